// g6_opmc.cu -- umbrella Monte Carlo on an order parameter (mc2.F90:505-520,
// 684-830 with OP_Q6T, OP_TRIANGLE and OP_EP).
//
// Order parameters of one chain (one CTA per chain):
//   Q6 (Q6Local.F90): bonds are the pairs within 3 A; the neighbourhood of k
//      is k and the molecules within 5 A; q6(k) = sqrt(4 pi/13 sum_m
//      |Q_m(k)|^2) / nbond(k), Q_m(k) summing Y_6m over the directed bonds
//      whose two ends are both in k's neighbourhood; op = mean of q6.
//   TRIANGLE (Triangle.F90): the cosines of the angles that the (at most) 4
//      nearest neighbours within 5 A span at each molecule, in 21 bins on
//      [-1, 1]; op = Kullback divergence from a reference histogram (or its
//      log).
//   EP: the chain's potential energy.
// State on the device (g6_op.cuh): per molecule its neighbours within 5 A
// with their vectors, for Q6 its bonds with their Y_6m, Q_m, nbond and q6;
// per chain the triangle counts and op.  k_op_prepare builds it from scratch
// (sq6system_prepareall, sTriangle_prepareall).
//
// A trial (k_mc_op): the energy warps sum dE as k_mc does and keep the
// molecules within 5 A of either pose of the target (a float pre-test with a
// margin, then the reference's FP64 image arithmetic); the whole CTA then
// evaluates the trial's order parameter incrementally (Differentiate):
//   Q6: only the target's bonds change.  Every molecule k within 5 A of
//      either pose loses 2 Y_6m of each old bond (t,j) with t and j in its old
//      neighbourhood and gains 2 Y_6m of each new bond with t and j in its new
//      one; the target's own Q_m is summed afresh over the directed bonds
//      inside its new neighbourhood; op is the fresh mean of q6 over the
//      chain, as the reference's sumq6.
//   TRIANGLE: the molecules whose 4 nearest include the target at either pose
//      (and the target) take their old angles out of the histogram and put
//      their new ones in; the counts are integers, so the incremental
//      histogram equals the fresh one exactly.
// The umbrella coeff (op - center)^2 enters the Metropolis test with dE
// (mc2.F90:700-722); an accepted trial commits the lists, bonds, sums and
// counts (Integrate), a rejected one leaves them as they were (Reject).
// Equal distances among a molecule's neighbours are ordered by label (the
// reference keeps its pair-list order).
#include <cuda_runtime.h>

#include <type_traits>

#include "g6_internal.cuh"
#include "g6_mctrial.cuh"
#include "g6_op.cuh"

namespace g6 {

constexpr int OP_POOL = 64;         // molecules within 5 A (+ margin) of either pose of a trial
constexpr int OP_WSEG = 16;         // per energy warp before the pool is compacted
constexpr float OP_PRE2 = 26.5f;    // float pre-test of |d|^2 [A^2] for the 5 A neighbourhoods
constexpr double OP_R5 = 25.0, OP_R3 = 9.0;

// Vector a -> b as neighbors_all2 stores it (Neighbor.F90:85-130): -(ca - cb
// - o) with the Compress2 image o; returns dd = dx^2 + dy^2 + dz^2.  Rounding
// is spelled out, so b -> a is exactly the negated vector with the same dd.
__device__ __forceinline__ double op_vec(const double* a, const double* b, const double L[3], const double iL[3],
                                         double v[3]) {
  double d[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const double delta = xsub(a[k], b[k]);
    d[k] = xsub(delta, xmul(xdnint(xmul(delta, iL[k])), L[k]));
    v[k] = -d[k];
  }
  return xadd(xadd(xmul(d[0], d[0]), xmul(d[1], d[1])), xmul(d[2], d[2]));
}

__device__ __forceinline__ double2 cmul_rn(double2 a, double2 b) {
  return make_double2(xsub(xmul(a.x, b.x), xmul(a.y, b.y)), xadd(xmul(a.x, b.y), xmul(a.y, b.x)));
}

// Associated Legendre function P_6^m(x) (the upward recurrence of q6.F90
// plgndr :69-100).
__device__ double legendre_6m(int m, double x) {
  double pmm = 1.0;
  if (m > 0) {
    const double somx2 = sqrt(xmul(xsub(1.0, x), xadd(1.0, x)));
    double fact = 1.0;
    for (int i = 1; i <= m; ++i) {
      pmm = xmul(xmul(-pmm, fact), somx2);
      fact = xadd(fact, 2.0);
    }
  }
  if (m == 6) return pmm;
  double pmmp1 = xmul(xmul(x, (double)(2 * m + 1)), pmm);
  if (m == 5) return pmmp1;
  double pll = 0.0;
  for (int ll = m + 2; ll <= 6; ++ll) {
    pll = xsub(xmul(xmul(x, (double)(2 * ll - 1)), pmmp1), xmul((double)(ll + m - 1), pmm)) / (double)(ll - m);
    pmm = pmmp1;
    pmmp1 = pll;
  }
  return pll;
}

// Y_6m and Y_6,-m (m >= 0) of the unit vector (x, y, z): cos(theta) = z,
// e^{i phi} = (x + iy)/sqrt(x^2 + y^2) (q6.F90 qlm, ylm2, ylm :24-66).
__device__ void y6m_pair(int m, double x, double y, double z, double2& pos, double2& neg) {
  const double fact[13] = {1.0, 1.0, 2.0, 6.0, 24.0, 120.0, 720.0, 5040.0, 40320.0, 362880.0, 3628800.0,
                           39916800.0, 479001600.0};
  const double rxy = sqrt(xadd(xmul(x, x), xmul(y, y)));
  const double2 w = make_double2(x / rxy, y / rxy);
  double2 wm = make_double2(1.0, 0.0);
  for (int q = 0; q < m; ++q) wm = cmul_rn(wm, w);
  const double norm = sqrt(xmul(13.0, fact[6 - m]) / xmul(xmul(4.0, PI), fact[6 + m]));
  const double p = xmul(norm, legendre_6m(m, z));
  pos = make_double2(xmul(p, wm.x), xmul(p, wm.y));
  const double sg = (m & 1) ? -1.0 : 1.0;
  neg = make_double2(sg * pos.x, -sg * pos.y);
}

// The 13 Y_6m of a bond along v (|v|^2 = dd), one thread.
__device__ void y6_bond(const double v[3], double dd, double2* out) {
  const double pp = 1.0 / sqrt(dd);
  const double x = xmul(v[0], pp), y = xmul(v[1], pp), z = xmul(v[2], pp);
  for (int m = 0; m <= 6; ++m) {
    double2 a, b;
    y6m_pair(m, x, y, z, a, b);
    out[6 + m] = a;
    if (m > 0) out[6 - m] = b;
  }
}

__device__ __forceinline__ double q6_value(const double2* q, int nb) {
  double s2 = 0.0;
#pragma unroll
  for (int m = 0; m < OP_NM; ++m) {
    const double a = hypot(q[m].x, q[m].y);
    s2 = xadd(s2, xmul(a, a));
  }
  return sqrt(xmul(xmul(s2, 4.0), PI) / 13.0) / (double)nb;
}

// Histogram bin of a cosine (histogram_accumulate, DistribModule.F90): nint((x
// - (-1)) / 0.1), or -1 outside the 21 bins.
__device__ __forceinline__ int tri_bin(double c) {
  const int b = (int)round(__ddiv_rn(xsub(c, -1.0), 0.1));
  return (b >= 0 && b < OP_NBIN) ? b : -1;
}

// Cosine of the angle between a and b at a molecule (Triangle.F90:80-82).
__device__ __forceinline__ double tri_cos(const double4& a, const double4& b) {
  const double dot = xadd(xadd(xmul(a.x, b.x), xmul(a.y, b.y)), xmul(a.z, b.z));
  return __ddiv_rn(dot, sqrt(xmul(a.w, b.w)));
}

// kullback_div (DistribModule.F90:304-326) of counts h against ref.
__device__ double tri_divergence(const int* h, const double* ref, int logarithmic) {
  double s1 = 0.0, s2 = 0.0;
  for (int i = 0; i < OP_NBIN; ++i) { s1 = xadd(s1, (double)h[i]); s2 = xadd(s2, ref[i]); }
  double div = 0.0;
  for (int i = 0; i < OP_NBIN; ++i) {
    const double p = __ddiv_rn((double)h[i], s1);
    double q = __ddiv_rn(ref[i], s2);
    if (q == 0.0) q = p;
    if (p != 0.0) div = xadd(div, xmul(p, log(__ddiv_rn(p, q))));
  }
  return logarithmic ? log(div) : div;
}

// The (at most) 4 nearest of a neighbour list, by (dd, label).
struct Near4 {
  int n;
  int j[4];
  double4 v[4];
  __device__ void clear() { n = 0; }
  __device__ void offer(int lj, const double4& lv) {
    int pos = n;
    while (pos > 0 && (lv.w < v[pos - 1].w || (lv.w == v[pos - 1].w && lj < j[pos - 1]))) --pos;
    if (pos >= 4) return;
    const int last = n < 4 ? n : 3;
    for (int q = last; q > pos; --q) { j[q] = j[q - 1]; v[q] = v[q - 1]; }
    j[pos] = lj;
    v[pos] = lv;
    if (n < 4) ++n;
  }
  __device__ bool has(int lj) const {
    for (int q = 0; q < n; ++q)
      if (j[q] == lj) return true;
    return false;
  }
  // its angles into the histogram with weight w
  __device__ void angles(int* dh, int w) const {
    for (int a = 0; a < n; ++a)
      for (int b = a + 1; b < n; ++b) {
        const int bin = tri_bin(tri_cos(v[a], v[b]));
        if (bin >= 0) atomicAdd(dh + bin, w);
      }
  }
};

__device__ __forceinline__ double block_sum(double v, double* red) {
#pragma unroll
  for (int m = 16; m >= 1; m >>= 1) v += __shfl_xor_sync(0xffffffffu, v, m);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double s = 0.0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
  return s;
}

__device__ __forceinline__ bool in_n5(const OpDev& o, int k, int j) {
  const int cnt = o.n5c[k];
  const int* lj = o.n5j + (size_t)k * OP_N5;
  for (int s = 0; s < cnt; ++s)
    if (lj[s] == j) return true;
  return false;
}

// ---------------------------------------------------------------------------
// State from scratch (sq6system_prepareall, sTriangle_prepareall)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(MC_NT) k_op_prepare(McArgs a, OpDev o) {
  __shared__ double s_red[32];
  __shared__ int s_h[OP_NBIN];
  const int c = blockIdx.x;
  const int i0 = a.rep.off[c], i1 = a.rep.off[c + 1], nc = i1 - i0, n = a.n;
  double L[3], iL[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) { L[k] = a.rep.L[3 * c + k]; iL[k] = a.rep.invL[3 * c + k]; }
  const float fs[3] = {a.rep.fscale[3 * c], a.rep.fscale[3 * c + 1], a.rep.fscale[3 * c + 2]};
  if (threadIdx.x < OP_NBIN) s_h[threadIdx.x] = 0;
  // neighbours within 5 A, by label
  for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
    const uint32_t fi[3] = {a.fix[i], a.fix[n + i], a.fix[2 * n + i]};
    const double ci[3] = {a.st[i], a.st[(size_t)n + i], a.st[2 * (size_t)n + i]};
    int cnt = 0;
    for (int j = i0; j < i1; ++j) {
      if (j == i) continue;
      const uint32_t fj[3] = {a.fix[j], a.fix[n + j], a.fix[2 * n + j]};
      float e[3];
      if (fvec_fix(fi, fj, fs, e) >= OP_PRE2) continue;
      const double cj[3] = {a.st[j], a.st[(size_t)n + j], a.st[2 * (size_t)n + j]};
      double v[3];
      const double dd = op_vec(ci, cj, L, iL, v);
      if (OP_R5 < dd) continue;
      if (cnt < OP_N5) {
        o.n5j[(size_t)i * OP_N5 + cnt] = j;
        o.n5v[(size_t)i * OP_N5 + cnt] = make_double4(v[0], v[1], v[2], dd);
      } else {
        *o.flag = 1;
      }
      ++cnt;
    }
    o.n5c[i] = min(cnt, OP_N5);
  }
  __syncthreads();
  double op = 0.0;
  if (o.kind == G6_OP_Q6) {
    // bonds and their Y_6m
    for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
      int nbd = 0;
      for (int s = 0; s < o.n5c[i]; ++s) {
        const double4 e = o.n5v[(size_t)i * OP_N5 + s];
        if (OP_R3 < e.w) continue;
        if (nbd < OP_NB) {
          const double v[3] = {e.x, e.y, e.z};
          o.bj[(size_t)i * OP_NB + nbd] = o.n5j[(size_t)i * OP_N5 + s];
          y6_bond(v, e.w, o.bq + ((size_t)i * OP_NB + nbd) * OP_NM);
        } else {
          *o.flag = 1;
        }
        ++nbd;
      }
      o.bc[i] = min(nbd, OP_NB);
    }
    __syncthreads();
    // Q_m(k) over the directed bonds with both ends in k's neighbourhood
    double part = 0.0;
    for (int k = i0 + threadIdx.x; k < i1; k += blockDim.x) {
      double2 q[OP_NM];
#pragma unroll
      for (int m = 0; m < OP_NM; ++m) q[m] = make_double2(0.0, 0.0);
      int nbk = 0;
      const int nk = o.n5c[k];
      for (int s = -1; s < nk; ++s) {
        const int i = s < 0 ? k : o.n5j[(size_t)k * OP_N5 + s];
        for (int b = 0; b < o.bc[i]; ++b) {
          const int j = o.bj[(size_t)i * OP_NB + b];
          if (j != k && !in_n5(o, k, j)) continue;
          ++nbk;
          const double2* bq = o.bq + ((size_t)i * OP_NB + b) * OP_NM;
#pragma unroll
          for (int m = 0; m < OP_NM; ++m) q[m] = make_double2(xadd(q[m].x, bq[m].x), xadd(q[m].y, bq[m].y));
        }
      }
#pragma unroll
      for (int m = 0; m < OP_NM; ++m) o.qs[(size_t)k * OP_NM + m] = q[m];
      o.nb[k] = nbk;
      const double v = q6_value(q, nbk);
      o.q6[k] = v;
      part += v;
    }
    op = block_sum(part, s_red) / (double)nc;
  } else if (o.kind == G6_OP_TRIANGLE) {
    for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
      Near4 nr;
      nr.clear();
      for (int s = 0; s < o.n5c[i]; ++s) nr.offer(o.n5j[(size_t)i * OP_N5 + s], o.n5v[(size_t)i * OP_N5 + s]);
      nr.angles(s_h, 1);
    }
    __syncthreads();
    if (threadIdx.x < OP_NBIN) o.hist[c * OP_NBIN + threadIdx.x] = s_h[threadIdx.x];
    op = tri_divergence(s_h, o.ref, o.logarithmic);
  } else {
    op = a.energy[c];
  }
  if (threadIdx.x == 0) o.op[c] = op;
}

cudaError_t launch_op_prepare(const McArgs& a, const OpDev& o, cudaStream_t s) {
  k_op_prepare<<<a.rep.nrep, MC_NT, 0, s>>>(a, o);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Umbrella chains
// ---------------------------------------------------------------------------
template <int NQ, bool TAPER, bool MIXED, int KIND>
__global__ void __launch_bounds__(MC_NT) k_mc_op(McArgs a, OpDev o) {
  using R = typename std::conditional<MIXED, float, double>::type;
  using P = PoseRead<NQ, MIXED>;
  using TP = TrialPose<R, NQ>;
  constexpr bool Q6 = KIND == G6_OP_Q6, TRI = KIND == G6_OP_TRIANGLE, POOL = Q6 || TRI;
  constexpr int E0 = 32, NE = MC_NT - E0, NEW = NE / 32;
  constexpr int W64 = P::W64, NPK = P::NPK;
  __shared__ typename std::conditional<MIXED, float, double>::type s_lu[MC_NB];
  __shared__ R s_g[6][MC_NB];
  __shared__ int s_tg[MC_NB];
  __shared__ TP s_pose;
  __shared__ R s_part[NEW];
  __shared__ int s_seg[NEW][MC_SEG];
  __shared__ int s_wseg[NEW][OP_WSEG];   // each energy warp's molecules near either pose
  __shared__ int s_wcnt[NEW];
  __shared__ int s_np, s_accept;
  __shared__ int s_pj[OP_POOL];          // the trial's pool: molecule
  __shared__ double4 s_po[OP_POOL];      // vector target(old) -> molecule, dd
  __shared__ double4 s_pn[OP_POOL];      // vector target(new) -> molecule, dd
  __shared__ double s_red[32];
  __shared__ double s_opnew;
  // Q6
  __shared__ int s_nbo, s_nbn, s_bold[OP_NB], s_bnew[OP_NB], s_pnb[OP_POOL];
  __shared__ double2 s_qn[OP_NB][OP_NM];   // Y_6m of the target's new bonds
  __shared__ unsigned s_mask[OP_POOL];     // bit b: bond b (old bonds, then new) has both ends in the molecule's neighbourhood
  __shared__ double2 s_dq[OP_POOL][OP_NM];
  __shared__ int s_dnb[OP_POOL];
  __shared__ double s_q6n[OP_POOL];
  __shared__ double2 s_qt[OP_NM];
  __shared__ int s_nbt;
  __shared__ double s_q6t;
  // TRIANGLE
  __shared__ int s_dh[OP_NBIN];
  // per molecule of the chain: pool index + 1 (s_aff), in the target's new neighbourhood (s_innew)
  extern __shared__ unsigned char s_dyn[];
  unsigned short* s_aff = reinterpret_cast<unsigned short*>(s_dyn);
  unsigned char* s_innew = s_dyn + 2 * (size_t)a.ncmax;

  const int c = blockIdx.x;
  const int i0 = a.rep.off[c], i1 = a.rep.off[c + 1], nc = i1 - i0;
  const int n = a.n;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double L[3], iL[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) { L[k] = a.rep.L[3 * c + k]; iL[k] = a.rep.invL[3 * c + k]; }
  const float fs[3] = {a.rep.fscale[3 * c], a.rep.fscale[3 * c + 1], a.rep.fscale[3 * c + 2]};
  const double beta = a.beta[c];
  const float fbeta_e = (float)(I2J * J2K * beta);
  const R sig_t_fixed = (R)sqrt(a.sigma_t[c] * a.sigma_t[c]);
  const R sig_r_fixed = (R)sqrt(a.sigma_r[c] * a.sigma_r[c]);
  const float fsi[3] = {(float)(4294967296.0 * iL[0]), (float)(4294967296.0 * iL[1]), (float)(4294967296.0 * iL[2])};
  const double ucen = o.umb[2 * c], ucoef = o.umb[2 * c + 1];
  for (int i = threadIdx.x; i < nc; i += blockDim.x) { s_aff[i] = 0; s_innew[i] = 0; }
  if (threadIdx.x < OP_NBIN) s_dh[threadIdx.x] = 0;
  if (threadIdx.x == 0) s_pose.trial = -1;
  __syncthreads();

  const R rin2 = MIXED ? (R)a.cc.frin2 : (R)a.cc.rin2, rin = MIXED ? (R)a.cc.frin : (R)a.cc.rin;
  const R rout = MIXED ? (R)a.cc.frout : (R)a.cc.rout, c1 = MIXED ? (R)a.cc.fc1 : (R)a.cc.c1;
  // the running energy and order parameter live in warp 0 (thread 0 writes them back)
  double energy = a.energy[c];
  double op = POOL ? o.op[c] : energy;
  long long nacc = 0;
  int nsample = 0;

  for (int t = 0; t < a.ntrial; ++t) {
    const int tb = t % MC_NB;
    if (tb == 0) {   // draws of the next MC_NB trials, as k_mc
      __syncthreads();
      const int tt = t + (int)threadIdx.x;
      if (threadIdx.x < MC_NB && tt < a.ntrial) {
        const uint64_t trial = a.counter + (uint64_t)tt;
        const uint32_t lo = (uint32_t)trial, hi = (uint32_t)(trial >> 32);
        double u[2];
        uniform2(a.seed, (uint32_t)c, lo, hi, 0u, u);
        int tg = (int)(u[0] * nc);
        if (tg >= nc) tg = nc - 1;
        s_tg[threadIdx.x] = tg;
        if constexpr (MIXED) s_lu[threadIdx.x] = logf((float)u[1]);
        else s_lu[threadIdx.x] = log(u[1]);
#pragma unroll 1
        for (int k = 0; k < 6; ++k) {
          uniform2(a.seed, (uint32_t)c, lo, hi, 1u + k, u);
          if constexpr (MIXED) s_g[k][threadIdx.x] = sqrtf(-2.0f * logf((float)u[0])) * sinpif(2.0f * (float)u[1]);
          else s_g[k][threadIdx.x] = sqrt(-2.0 * log(u[0])) * sin(2.0 * PI * u[1]);
        }
      }
      __syncthreads();
    }
    const int tg = i0 + s_tg[tb];
    TP& cur = s_pose;
    if (warp == 0) build_trial<R, NQ, MIXED, MIXED>(a, cur, t, tg, s_g, tb, sig_t_fixed, sig_r_fixed, iL, fsi);
    __syncthreads();
    if ((int)threadIdx.x >= E0) {
      // ---- energy warps: dE over every other molecule (k_mc's two passes) ----
      R acc = R(0);
      R ro[NQ + 1][3], rn[NQ + 1][3];
#pragma unroll
      for (int s = 0; s <= NQ; ++s)
#pragma unroll
        for (int k = 0; k < 3; ++k) { ro[s][k] = cur.oo[s][k]; rn[s][k] = cur.on[s][k]; }
      const uint32_t fo[3] = {cur.fo[0], cur.fo[1], cur.fo[2]}, fn[3] = {cur.fn[0], cur.fn[1], cur.fn[2]};
      const double co[3] = {cur.co[0], cur.co[1], cur.co[2]}, cn[3] = {cur.cn[0], cur.cn[1], cur.cn[2]};
      auto separations = [&](int j, R (&dO)[3], R (&dN)[3], R& ddO, R& ddN, bool& inO, bool& inN) {
        if (MIXED) {
          uint32_t fj[3];
          P::fix(a, j, fj);
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            dO[k] = (R)((float)(int)(fo[k] - fj[k]) * fs[k]);
            dN[k] = (R)((float)(int)(fn[k] - fj[k]) * fs[k]);
          }
          ddO = dO[0] * dO[0] + dO[1] * dO[1] + dO[2] * dO[2];
          ddN = dN[0] * dN[0] + dN[1] * dN[1] + dN[2] * dN[2];
          inO = ddO < (R)a.cc.frout2;
          inN = ddN < (R)a.cc.frout2;
          const bool bandO = fabsf((float)ddO - a.cc.frout2) < 1e-3f, bandN = fabsf((float)ddN - a.cc.frout2) < 1e-3f;
          if (bandO || bandN) {
            double cj[3], oo[3], dx[3];
            P::com(a, j, cj);
            if (bandO) inO = exact_dd(co, cj, L, iL, oo, dx) < a.cc.rout2;
            if (bandN) inN = exact_dd(cn, cj, L, iL, oo, dx) < a.cc.rout2;
          }
        } else {
          double cj[3], oo[3], dx[3];
          P::com(a, j, cj);
          const double d0 = exact_dd(co, cj, L, iL, oo, dx);
          dO[0] = dx[0]; dO[1] = dx[1]; dO[2] = dx[2];
          ddO = (R)d0;
          inO = d0 < a.cc.rout2;
          const double d1 = exact_dd(cn, cj, L, iL, oo, dx);
          dN[0] = dx[0]; dN[1] = dx[1]; dN[2] = dx[2];
          ddN = (R)d1;
          inN = d1 < a.cc.rout2;
        }
      };
      auto pair_dE = [&](int j, const R (&dO)[3], const R (&dN)[3], R ddO, R ddN, bool inO, bool inN) {
        R rj[NQ + 1][3];
#pragma unroll
        for (int s = 0; s <= NQ; ++s)
#pragma unroll
          for (int k = 0; k < 3; ++k)
            rj[s][k] = MIXED ? (R)a.pk32f[(size_t)j * 4 * NPK + 3 + 3 * s + k] : (R)a.pk64[(size_t)j * W64 + 3 + 3 * s + k];
        R v = R(0);
        if (inO) v -= pair_energy<NQ, TAPER, R>(dO, ddO, ro, rj, a.pc, rin2, rin, rout, c1);
        if (inN) v += pair_energy<NQ, TAPER, R>(dN, ddN, rn, rj, a.pc, rin2, rin, rout, c1);
        return v;
      };
      const int ew = warp - 1;
      int* seg = s_seg[ew];
      int nseg = 0, nw = 0;
      for (int j0 = i0 + 32 * ew; j0 < i1; j0 += NE) {
        const int j = j0 + lane;
        R dO[3] = {R(0), R(0), R(0)}, dN[3] = {R(0), R(0), R(0)}, ddO = R(0), ddN = R(0);
        bool inO = false, inN = false;
        const bool valid = j < i1 && j != tg;
        if (valid) separations(j, dO, dN, ddO, ddN, inO, inN);
        const bool take = inO || inN;
        const unsigned m = __ballot_sync(0xffffffffu, take);
        if (take) {
          const int pos = nseg + __popc(m & ((1u << lane) - 1u));
          if (pos < MC_SEG) seg[pos] = j;
          else acc += pair_dE(j, dO, dN, ddO, ddN, inO, inN);
        }
        nseg += __popc(m);
        if constexpr (POOL) {
          const bool near = valid && ((float)ddO < OP_PRE2 || (float)ddN < OP_PRE2);
          const unsigned mw = __ballot_sync(0xffffffffu, near);
          if (near) {
            const int pos = nw + __popc(mw & ((1u << lane) - 1u));
            if (pos < OP_WSEG) s_wseg[ew][pos] = j;
            else *o.flag = 1;
          }
          nw += __popc(mw);
        }
      }
      if (POOL && lane == 0) s_wcnt[ew] = min(nw, OP_WSEG);
      __syncwarp();
      const int ns = min(nseg, MC_SEG);
      for (int q = lane; q < ns; q += 32) {
        const int j = seg[q];
        R dO[3], dN[3], ddO, ddN;
        bool inO, inN;
        separations(j, dO, dN, ddO, ddN, inO, inN);
        acc += pair_dE(j, dO, dN, ddO, ddN, inO, inN);
      }
#pragma unroll
      for (int m = 16; m >= 1; m >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, m);
      if (lane == 0) s_part[ew] = acc;
    }
    __syncthreads();

    if constexpr (POOL) {
      // ---- the pool: molecules near either pose, FP64 vectors from the target ----
      {
        const int ew = threadIdx.x / OP_WSEG, q = threadIdx.x % OP_WSEG;
        if (ew < NEW && q < s_wcnt[ew]) {
          int off = 0;
          for (int w = 0; w < ew; ++w) off += s_wcnt[w];
          const int p = off + q;
          if (p < OP_POOL) {
            const int j = s_wseg[ew][q];
            double cj[3], v[3];
            P::com(a, j, cj);
            const double co[3] = {cur.co[0], cur.co[1], cur.co[2]}, cn[3] = {cur.cn[0], cur.cn[1], cur.cn[2]};
            const double ddo = op_vec(co, cj, L, iL, v);
            s_po[p] = make_double4(v[0], v[1], v[2], ddo);
            const double ddn = op_vec(cn, cj, L, iL, v);
            s_pn[p] = make_double4(v[0], v[1], v[2], ddn);
            s_pj[p] = j;
            s_aff[j - i0] = (unsigned short)(p + 1);
            if (!(OP_R5 < ddn)) s_innew[j - i0] = 1;
          } else {
            *o.flag = 1;
          }
        }
        if (threadIdx.x == 0) {
          int tot = 0;
          for (int w = 0; w < NEW; ++w) tot += s_wcnt[w];
          s_np = min(tot, OP_POOL);
        }
      }
      __syncthreads();
      const int np = s_np;
      if constexpr (Q6) {
        // old bonds of the target; new bonds = pool molecules within 3 A of the new pose (pool order)
        if (warp == 0) {
          const int nbo = o.bc[tg];
          if (lane < nbo) s_bold[lane] = o.bj[(size_t)tg * OP_NB + lane];
          int nbn = 0;
          for (int p0 = 0; p0 < np; p0 += 32) {
            const int p = p0 + lane;
            const bool bond = p < np && !(OP_R3 < s_pn[p].w);
            const unsigned m = __ballot_sync(0xffffffffu, bond);
            if (p < np) s_pnb[p] = -1;
            if (bond) {
              const int b = nbn + __popc(m & ((1u << lane) - 1u));
              if (b < OP_NB) { s_bnew[b] = p; s_pnb[p] = b; }
              else *o.flag = 1;
            }
            nbn += __popc(m);
          }
          if (lane == 0) { s_nbo = nbo; s_nbn = min(nbn, OP_NB); }
        }
        __syncthreads();
        const int nbo = s_nbo, nbn = s_nbn;
        // Y_6m of the new bonds (one thread per bond and |m|) and the
        // neighbourhood masks (one thread per pool molecule and bond)
        for (int x = threadIdx.x; x < nbn * 7; x += blockDim.x) {
          const int b = x / 7, m = x % 7;
          const double4 e = s_pn[s_bnew[b]];
          const double pp = 1.0 / sqrt(e.w);
          double2 ps, ng;
          y6m_pair(m, xmul(e.x, pp), xmul(e.y, pp), xmul(e.z, pp), ps, ng);
          s_qn[b][6 + m] = ps;
          if (m > 0) s_qn[b][6 - m] = ng;
        }
        for (int p = threadIdx.x; p < np; p += blockDim.x) s_mask[p] = 0u;
        __syncthreads();
        for (int x = threadIdx.x; x < np * (nbo + nbn); x += blockDim.x) {
          const int p = x / (nbo + nbn), b = x % (nbo + nbn);
          const int k = s_pj[p];
          const int j = b < nbo ? s_bold[b] : s_pj[s_bnew[b - nbo]];
          if (j == k || in_n5(o, k, j)) atomicOr(&s_mask[p], 1u << b);
        }
        __syncthreads();
        // dQ_m of every pool molecule: -2 Y of old bonds (target in its old
        // neighbourhood), +2 Y of new bonds (target in its new one)
        for (int x = threadIdx.x; x < np * OP_NM; x += blockDim.x) {
          const int p = x / OP_NM, m = x % OP_NM;
          const bool inO = !(OP_R5 < s_po[p].w), inN = !(OP_R5 < s_pn[p].w);
          const unsigned mk = s_mask[p];
          double2 d = make_double2(0.0, 0.0);
          int dn = 0;
          if (inO)
            for (int b = 0; b < nbo; ++b)
              if (mk & (1u << b)) {
                const double2 y = o.bq[((size_t)tg * OP_NB + b) * OP_NM + m];
                d = make_double2(xsub(d.x, xmul(2.0, y.x)), xsub(d.y, xmul(2.0, y.y)));
                dn -= 2;
              }
          if (inN)
            for (int b = 0; b < nbn; ++b)
              if (mk & (1u << (nbo + b))) {
                const double2 y = s_qn[b][m];
                d = make_double2(xadd(d.x, xmul(2.0, y.x)), xadd(d.y, xmul(2.0, y.y)));
                dn += 2;
              }
          s_dq[p][m] = d;
          if (m == 0) s_dnb[p] = dn;
        }
        // the target's Q_m afresh: warp m sums the directed bonds inside its new neighbourhood
        if (warp < OP_NM) {
          const int m = warp;
          double re = 0.0, im = 0.0;
          int cnt = 0;
          for (int p = lane; p < np; p += 32) {
            if (OP_R5 < s_pn[p].w) continue;
            const int i = s_pj[p];
            for (int b = 0; b < o.bc[i]; ++b) {
              const int j = o.bj[(size_t)i * OP_NB + b];
              if (j == tg || !s_innew[j - i0]) continue;
              const double2 y = o.bq[((size_t)i * OP_NB + b) * OP_NM + m];
              re = xadd(re, y.x);
              im = xadd(im, y.y);
              ++cnt;
            }
          }
#pragma unroll
          for (int s = 16; s >= 1; s >>= 1) {
            re += __shfl_xor_sync(0xffffffffu, re, s);
            im += __shfl_xor_sync(0xffffffffu, im, s);
            cnt += __shfl_xor_sync(0xffffffffu, cnt, s);
          }
          if (lane == 0) {
            for (int b = 0; b < nbn; ++b) {   // (t -> j) and (j -> t) of the new bonds
              re = xadd(re, xmul(2.0, s_qn[b][m].x));
              im = xadd(im, xmul(2.0, s_qn[b][m].y));
            }
            s_qt[m] = make_double2(re, im);
            if (m == 0) s_nbt = cnt + 2 * nbn;
          }
        }
        __syncthreads();
        // q6 at the trial: pool molecules and the target
        for (int p = threadIdx.x; p < np; p += blockDim.x) {
          const int k = s_pj[p];
          const bool hit = !(OP_R5 < s_po[p].w) || !(OP_R5 < s_pn[p].w);
          double v = o.q6[k];
          if (hit) {
            double2 q[OP_NM];
#pragma unroll
            for (int m = 0; m < OP_NM; ++m) {
              const double2 a0 = o.qs[(size_t)k * OP_NM + m], d = s_dq[p][m];
              q[m] = make_double2(xadd(a0.x, d.x), xadd(a0.y, d.y));
            }
            v = q6_value(q, o.nb[k] + s_dnb[p]);
          }
          s_q6n[p] = v;
        }
        if (threadIdx.x == blockDim.x - 1) s_q6t = q6_value(s_qt, s_nbt);
        __syncthreads();
        // op of the trial: the fresh mean of q6 over the chain
        double part = 0.0;
        for (int i = threadIdx.x; i < nc; i += blockDim.x) {
          const int k = i0 + i;
          part += k == tg ? s_q6t : (s_aff[i] ? s_q6n[s_aff[i] - 1] : o.q6[k]);
        }
        const double sum = block_sum(part, s_red);
        if (threadIdx.x == 0) s_opnew = sum / (double)nc;
      } else {
        // ---- TRIANGLE: old angles out, new angles in, for every molecule whose 4 nearest hold the target ----
        for (int p = threadIdx.x; p < np; p += blockDim.x) {
          const int k = s_pj[p];
          const bool inO = !(OP_R5 < s_po[p].w), inN = !(OP_R5 < s_pn[p].w);
          if (!inO && !inN) continue;
          Near4 a4, b4;
          a4.clear();
          b4.clear();
          const int cnt = o.n5c[k];
          for (int s = 0; s < cnt; ++s) {
            const int j = o.n5j[(size_t)k * OP_N5 + s];
            const double4 v = o.n5v[(size_t)k * OP_N5 + s];
            a4.offer(j, v);
            if (j != tg) b4.offer(j, v);
          }
          if (inN) {
            const double4 e = s_pn[p];
            b4.offer(tg, make_double4(-e.x, -e.y, -e.z, e.w));
          }
          if (!a4.has(tg) && !b4.has(tg)) continue;
          a4.angles(s_dh, -1);
          b4.angles(s_dh, 1);
        }
        if (threadIdx.x == blockDim.x - 1) {   // the target
          Near4 a4, b4;
          a4.clear();
          b4.clear();
          for (int s = 0; s < o.n5c[tg]; ++s) a4.offer(o.n5j[(size_t)tg * OP_N5 + s], o.n5v[(size_t)tg * OP_N5 + s]);
          for (int p = 0; p < np; ++p)
            if (!(OP_R5 < s_pn[p].w)) b4.offer(s_pj[p], s_pn[p]);
          a4.angles(s_dh, -1);
          b4.angles(s_dh, 1);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
          int h[OP_NBIN];
          for (int b = 0; b < OP_NBIN; ++b) h[b] = o.hist[c * OP_NBIN + b] + s_dh[b];
          s_opnew = tri_divergence(h, o.ref, o.logarithmic);
        }
      }
    }
    __syncthreads();
    // ---- warp 0: Metropolis test with the umbrella, the accepted pose ----
    if (warp == 0) {
      R v = lane < NEW ? s_part[lane] : R(0);
#pragma unroll
      for (int m = 16; m >= 1; m >>= 1) v += __shfl_xor_sync(0xffffffffu, v, m);
      const R dEr = __shfl_sync(0xffffffffu, v, 0);
      const double dE = (double)dEr;
      const double newop = POOL ? s_opnew : energy + dE;
      int acc_flag = 0;
      if (lane == 0) {
        const double dU = ucoef * ((newop - ucen) * (newop - ucen)) - ucoef * ((op - ucen) * (op - ucen));
        bool ok;
        if (MIXED) {
          const float x = -(float)(dE + dU) * fbeta_e;
          ok = x >= 0.0f || (float)s_lu[tb] < x;
        } else {
          const double x = -((dE + dU) * I2J * J2K) * beta;
          ok = x >= 0.0 || (double)s_lu[tb] < x;
        }
        acc_flag = ok ? 1 : 0;
        s_accept = acc_flag;
      }
      acc_flag = __shfl_sync(0xffffffffu, acc_flag, 0);
      if (acc_flag) {
        const double q64 = cur.q64[lane & 3];
        double* pp = a.pk64 + (size_t)tg * W64;
        float* pf = a.pk32f + (size_t)tg * 4 * NPK;
        if (lane < 4) a.st[(size_t)(33 + lane) * n + tg] = q64;
        if (lane < 3) {
          const double cn = cur.cn[lane];
          const uint32_t fw = cur.fn[lane];
          a.st[(size_t)lane * n + tg] = cn;
          pp[lane] = cn;
          pf[lane] = __uint_as_float(fw);
          a.fix[(size_t)lane * n + tg] = fw;
        }
        if (lane < 3 * (NQ + 1)) {
          const R ov = (&cur.on[0][0])[lane];
          pf[3 + lane] = (float)ov;
          if (!MIXED) pp[3 + lane] = (double)ov;
        }
        energy += dE;
        op = newop;
        if (lane == 0) ++nacc;
      }
      if (lane == 0) {
        if (a.trace) {
          double* tr = a.trace + ((size_t)c * a.ntrial + t) * 5;
          tr[0] = dE; tr[1] = energy; tr[2] = (double)acc_flag; tr[3] = (double)(tg - i0); tr[4] = op;
        }
        if (a.sample_every > 0 && (t + 1) % a.sample_every == 0) {
          if (a.samples) a.samples[(size_t)c * a.nsamples + nsample] = energy;
          if (o.opsamp) o.opsamp[(size_t)c * a.nsamples + nsample] = op;
        }
      }
    }
    __syncthreads();
    if constexpr (POOL) {
      // ---- Integrate (accepted) or Reject: commit the trial's lists, then clear the marks ----
      const bool accepted = s_accept != 0;
      const int np = s_np;
      for (int p = threadIdx.x; p < np; p += blockDim.x) {
        const int k = s_pj[p];
        if (accepted) {
          const double4 eo = s_po[p], en = s_pn[p];
          const bool inO = !(OP_R5 < eo.w), inN = !(OP_R5 < en.w);
          int* lj = o.n5j + (size_t)k * OP_N5;
          double4* lv = o.n5v + (size_t)k * OP_N5;
          const double4 back = make_double4(-en.x, -en.y, -en.z, en.w);   // k -> target (new)
          if (inO) {
            int s = 0;
            const int cnt = o.n5c[k];
            while (s < cnt && lj[s] != tg) ++s;
            if (s < cnt) {
              if (inN) {
                lv[s] = back;
              } else {
                lj[s] = lj[cnt - 1];
                lv[s] = lv[cnt - 1];
                o.n5c[k] = cnt - 1;
              }
            }
          } else if (inN) {
            const int cnt = o.n5c[k];
            if (cnt < OP_N5) { lj[cnt] = tg; lv[cnt] = back; o.n5c[k] = cnt + 1; }
            else *o.flag = 1;
          }
          if constexpr (Q6) {
            const bool bO = !(OP_R3 < eo.w), bN = !(OP_R3 < en.w) && s_pnb[p] >= 0;
            int* bj = o.bj + (size_t)k * OP_NB;
            double2* bq = o.bq + (size_t)k * OP_NB * OP_NM;
            if (bO) {
              int s = 0;
              const int cnt = o.bc[k];
              while (s < cnt && bj[s] != tg) ++s;
              if (s < cnt) {
                if (bN) {
                  for (int m = 0; m < OP_NM; ++m) bq[s * OP_NM + m] = s_qn[s_pnb[p]][m];
                } else {
                  bj[s] = bj[cnt - 1];
                  for (int m = 0; m < OP_NM; ++m) bq[s * OP_NM + m] = bq[(cnt - 1) * OP_NM + m];
                  o.bc[k] = cnt - 1;
                }
              }
            } else if (bN) {
              const int cnt = o.bc[k];
              if (cnt < OP_NB) {
                bj[cnt] = tg;
                for (int m = 0; m < OP_NM; ++m) bq[cnt * OP_NM + m] = s_qn[s_pnb[p]][m];
                o.bc[k] = cnt + 1;
              } else {
                *o.flag = 1;
              }
            }
            if (inO || inN) {
              for (int m = 0; m < OP_NM; ++m) {
                double2& q = o.qs[(size_t)k * OP_NM + m];
                q = make_double2(xadd(q.x, s_dq[p][m].x), xadd(q.y, s_dq[p][m].y));
              }
              o.nb[k] += s_dnb[p];
              o.q6[k] = s_q6n[p];
            }
          }
        }
        s_aff[k - i0] = 0;
        s_innew[k - i0] = 0;
      }
      if (accepted && warp == 1) {   // the target's own lists
        int cnt = 0;
        for (int p0 = 0; p0 < np; p0 += 32) {
          const int p = p0 + lane;
          const bool in = p < np && !(OP_R5 < s_pn[p].w);
          const unsigned m = __ballot_sync(0xffffffffu, in);
          if (in) {
            const int s = cnt + __popc(m & ((1u << lane) - 1u));
            if (s < OP_N5) { o.n5j[(size_t)tg * OP_N5 + s] = s_pj[p]; o.n5v[(size_t)tg * OP_N5 + s] = s_pn[p]; }
            else *o.flag = 1;
          }
          cnt += __popc(m);
        }
        if (lane == 0) o.n5c[tg] = min(cnt, OP_N5);
        if constexpr (Q6) {
          const int nbn = s_nbn;
          if (lane < nbn) o.bj[(size_t)tg * OP_NB + lane] = s_pj[s_bnew[lane]];
          for (int x = lane; x < nbn * OP_NM; x += 32)
            o.bq[(size_t)tg * OP_NB * OP_NM + x] = s_qn[x / OP_NM][x % OP_NM];
          if (lane < OP_NM) o.qs[(size_t)tg * OP_NM + lane] = s_qt[lane];
          if (lane == 0) { o.bc[tg] = nbn; o.nb[tg] = s_nbt; o.q6[tg] = s_q6t; }
        }
      }
      if constexpr (TRI) {
        if (threadIdx.x < OP_NBIN) {
          if (accepted) o.hist[c * OP_NBIN + threadIdx.x] += s_dh[threadIdx.x];
          s_dh[threadIdx.x] = 0;
        }
      }
      __syncthreads();
    }
    if (a.sample_every > 0 && (t + 1) % a.sample_every == 0) ++nsample;
  }
  if (threadIdx.x == 0) {
    a.energy[c] = energy;
    a.counts[2 * c] += nacc;
    a.counts[2 * c + 1] += a.ntrial;
    o.op[c] = op;
  }
}

template <int NQ, bool TAPER, bool MIXED, int KIND>
static cudaError_t launch_mc_op_k(const McArgs& a, const OpDev& o, cudaStream_t s) {
  const size_t dyn = 3 * (size_t)a.ncmax;
  k_mc_op<NQ, TAPER, MIXED, KIND><<<a.rep.nrep, MC_NT, dyn, s>>>(a, o);
  return cudaGetLastError();
}

template <int NQ, bool TAPER, bool MIXED>
static cudaError_t launch_mc_op_m(const McArgs& a, const OpDev& o, cudaStream_t s) {
  if (o.kind == G6_OP_Q6) return launch_mc_op_k<NQ, TAPER, MIXED, G6_OP_Q6>(a, o, s);
  if (o.kind == G6_OP_TRIANGLE) return launch_mc_op_k<NQ, TAPER, MIXED, G6_OP_TRIANGLE>(a, o, s);
  return launch_mc_op_k<NQ, TAPER, MIXED, G6_OP_EP>(a, o, s);
}

template <int NQ, bool TAPER>
static cudaError_t launch_mc_op_t(const McArgs& a, const OpDev& o, bool mixed, cudaStream_t s) {
  return mixed ? launch_mc_op_m<NQ, TAPER, true>(a, o, s) : launch_mc_op_m<NQ, TAPER, false>(a, o, s);
}

cudaError_t launch_mc_op(const McArgs& a, const OpDev& o, int model, bool mixed, cudaStream_t s) {
  if (model_nq(model) == 3) return launch_mc_op_t<3, false>(a, o, mixed, s);
  if (a.pc.taper) return launch_mc_op_t<4, true>(a, o, mixed, s);
  return launch_mc_op_t<4, false>(a, o, mixed, s);
}

}  // namespace g6
