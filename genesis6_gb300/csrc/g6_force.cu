// g6_force.cu -- site-site Lennard-Jones + Coulomb under the COM switch.
//
// k_force<Model, LPI, FUSED>: the FP64 (plain) force kernel.  LPI lanes
// cooperate on one i-molecule and walk its neighbour-list row (full list, both
// directions, so no scatter to j and no atomics); each lane keeps FP64 partial
// sums of the i-site forces, the COM-site switch force, the pair energy and
// the 3x3 molecular virial, and the lanes are combined with warp shuffles.
// The epilogue is rigid_collectforce: F = sum of site forces, lab torque = sum
// r_s x f_s; in the fused MD step one warp of the block then runs the FP64
// Gear corrector for the block's molecules.  The mixed-precision kernels are
// in g6_pairs.cu.
//
// The per-pair arithmetic (pair_math) is in g6_pairmath.cuh.
#include <cuda_runtime.h>

#include <cstring>

#include "g6_internal.cuh"
#include "g6_pairmath.cuh"
#include "g6_rigid.cuh"

namespace g6 {

// ---------------------------------------------------------------------------
// k_force: neighbour-list force kernel.
// ---------------------------------------------------------------------------
// Molecules per block of the fused step kernel: the block is MPB x LPI
// threads (128, or 256 at 32 lanes) and one of its warps runs the integrator
// with one molecule per lane.  Small blocks let several blocks share an SM, so one
// block's integrator epilogue overlaps the site loops of the others; at least 8
// molecules per epilogue warp keep the FP64 instruction count low.
template <int LPI>
struct StepShape {
  static constexpr int MPB = (128 / LPI) > 8 ? (128 / LPI) : 8;
  static constexpr int THREADS = MPB * LPI;
};

// HALF (with FUSED = false): the pair kernel of the FP64 step on half rows --
// each pair within rc once, i-side sums as in the force-only form but with
// the virial trace only, the partner's share (minus the pair force, its lab
// torque) added with FP64 atomics to a.jacc64 for k_integrate_fp64.
template <class M, int LPI, bool FUSED, bool HALF = false>
__global__ void __launch_bounds__(FUSED ? StepShape<LPI>::THREADS : 128, 1) k_force(ForceArgs a, StepArgs sa) {
  using R = double;
  constexpr int NW = (FUSED || HALF) ? 1 : 9;
  int step = 0;
  if (a.ctrl) step = a.ctrl[1];
  const bool odd = (step & 1) != 0;
  const double* pk64 = odd ? a.pk64_1 : a.pk64;
  const float4* pk32 = odd ? a.pk32_1 : a.pk32;
  const int gt = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = gt / LPI;
  const int sub = gt % LPI;
  const bool valid = i < a.n;
  const int n = a.n;

  Acc<M, R, NW> acc;
  acc.zero();
  R ri[M::NQ + 1][3];
  int npin = 0;
  if (valid) {
    const int r = a.rep.mol_rep[i];
    double Ld[3], iLd[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) { Ld[k] = a.rep.L[3 * r + k]; iLd[k] = a.rep.invL[3 * r + k]; }
    const double* pi = pk64 + (size_t)i * M::W64;
    double ci[3] = {pi[0], pi[1], pi[2]};
    const int nn = a.nnb[i];
    const int* row = a.nbr + (size_t)i * a.cap;
    {
#pragma unroll
      for (int s = 0; s <= M::NQ; ++s)
#pragma unroll
        for (int k = 0; k < 3; ++k) ri[s][k] = (R)pi[3 + 3 * s + k];
      for (int k = sub; k < nn; k += LPI) {
        const int j = row[k];
        const double* pj = pk64 + (size_t)j * M::W64;
        double cj[3] = {pj[0], pj[1], pj[2]}, o[3], dx[3];
        double dd = exact_dd(ci, cj, Ld, iLd, o, dx);
        if (!(dd < a.cc.rout2)) continue;
        ++npin;
        R rj[M::NQ + 1][3];
#pragma unroll
        for (int s = 0; s <= M::NQ; ++s)
#pragma unroll
          for (int q = 0; q < 3; ++q) rj[s][q] = (R)pj[3 + 3 * s + q];
        R dr[3] = {(R)dx[0], (R)dx[1], (R)dx[2]};
        if constexpr (HALF) {
          PairJ<R> pj;
          pair_math<M, R, NW, true>(dr, (R)dd, ri, rj, a.pc, (R)a.cc.rin2, (R)a.cc.rin, (R)a.cc.rout, (R)a.cc.c1,
                                    (R)a.cc.c2, (R)a.pc.rl, (R)a.pc.ru, (R)a.pc.w3, acc, &pj);
#pragma unroll
          for (int q = 0; q < 3; ++q) {
            atomicAdd(a.jacc64 + (size_t)q * n + j, pj.f[q]);
            atomicAdd(a.jacc64 + (size_t)(3 + q) * n + j, pj.t[q]);
          }
        } else {
          pair_math<M, R, NW>(dr, (R)dd, ri, rj, a.pc, (R)a.cc.rin2, (R)a.cc.rin, (R)a.cc.rout, (R)a.cc.c1,
                              (R)a.cc.c2, (R)a.pc.rl, (R)a.pc.ru, (R)a.pc.w3, acc);
        }
      }
    }
  }
  // rigid_collectforce on the lane partials: F, lab torque, energy, virial
  R fo[3], to[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    R t = acc.fc[k];
#pragma unroll
    for (int q = 0; q <= M::NQ; ++q) t += acc.fs[q][k];
    fo[k] = t;
  }
  {
    R tx = 0, ty = 0, tz = 0;
#pragma unroll
    for (int q = 0; q <= M::NQ; ++q) {
      tx += ri[q][1] * acc.fs[q][2] - ri[q][2] * acc.fs[q][1];
      ty += ri[q][2] * acc.fs[q][0] - ri[q][0] * acc.fs[q][2];
      tz += ri[q][0] * acc.fs[q][1] - ri[q][1] * acc.fs[q][0];
    }
    to[0] = tx; to[1] = ty; to[2] = tz;
  }
  int np_tot = npin;
#pragma unroll
  for (int m = LPI / 2; m >= 1; m >>= 1) np_tot += __shfl_xor_sync(0xffffffffu, np_tot, m);
  if constexpr (HALF) {
    // each pair once: the molecule's own sums in full (energy, virial trace, count)
    double v[8];
#pragma unroll
    for (int k = 0; k < 3; ++k) { v[k] = group_sum<LPI>((double)fo[k]); v[3 + k] = group_sum<LPI>((double)to[k]); }
    v[6] = group_sum<LPI>((double)acc.e);
    v[7] = group_sum<LPI>((double)acc.w[0]);
    if (valid && sub == 0) {
#pragma unroll
      for (int k = 0; k < 3; ++k) { a.F[k * n + i] = v[k]; a.tl[k * n + i] = v[3 + k]; }
      a.emol[i] = v[6];
      a.wmol[i] = v[7];
      a.npair_in[i] = np_tot;
    }
  } else if constexpr (!FUSED) {
    // combine the LPI lanes in FP64
    double v[16];
#pragma unroll
    for (int k = 0; k < 3; ++k) { v[k] = (double)fo[k]; v[3 + k] = (double)to[k]; }
    v[6] = (double)acc.e;
#pragma unroll
    for (int k = 0; k < 9; ++k) v[7 + k] = (double)acc.w[k];
#pragma unroll
    for (int k = 0; k < 16; ++k) v[k] = group_sum<LPI>(v[k]);
    if (valid && sub == 0) {
#pragma unroll
      for (int k = 0; k < 3; ++k) { a.F[k * n + i] = v[k]; a.tl[k * n + i] = v[3 + k]; }
      a.emol[i] = 0.5 * v[6];
#pragma unroll
      for (int k = 0; k < 9; ++k) a.wmol[k * n + i] = 0.5 * v[7 + k];
      if (a.npair_in) a.npair_in[i] = np_tot;
    }
  } else {
    // fused FP64 step: FP64 lane combine, FP64 integrator in warp 0
    constexpr int MPB = StepShape<LPI>::MPB;
    const bool predict_next = step + 1 < sa.ctrl[2];
    double v8[8];
#pragma unroll
    for (int k = 0; k < 3; ++k) { v8[k] = group_sum<LPI>((double)fo[k]); v8[3 + k] = group_sum<LPI>((double)to[k]); }
    v8[6] = group_sum<LPI>((double)acc.e);
    v8[7] = group_sum<LPI>((double)acc.w[0]);
    __shared__ double smd[MPB][9];
    if (sub == 0) {
      const int m = threadIdx.x / LPI;
#pragma unroll
      for (int k = 0; k < 8; ++k) smd[m][k] = v8[k];
      smd[m][8] = (double)np_tot;
    }
    __syncthreads();
    double vv[NRED];
#pragma unroll
    for (int k = 0; k < NRED; ++k) vv[k] = 0.0;
    double dmax2 = 0.0;
    int bad = 0, rr = -1;
    // the integrator warp rotates with the block so that the blocks resident on an
    // SM spread their FP64 work over its four schedulers
    const int ew = blockIdx.x % (StepShape<LPI>::THREADS / 32);
    if ((int)(threadIdx.x >> 5) == ew && (threadIdx.x & 31) < MPB) {
      const int m = threadIdx.x & 31;
      const int im = blockIdx.x * MPB + m;
      if (im < n) {
        rr = a.rep.mol_rep[im];
        const double F[3] = {smd[m][0], smd[m][1], smd[m][2]}, tl[3] = {smd[m][3], smd[m][4], smd[m][5]};
        correct_one(sa, im, sa.p.st, n, im, F, tl, 0.5 * smd[m][6], 0.5 * smd[m][7], 0.5 * smd[m][8], step,
                    predict_next, pose_buf(sa, odd ? 1 : 0), vv, bad);
        if (predict_next) place_next(sa, im, pose_buf(sa, odd ? 0 : 1), dmax2, bad);
      }
    }
    step_reduce<double>(sa, vv, rr, (float)dmax2, bad, MPB, step, ew);
  }
}

template <class M, int LPI, bool FUSED, bool HALF>
static cudaError_t launch_force_t(const ForceArgs& a, const StepArgs& sa, cudaStream_t s) {
  // force only: 128 threads; fused step: MPB molecules (MPB x LPI threads) per block
  const int threads = FUSED ? StepShape<LPI>::THREADS : 128;
  const long long total = (long long)a.n * LPI;
  const int blocks = (int)((total + threads - 1) / threads);
  if (blocks == 0) return cudaSuccess;
  k_force<M, LPI, FUSED, HALF><<<blocks, threads, 0, s>>>(a, sa);
  return cudaGetLastError();
}

template <class M, bool FUSED, bool HALF>
static cudaError_t launch_force_l(const ForceArgs& a, const StepArgs& sa, int lpi, cudaStream_t s) {
  switch (lpi) {
    case 4: return launch_force_t<M, 4, FUSED, HALF>(a, sa, s);
    case 8: return launch_force_t<M, 8, FUSED, HALF>(a, sa, s);
    case 16: return launch_force_t<M, 16, FUSED, HALF>(a, sa, s);
    default: return launch_force_t<M, 32, FUSED, HALF>(a, sa, s);
  }
}

template <bool FUSED, bool HALF = false>
static cudaError_t launch_force_any(const ForceArgs& a, const StepArgs& sa, int model, int lpi, cudaStream_t s) {
  if (model_nq(model) == 3) return launch_force_l<MT<3, false>, FUSED, HALF>(a, sa, lpi, s);
  if (a.pc.taper) return launch_force_l<MT<4, true>, FUSED, HALF>(a, sa, lpi, s);
  return launch_force_l<MT<4, false>, FUSED, HALF>(a, sa, lpi, s);
}

// The FP64 MD step on half rows, second kernel: each molecule's force and lab
// torque (its own pairs' sums minus / plus the shares its partners added to
// jacc64, which are cleared for the next step), then the Gear corrector, the
// next predict and placement and the step's reductions as in the fused step;
// one molecule per lane, 32 per block (an FP64 instruction costs a warp the
// same whatever the number of active lanes).
__global__ void __launch_bounds__(32) k_integrate_fp64(ForceArgs a, StepArgs sa) {
  const int n = a.n;
  const int step = a.ctrl[1];
  const bool odd = (step & 1) != 0;
  const bool predict_next = step + 1 < sa.ctrl[2];
  const int im = blockIdx.x * 32 + threadIdx.x;
  double vv[NRED];
#pragma unroll
  for (int k = 0; k < NRED; ++k) vv[k] = 0.0;
  double dmax2 = 0.0;
  int bad = 0, rr = -1;
  if (im < n) {
    rr = a.rep.mol_rep[im];
    double F[3], tl[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      double* jf = a.jacc64 + (size_t)k * n + im;
      double* jt = a.jacc64 + (size_t)(3 + k) * n + im;
      F[k] = a.F[(size_t)k * n + im] - *jf;
      tl[k] = a.tl[(size_t)k * n + im] + *jt;
      *jf = 0.0;
      *jt = 0.0;
    }
    // the molecule's record in registers: the corrector's read-modify-write
    // chain then waits on no memory round trip (in the fused step it does, but
    // other blocks' pair work hides it)
    double rs[REC];
#pragma unroll
    for (int c = 0; c < REC; ++c) rs[c] = sa.p.st[(size_t)c * n + im];
    correct_one(sa, im, rs, 1, 0, F, tl, a.emol[im], a.wmol[im], (double)a.npair_in[im], step, predict_next,
                pose_buf(sa, odd ? 1 : 0), vv, bad);
#pragma unroll
    for (int c = 0; c < REC; ++c) sa.p.st[(size_t)c * n + im] = rs[c];
    if (predict_next) place_next(sa, im, pose_buf(sa, odd ? 0 : 1), dmax2, bad);
  }
  step_reduce<double>(sa, vv, rr, (float)dmax2, bad, 32, step, 0);
}

// Force only (outputs F, lab torque, per-molecule energy and virial); the
// mixed precision runs the list kernel of g6_pairs.cu.
cudaError_t launch_force(const ForceArgs& a, int model, bool mixed, int lpi, cudaStream_t s) {
  if (mixed) return launch_pairs_force(a, model, lpi, s);
  StepArgs none;
  memset(&none, 0, sizeof none);
  return launch_force_any<false>(a, none, model, lpi, s);
}

// One fused FP64 MD step: force, then the Gear corrector, reductions and the
// next step's predict + placement in the kernel's epilogue.
cudaError_t launch_step_fp64(const ForceArgs& a, const StepArgs& sa, int model, int lpi, cudaStream_t s) {
  return launch_force_any<true>(a, sa, model, lpi, s);
}

cudaError_t launch_step_fp64_half(const ForceArgs& a, const StepArgs& sa, int model, int lpi, cudaStream_t s) {
  cudaError_t e = launch_force_any<false, true>(a, sa, model, lpi, s);
  if (e != cudaSuccess || a.n == 0) return e;
  k_integrate_fp64<<<(a.n + 31) / 32, 32, 0, s>>>(a, sa);
  return cudaGetLastError();
}

int pk64_width(int model) { return model_nq(model) == 3 ? MT<3, false>::W64 : MT<4, false>::W64; }
int pk32_width(int model) { return model_nq(model) == 3 ? MT<3, false>::NPK : MT<4, false>::NPK; }

// ---------------------------------------------------------------------------
// Pair-list kernels for the reference-facing calls g6_force_sites and
// g6_pair_potential: one thread per pair of the caller's compressed list,
// absolute FP64 site positions (site%x of the reference), site forces
// scattered with FP64 atomics (i: +, j: -), per-pair ep, block-reduced virial.
// ---------------------------------------------------------------------------

template <int NQ, bool TAPER>
__global__ void __launch_bounds__(128) k_force_sites(SitesArgs a) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double w[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  if (k < a.npair) {
    const int ns = a.nsite, last = ns - 1;
    const int ii = a.pi[k] * ns, jj = a.pj[k] * ns;
    int st[NQ + 1];   // reference site of the LJ site and of each charged site
#pragma unroll
    for (int s = 0; s <= NQ; ++s) st[s] = a.site[s];
    const double ox = a.ox[k], oy = a.oy[k], oz = a.oz[k];
    const double hh = a.hh[k], dh = a.with_force ? a.dh[k] : 0.0;
    double d[3] = {a.x[ii + last] - a.x[jj + last] - ox, a.y[ii + last] - a.y[jj + last] - oy,
                   a.z[ii + last] - a.z[jj + last] - oz};
    double fi[NQ + 2][3], fj[NQ + 2][3];
#pragma unroll
    for (int s = 0; s < NQ + 2; ++s)
#pragma unroll
      for (int c = 0; c < 3; ++c) fi[s][c] = fj[s][c] = 0.0;
    // LJ site pair
    double vx = a.x[ii + st[0]] - a.x[jj + st[0]] - ox, vy = a.y[ii + st[0]] - a.y[jj + st[0]] - oy,
           vz = a.z[ii + st[0]] - a.z[jj + st[0]] - oz;
    double inv = 1.0 / (vx * vx + vy * vy + vz * vz);
    double d6 = inv * inv * inv, d12 = d6 * d6;
    double elj = a.pc.aa * d12 + a.pc.bb * d6;
    double flj = inv * (a.pc.aa * 12.0 * d12 + a.pc.bb * 6.0 * d6);
    fi[0][0] = fj[0][0] = vx * flj; fi[0][1] = fj[0][1] = vy * flj; fi[0][2] = fj[0][2] = vz * flj;
    double ec = 0;
#pragma unroll
    for (int p = 1; p <= NQ; ++p)
#pragma unroll
      for (int q = 1; q <= NQ; ++q) {
        double x = a.x[ii + st[p]] - a.x[jj + st[q]] - ox, y = a.y[ii + st[p]] - a.y[jj + st[q]] - oy,
               z = a.z[ii + st[p]] - a.z[jj + st[q]] - oz;
        double dd = 1.0 / (x * x + y * y + z * z);
        double ri = sqrt(dd);
        double e0 = a.pc.qq[p - 1][q - 1] * ri;
        double f0 = e0 * dd;
        ec += e0;
        fi[p][0] += x * f0; fi[p][1] += y * f0; fi[p][2] += z * f0;
        fj[q][0] += x * f0; fj[q][1] += y * f0; fj[q][2] += z * f0;
      }
    double scc = hh, dcc = dh;
    if (TAPER) {
      double s12, ds12;
      double d12c = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
      if (d12c < a.pc.ru * a.pc.ru) {
        if (d12c < a.pc.rl * a.pc.rl) { s12 = 0; ds12 = 0; }
        else {
          double r12 = sqrt(d12c);
          s12 = (r12 - a.pc.rl) * (r12 - a.pc.rl) * (3.0 * a.pc.ru - a.pc.rl - 2.0 * r12) / a.pc.w3;
          ds12 = -(6.0 * (r12 - a.pc.rl) * (a.pc.ru - r12) / a.pc.w3) / r12;
        }
      } else { s12 = 1; ds12 = 0; }
      scc = hh * s12;
      dcc = dh * s12 + hh * ds12;
    }
    a.ep[k] = hh * elj + scc * ec;
    if (a.with_force) {
      double fcom = dh * elj + dcc * ec;
      double fp[3] = {0, 0, 0};
#pragma unroll
      for (int s = 0; s < NQ + 1; ++s) {
        double sc = (s == 0) ? hh : scc;
#pragma unroll
        for (int c = 0; c < 3; ++c) { fi[s][c] *= sc; fj[s][c] *= sc; fp[c] += fi[s][c]; }
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) { fi[NQ + 1][c] = fcom * d[c]; fj[NQ + 1][c] = fcom * d[c]; fp[c] += fcom * d[c]; }
      // the COM is the last reference site; the others map through st
#pragma unroll
      for (int s = 0; s < NQ + 2; ++s) {
        int si = (s == NQ + 1) ? last : st[s];
        atomicAdd(&a.fx[ii + si], fi[s][0]); atomicAdd(&a.fy[ii + si], fi[s][1]); atomicAdd(&a.fz[ii + si], fi[s][2]);
        atomicAdd(&a.fx[jj + si], -fj[s][0]); atomicAdd(&a.fy[jj + si], -fj[s][1]); atomicAdd(&a.fz[jj + si], -fj[s][2]);
      }
#pragma unroll
      for (int p = 0; p < 3; ++p)
#pragma unroll
        for (int q = 0; q < 3; ++q) w[3 * p + q] = d[p] * fp[q];
    }
  }
  if (a.with_force) {
    __shared__ double sw[9][4];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int c = 0; c < 9; ++c) {
      double v = w[c];
#pragma unroll
      for (int m = 16; m >= 1; m >>= 1) v += __shfl_xor_sync(0xffffffffu, v, m);
      if (lane == 0) sw[c][warp] = v;
    }
    __syncthreads();
    if (threadIdx.x < 9) {
      double v = 0;
      for (int q = 0; q < (int)(blockDim.x >> 5); ++q) v += sw[threadIdx.x][q];
      atomicAdd(&a.vir[threadIdx.x], v);
    }
  }
}

cudaError_t launch_force_sites(const SitesArgs& a, int model, cudaStream_t s) {
  const int threads = 128;
  const long long blocks = (a.npair + threads - 1) / threads;
  if (blocks == 0) return cudaSuccess;
  if (model_nq(model) == 3) k_force_sites<3, false><<<(unsigned)blocks, threads, 0, s>>>(a);
  else if (a.pc.taper) k_force_sites<4, true><<<(unsigned)blocks, threads, 0, s>>>(a);
  else k_force_sites<4, false><<<(unsigned)blocks, threads, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace g6
