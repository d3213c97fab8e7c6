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

// Component c of qdot(w, q) (RigidModule.F90:1337-1348) from the three
// quaternion components it uses, qo[k] = q[c ^ (k + 1)]: every component is
// sum_k s_ck w_k qo[k] with the signs of qdot (the bits of 0xF5, three per
// component), so the four lanes of a quad run one instruction stream.
__device__ __forceinline__ double qdot64_c(const double w[3], const double qo[3], int c) {
  const int b = 3 * c;
  const double s0 = ((0xF5 >> b) & 1) ? -1.0 : 1.0;
  const double s1 = ((0xF5 >> (b + 1)) & 1) ? -1.0 : 1.0;
  const double s2 = ((0xF5 >> (b + 2)) & 1) ? -1.0 : 1.0;
  return (s0 * w[0]) * qo[0] + (s1 * w[1]) * qo[1] + (s2 * w[2]) * qo[2];
}

// The FP64 MD step on half rows, second kernel: each molecule's force and lab
// torque (its own pairs' sums minus / plus the shares its partners added to
// jacc64, which are cleared for the next step), then the FP64 Gear corrector
// and the next step's predict (the arithmetic of correct_one and predict_one),
// placement and the step's reductions.  Four lanes per molecule, lane c owning
// component c of every vector (x, y, z for c < 3; quaternion component c) and
// the state columns of that component, full vectors by shuffles within the
// quad: an FP64 instruction costs a warp 64 cycles however few lanes are
// active, so the quad's lanes split the corrector's chain (about a quarter of
// the instructions per warp of one molecule per lane) and the 8 molecules of a
// warp share each instruction.  32 molecules per block of 128 threads; the
// placement (place_to) runs on the quad's first lane.
__global__ void __launch_bounds__(128) k_integrate_fp64(ForceArgs a, StepArgs sa) {
  __shared__ double s_vv[32][NRED];
  __shared__ float s_dm[32];
  __shared__ int s_bad[32], s_rr[32];
  const int n = a.n;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, c = lane & 3;
  const int m = warp * 8 + (lane >> 2);
  const int im = blockIdx.x * 32 + m;
  const bool ok = im < n;
  const bool v3 = c < 3;
  const int ii = ok ? im : 0;   // a lane without a molecule computes on molecule 0 and stores nothing
  const int step = a.ctrl[1];
  const bool odd = (step & 1) != 0;
  const bool predict_next = step + 1 < sa.ctrl[2];
  double* st = sa.p.st;
  const int r = sa.p.rep.mol_rep[ii];
  const ThermoDev th = sa.th[r];
  const double dt = sa.dt;
  // the state columns of component c: x[k] = column 3k + c (com, d1..d5),
  // w[k] = 18 + 3k + c (w1..w5), q[k] = 33 + 4k + c (q, q2..q5)
  double x[6], w[5], q[5];
#pragma unroll
  for (int k = 0; k < 6; ++k) x[k] = v3 ? st[(size_t)(3 * k + c) * n + ii] : 0.0;
#pragma unroll
  for (int k = 0; k < 5; ++k) w[k] = v3 ? st[(size_t)(18 + 3 * k + c) * n + ii] : 0.0;
#pragma unroll
  for (int k = 0; k < 5; ++k) q[k] = st[(size_t)(33 + 4 * k + c) * n + ii];
  double Fc = 0.0, tlc = 0.0;
  if (v3 && ok) {
    double* jf = a.jacc64 + (size_t)c * n + im;
    double* jt = a.jacc64 + (size_t)(3 + c) * n + im;
    Fc = a.F[(size_t)c * n + im] - *jf;
    tlc = a.tl[(size_t)c * n + im] + *jt;
    *jf = 0.0;
    *jt = 0.0;
  }
  // body torque component c: column c of the rotation against the lab torque
  const PoseBuf cur = pose_buf(sa, odd ? 1 : 0);
  const double tl0 = qsh(tlc, 0), tl1 = qsh(tlc, 1), tl2 = qsh(tlc, 2);
  double tauc = 0.0;
  if (v3)
    tauc = cur.tmat[(size_t)c * n + ii] * tl0 + cur.tmat[(size_t)(3 + c) * n + ii] * tl1 +
           cur.tmat[(size_t)(6 + c) * n + ii] * tl2;
  int bd = (v3 && ok && !(isfinite(Fc) && isfinite(tauc))) ? 1 : 0;
  double ext_t = 0.0, ext_r = 0.0;
  if (th.kind == G6_NOSE) {
    const double nc = th.z[0] * dt;
    ext_t = nc * 0.5;
    ext_r = nc;
  }
  const double massi = 1.0 / sa.mass;
  // COM: Gear-5
  if (v3) {
    double nf = Fc * (dt * dt * 0.5 * massi);
    nf = nf - x[1] * ext_t;
    const double delta = nf - x[2];
    x[0] = x[0] + G50 * delta;
    x[1] = x[1] + G51 * delta;
    x[2] = nf;
    x[3] = x[3] + G53 * delta;
    x[4] = x[4] + G54 * delta;
    x[5] = x[5] + G55 * delta;
  }
  // quaternion value, from the angular velocity before its correction
  const double w1v[3] = {qsh(w[0], 0), qsh(w[0], 1), qsh(w[0], 2)};
  {
    const double qo[3] = {qsh(q[0], c ^ 1), qsh(q[0], c ^ 2), qsh(q[0], c ^ 3)};
    const double dw = qdot64_c(w1v, qo, c) * dt * 0.5 - q[1];
    q[0] = q[0] + G40 * dw;
  }
  // angular velocity: Gear-4 with Euler's equations (axis c, cyclic c1, c2)
  if (v3) {
    const int c1 = c == 2 ? 0 : c + 1, c2 = c == 0 ? 2 : c - 1;
    const double Ic = c == 0 ? sa.I[0] : (c == 1 ? sa.I[1] : sa.I[2]);
    const double I1 = c1 == 0 ? sa.I[0] : (c1 == 1 ? sa.I[1] : sa.I[2]);
    const double I2 = c2 == 0 ? sa.I[0] : (c2 == 1 ? sa.I[1] : sa.I[2]);
    const double wa = c1 == 0 ? w1v[0] : (c1 == 1 ? w1v[1] : w1v[2]);
    const double wb = c2 == 0 ? w1v[0] : (c2 == 1 ? w1v[1] : w1v[2]);
    double nf = (tauc + (I1 - I2) * wa * wb) * dt * (1.0 / Ic);
    nf = nf - w[0] * ext_r;
    const double delta = nf - w[1];
    w[0] = w[0] + G40 * delta;
    w[1] = nf;
    w[2] = w[2] + G42 * delta;
    w[3] = w[3] + G43 * delta;
    w[4] = w[4] + G44 * delta;
  }
  // stochastic collisions: every lane of the quad draws the same numbers
  if (th.kind == G6_ANDERSEN) {
    double u[2];
    const uint32_t sc = (uint32_t)(sa.ctrl[6] + step);
    uniform2(sa.seed, (uint32_t)im, sc, 0x41u, 0u, u);
    if (u[0] <= th.rate * dt) {
      const double kT = th.temp * RGAS * J2I;
      double z[6];
      for (int p = 0; p < 3; ++p) {
        double g[2];
        uniform2(sa.seed, (uint32_t)im, sc, 0x41u, (uint32_t)(p + 1), g);
        z[2 * p] = normal_pair(g[0], g[1], z[2 * p + 1]);
      }
      const double sv = sqrt(kT * massi) * dt;
      if (v3) {
        const double Ic = c == 0 ? sa.I[0] : (c == 1 ? sa.I[1] : sa.I[2]);
        x[1] = (c == 0 ? z[0] : (c == 1 ? z[1] : z[2])) * sv;
        w[0] = (c == 0 ? z[3] : (c == 1 ? z[4] : z[5])) * sqrt(kT / Ic);
      }
    }
  }
  // quaternion derivative stacks from the corrected angular-velocity stack
  double W[4][3];
#pragma unroll
  for (int k = 0; k < 4; ++k)
#pragma unroll
    for (int j = 0; j < 3; ++j) W[k][j] = qsh(w[k], j);
  double a0[3], a1[3], a2[3], a3[3];
  a0[0] = qsh(q[0], c ^ 1); a0[1] = qsh(q[0], c ^ 2); a0[2] = qsh(q[0], c ^ 3);
  q[1] = qdot64_c(W[0], a0, c) * dt * 0.5;
  a1[0] = qsh(q[1], c ^ 1); a1[1] = qsh(q[1], c ^ 2); a1[2] = qsh(q[1], c ^ 3);
  q[2] = (qdot64_c(W[1], a0, c) + qdot64_c(W[0], a1, c)) * dt * 0.25;
  a2[0] = qsh(q[2], c ^ 1); a2[1] = qsh(q[2], c ^ 2); a2[2] = qsh(q[2], c ^ 3);
  q[3] = (qdot64_c(W[2], a0, c) + qdot64_c(W[0], a2, c) + qdot64_c(W[1], a1, c)) * dt * (1.0 / 6.0);
  a3[0] = qsh(q[3], c ^ 1); a3[1] = qsh(q[3], c ^ 2); a3[2] = qsh(q[3], c ^ 3);
  q[4] = (qdot64_c(W[3], a0, c) + qdot64_c(W[2], a1, c) + qdot64_c(W[1], a2, c) + qdot64_c(W[0], a3, c)) * dt *
         (1.0 / 8.0);
  // reductions: kinetic sums (Rigid_Ek) over the quad
  const double ekt = quad_sum(v3 ? x[1] * x[1] : 0.0);
  const double Icw = v3 ? (c == 0 ? sa.I[0] : (c == 1 ? sa.I[1] : sa.I[2])) : 0.0;
  const double ekr = quad_sum(Icw * (W[0][c == 3 ? 0 : c] * W[0][c == 3 ? 0 : c]));
  // the next step's predict (predict_one)
  if (predict_next) {
    if (v3) {
      const double d1 = x[1], d2 = x[2], d3 = x[3], d4 = x[4], d5 = x[5];
      x[0] = x[0] + d1 + d2 + d3 + d4 + d5;
      x[1] = d1 + 2.0 * d2 + 3.0 * d3 + 4.0 * d4 + 5.0 * d5;
      x[2] = d2 + 3.0 * d3 + 6.0 * d4 + 10.0 * d5;
      x[3] = d3 + 4.0 * d4 + 10.0 * d5;
      x[4] = d4 + 5.0 * d5;
      const double w1 = w[0], w2 = w[1], w3 = w[2], w4 = w[3], w5 = w[4];
      w[0] = w1 + w2 + w3 + w4 + w5;
      w[1] = w2 + 2.0 * w3 + 3.0 * w4 + 4.0 * w5;
      w[2] = w3 + 3.0 * w4 + 6.0 * w5;
      w[3] = w4 + 4.0 * w5;
    }
    const double qs = q[0] + q[1] + q[2] + q[3] + q[4];
    q[1] = q[1] + 2.0 * q[2] + 3.0 * q[3] + 4.0 * q[4];
    const double re = 1.0 / sqrt(quad_sum(qs * qs));
    q[0] = qs * re;
  }
  if (ok) {
    if (v3) {
#pragma unroll
      for (int k = 0; k < 6; ++k) st[(size_t)(3 * k + c) * n + im] = x[k];
#pragma unroll
      for (int k = 0; k < 5; ++k) st[(size_t)(18 + 3 * k + c) * n + im] = w[k];
    }
#pragma unroll
    for (int k = 0; k < 5; ++k) st[(size_t)(33 + 4 * k + c) * n + im] = q[k];
  }
  bd = quad_sum(bd);
  __syncwarp();   // the quad's columns are written before its first lane places the molecule
  if (c == 0) {
    double dmax2 = 0.0;
    int bad = bd ? 1 : 0;
    if (ok && predict_next) place_next(sa, im, pose_buf(sa, odd ? 0 : 1), dmax2, bad);
    s_vv[m][0] = ok ? a.emol[im] : 0.0;
    s_vv[m][1] = ok ? a.wmol[im] : 0.0;
    s_vv[m][2] = ok ? ekt : 0.0;
    s_vv[m][3] = ok ? ekr : 0.0;
    s_vv[m][4] = ok ? (double)a.npair_in[im] : 0.0;
    s_dm[m] = (float)dmax2;
    s_bad[m] = ok ? bad : 0;
    s_rr[m] = ok ? r : -1;
  }
  __syncthreads();
  double vv[NRED];
  float dm = 0.0f;
  int bdd = 0, rr = -1;
#pragma unroll
  for (int k = 0; k < NRED; ++k) vv[k] = 0.0;
  if (warp == 0) {
#pragma unroll
    for (int k = 0; k < NRED; ++k) vv[k] = s_vv[lane][k];
    dm = s_dm[lane]; bdd = s_bad[lane]; rr = s_rr[lane];
  }
  step_reduce<double>(sa, vv, rr, dm, bdd, 32, step, 0);
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
  k_integrate_fp64<<<(a.n + 31) / 32, 128, 0, s>>>(a, sa);
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
