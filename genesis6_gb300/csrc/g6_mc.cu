// g6_mc.cu -- single-molecule Monte Carlo on the device (mc2.F90:544-832).
//
// One CTA advances one chain (= one replica of the context) through ntrial
// sequential trials.  Per trial:
//   warp 0   reads the trial's draws (target, Gaussian rotation vector and
//            translation: the sine branch of Random_Normal, RandomModule.F90:20-28)
//            from a shared-memory batch that all threads fill in parallel once
//            per MC_NB trials, scales them by the widths, and builds the new
//            quaternion with qinfrotator + qadd (QuatModule.F90:108-133, 203-223)
//            and the new site offsets (rigid_setsiteposition) -- normally one
//            trial ahead, while the previous trial's energies are summed, and
//            again here only when the previous acceptance made that pose stale;
//   others   sum e(new, j) - e(old, j) over every other molecule j of the chain
//            with the PairPotential arithmetic (strict rc test, COM switch, ST2
//            Coulomb taper on the custom path), one molecule j per thread;
//   warp 0   Metropolis test (mc2.F90:712-722) as log(u) < -dE*I2J*J2K*beta
//            (+ the Hastings term), and on acceptance writes the new pose.
// Unlike mc2 (which subtracts stored pair energies of the neighbours of the
// new pose only and adapts the step width after every trial), dE runs over all
// neighbours of both poses and the widths are fixed, so the Markov chain is
// exactly Metropolis-Hastings for the chosen widths.  The draws come from the
// same Philox stream as the oracle (counter = chain, trial, draw), so short
// FP64 chains replay the CPU chain trial by trial.
//
// Mixed precision: the trial pose and the pair energies are FP32; the FP64
// state (COM, quaternion, FP64 offsets) is rebuilt from the FP64 draws only
// when a trial is accepted, and the FP32 offsets the trial used are the ones
// stored in the packed pose, so later trials see exactly the pose whose energy
// was accepted.
//
// Learned widths (G6_MC_LEARNED): the proposal widths come from a 24-64-64-2
// MLP on local-environment features.  The features of every molecule at its
// current pose are kept in an integer cache (exact sums, see g6_mlp.cuh): the
// widths at the old pose come from the cache.  The energy warps, which test
// every molecule against both poses anyway, keep the molecules within 6 A of
// either pose, add the target's terms of the new-pose ones into its new
// features and prepare each neighbour's own terms of the pair; they then
// signal warp 0 (named barrier 1), which runs the network on the new features
// while they sum the pair energies.  An accepted move writes the moved
// molecule's new features and adds the prepared terms to its neighbours'
// rows.  The Hastings ratio uses the widths of both poses.  G6_MC_COLLECT runs
// the fixed widths and writes one training record per trial.
#include <cuda_runtime.h>

#include <type_traits>

#include "g6_internal.cuh"
#include "g6_mctrial.cuh"
#include "g6_mlp.cuh"

namespace g6 {

// Features of every molecule of the chain at its current pose (integer cache).
template <int NQ, bool MIXED>
__device__ __noinline__ void init_features(const McArgs& a, int i0, int i1, const float fs[3], const double L[3],
                              const double iL[3], int* fcl) {
  using P = PoseRead<NQ, MIXED>;
  for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
    float o[(NQ + 1) * 3], u[4][3];
    P::offsets(a, i, o);
    site_dirs<NQ>(o, u);
#pragma unroll
    for (int s = 0; s < 4; ++s)
#pragma unroll
      for (int k = 0; k < 3; ++k) a.udir[(size_t)i * 12 + 3 * s + k] = u[s][k];
    int f[MLP_IN];
#pragma unroll
    for (int k = 0; k < MLP_IN; ++k) f[k] = 0;
    uint32_t fi[3];
    double ci[3];
    if (MIXED) P::fix(a, i, fi); else P::com(a, i, ci);
    for (int j = i0; j < i1; ++j) {
      if (j == i) continue;
      float e[3], r2;
      if (MIXED) { uint32_t fj[3]; P::fix(a, j, fj); r2 = fvec_fix(fi, fj, fs, e); }
      else { double cj[3]; P::com(a, j, cj); r2 = fvec_64(ci, cj, L, iL, e); }
      if (r2 < FEAT_RC2 && r2 > 0.0f) feat_terms(e, r2, u, 1, f);
    }
#pragma unroll
    for (int k = 0; k < MLP_IN; ++k) fcl[(size_t)(i - i0) * MLP_IN + k] = f[k];
  }
}

// The proposal-width network in shared memory, transposed for conflict-free
// reads (lane o reads column o).
struct MlpShared {
  float2 w1p[MLP_IN][MLP_H / 2];   // lane l holds outputs 2l, 2l+1: w1p[k][l] = (W1[2l][k], W1[2l+1][k])
  float2 b1p[MLP_H / 2];
  float2 w2p[MLP_H][MLP_H / 2];
  float2 b2p[MLP_H / 2];
  float2 w3p[MLP_OUT][MLP_H / 2];
  float b3[MLP_OUT];
  float mean[MLP_IN], istd[MLP_IN];
  float4 x[2][MLP_IN / 4];   // per-warp scratch (warps 0 and 1 evaluate the network concurrently)
  float4 h[2][MLP_H / 4];
  float s0t, s0r;            // reference widths sigma0
  double s0t_d, s0r_d;
};

__device__ void mlp_load(MlpShared& m, const MlpDev& d) {
  for (int p = threadIdx.x; p < MLP_H * MLP_IN; p += blockDim.x) {
    const int o = p / MLP_IN, k = p % MLP_IN;
    float* w = reinterpret_cast<float*>(&m.w1p[k][o >> 1]);
    w[o & 1] = d.w[MLP_W1 + p];
  }
  for (int p = threadIdx.x; p < MLP_H * MLP_H; p += blockDim.x) {
    const int o = p / MLP_H, k = p % MLP_H;
    float* w = reinterpret_cast<float*>(&m.w2p[k][o >> 1]);
    w[o & 1] = d.w[MLP_W2 + p];
  }
  for (int p = threadIdx.x; p < MLP_H; p += blockDim.x) {
    reinterpret_cast<float*>(m.b1p)[p] = d.w[MLP_B1 + p];
    reinterpret_cast<float*>(m.b2p)[p] = d.w[MLP_B2 + p];
    reinterpret_cast<float*>(m.w3p[0])[p] = d.w[MLP_W3 + p];
    reinterpret_cast<float*>(m.w3p[1])[p] = d.w[MLP_W3 + MLP_H + p];
  }
  if (threadIdx.x < MLP_OUT) m.b3[threadIdx.x] = d.w[MLP_B3 + threadIdx.x];
  if (threadIdx.x < MLP_IN) { m.mean[threadIdx.x] = d.feat_mean[threadIdx.x]; m.istd[threadIdx.x] = d.feat_inv_std[threadIdx.x]; }
  if (threadIdx.x == 0) { m.s0t = (float)d.sigma0_t; m.s0r = (float)d.sigma0_r; m.s0t_d = d.sigma0_t; m.s0r_d = d.sigma0_r; }
}

// Widths from integer features feat[] (one whole warp; lane 0's result is the
// one used).  w selects the warp's scratch rows.  R: the pose precision.  Lane
// l computes hidden units 2l and 2l+1 with one 8-byte weight load per input
// and four independent partial sums per unit; inputs are read four at a time.
// Not inlined (nor are build_trial and init_features): one copy of the code
// serves every call site, which keeps the kernel's instruction footprint small
// (about 7% faster per trial than inlined copies).
// tanh of a hidden unit: the single-instruction approximation (PTX
// tanh.approx.f32) for mixed-precision chains, tanhf for the FP64 chains that
// replay the FP64 reference.
template <class R>
__device__ __forceinline__ float mlp_tanh(float x) {
  if constexpr (sizeof(R) == 4) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
  } else {
    return tanhf(x);
  }
}

template <class R>
__device__ __noinline__ void mlp_widths_warp(MlpShared& m, int w, const int* feat, R& st, R& sr) {
  const int lane = threadIdx.x & 31;
  float* xs = reinterpret_cast<float*>(m.x[w]);
  if (lane < MLP_IN) xs[lane] = ((float)feat[lane] * FEAT_IQ - m.mean[lane]) * m.istd[lane];
  __syncwarp();
  float a0[4] = {0.0f, 0.0f, 0.0f, 0.0f}, a1[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
  for (int k4 = 0; k4 < MLP_IN / 4; ++k4) {
    const float4 x = m.x[w][k4];
    const float xv[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const float2 wt = m.w1p[4 * k4 + u][lane];
      a0[u] = fmaf(wt.x, xv[u], a0[u]);
      a1[u] = fmaf(wt.y, xv[u], a1[u]);
    }
  }
  const float2 b1 = m.b1p[lane];
  const float h1a = mlp_tanh<R>(b1.x + ((a0[0] + a0[1]) + (a0[2] + a0[3])));
  const float h1b = mlp_tanh<R>(b1.y + ((a1[0] + a1[1]) + (a1[2] + a1[3])));
  reinterpret_cast<float2*>(m.h[w])[lane] = make_float2(h1a, h1b);
  __syncwarp();
#pragma unroll
  for (int u = 0; u < 4; ++u) { a0[u] = 0.0f; a1[u] = 0.0f; }
#pragma unroll
  for (int k4 = 0; k4 < MLP_H / 4; ++k4) {
    const float4 x = m.h[w][k4];
    const float xv[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const float2 wt = m.w2p[4 * k4 + u][lane];
      a0[u] = fmaf(wt.x, xv[u], a0[u]);
      a1[u] = fmaf(wt.y, xv[u], a1[u]);
    }
  }
  const float2 b2 = m.b2p[lane];
  const float h2a = mlp_tanh<R>(b2.x + ((a0[0] + a0[1]) + (a0[2] + a0[3])));
  const float h2b = mlp_tanh<R>(b2.y + ((a1[0] + a1[1]) + (a1[2] + a1[3])));
  float z[MLP_OUT];
#pragma unroll
  for (int q = 0; q < MLP_OUT; ++q) {
    const float2 w3 = m.w3p[q][lane];
    float s = w3.x * h2a + w3.y * h2b;
#pragma unroll
    for (int mm = 16; mm >= 1; mm >>= 1) s += __shfl_xor_sync(0xffffffffu, s, mm);
    z[q] = __shfl_sync(0xffffffffu, s, 0) + m.b3[q];   // lane 0's sum on every lane
  }
  __syncwarp();
  if constexpr (sizeof(R) == 4) {
    st = m.s0t * ((float)MLP_SMIN + (float)MLP_SSPAN * mlp_sigmoid(z[0]));
    sr = m.s0r * ((float)MLP_SMIN + (float)MLP_SSPAN * mlp_sigmoid(z[1]));
  } else {
    st = m.s0t_d * (MLP_SMIN + MLP_SSPAN * (double)mlp_sigmoid(z[0]));
    sr = m.s0r_d * (MLP_SMIN + MLP_SSPAN * (double)mlp_sigmoid(z[1]));
  }
}

// Control warps of a chain's CTA (they build poses and run the network; the
// others are energy warps).
__host__ __device__ constexpr int mc_ctrl_warps(int mode) { return mode == G6_MC_LEARNED ? 2 : 1; }

template <int NQ, bool TAPER, bool MIXED, int MODE>
__global__ void __launch_bounds__(MC_NT) k_mc(McArgs a) {
  using R = typename std::conditional<MIXED, float, double>::type;
  using P = PoseRead<NQ, MIXED>;
  using TP = TrialPose<R, NQ>;
  constexpr bool FEAT = MODE != G6_MC_PLAIN;
  constexpr bool LEARN = MODE == G6_MC_LEARNED;
  // the FP64 quaternion an acceptance writes is prepared with the pose
  constexpr bool Q64 = MIXED;
  // control warps build the next trial's pose (and, with learned widths, run
  // the network) while the others sum energies
  constexpr int NCTRL = mc_ctrl_warps(MODE);
  constexpr int E0 = 32 * NCTRL, NE = MC_NT - E0, NEW = NE / 32;
  constexpr int W64 = P::W64, NPK = P::NPK;
  __shared__ typename std::conditional<MIXED, float, double>::type s_lu[MC_NB];   // log of the test uniform
  __shared__ R s_g[6][MC_NB];   // unit normals of the rotation (0-2) and translation (3-5)
  __shared__ int s_tg[MC_NB];
  __shared__ TP s_pose[2];
  __shared__ int s_feat[MLP_IN];   // the target's features at the trial pose
  __shared__ R s_part[NEW];
  __shared__ int s_seg[NEW][MC_SEG];   // each energy warp's molecules within rc of either pose
  __shared__ int s_pool;   // feature neighbours kept so far: new pose (low 16 bits), old pose (high 16 bits)
  __shared__ int s_accept, s_hit;
  __shared__ QForm s_qf_new;   // proposal density form of the learned widths at the trial pose
  __shared__ typename std::conditional<LEARN, MlpShared, int>::type s_mlp;

  const int c = blockIdx.x;
  const int i0 = a.rep.off[c], i1 = a.rep.off[c + 1], nc = i1 - i0;
  const int n = a.n;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double L[3], iL[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) { L[k] = a.rep.L[3 * c + k]; iL[k] = a.rep.invL[3 * c + k]; }
  const float fs[3] = {a.rep.fscale[3 * c], a.rep.fscale[3 * c + 1], a.rep.fscale[3 * c + 2]};
  const double beta = a.beta[c];
  const float fbeta_e = (float)(I2J * J2K * beta);   // mixed test: x = -dE * fbeta_e + log Hastings
  // fixed widths enter as sqrt(sigma^2), the variance form of mc2's Random_Normal call
  const R sig_t_fixed = (R)sqrt(a.sigma_t[c] * a.sigma_t[c]);
  const R sig_r_fixed = (R)sqrt(a.sigma_r[c] * a.sigma_r[c]);
  const float fsi[3] = {(float)(4294967296.0 * iL[0]), (float)(4294967296.0 * iL[1]), (float)(4294967296.0 * iL[2])};
  if constexpr (LEARN) mlp_load(s_mlp, a.mlp);
  // dynamic shared memory: the chain's feature cache when it fits (else its rows
  // of a.fcache), then the feature neighbours of the new pose and of the old pose
  // (MC_POOL entries each)
  extern __shared__ __align__(16) int s_dyn[];
  int* const fcl = a.fc_smem ? s_dyn : a.fcache + (size_t)i0 * MLP_IN;
  FeEntry* const pool_new = reinterpret_cast<FeEntry*>(s_dyn + (a.fc_smem ? (size_t)a.ncmax * MLP_IN : 0));
  FeEntry* const pool_old = pool_new + MC_POOL;
  if constexpr (FEAT) init_features<NQ, MIXED>(a, i0, i1, fs, L, iL, fcl);
  if (threadIdx.x == 0) { s_pose[0].trial = -1; s_pose[1].trial = -1; }
  __syncthreads();

  const R rin2 = MIXED ? (R)a.cc.frin2 : (R)a.cc.rin2, rin = MIXED ? (R)a.cc.frin : (R)a.cc.rin;
  const R rout = MIXED ? (R)a.cc.frout : (R)a.cc.rout, c1 = MIXED ? (R)a.cc.fc1 : (R)a.cc.c1;
  double energy = a.energy[c];
  long long nacc = 0;
  int nsample = 0;

  for (int t = 0; t < a.ntrial; ++t) {
    const int tb = t % MC_NB;
    if (tb == 0) {   // draws of the next MC_NB trials, one trial per thread
      __syncthreads();
      const int tt = t + (int)threadIdx.x;
      if (threadIdx.x < MC_NB && tt < a.ntrial) {
        const uint64_t trial = a.counter + (uint64_t)tt;
        const uint32_t lo = (uint32_t)trial, hi = (uint32_t)(trial >> 32);
        double u[2];
        uniform2(a.seed, (uint32_t)c, lo, hi, 0u, u);
        int tg = (int)(u[0] * nc);
        if (tg >= nc) tg = nc - 1;   // u = 1 would select nc (mc2.F90:551 quirk)
        s_tg[threadIdx.x] = tg;
        // Box-Muller normals (sine branch): FP32 functions for the FP32 trial poses
        // of mixed precision (FP64 transcendentals cost tens of 64-cycle FP64
        // instructions each), FP64 in the FP64 mode that replays the oracle
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
    TP& cur = s_pose[t & 1];
    const bool next_in_batch = tb + 1 < MC_NB && t + 1 < a.ntrial;
    const int tg1 = next_in_batch ? i0 + s_tg[tb + 1] : -1;   // the next trial's target
    if (FEAT && threadIdx.x == 0) { s_hit = 0; s_pool = 0; }
    if (FEAT && threadIdx.x < MLP_IN) s_feat[threadIdx.x] = 0;
    // ---- warp 0: the trial pose, unless it was built during the previous trial ----
    if (warp == 0 && cur.trial != t) {
      R st_w = sig_t_fixed, sr_w = sig_r_fixed;
      if constexpr (LEARN) mlp_widths_warp<R>(s_mlp, 0, fcl + (size_t)(tg - i0) * MLP_IN, st_w, sr_w);
      build_trial<R, NQ, MIXED, Q64>(a, cur, t, tg, s_g, tb, st_w, sr_w, iL, fsi);
    }
    __syncthreads();
    if ((int)threadIdx.x >= E0) {
      // ---- energy warps: dE over every other molecule of the chain ----
      R acc = R(0);
      R ro[NQ + 1][3], rn[NQ + 1][3];
#pragma unroll
      for (int s = 0; s <= NQ; ++s)
#pragma unroll
        for (int k = 0; k < 3; ++k) { ro[s][k] = cur.oo[s][k]; rn[s][k] = cur.on[s][k]; }
      const uint32_t fo[3] = {cur.fo[0], cur.fo[1], cur.fo[2]}, fn[3] = {cur.fn[0], cur.fn[1], cur.fn[2]};
      const double co[3] = {cur.co[0], cur.co[1], cur.co[2]}, cn[3] = {cur.cn[0], cur.cn[1], cur.cn[2]};
      // separation of molecule j from both poses (j -> pose) and the strict rc tests
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
          if (bandO || bandN) {   // borderline: the reference's FP64 test
            double cj[3], o[3], dx[3];
            P::com(a, j, cj);
            if (bandO) inO = exact_dd(co, cj, L, iL, o, dx) < a.cc.rout2;
            if (bandN) inN = exact_dd(cn, cj, L, iL, o, dx) < a.cc.rout2;
          }
        } else {
          double cj[3], o[3], dx[3];
          P::com(a, j, cj);
          const double d0 = exact_dd(co, cj, L, iL, o, dx);
          dO[0] = dx[0]; dO[1] = dx[1]; dO[2] = dx[2];
          ddO = (R)d0;
          inO = d0 < a.cc.rout2;
          const double d1 = exact_dd(cn, cj, L, iL, o, dx);
          dN[0] = dx[0]; dN[1] = dx[1]; dN[2] = dx[2];
          ddN = (R)d1;
          inN = d1 < a.cc.rout2;
        }
      };
      // e(new, j) - e(old, j)
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
      const int ew = warp - NCTRL;
      // a feature neighbour kept in slot pos: its separation and, asynchronously,
      // its site directions
      auto keep = [&](FeEntry* base, int pos, int j, const float (&e)[3]) {
        FeEntry& E = base[pos];
        E.j = j;
        E.e[0] = e[0]; E.e[1] = e[1]; E.e[2] = e[2];
        const unsigned dst = (unsigned)__cvta_generic_to_shared(E.u);
        const float* src = a.udir + (size_t)j * 12;
        asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
        asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" ::"r"(dst + 16), "l"(src + 4) : "memory");
        asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" ::"r"(dst + 32), "l"(src + 8) : "memory");
      };
      // Pass 1: the rc tests for this warp's molecules, the ones within rc of
      // either pose appended (ballot order) to the warp's segment, so that the
      // pair energies below run with full lanes instead of one site-loop pass
      // per 32 molecules with a few lanes each.  Entries beyond the segment's
      // capacity are summed at once.  Both passes run in a fixed order.  With
      // features, the molecules within 6 A of either pose are kept as well.
      int* seg = s_seg[ew];
      int nseg = 0;
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
        if constexpr (FEAT) {
          // the same separations as float: bitwise those of the cache's own
          // evaluation (fvec_fix / fvec_64), tested with the exactly rounded |e|^2
          const float eo[3] = {(float)dO[0], (float)dO[1], (float)dO[2]};
          const float en[3] = {(float)dN[0], (float)dN[1], (float)dN[2]};
          bool qo = false, qn = false;
          if (valid) {
            const float r2o = dot3_rn(eo, eo), r2n = dot3_rn(en, en);
            qo = r2o < FEAT_RC2 && r2o > 0.0f;
            qn = r2n < FEAT_RC2 && r2n > 0.0f;
          }
          const unsigned mo = __ballot_sync(0xffffffffu, qo), mn = __ballot_sync(0xffffffffu, qn);
          const unsigned lt = (1u << lane) - 1u;
          if ((qo || qn) && j == tg1) s_hit = 1;
          if (mn | mo) {   // slots in both pools from one shared atomic per chunk
            int b = 0;
            if (lane == 0) b = atomicAdd(&s_pool, __popc(mn) + (__popc(mo) << 16));
            b = __shfl_sync(0xffffffffu, b, 0);
            const int bn = (b & 0xffff) + __popc(mn & lt), bo = (b >> 16) + __popc(mo & lt);
            if (qn) {
              if (bn < MC_POOL) keep(pool_new, bn, j, en); else *a.flag = 1;
            }
            if (qo) {
              if (bo < MC_POOL) keep(pool_old, bo, j, eo); else *a.flag = 1;
            }
          }
        }
      }
      if constexpr (FEAT) {
        asm volatile("cp.async.wait_all;" ::: "memory");
        // every energy warp's entries are complete (named barrier 2, energy warps only)
        asm volatile("bar.sync 2, %0;" ::"n"(NE) : "memory");
        const int nn = min(s_pool & 0xffff, MC_POOL), no = min(s_pool >> 16, MC_POOL);
        // The terms of the kept pairs, one kind of term per warp and one pair per
        // lane (no divergence): for the new pose the radial shells (the same for
        // both molecules of a pair: into the target's features and the
        // neighbour's entry), the target's direction terms and the neighbour's;
        // for the old pose the neighbour's radial and direction terms.
        const int bn = (nn + 31) >> 5, bo = (no + 31) >> 5;
        auto task = [&](int wt) {
          const bool nw = wt < 6 * bn;
          const int kind = nw ? wt / bn : 6 + (wt - 6 * bn) / bo;
          const int q = 32 * (nw ? wt % bn : (wt - 6 * bn) % bo) + lane;
          const bool ok = q < (nw ? nn : no);
          FeEntry& E = nw ? pool_new[ok ? q : 0] : pool_old[ok ? q : 0];
          float e[3] = {E.e[0], E.e[1], E.e[2]};
          const bool tgt = kind == 2 || kind == 3;   // the target's terms: e from the target's side
          if (tgt) { e[0] = -e[0]; e[1] = -e[1]; e[2] = -e[2]; }
          const int part = kind < 6 ? (kind < 2 ? kind : (kind < 4 ? kind : kind - 2)) : kind - 6;
          int v[8];
          feat_part(part, e, dot3_rn(e, e), tgt ? &cur.un[0][0] : E.u, v);
          const int nv = part < 2 ? 8 : 4;
          if (ok && kind != 2 && kind != 3) {
#pragma unroll
            for (int k = 0; k < 8; ++k)
              if (k < nv) E.d[part_index(part, k)] = v[k];
          }
          if (kind < 4) {   // into the target's features: a warp sum per feature
            int mine = 0;
#pragma unroll
            for (int k = 0; k < 8; ++k) {
              const int sum = __reduce_add_sync(0xffffffffu, ok ? v[k] : 0);
              if (lane == k) mine = sum;
            }
            if (lane < nv && mine != 0) atomicAdd(s_feat + part_index(part, lane), mine);
          }
        };
        // the target's terms (kinds 0-3) first, on the warps with the fewest
        // molecules in pass 1; each warp signals warp 0 once its share of them is
        // done, and then takes its neighbours' terms
        int wt = NEW - 1 - ew;
        for (; wt < 4 * bn; wt += NEW) task(wt);
        // the target's new features are complete once every energy warp has arrived
        if constexpr (LEARN) asm volatile("bar.arrive 1, %0;" ::"n"(32 + NE) : "memory");
        for (; wt < 6 * bn + 4 * bo; wt += NEW) task(wt);
      }
      __syncwarp();
      // Pass 2: the segment, one molecule per lane
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
      if (lane == 0) s_part[warp - NCTRL] = acc;
    } else if (warp == 0) {
      if constexpr (LEARN) {
        // ---- warp 0: widths at the trial pose from the energy warps' features ----
        asm volatile("bar.sync 1, %0;" ::"n"(32 + NE) : "memory");
        R st2, sr2;
        mlp_widths_warp<R>(s_mlp, 0, s_feat, st2, sr2);
        if (lane == 0) s_qf_new = q_form((float)st2, (float)sr2);
      } else if (next_in_batch) {   // the next trial's pose (fixed widths)
        build_trial<R, NQ, MIXED, Q64>(a, s_pose[(t + 1) & 1], t + 1, tg1, s_g, tb + 1, sig_t_fixed, sig_r_fixed, iL,
                                       fsi);
      }
    } else if constexpr (LEARN) {
      // ---- warp 1: widths of the next trial's target at its current pose, and its trial pose ----
      if (next_in_batch) {
        R st1, sr1;
        mlp_widths_warp<R>(s_mlp, 1, fcl + (size_t)(tg1 - i0) * MLP_IN, st1, sr1);
        build_trial<R, NQ, MIXED, Q64>(a, s_pose[(t + 1) & 1], t + 1, tg1, s_g, tb + 1, st1, sr1, iL, fsi);
      }
    }
    __syncthreads();
    // ---- warp 0: acceptance, state update, the moved molecule's cache row ----
    if (warp == 0) {
      R v = lane < NEW ? s_part[lane] : R(0);
#pragma unroll
      for (int m = 16; m >= 1; m >>= 1) v += __shfl_xor_sync(0xffffffffu, v, m);
      const R dEr = __shfl_sync(0xffffffffu, v, 0);
      int acc_flag = 0;
      if (lane == 0) {
        float logh = 0.0f;
        if (LEARN)
          logh = (s_qf_new.lq - cur.qf.lq) - cur.d2 * (s_qf_new.it - cur.qf.it) - cur.r2 * (s_qf_new.ir - cur.qf.ir);
        // Metropolis-Hastings test in the precision of the energies
        bool ok;
        if (MIXED) {
          const float x = fmaf(-(float)dEr, fbeta_e, logh);
          ok = x >= 0.0f || (float)s_lu[tb] < x;
        } else {
          const double x = -((double)dEr * I2J * J2K) * beta + (double)logh;
          ok = x >= 0.0 || (double)s_lu[tb] < x;
        }
        acc_flag = ok ? 1 : 0;
      }
      acc_flag = __shfl_sync(0xffffffffu, acc_flag, 0);
      const double dE = (double)dEr;
      if (acc_flag) {
        // the accepted pose, one component per lane.  In mixed precision the FP64
        // site offsets of the packed pose are not kept during a run: the Monte
        // Carlo kernel reads only the COM of pk64, and every other caller places
        // the molecules again from the state.
        const double q64 = cur.q64[lane & 3];
        double* p = a.pk64 + (size_t)tg * W64;
        float* pf = a.pk32f + (size_t)tg * 4 * NPK;
        if (lane < 4) a.st[(size_t)(33 + lane) * n + tg] = q64;
        if (lane < 3) {
          const double cn = cur.cn[lane];
          const uint32_t fw = cur.fn[lane];
          a.st[(size_t)lane * n + tg] = cn;
          p[lane] = cn;
          pf[lane] = __uint_as_float(fw);
          a.fix[(size_t)lane * n + tg] = fw;
        }
        if (lane < 3 * (NQ + 1)) {
          const R o = (&cur.on[0][0])[lane];
          pf[3 + lane] = (float)o;
          if (!MIXED) p[3 + lane] = (double)o;
        }
        if (lane == 0) {
          energy += dE;
          ++nacc;
          // the next trial's prepared pose is stale when it moves the same molecule,
          // or, with learned widths, when its widths came from a cache row this move changes
          if (s_pose[(t + 1) & 1].trial == t + 1 && (tg1 == tg || (LEARN && s_hit))) s_pose[(t + 1) & 1].trial = -1;
        }
      }
      if (lane == 0) {
        if (a.trace) {
          double* tr = a.trace + ((size_t)c * a.ntrial + t) * 4;
          tr[0] = dE; tr[1] = energy; tr[2] = (double)acc_flag; tr[3] = (double)(tg - i0);
        }
        if (a.samples && a.sample_every > 0 && (t + 1) % a.sample_every == 0)
          a.samples[(size_t)c * a.nsamples + nsample] = energy;
      }
      __syncwarp();
      if constexpr (FEAT) {
        if (MODE == G6_MC_COLLECT && a.records) {   // training record of this trial
          float* rr = a.records + ((size_t)c * a.ntrial + t) * MLP_REC;
          if (lane < MLP_IN) {
            rr[lane] = (float)fcl[(size_t)(tg - i0) * MLP_IN + lane] * FEAT_IQ;
            rr[MLP_IN + lane] = (float)s_feat[lane] * FEAT_IQ;
          }
          if (lane == 0) {
            rr[2 * MLP_IN] = cur.d2;
            rr[2 * MLP_IN + 1] = cur.r2;
            rr[2 * MLP_IN + 2] = (float)((double)dEr * I2J * J2K * beta);
          }
        }
        if (lane == 0) s_accept = acc_flag;
        __syncwarp();
        if (acc_flag) {   // the moved molecule's own cache entries: its new-pose features and site directions
          if (lane < MLP_IN) fcl[(size_t)(tg - i0) * MLP_IN + lane] = s_feat[lane];
          if (lane < 12) a.udir[(size_t)tg * 12 + lane] = cur.un[lane / 3][lane % 3];
        }
      }
      __syncwarp();
    }
    if constexpr (FEAT) {
      // ---- accepted move: the neighbours' prepared terms (new pose added, old
      //      pose subtracted) added to their cache rows, one term per thread ----
      __syncthreads();
      if (s_accept) {
        const int nn = min(s_pool & 0xffff, MC_POOL), no = min(s_pool >> 16, MC_POOL);
        for (int p = threadIdx.x; p < MLP_IN * (nn + no); p += MC_NT) {
          const int q = p / MLP_IN, k = p - q * MLP_IN;
          const bool nw = q < nn;
          const FeEntry& E = nw ? pool_new[q] : pool_old[q - nn];
          const int v = E.d[k];
          if (v != 0) atomicAdd(fcl + (size_t)(E.j - i0) * MLP_IN + k, nw ? v : -v);
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
  }
}

// Shared memory a CTA may give to its chain's feature cache (the rest of the
// 227 KB holds the energy warps' feature neighbours, the network and the L1
// that caches the chain's packed poses).
constexpr size_t MC_FC_SMEM_MAX = 100 * 1024;

template <int NQ, bool TAPER, bool MIXED, int MODE>
static cudaError_t launch_mc_k(McArgs a, cudaStream_t s) {
  const size_t fc_bytes = (size_t)a.ncmax * MLP_IN * sizeof(int);
  size_t dyn = 0;
  a.fc_smem = 0;
  if (MODE != G6_MC_PLAIN) {
    a.fc_smem = fc_bytes <= MC_FC_SMEM_MAX;
    dyn = (a.fc_smem ? fc_bytes : 0) + (size_t)2 * MC_POOL * sizeof(FeEntry);
    cudaError_t e = cudaFuncSetAttribute(k_mc<NQ, TAPER, MIXED, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)dyn);
    if (e != cudaSuccess) return e;
  }
  k_mc<NQ, TAPER, MIXED, MODE><<<a.rep.nrep, MC_NT, dyn, s>>>(a);
  return cudaGetLastError();
}

template <int NQ, bool TAPER, bool MIXED>
static cudaError_t launch_mc_m(const McArgs& a, int mode, cudaStream_t s) {
  if (mode == G6_MC_LEARNED) return launch_mc_k<NQ, TAPER, MIXED, G6_MC_LEARNED>(a, s);
  if (mode == G6_MC_COLLECT) return launch_mc_k<NQ, TAPER, MIXED, G6_MC_COLLECT>(a, s);
  return launch_mc_k<NQ, TAPER, MIXED, G6_MC_PLAIN>(a, s);
}

template <int NQ, bool TAPER>
static cudaError_t launch_mc_t(const McArgs& a, bool mixed, int mode, cudaStream_t s) {
  return mixed ? launch_mc_m<NQ, TAPER, true>(a, mode, s) : launch_mc_m<NQ, TAPER, false>(a, mode, s);
}

cudaError_t launch_mc(const McArgs& a, int model, bool mixed, int mode, cudaStream_t s) {
  if (model_nq(model) == 3) return launch_mc_t<3, false>(a, mixed, mode, s);
  if (a.pc.taper) return launch_mc_t<4, true>(a, mixed, mode, s);
  return launch_mc_t<4, false>(a, mixed, mode, s);
}

}  // namespace g6
