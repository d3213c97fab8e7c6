// g6_mc.cu -- single-molecule Monte Carlo on the device (mc2.F90:544-832).
//
// One CTA advances one chain (= one replica of the context) through ntrial
// sequential trials.  Per trial:
//   thread 0   picks the target (uniform), draws the rotation vector and the
//              translation (Gaussian, the sine branch of Random_Normal,
//              RandomModule.F90:20-28), builds the new quaternion with
//              qinfrotator + qadd (QuatModule.F90:108-133, 203-223) and the new
//              site offsets (rigid_setsiteposition);
//   all        sum e(new, j) - e(old, j) over every other molecule j of the
//              chain with the PairPotential arithmetic (strict rc test, COM
//              switch, ST2 Coulomb taper on the custom path), per-thread
//              partials combined in FP64 in a fixed order;
//   thread 0   Metropolis test exp(-dE * I2J * J2K * beta) (mc2.F90:712-722),
//              and on acceptance writes the new pose.
// Unlike mc2 (which subtracts stored pair energies of the neighbours of the
// new pose only and adapts the step width after every trial), dE runs over all
// neighbours of both poses and the widths are fixed, so the Markov chain is
// exactly Metropolis-Hastings for the chosen widths.  The draws come from the
// same Philox stream as the oracle (counter = chain, trial, draw), so short
// chains can be replayed step by step on the CPU.
//
// Learned widths (LEARNED = true): the proposal widths come from a 24-64-64-2
// MLP on local-environment features, evaluated at the old pose before the draw
// and at the new pose after it; the Hastings ratio includes both densities.
#include <cuda_runtime.h>

#include "g6_internal.cuh"
#include "g6_mlp.cuh"

namespace g6 {

template <int NQ, bool TAPER, class R>
__device__ __forceinline__ R pair_energy(const R d[3], R dd, const R (&ri)[NQ + 1][3], const R (&rj)[NQ + 1][3],
                                         const PairConst& pc, R rin2, R rin, R rout, R c1, R c2) {
  R hh, dh;
  if (dd > rin2) {
    R r = sqrt(dd);
    R u = r - rout, l = r - rin, uu = u * u, ll = l * l;
    hh = c1 * uu * u * (R(10) * ll - R(5) * u * l + uu);
  } else {
    hh = R(1);
  }
  (void)dh;
  R v[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) v[k] = d[k] + ri[0][k] - rj[0][k];
  const R inv = R(1) / (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  const R d6 = inv * inv * inv;
  const R aa = sizeof(R) == 8 ? (R)pc.aa : (R)pc.faa, bb = sizeof(R) == 8 ? (R)pc.bb : (R)pc.fbb;
  const R elj = aa * d6 * d6 + bb * d6;
  R ec = R(0);
#pragma unroll
  for (int a = 1; a <= NQ; ++a)
#pragma unroll
    for (int b = 1; b <= NQ; ++b) {
      R x = d[0] + ri[a][0] - rj[b][0], y = d[1] + ri[a][1] - rj[b][1], z = d[2] + ri[a][2] - rj[b][2];
      const R q = sizeof(R) == 8 ? (R)pc.qq[a - 1][b - 1] : (R)pc.fqq[a - 1][b - 1];
      ec += q * (sizeof(R) == 8 ? (R)rsqrt((double)(x * x + y * y + z * z)) : (R)rsqrtf((float)(x * x + y * y + z * z)));
    }
  R scc = hh;
  if (TAPER) {
    const R rl = sizeof(R) == 8 ? (R)pc.rl : (R)pc.frl, ru = sizeof(R) == 8 ? (R)pc.ru : (R)pc.fru;
    const R w3 = sizeof(R) == 8 ? (R)pc.w3 : (R)pc.fw3;
    R s12;
    if (dd < ru * ru) {
      if (dd < rl * rl) s12 = R(0);
      else {
        R r12 = sqrt(dd);
        s12 = (r12 - rl) * (r12 - rl) * (R(3) * ru - rl - R(2) * r12) / w3;
      }
    } else {
      s12 = R(1);
    }
    scc = hh * s12;
  }
  return hh * elj + scc * ec;
}

// QuatModule.F90:108-133: a1 <- a1 (x) a2, then the shorter of the two signs.
__device__ __forceinline__ void qadd(double q1[4], const double q2[4]) {
  const double a1 = q1[0], b1 = q1[1], c1 = q1[2], d1 = q1[3];
  const double a2 = q2[0], b2 = q2[1], c2 = q2[2], d2 = q2[3];
  double a3 = a1 * a2 - b1 * b2 - c1 * c2 - d1 * d2;
  double b3 = a1 * b2 + b1 * a2 + c1 * d2 - d1 * c2;
  double c3 = a1 * c2 + c1 * a2 - b1 * d2 + d1 * b2;
  double d3 = a1 * d2 + d1 * a2 + b1 * c2 - c1 * b2;
  if (a3 < 0) { a3 = -a3; b3 = -b3; c3 = -c3; d3 = -d3; }
  q1[0] = a3; q1[1] = b3; q1[2] = c3; q1[3] = d3;
}

__device__ __forceinline__ double mc_normal(uint64_t seed, uint32_t chain, uint64_t trial, uint32_t k, double var) {
  double u[2];
  uniform2(seed, chain, (uint32_t)trial, (uint32_t)(trial >> 32), k, u);
  return sqrt(-2.0 * log(u[0])) * sin(2.0 * PI * u[1]) * sqrt(var);
}

struct McShared {
  double com_new[3], q_new[4], off_new[MAXQ + 1][3];
  double com_old[3], off_old[MAXQ + 1][3];
  float off_new_f[MAXQ + 1][3];
  uint32_t fix_new[3];
  int target;
  double sig_t, sig_r, logq_fwd;
  double rot[3], dx[3];
  float feat_old[MLP_IN], feat_new[MLP_IN];
  double part[32];
  double dE;
  int accept;
};

template <int NQ, bool TAPER, bool MIXED, bool LEARNED>
__global__ void __launch_bounds__(256) k_mc(McArgs a) {
  using R = typename std::conditional<MIXED, float, double>::type;
  constexpr int W64 = ((6 + 3 * NQ) + 1) / 2 * 2;
  constexpr int NPK = ((6 + 3 * NQ) + 3) / 4;
  __shared__ McShared sh;
  const int c = blockIdx.x;
  const int i0 = a.rep.off[c], i1 = a.rep.off[c + 1], nc = i1 - i0;
  const int n = a.n;
  double L[3], iL[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) { L[k] = a.rep.L[3 * c + k]; iL[k] = a.rep.invL[3 * c + k]; }
  const float fs[3] = {a.rep.fscale[3 * c], a.rep.fscale[3 * c + 1], a.rep.fscale[3 * c + 2]};
  const double beta = a.beta[c];
  double energy = a.energy[c];
  long long nacc = 0;
  int nsample = 0;
  for (int t = 0; t < a.ntrial; ++t) {
    const uint64_t trial = a.counter + (uint64_t)t;
    if (threadIdx.x == 0) {
      double u[2];
      uniform2(a.seed, (uint32_t)c, (uint32_t)trial, (uint32_t)(trial >> 32), 0u, u);
      int tg = (int)(u[0] * nc);
      if (tg >= nc) tg = nc - 1;   // u = 1 would select nc (mc2.F90:551 quirk)
      sh.target = i0 + tg;
      sh.sig_t = a.sigma_t[c];
      sh.sig_r = a.sigma_r[c];
    }
    __syncthreads();
    const int tg = sh.target;
    if (LEARNED) {
      if (threadIdx.x == 0) {
        const double* po = a.pk64 + (size_t)tg * W64;
        for (int k = 0; k < 3; ++k) sh.com_old[k] = po[k];
        for (int s = 0; s <= NQ; ++s)
          for (int k = 0; k < 3; ++k) sh.off_old[s][k] = po[3 + 3 * s + k];
      }
      __syncthreads();
      mc_features<NQ>(a, tg, sh.com_old, sh.off_old, sh.feat_old, i0, i1, L, iL);   // block-wide
      if (threadIdx.x < 32) mlp_widths(a.mlp, sh.feat_old, &sh.sig_t, &sh.sig_r);
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      const double sr = sh.sig_r, st = sh.sig_t;
      double rot[3], dx[3];
      for (int k = 0; k < 3; ++k) rot[k] = mc_normal(a.seed, c, trial, 1u + k, sr * sr);
      for (int k = 0; k < 3; ++k) dx[k] = mc_normal(a.seed, c, trial, 4u + k, st * st);
      // qinfrotator: normalise (1, x, y, z)
      double qr[4] = {1.0, rot[0], rot[1], rot[2]};
      const double rn = 1.0 / sqrt(qr[0] * qr[0] + qr[1] * qr[1] + qr[2] * qr[2] + qr[3] * qr[3]);
      for (int k = 0; k < 4; ++k) qr[k] *= rn;
      double qo[4];
      for (int k = 0; k < 4; ++k) qo[k] = a.st[(size_t)(33 + k) * n + tg];
      qadd(qr, qo);
      double tm[9];
      {
        const double qa = qr[0], qb = qr[1], qc = qr[2], qd = qr[3];
        tm[0] = (qa * qa + qb * qb - (qc * qc + qd * qd)); tm[1] = -2.0 * (qa * qd + qb * qc);
        tm[2] = 2.0 * (qb * qd - qa * qc); tm[3] = 2.0 * (qa * qd - qb * qc);
        tm[4] = qa * qa + qc * qc - (qb * qb + qd * qd); tm[5] = -2.0 * (qa * qb + qc * qd);
        tm[6] = 2.0 * (qa * qc + qb * qd); tm[7] = 2.0 * (qa * qb - qc * qd);
        tm[8] = qa * qa + qd * qd - (qb * qb + qc * qc);
      }
      for (int k = 0; k < 4; ++k) sh.q_new[k] = qr[k];
      for (int k = 0; k < 3; ++k) { sh.com_new[k] = a.st[(size_t)k * n + tg] + dx[k]; sh.rot[k] = rot[k]; sh.dx[k] = dx[k]; }
      for (int s = 0; s <= NQ; ++s) {
        const double bx = a.body[s][0], by = a.body[s][1], bz = a.body[s][2];
        const double o[3] = {tm[0] * bx + tm[1] * by + tm[2] * bz, tm[3] * bx + tm[4] * by + tm[5] * bz,
                             tm[6] * bx + tm[7] * by + tm[8] * bz};
        for (int k = 0; k < 3; ++k) { sh.off_new[s][k] = o[k]; sh.off_new_f[s][k] = (float)o[k]; }
      }
      for (int k = 0; k < 3; ++k) sh.fix_new[k] = to_fixed(sh.com_new[k], iL[k]);
    }
    __syncthreads();
    // dE over all other molecules of the chain
    double part = 0.0;
    {
      const double* po = a.pk64 + (size_t)tg * W64;
      double co[3] = {po[0], po[1], po[2]};
      R ro[NQ + 1][3], rn[NQ + 1][3];
      uint32_t fo[3] = {a.fix[tg], a.fix[n + tg], a.fix[2 * n + tg]};
#pragma unroll
      for (int s = 0; s <= NQ; ++s)
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          ro[s][k] = MIXED ? (R)a.pk32f[(size_t)tg * 4 * NPK + 3 + 3 * s + k] : (R)po[3 + 3 * s + k];
          rn[s][k] = MIXED ? (R)sh.off_new_f[s][k] : (R)sh.off_new[s][k];
        }
      const R rin2 = MIXED ? (R)a.cc.frin2 : (R)a.cc.rin2, rin = MIXED ? (R)a.cc.frin : (R)a.cc.rin;
      const R rout = MIXED ? (R)a.cc.frout : (R)a.cc.rout;
      const R c1 = MIXED ? (R)a.cc.fc1 : (R)a.cc.c1, c2 = MIXED ? (R)a.cc.fc2 : (R)a.cc.c2;
      R acc = R(0);
      for (int j = i0 + threadIdx.x; j < i1; j += blockDim.x) {
        if (j == tg) continue;
        const double* pj = a.pk64 + (size_t)j * W64;
        R rj[NQ + 1][3];
        for (int pose = 0; pose < 2; ++pose) {
          R d[3];
          R dd;
          bool in;
          if (MIXED) {
            const uint32_t* f = pose ? sh.fix_new : fo;
            d[0] = (R)((float)(int)(f[0] - a.fix[j]) * fs[0]);
            d[1] = (R)((float)(int)(f[1] - a.fix[n + j]) * fs[1]);
            d[2] = (R)((float)(int)(f[2] - a.fix[2 * n + j]) * fs[2]);
            dd = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            in = dd < (R)a.cc.frout2;
            if (fabs((double)dd - a.cc.rout2) < 1e-3) {
              double cj[3] = {pj[0], pj[1], pj[2]}, o[3], dx[3];
              in = exact_dd(pose ? sh.com_new : co, cj, L, iL, o, dx) < a.cc.rout2;
            }
          } else {
            double cj[3] = {pj[0], pj[1], pj[2]}, o[3], dx[3];
            const double ddd = exact_dd(pose ? sh.com_new : co, cj, L, iL, o, dx);
            in = ddd < a.cc.rout2;
            d[0] = (R)dx[0]; d[1] = (R)dx[1]; d[2] = (R)dx[2];
            dd = (R)ddd;
          }
          if (!in) continue;
#pragma unroll
          for (int s = 0; s <= NQ; ++s)
#pragma unroll
            for (int k = 0; k < 3; ++k)
              rj[s][k] = MIXED ? (R)a.pk32f[(size_t)j * 4 * NPK + 3 + 3 * s + k] : (R)pj[3 + 3 * s + k];
          const R e = pose ? pair_energy<NQ, TAPER, R>(d, dd, rn, rj, a.pc, rin2, rin, rout, c1, c2)
                           : pair_energy<NQ, TAPER, R>(d, dd, ro, rj, a.pc, rin2, rin, rout, c1, c2);
          acc += pose ? e : -e;
        }
      }
      part = (double)acc;
    }
    // fixed-order block reduction in FP64
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) part += __shfl_xor_sync(0xffffffffu, part, m);
    if ((threadIdx.x & 31) == 0) sh.part[threadIdx.x >> 5] = part;
    if (LEARNED) mc_features<NQ>(a, tg, sh.com_new, sh.off_new, sh.feat_new, i0, i1, L, iL);
    __syncthreads();
    if (LEARNED && threadIdx.x < 32) {
      double st2, sr2;
      mlp_widths(a.mlp, sh.feat_new, &st2, &sr2);
      if (threadIdx.x == 0) {
        // log q(old|new) - log q(new|old) for isotropic Gaussians in translation and rotation vector
        double d2 = sh.dx[0] * sh.dx[0] + sh.dx[1] * sh.dx[1] + sh.dx[2] * sh.dx[2];
        double r2 = sh.rot[0] * sh.rot[0] + sh.rot[1] * sh.rot[1] + sh.rot[2] * sh.rot[2];
        const double lf = -3.0 * log(sh.sig_t) - d2 / (2.0 * sh.sig_t * sh.sig_t) - 3.0 * log(sh.sig_r) -
                          r2 / (2.0 * sh.sig_r * sh.sig_r);
        const double lr = -3.0 * log(st2) - d2 / (2.0 * st2 * st2) - 3.0 * log(sr2) - r2 / (2.0 * sr2 * sr2);
        sh.logq_fwd = lr - lf;
      }
    }
    if (threadIdx.x == 0) {
      double dE = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) dE += sh.part[w];
      double u[2];
      uniform2(a.seed, (uint32_t)c, (uint32_t)trial, (uint32_t)(trial >> 32), 0u, u);
      const double logh = LEARNED ? sh.logq_fwd : 0.0;
      bool acc = false;
      const double x = -(dE * I2J * J2K) * beta + logh;
      if (x >= 0.0) acc = true;
      else acc = u[1] < exp(x);
      sh.accept = acc ? 1 : 0;
      sh.dE = dE;
      if (LEARNED && a.records) {   // training record of this trial
        float* rr = a.records + ((size_t)c * a.ntrial + t) * MLP_REC;
        for (int k = 0; k < MLP_IN; ++k) { rr[k] = sh.feat_old[k]; rr[MLP_IN + k] = sh.feat_new[k]; }
        rr[2 * MLP_IN] = (float)(sh.dx[0] * sh.dx[0] + sh.dx[1] * sh.dx[1] + sh.dx[2] * sh.dx[2]);
        rr[2 * MLP_IN + 1] = (float)(sh.rot[0] * sh.rot[0] + sh.rot[1] * sh.rot[1] + sh.rot[2] * sh.rot[2]);
        rr[2 * MLP_IN + 2] = (float)(dE * I2J * J2K * beta);
      }
      if (a.trace) a.trace[((size_t)c * a.ntrial + t) * 4 + 0] = dE;
    }
    __syncthreads();
    if (sh.accept) {
      // write the new pose (state, packed poses, fixed point); one thread per field group
      if (threadIdx.x == 0) {
        for (int k = 0; k < 3; ++k) a.st[(size_t)k * n + tg] = sh.com_new[k];
        for (int k = 0; k < 4; ++k) a.st[(size_t)(33 + k) * n + tg] = sh.q_new[k];
        double* p = a.pk64 + (size_t)tg * W64;
        for (int k = 0; k < 3; ++k) p[k] = sh.com_new[k];
        for (int s = 0; s <= NQ; ++s)
          for (int k = 0; k < 3; ++k) p[3 + 3 * s + k] = sh.off_new[s][k];
        float* pf = a.pk32f + (size_t)tg * 4 * NPK;
        for (int k = 0; k < 3; ++k) pf[k] = __uint_as_float(sh.fix_new[k]);
        for (int s = 0; s <= NQ; ++s)
          for (int k = 0; k < 3; ++k) pf[3 + 3 * s + k] = sh.off_new_f[s][k];
        for (int k = 0; k < 3; ++k) a.fix[(size_t)k * n + tg] = sh.fix_new[k];
      }
      energy += sh.dE;
      ++nacc;
    }
    if (threadIdx.x == 0 && a.trace) {
      a.trace[((size_t)c * a.ntrial + t) * 4 + 1] = energy;
      a.trace[((size_t)c * a.ntrial + t) * 4 + 2] = (double)sh.accept;
      a.trace[((size_t)c * a.ntrial + t) * 4 + 3] = (double)(tg - i0);
    }
    if (a.samples && a.sample_every > 0 && (t + 1) % a.sample_every == 0 && threadIdx.x == 0) {
      a.samples[(size_t)c * a.nsamples + nsample] = energy;
    }
    if (a.sample_every > 0 && (t + 1) % a.sample_every == 0) ++nsample;
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    a.energy[c] = energy;
    a.counts[2 * c] += nacc;
    a.counts[2 * c + 1] += a.ntrial;
  }
}

template <int NQ, bool TAPER>
static cudaError_t launch_mc_t(const McArgs& a, bool mixed, bool learned, cudaStream_t s) {
  const int nb = a.rep.nrep;
  if (mixed) {
    if (learned) k_mc<NQ, TAPER, true, true><<<nb, 256, 0, s>>>(a);
    else k_mc<NQ, TAPER, true, false><<<nb, 256, 0, s>>>(a);
  } else {
    if (learned) k_mc<NQ, TAPER, false, true><<<nb, 256, 0, s>>>(a);
    else k_mc<NQ, TAPER, false, false><<<nb, 256, 0, s>>>(a);
  }
  return cudaGetLastError();
}

cudaError_t launch_mc(const McArgs& a, int model, bool mixed, bool learned, cudaStream_t s) {
  if (model == G6_TIP4P) return launch_mc_t<3, false>(a, mixed, learned, s);
  if (a.pc.taper) return launch_mc_t<4, true>(a, mixed, learned, s);
  return launch_mc_t<4, false>(a, mixed, learned, s);
}

}  // namespace g6
