// g6_md.cu -- rigid-body Gear predictor-corrector and per-step reductions.
//
// k_predict_place: rigid_predict (RigidModule.F90:480-559) and site placement
//   (rigid_setmatrix :62-83, rigid_setsiteposition0 :88-144) for one molecule
//   per thread, writing the packed poses the force kernel reads.
// k_correct_step: rigid_correct (RigidModule.F90:1255-1487) with Nose friction,
//   the optional stochastic-collision thermostat, Rigid_Ek / Rigid_PressureTensor
//   partials (:576-619), then the next step's predict + placement and the
//   displacement test of the neighbour list.  Per-replica sums are reduced
//   per block (segmented by replica) and the last block to finish reduces the
//   block partials in a fixed order (deterministic), computes T, P and the
//   conserved quantity (Mixture.F90:2251-2264, 2431-2453), runs Nose_Correct
//   and the next Nose_Predict (NoseModule.F90:43-87), and sets the rebuild flag.
// Everything here is FP64.
#include <cuda_runtime.h>

#include "g6_internal.cuh"

namespace g6 {




#define ST(c) st[(size_t)(c) * n + i]

__device__ __forceinline__ void setmatrix(const double q[4], double t[9]) {
  const double qa = q[0], qb = q[1], qc = q[2], qd = q[3];
  t[0] = (qa * qa + qb * qb - (qc * qc + qd * qd));
  t[1] = -2.0 * (qa * qd + qb * qc);
  t[2] = 2.0 * (qb * qd - qa * qc);
  t[3] = 2.0 * (qa * qd - qb * qc);
  t[4] = qa * qa + qc * qc - (qb * qb + qd * qd);
  t[5] = -2.0 * (qa * qb + qc * qd);
  t[6] = 2.0 * (qa * qc + qb * qd);
  t[7] = 2.0 * (qa * qb - qc * qd);
  t[8] = qa * qa + qd * qd - (qb * qb + qc * qc);
}

__device__ void predict_one(double* st, int n, int i) {
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    double d1 = ST(3 + a), d2 = ST(6 + a), d3 = ST(9 + a), d4 = ST(12 + a), d5 = ST(15 + a);
    ST(a) = ST(a) + d1 + d2 + d3 + d4 + d5;
    ST(3 + a) = d1 + 2.0 * d2 + 3.0 * d3 + 4.0 * d4 + 5.0 * d5;
    ST(6 + a) = d2 + 3.0 * d3 + 6.0 * d4 + 10.0 * d5;
    ST(9 + a) = d3 + 4.0 * d4 + 10.0 * d5;
    ST(12 + a) = d4 + 5.0 * d5;
  }
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    double w1 = ST(18 + a), w2 = ST(21 + a), w3 = ST(24 + a), w4 = ST(27 + a), w5 = ST(30 + a);
    ST(18 + a) = w1 + w2 + w3 + w4 + w5;
    ST(21 + a) = w2 + 2.0 * w3 + 3.0 * w4 + 4.0 * w5;
    ST(24 + a) = w3 + 3.0 * w4 + 6.0 * w5;
    ST(27 + a) = w4 + 4.0 * w5;
  }
  double q[4];
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    double q1 = ST(33 + a), q2 = ST(37 + a), q3 = ST(41 + a), q4 = ST(45 + a), q5 = ST(49 + a);
    q[a] = q1 + q2 + q3 + q4 + q5;
    ST(37 + a) = q2 + 2.0 * q3 + 3.0 * q4 + 4.0 * q5;
  }
  double re = 1.0 / sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
#pragma unroll
  for (int a = 0; a < 4; ++a) ST(33 + a) = q[a] * re;
}

__device__ void place_one(const PlaceArgs& a, int i) {
  const int n = a.n;
  double* st = a.st;
  double q[4] = {ST(33), ST(34), ST(35), ST(36)};
  double t[9];
  setmatrix(q, t);
#pragma unroll
  for (int k = 0; k < 9; ++k) a.tmat[(size_t)k * n + i] = t[k];
  const int r = a.rep.mol_rep[i];
  const double com[3] = {ST(0), ST(1), ST(2)};
  double* p64 = a.pk64 + (size_t)i * a.w64;
  p64[0] = com[0]; p64[1] = com[1]; p64[2] = com[2];
  float w[24];
#pragma unroll
  for (int k = 0; k < 24; ++k) w[k] = 0.0f;
  uint32_t fx = to_fixed(com[0], a.rep.invL[3 * r]);
  uint32_t fy = to_fixed(com[1], a.rep.invL[3 * r + 1]);
  uint32_t fz = to_fixed(com[2], a.rep.invL[3 * r + 2]);
  a.fix[i] = fx; a.fix[n + i] = fy; a.fix[2 * n + i] = fz;
  w[0] = __uint_as_float(fx); w[1] = __uint_as_float(fy); w[2] = __uint_as_float(fz);
  for (int s = 0; s <= a.nq; ++s) {   // LJ site then charged sites; the COM site offset is zero
    const double bx = a.body[s][0], by = a.body[s][1], bz = a.body[s][2];
    double o[3] = {t[0] * bx + t[1] * by + t[2] * bz, t[3] * bx + t[4] * by + t[5] * bz,
                   t[6] * bx + t[7] * by + t[8] * bz};
    for (int k = 0; k < 3; ++k) { p64[3 + 3 * s + k] = o[k]; w[3 + 3 * s + k] = (float)o[k]; }
  }
  for (int k = 3 + 3 * (a.nq + 1); k < a.w64; ++k) p64[k] = 0.0;
  for (int q4 = 0; q4 < a.npk; ++q4)
    a.pk32[(size_t)i * a.npk + q4] = make_float4(w[4 * q4], w[4 * q4 + 1], w[4 * q4 + 2], w[4 * q4 + 3]);
}

__global__ void k_predict_place(PlaceArgs a, int do_predict, ThermoDev* th, int nose_predict) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (nose_predict && blockIdx.x == 0) {
    for (int r = threadIdx.x; r < a.rep.nrep; r += blockDim.x) {
      ThermoDev& T = th[r];
      if (T.kind == G6_NOSE) {   // Nose_Predict
        T.z[0] = T.z[0] + T.z[1] + T.z[2] + T.z[3] + T.z[4];
        T.z[1] = T.z[1] + 2.0 * T.z[2] + 3.0 * T.z[3] + 4.0 * T.z[4];
        T.z[2] = T.z[2] + 3.0 * T.z[3] + 6.0 * T.z[4];
        T.z[3] = T.z[3] + 4.0 * T.z[4];
      }
    }
  }
  if (i >= a.n) return;
  if (do_predict) predict_one(a.st, a.n, i);
  place_one(a, i);
}

cudaError_t launch_predict_place(const PlaceArgs& a, int do_predict, ThermoDev* th, int nose_predict,
                                 cudaStream_t s) {
  const int blocks = a.n > 0 ? (a.n + 127) / 128 : 1;
  k_predict_place<<<blocks, 128, 0, s>>>(a, do_predict, th, nose_predict);
  return cudaGetLastError();
}

// (1/2) W(w) q pattern of RigidModule.F90:1337-1348
__device__ __forceinline__ void qdot(const double w[3], const double q[4], double o[4]) {
  o[0] = (-w[0] * q[1] + w[1] * q[2] - w[2] * q[3]);
  o[1] = (w[0] * q[0] - w[1] * q[3] - w[2] * q[2]);
  o[2] = (-w[0] * q[3] - w[1] * q[0] + w[2] * q[1]);
  o[3] = (w[0] * q[2] + w[1] * q[1] + w[2] * q[0]);
}

__device__ __forceinline__ double normal_pair(double u1, double u2, double& second) {
  double r = sqrt(-2.0 * log(u1));
  double s, c;
  sincospi(2.0 * u2, &s, &c);
  second = r * c;
  return r * s;
}

// Segmented (by replica) block reduction of NV values; molecules are in
// replica order so a block spans replicas rfirst..rlast (<= MAXREP_PER_BLOCK).
template <int NV>
__device__ void block_segmented_sum(const double (&v)[NV], int r, int rfirst, int nslots, double* out_part) {
  __shared__ double sh[RED_BLOCK / 32][NV];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int s = 0; s < nslots; ++s) {
    const bool mine = (r == rfirst + s);
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double x = mine ? v[k] : 0.0;
#pragma unroll
      for (int m = 16; m >= 1; m >>= 1) x += __shfl_xor_sync(0xffffffffu, x, m);
      if (lane == 0) sh[warp][k] = x;
    }
    __syncthreads();
    if (threadIdx.x < NV) {
      double x = 0.0;
      for (int w = 0; w < RED_BLOCK / 32; ++w) x += sh[w][threadIdx.x];
      out_part[s * NV + threadIdx.x] = x;
    }
    __syncthreads();
  }
}

__global__ void __launch_bounds__(RED_BLOCK) k_correct_step(StepArgs a) {
  const int n = a.p.n;
  double* st = a.p.st;
  const int i = blockIdx.x * RED_BLOCK + threadIdx.x;
  const bool valid = i < n;
  const int step = a.ctrl[1];
  const bool predict_next = step + 1 < a.ctrl[2];
  const int r = valid ? a.p.rep.mol_rep[i] : -1;
  double v[NRED];
#pragma unroll
  for (int k = 0; k < NRED; ++k) v[k] = 0.0;
  double dmax2 = 0.0;
  int bad = 0;
  if (valid) {
    const ThermoDev th = a.th[r];
    const double dt = a.dt;
    // body torque = T^T tau_lab (rigid_collectforce :305-310)
    double t[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) t[k] = a.p.tmat[(size_t)k * n + i];
    const double F[3] = {a.F[i], a.F[n + i], a.F[2 * n + i]};
    const double tl[3] = {a.tl[i], a.tl[n + i], a.tl[2 * n + i]};
    const double tau[3] = {t[0] * tl[0] + t[3] * tl[1] + t[6] * tl[2], t[1] * tl[0] + t[4] * tl[1] + t[7] * tl[2],
                           t[2] * tl[0] + t[5] * tl[1] + t[8] * tl[2]};
    if (!(isfinite(F[0]) && isfinite(F[1]) && isfinite(F[2]) && isfinite(tau[0]) && isfinite(tau[1]) &&
          isfinite(tau[2])))
      bad = 1;
    double ext_t = 0.0, ext_r = 0.0;
    if (th.kind == G6_NOSE) {
      const double nc = th.z[0] * dt;
      ext_t = nc * 0.5;
      ext_r = nc;
    }
    // COM: Gear-5
    const double massi = 1.0 / a.mass;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      double nf = F[c] * (dt * dt * 0.5 * massi);
      nf = nf - ST(3 + c) * ext_t;
      const double delta = nf - ST(6 + c);
      ST(c) = ST(c) + G50 * delta;
      ST(3 + c) = ST(3 + c) + G51 * delta;
      ST(6 + c) = nf;
      ST(9 + c) = ST(9 + c) + G53 * delta;
      ST(12 + c) = ST(12 + c) + G54 * delta;
      ST(15 + c) = ST(15 + c) + G55 * delta;
    }
    // quaternion value
    double q1[4] = {ST(33), ST(34), ST(35), ST(36)};
    double w1[3] = {ST(18), ST(19), ST(20)};
    double nw[4];
    qdot(w1, q1, nw);
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const double dw = nw[c] * dt * 0.5 - ST(37 + c);
      q1[c] = q1[c] + G40 * dw;
      ST(33 + c) = q1[c];
    }
    // angular velocity: Gear-4 with Euler's equations
    const double Ix = a.I[0], Iy = a.I[1], Iz = a.I[2];
    double nf[3];
    nf[0] = (tau[0] + (Iy - Iz) * w1[1] * w1[2]) * dt * (1.0 / Ix);
    nf[1] = (tau[1] + (Iz - Ix) * w1[2] * w1[0]) * dt * (1.0 / Iy);
    nf[2] = (tau[2] + (Ix - Iy) * w1[0] * w1[1]) * dt * (1.0 / Iz);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      nf[c] = nf[c] - w1[c] * ext_r;
      const double delta = nf[c] - ST(21 + c);
      ST(18 + c) = ST(18 + c) + G40 * delta;
      ST(21 + c) = nf[c];
      ST(24 + c) = ST(24 + c) + G42 * delta;
      ST(27 + c) = ST(27 + c) + G43 * delta;
      ST(30 + c) = ST(30 + c) + G44 * delta;
    }
    // stochastic collisions (new thermostat; velocity resampled from Maxwell-Boltzmann)
    if (th.kind == G6_ANDERSEN) {
      double u[2];
      const uint32_t sc = (uint32_t)(a.ctrl[6] + step);
      uniform2(a.seed, (uint32_t)i, sc, 0x41u, 0u, u);
      if (u[0] <= th.rate * dt) {
        const double kT = th.temp * RGAS * J2I;
        double z[6];
        for (int p = 0; p < 3; ++p) {
          double g[2];
          uniform2(a.seed, (uint32_t)i, sc, 0x41u, (uint32_t)(p + 1), g);
          z[2 * p] = normal_pair(g[0], g[1], z[2 * p + 1]);
        }
        const double sv = sqrt(kT * massi) * dt;
        for (int c = 0; c < 3; ++c) ST(3 + c) = z[c] * sv;
        ST(18) = z[3] * sqrt(kT / Ix);
        ST(19) = z[4] * sqrt(kT / Iy);
        ST(20) = z[5] * sqrt(kT / Iz);
      }
    }
    // quaternion derivative stacks from the corrected angular-velocity stack
    double W[5][3], Q[5][4], tq[4], uq[4], vq[4], xq[4];
#pragma unroll
    for (int k = 0; k < 5; ++k)
#pragma unroll
      for (int c = 0; c < 3; ++c) W[k][c] = ST(18 + 3 * k + c);
#pragma unroll
    for (int c = 0; c < 4; ++c) Q[0][c] = q1[c];
    qdot(W[0], Q[0], tq);
#pragma unroll
    for (int c = 0; c < 4; ++c) Q[1][c] = tq[c] * dt * 0.5;
    qdot(W[1], Q[0], tq); qdot(W[0], Q[1], uq);
#pragma unroll
    for (int c = 0; c < 4; ++c) Q[2][c] = (tq[c] + uq[c]) * dt * 0.25;
    qdot(W[2], Q[0], tq); qdot(W[0], Q[2], uq); qdot(W[1], Q[1], vq);
#pragma unroll
    for (int c = 0; c < 4; ++c) Q[3][c] = (tq[c] + uq[c] + vq[c]) * dt * (1.0 / 6.0);
    qdot(W[3], Q[0], tq); qdot(W[2], Q[1], uq); qdot(W[1], Q[2], vq); qdot(W[0], Q[3], xq);
#pragma unroll
    for (int c = 0; c < 4; ++c) Q[4][c] = (tq[c] + uq[c] + vq[c] + xq[c]) * dt * (1.0 / 8.0);
#pragma unroll
    for (int k = 1; k < 5; ++k)
#pragma unroll
      for (int c = 0; c < 4; ++c) ST(33 + 4 * k + c) = Q[k][c];
    // reductions: Epot, virial, kinetic sums, kinetic tensor, pairs
    const double d1[3] = {ST(3), ST(4), ST(5)};
    v[0] = a.emol[i];
#pragma unroll
    for (int k = 0; k < 9; ++k) v[1 + k] = a.wmol[(size_t)k * n + i];
    v[10] = d1[0] * d1[0] + d1[1] * d1[1] + d1[2] * d1[2];
    v[11] = W[0][0] * W[0][0];
    v[12] = W[0][1] * W[0][1];
    v[13] = W[0][2] * W[0][2];
#pragma unroll
    for (int p = 0; p < 3; ++p)
#pragma unroll
      for (int q = 0; q < 3; ++q) v[14 + 3 * p + q] = d1[p] * d1[q];
    v[23] = a.npin ? 0.5 * (double)a.npin[i] : 0.0;
    if (predict_next) {
      predict_one(st, n, i);
      place_one(a.p, i);
      const double dx = ST(0) - a.com_build[i], dy = ST(1) - a.com_build[n + i], dz = ST(2) - a.com_build[2 * n + i];
      dmax2 = dx * dx + dy * dy + dz * dz;
      if (!isfinite(dmax2)) { bad = 1; dmax2 = 1e300; }
    }
  }
  // per-block, per-replica partial sums
  const int first_i = blockIdx.x * RED_BLOCK;
  const int last_i = min(n, first_i + RED_BLOCK) - 1;
  const int rfirst = a.p.rep.mol_rep[first_i];
  const int nslots = a.p.rep.mol_rep[last_i] - rfirst + 1;
  block_segmented_sum<NRED>(v, r, rfirst, nslots, a.part + (size_t)blockIdx.x * MAXREP_PER_BLOCK * NRED);
  {
    __shared__ double shm[RED_BLOCK / 32];
    __shared__ int shbad[RED_BLOCK / 32];
    double m = dmax2;
    int b = bad;
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
      m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
      b |= __shfl_xor_sync(0xffffffffu, b, o);
    }
    if ((threadIdx.x & 31) == 0) { shm[threadIdx.x >> 5] = m; shbad[threadIdx.x >> 5] = b; }
    __syncthreads();
    if (threadIdx.x == 0) {
      double mm = 0.0;
      int bb = 0;
      for (int w = 0; w < RED_BLOCK / 32; ++w) { mm = fmax(mm, shm[w]); bb |= shbad[w]; }
      a.partmax[blockIdx.x] = mm;
      if (bb) atomicOr(&a.ctrl[3], 1);
    }
  }
  // last block finalises the step
  __shared__ int am_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) am_last = (atomicAdd(a.done, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!am_last) return;
  __threadfence();
  const int nrep = a.p.rep.nrep;
  for (int task = threadIdx.x; task < nrep * NRED; task += RED_BLOCK) {
    const int rr = task / NRED, k = task % NRED;
    const int b0 = a.p.rep.off[rr] / RED_BLOCK, b1 = (a.p.rep.off[rr + 1] - 1) / RED_BLOCK;
    double s = 0.0;
    for (int b = b0; b <= b1; ++b) {
      const int slot = rr - a.p.rep.mol_rep[b * RED_BLOCK];
      s += __ldcg(&a.part[((size_t)b * MAXREP_PER_BLOCK + slot) * NRED + k]);
    }
    a.red[task] = s;
  }
  __shared__ double gmax;
  if (threadIdx.x == 0) {
    double m = 0.0;
    for (int b = 0; b < (int)gridDim.x; ++b) m = fmax(m, __ldcg(&a.partmax[b]));
    gmax = m;
  }
  __threadfence_block();
  __syncthreads();
  const int logcap = a.ctrl[5];
  for (int rr = threadIdx.x; rr < nrep; rr += RED_BLOCK) {
    const double* s = a.red + (size_t)rr * NRED;
    ThermoDev& th = a.th[rr];
    const int nm = a.p.rep.off[rr + 1] - a.p.rep.off[rr];
    const double dof = 6.0 * nm;
    const double dt = a.dt;
    const double ekt = s[10] * a.mass * 0.5 * (1.0 / (dt * dt));
    const double ekr = (s[11] * a.I[0] + s[12] * a.I[1] + s[13] * a.I[2]) * 0.5;
    const double temperature = I2J * 2.0 * (ekt + ekr) / (RGAS * dof);
    const double pkin = (s[14] + s[18] + s[22]) * a.mass * (1.0 / (dt * dt));
    const double vp = pkin + s[1] + s[5] + s[9];
    const double V = a.p.rep.L[3 * rr] * a.p.rep.L[3 * rr + 1] * a.p.rep.L[3 * rr + 2];
    const double pressure = (vp / 3.0) * I2J * (1.0 / A2P) / (V * NA * ANG2M * ANG2M * ANG2M);
    if (th.kind == G6_NOSE) {   // Nose_Correct
      const double zetaf = (temperature - th.temp) / th.q - th.dump * th.z[0];
      const double dz2 = zetaf - th.z[1];
      th.z[0] = th.z[0] + G40 * dz2;
      th.z[1] = zetaf;
      th.z[2] = th.z[2] + G42 * dz2;
      th.z[3] = th.z[3] + G43 * dz2;
      th.z[4] = th.z[4] + G44 * dz2;
      th.zsum = th.zsum + th.z[0];
    }
    double nose_ek = 0.0, nose_ep = 0.0;
    if (th.kind == G6_NOSE) {
      nose_ek = (th.z[0] * th.z[0] * th.q * dt * dof * 0.5) * RGAS;
      nose_ep = (dof * th.temp * (th.zsum - 0.5 * th.z[0]) * dt) * RGAS;
    }
    if (a.log && step < logcap) {
      double* lg = a.log + ((size_t)step * nrep + rr) * G6_LOG_WIDTH;
      lg[0] = s[0]; lg[1] = ekt; lg[2] = ekr; lg[3] = temperature; lg[4] = pressure;
      lg[5] = (s[0] + ekt + ekr) * I2J + nose_ep + nose_ek;
      lg[6] = s[23]; lg[7] = th.z[0]; lg[8] = (double)a.ctrl[0]; lg[9] = (double)step;
    }
    if (predict_next && th.kind == G6_NOSE) {   // Nose_Predict for the next step
      th.z[0] = th.z[0] + th.z[1] + th.z[2] + th.z[3] + th.z[4];
      th.z[1] = th.z[1] + 2.0 * th.z[2] + 3.0 * th.z[3] + 4.0 * th.z[4];
      th.z[2] = th.z[2] + 3.0 * th.z[3] + 6.0 * th.z[4];
      th.z[3] = th.z[3] + 4.0 * th.z[4];
    }
  }
  if (threadIdx.x == 0) {
    a.ctrl[0] = (predict_next && gmax > a.half_skin2) ? 1 : 0;
    a.ctrl[1] = step + 1;
    *a.done = 0u;
  }
}

cudaError_t launch_correct_step(const StepArgs& a, cudaStream_t s) {
  const int blocks = (a.p.n + RED_BLOCK - 1) / RED_BLOCK;
  k_correct_step<<<blocks, RED_BLOCK, 0, s>>>(a);
  return cudaGetLastError();
}

// Replica exchange for neighbouring temperature pairs (replica_exchange_trial,
// Replica.F90:7-73) with the MD side effects of Mixture.F90:1616-1653: the
// replica that changes temperature has its first derivatives scaled by
// sqrt(T_new/T_old) (Rigid_ScaleVelocity) and its Nose zeta stack zeroed.

__global__ void k_exchange(ExchArgs a) {
  for (int r = threadIdx.x; r < a.nrep; r += blockDim.x) a.scale[r] = 1.0;
  __syncthreads();
  for (int r = threadIdx.x; r + 1 < a.nrep; r += blockDim.x) {
    if ((r & 1) != a.parity) continue;
    const int r1 = r + 1;
    const double a0 = a.epot[r], a1 = a.epot[r1];
    const double b0 = a.beta[r], b1 = a.beta[r1];
    const double acc0 = -(a0 * b0 + a1 * b1) * I2J * J2K;
    const double acc1 = -(a0 * b1 + a1 * b0) * I2J * J2K;
    bool accept = false;
    if (acc0 < acc1) accept = true;
    else {
      double u[2];
      uniform2(a.seed, (uint32_t)r, (uint32_t)a.counter, (uint32_t)(a.counter >> 32), 0x52u, u);
      accept = u[0] < exp(acc1 - acc0);
    }
    if (a.accepted) a.accepted[r] = accept ? 1 : 0;
    if (accept) {
      a.beta[r] = b1; a.beta[r1] = b0;
      const double t0 = a.th[r].temp, t1 = a.th[r1].temp;
      a.scale[r] = sqrt(t1 / t0);
      a.scale[r1] = sqrt(t0 / t1);
      a.th[r].temp = t1; a.th[r1].temp = t0;
      for (int k = 0; k < 5; ++k) { a.th[r].z[k] = 0.0; a.th[r1].z[k] = 0.0; }
    }
  }
}

__global__ void k_scale_velocity(double* st, int n, const int* mol_rep, const double* scale) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double f = scale[mol_rep[i]];
  if (f == 1.0) return;
  for (int c = 0; c < 3; ++c) { ST(3 + c) *= f; ST(18 + c) *= f; }
}

cudaError_t launch_exchange(const ExchArgs& a, double* st, int n, const int* mol_rep, cudaStream_t s) {
  k_exchange<<<1, 128, 0, s>>>(a);
  if (n > 0) k_scale_velocity<<<(n + 127) / 128, 128, 0, s>>>(st, n, mol_rep, a.scale);
  return cudaGetLastError();
}

// AoS rigid records (n x 53) <-> SoA device state (53 x n).
__global__ void k_rec_transpose(double* aos, double* soa, int n, int to_soa) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)n * REC) return;
  const int c = (int)(t / n), i = (int)(t % n);
  if (to_soa) soa[t] = aos[(size_t)i * REC + c];
  else aos[(size_t)i * REC + c] = soa[t];
}

cudaError_t launch_rec_transpose(double* aos, double* soa, int n, int to_soa, cudaStream_t s) {
  const long long total = (long long)n * REC;
  if (total == 0) return cudaSuccess;
  k_rec_transpose<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(aos, soa, n, to_soa);
  return cudaGetLastError();
}

}  // namespace g6
