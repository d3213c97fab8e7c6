// g6_rigid.cuh -- rigid-body Gear predictor-corrector, site placement and the
// per-step reductions, as device functions shared by the placement kernel
// (g6_md.cu) and the fused force+integrator step kernel (g6_force.cu).
//
//   predict_one   rigid_predict (RigidModule.F90:480-559)
//   place_to      rigid_setmatrix + rigid_setsiteposition0 (RigidModule.F90:62-144):
//                 rotation matrix and the packed poses the site loop reads
//   correct_one   rigid_correct (RigidModule.F90:1255-1487) with Nose friction and
//                 the stochastic-collision thermostat, the Rigid_Ek /
//                 Rigid_PressureTensor terms (:576-619) of one molecule, then the next
//                 step's predict + placement and the neighbour-list displacement test
//   step_reduce   per-block, per-replica partial sums of the step; the last block
//                 of each replica runs finish_replica, the last block overall
//                 advances the step counter
//   finish_replica per-replica sums in a fixed order, T, P and the conserved
//                 quantity (Mixture.F90:2251-2264, 2431-2453), Nose_Correct and the
//                 next Nose_Predict (NoseModule.F90:43-87), the step log
// The plain path is all FP64; the mixed path (correct_mixed, predict_mixed,
// place_mixed) keeps FP64 for com, d1, w1 and q and float for the rest.
#pragma once

#include "g6_internal.cuh"

namespace g6 {

#define G6_ST(c) st[(size_t)(c) * n + i]
// correct_one's state: column c of the molecule's record at sst[c * sn + si]
// (the state columns, or a copy in registers with sn = 1, si = 0)
#define G6_SS(c) sst[(size_t)(c) * sn + si]

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

// The mixed list kernel's record of molecule i (pkq): fixed-point COM words
// and the float quaternion the offsets were built from.
__device__ __forceinline__ void write_pose_q(float4* pkq, int i, const float w[3], const float q[4]) {
  pkq[2 * (size_t)i] = make_float4(w[0], w[1], w[2], q[0]);
  pkq[2 * (size_t)i + 1] = make_float4(q[1], q[2], q[3], 0.0f);
}

__device__ __forceinline__ void predict_one(double* st, int n, int i) {
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    double d1 = G6_ST(3 + a), d2 = G6_ST(6 + a), d3 = G6_ST(9 + a), d4 = G6_ST(12 + a), d5 = G6_ST(15 + a);
    G6_ST(a) = G6_ST(a) + d1 + d2 + d3 + d4 + d5;
    G6_ST(3 + a) = d1 + 2.0 * d2 + 3.0 * d3 + 4.0 * d4 + 5.0 * d5;
    G6_ST(6 + a) = d2 + 3.0 * d3 + 6.0 * d4 + 10.0 * d5;
    G6_ST(9 + a) = d3 + 4.0 * d4 + 10.0 * d5;
    G6_ST(12 + a) = d4 + 5.0 * d5;
  }
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    double w1 = G6_ST(18 + a), w2 = G6_ST(21 + a), w3 = G6_ST(24 + a), w4 = G6_ST(27 + a), w5 = G6_ST(30 + a);
    G6_ST(18 + a) = w1 + w2 + w3 + w4 + w5;
    G6_ST(21 + a) = w2 + 2.0 * w3 + 3.0 * w4 + 4.0 * w5;
    G6_ST(24 + a) = w3 + 3.0 * w4 + 6.0 * w5;
    G6_ST(27 + a) = w4 + 4.0 * w5;
  }
  double q[4];
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    double q1 = G6_ST(33 + a), q2 = G6_ST(37 + a), q3 = G6_ST(41 + a), q4 = G6_ST(45 + a), q5 = G6_ST(49 + a);
    q[a] = q1 + q2 + q3 + q4 + q5;
    G6_ST(37 + a) = q2 + 2.0 * q3 + 3.0 * q4 + 4.0 * q5;
  }
  double re = 1.0 / sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
#pragma unroll
  for (int a = 0; a < 4; ++a) G6_ST(33 + a) = q[a] * re;
}

// Placement of molecule i (its current com and q in st) into one buffer set.
__device__ __forceinline__ void place_to(const PlaceArgs& a, int i, double* tmat, double* pk64, float4* pk32,
                                         float4* pkq, uint32_t* fix) {
  const int n = a.n;
  const double* st = a.st;
  double q[4] = {G6_ST(33), G6_ST(34), G6_ST(35), G6_ST(36)};
  double t[9];
  setmatrix(q, t);
#pragma unroll
  for (int k = 0; k < 9; ++k) tmat[(size_t)k * n + i] = t[k];
  const int r = a.rep.mol_rep[i];
  const double com[3] = {G6_ST(0), G6_ST(1), G6_ST(2)};
  double* p64 = pk64 + (size_t)i * a.w64;
  p64[0] = com[0]; p64[1] = com[1]; p64[2] = com[2];
  float w[24];
#pragma unroll
  for (int k = 0; k < 24; ++k) w[k] = 0.0f;
  const uint32_t fx = to_fixed(com[0], a.rep.invL[3 * r]);
  const uint32_t fy = to_fixed(com[1], a.rep.invL[3 * r + 1]);
  const uint32_t fz = to_fixed(com[2], a.rep.invL[3 * r + 2]);
  fix[i] = fx; fix[n + i] = fy; fix[2 * n + i] = fz;
  w[0] = __uint_as_float(fx); w[1] = __uint_as_float(fy); w[2] = __uint_as_float(fz);
  for (int s = 0; s <= a.nq; ++s) {   // LJ site then charged sites; the COM site offset is zero
    const double bx = a.body[s][0], by = a.body[s][1], bz = a.body[s][2];
    const double o[3] = {t[0] * bx + t[1] * by + t[2] * bz, t[3] * bx + t[4] * by + t[5] * bz,
                         t[6] * bx + t[7] * by + t[8] * bz};
    for (int k = 0; k < 3; ++k) { p64[3 + 3 * s + k] = o[k]; w[3 + 3 * s + k] = (float)o[k]; }
  }
  for (int k = 3 + 3 * (a.nq + 1); k < a.w64; ++k) p64[k] = 0.0;
  for (int q4 = 0; q4 < a.npk; ++q4)
    pk32[(size_t)i * a.npk + q4] = make_float4(w[4 * q4], w[4 * q4 + 1], w[4 * q4 + 2], w[4 * q4 + 3]);
  if (pkq) {
    const float qf[4] = {(float)q[0], (float)q[1], (float)q[2], (float)q[3]};
    write_pose_q(pkq, i, w, qf);
  }
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

// Buffer set (0 or 1) of the packed poses.
struct PoseBuf {
  double* tmat;
  double* pk64;
  float4* pk32;
  float4* pkq;
  uint32_t* fix;
};
__device__ __forceinline__ PoseBuf pose_buf(const StepArgs& a, int which) {
  PoseBuf b;
  if (which == 0) { b.tmat = a.p.tmat; b.pk64 = a.p.pk64; b.pk32 = a.p.pk32; b.pkq = a.p.pkq; b.fix = a.p.fix; }
  else { b.tmat = a.tmat1; b.pk64 = a.pk64_1; b.pk32 = a.pk32_1; b.pkq = a.pkq_1; b.fix = a.fix1; }
  return b;
}

// rigid_correct + energy/virial/kinetic terms + the next predict and placement
// for molecule i.  F: COM force; tl: lab-frame torque; cur/next: pose buffers.
__device__ __forceinline__ void correct_one(const StepArgs& a, int i, double* sst, int sn, int si, const double F[3],
                                            const double tl[3], double emol, double wtr, double npair_half, int step,
                                            bool predict_next, const PoseBuf& cur, double (&v)[NRED], int& bad) {
  const int n = a.p.n;
  const int r = a.p.rep.mol_rep[i];
  const ThermoDev th = a.th[r];
  const double dt = a.dt;
  // body torque = T^T tau_lab (rigid_collectforce RigidModule.F90:305-310)
  double t[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) t[k] = cur.tmat[(size_t)k * n + i];
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
    nf = nf - G6_SS(3 + c) * ext_t;
    const double delta = nf - G6_SS(6 + c);
    G6_SS(c) = G6_SS(c) + G50 * delta;
    G6_SS(3 + c) = G6_SS(3 + c) + G51 * delta;
    G6_SS(6 + c) = nf;
    G6_SS(9 + c) = G6_SS(9 + c) + G53 * delta;
    G6_SS(12 + c) = G6_SS(12 + c) + G54 * delta;
    G6_SS(15 + c) = G6_SS(15 + c) + G55 * delta;
  }
  // quaternion value
  double q1[4] = {G6_SS(33), G6_SS(34), G6_SS(35), G6_SS(36)};
  double w1[3] = {G6_SS(18), G6_SS(19), G6_SS(20)};
  double nw[4];
  qdot(w1, q1, nw);
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const double dw = nw[c] * dt * 0.5 - G6_SS(37 + c);
    q1[c] = q1[c] + G40 * dw;
    G6_SS(33 + c) = q1[c];
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
    const double delta = nf[c] - G6_SS(21 + c);
    G6_SS(18 + c) = G6_SS(18 + c) + G40 * delta;
    G6_SS(21 + c) = nf[c];
    G6_SS(24 + c) = G6_SS(24 + c) + G42 * delta;
    G6_SS(27 + c) = G6_SS(27 + c) + G43 * delta;
    G6_SS(30 + c) = G6_SS(30 + c) + G44 * delta;
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
      for (int c = 0; c < 3; ++c) G6_SS(3 + c) = z[c] * sv;
      G6_SS(18) = z[3] * sqrt(kT / Ix);
      G6_SS(19) = z[4] * sqrt(kT / Iy);
      G6_SS(20) = z[5] * sqrt(kT / Iz);
    }
  }
  // quaternion derivative stacks from the corrected angular-velocity stack
  double W[5][3], Q[5][4], tq[4], uq[4], vq[4], xq[4];
#pragma unroll
  for (int k = 0; k < 5; ++k)
#pragma unroll
    for (int c = 0; c < 3; ++c) W[k][c] = G6_SS(18 + 3 * k + c);
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
    for (int c = 0; c < 4; ++c) G6_SS(33 + 4 * k + c) = Q[k][c];
  // reductions: Epot, virial trace, kinetic sums (Rigid_Ek), pairs
  const double d1[3] = {G6_SS(3), G6_SS(4), G6_SS(5)};
  v[0] = emol;
  v[1] = wtr;
  v[2] = d1[0] * d1[0] + d1[1] * d1[1] + d1[2] * d1[2];
  v[3] = a.I[0] * (W[0][0] * W[0][0]) + a.I[1] * (W[0][1] * W[0][1]) + a.I[2] * (W[0][2] * W[0][2]);
  v[4] = npair_half;
  if (predict_next) predict_one(sst, sn, si);
}

// After correct_one with the next step predicted and the state in the
// columns: placement into the next pose buffer and the displacement since the
// last list build.
__device__ __forceinline__ void place_next(const StepArgs& a, int i, const PoseBuf& next, double& dmax2, int& bad) {
  const int n = a.p.n;
  const double* st = a.p.st;
  place_to(a.p, i, next.tmat, next.pk64, next.pk32, next.pkq, next.fix);
  const double dx = G6_ST(0) - a.com_build[i], dy = G6_ST(1) - a.com_build[n + i],
               dz = G6_ST(2) - a.com_build[2 * n + i];
  dmax2 = dx * dx + dy * dy + dz * dz;
  if (!isfinite(dmax2)) { bad = 1; dmax2 = 1e300; }
}

// ---------------------------------------------------------------------------
// Mixed precision: the FP64 state holds com, d1, w1 and q; the small Gear
// terms live in the float SoA stf.  Every FP64 instruction here is one the
// update of a FP64 quantity needs (GB300 issues FP64 at 1/64 of the FP32 rate).
// ---------------------------------------------------------------------------
#define G6_SF(c) stf[(size_t)(c) * n + i]

// setmatrix in float with every rounding spelled out (no contraction left to
// the compiler): the placement and the mixed list kernel, which rebuilds a
// neighbour's site offsets from its quaternion, get the same bits.
__device__ __forceinline__ void setmatrix_f(const float q[4], float t[9]) {
  const float qa = q[0], qb = q[1], qc = q[2], qd = q[3];
  const float aa = __fmul_rn(qa, qa), bb = __fmul_rn(qb, qb), cc = __fmul_rn(qc, qc), dd = __fmul_rn(qd, qd);
  t[0] = __fsub_rn(__fadd_rn(aa, bb), __fadd_rn(cc, dd));
  t[1] = __fmul_rn(-2.0f, __fmaf_rn(qa, qd, __fmul_rn(qb, qc)));
  t[2] = __fmul_rn(2.0f, __fmaf_rn(qb, qd, __fmul_rn(-qa, qc)));
  t[3] = __fmul_rn(2.0f, __fmaf_rn(qa, qd, __fmul_rn(-qb, qc)));
  t[4] = __fsub_rn(__fadd_rn(aa, cc), __fadd_rn(bb, dd));
  t[5] = __fmul_rn(-2.0f, __fmaf_rn(qa, qb, __fmul_rn(qc, qd)));
  t[6] = __fmul_rn(2.0f, __fmaf_rn(qa, qc, __fmul_rn(qb, qd)));
  t[7] = __fmul_rn(2.0f, __fmaf_rn(qa, qb, __fmul_rn(-qc, qd)));
  t[8] = __fsub_rn(__fadd_rn(aa, dd), __fadd_rn(bb, cc));
}

// Lab-frame offset t * b of a body-frame site, rounding spelled out.
__device__ __forceinline__ void site_off_f(const float t[9], float bx, float by, float bz, float o[3]) {
  o[0] = __fmaf_rn(t[0], bx, __fmaf_rn(t[1], by, __fmul_rn(t[2], bz)));
  o[1] = __fmaf_rn(t[3], bx, __fmaf_rn(t[4], by, __fmul_rn(t[5], bz)));
  o[2] = __fmaf_rn(t[6], bx, __fmaf_rn(t[7], by, __fmul_rn(t[8], bz)));
}

__device__ __forceinline__ void qdot_f(const float w[3], const float q[4], float o[4]) {
  o[0] = (-w[0] * q[1] + w[1] * q[2] - w[2] * q[3]);
  o[1] = (w[0] * q[0] - w[1] * q[3] - w[2] * q[2]);
  o[2] = (-w[0] * q[3] - w[1] * q[0] + w[2] * q[1]);
  o[3] = (w[0] * q[2] + w[1] * q[1] + w[2] * q[0]);
}

// Uniform in (0, 1] from one Philox output word, and a float normal pair.
__device__ __forceinline__ float uniform_f(uint32_t x) { return ((float)(x >> 8) + 1.0f) * (1.0f / 16777216.0f); }

// Placement into a pose buffer from the FP64 com and (normalised) q:
// fixed-point com (x * 2^32 / L, wrapped), float site offsets, FP64 com.
template <int NQ>
__device__ __forceinline__ void place_mixed(const PlaceArgs& a, int i, const double x[3], const double q[4],
                                            double* pk64, float4* pk32, float4* pkq, uint32_t* fix) {
  constexpr int NPK = ((6 + 3 * NQ) + 3) / 4;
  const int n = a.n;
  const int r = a.rep.mol_rep[i];
  const float qf[4] = {(float)q[0], (float)q[1], (float)q[2], (float)q[3]};
  float t[9];
  setmatrix_f(qf, t);
  float w[24];
#pragma unroll
  for (int k = 0; k < 24; ++k) w[k] = 0.0f;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const uint32_t f = (uint32_t)(unsigned long long)__double2ll_rn(x[k] * (a.rep.invL[3 * r + k] * 4294967296.0));
    fix[(size_t)k * n + i] = f;
    w[k] = __uint_as_float(f);
    pk64[(size_t)i * a.w64 + k] = x[k];
  }
#pragma unroll
  for (int s = 0; s <= NQ; ++s) site_off_f(t, a.fbody[s][0], a.fbody[s][1], a.fbody[s][2], w + 3 + 3 * s);
#pragma unroll
  for (int q4 = 0; q4 < NPK; ++q4)
    pk32[(size_t)i * NPK + q4] = make_float4(w[4 * q4], w[4 * q4 + 1], w[4 * q4 + 2], w[4 * q4 + 3]);
  write_pose_q(pkq, i, w, qf);
}

// rigid_predict (RigidModule.F90:480-559) with the small terms in float.
__device__ __forceinline__ void predict_mixed(double* st, float* stf, int n, int i, double x[3], double q[4]) {
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float d2 = G6_SF(STF_D2 + c), d3 = G6_SF(STF_D2 + 3 + c), d4 = G6_SF(STF_D2 + 6 + c),
                d5 = G6_SF(STF_D2 + 9 + c);
    const double d1 = G6_ST(3 + c);
    x[c] = G6_ST(c) + d1 + (double)(d2 + d3 + d4 + d5);
    G6_ST(c) = x[c];
    G6_ST(3 + c) = d1 + (double)(2.0f * d2 + 3.0f * d3 + 4.0f * d4 + 5.0f * d5);
    G6_SF(STF_D2 + c) = d2 + 3.0f * d3 + 6.0f * d4 + 10.0f * d5;
    G6_SF(STF_D2 + 3 + c) = d3 + 4.0f * d4 + 10.0f * d5;
    G6_SF(STF_D2 + 6 + c) = d4 + 5.0f * d5;
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float w2 = G6_SF(STF_W2 + c), w3 = G6_SF(STF_W2 + 3 + c), w4 = G6_SF(STF_W2 + 6 + c),
                w5 = G6_SF(STF_W2 + 9 + c);
    G6_ST(18 + c) = G6_ST(18 + c) + (double)(w2 + w3 + w4 + w5);
    G6_SF(STF_W2 + c) = w2 + 2.0f * w3 + 3.0f * w4 + 4.0f * w5;
    G6_SF(STF_W2 + 3 + c) = w3 + 3.0f * w4 + 6.0f * w5;
    G6_SF(STF_W2 + 6 + c) = w4 + 4.0f * w5;
  }
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const float q2 = G6_SF(STF_Q2 + c), q3 = G6_SF(STF_Q2 + 4 + c), q4 = G6_SF(STF_Q2 + 8 + c),
                q5 = G6_SF(STF_Q2 + 12 + c);
    q[c] = G6_ST(33 + c) + (double)(q2 + q3 + q4 + q5);
    G6_SF(STF_Q2 + c) = q2 + 2.0f * q3 + 3.0f * q4 + 4.0f * q5;
  }
  // 1/|q|: float estimate, one Newton step in FP64 (|q|^2 = 1 + O(1e-6))
  const double n2 = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
  double re = (double)rsqrtf((float)n2);
  re = re * (1.5 - 0.5 * n2 * re * re);
#pragma unroll
  for (int c = 0; c < 4; ++c) { q[c] *= re; G6_ST(33 + c) = q[c]; }
}

// rigid_correct (RigidModule.F90:1255-1487) followed by the next step's
// rigid_predict (:480-559), with FP64 only for com, d1, w1 and q.  Every FP64
// or conversion instruction costs a warp 64 cycles on GB300, so the float
// increments of the corrector and of the predictor are summed in float and
// each FP64 quantity receives them in one FP64 addition.  F: COM force, tl: lab
// torque (float); outputs the kinetic sums and the displacement test.
// The inputs of correct_mixed that depend neither on the step's forces nor on
// the thermostat (which the pair kernel's first blocks finish): loaded
// together, before the integrator waits for the pair kernel, so that their
// latencies overlap each other and the pair kernel's tail.
struct MixedIn {
  double xd[3], d1d[3], w1d[3], qd[4];   // com, d1, w1, q (FP64 state)
  float sd[12], sw[12], sq[4];           // d2..d5, w2..w5, q2 (float small terms)
  double fixs[3];                        // 2^32 / L of the molecule's replica
  uint32_t fixb[3];                      // fixed-point COM at the last list build
  float fs[3];                           // L / 2^32
  int r;                                 // replica
};

__device__ __forceinline__ void load_mixed(const StepArgs& a, int i, MixedIn& m) {
  const int n = a.p.n;
  const double* st = a.p.st;
  const float* stf = a.stf;
  m.r = a.p.rep.mol_rep[i];
#pragma unroll
  for (int c = 0; c < 3; ++c) { m.xd[c] = G6_ST(c); m.d1d[c] = G6_ST(3 + c); m.w1d[c] = G6_ST(18 + c); }
#pragma unroll
  for (int c = 0; c < 4; ++c) { m.qd[c] = G6_ST(33 + c); m.sq[c] = G6_SF(STF_Q2 + c); }
#pragma unroll
  for (int c = 0; c < 12; ++c) { m.sd[c] = G6_SF(STF_D2 + c); m.sw[c] = G6_SF(STF_W2 + c); }
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    m.fixs[c] = a.fixs[3 * m.r + c];
    m.fixb[c] = a.fix_build[(size_t)c * n + i];
    m.fs[c] = a.p.rep.fscale[3 * m.r + c];
  }
}

template <int NQ>
__device__ __forceinline__ void correct_mixed(const StepArgs& a, int i, const MixedIn& m, const float F[3],
                                              const float tl[3], int step, bool predict_next, const PoseBuf& next,
                                              float& ekt2, float& ekr2, float& dmax2, int& bad) {
  const int n = a.p.n;
  double* st = a.p.st;
  float* stf = a.stf;
  const int r = m.r;
  const ThermoDev& th = a.th[r];
  const int kind = th.kind;
  const float dt = a.fdt;
  double xd[3], d1d[3], w1d[3], qd[4];
#pragma unroll
  for (int c = 0; c < 3; ++c) { xd[c] = m.xd[c]; d1d[c] = m.d1d[c]; w1d[c] = m.w1d[c]; }
#pragma unroll
  for (int c = 0; c < 4; ++c) qd[c] = m.qd[c];
  float d1f[3], w1f[3], qf[4];
#pragma unroll
  for (int c = 0; c < 3; ++c) { d1f[c] = (float)d1d[c]; w1f[c] = (float)w1d[c]; }
#pragma unroll
  for (int c = 0; c < 4; ++c) qf[c] = (float)qd[c];
  float t[9];
  setmatrix_f(qf, t);
  const float tau[3] = {t[0] * tl[0] + t[3] * tl[1] + t[6] * tl[2], t[1] * tl[0] + t[4] * tl[1] + t[7] * tl[2],
                        t[2] * tl[0] + t[5] * tl[1] + t[8] * tl[2]};
  if (!(isfinite(F[0]) && isfinite(F[1]) && isfinite(F[2]) && isfinite(tau[0]) && isfinite(tau[1]) &&
        isfinite(tau[2])))
    bad = 1;
  const float ext_r = kind == G6_NOSE ? th.fext : 0.0f, ext_t = 0.5f * ext_r;
  // COM: Gear-5 corrector (float increments of x and d1)
  float D[4][3], dx_c[3], dd1_c[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float nf = F[c] * a.fcf - d1f[c] * ext_t;
    const float delta = nf - m.sd[c];
    dx_c[c] = (float)G50 * delta;
    dd1_c[c] = (float)G51 * delta;
    D[0][c] = nf;
    D[1][c] = m.sd[3 + c] + (float)G53 * delta;
    D[2][c] = m.sd[6 + c] + (float)G54 * delta;
    D[3][c] = m.sd[9 + c] + (float)G55 * delta;
  }
  // quaternion value
  float nw[4], dq_c[4];
  qdot_f(w1f, qf, nw);
#pragma unroll
  for (int c = 0; c < 4; ++c) dq_c[c] = (float)G40 * (nw[c] * dt * 0.5f - m.sq[c]);
  // angular velocity: Gear-4 with Euler's equations
  const float Ix = a.fI[0], Iy = a.fI[1], Iz = a.fI[2];
  float nfw[3], Wk[4][3], dw1_c[3];
  nfw[0] = (tau[0] + (Iy - Iz) * w1f[1] * w1f[2]) * dt / Ix - w1f[0] * ext_r;
  nfw[1] = (tau[1] + (Iz - Ix) * w1f[2] * w1f[0]) * dt / Iy - w1f[1] * ext_r;
  nfw[2] = (tau[2] + (Ix - Iy) * w1f[0] * w1f[1]) * dt / Iz - w1f[2] * ext_r;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float delta = nfw[c] - m.sw[c];
    dw1_c[c] = (float)G40 * delta;
    Wk[0][c] = nfw[c];
    Wk[1][c] = m.sw[3 + c] + (float)G42 * delta;
    Wk[2][c] = m.sw[6 + c] + (float)G43 * delta;
    Wk[3][c] = m.sw[9 + c] + (float)G44 * delta;
  }
  // corrected d1, w1 in float (kinetic sums, quaternion stacks)
  float d1c[3], w1c[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) { d1c[c] = d1f[c] + dd1_c[c]; w1c[c] = w1f[c] + dw1_c[c]; }
  if (kind == G6_ANDERSEN) {   // stochastic collisions (float draws)
    uint32_t ctr[4] = {(uint32_t)i, (uint32_t)(a.ctrl[6] + step), 0x41u, 0u};
    philox4x32(ctr, (uint32_t)a.seed, (uint32_t)(a.seed >> 32));
    if (uniform_f(ctr[0]) <= th.frdt) {
      const float kT = th.fkT;
      float z[6];
      for (int p = 0; p < 3; ++p) {
        uint32_t g[4] = {(uint32_t)i, (uint32_t)(a.ctrl[6] + step), 0x41u, (uint32_t)(p + 1)};
        philox4x32(g, (uint32_t)a.seed, (uint32_t)(a.seed >> 32));
        const float rr = sqrtf(-2.0f * logf(uniform_f(g[0])));
        float sn, cs;
        sincospif(2.0f * uniform_f(g[1]), &sn, &cs);
        z[2 * p] = rr * sn;
        z[2 * p + 1] = rr * cs;
      }
      const float sv = sqrtf(kT / a.fmass) * dt;
      for (int c = 0; c < 3; ++c) { d1c[c] = z[c] * sv; d1d[c] = 0.0; dd1_c[c] = d1c[c]; }
      w1c[0] = z[3] * sqrtf(kT / Ix);
      w1c[1] = z[4] * sqrtf(kT / Iy);
      w1c[2] = z[5] * sqrtf(kT / Iz);
      for (int c = 0; c < 3; ++c) { w1d[c] = 0.0; dw1_c[c] = w1c[c]; }
    }
  }
  // quaternion stacks from the corrected angular-velocity stack
  float W[5][3], Q[5][4], tq[4], uq[4], vq[4], xq[4];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    W[0][c] = w1c[c];
#pragma unroll
    for (int k = 1; k < 5; ++k) W[k][c] = Wk[k - 1][c];
  }
#pragma unroll
  for (int c = 0; c < 4; ++c) Q[0][c] = qf[c] + dq_c[c];
  qdot_f(W[0], Q[0], tq);
#pragma unroll
  for (int c = 0; c < 4; ++c) Q[1][c] = tq[c] * dt * 0.5f;
  qdot_f(W[1], Q[0], tq); qdot_f(W[0], Q[1], uq);
#pragma unroll
  for (int c = 0; c < 4; ++c) Q[2][c] = (tq[c] + uq[c]) * dt * 0.25f;
  qdot_f(W[2], Q[0], tq); qdot_f(W[0], Q[2], uq); qdot_f(W[1], Q[1], vq);
#pragma unroll
  for (int c = 0; c < 4; ++c) Q[3][c] = (tq[c] + uq[c] + vq[c]) * dt * (1.0f / 6.0f);
  qdot_f(W[3], Q[0], tq); qdot_f(W[2], Q[1], uq); qdot_f(W[1], Q[2], vq); qdot_f(W[0], Q[3], xq);
#pragma unroll
  for (int c = 0; c < 4; ++c) Q[4][c] = (tq[c] + uq[c] + vq[c] + xq[c]) * dt * (1.0f / 8.0f);
  // kinetic sums (Rigid_Ek)
  ekt2 = d1c[0] * d1c[0] + d1c[1] * d1c[1] + d1c[2] * d1c[2];
  ekr2 = Ix * (W[0][0] * W[0][0]) + Iy * (W[0][1] * W[0][1]) + Iz * (W[0][2] * W[0][2]);
  if (!predict_next) {   // last step of a run: the corrected state
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      G6_ST(c) = xd[c] + (double)dx_c[c];
      G6_ST(3 + c) = d1d[c] + (double)dd1_c[c];
      G6_ST(18 + c) = w1d[c] + (double)dw1_c[c];
#pragma unroll
      for (int k = 0; k < 4; ++k) { G6_SF(STF_D2 + 3 * k + c) = D[k][c]; G6_SF(STF_W2 + 3 * k + c) = W[k + 1][c]; }
    }
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      G6_ST(33 + c) = qd[c] + (double)dq_c[c];
#pragma unroll
      for (int k = 1; k < 5; ++k) G6_SF(STF_Q2 + 4 * (k - 1) + c) = Q[k][c];
    }
    return;
  }
  // the next step's prediction, added to the corrected state in one FP64 add each
  double x[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float dsum = D[0][c] + D[1][c] + D[2][c] + D[3][c];
    x[c] = (xd[c] + d1d[c]) + (double)(dx_c[c] + dd1_c[c] + dsum);
    G6_ST(c) = x[c];
    G6_ST(3 + c) = d1d[c] + (double)(dd1_c[c] + 2.0f * D[0][c] + 3.0f * D[1][c] + 4.0f * D[2][c] + 5.0f * D[3][c]);
    G6_SF(STF_D2 + c) = D[0][c] + 3.0f * D[1][c] + 6.0f * D[2][c] + 10.0f * D[3][c];
    G6_SF(STF_D2 + 3 + c) = D[1][c] + 4.0f * D[2][c] + 10.0f * D[3][c];
    G6_SF(STF_D2 + 6 + c) = D[2][c] + 5.0f * D[3][c];
    G6_SF(STF_D2 + 9 + c) = D[3][c];
    G6_ST(18 + c) = w1d[c] + (double)(dw1_c[c] + W[1][c] + W[2][c] + W[3][c] + W[4][c]);
    G6_SF(STF_W2 + c) = W[1][c] + 2.0f * W[2][c] + 3.0f * W[3][c] + 4.0f * W[4][c];
    G6_SF(STF_W2 + 3 + c) = W[2][c] + 3.0f * W[3][c] + 6.0f * W[4][c];
    G6_SF(STF_W2 + 6 + c) = W[3][c] + 4.0f * W[4][c];
    G6_SF(STF_W2 + 9 + c) = W[4][c];
  }
  double q[4];
  float qp[4];
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const float qsum = dq_c[c] + Q[1][c] + Q[2][c] + Q[3][c] + Q[4][c];
    q[c] = qd[c] + (double)qsum;
    qp[c] = qf[c] + qsum;
    G6_SF(STF_Q2 + c) = Q[1][c] + 2.0f * Q[2][c] + 3.0f * Q[3][c] + 4.0f * Q[4][c];
    G6_SF(STF_Q2 + 4 + c) = Q[2][c];
    G6_SF(STF_Q2 + 8 + c) = Q[3][c];
    G6_SF(STF_Q2 + 12 + c) = Q[4][c];
  }
  // 1/|q| = 1 - e/2 + 3e^2/8 for |q|^2 = 1 + e (|e| ~ 1e-6): the small factor in float
  const double e2 = (q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]) - 1.0;
  const float ef = (float)e2;
  const float cfac = ef * (-0.5f + 0.375f * ef);
  const double cd = (double)cfac;
#pragma unroll
  for (int c = 0; c < 4; ++c) { q[c] = q[c] + q[c] * cd; G6_ST(33 + c) = q[c]; qp[c] = qp[c] + qp[c] * cfac; }
  // placement of the predicted pose: fixed-point COM, FP64 COM, float offsets
  constexpr int NPK = ((6 + 3 * NQ) + 3) / 4;
  float tp[9];
  setmatrix_f(qp, tp);
  float w[24];
#pragma unroll
  for (int k = 0; k < 24; ++k) w[k] = 0.0f;
  float dd = 0.0f;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const uint32_t fw = (uint32_t)(unsigned long long)__double2ll_rn(x[c] * m.fixs[c]);
    next.fix[(size_t)c * n + i] = fw;
    w[c] = __uint_as_float(fw);
    next.pk64[(size_t)i * a.p.w64 + c] = x[c];
    const float e = (float)(int)(fw - m.fixb[c]) * m.fs[c];
    dd += e * e;
  }
#pragma unroll
  for (int s = 0; s <= NQ; ++s) site_off_f(tp, a.p.fbody[s][0], a.p.fbody[s][1], a.p.fbody[s][2], w + 3 + 3 * s);
#pragma unroll
  for (int q4 = 0; q4 < NPK; ++q4)
    next.pk32[(size_t)i * NPK + q4] = make_float4(w[4 * q4], w[4 * q4 + 1], w[4 * q4 + 2], w[4 * q4 + 3]);
  write_pose_q(next.pkq, i, w, qp);
  dmax2 = dd;
  if (!isfinite(dd)) { bad = 1; dmax2 = 3.0e38f; }
}


// ---------------------------------------------------------------------------
// Component-parallel corrector (the mixed MD step's k_integrate_quad): four
// lanes per molecule, lane c = lane & 3 owning component c of every vector
// (x, y, z for c < 3; quaternion component c), so a molecule's chain of
// dependent instructions is about a third of correct_mixed's.  The same
// arithmetic per component as correct_mixed; full vectors come from the
// quad's lanes by warp shuffles, and a quaternion product takes the three
// components it needs from the lanes that own them.  Every lane of the warp
// calls it (ok = false for a lane whose molecule does not exist: no stores).
// ---------------------------------------------------------------------------
struct QuadIn {
  double xd, d1d, w1d, qd;   // component c of com, d1, w1 (c < 3) and of q
  float sd[4], sw[4];        // component c of d2..d5 and of w2..w5 (c < 3)
  float sq;                  // component c of q2
  double fixs;               // 2^32 / L on axis c
  uint32_t fixb;             // fixed-point COM word c at the last list build
  float fs;                  // L / 2^32 on axis c
  int r;
};

__device__ __forceinline__ void load_quad(const StepArgs& a, int i, int c, QuadIn& m) {
  const int n = a.p.n;
  const double* st = a.p.st;
  const float* stf = a.stf;
  m.r = a.p.rep.mol_rep[i];
  m.qd = G6_ST(33 + c);
  m.sq = G6_SF(STF_Q2 + c);
  if (c < 3) {
    m.xd = G6_ST(c); m.d1d = G6_ST(3 + c); m.w1d = G6_ST(18 + c);
#pragma unroll
    for (int k = 0; k < 4; ++k) { m.sd[k] = G6_SF(STF_D2 + 3 * k + c); m.sw[k] = G6_SF(STF_W2 + 3 * k + c); }
    m.fixs = a.fixs[3 * m.r + c];
    m.fixb = a.fix_build[(size_t)c * n + i];
    m.fs = a.p.rep.fscale[3 * m.r + c];
  } else {
    m.xd = m.d1d = m.w1d = 0.0;
#pragma unroll
    for (int k = 0; k < 4; ++k) { m.sd[k] = 0.0f; m.sw[k] = 0.0f; }
    m.fixs = 0.0; m.fixb = 0u; m.fs = 0.0f;
  }
}

__device__ __forceinline__ void quad_dummy(int c, QuadIn& m) {
  m.r = 0; m.qd = c == 0 ? 1.0 : 0.0; m.sq = 0.0f; m.xd = m.d1d = m.w1d = 0.0;
#pragma unroll
  for (int k = 0; k < 4; ++k) { m.sd[k] = 0.0f; m.sw[k] = 0.0f; }
  m.fixs = 0.0; m.fixb = 0u; m.fs = 0.0f;
}

// value of lane (quad base | k)
template <class T>
__device__ __forceinline__ T qsh(T v, int k) { return __shfl_sync(0xffffffffu, v, (int)((threadIdx.x & 31) & ~3) | k); }
template <class T>
__device__ __forceinline__ T quad_sum(T v) {
  v += __shfl_xor_sync(0xffffffffu, v, 1);
  v += __shfl_xor_sync(0xffffffffu, v, 2);
  return v;
}
__device__ __forceinline__ float sel3(int c, float a0, float a1, float a2) { return c == 0 ? a0 : (c == 1 ? a1 : a2); }

// The quaternion product of qdot_f, component c: o_c = sum_k s_ck w_k q[c ^ (k + 1)]
// with the signs of qdot_f (negative terms: c = 0: k 0, 2; c = 1: k 1, 2; c = 2: k 0, 1).
struct QuadQ {   // the three components of one quaternion that lane c's products need
  float q0, q1, q2;
  __device__ void load(float own, int c) { q0 = qsh(own, c ^ 1); q1 = qsh(own, c ^ 2); q2 = qsh(own, c ^ 3); }
};
__device__ __forceinline__ float qdot_c(const float w[3], const QuadQ& q, int c) {
  const int b = 3 * c;
  const float s0 = ((0xF5 >> b) & 1) ? -1.0f : 1.0f;
  const float s1 = ((0xF5 >> (b + 1)) & 1) ? -1.0f : 1.0f;
  const float s2 = ((0xF5 >> (b + 2)) & 1) ? -1.0f : 1.0f;
  return (s0 * w[0]) * q.q0 + (s1 * w[1]) * q.q1 + (s2 * w[2]) * q.q2;
}

template <int NQ>
__device__ __forceinline__ void correct_quad(const StepArgs& a, int i, bool ok, int c, const QuadIn& m, float Fc,
                                             const float tl[3], int step, bool predict_next, const PoseBuf& next,
                                             float& ekt2, float& ekr2, float& dmax2, int& bad) {
  const int n = a.p.n;
  double* st = a.p.st;
  float* stf = a.stf;
  const bool v3 = c < 3;   // owns a vector component
  const ThermoDev& th = a.th[m.r];
  const int kind = th.kind;
  const float dt = a.fdt;
  double xd = m.xd, d1d = m.d1d, w1d = m.w1d;
  const double qd = m.qd;
  const float d1f = (float)d1d, w1f = (float)w1d, qf = (float)qd;
  float w[3], q4[4];
#pragma unroll
  for (int k = 0; k < 3; ++k) w[k] = qsh(w1f, k);
#pragma unroll
  for (int k = 0; k < 4; ++k) q4[k] = qsh(qf, k);
  float t[9];
  setmatrix_f(q4, t);
  const float tau = sel3(c, t[0], t[1], t[2]) * tl[0] + sel3(c, t[3], t[4], t[5]) * tl[1] +
                    sel3(c, t[6], t[7], t[8]) * tl[2];
  int bd = (v3 && !(isfinite(Fc) && isfinite(tau))) ? 1 : 0;
  const float ext_r = kind == G6_NOSE ? th.fext : 0.0f, ext_t = 0.5f * ext_r;
  // COM: Gear-5 corrector
  const float nf = Fc * a.fcf - d1f * ext_t;
  const float delta = nf - m.sd[0];
  float dx_c = (float)G50 * delta, dd1_c = (float)G51 * delta;
  const float D0 = nf, D1 = m.sd[1] + (float)G53 * delta, D2 = m.sd[2] + (float)G54 * delta,
              D3 = m.sd[3] + (float)G55 * delta;
  // quaternion value
  QuadQ qq;
  qq.load(qf, c);
  const float nw = qdot_c(w, qq, c);
  const float dq_c = (float)G40 * (nw * dt * 0.5f - m.sq);
  // angular velocity: Gear-4 with Euler's equations (axis c, cyclic c+1, c+2)
  const float I0 = sel3(c, a.fI[0], a.fI[1], a.fI[2]);
  const float I1 = sel3(c, a.fI[1], a.fI[2], a.fI[0]);
  const float I2 = sel3(c, a.fI[2], a.fI[0], a.fI[1]);
  const float wa = sel3(c, w[1], w[2], w[0]), wb = sel3(c, w[2], w[0], w[1]);
  const float nfw = (tau + (I1 - I2) * wa * wb) * dt / I0 - w1f * ext_r;
  const float dlw = nfw - m.sw[0];
  float dw1_c = (float)G40 * dlw;
  const float Wk0 = nfw, Wk1 = m.sw[1] + (float)G42 * dlw, Wk2 = m.sw[2] + (float)G43 * dlw,
              Wk3 = m.sw[3] + (float)G44 * dlw;
  float d1c = d1f + dd1_c, w1c = w1f + dw1_c;
  if (kind == G6_ANDERSEN) {   // stochastic collisions: the quad draws the same numbers
    uint32_t ctr[4] = {(uint32_t)i, (uint32_t)(a.ctrl[6] + step), 0x41u, 0u};
    philox4x32(ctr, (uint32_t)a.seed, (uint32_t)(a.seed >> 32));
    if (uniform_f(ctr[0]) <= th.frdt) {
      const float kT = th.fkT;
      float z[6];
      for (int p = 0; p < 3; ++p) {
        uint32_t g[4] = {(uint32_t)i, (uint32_t)(a.ctrl[6] + step), 0x41u, (uint32_t)(p + 1)};
        philox4x32(g, (uint32_t)a.seed, (uint32_t)(a.seed >> 32));
        const float rr = sqrtf(-2.0f * logf(uniform_f(g[0])));
        float sn, cs;
        sincospif(2.0f * uniform_f(g[1]), &sn, &cs);
        z[2 * p] = rr * sn;
        z[2 * p + 1] = rr * cs;
      }
      const float sv = sqrtf(kT / a.fmass) * dt;
      d1c = sel3(c, z[0], z[1], z[2]) * sv; d1d = 0.0; dd1_c = d1c;
      w1c = sel3(c, z[3], z[4], z[5]) * sqrtf(kT / I0); w1d = 0.0; dw1_c = w1c;
    }
  }
  if (!v3) { d1c = 0.0f; w1c = 0.0f; }
  // quaternion stacks from the corrected angular-velocity stack
  float W0[3], W1[3], W2[3], W3[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) { W0[k] = qsh(w1c, k); W1[k] = qsh(Wk0, k); W2[k] = qsh(Wk1, k); W3[k] = qsh(Wk2, k); }
  const float Q0 = qf + dq_c;
  QuadQ a0, a1, a2, a3;
  a0.load(Q0, c);
  const float Q1 = qdot_c(W0, a0, c) * dt * 0.5f;
  a1.load(Q1, c);
  const float Q2 = (qdot_c(W1, a0, c) + qdot_c(W0, a1, c)) * dt * 0.25f;
  a2.load(Q2, c);
  const float Q3 = (qdot_c(W2, a0, c) + qdot_c(W0, a2, c) + qdot_c(W1, a1, c)) * dt * (1.0f / 6.0f);
  a3.load(Q3, c);
  const float Q4 = (qdot_c(W3, a0, c) + qdot_c(W2, a1, c) + qdot_c(W1, a2, c) + qdot_c(W0, a3, c)) * dt * (1.0f / 8.0f);
  // kinetic sums (Rigid_Ek)
  ekt2 = quad_sum(d1c * d1c);
  ekr2 = quad_sum(I0 * (w1c * w1c));   // w1c is 0 on lane 3
  if (!predict_next) {   // last step of a run: the corrected state
    if (ok) {
      if (v3) {
        G6_ST(c) = xd + (double)dx_c;
        G6_ST(3 + c) = d1d + (double)dd1_c;
        G6_ST(18 + c) = w1d + (double)dw1_c;
        const float Dk[4] = {D0, D1, D2, D3}, Wn[4] = {Wk0, Wk1, Wk2, Wk3};
#pragma unroll
        for (int k = 0; k < 4; ++k) { G6_SF(STF_D2 + 3 * k + c) = Dk[k]; G6_SF(STF_W2 + 3 * k + c) = Wn[k]; }
      }
      G6_ST(33 + c) = qd + (double)dq_c;
      G6_SF(STF_Q2 + c) = Q1; G6_SF(STF_Q2 + 4 + c) = Q2; G6_SF(STF_Q2 + 8 + c) = Q3; G6_SF(STF_Q2 + 12 + c) = Q4;
    }
    if (quad_sum(bd)) bad = 1;
    dmax2 = 0.0f;
    return;
  }
  // the next step's prediction, added to the corrected state in one FP64 add each
  double x = 0.0;
  if (v3) {
    const float dsum = D0 + D1 + D2 + D3;
    x = (xd + d1d) + (double)(dx_c + dd1_c + dsum);
    if (ok) {
      G6_ST(c) = x;
      G6_ST(3 + c) = d1d + (double)(dd1_c + 2.0f * D0 + 3.0f * D1 + 4.0f * D2 + 5.0f * D3);
      G6_SF(STF_D2 + c) = D0 + 3.0f * D1 + 6.0f * D2 + 10.0f * D3;
      G6_SF(STF_D2 + 3 + c) = D1 + 4.0f * D2 + 10.0f * D3;
      G6_SF(STF_D2 + 6 + c) = D2 + 5.0f * D3;
      G6_SF(STF_D2 + 9 + c) = D3;
      G6_ST(18 + c) = w1d + (double)(dw1_c + Wk0 + Wk1 + Wk2 + Wk3);
      G6_SF(STF_W2 + c) = Wk0 + 2.0f * Wk1 + 3.0f * Wk2 + 4.0f * Wk3;
      G6_SF(STF_W2 + 3 + c) = Wk1 + 3.0f * Wk2 + 6.0f * Wk3;
      G6_SF(STF_W2 + 6 + c) = Wk2 + 4.0f * Wk3;
      G6_SF(STF_W2 + 9 + c) = Wk3;
    }
  }
  const float qsum = dq_c + Q1 + Q2 + Q3 + Q4;
  double q = qd + (double)qsum;
  float qp = qf + qsum;
  if (ok) {
    G6_SF(STF_Q2 + c) = Q1 + 2.0f * Q2 + 3.0f * Q3 + 4.0f * Q4;
    G6_SF(STF_Q2 + 4 + c) = Q2;
    G6_SF(STF_Q2 + 8 + c) = Q3;
    G6_SF(STF_Q2 + 12 + c) = Q4;
  }
  // 1/|q| = 1 - e/2 + 3e^2/8 for |q|^2 = 1 + e: the small factor in float
  const double e2 = quad_sum(q * q) - 1.0;
  const float ef = (float)e2;
  const float cfac = ef * (-0.5f + 0.375f * ef);
  const double cd = (double)cfac;
  q = q + q * cd;
  qp = qp + qp * cfac;
  if (ok) G6_ST(33 + c) = q;
  // placement of the predicted pose: fixed-point COM, FP64 COM, float offsets, the pose record
  constexpr int NPK = ((6 + 3 * NQ) + 3) / 4;
  float qv[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) qv[k] = qsh(qp, k);
  float tp[9];
  setmatrix_f(qv, tp);
  float e = 0.0f;
  uint32_t fw = 0u;
  if (v3) {
    fw = (uint32_t)(unsigned long long)__double2ll_rn(x * m.fixs);
    e = (float)(int)(fw - m.fixb) * m.fs;
  }
  const float dd = quad_sum(e * e);
  if (ok) {
    float* pf = reinterpret_cast<float*>(next.pk32) + (size_t)i * 4 * NPK;
    float* qf8 = reinterpret_cast<float*>(next.pkq) + 8 * (size_t)i;
    if (v3) {
      next.fix[(size_t)c * n + i] = fw;
      next.pk64[(size_t)i * a.p.w64 + c] = x;
      pf[c] = __uint_as_float(fw);
      qf8[c] = __uint_as_float(fw);
    }
    qf8[3 + c] = qp;
    if (c == 3) qf8[7] = 0.0f;
    // site c (and, with 4 charged sites, site 4 on lane 0)
    if (c <= NQ) {
      float o[3];
      site_off_f(tp, a.p.fbody[c][0], a.p.fbody[c][1], a.p.fbody[c][2], o);
#pragma unroll
      for (int k = 0; k < 3; ++k) pf[3 + 3 * c + k] = o[k];
    }
    if (NQ == 4 && c == 0) {
      float o[3];
      site_off_f(tp, a.p.fbody[4][0], a.p.fbody[4][1], a.p.fbody[4][2], o);
#pragma unroll
      for (int k = 0; k < 3; ++k) pf[15 + k] = o[k];
    }
    if (c == 3)
      for (int k = 3 + 3 * (NQ + 1); k < 4 * NPK; ++k) pf[k] = 0.0f;
  }
  dmax2 = dd;
  const int anybad = quad_sum(bd);
  if (anybad) bad = 1;
  if (!isfinite(dd)) { bad = 1; dmax2 = 3.0e38f; }
}

#undef G6_SF

// ---------------------------------------------------------------------------
// Per-step reductions.  Warp 0 of each block holds one molecule per lane; it
// sums the NRED quantities per replica slot (FP64 in the plain path, float
// pairs with error-free addition in the mixed path), writes the block
// partials, and the last block to arrive sums the partials in a fixed order.
// ---------------------------------------------------------------------------
struct FF {
  float hi, lo;
};
__device__ __forceinline__ FF ff_add(FF a, FF b) {
  const float s = a.hi + b.hi;
  const float bp = s - a.hi;
  const float e = (a.hi - (s - bp)) + (b.hi - bp);
  const float t = e + (a.lo + b.lo);
  const float h = s + t;
  return FF{h, t - (h - s)};
}
__device__ __forceinline__ FF red_zero(FF) { return FF{0.0f, 0.0f}; }
__device__ __forceinline__ double red_zero(double) { return 0.0; }
__device__ __forceinline__ FF red_add(FF a, FF b) { return ff_add(a, b); }
__device__ __forceinline__ double red_add(double a, double b) { return a + b; }
__device__ __forceinline__ FF red_shfl(FF v, int m) {
  return FF{__shfl_xor_sync(0xffffffffu, v.hi, m), __shfl_xor_sync(0xffffffffu, v.lo, m)};
}
__device__ __forceinline__ double red_shfl(double v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }
__device__ __forceinline__ double red_double(FF v) { return (double)v.hi + (double)v.lo; }
__device__ __forceinline__ double red_double(double v) { return v; }

// Reductions, thermostat and log of replica rr for the step (block-wide; run
// by the last block of the replica to finish): the replica's block partials
// summed in a fixed order, T, P and the conserved quantity
// (Mixture.F90:2251-2264, 2431-2453), Nose_Correct and the next Nose_Predict
// (NoseModule.F90:43-87).
__device__ inline void finish_replica(const StepArgs& a, int rr, int mpb, int step, int rebuilt) {
  __shared__ double wsum[32][NRED];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = (blockDim.x + 31) >> 5;
  const int b0 = a.p.rep.off[rr] / mpb, b1 = (a.p.rep.off[rr + 1] - 1) / mpb;
  const int slot0 = rr - a.p.rep.mol_rep[b0 * mpb];   // later blocks start inside replica rr
  double sum[NRED];
#pragma unroll
  for (int k = 0; k < NRED; ++k) sum[k] = 0.0;
#pragma unroll 4
  for (int b = b0 + (int)threadIdx.x; b <= b1; b += blockDim.x) {
    const double* src = a.part + ((size_t)b * MAXREP_PER_BLOCK + (b == b0 ? slot0 : 0)) * NRED;
#pragma unroll
    for (int k = 0; k < NRED; ++k) sum[k] += __ldcg(src + k);
  }
#pragma unroll
  for (int k = 0; k < NRED; ++k) {
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) sum[k] += __shfl_xor_sync(0xffffffffu, sum[k], m);
    if (lane == 0) wsum[warp][k] = sum[k];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double s[NRED];
#pragma unroll
    for (int k = 0; k < NRED; ++k) {
      double x = 0.0;
      for (int w = 0; w < nwarp; ++w) x += wsum[w][k];
      s[k] = x;
      a.red[(size_t)rr * NRED + k] = x;
    }
    const bool predict_next = step + 1 < a.ctrl[2];
    ThermoDev& th = a.th[rr];
    const double dt = a.dt;
    const int nm = a.p.rep.off[rr + 1] - a.p.rep.off[rr];
    const double dof = 6.0 * nm;
    const double ekt = s[2] * a.mass * 0.5 * a.inv_dt2;
    const double ekr = s[3] * 0.5;
    const double temperature = (ekt + ekr) * a.rfac[2 * rr];
    const double pkin = s[2] * a.mass * a.inv_dt2;
    const double pressure = (pkin + s[1]) * a.rfac[2 * rr + 1];
    if (th.kind == G6_NOSE) {   // Nose_Correct
      const double zetaf = (temperature - th.temp) * th.inv_q - th.dump * th.z[0];
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
    if (a.log && step < a.ctrl[5]) {
      double* lg = a.log + ((size_t)step * a.p.rep.nrep + rr) * G6_LOG_WIDTH;
      lg[0] = s[0]; lg[1] = ekt; lg[2] = ekr; lg[3] = temperature; lg[4] = pressure;
      lg[5] = (s[0] + ekt + ekr) * I2J + nose_ep + nose_ek;
      lg[6] = s[4]; lg[7] = th.z[0]; lg[8] = (double)rebuilt; lg[9] = (double)step;
    }
    if (predict_next && th.kind == G6_NOSE) {   // Nose_Predict for the next step
      th.z[0] = th.z[0] + th.z[1] + th.z[2] + th.z[3] + th.z[4];
      th.z[1] = th.z[1] + 2.0 * th.z[2] + 3.0 * th.z[3] + 4.0 * th.z[4];
      th.z[2] = th.z[2] + 3.0 * th.z[3] + 6.0 * th.z[4];
      th.z[3] = th.z[3] + 4.0 * th.z[4];
      th.fext = (float)(th.z[0] * dt);
    }
  }
  __syncthreads();
}

// Block partials of the step (warp ew holds one molecule per lane): per replica
// slot, sums over the lanes (FP64 in the plain path, float pairs with error-free
// addition in the mixed path); the largest displacement goes to an atomic max
// word.  The last block of each replica to arrive finishes that replica
// (finish_replica); the last block overall advances the step counter.
// The last block of step `step` (every block's displacement maximum is in
// gmax[step & 1]): the next step's list decision for its head, ctrl[0] = 1
// when some molecule has moved more than half the skin since the last build,
// and the word the next step's blocks raise reset to 0.
__device__ __forceinline__ void next_step_decision(const StepArgs& a, int step) {
  __threadfence();
  const double gm = (double)__uint_as_float(__ldcg(&a.gmax[step & 1]));
  a.ctrl[0] = (step + 1 < a.ctrl[2] && gm > a.half_skin2) ? 1 : 0;
  a.gmax[(step + 1) & 1] = 0u;
}

template <class V>
__device__ void step_reduce(const StepArgs& a, const V (&v)[NRED], int r, float dmax2, int bad, int mpb, int step,
                            int ew) {
  const int n = a.p.n;
  __shared__ int s_rfirst, s_nslots;
  __shared__ int s_last[MAXREP_PER_BLOCK];
  if ((int)(threadIdx.x >> 5) == ew) {
    const int lane = threadIdx.x & 31;
    const int first_i = blockIdx.x * mpb;
    const int last_i = min(n, first_i + mpb) - 1;
    const int rfirst = a.p.rep.mol_rep[first_i];
    const int nslots = a.p.rep.mol_rep[last_i] - rfirst + 1;
    for (int s = 0; s < nslots; ++s) {
      const bool mine = (r == rfirst + s);
#pragma unroll
      for (int k = 0; k < NRED; ++k) {
        V x = mine ? v[k] : red_zero(v[k]);
#pragma unroll
        for (int m = 16; m >= 1; m >>= 1) x = red_add(x, red_shfl(x, m));
        if (lane == 0) a.part[((size_t)blockIdx.x * MAXREP_PER_BLOCK + s) * NRED + k] = red_double(x);
      }
    }
    float m = dmax2;
    int b = bad;
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
      m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
      b |= __shfl_xor_sync(0xffffffffu, b, o);
    }
    if (lane == 0) {
      // non-negative floats order like their bit patterns: an exact, order-free maximum
      if (m > 0.0f) atomicMax(&a.gmax[step & 1], __float_as_uint(m));
      if (b) atomicOr(&a.ctrl[3], 1);
      s_rfirst = rfirst;
      s_nslots = nslots;
    }
  }
  // publish the partials, then count the block in for each of its replicas
  __threadfence();
  __syncthreads();
  if ((int)threadIdx.x < s_nslots) {
    const int rr = s_rfirst + threadIdx.x;
    const int nb = (a.p.rep.off[rr + 1] - 1) / mpb - a.p.rep.off[rr] / mpb + 1;
    s_last[threadIdx.x] = atomicAdd(&a.repcnt[rr], 1) == nb - 1;
  }
  __syncthreads();
  for (int sl = 0; sl < s_nslots; ++sl) {
    if (!s_last[sl]) continue;
    __threadfence();
    finish_replica(a, s_rfirst + sl, mpb, step, a.ctrl[0]);
    if (threadIdx.x == 0) a.repcnt[s_rfirst + sl] = 0;
  }
  // (every block has read ctrl[0] and ctrl[1] before it arrives at the counter)
  if (threadIdx.x == 0 && atomicAdd(a.done, 1u) == gridDim.x - 1) {
    next_step_decision(a, step);
    a.ctrl[1] = step + 1;
    a.ctrl[4] = 1;
    *a.done = 0u;
  }
}

// Mixed MD step: the block partials of step_reduce without the replica finish,
// which runs in the next kernel (finish_pending): per replica slot the sums
// over the block's molecules (warp ew holds one per lane), the displacement
// maximum and the error flag; the last block overall keeps the step's rebuild
// flag for the log (ctrl[7]) and advances the step counter.
template <class V>
__device__ void step_partials(const StepArgs& a, const V (&v)[NRED], int r, float dmax2, int bad, int mpb, int step,
                              int ew) {
  const int n = a.p.n;
  if ((int)(threadIdx.x >> 5) == ew) {
    const int lane = threadIdx.x & 31;
    const int first_i = blockIdx.x * mpb;
    const int last_i = min(n, first_i + mpb) - 1;
    const int rfirst = a.p.rep.mol_rep[first_i];
    const int nslots = a.p.rep.mol_rep[last_i] - rfirst + 1;
    for (int s = 0; s < nslots; ++s) {
      const bool mine = (r == rfirst + s);
#pragma unroll
      for (int k = 0; k < NRED; ++k) {
        V x = mine ? v[k] : red_zero(v[k]);
#pragma unroll
        for (int m = 16; m >= 1; m >>= 1) x = red_add(x, red_shfl(x, m));
        if (lane == 0) a.part[((size_t)blockIdx.x * MAXREP_PER_BLOCK + s) * NRED + k] = red_double(x);
      }
    }
    float m = dmax2;
    int b = bad;
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
      m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
      b |= __shfl_xor_sync(0xffffffffu, b, o);
    }
    if (lane == 0) {
      if (m > 0.0f) atomicMax(&a.gmax[step & 1], __float_as_uint(m));
      if (b) atomicOr(&a.ctrl[3], 1);
    }
  }
  __syncthreads();
  // (every block has read ctrl[0] and ctrl[1] before it arrives at the counter;
  // its displacement maximum is published before it does)
  if (threadIdx.x == 0) __threadfence();
  if (threadIdx.x == 0 && atomicAdd(a.done, 1u) == gridDim.x - 1) {
    a.ctrl[7] = a.ctrl[0];
    next_step_decision(a, step);
    a.ctrl[1] = step + 1;
    a.ctrl[4] = 1;
    *a.done = 0u;
  }
}

// The deferred replica finish of the mixed MD step (block-wide, one replica
// per block): sums, thermostat, log and the next Nose_Predict of step
// ctrl[1]-1, from the partials its integrator kernel wrote.  Runs in the next
// step's pair kernel, overlapped with its pair work, or after the last step.
__device__ inline void finish_pending(const StepArgs& a, int rr, int mpb) {
  if (!a.ctrl[4]) return;   // no step of this run has finished yet
  finish_replica(a, rr, mpb, a.ctrl[1] - 1, a.ctrl[7]);
}

#undef G6_ST
#undef G6_SS

}  // namespace g6
