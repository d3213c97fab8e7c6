// g6_mctrial.cuh -- pieces of a Monte Carlo trial shared by the chain kernels
// (g6_mc.cu: plain, learned-width and record-collecting chains; g6_opmc.cu:
// umbrella chains on an order parameter): the trial pair energy
// (PairPotential), the trial rotation (qinfrotator + qadd), the feature terms
// of the learned proposal, the pose readers and the warp-cooperative build of
// one trial's proposal (mc2.F90:544-620).
#pragma once

#include <cuda_runtime.h>

#include "g6_internal.cuh"
#include "g6_mlp.cuh"

namespace g6 {
constexpr int MC_NT = 512;            // threads per chain
constexpr int MC_NB = 128;            // trials per batch of pre-computed draws
constexpr float FEAT_Q = 1048576.0f;  // feature terms are integers of 2^-20
constexpr float FEAT_IQ = 1.0f / 1048576.0f;
constexpr float FEAT_RC2 = 6.0f * 6.0f;
constexpr int MC_SEG = 96;            // molecules within rc kept per energy warp and trial
constexpr int MC_POOL = 64;           // feature neighbours kept per pose (about 31 in liquid water)

template <int NQ, bool TAPER, class R>
__device__ __forceinline__ R pair_energy(const R d[3], R dd, const R (&ri)[NQ + 1][3], const R (&rj)[NQ + 1][3],
                                         const PairConst& pc, R rin2, R rin, R rout, R c1) {
  R hh;
  if (dd > rin2) {
    R r, ir;
    root_r(dd, r, ir);
    R u = r - rout, l = r - rin, uu = u * u, ll = l * l;
    hh = c1 * uu * u * (R(10) * ll - R(5) * u * l + uu);
  } else {
    hh = R(1);
  }
  R v[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) v[k] = d[k] + ri[0][k] - rj[0][k];
  const R inv = rcp_r(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
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
      ec += q * rsqrt_r(x * x + y * y + z * z);
    }
  R scc = hh;
  if (TAPER) {
    const R rl = sizeof(R) == 8 ? (R)pc.rl : (R)pc.frl, ru = sizeof(R) == 8 ? (R)pc.ru : (R)pc.fru;
    const R w3 = sizeof(R) == 8 ? (R)pc.w3 : (R)pc.fw3;
    R s12;
    if (dd < ru * ru) {
      if (dd < rl * rl) s12 = R(0);
      else {
        R r12, ir12;
        root_r(dd, r12, ir12);
        s12 = (r12 - rl) * (r12 - rl) * (R(3) * ru - rl - R(2) * r12) / w3;
      }
    } else {
      s12 = R(1);
    }
    scc = hh * s12;
  }
  return hh * elj + scc * ec;
}

// QuatModule.F90:108-133: a1 <- a1 (x) a2, then the sign with a >= 0.
template <class R>
__device__ __forceinline__ void qadd(R q1[4], const R q2[4]) {
  const R a1 = q1[0], b1 = q1[1], c1 = q1[2], d1 = q1[3];
  const R a2 = q2[0], b2 = q2[1], c2 = q2[2], d2 = q2[3];
  R a3 = a1 * a2 - b1 * b2 - c1 * c2 - d1 * d2;
  R b3 = a1 * b2 + b1 * a2 + c1 * d2 - d1 * c2;
  R c3 = a1 * c2 + c1 * a2 - b1 * d2 + d1 * b2;
  R d3 = a1 * d2 + d1 * a2 + b1 * c2 - c1 * b2;
  if (a3 < R(0)) { a3 = -a3; b3 = -b3; c3 = -c3; d3 = -d3; }
  q1[0] = a3; q1[1] = b3; q1[2] = c3; q1[3] = d3;
}

// qinfrotator (QuatModule.F90:203-223) composed with the old orientation, the
// rotation matrix of rigid_setmatrix and the lab offsets of sites 0..NQ.
template <class R, int NQ, class B>
__device__ __forceinline__ void trial_rotation(const R rot[3], const R* qold, const B (&body)[MAXSITE][3],
                                               R qn[4], R (&off)[NQ + 1][3]) {
  R qr[4] = {R(1), rot[0], rot[1], rot[2]};
  const R nn = qr[0] * qr[0] + qr[1] * qr[1] + qr[2] * qr[2] + qr[3] * qr[3];
  R rn;
  if constexpr (sizeof(R) == 4) rn = rsqrtf(nn);   // FP32 trial poses: the hardware reciprocal square root
  else rn = R(1) / sqrt(nn);
#pragma unroll
  for (int k = 0; k < 4; ++k) qr[k] *= rn;
  R qo[4] = {qold[0], qold[1], qold[2], qold[3]};
  qadd(qr, qo);
  const R qa = qr[0], qb = qr[1], qc = qr[2], qd = qr[3];
  R tm[9];
  tm[0] = (qa * qa + qb * qb - (qc * qc + qd * qd)); tm[1] = -R(2) * (qa * qd + qb * qc);
  tm[2] = R(2) * (qb * qd - qa * qc); tm[3] = R(2) * (qa * qd - qb * qc);
  tm[4] = qa * qa + qc * qc - (qb * qb + qd * qd); tm[5] = -R(2) * (qa * qb + qc * qd);
  tm[6] = R(2) * (qa * qc + qb * qd); tm[7] = R(2) * (qa * qb - qc * qd);
  tm[8] = qa * qa + qd * qd - (qb * qb + qc * qc);
#pragma unroll
  for (int k = 0; k < 4; ++k) qn[k] = qr[k];
#pragma unroll
  for (int s = 0; s <= NQ; ++s) {
    const R bx = (R)body[s][0], by = (R)body[s][1], bz = (R)body[s][2];
    off[s][0] = tm[0] * bx + tm[1] * by + tm[2] * bz;
    off[s][1] = tm[3] * bx + tm[4] * by + tm[5] * bz;
    off[s][2] = tm[6] * bx + tm[7] * by + tm[8] * bz;
  }
}

// ---------------------------------------------------------------------------
// Features with correctly rounded single operations only (no contraction), so
// the same pair gives the same integer terms at every call site.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float dot3_rn(const float a[3], const float b[3]) {
  return __fadd_rn(__fadd_rn(__fmul_rn(a[0], b[0]), __fmul_rn(a[1], b[1])), __fmul_rn(a[2], b[2]));
}
// exp(-t^2) with the single hardware base-2 exponential (PTX ex2.approx.ftz:
// results below 2^-126 flush to zero, far below the 2^-20 quantum of a term)
__device__ __forceinline__ float gauss_rn(float t) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(__fmul_rn(-__fmul_rn(t, t), 1.44269504f)));
  return y;
}
// Nearest integer (ties to even, as __float2int_rn) of the term in units of
// 2^-20 by the 1.5 * 2^23 bit pattern (exact below 2^22; terms are in [0, 1]):
// a float-to-int conversion issues on the FP64 pipe of this GPU.
__device__ __forceinline__ int feat_q(float x) {
  return __float_as_int(__fadd_rn(__fmul_rn(x, FEAT_Q), 12582912.0f)) - 0x4B400000;
}

// Unit direction of one site offset v.  rsqrtf is a fixed function of its
// argument, so every call site gets the same bits for the same v.
__device__ __forceinline__ void site_dir1(const float v[3], float u[3]) {
  const float inv = rsqrtf(dot3_rn(v, v));
#pragma unroll
  for (int k = 0; k < 3; ++k) u[k] = __fmul_rn(v[k], inv);
}

// Unit directions of the charged sites 1..NQ from their offsets o[(NQ+1)*3].
template <int NQ>
__device__ __forceinline__ void site_dirs(const float* o, float (&u)[4][3]) {
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    if (s < NQ) {
      const float v[3] = {o[3 * (s + 1)], o[3 * (s + 1) + 1], o[3 * (s + 1) + 2]};
      site_dir1(v, u[s]);
    } else {
      u[s][0] = u[s][1] = u[s][2] = 0.0f;
    }
  }
}

// The single terms of one neighbour at distance r (1/r = ir) along e.  Every
// call site builds a term from these helpers, so a pair gives the same integer
// whichever molecule of the pair is being updated.
__device__ __forceinline__ void feat_r(float r2, float& r, float& ir) {
  ir = rsqrtf(r2);
  r = __fmul_rn(r2, ir);
}
template <int K>
__device__ __forceinline__ int feat_radial(float r) {
  return feat_q(gauss_rn(__fmul_rn(__fsub_rn(r, 2.4f + 0.225f * K), 4.0f)));
}
__device__ __forceinline__ float feat_g1(float r) { return gauss_rn(__fmul_rn(__fsub_rn(r, 2.9f), 1.0f / 0.35f)); }
__device__ __forceinline__ float feat_g2(float r) { return gauss_rn(__fmul_rn(__fsub_rn(r, 4.5f), 2.0f)); }
__device__ __forceinline__ float feat_c4(const float u[3], const float e[3], float ir) {
  const float c = fmaxf(__fmul_rn(dot3_rn(u, e), ir), 0.0f);
  const float c2 = __fmul_rn(c, c);
  return __fmul_rn(c2, c2);
}
template <int K0, int NK>
__device__ __forceinline__ void feat_radials(float r, int sign, int (&f)[MLP_IN]) {
  if constexpr (NK > 0) {
    f[K0] += sign * feat_radial<K0>(r);
    feat_radials<K0 + 1, NK - 1>(r, sign, f);
  }
}

// Integer feature terms of one neighbour at e (molecule -> neighbour, |e|^2 = r2).
__device__ __forceinline__ void feat_terms(const float e[3], float r2, const float (&u)[4][3], int sign,
                                           int (&f)[MLP_IN]) {
  float r, ir;
  feat_r(r2, r, ir);
  feat_radials<0, 16>(r, sign, f);
  const float g1 = feat_g1(r), g2 = feat_g2(r);
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    const float c4 = feat_c4(u[s], e, ir);
    f[16 + s] += sign * feat_q(__fmul_rn(g1, c4));
    f[20 + s] += sign * feat_q(__fmul_rn(g2, c4));
  }
}

// A quarter of the terms of one neighbour: part 0 and 1 the radial shells 0-7
// and 8-15, part 2 and 3 the direction terms of charged sites 0-1 and 2-3 (u =
// the molecule's 12 site-direction floats).  v[q] is the term of feature
// part_index(part, q); parts 2 and 3 fill v[0..3].
__device__ __forceinline__ int part_index(int part, int q) {
  return part < 2 ? 8 * part + q : 16 + 4 * (q >> 1) + 2 * (part - 2) + (q & 1);
}
__device__ __forceinline__ void feat_part(int part, const float e[3], float r2, const float* u, int (&v)[8]) {
  float r, ir;
  feat_r(r2, r, ir);
  int f[MLP_IN];
#pragma unroll
  for (int k = 0; k < MLP_IN; ++k) f[k] = 0;
  if (part == 0) {
    feat_radials<0, 8>(r, 1, f);
#pragma unroll
    for (int q = 0; q < 8; ++q) v[q] = f[q];
  } else if (part == 1) {
    feat_radials<8, 8>(r, 1, f);
#pragma unroll
    for (int q = 0; q < 8; ++q) v[q] = f[8 + q];
  } else {
    const float g1 = feat_g1(r), g2 = feat_g2(r);
    const int s0 = 2 * (part - 2);
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const float us[3] = {u[3 * (s0 + q)], u[3 * (s0 + q) + 1], u[3 * (s0 + q) + 2]};
      const float c4 = feat_c4(us, e, ir);
      v[q] = feat_q(__fmul_rn(g1, c4));
      v[2 + q] = feat_q(__fmul_rn(g2, c4));
    }
#pragma unroll
    for (int q = 4; q < 8; ++q) v[q] = 0;
  }
}

// One feature neighbour of a trial pose as an energy warp keeps it: the
// neighbour's site directions (copied asynchronously), the separation
// neighbour -> target pose, the neighbour, and the neighbour's own terms of the
// pair, added to (new pose) or subtracted from (old pose) its cache row when
// the move is accepted.  160 bytes, so that u stays 16-byte aligned.
struct FeEntry {
  float u[12];
  float e[3];
  int j;
  int d[MLP_IN];
};

// Separation a -> b of two molecules: fixed-point COMs (mixed) or the FP64
// minimum image (plain), as float.
__device__ __forceinline__ float fvec_fix(const uint32_t a[3], const uint32_t b[3], const float fs[3], float e[3]) {
#pragma unroll
  for (int k = 0; k < 3; ++k) e[k] = __fmul_rn((float)(int)(b[k] - a[k]), fs[k]);
  return dot3_rn(e, e);
}
__device__ __forceinline__ float fvec_64(const double a[3], const double b[3], const double L[3], const double iL[3],
                                         float e[3]) {
  double o[3], d[3];
  exact_dd(b, a, L, iL, o, d);
#pragma unroll
  for (int k = 0; k < 3; ++k) e[k] = (float)d[k];
  return dot3_rn(e, e);
}

template <int NQ, bool MIXED>
struct PoseRead {
  static constexpr int W64 = ((6 + 3 * NQ) + 1) / 2 * 2;
  static constexpr int NPK = ((6 + 3 * NQ) + 3) / 4;
  // float offsets of sites 0..NQ of molecule j as the trial energies see them
  __device__ static void offsets(const McArgs& a, int j, float (&o)[(NQ + 1) * 3]) {
#pragma unroll
    for (int k = 0; k < (NQ + 1) * 3; ++k)
      o[k] = MIXED ? a.pk32f[(size_t)j * 4 * NPK + 3 + k] : (float)a.pk64[(size_t)j * W64 + 3 + k];
  }
  __device__ static void fix(const McArgs& a, int j, uint32_t (&f)[3]) {
    f[0] = a.fix[j]; f[1] = a.fix[a.n + j]; f[2] = a.fix[2 * a.n + j];
  }
  __device__ static void com(const McArgs& a, int j, double (&c)[3]) {
    const double* p = a.pk64 + (size_t)j * W64;
    c[0] = p[0]; c[1] = p[1]; c[2] = p[2];
  }
};

// The proposal density of a move (isotropic Gaussians in the translation and
// in the rotation vector) as three numbers of its widths, so that the log of
// the density, -3 ln st - 3 ln sr - d2/(2 st^2) - r2/(2 sr^2), is
// lq - d2 * it - r2 * ir.
struct QForm {
  float lq, it, ir;
};
__device__ __forceinline__ QForm q_form(float st, float sr) {
  return QForm{-3.0f * (__logf(st) + __logf(sr)), 0.5f / (st * st), 0.5f / (sr * sr)};
}

// One trial's proposal: widths, draws, the trial pose of the target and its
// current pose.  Built by one whole warp; two of them alternate so that the
// next trial's pose is built while the current trial's energies are summed.
template <class R, int NQ>
struct TrialPose {
  R on[NQ + 1][3], oo[NQ + 1][3];   // new / old site offsets
  double cn[3], co[3];              // new / old FP64 COM
  R rot[3], dx[3];                  // rotation vector and translation
  QForm qf;                         // proposal density form of the widths at the old pose
  R qn[4];                          // trial quaternion (the pose's precision)
  double qo64[4];                   // FP64 quaternion before the move
  double q64[4];                    // FP64 quaternion after the move
  uint32_t fn[3], fo[3];            // new / old fixed-point COM
  float un[4][3];                   // charged-site directions at the new pose
  float d2, r2;                     // |dx|^2, |rot|^2
  int trial;                        // trial number the pose belongs to (-1: none)
};

// FP64 quaternion of an accepted mixed-precision trial, component `lane` on
// lanes 0-3 (all lanes call): qadd of QuatModule.F90:108-133 applied to the
// FP64 quaternion as a float increment (qinfrotator(rot) - identity) (x) q_old,
// with 1/sqrt(1+s) - 1 written without cancellation as
// -s / (sqrt(1+s) (1 + sqrt(1+s))); then the sign with a >= 0 and |q| = 1
// restored by the factor 1 - e/2 + 3e^2/8.
template <class TP>
__device__ __forceinline__ double accepted_q64(const TP& P, int lane) {
  const double qv = lane < 4 ? P.qo64[lane & 3] : 0.0;
  const float qf = (float)qv;
  const float of0 = __shfl_sync(0xffffffffu, qf, 0), of1 = __shfl_sync(0xffffffffu, qf, 1);
  const float of2 = __shfl_sync(0xffffffffu, qf, 2), of3 = __shfl_sync(0xffffffffu, qf, 3);
  const float r0 = (float)P.rot[0], r1 = (float)P.rot[1], r2 = (float)P.rot[2];
  const float s2 = r0 * r0 + r1 * r1 + r2 * r2, rs = sqrtf(1.0f + s2), inv = 1.0f / rs;
  const float m0 = -s2 / (rs * (1.0f + rs)), b1 = r0 * inv, c1 = r1 * inv, d1 = r2 * inv;
  const float dq0 = m0 * of0 - b1 * of1 - c1 * of2 - d1 * of3;
  const float dq1 = m0 * of1 + b1 * of0 + c1 * of3 - d1 * of2;
  const float dq2 = m0 * of2 + c1 * of0 - b1 * of3 + d1 * of1;
  const float dq3 = m0 * of3 + d1 * of0 + b1 * of2 - c1 * of1;
  const float dq = lane == 0 ? dq0 : (lane == 1 ? dq1 : (lane == 2 ? dq2 : dq3));
  double q64 = qv + (double)dq;
  if (of0 + dq0 < 0.0f) q64 = -q64;
  double sq = lane < 4 ? q64 * q64 : 0.0;
  sq += __shfl_xor_sync(0xffffffffu, sq, 1);
  sq += __shfl_xor_sync(0xffffffffu, sq, 2);
  const float ef = (float)(sq - 1.0);
  return q64 + q64 * (double)(ef * (-0.5f + 0.375f * ef));
}

// Warp-cooperative build of trial `trial` (target tg, unit normals g[0..5][slot],
// widths st_w, sr_w).  Register arrays are indexed with constants only
// (selects), never by lane.  Mixed precision builds the pose in FP32 with no
// FP64 arithmetic but the trial COM and, with Q64, the FP64 quaternion an
// acceptance would write (accepted_q64); the FP64 mode follows mc2's serial formulas in
// FP64, component k on lane k, since an FP64 warp instruction costs the same
// whatever the number of active lanes.
template <class R, int NQ, bool MIXED, bool Q64>
__device__ __noinline__ void build_trial(const McArgs& a, TrialPose<R, NQ>& P, int trial, int tg, const R (*g)[MC_NB], int slot,
                            R st_w, R sr_w, const double iL[3], const float fsi[3]) {
  using Pr = PoseRead<NQ, MIXED>;
  const int lane = threadIdx.x & 31;
  const int n = a.n;
  double qv = 0.0, cv = 0.0;
  R rk = R(0), dk = R(0), ov = R(0);
  uint32_t fv = 0u;
  if (lane < 4) qv = a.st[(size_t)(33 + lane) * n + tg];
  if (lane < 3) {
    cv = a.st[(size_t)lane * n + tg];
    fv = a.fix[(size_t)lane * n + tg];
    rk = g[lane][slot] * sr_w;
    dk = g[3 + lane][slot] * st_w;
  }
  if (lane < 3 * (NQ + 1))
    ov = MIXED ? (R)a.pk32f[(size_t)tg * 4 * Pr::NPK + 3 + lane] : (R)a.pk64[(size_t)tg * Pr::W64 + 3 + lane];
  const R qr = (R)qv;   // the conversion on the owning lanes only
  R qold[4], rot[3];
#pragma unroll
  for (int k = 0; k < 4; ++k) qold[k] = __shfl_sync(0xffffffffu, qr, k);
#pragma unroll
  for (int k = 0; k < 3; ++k) rot[k] = __shfl_sync(0xffffffffu, rk, k);
  R qn[4], off[NQ + 1][3];
  if constexpr (MIXED) trial_rotation<R, NQ>(rot, qold, a.fbody, qn, off);
  else trial_rotation<R, NQ>(rot, qold, a.body, qn, off);
  if (lane < 4) {
    P.qo64[lane] = qv;
    if (!MIXED) P.q64[lane] = (double)(lane == 0 ? qn[0] : (lane == 1 ? qn[1] : (lane == 2 ? qn[2] : qn[3])));
  }
  if (lane < 3) {
    const double cn = cv + (double)dk;
    P.co[lane] = cv;
    P.cn[lane] = cn;
    P.fo[lane] = fv;
    if (MIXED) {
      // the fixed-point trial COM: old word + rounded translation, so that the
      // reverse move (-dk) returns to the same word
      const float s = lane == 0 ? fsi[0] : (lane == 1 ? fsi[1] : fsi[2]);
      P.fn[lane] = fv + (uint32_t)__float2int_rn((float)dk * s);
    } else {
      const double il = lane == 0 ? iL[0] : (lane == 1 ? iL[1] : iL[2]);
      P.fn[lane] = to_fixed(cn, il);
    }
    P.rot[lane] = rk;
    P.dx[lane] = dk;
  }
  R d2 = dk * dk, r2 = rk * rk;   // nonzero on lanes 0-2 only
  d2 += __shfl_xor_sync(0xffffffffu, d2, 1);
  r2 += __shfl_xor_sync(0xffffffffu, r2, 1);
  d2 += __shfl_sync(0xffffffffu, d2, 2);
  r2 += __shfl_sync(0xffffffffu, r2, 2);
  // old and new offsets: value 3s+k on lane 3s+k
  R onv = R(0);
#pragma unroll
  for (int s = 0; s <= NQ; ++s)
#pragma unroll
    for (int k = 0; k < 3; ++k)
      if (lane == 3 * s + k) onv = off[s][k];
  if (lane < 3 * (NQ + 1)) {
    (&P.oo[0][0])[lane] = ov;
    (&P.on[0][0])[lane] = onv;
  }
  if (lane < 4) P.qn[lane] = lane == 0 ? qn[0] : (lane == 1 ? qn[1] : (lane == 2 ? qn[2] : qn[3]));
  // unit direction of charged site s at the new pose on lane 16 + 3s .. 16 + 3s + 2
  {
    const int s = (lane - 16) / 3;
    float v[3] = {1.0f, 0.0f, 0.0f};
#pragma unroll
    for (int q = 0; q < NQ; ++q)
      if (s == q) { v[0] = (float)off[q + 1][0]; v[1] = (float)off[q + 1][1]; v[2] = (float)off[q + 1][2]; }
    float u[3];
    site_dir1(v, u);
    if (lane >= 16 && lane < 28) {
      const int k = (lane - 16) - 3 * s;
      (&P.un[0][0])[lane - 16] = s < NQ ? (k == 0 ? u[0] : (k == 1 ? u[1] : u[2])) : 0.0f;
    }
  }
  if (lane == 0) {
    P.d2 = (float)d2;
    P.r2 = (float)r2;
    P.qf = q_form((float)st_w, (float)sr_w);
    P.trial = trial;
  }
  __syncwarp();
  if constexpr (Q64) {   // the FP64 quaternion an acceptance writes, prepared off the acceptance path
    const double q = accepted_q64(P, lane);
    if (lane < 4) P.q64[lane] = q;
    __syncwarp();
  }
}

}  // namespace g6
