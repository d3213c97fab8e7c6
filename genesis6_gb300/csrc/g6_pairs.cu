// g6_pairs.cu -- mixed-precision site-site forces over the Verlet list, and the
// integrator kernels of the mixed MD step.
//
// k_pairs<Model, LPI, MODE, HALF>: LPI lanes cooperate on one molecule i; a
// warp holds 32/LPI molecules and never waits for another warp (no block
// barrier).  Per molecule, two phases:
//   1. test: the lanes read the neighbour row (coalesced) and the 32-bit
//      fixed-point COM of each listed j (one 16-byte load), keep the pairs
//      with |d|^2 < rc^2 (an FP32 distance from the integer COM differences
//      without their low 9 bits; within a band of rc^2 that covers that
//      truncation the reference's FP64 test decides) and append them to the
//      molecule's row in shared memory with a ballot and a prefix count.  Up
//      to six row entries per lane are in flight at a time.
//   2. pairs: the lanes share out the compacted row (every lane of a group has
//      an in-range pair until the row's tail), load j's pose record one pair
//      ahead and run the FP32 site loop of pair_math, keeping per-lane sums of
//      the i-site forces, the COM switch force, the energy and the virial.
// HALF (the MD step's default): the rows hold only the pairs i evaluates
// (half_keep), the record is the 32-byte pkq (fixed-point COM and float
// quaternion, one 256-bit load) whose quaternion gives j's site offsets again
// (two rotation columns for the planar TIP4P/SPC-E layout), and each pair's
// force and torque on j go to jacc by two vector float atomics.  The full
// list (MODE 0, and the MD step when chosen) evaluates every pair from both
// molecules with the 64-byte pk32 record (offsets included, two loads).
// The lanes of a molecule are then combined: in FP64 for the force-only call
// (MODE 0: F, lab torque, energy, full virial), by a reduce-scatter of
// error-free float pairs for the MD step (MODE 1: F, lab torque, energy and
// virial trace as float pairs in fres, read by the integrator).
//
// k_integrate_mixed<NQ, MPW> (one lane per molecule) and k_integrate_quad<NQ>
// (four lanes per molecule, one per component): rigid_correct with the small
// Gear terms in float, the next predict and placement, and the per-step
// partial sums (step_partials; the replica finish runs in the next pair
// kernel's first blocks).
#include <cuda_runtime.h>

#include <cstring>

#include "g6_internal.cuh"
#include "g6_pairmath.cuh"
#include "g6_rigid.cuh"

namespace g6 {

// Residency of k_pairs: 128 threads per block, at least MINB blocks per SM
// (5: 96 registers, enough for the 3-charge models in the MD step without
// spills; 4: 128 registers for the 4-charge models and the full virial).
// Blocks of 32 or 64 threads measured the same (the SMs' 3-or-4-block split
// of a 4,096-molecule grid is not what leaves them idle at its end).
template <int LPI>
struct PairShape {
  static constexpr int THREADS = 128;
  static constexpr int GROUPS = 32 / LPI;   // molecules per warp
  // row entries per lane in flight during the test (4 to 6: deeper unrolling
  // spills the 3-charge MD variant at its 96-register budget)
  static constexpr int UNROLL = (160 / LPI) > 6 ? 6 : ((160 / LPI) < 4 ? 4 : (160 / LPI));
};
template <class M, int MODE>
struct PairMinBlocks {
  static constexpr int value = (M::NQ == 3 && MODE == 1) ? 5 : 4;
};

// The 32-byte record of molecule j (pkq: fixed-point COM words, float
// quaternion, zero) in one 256-bit load through the non-coherent path: no
// pose buffer is written while a pair kernel runs.
__device__ __forceinline__ void load_pose_q(const float4* pkq, int j, float (&v)[8]) {
  asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
      : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7])
      : "l"(pkq + 2 * (size_t)j));
}

// Float site offsets (LJ site, charged sites) from the record's quaternion:
// the placement's arithmetic (setmatrix_f, site_off_f), so the same bits as
// the offsets it wrote to pk32.  A planar model (M::PLANAR: body x = 0 for
// every site, y = 0 for sites 0 and 1, sites 2 and 3 at (0, +-y, z)) needs only
// the rotation's second and third columns; its terms with a zero body
// coordinate are left out, which changes no value (x * 0 + y = y), and the
// two mirror sites share their z term.
template <class M>
__device__ __forceinline__ void sites_from_q(const ForceArgs& a, const float* q, float (&r)[M::NQ + 1][3]) {
  if constexpr (M::PLANAR) {
    const float qa = q[0], qb = q[1], qc = q[2], qd = q[3];
    const float aa = __fmul_rn(qa, qa), bb = __fmul_rn(qb, qb), cc = __fmul_rn(qc, qc), dd = __fmul_rn(qd, qd);
    const float t1 = __fmul_rn(-2.0f, __fmaf_rn(qa, qd, __fmul_rn(qb, qc)));
    const float t2 = __fmul_rn(2.0f, __fmaf_rn(qb, qd, __fmul_rn(-qa, qc)));
    const float t4 = __fsub_rn(__fadd_rn(aa, cc), __fadd_rn(bb, dd));
    const float t5 = __fmul_rn(-2.0f, __fmaf_rn(qa, qb, __fmul_rn(qc, qd)));
    const float t7 = __fmul_rn(2.0f, __fmaf_rn(qa, qb, __fmul_rn(-qc, qd)));
    const float t8 = __fsub_rn(__fadd_rn(aa, dd), __fadd_rn(bb, cc));
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const float z = a.fbody[s][2];
      r[s][0] = __fmul_rn(t2, z); r[s][1] = __fmul_rn(t5, z); r[s][2] = __fmul_rn(t8, z);
    }
    const float y = a.fbody[2][1], z = a.fbody[2][2];
    const float zx = __fmul_rn(t2, z), zy = __fmul_rn(t5, z), zz = __fmul_rn(t8, z);
    r[2][0] = __fmaf_rn(t1, y, zx); r[2][1] = __fmaf_rn(t4, y, zy); r[2][2] = __fmaf_rn(t7, y, zz);
    r[3][0] = __fmaf_rn(t1, -y, zx); r[3][1] = __fmaf_rn(t4, -y, zy); r[3][2] = __fmaf_rn(t7, -y, zz);
  } else {
    float t[9];
    setmatrix_f(q, t);
#pragma unroll
    for (int s = 0; s <= M::NQ; ++s) site_off_f(t, a.fbody[s][0], a.fbody[s][1], a.fbody[s][2], r[s]);
  }
}

// The pose record a pair kernel reads per molecule: the 64-byte pk32 record
// (fixed-point COM words, float offsets of the LJ site and the three charged
// sites) in two 256-bit loads, or the 32-byte pkq record, whose quaternion
// gives the offsets again with the placement's roundings (the same bits).
// OFFS = the pk32 record: the full list of the 3-charge models, where each
// record load is followed by a pair's whole site loop.  The half list does half
// the site work per row and is bound by the L1 line gathers of the records, so
// it takes the quarter-size pkq record; 4-charge models always do (their
// 80-byte pk32 record is not 32-byte aligned).  Measured on TIP4P: full list
// 59.7 (pk32) vs 61.8 us (pkq) at 32,768 molecules; half list 54.9 vs 49.1 us.
template <class M, bool HALF>
struct PoseRec {
  static constexpr bool OFFS = M::NPK == 4 && !HALF;
  static constexpr int W = OFFS ? 16 : 8;   // floats
};
template <class M, bool HALF>
__device__ __forceinline__ void load_rec(const float4* pk32, const float4* pkq, int j,
                                         float (&v)[PoseRec<M, HALF>::W]) {
  if constexpr (PoseRec<M, HALF>::OFFS) {
    const float4* p = pk32 + 4 * (size_t)j;
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7])
        : "l"(p));
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=f"(v[8]), "=f"(v[9]), "=f"(v[10]), "=f"(v[11]), "=f"(v[12]), "=f"(v[13]), "=f"(v[14]), "=f"(v[15])
        : "l"(p + 2));
  } else {
    load_pose_q(pkq, j, v);
  }
}
template <class M, bool HALF>
__device__ __forceinline__ void rec_sites(const ForceArgs& a, const float (&v)[PoseRec<M, HALF>::W],
                                          float (&r)[M::NQ + 1][3]) {
  if constexpr (PoseRec<M, HALF>::OFFS) {
#pragma unroll
    for (int s = 0; s <= M::NQ; ++s)
#pragma unroll
      for (int k = 0; k < 3; ++k) r[s][k] = v[3 + 3 * s + k];
  } else {
    sites_from_q<M>(a, v + 3, r);
  }
}
// The first float4 of a record: the fixed-point COM words.
template <class M, bool HALF>
__device__ __forceinline__ float4 load_com(const float4* pk32, const float4* pkq, int j) {
  if constexpr (PoseRec<M, HALF>::OFFS) return __ldg(pk32 + 4 * (size_t)j);
  else return __ldg(pkq + 2 * (size_t)j);
}

// The row test's COM separation: the integer difference without its low 9
// bits (|h| < 2^22, converted exactly by the 1.5 * 2^23 bit pattern), times
// 512 L/2^32.  Each component is low by less than L/2^23 (the band that
// sends a pair to the FP64 test covers it); 5 instructions per component
// instead of fix_delta's 9.
__device__ __forceinline__ float coarse_delta(uint32_t xi, uint32_t xj, float s512) {
  const int h = (int)(xi - xj) >> 9;
  return (__int_as_float(0x4B400000 + h) - 12582912.0f) * s512;
}

// Fixed-point COM difference (units L/2^32, the wrap is the minimum image) to A.
__device__ __forceinline__ void fix_delta(uint32_t xi, uint32_t yi, uint32_t zi, const float4& qj, float sx, float sy,
                                          float sz, float d[3]) {
  d[0] = i32_to_f32((int)(xi - __float_as_uint(qj.x))) * sx;
  d[1] = i32_to_f32((int)(yi - __float_as_uint(qj.y))) * sy;
  d[2] = i32_to_f32((int)(zi - __float_as_uint(qj.z))) * sz;
}

// The LPI lanes of a molecule combine their 8 float-pair partials by a
// butterfly that halves the values each lane carries at every level
// (reduce-scatter): 4 + 2 + 1 float-pair exchanges instead of 8 per level.
// Lane sub ends with the sums of values idx .. idx + 8/LPI - 1 (LPI <= 8) or
// of value idx (LPI > 8, after all-reducing that value over the groups of 8).
template <int CNT>
__device__ __forceinline__ void scatter_level(FF (&v)[8], int sub, int m, int& idx) {
  constexpr int H = CNT / 2;
  const bool up = (sub & m) != 0;
#pragma unroll
  for (int k = 0; k < H; ++k) {
    const FF keep = up ? v[k + H] : v[k];
    const FF send = up ? v[k] : v[k + H];
    v[k] = ff_add(keep, red_shfl(send, m));
  }
  if (up) idx += H;
}
template <int LPI>
__device__ __forceinline__ int ff_reduce_scatter8(FF (&v)[8], int sub) {
  int idx = 0;
  if constexpr (LPI >= 2) scatter_level<8>(v, sub, LPI / 2, idx);
  if constexpr (LPI >= 4) scatter_level<4>(v, sub, LPI / 4, idx);
  if constexpr (LPI >= 8) scatter_level<2>(v, sub, LPI / 8, idx);
#pragma unroll
  for (int m = LPI / 16; m >= 1; m >>= 1) v[0] = ff_add(v[0], red_shfl(v[0], m));
  return idx;
}

// MODE 0: force only; 1: MD step.  HALF (MD step only): each pair within rc is
// evaluated once, by the molecule that keeps it (half_keep: rows built for a
// half-list run hold only those; a full row is filtered here); j's force and
// torque go to a.jacc with vector float atomics, read and cleared by the
// integrator kernel.
template <class M, int LPI, int MODE, bool HALF>
__global__ void __launch_bounds__(PairShape<LPI>::THREADS, (PairMinBlocks<M, MODE>::value))
    k_pairs(ForceArgs a, StepArgs sa) {
  static_assert(!HALF || MODE == 1, "the half list is an MD-step variant");
  constexpr int NW = MODE == 0 ? 9 : 1;
  int bid = blockIdx.x;
  if constexpr (MODE == 1) {
    // the integrator kernel (a programmatic dependent launch) may start its
    // loads now; it waits for this grid before reading forces or thermostats
    asm volatile("griddepcontrol.launch_dependents;");
    // the first nrep blocks finish the previous step's replicas (sums,
    // thermostat, log), overlapped with the pair work of the others
    if (bid < a.rep.nrep) {
      finish_pending(sa, bid, 32);
      return;
    }
    bid -= a.rep.nrep;
  }
  constexpr int G = PairShape<LPI>::GROUPS;
  constexpr int U = PairShape<LPI>::UNROLL;
  extern __shared__ int s_rows[];
  const int n = a.n;
  const int step = a.ctrl ? a.ctrl[1] : 0;
  const bool odd = (step & 1) != 0;
  const double* pk64 = odd ? a.pk64_1 : a.pk64;
  const float4* pkq = odd ? a.pkq_1 : a.pkq;
  const float4* pk32 = odd ? a.pk32_1 : a.pk32;
  constexpr int RW = PoseRec<M, HALF>::W;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int g = lane / LPI, sub = lane % LPI;
  const int i = (bid * blockDim.x + threadIdx.x) / LPI;
  const bool valid = i < n;
  int* srow = s_rows + (size_t)(warp * G + g) * a.ccap;

  // pose of i: fixed-point COM and float site offsets
  float ri[M::NQ + 1][3];
  uint32_t xi = 0, yi = 0, zi = 0;
  float sx = 0.f, sy = 0.f, sz = 0.f;
  int r = 0, nn = 0;
  if (valid) {
    float wi[RW];
    load_rec<M, HALF>(pk32, pkq, i, wi);
    if (a.rep.nrep == 1) {   // one replica: the scales are kernel arguments (no dependent load)
      sx = a.fs1[0]; sy = a.fs1[1]; sz = a.fs1[2];
    } else {
      r = a.rep.mol_rep[i];
      sx = a.rep.fscale[3 * r]; sy = a.rep.fscale[3 * r + 1]; sz = a.rep.fscale[3 * r + 2];
    }
    xi = __float_as_uint(wi[0]); yi = __float_as_uint(wi[1]); zi = __float_as_uint(wi[2]);
    rec_sites<M, HALF>(a, wi, ri);
    nn = a.nnb[i];
  } else {
#pragma unroll
    for (int s = 0; s <= M::NQ; ++s) ri[s][0] = ri[s][1] = ri[s][2] = 0.f;
  }

  // ---- phase 1: in-range entries of the row into shared memory ----
  int nmax = nn;
#pragma unroll
  for (int m = 16; m >= 1; m >>= 1) nmax = max(nmax, __shfl_xor_sync(0xffffffffu, nmax, m));
  const int* row = a.nbr + (size_t)(valid ? i : 0) * a.cap;
  const float rout2 = a.cc.frout2;
  const float band = a.band;   // above the test's error (coarse_delta, FP32 rounding); set per system
  const float sx5 = sx * 512.0f, sy5 = sy * 512.0f, sz5 = sz * 512.0f;
  int cnt = 0;
  // the row entries of the next batch are loaded while this batch's COM words
  // are in flight (one round trip of row loads in all, not one per batch);
  // the first batch's are loaded within the row's capacity before its length
  // arrives and masked by it afterwards
  int jn[U];
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int k = u * LPI + sub;
    jn[u] = (valid && k < a.cap) ? __ldg(row + k) : -1;
  }
  for (int base = 0; base < nmax; base += LPI * U) {
    int jj[U];
    float4 qj[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      jj[u] = base + u * LPI + sub < nn ? jn[u] : -1;
      if (HALF && jj[u] >= 0 && !half_keep(i, jj[u])) jj[u] = -1;
    }
#pragma unroll
    for (int u = 0; u < U; ++u) qj[u] = jj[u] >= 0 ? load_com<M, HALF>(pk32, pkq, jj[u]) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int k = base + LPI * U + u * LPI + sub;
      jn[u] = k < nn ? __ldg(row + k) : -1;
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      bool in = false;
      if (jj[u] >= 0) {
        const float d0 = coarse_delta(xi, __float_as_uint(qj[u].x), sx5);
        const float d1 = coarse_delta(yi, __float_as_uint(qj[u].y), sy5);
        const float d2 = coarse_delta(zi, __float_as_uint(qj[u].z), sz5);
        const float dd = d0 * d0 + d1 * d1 + d2 * d2;
        in = dd < rout2;
        if (fabsf(dd - rout2) < band) {
          // borderline: decide with the reference's FP64 arithmetic (Interaction_Compress2)
          const double* pi = pk64 + (size_t)i * M::W64;
          const double* pj = pk64 + (size_t)jj[u] * M::W64;
          const double ci[3] = {pi[0], pi[1], pi[2]}, cj[3] = {pj[0], pj[1], pj[2]};
          const double Ld[3] = {a.rep.L[3 * r], a.rep.L[3 * r + 1], a.rep.L[3 * r + 2]};
          const double iLd[3] = {a.rep.invL[3 * r], a.rep.invL[3 * r + 1], a.rep.invL[3 * r + 2]};
          double o[3], dx[3];
          in = exact_dd(ci, cj, Ld, iLd, o, dx) < a.cc.rout2;
        }
      }
      const unsigned bal = __ballot_sync(0xffffffffu, in);
      const unsigned mine = LPI == 32 ? bal : (bal >> (g * LPI)) & ((1u << LPI) - 1u);
      if (in) {
        const int pos = cnt + __popc(mine & ((1u << sub) - 1u));
        if (pos < a.ccap) srow[pos] = jj[u];
      }
      cnt += __popc(mine);
    }
  }
  if (cnt > a.ccap) {   // more in-range pairs than the shared row holds: reported, the run is repeated
    if (sub == 0) atomicExch(a.overflow, 1);
    cnt = a.ccap;
  }
  __syncwarp();

  // ---- phase 2: site loops over the compacted row ----
  Acc<M, float, NW> acc;
  acc.zero();
  {
    const float frin2 = a.cc.frin2, frin = a.cc.frin, frout = a.cc.frout, fc1 = a.cc.fc1, fc2 = a.cc.fc2;
    int t = sub;
    float tn[RW];
    if (t < cnt) load_rec<M, HALF>(pk32, pkq, srow[t], tn);
    for (; t < cnt; t += LPI) {
      float wj[RW];
#pragma unroll
      for (int k = 0; k < RW; ++k) wj[k] = tn[k];
      if (t + LPI < cnt) load_rec<M, HALF>(pk32, pkq, srow[t + LPI], tn);   // the next pair's record, one pair ahead
      float d[3];
      fix_delta(xi, yi, zi, make_float4(wj[0], wj[1], wj[2], 0.f), sx, sy, sz, d);
      const float dd = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
      float rj[M::NQ + 1][3];
      rec_sites<M, HALF>(a, wj, rj);
      if constexpr (HALF) {
        const int jc = srow[t];
        PairJ<float> pj;
        pair_math<M, float, NW, true>(d, dd, ri, rj, a.pc, frin2, frin, frout, fc1, fc2, a.pc.frl, a.pc.fru, a.pc.fw3,
                                      acc, &pj);
        atomicAdd(a.jacc + 2 * (size_t)jc, make_float4(pj.f[0], pj.f[1], pj.f[2], 0.f));
        atomicAdd(a.jacc + 2 * (size_t)jc + 1, make_float4(pj.t[0], pj.t[1], pj.t[2], 0.f));
      } else {
        pair_math<M, float, NW>(d, dd, ri, rj, a.pc, frin2, frin, frout, fc1, fc2, a.pc.frl, a.pc.fru, a.pc.fw3, acc);
      }
    }
  }

  // ---- lane partials -> F, lab torque (rigid_collectforce), energy, virial ----
  float fo[3], to[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    float t = acc.fc[k];
#pragma unroll
    for (int q = 0; q <= M::NQ; ++q) t += acc.fs[q][k];
    fo[k] = t;
  }
  {
    float tx = 0.f, ty = 0.f, tz = 0.f;
#pragma unroll
    for (int q = 0; q <= M::NQ; ++q) {
      tx += ri[q][1] * acc.fs[q][2] - ri[q][2] * acc.fs[q][1];
      ty += ri[q][2] * acc.fs[q][0] - ri[q][0] * acc.fs[q][2];
      tz += ri[q][0] * acc.fs[q][1] - ri[q][1] * acc.fs[q][0];
    }
    to[0] = tx; to[1] = ty; to[2] = tz;
  }
  if constexpr (MODE == 0) {
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
      if (a.npair_in) a.npair_in[i] = cnt;
    }
  } else {
    FF q8[8];
#pragma unroll
    for (int k = 0; k < 3; ++k) { q8[k] = FF{fo[k], 0.0f}; q8[3 + k] = FF{to[k], 0.0f}; }
    q8[6] = FF{acc.e, 0.0f};
    q8[7] = FF{acc.w[0], 0.0f};
    const int idx = ff_reduce_scatter8<LPI>(q8, sub);
    constexpr int C = LPI >= 8 ? 1 : 8 / LPI;   // values each lane ends with
    if (valid && (LPI <= 8 || (sub & (LPI / 8 - 1)) == 0)) {
      // fres: [F.hi, E.hi] [F.lo, E.lo] [tau.hi, W.hi] [tau.lo, W.lo]
      float* o = (float*)(a.fres + (size_t)4 * i);
#pragma unroll
      for (int c = 0; c < C; ++c) {
        const int k = idx + c;
        const int pos = k < 3 ? k : (k < 6 ? 5 + k : (k == 6 ? 3 : 11));
        o[pos] = q8[c].hi;
        o[pos + 4] = q8[c].lo;
      }
    }
    if (valid && sub == 0) a.npair_in[i] = cnt;
  }
}

// Half list: the j side the pair kernel accumulated for molecule im (the
// sum of its partners' pair forces, which the caller subtracts, and its lab
// torque from those pairs), cleared for the next step's atomics.
__device__ __forceinline__ void take_jside(const ForceArgs& a, int im, float4& jf, float4& jt) {
  float4* p = a.jacc + 2 * (size_t)im;
  jf = p[0];
  jt = p[1];
  p[0] = make_float4(0.f, 0.f, 0.f, 0.f);
  p[1] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// Mixed MD step, second kernel: Gear corrector, next predict + placement and
// the step's reductions for 32 molecules per block.  MPW molecules per warp
// (32 / MPW warps per block): the corrector's FP64 instructions cost a warp
// 64 cycles each whatever the number of active lanes, so fewer molecules per
// warp spread them over more schedulers (small systems, latency) and more
// molecules per warp issue fewer of them (large systems, FP64 throughput).
// The block's 32 results meet in shared memory for step_reduce.
template <int NQ, int MPW>
__global__ void __launch_bounds__(32 * (32 / MPW)) k_integrate_mixed(ForceArgs a, StepArgs sa) {
  __shared__ FF s_vv[32][NRED];
  __shared__ float s_dm[32];
  __shared__ int s_bad[32], s_rr[32];
  const int n = a.n;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // the state of this lane's molecule, before the pair kernel has finished
  MixedIn min;
  {
    const int im = blockIdx.x * 32 + warp * MPW + lane;
    if (lane < MPW && im < n) load_mixed(sa, im, min);
  }
  // forces, the thermostats and the control words are the pair kernel's (and
  // its replica finish's) results: wait for that grid (a no-op when the kernel
  // was not launched as its programmatic dependent)
  asm volatile("griddepcontrol.wait;" ::: "memory");
  const int step = a.ctrl[1];
  const bool odd = (step & 1) != 0;
  const bool predict_next = step + 1 < sa.ctrl[2];
  if (lane < MPW) {
    const int m = warp * MPW + lane;
    const int im = blockIdx.x * 32 + m;
    FF vv[NRED];
#pragma unroll
    for (int k = 0; k < NRED; ++k) vv[k] = FF{0.0f, 0.0f};
    float dmax2 = 0.0f;
    int bad = 0, rr = -1;
    if (im < n) {
      rr = a.rep.mol_rep[im];
      const float4* o = a.fres + (size_t)4 * im;
      const float4 h0 = o[0], l0 = o[1], h1 = o[2], l1 = o[3];
      float4 jf = make_float4(0.f, 0.f, 0.f, 0.f), jt = jf;
      if (a.half) take_jside(a, im, jf, jt);
      const float F[3] = {h0.x + (l0.x - jf.x), h0.y + (l0.y - jf.y), h0.z + (l0.z - jf.z)};
      const float tl[3] = {h1.x + (l1.x + jt.x), h1.y + (l1.y + jt.y), h1.z + (l1.z + jt.z)};
      float ekt2, ekr2;
      correct_mixed<NQ>(sa, im, min, F, tl, step, predict_next, pose_buf(sa, odd ? 0 : 1), ekt2, ekr2, dmax2, bad);
      const float pf = a.half ? 1.0f : 0.5f;   // a full list holds every pair twice
      vv[0] = FF{pf * h0.w, pf * l0.w};
      vv[1] = FF{pf * h1.w, pf * l1.w};
      vv[2] = FF{ekt2, 0.0f};
      vv[3] = FF{ekr2, 0.0f};
      vv[4] = FF{pf * (float)a.npair_in[im], 0.0f};
    }
#pragma unroll
    for (int k = 0; k < NRED; ++k) s_vv[m][k] = vv[k];
    s_dm[m] = dmax2; s_bad[m] = bad; s_rr[m] = rr;
  }
  __syncthreads();
  FF vv[NRED];
  float dmax2 = 0.0f;
  int bad = 0, rr = -1;
  if (warp == 0) {
#pragma unroll
    for (int k = 0; k < NRED; ++k) vv[k] = s_vv[lane][k];
    dmax2 = s_dm[lane]; bad = s_bad[lane]; rr = s_rr[lane];
  }
  step_partials<FF>(sa, vv, rr, dmax2, bad, 32, step, 0);
}

// The component-parallel integrator: four lanes per molecule (correct_quad),
// 8 molecules per warp, 32 per block of 128 threads.
template <int NQ>
__global__ void __launch_bounds__(128) k_integrate_quad(ForceArgs a, StepArgs sa) {
  __shared__ FF s_vv[32][NRED];
  __shared__ float s_dm[32];
  __shared__ int s_bad[32], s_rr[32];
  const int n = a.n;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, c = lane & 3;
  const int m = warp * 8 + (lane >> 2);
  const int im = blockIdx.x * 32 + m;
  const bool ok = im < n;
  QuadIn qin;
  if (ok) load_quad(sa, im, c, qin);
  else quad_dummy(c, qin);
  asm volatile("griddepcontrol.wait;" ::: "memory");   // forces, thermostats, control words (see k_integrate_mixed)
  const int step = a.ctrl[1];
  const bool odd = (step & 1) != 0;
  const bool predict_next = step + 1 < sa.ctrl[2];
  float4 h0 = make_float4(0.f, 0.f, 0.f, 0.f), l0 = h0, h1 = h0, l1 = h0, jf = h0, jt = h0;
  if (ok) {
    const float4* o = a.fres + (size_t)4 * im;
    h0 = o[0]; l0 = o[1]; h1 = o[2]; l1 = o[3];
    if (a.half) {
      jf = a.jacc[2 * (size_t)im];
      jt = a.jacc[2 * (size_t)im + 1];
    }
  }
  if (a.half) {
    __syncwarp();   // every lane of the quad has read the j side before lane 0 clears it
    if (ok && c == 0) {
      a.jacc[2 * (size_t)im] = make_float4(0.f, 0.f, 0.f, 0.f);
      a.jacc[2 * (size_t)im + 1] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
  }
  const float Fc = c == 0 ? h0.x + (l0.x - jf.x) : (c == 1 ? h0.y + (l0.y - jf.y) : (c == 2 ? h0.z + (l0.z - jf.z) : 0.0f));
  const float tl[3] = {h1.x + (l1.x + jt.x), h1.y + (l1.y + jt.y), h1.z + (l1.z + jt.z)};
  float ekt2 = 0.0f, ekr2 = 0.0f, dmax2 = 0.0f;
  int bad = 0;
  correct_quad<NQ>(sa, im, ok, c, qin, Fc, tl, step, predict_next, pose_buf(sa, odd ? 0 : 1), ekt2, ekr2, dmax2, bad);
  if (c == 0) {
    FF vv[NRED];
#pragma unroll
    for (int k = 0; k < NRED; ++k) vv[k] = FF{0.0f, 0.0f};
    int rr = -1;
    if (ok) {
      rr = qin.r;
      const float pf = a.half ? 1.0f : 0.5f;   // a full list holds every pair twice
      vv[0] = FF{pf * h0.w, pf * l0.w};
      vv[1] = FF{pf * h1.w, pf * l1.w};
      vv[2] = FF{ekt2, 0.0f};
      vv[3] = FF{ekr2, 0.0f};
      vv[4] = FF{pf * (float)a.npair_in[im], 0.0f};
    } else {
      dmax2 = 0.0f;
      bad = 0;
    }
#pragma unroll
    for (int k = 0; k < NRED; ++k) s_vv[m][k] = vv[k];
    s_dm[m] = dmax2; s_bad[m] = bad; s_rr[m] = rr;
  }
  __syncthreads();
  FF vv[NRED];
  float dm = 0.0f;
  int bd = 0, rr = -1;
  if (warp == 0) {
#pragma unroll
    for (int k = 0; k < NRED; ++k) vv[k] = s_vv[lane][k];
    dm = s_dm[lane]; bd = s_bad[lane]; rr = s_rr[lane];
  }
  step_partials<FF>(sa, vv, rr, dm, bd, 32, step, 0);
}

// Finish of the last step of a mixed run (one replica per block).
__global__ void __launch_bounds__(128) k_finish_step(StepArgs sa) { finish_pending(sa, blockIdx.x, 32); }

template <int LPI>
size_t pairs_smem_bytes(int cap) {
  return (size_t)(PairShape<LPI>::THREADS / 32) * PairShape<LPI>::GROUPS * cap * sizeof(int);
}

template <class M, int LPI, int MODE, bool HALF>
static cudaError_t launch_pairs_t(const ForceArgs& a, const StepArgs& sa, cudaStream_t s) {
  const int threads = PairShape<LPI>::THREADS;
  const long long total = (long long)a.n * LPI;
  const int blocks = (int)((total + threads - 1) / threads) + (MODE == 1 ? a.rep.nrep : 0);
  if (blocks == 0) return cudaSuccess;
  const size_t smem = pairs_smem_bytes<LPI>(a.ccap);
  if (smem > 48 * 1024) {
    cudaError_t e =
        cudaFuncSetAttribute(k_pairs<M, LPI, MODE, HALF>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  k_pairs<M, LPI, MODE, HALF><<<blocks, threads, smem, s>>>(a, sa);
  return cudaGetLastError();
}

template <class M, int MODE, bool HALF>
static cudaError_t launch_pairs_h(const ForceArgs& a, const StepArgs& sa, int lpi, cudaStream_t s) {
  switch (lpi) {
    case 4: return launch_pairs_t<M, 4, MODE, HALF>(a, sa, s);
    case 8: return launch_pairs_t<M, 8, MODE, HALF>(a, sa, s);
    case 16: return launch_pairs_t<M, 16, MODE, HALF>(a, sa, s);
    default: return launch_pairs_t<M, 32, MODE, HALF>(a, sa, s);
  }
}

template <class M, int MODE>
static cudaError_t launch_pairs_l(const ForceArgs& a, const StepArgs& sa, int lpi, cudaStream_t s) {
  if constexpr (MODE == 1) {
    if (a.half) return launch_pairs_h<M, 1, true>(a, sa, lpi, s);
  }
  return launch_pairs_h<M, MODE, false>(a, sa, lpi, s);
}

template <int MODE>
static cudaError_t launch_pairs_any(const ForceArgs& a, const StepArgs& sa, int model, int lpi, cudaStream_t s) {
  if (model_nq(model) == 3) {
    if (MODE == 1 && a.planar) return launch_pairs_l<MT<3, false, true>, MODE>(a, sa, lpi, s);
    return launch_pairs_l<MT<3, false>, MODE>(a, sa, lpi, s);
  }
  if (a.pc.taper) return launch_pairs_l<MT<4, true>, MODE>(a, sa, lpi, s);
  return launch_pairs_l<MT<4, false>, MODE>(a, sa, lpi, s);
}

// Largest row capacity (entries) whose shared-memory rows fit one block.
int pairs_max_cap(int lpi) {
  const size_t lim = 200 * 1024;
  switch (lpi) {
    case 4: return (int)(lim / pairs_smem_bytes<4>(1));
    case 8: return (int)(lim / pairs_smem_bytes<8>(1));
    case 16: return (int)(lim / pairs_smem_bytes<16>(1));
    default: return (int)(lim / pairs_smem_bytes<32>(1));
  }
}

// Mixed force only: F, lab torque, per-molecule energy and virial in FP64.
cudaError_t launch_pairs_force(const ForceArgs& a, int model, int lpi, cudaStream_t s) {
  StepArgs none;
  memset(&none, 0, sizeof none);
  ForceArgs f = a;
  f.half = 0;
  return launch_pairs_any<0>(f, none, model, lpi, s);
}

// After the last step of a mixed run: its replica finish.
cudaError_t launch_finish_step(const StepArgs& sa, int nrep, cudaStream_t s) {
  k_finish_step<<<nrep, 128, 0, s>>>(sa);
  return cudaGetLastError();
}

// The integrator as a programmatic dependent of the pair kernel launched just
// before it (pdl), so that its blocks start and load the state during the pair
// kernel's tail; a plain launch when an event separates the two.
template <int NQ, int MPW>
static cudaError_t launch_integrate_k(const ForceArgs& a, const StepArgs& sa, int blocks, bool pdl, cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(blocks);
  cfg.blockDim = dim3(32 * (32 / MPW));
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = pdl ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, k_integrate_mixed<NQ, MPW>, a, sa);
}

template <int NQ>
static cudaError_t launch_integrate_quad(const ForceArgs& a, const StepArgs& sa, int blocks, bool pdl, cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(blocks);
  cfg.blockDim = dim3(128);
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = pdl ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, k_integrate_quad<NQ>, a, sa);
}

// mpw: molecules per warp of the one-lane-per-molecule integrator (8, 16 or
// 32), or 4 for the component-parallel one (4 lanes per molecule).
template <int NQ>
static cudaError_t launch_integrate(const ForceArgs& a, const StepArgs& sa, int mpw, int blocks, bool pdl,
                                    cudaStream_t s) {
  switch (mpw) {
    case 4: return launch_integrate_quad<NQ>(a, sa, blocks, pdl, s);
    case 8: return launch_integrate_k<NQ, 8>(a, sa, blocks, pdl, s);
    case 16: return launch_integrate_k<NQ, 16>(a, sa, blocks, pdl, s);
    default: return launch_integrate_k<NQ, 32>(a, sa, blocks, pdl, s);
  }
}

// The forces of the MD step's pair kernel without the integrator: fres (and,
// for the half list, minus the partner share in jacc, which is cleared) to
// FP64 F and lab torque, the energy share to emol.
__global__ void __launch_bounds__(128) k_step_forces(ForceArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const float4* o = a.fres + (size_t)4 * i;
  const float4 h0 = o[0], l0 = o[1], h1 = o[2], l1 = o[3];
  double f[3] = {(double)h0.x + (double)l0.x, (double)h0.y + (double)l0.y, (double)h0.z + (double)l0.z};
  double t[3] = {(double)h1.x + (double)l1.x, (double)h1.y + (double)l1.y, (double)h1.z + (double)l1.z};
  if (a.half) {
    float4 jf, jt;
    take_jside(a, i, jf, jt);
    f[0] -= jf.x; f[1] -= jf.y; f[2] -= jf.z;
    t[0] += jt.x; t[1] += jt.y; t[2] += jt.z;
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) { a.F[(size_t)k * a.n + i] = f[k]; a.tl[(size_t)k * a.n + i] = t[k]; }
  a.emol[i] = (a.half ? 1.0 : 0.5) * ((double)h0.w + (double)l0.w);
}

cudaError_t launch_step_pair_forces(const ForceArgs& a, const StepArgs& sa, int model, int lpi, cudaStream_t s) {
  cudaError_t e = launch_pairs_any<1>(a, sa, model, lpi, s);
  if (e != cudaSuccess || a.n == 0) return e;
  k_step_forces<<<(a.n + 127) / 128, 128, 0, s>>>(a);
  return cudaGetLastError();
}

// Mixed MD step: pair kernel, then the integrator kernel (mpw molecules per warp).
cudaError_t launch_step_mixed(const ForceArgs& a, const StepArgs& sa, int model, int lpi, int mpw, cudaStream_t s,
                              cudaEvent_t between) {
  cudaError_t e = launch_pairs_any<1>(a, sa, model, lpi, s);
  if (e != cudaSuccess) return e;
  if (between) {
    e = cudaEventRecordWithFlags(between, s, cudaEventRecordExternal);
    if (e != cudaSuccess) return e;
  }
  const int blocks = (a.n + 31) / 32;
  if (blocks == 0) return cudaSuccess;
  const bool pdl = between == nullptr;
  return model_nq(model) == 3 ? launch_integrate<3>(a, sa, mpw, blocks, pdl, s)
                              : launch_integrate<4>(a, sa, mpw, blocks, pdl, s);
}

}  // namespace g6
