// g6_pairmath.cuh -- the site-site arithmetic of one molecule pair, shared by
// the force kernels (g6_force.cu: FP64 and force-only paths; g6_pairs.cu: the
// mixed-precision list kernel of the MD step).
//
// Physics per molecule pair (i,j), restating StdForce StdInteraction.F90:201-604,
// interaction_force_tip4p TIP4PModule.F90:187-758 and force_st2
// ST2Module.F90:187-750:
//   d   = com_i - com_j - image                     (Interaction_Compress2)
//   hh, dh = cutoff_func(|d|^2)                      (CutoffModule.F90:38-59)
//   e_lj = aa/r^12 + bb/r^6 on the LJ site pair, e_c = sum qq/r on charged pairs
//   f_site = hh * (site-site force) [ST2 custom path: charged pairs x hh*s12]
//   f_COM  = dh*e*d  [ST2: dh*e_lj*d + (dh*s12 + hh*ds12)*e_c*d]
//   e_pair = hh*e    [ST2: e_c*hh*s12 + e_lj*hh]
//   W     += d (x) (sum of i-site forces incl. f_COM)
#pragma once

#include <cuda_runtime.h>

#include "g6_internal.cuh"

namespace g6 {

// PLANAR_ (3-charge models): every site has body x = 0, the LJ site and the
// first charged site lie on the z axis and the other two charged sites are
// mirror images in y with one z (TIP4P, SPC/E), so a site offset needs only
// two columns of the rotation.
template <int NQ_, bool TAPER_, bool PLANAR_ = false>
struct MT {
  static constexpr int NQ = NQ_;
  static constexpr bool TAPER = TAPER_;
  static constexpr bool PLANAR = PLANAR_;
  static constexpr int W64 = ((6 + 3 * NQ_) + 1) / 2 * 2;   // doubles per molecule in pk64
  static constexpr int NPK = ((6 + 3 * NQ_) + 3) / 4;        // float4 per molecule in pk32
};


// ---------------------------------------------------------------------------
// Switch and taper in either precision.
// ---------------------------------------------------------------------------
template <class R>
__device__ __forceinline__ void switch_fn(R dd, R rin2, R rin, R rout, R c1, R c2, R& hh, R& dh) {
  if (dd > rin2) {
    R r, ir;
    root_r(dd, r, ir);
    R u = r - rout, l = r - rin, uu = u * u, ll = l * l;
    hh = c1 * uu * u * (R(10) * ll - R(5) * u * l + uu);
    dh = div_r(-c2 * uu * ll, r, ir);
  } else {
    hh = R(1);
    dh = R(0);
  }
}
template <class R>
__device__ __forceinline__ void taper_fn(R d12, R rl, R ru, R w3, R& s12, R& ds12) {
  if (d12 < ru * ru) {
    if (d12 < rl * rl) {
      s12 = R(0); ds12 = R(0);
    } else {
      R r12, ir12;
      root_r(d12, r12, ir12);
      s12 = (r12 - rl) * (r12 - rl) * (R(3) * ru - rl - R(2) * r12) / w3;
      ds12 = div_r(-(R(6) * (r12 - rl) * (ru - r12) / w3), r12, ir12);
    }
  } else {
    s12 = R(1); ds12 = R(0);
  }
}

template <class R> struct Prm;
template <> struct Prm<double> {
  __device__ static double qq(const PairConst& p, int a, int b) { return p.qq[a][b]; }
  __device__ static double aa(const PairConst& p) { return p.aa; }
  __device__ static double bb(const PairConst& p) { return p.bb; }
};
template <> struct Prm<float> {
  __device__ static float qq(const PairConst& p, int a, int b) { return p.fqq[a][b]; }
  __device__ static float aa(const PairConst& p) { return p.faa; }
  __device__ static float bb(const PairConst& p) { return p.fbb; }
};

// Site-site loop of one molecule pair.  ri/rj: site offsets from their COM
// (index 0 = LJ site, 1..NQ = charged sites).  Adds i-side results to acc.
// NW = 9: full 3x3 molecular virial; NW = 1: its trace only (MD step).
template <class M, class R, int NW>
struct Acc {
  R fs[M::NQ + 1][3];
  R fc[3];
  R e;
  R w[NW];
  __device__ void zero() {
#pragma unroll
    for (int s = 0; s <= M::NQ; ++s) fs[s][0] = fs[s][1] = fs[s][2] = R(0);
    fc[0] = fc[1] = fc[2] = R(0);
    e = R(0);
#pragma unroll
    for (int k = 0; k < NW; ++k) w[k] = R(0);
  }
};

// The j side of one pair for the half list (each pair evaluated once): the
// force on j is minus the pair force on i (f holds the pair force on i; the
// consumer subtracts it), and j's torque about its COM
// follows from the site forces being central: (d + r_ia - r_jb) x f_ab = 0, so
// sum_ab r_jb x (-f_ab) = -sum_a (d + r_ia) x F_ia with F_ia the (switched)
// force on i's site a from all of j's sites.  The COM switch force acts along
// d and turns neither molecule.
template <class R>
struct PairJ {
  R f[3];
  R t[3];
};

template <class M, class R, int NW, bool HALF = false>
__device__ __forceinline__ void pair_math(const R d[3], R dd, const R (&ri)[M::NQ + 1][3],
                                          const R (&rj)[M::NQ + 1][3], const PairConst& pc, R rin2, R rin, R rout,
                                          R c1, R c2, R trl, R tru, R tw3, Acc<M, R, NW>& acc,
                                          PairJ<R>* pj = nullptr) {
  R hh, dh;
  switch_fn<R>(dd, rin2, rin, rout, c1, c2, hh, dh);
  // LJ site pair (site 0 - site 0)
  R v[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) v[k] = d[k] + ri[0][k] - rj[0][k];
  R inv = rcp_r(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  R d6 = inv * inv * inv, d12 = d6 * d6;
  const R aa = Prm<R>::aa(pc), bb = Prm<R>::bb(pc);
  R elj = aa * d12 + bb * d6;
  R flj = inv * (aa * R(12) * d12 + bb * R(6) * d6);
  R fsite[M::NQ + 1][3];
#pragma unroll
  for (int k = 0; k < 3; ++k) fsite[0][k] = v[k] * flj;
  // charged site pairs
  R ec = R(0);
#pragma unroll
  for (int a = 1; a <= M::NQ; ++a) {
    R fa0 = R(0), fa1 = R(0), fa2 = R(0);
#pragma unroll
    for (int b = 1; b <= M::NQ; ++b) {
      R x = d[0] + ri[a][0] - rj[b][0];
      R y = d[1] + ri[a][1] - rj[b][1];
      R z = d[2] + ri[a][2] - rj[b][2];
      R rr = rsqrt_r(x * x + y * y + z * z);
      R e0 = Prm<R>::qq(pc, a - 1, b - 1) * rr;
      R f0 = e0 * rr * rr;
      ec += e0;
      fa0 += x * f0; fa1 += y * f0; fa2 += z * f0;
    }
    fsite[a][0] = fa0; fsite[a][1] = fa1; fsite[a][2] = fa2;
  }
  R scc = hh, dcc = dh;
  if (M::TAPER) {
    R s12, ds12;
    taper_fn<R>(dd, trl, tru, tw3, s12, ds12);
    scc = hh * s12;
    dcc = dh * s12 + hh * ds12;
  }
  R fcom = dh * elj + dcc * ec;
  R fp[3];
  R us[M::NQ + 1][3];   // switched site forces on i
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    R t = hh * fsite[0][k];
    us[0][k] = t;
    acc.fs[0][k] += t;
    R sum = t;
#pragma unroll
    for (int a = 1; a <= M::NQ; ++a) {
      R u = scc * fsite[a][k];
      us[a][k] = u;
      acc.fs[a][k] += u;
      sum += u;
    }
    R c = fcom * d[k];
    acc.fc[k] += c;
    fp[k] = sum + c;
  }
  acc.e += hh * elj + scc * ec;
  if constexpr (HALF) {
    R tx = R(0), ty = R(0), tz = R(0);
#pragma unroll
    for (int a = 0; a <= M::NQ; ++a) {
      const R vx = d[0] + ri[a][0], vy = d[1] + ri[a][1], vz = d[2] + ri[a][2];
      tx += vz * us[a][1] - vy * us[a][2];
      ty += vx * us[a][2] - vz * us[a][0];
      tz += vy * us[a][0] - vx * us[a][1];
    }
    pj->t[0] = tx; pj->t[1] = ty; pj->t[2] = tz;
    pj->f[0] = fp[0]; pj->f[1] = fp[1]; pj->f[2] = fp[2];
  }
  if constexpr (NW == 9) {
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = 0; b < 3; ++b) acc.w[3 * a + b] += d[a] * fp[b];
  } else {
    acc.w[0] += d[0] * fp[0] + d[1] * fp[1] + d[2] * fp[2];
  }
}

__device__ __forceinline__ double shfl_xor_d(double v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }

template <int LPI>
__device__ __forceinline__ double group_sum(double v) {
#pragma unroll
  for (int m = LPI / 2; m >= 1; m >>= 1) v += shfl_xor_d(v, m);
  return v;
}


}  // namespace g6
