// g6_internal.cuh -- shared definitions of the sm_103a rigid-water library.
//
// Device data layout (one context = one system of nrep replicas, n molecules
// in replica order):
//   st      FP64 SoA rigid state, st[c*n + i], c in [0,53): com[3], d[5][3],
//           w[5][3], q[5][4] (the 53-double record of g6gpu.h)
//   tmat    FP64 SoA rotation matrices (body -> lab), tmat[k*n + i]
//   pk64    FP64 AoS packed pose per molecule for the site loop:
//           com[3], LJ-site offset[3], charged-site offsets[3*NQ] (+pad)
//   pk32    float4 AoS packed pose for the mixed site loop: 32-bit fixed-point
//           COM (x,y,z as uint32 in units of L/2^32), then float offsets of
//           the LJ site and the charged sites relative to the COM
//   pkq     2 float4 per molecule for the mixed list kernel: the fixed-point
//           COM words, then the float quaternion (q0..q3) and a zero; the
//           kernel rebuilds the float site offsets from the quaternion
//           (rotmat_f / site_off_f, the same roundings as the placement's)
//   fix     uint32 SoA fixed-point COM (list building and cell-free tests)
//   F, tl   per-molecule force and lab-frame torque (FP64 SoA)
//   emol, wmol  per-molecule energy (1/2 of its pair sum) and virial rows
// Cells are counting-sorted molecule ids (cell_mol) with start offsets; the
// neighbour list is a fixed-capacity row per molecule (nbr[i*cap + k]).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/g6gpu.h"

namespace g6 {

constexpr int REC = 53;
constexpr int MAXSITE = 6;  // sites per molecule including the COM site
constexpr int MAXQ = 4;     // charged sites per molecule
constexpr int MAXREP_PER_BLOCK = 8;
constexpr int RED_BLOCK = 64;    // block size of the per-molecule update kernels (FP64-bound: spread over SMs)
constexpr int NRED = 5;          // reduced quantities per replica: Epot, virial trace, sum |d1|^2, sum I w^2, pairs
// Mixed-precision MD keeps the small Gear terms in a float SoA (stf[c*n + i]):
// d2..d5 (com), w2..w5 (angular velocity) and the quaternion stacks q2..q5.
constexpr int STF_D2 = 0, STF_W2 = 12, STF_Q2 = 24, STF_COLS = 40;

// ---------------------------------------------------------------------------
// Model constants (host computes them from the reference formulas; the device
// receives them by value in kernel arguments).
// ---------------------------------------------------------------------------
struct PairConst {
  double qq[MAXQ][MAXQ];   // charged-site pair prefactors (already x100 internal units)
  double aa, bb;           // LJ site pair: e = aa/r^12 + bb/r^6
  float fqq[MAXQ][MAXQ];
  float faa, fbb;
  int taper;               // ST2 Coulomb taper (force_st2 / pairpotential_st2)
  double rl, ru, w3;       // taper range and (ru-rl)^3
  float frl, fru, fw3;
};

struct CutConst {
  double rin, rout, rin2, rout2, c1, c2;
  float frin, frout, frin2, frout2, fc1, fc2;
};

// Per-replica geometry of one cell grid.
struct GridDev {
  int ncell_total;
  const int* nd;         // 3*nrep
  const double* cell;    // 3*nrep cell edge
  const double* icell;   // 3*nrep 1/cell
  const int* cell_off;   // nrep+1
};

struct RepDev {
  int nrep;
  const int* off;        // nrep+1 molecule offsets
  const int* mol_rep;    // n
  const double* L;       // 3*nrep
  const double* invL;    // 3*nrep
  const float* fscale;   // 3*nrep  L / 2^32
};

// ---------------------------------------------------------------------------
// Exact FP64 helpers: explicit round-to-nearest intrinsics are never fused
// into FMAs, so these reproduce the reference's separate multiply/add steps.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double xmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double xadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double xsub(double a, double b) { return __dsub_rn(a, b); }
// Fortran dnint: round half away from zero.
__device__ __forceinline__ double xdnint(double x) { return round(x); }

// ---------------------------------------------------------------------------
// Reciprocal, reciprocal square root and square root in either precision.  The
// FP32 (mixed) site loops use the single hardware instructions (PTX
// rcp/rsqrt.approx.ftz: about one ulp, no subnormal handling; squared site
// separations are far from the subnormal range); the FP64 mode keeps IEEE
// division and sqrt.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float rsqrt_r(float x) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ double rsqrt_r(double x) { return rsqrt(x); }
__device__ __forceinline__ float rcp_r(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ double rcp_r(double x) { return 1.0 / x; }
// r from r^2, and y / r
__device__ __forceinline__ void root_r(float x, float& r, float& ir) { ir = rsqrt_r(x); r = x * ir; }
__device__ __forceinline__ void root_r(double x, double& r, double& ir) { r = sqrt(x); ir = 0.0; }
__device__ __forceinline__ float div_r(float y, float, float ir) { return y * ir; }
__device__ __forceinline__ double div_r(double y, double r, double) { return y / r; }

// Minimum-image COM separation exactly as Interaction_Compress2
// (InteractionModule.F90:454-465): o = dnint(delta*invL)*L, d = delta - o,
// dd = (dx^2 + dy^2) + dz^2.
__device__ __forceinline__ double exact_dd(const double ci[3], const double cj[3], const double L[3],
                                           const double iL[3], double o[3], double d[3]) {
  for (int k = 0; k < 3; ++k) {
    double delta = xsub(ci[k], cj[k]);
    o[k] = xmul(xdnint(xmul(delta, iL[k])), L[k]);
    d[k] = xsub(delta, o[k]);
  }
  return xadd(xadd(xmul(d[0], d[0]), xmul(d[1], d[1])), xmul(d[2], d[2]));
}

// Fixed-point COM: x -> round(frac(x/L) * 2^32) as uint32.  Differences of
// two such words, read as int32, are the minimum-image separation in units of
// L/2^32.
// int32 -> float rounded once, without a conversion instruction (conversions
// issue on the FP64 pipe of this GPU): the two 16-bit halves are exact floats
// through the 1.5 * 2^23 and 2^23 bit patterns, then hi * 2^16 + lo in one fma.
__device__ __forceinline__ float i32_to_f32(int x) {
  const float fh = __int_as_float(0x4B400000 + (x >> 16)) - 12582912.0f;
  const float fl = __int_as_float(0x4B000000 + (x & 0xFFFF)) - 8388608.0f;
  return fmaf(fh, 65536.0f, fl);
}
// Nearest integer of |t| < 2^22 as an int and as a float (ties to even),
// without a conversion instruction.
__device__ __forceinline__ int nearest_i32(float t, float& rf) {
  const float m = t + 12582912.0f;
  rf = m - 12582912.0f;
  return __float_as_int(m) - 0x4B400000;
}

__device__ __forceinline__ uint32_t to_fixed(double x, double invL) {
  double f = x * invL;
  f = f - floor(f);
  unsigned long long u = __double2ull_rn(f * 4294967296.0);
  return (uint32_t)(u & 0xffffffffull);
}

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon et al., SC'11), identical to the oracle's generator.
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ void philox4x32(uint32_t c[4], uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)M0 * c[0];
    uint64_t p1 = (uint64_t)M1 * c[2];
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
    k0 += W0; k1 += W1;
  }
}
// Two uniforms in (0,1] with 53-bit resolution.
__host__ __device__ __forceinline__ void uniform2(uint64_t seed, uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                                  double out[2]) {
  uint32_t c[4] = {c0, c1, c2, c3};
  philox4x32(c, (uint32_t)seed, (uint32_t)(seed >> 32));
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    uint64_t u = ((uint64_t)(c[2 * k] >> 5) << 26) | (uint64_t)(c[2 * k + 1] >> 6);
    out[k] = ((double)u + 1.0) * (1.0 / 9007199254740992.0);
  }
}

// Physical constants (PhysConst.F90:4-62).
constexpr double PI = 3.1415926535897932;
constexpr double NA = 6.0225e23;
constexpr double KB = 1.380066e-23;
constexpr double RGAS = NA * KB;
constexpr double CA = 4.184;
constexpr double COEFF = CA * 332.17752;
constexpr double I2J = 10.0;
constexpr double J2I = 1.0 / 10.0;
constexpr double J2K = 0.120273;
constexpr double KX2X = 1000.0;
constexpr double A2P = 101326.0;
constexpr double ANG2M = 1e-10;

// Gear coefficients, PhysConst.F90:7-15
constexpr double G50 = 3.0 / 16.0, G51 = 251.0 / 360.0, G53 = 11.0 / 18.0, G54 = 1.0 / 6.0, G55 = 1.0 / 60.0;
constexpr double G40 = 251.0 / 720.0, G42 = 11.0 / 12.0, G43 = 1.0 / 3.0, G44 = 1.0 / 24.0;

// ---------------------------------------------------------------------------
// Kernel argument blocks (passed by value).
// ---------------------------------------------------------------------------
struct ForceArgs {
  int n, cap, stride_pk32;
  const double* pk64_1;   // pose buffer 1, used when ctrl != NULL and the step is odd
  const float4* pk32_1;
  const int* ctrl;
  const int* nbr;
  const int* nnb;
  RepDev rep;
  const double* pk64;
  const float4* pk32;
  PairConst pc;
  CutConst cc;
  double* F;      // 3 SoA
  double* tl;     // 3 SoA lab torque
  double* emol;   // n
  double* wmol;   // 9 SoA
  int* npair_in;  // per molecule: pairs within rc (diagnostic, optional; required by the mixed MD step)
  float4* fres;   // mixed MD step: per molecule 4 float4 of float pairs (F, energy; lab torque, virial trace)
  int ccap;       // mixed list kernel: in-range entries per molecule its shared-memory rows hold (<= cap)
  int* overflow;  // set to 1 when a row holds more in-range entries than ccap
  const float4* pkq;     // mixed list kernel: 2 float4 per molecule (fixed-point COM, float quaternion)
  const float4* pkq_1;   // the same for pose buffer 1
  float fbody[MAXSITE][3];   // body-frame site coordinates (LJ site, charged sites) as float
  float4* jacc;   // mixed MD step, half list: per molecule 2 float4 (minus its force, its lab torque) from the
                  // pairs others hold
  double* jacc64; // FP64 MD step, half list: 6 SoA columns per molecule (minus-force share, lab torque share)
  int half;       // MD step: 1 = half list (each pair once, j side by atomics), 0 = full list
  int planar;     // 3-charge model with the planar site layout of MT::PLANAR
  float band;     // mixed row test: |d^2 - rc^2| below this (A^2) is decided by the FP64 test
  float fs1[3];   // one replica: its fixed-point scales L/2^32 (rep.fscale[0..2]), read without a load
};

struct SitesArgs {
  int nsite, nq;
  int site[MAXSITE];   // reference site index of kernel site s (LJ site, charged sites)
  long long npair;
  const double *x, *y, *z;
  double *fx, *fy, *fz;
  const int *pi, *pj;
  const double *ox, *oy, *oz, *hh, *dh;
  double* ep;
  double* vir;   // 9, accumulated with atomics
  PairConst pc;
  int with_force;
};

struct CellArgs {
  int n;
  RepDev rep;
  GridDev g;
  const double* com;   // SoA (x: com[i], y: com[n+i], z: com[2n+i])
  int* cell;           // n
  int* slot;           // n
  int* count;          // ncell_total
  const int* ctrl;     // optional: ctrl[0] == 0 -> skip (no rebuild this step)
};

struct ListArgs {
  int n, cap;
  RepDev rep;
  GridDev g;
  const int* cell;
  const int* start;
  const int* cellmol;
  const uint32_t* fix;   // SoA 3n
  const uint32_t* fix1;  // buffer 1 (odd steps when ctrl != NULL)
  const double* com;     // SoA 3n (state)
  double* com_build;     // SoA 3n
  uint32_t* fix_build;   // SoA 3n fixed-point COM at the build
  float rlist2;
  int* nbr;
  int* nnb;
  int* overflow;
  const int* ctrl;
  uint4* cellfix;        // n: (fixed-point COM, molecule) of each cell-sorted slot, filled before the rows
  int half;              // 1: each row keeps only the pairs its molecule evaluates in a half-list step (half_keep)
};

// Half list: of the two row entries of a pair, molecule i keeps j when i and j
// have the same parity and j > i, or different parity and j < i, so every
// molecule keeps about half of its row whatever the index order.
__device__ __forceinline__ bool half_keep(int i, int j) { return ((i ^ j) & 1) ? (j < i) : (j > i); }

struct PairSetArgs {
  int n;
  RepDev rep;
  GridDev g;
  const int* cell;
  const int* start;
  const int* cellmol;
  const int* sten;       // (x,y,z,kind) per entry; kind 0 half shell, 1 self-mirror (j > i)
  const int* sten_off;   // nrep+1
  const double* com;     // SoA 3n
  double rout2, rin2, rin, rout, c1, c2;
  long long* cnt;        // n+1 (pass 0 writes counts; the scan turns them into offsets)
  const long long* off;  // pass 1
  int pass;
  int* pi; int* pj;
  double *ox, *oy, *oz, *hh, *dh;
};

struct ThermoDev {
  int kind;
  double temp, q, dump, inv_q;
  float fext;        // zeta0 * dt of the current step (mixed corrector)
  float fkT, frdt;   // kT and collision probability per step (mixed corrector)
  double z[5];
  double zsum;
  double rate;
};

struct PlaceArgs {
  int n, nq, npk, w64;
  RepDev rep;
  double body[MAXSITE][3];
  float fbody[MAXSITE][3];
  double* st;
  double* tmat;
  double* pk64;
  float4* pk32;
  float4* pkq;   // 2 float4 per molecule (layout above)
  uint32_t* fix;
};

struct StepArgs {
  PlaceArgs p;         // constants, the state st and pose buffer 0
  double* tmat1;       // pose buffer 1 (the buffers alternate with the step parity)
  double* pk64_1;
  float4* pk32_1;
  float4* pkq_1;
  uint32_t* fix1;
  double mass, I[3], dt;
  double inv_dt2;      // 1 / dt^2
  float fdt, fcf, fmass, fI[3];   // dt, dt^2 / (2 mass), mass, inertia as float (mixed corrector)
  const double* rfac;  // per replica: I2J*2/(RGAS*dof) (temperature), I2J/(3*A2P*V*NA*ANG2M^3) (pressure)
  const double* fixs;  // per replica and axis: 2^32 / L (fixed-point COM scale)
  const double* com_build;
  const uint32_t* fix_build;
  float* stf;          // mixed precision: float SoA of the small Gear terms (STF_*)
  double half_skin2;
  ThermoDev* th;
  double* part;        // blocks * MAXREP_PER_BLOCK * NRED
  unsigned int* gmax;  // 2 words: largest squared displacement of the steps of each parity (float bits)
  int* repcnt;         // per replica: blocks of the step that have written their partials
  double* red;         // nrep * NRED (finalize scratch)
  unsigned int* done;
  int* ctrl;           // [0] list rebuilt at the start of this step, [1] step, [2] nsteps, [3] error bits,
                       // [4] a step of this run has finished, [5] log capacity, [6] step base
  double* log;         // [step][rep][G6_LOG_WIDTH]
  unsigned long long seed;
};

struct ExchArgs {
  int nrep, parity;
  unsigned long long seed, counter;
  const double* epot;   // per replica
  double* beta;
  ThermoDev* th;
  int* accepted;
  double* scale;        // per replica velocity scale (1 if unchanged)
  int numb;             // parabolic umbrellas per replica (Umbrella.F90), 0 for none
  double* umb;          // (nrep, numb, 2): center, coefficient; swapped with beta on acceptance
  const double* op;     // (nrep, numb): the order parameters the umbrellas act on
  double* temp;         // scratch (nrep): thermostat targets, permuted with beta
  int* slot;            // scratch (nrep): replica of each temperature slot
  int* moved;           // scratch (nrep): 1 for a replica whose temperature changed
};

// ---------------------------------------------------------------------------
// Replica exchange, shared by the device kernel (one context) and the host
// plan (replicas spread over processes): replica_exchange_trial
// (Replica.F90:7-73) as the MD driver applies it (Mixture.F90:1589-1653).
// The reference keeps node_in_charge(j), the replica that holds temperature
// slot j, and tests neighbouring slots (j, jj); here the slots are the
// replicas ordered by decreasing beta (ties by index), which is
// node_in_charge for a ladder of distinct temperatures.  The pairs (j, j+1)
// with j % 2 == parity are tested in increasing j (disjoint pairs, so their
// order does not matter); pair j uses the uniform of Philox key seed, counter
// (j, counter, 0x52).  An accepted pair trades beta, the thermostat
// temperature and the umbrellas; both replicas get the velocity factor
// sqrt(T_new / T_old) and are marked moved (their Nose zeta is reset).
// ---------------------------------------------------------------------------
struct ExchangeIO {
  int nrep, parity;
  unsigned long long seed, counter;
  const double* epot;
  double* beta;
  double* temp;
  int numb;
  double* umb;
  const double* op;
  int* slot;
  double* scale;
  int* moved;
  int* accepted;   // optional: 1 for the replica in the lower slot of an accepted pair
};

__host__ __device__ inline double umbrella_sum(const ExchangeIO& x, int r, int u) {
  // coeffi (op - center)^2 of replica r's order parameters under replica u's umbrellas (Umbrella.F90:11-16)
  double a = 0.0;
  for (int k = 0; k < x.numb; ++k) {
    const double* uu = x.umb + ((size_t)u * x.numb + k) * 2;
    const double o = x.op[(size_t)r * x.numb + k];
    a = a + uu[1] * ((o - uu[0]) * (o - uu[0]));
  }
  return a;
}

__host__ __device__ inline void exchange_run(const ExchangeIO& x) {
  const int R = x.nrep;
  for (int r = 0; r < R; ++r) {
    x.scale[r] = 1.0;
    x.moved[r] = 0;
    if (x.accepted) x.accepted[r] = 0;
    x.slot[r] = r;
  }
  for (int j = 1; j < R; ++j) {   // slots: decreasing beta, stable
    const int v = x.slot[j];
    int q = j - 1;
    while (q >= 0 && x.beta[x.slot[q]] < x.beta[v]) { x.slot[q + 1] = x.slot[q]; --q; }
    x.slot[q + 1] = v;
  }
  for (int j = x.parity; j + 1 < R; j += 2) {
    const int n0 = x.slot[j], n1 = x.slot[j + 1];
    const double b0 = x.beta[n0], b1 = x.beta[n1];
    double a0 = x.epot[n0], a1 = x.epot[n1];
    if (x.numb > 0) { a0 = a0 + umbrella_sum(x, n0, n0); a1 = a1 + umbrella_sum(x, n1, n1); }
    const double acc0 = -(a0 * b0 + a1 * b1) * I2J * J2K;
    a0 = x.epot[n0]; a1 = x.epot[n1];
    if (x.numb > 0) { a0 = a0 + umbrella_sum(x, n0, n1); a1 = a1 + umbrella_sum(x, n1, n0); }
    const double acc1 = -(a0 * b1 + a1 * b0) * I2J * J2K;
    bool accept = acc0 < acc1;
    if (!accept) {
      double u[2];
      uniform2(x.seed, (uint32_t)j, (uint32_t)x.counter, (uint32_t)(x.counter >> 32), 0x52u, u);
      accept = u[0] < exp(acc1 - acc0);
    }
    if (x.accepted) x.accepted[n0] = accept ? 1 : 0;
    if (!accept) continue;
    x.beta[n0] = b1; x.beta[n1] = b0;
    for (int k = 0; k < 2 * x.numb; ++k) {
      const double t = x.umb[(size_t)n0 * x.numb * 2 + k];
      x.umb[(size_t)n0 * x.numb * 2 + k] = x.umb[(size_t)n1 * x.numb * 2 + k];
      x.umb[(size_t)n1 * x.numb * 2 + k] = t;
    }
    const double t0 = x.temp[n0], t1 = x.temp[n1];
    x.scale[n0] = sqrt(t1 / t0);
    x.scale[n1] = sqrt(t0 / t1);
    x.temp[n0] = t1; x.temp[n1] = t0;
    x.moved[n0] = 1; x.moved[n1] = 1;
    x.slot[j] = n1; x.slot[j + 1] = n0;
  }
}

// ---------------------------------------------------------------------------
// Host-side declarations shared between translation units.
// ---------------------------------------------------------------------------
// FP64 site positions of every molecule in the reference's site layout.
struct SitePosArgs {
  int n, nsite;
  double body[MAXSITE][3];
  const double* st;
  double* pos;   // (n, nsite, 3)
  float* off;    // (n, 16): R(q) body of sites 0..nsite-2 (3 floats each; the COM site's is 0) in FP32, zero padded
  uint32_t* fixc;   // (n, 4): the COM as 32-bit fixed point of its replica's box, zero padded
  RepDev rep;
};
// Site-site distance histograms over a pair set (g6_analysis.cu).
struct RdfArgs {
  long long npair;
  int nrep, nsite, nbin;
  double binwidth, minvalue;
  const int* off_rep;             // replica offsets (nrep + 1)
  const int *pi, *pj;
  const double *ox, *oy, *oz;
  const double* pos;
  const float* off;
  const uint32_t* fixc;           // COM fixed point (n, 4)
  const float* fscale;            // per replica: box edge / 2^32 (3 floats)
  int n;
  int fp64_only;                  // every distance in FP64 (cutoffs beyond the FP32 bound)
  unsigned long long* hist;       // (nrep, nsite, nsite, nbin), a <= b only
};
// Hydrogen bonds by O-H distance on a pair set (g6_analysis.cu).
struct HbArgs {
  long long npair;
  int nsite, osite, hsite[2];     // reference sites: the oxygen and the two hydrogens
  const int *pi, *pj;
  const double *ox, *oy, *oz;
  const double* pos;
  long long cap;                  // bonds the output arrays hold
  unsigned long long* count;      // bonds found (may exceed cap)
  int *from, *which, *to;         // per bond: donor, its hydrogen (1, 2), acceptor
};
cudaError_t launch_hbonds(const HbArgs& a, cudaStream_t s);

// Two-component pair lists and the site-pair-table force (g6_mixture.cu).
constexpr int TMAXS = 6;                     // sites per molecule (COM included)
constexpr int TMAX = (TMAXS - 1) * (TMAXS - 1);
struct TableArgs {
  int nsi, nsj, offi, offj, ntab;
  int si[TMAX], sj[TMAX];
  double qq[TMAX], aa[TMAX], bb[TMAX];
  int kind[TMAX];                            // bit 0: Coulomb, bit 1: LJ
  long long npair;
  const double *x, *y, *z;
  double *fx, *fy, *fz;
  const int *pi, *pj;
  const double *ox, *oy, *oz, *hh, *dh;
  double* ep;
  double* vir;
  int with_force;
};
struct HetOutputs {
  int *pi, *pj;
  double *ox, *oy, *oz, *hh, *dh;
};
struct ModelHost;
bool pair_table2(const ModelHost& mi, const ModelHost& mj, int path, TableArgs& t);
cudaError_t launch_table_force(const TableArgs& a, cudaStream_t s);
cudaError_t launch_pairsearch_hetero(const double L[3], const double req[3], const CutConst& cc, int na,
                                     const double* ca, int nb, const double* cb, char* scratch, size_t scratch_bytes,
                                     long long* total, cudaStream_t s, HetOutputs& out, bool write);
size_t pairsearch_hetero_scratch(const double L[3], const double req[3], int na, int nb);
cudaError_t launch_site_positions(const SitePosArgs& a, cudaStream_t s);
cudaError_t launch_rdf(const RdfArgs& a, int num_sms, cudaStream_t s);
size_t rdf_smem_bytes(int nrep, int nsite, int nbin);

// body/param: the kernels' site layout (LJ site, then the nq charged sites);
// rbody/rparam: the reference's site arrays (nref sites, the last one the COM);
// site[s]: reference index of kernel site s (SPC/E: the oxygen is both the LJ
// site and a charged site).
struct ModelHost {
  int model = 0, nsite = 0, nq = 0, nref = 0;
  double body[MAXSITE][3] = {};
  double param[MAXSITE][3] = {};   // q, eps, sig
  double rbody[MAXSITE][3] = {};
  double rparam[MAXSITE][3] = {};
  int site[MAXSITE] = {};
  double mass = 0, I[3] = {};
};
// charged sites of a model's kernels: 3 (TIP4P, SPC/E) or 4 (TIP5P, ST2)
inline int model_nq(int model) { return (model == G6_TIP4P || model == G6_SPCE) ? 3 : 4; }

// Band of the mixed row test (ForceArgs::band): its squared separation is off
// by less than 2 sqrt(3) rlist L/2^23 (coarse_delta drops 9 of the 32 bits of
// each fixed-point difference) plus a few FP32 roundings; 1e-3 A^2 at least.
inline float row_test_band(double rlist, double lmax) {
  const double b = 1.25 * 2.0 * 1.7320508075688772 * rlist * lmax / 8388608.0 + 1e-4;
  return (float)(b > 1e-3 ? b : 1e-3);
}

// The planar site layout of MT::PLANAR, checked on the float body coordinates.
inline bool planar_sites(int nq, const float (&b)[MAXSITE][3]) {
  if (nq != 3) return false;
  for (int s = 0; s < 4; ++s)
    if (b[s][0] != 0.0f) return false;
  return b[0][1] == 0.0f && b[1][1] == 0.0f && b[2][1] == -b[3][1] && b[2][2] == b[3][2];
}
bool make_model(int model, ModelHost& m);
void make_pair_const(const ModelHost& m, int path, PairConst& pc);
void make_cut_const(double rin, double rout, CutConst& cc);

cudaError_t launch_force(const ForceArgs& a, int model, bool mixed, int lpi, cudaStream_t s);
// Mixed-precision list kernel (g6_pairs.cu): force only, and the MD step as the
// pair kernel plus the integrator kernel (`between`, optional, is recorded
// between the two).
cudaError_t launch_pairs_force(const ForceArgs& a, int model, int lpi, cudaStream_t s);
cudaError_t launch_step_mixed(const ForceArgs& a, const StepArgs& sa, int model, int lpi, int mpw, cudaStream_t s,
                              cudaEvent_t between);
// The mixed MD step's pair kernel alone, its forces to F, tl and emol (FP64).
cudaError_t launch_step_pair_forces(const ForceArgs& a, const StepArgs& sa, int model, int lpi, cudaStream_t s);
int pairs_max_cap(int lpi);
cudaError_t launch_finish_step(const StepArgs& sa, int nrep, cudaStream_t s);
cudaError_t launch_force_sites(const SitesArgs& a, int model, cudaStream_t s);
int pk64_width(int model);
int pk32_width(int model);
cudaError_t launch_cells(const CellArgs& a, int* start, int* cellmol, cudaStream_t s);
cudaError_t launch_list(const ListArgs& a, cudaStream_t s);
int rebuild_grid_limit();
cudaError_t launch_rebuild(const CellArgs& c, const ListArgs& l, int* start, int* cellmol, int grid_limit,
                           const StepArgs* step, cudaStream_t s);
cudaError_t launch_pairset_count(PairSetArgs a, cudaStream_t s);
cudaError_t launch_pairset_write(PairSetArgs a, cudaStream_t s);
cudaError_t launch_predict_place(const PlaceArgs& a, int do_predict, ThermoDev* th, int nose_predict, cudaStream_t s);
cudaError_t launch_stf_move(double* st, float* stf, int n, int to_float, cudaStream_t s);
cudaError_t launch_begin_mixed(const PlaceArgs& a, float* stf, ThermoDev* th, double dt, cudaStream_t s);
// Host-buffer step of the mixed path: records in -> state + first predict; finish + state -> records out.
struct HostInArgs {
  const double* rec;          // the caller's records (device copy, or the page-locked buffer itself)
  double* keep;               // optional: device copy of rec kept for a repeat of the step (row overflow)
  const uint32_t* fix_build;  // fixed-point COM at the last list build
  unsigned int* gmax;         // gmax[1]: the largest squared displacement since that build (float bits)
  // optional: the run's control block read by block 0 from page-locked memory
  // into the device block (instead of a copy before the kernel); the 16-byte
  // word gmax16 holds gmax[0..3], of which gmax[1] is left to the other blocks'
  // atomics
  const uint4* ctl_up;
  uint4* ctl;
  int ctl_n16, gmax16;
};
// Optional read-back of the step's control words straight into page-locked
// memory by the replica-finish blocks of the records-out kernel (instead of a
// copy after it): per replica its thermostat and sums; block 0 also the
// control words and the overflow flag.  th_dn == nullptr: none.
struct HostOutArgs {
  double* rec;        // records out (page-locked or a device copy)
  ThermoDev* th_dn;
  double* red_dn;
  int* ctrl_dn;
  int* ovf_dn;
  const int* ovf;     // the device overflow flag
};
cudaError_t launch_host_in_mixed(const PlaceArgs& a, const HostInArgs& h, float* stf, ThermoDev* th, double dt,
                                 cudaStream_t s);
cudaError_t launch_host_out_mixed(const StepArgs& sa, const HostOutArgs& o, cudaStream_t s);
cudaError_t launch_step_fp64(const ForceArgs& f, const StepArgs& a, int model, int lpi, cudaStream_t s);
// The FP64 MD step on half rows: the pair kernel (own sums per molecule, the
// partner's share by FP64 atomics into f.jacc64), then the integrator kernel.
cudaError_t launch_step_fp64_half(const ForceArgs& f, const StepArgs& a, int model, int lpi, cudaStream_t s);
cudaError_t launch_feat_stats(const float* rec, long long nrec, float* mean, float* istd, cudaStream_t s);
cudaError_t launch_adam(float* w, const float* g, float* m, float* v, float lr, int t, cudaStream_t s);
cudaError_t launch_rec_transpose(double* aos, double* soa, int n, int to_soa, cudaStream_t s);
cudaError_t launch_exchange(const ExchArgs& a, double* st, int n, const int* mol_rep, cudaStream_t s);
cudaError_t launch_scale_velocity(double* st, int n, const int* mol_rep, const double* scale, cudaStream_t s);

}  // namespace g6
