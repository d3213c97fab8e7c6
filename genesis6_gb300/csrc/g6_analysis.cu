// g6_analysis.cu -- trajectory analysis on the device pair set.
//
// Site-site radial histograms (radialdistrib, RDFModule.F90:101-137): for every
// molecule pair of the within-cutoff pair set and every pair of reference
// sites (a on one molecule, b on the other), the distance
//     dx = x(i, a) - x(j, b) - ox,   r = sqrt(dx^2 + dy^2 + dz^2)
// goes to bin nint((r - minvalue) / binwidth) when that bin exists
// (Histogram_Accumulate, DistribModule.F90:149-158; nint rounds half away
// from zero).  The reference keeps one histogram per ordered pair of site
// types, which depends on which molecule of a pair its list names first; the
// count here is kept per unordered pair of sites (a <= b), the sum of both
// orders, which does not.  Site positions are FP64, com + R(q) body with the
// rotation matrix of rigid_setmatrix (RigidModule.F90:62-83) and every product
// and sum rounded separately (no contraction), the order of the CPU reference.
//
// The bin of a site pair comes from FP32 arithmetic: the COM difference is the
// exact difference of 32-bit fixed-point COM words (the minimum image by
// wrap-around) converted once to FP32, then the FP32 site offsets are added.
// For separations below 32 A (cutoffs up to ~30 A) that distance is within
// 1e-5 A of the FP64 one, so the bin is the FP64 bin unless the distance lies
// within RDF_TOL = 5e-5 A of a bin boundary.  Those cases (~0.2% at 0.05 A
// bins) are queued per block and then decided by the FP64 distance of the
// reference's formula, one case per thread, so that an FP64 instruction (1/64
// of the FP32 issue rate on this GPU) serves 32 of them.
#include <cuda_runtime.h>

#include "g6_internal.cuh"

namespace g6 {

__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }

__global__ void k_site_positions(SitePosArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const double qa = a.st[(size_t)33 * a.n + i], qb = a.st[(size_t)34 * a.n + i];
  const double qc = a.st[(size_t)35 * a.n + i], qd = a.st[(size_t)36 * a.n + i];
  double t[9];
  t[0] = sub(add(mul(qa, qa), mul(qb, qb)), add(mul(qc, qc), mul(qd, qd)));
  t[1] = mul(-2.0, add(mul(qa, qd), mul(qb, qc)));
  t[2] = mul(2.0, sub(mul(qb, qd), mul(qa, qc)));
  t[3] = mul(2.0, sub(mul(qa, qd), mul(qb, qc)));
  t[4] = sub(add(mul(qa, qa), mul(qc, qc)), add(mul(qb, qb), mul(qd, qd)));
  t[5] = mul(-2.0, add(mul(qa, qb), mul(qc, qd)));
  t[6] = mul(2.0, add(mul(qa, qc), mul(qb, qd)));
  t[7] = mul(2.0, sub(mul(qa, qb), mul(qc, qd)));
  t[8] = sub(add(mul(qa, qa), mul(qd, qd)), add(mul(qb, qb), mul(qc, qc)));
  const double c[3] = {a.st[i], a.st[(size_t)a.n + i], a.st[(size_t)2 * a.n + i]};
  for (int s = 0; s < a.nsite; ++s) {
    const double bx = a.body[s][0], by = a.body[s][1], bz = a.body[s][2];
    for (int k = 0; k < 3; ++k) {
      const double o = add(add(mul(t[3 * k], bx), mul(t[3 * k + 1], by)), mul(t[3 * k + 2], bz));
      a.pos[((size_t)i * a.nsite + s) * 3 + k] = add(c[k], o);
      if (s + 1 < a.nsite) a.off[(size_t)i * 16 + 3 * s + k] = (float)o;   // the COM site's offset is 0
    }
  }
  for (int k = 3 * (a.nsite - 1); k < 16; ++k) a.off[(size_t)i * 16 + k] = 0.0f;
  const int r = a.rep.mol_rep[i];
  for (int k = 0; k < 3; ++k) a.fixc[(size_t)i * 4 + k] = to_fixed(c[k], a.rep.invL[3 * r + k]);
  a.fixc[(size_t)i * 4 + 3] = 0u;
}

// replica of molecule i: the last r with off[r] <= i
__device__ __forceinline__ int replica_of(const int* off, int nrep, int i) {
  int lo = 0, hi = nrep - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (off[mid] <= i) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// One pair per thread (grid-stride); counts in a shared histogram of all
// replicas, added to the global int64 counts at the end of the block.
constexpr float RDF_TOL = 5e-5f;   // A: FP32 distance error bound (1e-5 A) with margin
constexpr int RDF_Q = 1024;        // queued boundary cases per block

__device__ __forceinline__ int rdf_bin64(const RdfArgs& a, long long p, int sa, int sb) {
  const int i = a.pi[p], j = a.pj[p], ns = a.nsite;
  const double* xi = a.pos + ((size_t)i * ns + sa) * 3;
  const double* xj = a.pos + ((size_t)j * ns + sb) * 3;
  const double dx = sub(sub(xi[0], xj[0]), a.ox[p]);
  const double dy = sub(sub(xi[1], xj[1]), a.oy[p]);
  const double dz = sub(sub(xi[2], xj[2]), a.oz[p]);
  const double rr = __dsqrt_rn(add(add(mul(dx, dx), mul(dy, dy)), mul(dz, dz)));
  return (int)round(__ddiv_rn(sub(rr, a.minvalue), a.binwidth));   // nint: half away from zero
}

// NS sites per molecule; each molecule's FP32 offsets are 16 floats (four
// 16-byte loads) and its fixed-point COM one 16-byte load.
template <int NS>
__global__ void __launch_bounds__(256) k_rdf(RdfArgs a) {
  extern __shared__ unsigned int s_hist[];
  __shared__ int s_nq;
  __shared__ int2 s_q[RDF_Q];   // (pair, 16 sa + sb)
  const int nb = a.nbin;
  const int per_rep = NS * NS * nb, total = a.nrep * per_rep;
  for (int k = threadIdx.x; k < total; k += blockDim.x) s_hist[k] = 0u;
  if (threadIdx.x == 0) s_nq = 0;
  __syncthreads();
  const float fw = (float)a.binwidth, finv = (float)(1.0 / a.binwidth), fmin = (float)a.minvalue;
  const float fnb = (float)nb + 1.0f;
  auto count = [&](int r, int sa, int sb, int bin) {
    if (bin >= 0 && bin < nb) {
      const int lo = sa < sb ? sa : sb, hi = sa < sb ? sb : sa;
      atomicAdd(&s_hist[(size_t)r * per_rep + (lo * NS + hi) * nb + bin], 1u);
    }
  };
  const uint4* fix4 = reinterpret_cast<const uint4*>(a.fixc);
  const float4* off4 = reinterpret_cast<const float4*>(a.off);
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < a.npair;
       p += (long long)gridDim.x * blockDim.x) {
    const int i = a.pi[p], j = a.pj[p];
    const uint4 ci = fix4[i], cj = fix4[j];
    // offsets of sites 0..NS-2, then the COM site's zero offset
    float oi[3 * NS > 16 ? 3 * NS : 16], oj[3 * NS > 16 ? 3 * NS : 16];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const float4 u = off4[(size_t)i * 4 + q], v = off4[(size_t)j * 4 + q];
      oi[4 * q] = u.x; oi[4 * q + 1] = u.y; oi[4 * q + 2] = u.z; oi[4 * q + 3] = u.w;
      oj[4 * q] = v.x; oj[4 * q + 1] = v.y; oj[4 * q + 2] = v.z; oj[4 * q + 3] = v.w;
    }
#pragma unroll
    for (int k = 3 * (NS - 1); k < 3 * NS; ++k) { oi[k] = 0.0f; oj[k] = 0.0f; }
    const int r = replica_of(a.off_rep, a.nrep, i);
    const float dc[3] = {i32_to_f32((int)(ci.x - cj.x)) * a.fscale[3 * r],
                         i32_to_f32((int)(ci.y - cj.y)) * a.fscale[3 * r + 1],
                         i32_to_f32((int)(ci.z - cj.z)) * a.fscale[3 * r + 2]};
#pragma unroll
    for (int sa = 0; sa < NS; ++sa) {
      const float ua[3] = {dc[0] + oi[3 * sa], dc[1] + oi[3 * sa + 1], dc[2] + oi[3 * sa + 2]};
#pragma unroll
      for (int sb = 0; sb < NS; ++sb) {
        const float ex = ua[0] - oj[3 * sb], ey = ua[1] - oj[3 * sb + 1], ez = ua[2] - oj[3 * sb + 2];
        const float t = (sqrtf(ex * ex + ey * ey + ez * ez) - fmin) * finv;
        if (!(t > -1.0f && t < fnb)) continue;   // far outside the histogram
        float rf;
        const int bin = nearest_i32(t, rf);
        if (!a.fp64_only && (0.5f - fabsf(t - rf)) * fw > RDF_TOL) {
          count(r, sa, sb, bin);
        } else {   // near a bin boundary: queued for the reference's FP64 distance
          const int slot = atomicAdd(&s_nq, 1);
          if (slot < RDF_Q) s_q[slot] = make_int2((int)p, 16 * sa + sb);
          else count(r, sa, sb, rdf_bin64(a, p, sa, sb));
        }
      }
    }
  }
  __syncthreads();
  const int nq = min(s_nq, RDF_Q);
  for (int q = threadIdx.x; q < nq; q += blockDim.x) {
    const int2 e = s_q[q];
    const int sa = e.y >> 4, sb = e.y & 15;
    count(replica_of(a.off_rep, a.nrep, a.pi[e.x]), sa, sb, rdf_bin64(a, e.x, sa, sb));
  }
  __syncthreads();
  for (int k = threadIdx.x; k < total; k += blockDim.x)
    if (s_hist[k]) atomicAdd(&a.hist[k], (unsigned long long)s_hist[k]);
}

// interaction_hb_by_oh_distance (InteractionModule.F90:682-777), one pair per
// thread: the squared O-H distances O(i)-H1(j), O(i)-H2(j), O(j)-H1(i),
// O(j)-H2(i) in that order (dx = x - x - o in FP64, the reference's order), the
// first strict minimum; below 2.5^2 A^2 the molecule whose hydrogen it is, is
// the donor (from), the other the acceptor (to).  Bonds are appended to the
// output (one atomic per warp), so their order is not the pair order.
__global__ void __launch_bounds__(256) k_hbonds(HbArgs a) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  bool bond = false;
  int f = -1, w = 0, t = -1;
  if (k < a.npair) {
  const int i = a.pi[k], j = a.pj[k], ns = a.nsite;
  const double o[3] = {a.ox[k], a.oy[k], a.oz[k]};
  double dmin = 1e10;
  int pmin = 0, wmin = 0, p = 0;
  for (int blk = 0; blk < 2; ++blk) {
    const int mo = blk == 0 ? i : j, mh = blk == 0 ? j : i;   // molecule of the O, of the H
    const double* xo = a.pos + ((size_t)mo * ns + a.osite) * 3;
    for (int h = 0; h < 2; ++h) {
      const double* xh = a.pos + ((size_t)mh * ns + a.hsite[h]) * 3;
      // the reference's dx = x(ii) - x(jj) - ox with ii on molecule i, jj on molecule j
      const double* xi = blk == 0 ? xo : xh;
      const double* xj = blk == 0 ? xh : xo;
      const double dx = sub(sub(xi[0], xj[0]), o[0]);
      const double dy = sub(sub(xi[1], xj[1]), o[1]);
      const double dz = sub(sub(xi[2], xj[2]), o[2]);
      const double d = add(add(mul(dx, dx), mul(dy, dy)), mul(dz, dz));
      ++p;
      if (d < dmin) { dmin = d; pmin = p; wmin = h + 1; }
    }
  }
  if (dmin < 6.25) {
    bond = true;
    f = pmin <= 2 ? j : i;
    w = wmin;
    t = pmin <= 2 ? i : j;
  }
  }
  const unsigned m = __ballot_sync(0xffffffffu, bond);
  if (m == 0u) return;
  unsigned long long base = 0;
  if (lane == __ffs(m) - 1) base = atomicAdd(a.count, (unsigned long long)__popc(m));
  base = __shfl_sync(0xffffffffu, base, __ffs(m) - 1);
  if (bond) {
    const long long pos = (long long)base + __popc(m & ((1u << lane) - 1u));
    if (pos < a.cap) { a.from[pos] = f; a.which[pos] = w; a.to[pos] = t; }
  }
}

cudaError_t launch_hbonds(const HbArgs& a, cudaStream_t s) {
  if (a.npair == 0) return cudaSuccess;
  k_hbonds<<<(unsigned)((a.npair + 255) / 256), 256, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_site_positions(const SitePosArgs& a, cudaStream_t s) {
  if (a.n == 0) return cudaSuccess;
  k_site_positions<<<(a.n + 127) / 128, 128, 0, s>>>(a);
  return cudaGetLastError();
}

size_t rdf_smem_bytes(int nrep, int nsite, int nbin) {
  return (size_t)nrep * nsite * nsite * nbin * sizeof(unsigned int);
}

cudaError_t launch_rdf(const RdfArgs& a, int num_sms, cudaStream_t s) {
  if (a.npair == 0) return cudaSuccess;
  const size_t smem = rdf_smem_bytes(a.nrep, a.nsite, a.nbin);
  const long long want = (a.npair + 255) / 256;
  const int blocks = (int)(want < 4LL * num_sms ? want : 4LL * num_sms);   // a few blocks per SM
  auto go = [&](auto kern) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<blocks, 256, smem, s>>>(a);
    return cudaGetLastError();
  };
  if (a.nsite == 4) return go(k_rdf<4>);
  if (a.nsite == 5) return go(k_rdf<5>);
  if (a.nsite == 6) return go(k_rdf<6>);
  return cudaErrorInvalidValue;
}

}  // namespace g6
