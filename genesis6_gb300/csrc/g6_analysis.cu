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
// The bin of a site pair comes from FP32 arithmetic (COM difference in FP64,
// rounded once to FP32, then FP32 site offsets): for separations below 32 A
// (cutoffs up to ~30 A) that distance is within 1e-5 A of the FP64 one (three
// roundings of at most half an FP32 ulp of 32 A per component, plus the norm),
// so the bin is the FP64 bin unless the distance lies within RDF_TOL = 5e-5 A
// of a bin boundary, where the FP64 distance of the reference's formula
// decides.  An FP64 instruction issues at 1/64 of the FP32 rate on this GPU.
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
      a.off[((size_t)i * a.nsite + s) * 3 + k] = (float)o;
    }
  }
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

__global__ void __launch_bounds__(256) k_rdf(RdfArgs a) {
  extern __shared__ unsigned int s_hist[];
  const int ns = a.nsite, nb = a.nbin;
  const int per_rep = ns * ns * nb, total = a.nrep * per_rep;
  for (int k = threadIdx.x; k < total; k += blockDim.x) s_hist[k] = 0u;
  __syncthreads();
  const double w = a.binwidth;   // divided by, as the reference does
  const float fw = (float)w, finv = (float)(1.0 / w), fmin = (float)a.minvalue;
  const int n = a.n;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < a.npair;
       p += (long long)gridDim.x * blockDim.x) {
    const int i = a.pi[p], j = a.pj[p];
    const int r = replica_of(a.off_rep, a.nrep, i);
    const double ox = a.ox[p], oy = a.oy[p], oz = a.oz[p];
    const float dc[3] = {(float)sub(sub(a.st[i], a.st[j]), ox), (float)sub(sub(a.st[n + i], a.st[n + j]), oy),
                         (float)sub(sub(a.st[2 * n + i], a.st[2 * n + j]), oz)};
    const float* fi = a.off + (size_t)i * ns * 3;
    const float* fj = a.off + (size_t)j * ns * 3;
    for (int sa = 0; sa < ns; ++sa) {
      const float ua[3] = {dc[0] + fi[3 * sa], dc[1] + fi[3 * sa + 1], dc[2] + fi[3 * sa + 2]};
      for (int sb = 0; sb < ns; ++sb) {
        const float ex = ua[0] - fj[3 * sb], ey = ua[1] - fj[3 * sb + 1], ez = ua[2] - fj[3 * sb + 2];
        const float t = (sqrtf(ex * ex + ey * ey + ez * ez) - fmin) * finv;
        const float fl = floorf(t);
        int bin;
        if (!a.fp64_only && fabsf(t - fl - 0.5f) * fw > RDF_TOL) {
          bin = (int)fl + (t - fl > 0.5f ? 1 : 0);
        } else {   // near a bin boundary: the reference's FP64 distance decides
          const double* xi = a.pos + ((size_t)i * ns + sa) * 3;
          const double* xj = a.pos + ((size_t)j * ns + sb) * 3;
          const double dx = sub(sub(xi[0], xj[0]), ox);
          const double dy = sub(sub(xi[1], xj[1]), oy);
          const double dz = sub(sub(xi[2], xj[2]), oz);
          const double rr = __dsqrt_rn(add(add(mul(dx, dx), mul(dy, dy)), mul(dz, dz)));
          bin = (int)round(__ddiv_rn(sub(rr, a.minvalue), w));   // nint: half away from zero
        }
        if (bin >= 0 && bin < nb) {
          const int lo = sa < sb ? sa : sb, hi = sa < sb ? sb : sa;
          atomicAdd(&s_hist[(size_t)r * per_rep + (lo * ns + hi) * nb + bin], 1u);
        }
      }
    }
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
  cudaError_t e = cudaFuncSetAttribute(k_rdf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const long long want = (a.npair + 255) / 256;
  const int blocks = (int)(want < 4LL * num_sms ? want : 4LL * num_sms);   // a few blocks per SM
  k_rdf<<<blocks, 256, smem, s>>>(a);
  return cudaGetLastError();
}

}  // namespace g6
