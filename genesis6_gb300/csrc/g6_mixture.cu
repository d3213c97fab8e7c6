// g6_mixture.cu -- two-component (hetero) pair search and forces on the
// reference's site store.
//
// The reference handles a mixture by calling its pair search and force once
// per component pair: Grid_NeighborList with the hetero stencil
// (NeighborCell_ListHetero, GridModule.F90:757-899) and two address tables,
// Interaction_Compress2 and CutOff_Dimmer2, then force(iv, mi, mj, ...)
// (Interaction2.F90:19-68), which picks the TIP4P-OPLS methanol hand kernel
// (interaction_force_tip4p_oplsmeoh, OPLSMeOHModule.F90:1201-1480) on the
// custom path and StdForce (StdInteraction.F90:63-630) otherwise.
//
// k_het_assign / k_pairset_hetero: the exact pair set (i in A, j in B) with the
//   reference's FP64 cell index and cutoff arithmetic, two passes (count, scan,
//   write) in cell / molecule / stencil / molecule order.
// k_table_force: one thread per pair of a caller's list, the pair's site loop
//   over a table of site pairs (charge product, LJ aa/bb) as StdForce walks
//   it, FP64, site forces scattered with atomics into one global site store
//   (component i at site offset offi, j at offj), per-pair energies and the
//   block-reduced virial.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "g6_internal.cuh"

namespace g6 {

// ---------------------------------------------------------------------------
// Hetero pair search
// ---------------------------------------------------------------------------
struct HetGrid {
  int nd[3];
  double L[3], iL[3], icell[3];
};

// Reference cell index (0-based) of one COM: box_renormalize, then
// dnint(delta * (1/cell)) wrapped into [0, ndiv) (GridModule.F90:503-531).
__device__ __forceinline__ int het_cell(const HetGrid& g, double x, double y, double z) {
  const double c[3] = {x, y, z};
  int j[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    double delta = c[d];
    const double cellv = xmul(xdnint(xmul(delta, g.iL[d])), g.L[d]);
    delta = xsub(delta, cellv);
    int jj = (int)xdnint(xmul(delta, g.icell[d]));
    if (jj < 0) jj += g.nd[d];
    if (jj >= g.nd[d]) jj -= g.nd[d];
    if (!(jj >= 0 && jj < g.nd[d])) jj = 0;
    j[d] = jj;
  }
  return (j[2] * g.nd[1] + j[1]) * g.nd[0] + j[0];
}

// Cell of every molecule (com row-major (n,3)) and the cell populations.
__global__ void k_het_assign(HetGrid g, int n, const double* com, int* cell, int* count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int c = het_cell(g, com[3 * i], com[3 * i + 1], com[3 * i + 2]);
  cell[i] = c;
  atomicAdd(&count[c], 1);
}

// Residents of each cell: scattered to free slots, then put in molecule
// order (Address_Assign keeps molecule order) by one thread per cell.
__global__ void k_het_fill(int n, const int* cell, const int* start, int* fillc, int* cellmol) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int c = cell[i];
  cellmol[start[c] + atomicAdd(&fillc[c], 1)] = i;
}
__global__ void k_het_sort(int ncell, const int* start, int* cellmol) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncell) return;
  for (int k = start[c] + 1; k < start[c + 1]; ++k) {
    const int v = cellmol[k];
    int q = k - 1;
    while (q >= start[c] && cellmol[q] > v) { cellmol[q + 1] = cellmol[q]; --q; }
    cellmol[q + 1] = v;
  }
}

struct HetPairArgs {
  HetGrid g;
  int na;
  const double* ca;       // (na,3)
  const double* cb;       // (nb,3)
  const int* cella;
  const int* startb;
  const int* cellmolb;
  int nsten;
  int sten[27][3];        // cell offsets in [0, ndiv)
  double rout2, rin2, rin, rout, c1, c2;
  long long* cnt;         // na + 1 (pass 0 counts; scanned into offsets)
  const long long* off;
  int pass;
  int *pi, *pj;
  double *ox, *oy, *oz, *hh, *dh;
};

__device__ __forceinline__ void het_switch(double dd, const HetPairArgs& a, double& hh, double& dh) {
  hh = 1.0; dh = 0.0;
  if (dd > a.rin2) {   // cutoff_func CutoffModule.F90:38-59
    const double dr = __dsqrt_rn(dd);
    const double u = xsub(dr, a.rout), l = xsub(dr, a.rin), uu = xmul(u, u), ll = xmul(l, l);
    const double poly = xadd(xsub(xmul(10.0, ll), xmul(xmul(5.0, u), l)), uu);
    hh = xmul(xmul(xmul(a.c1, uu), u), poly);
    dh = -__ddiv_rn(xmul(xmul(a.c2, uu), ll), dr);
  }
}

__global__ void k_pairset_hetero(HetPairArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.na) return;
  const HetGrid& g = a.g;
  const int c = a.cella[i];
  const int cx = c % g.nd[0], cy = (c / g.nd[0]) % g.nd[1], cz = c / (g.nd[0] * g.nd[1]);
  const double ci[3] = {a.ca[3 * i], a.ca[3 * i + 1], a.ca[3 * i + 2]};
  long long cnt = 0;
  long long w = a.pass ? a.off[i] : 0;
  for (int e = 0; e < a.nsten; ++e) {
    const int nx = (cx + a.sten[e][0]) % g.nd[0], ny = (cy + a.sten[e][1]) % g.nd[1], nz = (cz + a.sten[e][2]) % g.nd[2];
    const int cj = (nz * g.nd[1] + ny) * g.nd[0] + nx;
    for (int k = a.startb[cj]; k < a.startb[cj + 1]; ++k) {
      const int j = a.cellmolb[k];
      const double cj3[3] = {a.cb[3 * j], a.cb[3 * j + 1], a.cb[3 * j + 2]};
      double o[3], d[3];
      const double dd = exact_dd(ci, cj3, g.L, g.iL, o, d);
      if (!(dd < a.rout2)) continue;   // Interaction_Compress2: strict
      if (a.pass) {
        double h, dh;
        het_switch(dd, a, h, dh);
        a.pi[w] = i; a.pj[w] = j;
        a.ox[w] = o[0]; a.oy[w] = o[1]; a.oz[w] = o[2];
        a.hh[w] = h; a.dh[w] = dh;
        ++w;
      }
      ++cnt;
    }
  }
  if (!a.pass) a.cnt[i] = cnt;
}

// Exclusive scan of n counts (one block) into out[0..n]; out[n] = total.
template <class T>
__global__ void __launch_bounds__(1024) k_het_scan(const T* count, T* out, int n) {
  __shared__ T part[1024];
  const int t = threadIdx.x;
  const int per = (n + 1023) / 1024;
  const int b = t * per, e = min(n, b + per);
  T s = 0;
  for (int k = b; k < e; ++k) s += count[k];
  part[t] = s;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    const T v = t >= o ? part[t - o] : 0;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  T run = t == 0 ? 0 : part[t - 1];
  for (int k = b; k < e; ++k) { out[k] = run; run += count[k]; }
  if (t == 1023) out[n] = part[1023];
}

// ---------------------------------------------------------------------------
// Site-pair-table force
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_table_force(TableArgs a) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double w[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  if (k < a.npair) {
    const int ii = a.offi + a.pi[k] * a.nsi, jj = a.offj + a.pj[k] * a.nsj;
    const double ox = a.ox[k], oy = a.oy[k], oz = a.oz[k];
    double fi[TMAXS][3], fj[TMAXS][3];
#pragma unroll
    for (int s = 0; s < TMAXS; ++s)
#pragma unroll
      for (int c = 0; c < 3; ++c) fi[s][c] = fj[s][c] = 0.0;
    double e = 0.0;
    for (int t = 0; t < a.ntab; ++t) {   // StdInteraction.F90:201-560, one site pair at a time
      const int si = a.si[t], sj = a.sj[t];
      const double dx = a.x[ii + si] - a.x[jj + sj] - ox, dy = a.y[ii + si] - a.y[jj + sj] - oy,
                   dz = a.z[ii + si] - a.z[jj + sj] - oz;
      const double dd = 1.0 / (dx * dx + dy * dy + dz * dz);
      double e0 = 0.0, f0 = 0.0;
      if (a.kind[t] & 1) {
        const double r = sqrt(dd);
        e0 = a.qq[t] * r;
        f0 = a.qq[t] * r * dd;
      }
      if (a.kind[t] & 2) {
        const double d6 = dd * dd * dd, d12 = d6 * d6;
        e0 = e0 + a.aa[t] * d12 + a.bb[t] * d6;
        f0 = f0 + dd * (a.aa[t] * 12.0 * d12 + a.bb[t] * 6.0 * d6);
      }
      e += e0;
      // per-site sums in registers: the site index is a runtime value, so
      // the register arrays are updated through a small unrolled switch
#pragma unroll
      for (int s = 0; s < TMAXS; ++s) {
        if (s == si) { fi[s][0] += dx * f0; fi[s][1] += dy * f0; fi[s][2] += dz * f0; }
        if (s == sj) { fj[s][0] += dx * f0; fj[s][1] += dy * f0; fj[s][2] += dz * f0; }
      }
    }
    const double hh = a.hh[k];
    a.ep[k] = e * hh;
    if (a.with_force) {
      const int lasti = a.nsi - 1, lastj = a.nsj - 1;
      const double d00[3] = {a.x[ii + lasti] - a.x[jj + lastj] - ox, a.y[ii + lasti] - a.y[jj + lastj] - oy,
                             a.z[ii + lasti] - a.z[jj + lastj] - oz};
      const double dh = a.dh[k];
      double vr[3] = {0.0, 0.0, 0.0};
#pragma unroll
      for (int s = 0; s < TMAXS; ++s) {
        const bool ci = s < a.nsi, cj = s < a.nsj;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          double u = fi[s][c] * hh, v = fj[s][c] * hh;
          if (s == lasti) u += dh * d00[c] * e;    // COM switch force (StdInteraction.F90:545-559)
          if (s == lastj) v += dh * d00[c] * e;
          if (ci) { vr[c] += u; if (u != 0.0) atomicAdd(c == 0 ? &a.fx[ii + s] : c == 1 ? &a.fy[ii + s] : &a.fz[ii + s], u); }
          if (cj && v != 0.0) atomicAdd(c == 0 ? &a.fx[jj + s] : c == 1 ? &a.fy[jj + s] : &a.fz[jj + s], -v);
        }
      }
#pragma unroll
      for (int p = 0; p < 3; ++p)
#pragma unroll
        for (int q = 0; q < 3; ++q) w[3 * p + q] = d00[p] * vr[q];
    }
  }
  if (a.with_force) {
    __shared__ double sw[9][4];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int c = 0; c < 9; ++c) {
      double v = w[c];
#pragma unroll
      for (int m = 16; m >= 1; m >>= 1) v += __shfl_xor_sync(0xffffffffu, v, m);
      if (lane == 0) sw[c][warp] = v;
    }
    __syncthreads();
    if (threadIdx.x < 9) {
      double v = 0.0;
      for (int q = 0; q < (int)(blockDim.x >> 5); ++q) v += sw[threadIdx.x][q];
      atomicAdd(&a.vir[threadIdx.x], v);
    }
  }
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
static inline double pw6(double x) { const double x2 = x * x; return x2 * x2 * x2; }

// Site-pair table of force(iv, mi, mj, ...): StdForce's table
// (StdInteraction.F90:201-222: every site pair with a charge product or an LJ
// pair, LB mixing) or, on the custom path for TIP4P with OPLS methanol, the
// constants of interaction_force_tip4p_oplsmeoh (OPLSMeOHModule.F90:1-7,
// 1189-1198: water O against Me and O with LB-mixed EPSWO/SIGWO, the TIP4P
// charges against Me, O, H).  Returns false when the table does not fit.
bool pair_table2(const ModelHost& mi, const ModelHost& mj, int path, TableArgs& t) {
  t.ntab = 0;
  auto push = [&](int si, int sj, double qq, double aa, double bb, int kind) {
    if (t.ntab >= TMAX) return false;
    t.si[t.ntab] = si; t.sj[t.ntab] = sj; t.qq[t.ntab] = qq; t.aa[t.ntab] = aa; t.bb[t.ntab] = bb;
    t.kind[t.ntab] = kind;
    ++t.ntab;
    return true;
  };
  if (path == G6_PATH_CUSTOM && mi.model == G6_TIP4P && mj.model == G6_OPLSMEOH) {
    const double EPSWO = mi.rparam[0][1], SIGWO = mi.rparam[0][2];
    const double EPSM = mj.rparam[0][1], SIGM = mj.rparam[0][2], EPSO = mj.rparam[1][1], SIGO = mj.rparam[1][2];
    const double aomxs = pw6((SIGWO + SIGM) * 0.5) * pw6((SIGWO + SIGM) * 0.5) * 100.0;
    const double bomxs = pw6((SIGWO + SIGM) * 0.5) * 100.0;
    const double aooxs = pw6((SIGWO + SIGO) * 0.5) * pw6((SIGWO + SIGO) * 0.5) * 100.0;
    const double booxs = pw6((SIGWO + SIGO) * 0.5) * 100.0;
    if (!push(0, 0, 0.0, 4.0 * std::sqrt(EPSWO * EPSM) * aomxs, -4.0 * std::sqrt(EPSWO * EPSM) * bomxs, 2)) return false;
    if (!push(0, 1, 0.0, 4.0 * std::sqrt(EPSWO * EPSO) * aooxs, -4.0 * std::sqrt(EPSWO * EPSO) * booxs, 2)) return false;
    for (int a = 1; a <= 3; ++a)
      for (int b = 0; b < 3; ++b)
        if (!push(a, b, mi.rparam[a][0] * mj.rparam[b][0] * COEFF * 100.0, 0.0, 0.0, 1)) return false;
    return true;
  }
  for (int is = 0; is < mi.nref; ++is)
    for (int js = 0; js < mj.nref; ++js) {
      const double qq = mi.rparam[is][0] * mj.rparam[js][0] * COEFF * KX2X * J2I;
      const double ee = mi.rparam[is][1] * mj.rparam[js][1];
      if (qq == 0.0 && ee == 0.0) continue;
      double aa = 0.0, bb = 0.0;
      if (ee != 0.0) {
        const double ljeps = std::sqrt(ee), ljsig = pw6((mi.rparam[is][2] + mj.rparam[js][2]) * 0.5);
        aa = 4.0 * ljeps * ljsig * ljsig * KX2X * J2I;
        bb = -4.0 * ljeps * ljsig * KX2X * J2I;
      }
      if (!push(is, js, qq, aa, bb, (qq != 0.0 ? 1 : 0) | (ee != 0.0 ? 2 : 0))) return false;
    }
  return true;
}

cudaError_t launch_table_force(const TableArgs& a, cudaStream_t s) {
  const long long blocks = (a.npair + 127) / 128;
  if (blocks == 0) return cudaSuccess;
  k_table_force<<<(unsigned)blocks, 128, 0, s>>>(a);
  return cudaGetLastError();
}

// NeighborCell_ListHetero (maxradius == 0): offsets -1..1 per axis clipped to
// (ndiv-1)/2 and -ndiv/2, as cell offsets in [0, ndiv).
int hetero_stencil(const int nd[3], int st[27][3]) {
  int nmax[3], nmin[3];
  for (int d = 0; d < 3; ++d) {
    nmax[d] = std::min(1, (nd[d] - 1) / 2);
    nmin[d] = std::max(-1, -(nd[d] / 2));
  }
  int k = 0;
  for (int jz = nmin[2]; jz <= nmax[2]; ++jz)
    for (int jy = nmin[1]; jy <= nmax[1]; ++jy)
      for (int jx = nmin[0]; jx <= nmax[0]; ++jx) {
        st[k][0] = jx < 0 ? jx + nd[0] : jx;
        st[k][1] = jy < 0 ? jy + nd[1] : jy;
        st[k][2] = jz < 0 ? jz + nd[2] : jz;
        ++k;
      }
  return k;
}

// The hetero pair search on device arrays (ca (na,3), cb (nb,3)); scratch
// holds the cell tables; pair outputs are allocated by the caller through
// `grow` once the count is known.  Returns the pair count through *total.
cudaError_t launch_pairsearch_hetero(const double L[3], const double req[3], const CutConst& cc, int na,
                                     const double* ca, int nb, const double* cb, char* scratch, size_t scratch_bytes,
                                     long long* total, cudaStream_t s, HetOutputs& out, bool write) {
  HetPairArgs a;
  std::memset(&a, 0, sizeof a);
  int ncell = 1;
  for (int d = 0; d < 3; ++d) {
    int nd = (int)(L[d] / req[d]);
    a.g.nd[d] = nd < 1 ? 1 : nd;
    const double cell = L[d] / a.g.nd[d];
    a.g.L[d] = L[d]; a.g.iL[d] = 1.0 / L[d]; a.g.icell[d] = 1.0 / cell;
    ncell *= a.g.nd[d];
  }
  a.nsten = hetero_stencil(a.g.nd, a.sten);
  char* p = scratch;
  auto take = [&](size_t b) { char* q = p; p += (b + 255) / 256 * 256; return (void*)q; };
  int* cella = (int*)take((size_t)na * 4);
  int* cellb = (int*)take((size_t)nb * 4);
  int* countb = (int*)take((size_t)(ncell + 1) * 4);
  int* startb = (int*)take((size_t)(ncell + 1) * 4);
  int* cellmolb = (int*)take((size_t)nb * 4);
  int* fillb = (int*)take((size_t)(ncell + 1) * 4);
  long long* cnt = (long long*)take((size_t)(na + 1) * 8);
  long long* off = (long long*)take((size_t)(na + 1) * 8);
  if ((size_t)(p - scratch) > scratch_bytes) return cudaErrorInvalidValue;
  cudaError_t e = cudaMemsetAsync(countb, 0, (size_t)(ncell + 1) * 4, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(fillb, 0, (size_t)(ncell + 1) * 4, s);
  if (e != cudaSuccess) return e;
  if (na > 0) k_het_assign<<<(na + 127) / 128, 128, 0, s>>>(a.g, na, ca, cella, fillb);   // (A's counts unused)
  if (nb > 0) k_het_assign<<<(nb + 127) / 128, 128, 0, s>>>(a.g, nb, cb, cellb, countb);
  k_het_scan<int><<<1, 1024, 0, s>>>(countb, startb, ncell);
  e = cudaMemsetAsync(fillb, 0, (size_t)(ncell + 1) * 4, s);
  if (e != cudaSuccess) return e;
  if (nb > 0) k_het_fill<<<(nb + 127) / 128, 128, 0, s>>>(nb, cellb, startb, fillb, cellmolb);
  k_het_sort<<<(ncell + 127) / 128, 128, 0, s>>>(ncell, startb, cellmolb);
  a.na = na; a.ca = ca; a.cb = cb; a.cella = cella; a.startb = startb; a.cellmolb = cellmolb;
  a.rout2 = cc.rout2; a.rin2 = cc.rin2; a.rin = cc.rin; a.rout = cc.rout; a.c1 = cc.c1; a.c2 = cc.c2;
  a.cnt = cnt; a.off = off;
  if (!write) {
    a.pass = 0;
    if (na > 0) k_pairset_hetero<<<(na + 127) / 128, 128, 0, s>>>(a);
    k_het_scan<long long><<<1, 1024, 0, s>>>(cnt, off, na);
    e = cudaMemcpyAsync(total, off + na, sizeof(long long), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return e == cudaSuccess ? cudaGetLastError() : e;
  }
  a.pass = 1;
  a.pi = out.pi; a.pj = out.pj; a.ox = out.ox; a.oy = out.oy; a.oz = out.oz; a.hh = out.hh; a.dh = out.dh;
  if (na > 0) k_pairset_hetero<<<(na + 127) / 128, 128, 0, s>>>(a);
  return cudaGetLastError();
}

size_t pairsearch_hetero_scratch(const double L[3], const double req[3], int na, int nb) {
  size_t ncell = 1;
  for (int d = 0; d < 3; ++d) ncell *= (size_t)std::max(1, (int)(L[d] / req[d]));
  auto al = [](size_t b) { return (b + 255) / 256 * 256; };
  return al((size_t)na * 4) + al((size_t)nb * 4) + 3 * al((ncell + 1) * 4) + al((size_t)nb * 4) +
         2 * al((size_t)(na + 1) * 8);
}

}  // namespace g6
