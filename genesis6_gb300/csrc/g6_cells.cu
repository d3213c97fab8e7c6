// g6_cells.cu -- cell grid, exact pair set, and device neighbour list.
//
// K1 cell build (Address_Assign, GridModule.F90:503-552): every molecule gets
// the reference's cell index, computed with the reference's FP64 steps
// (box_renormalize, then dnint(delta * (1/cell)) wrapped into [0, ndiv)), a
// warp-aggregated atomic count per cell, an exclusive scan, a scatter, and a
// per-cell sort so that residents are listed in molecule order like the
// reference's resident table.
//
// K3 exact pair set (Grid_NeighborList GridModule.F90:557-752 +
// Interaction_Compress2 InteractionModule.F90:398-605 + CutOff_Dimmer2
// CutoffModule.F90:220-278): for every i, the half-shell stencil cells and the
// self-mirror cells with j > i, the strict FP64 test dd < rc^2, image offsets
// and the switch values.  Two passes (count, scan, write) give a
// deterministic order.
//
// Neighbour list: full list (both directions) over the 27 (distinct)
// surrounding cells of a grid whose edge is >= rc + skin, screened with the
// 32-bit fixed-point COM; compacted per warp with ballots.
#include <cuda_runtime.h>

#include <cooperative_groups.h>

#include <cstring>

#include "g6_internal.cuh"
#include "g6_rigid.cuh"

namespace cg = cooperative_groups;

namespace g6 {


__device__ __forceinline__ bool skip_ctrl(const int* ctrl) { return ctrl != nullptr && ctrl[0] == 0; }

__global__ void k_cell_clear(int* count, int ncell, const int* ctrl) {
  if (skip_ctrl(ctrl)) return;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c <= ncell; c += gridDim.x * blockDim.x) count[c] = 0;
}

// Reference cell index of one molecule (0-based, global over replicas).
__device__ __forceinline__ int ref_cell(const RepDev& rep, const GridDev& g, int r, double x, double y, double z) {
  double c[3] = {x, y, z};
  int j[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const double L = rep.L[3 * r + d], iL = rep.invL[3 * r + d];
    double delta = c[d];
    double cellv = xmul(xdnint(xmul(delta, iL)), L);
    delta = xsub(delta, cellv);
    int nd = g.nd[3 * r + d];
    int jj = (int)xdnint(xmul(delta, g.icell[3 * r + d]));
    if (jj < 0) jj += nd;
    if (jj >= nd) jj -= nd;
    // non-finite or absurd coordinates cannot index outside the grid; the
    // integrator reports them separately (G6_ERR_NONFINITE)
    if (!(jj >= 0 && jj < nd)) jj = 0;
    j[d] = jj;
  }
  const int nx = g.nd[3 * r], ny = g.nd[3 * r + 1];
  return g.cell_off[r] + (j[2] * ny + j[1]) * nx + j[0];
}

__global__ void k_cell_assign(CellArgs a) {
  if (skip_ctrl(a.ctrl)) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = i < a.n;
  int c = -1;
  if (valid) {
    const int r = a.rep.mol_rep[i];
    c = ref_cell(a.rep, a.g, r, a.com[i], a.com[a.n + i], a.com[2 * a.n + i]);
    a.cell[i] = c;
  }
  // warp-aggregated atomic increment of the cell population
  const unsigned act = __ballot_sync(0xffffffffu, valid);
  if (!valid) return;
  const unsigned peers = __match_any_sync(act, c);
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(peers) - 1;
  const int rank = __popc(peers & ((1u << lane) - 1u));
  int base = 0;
  if (lane == leader) base = atomicAdd(&a.count[c], __popc(peers));
  base = __shfl_sync(peers, base, leader);
  a.slot[i] = base + rank;
}

// Exclusive scan of count[0..m) into start[0..m] with one block of 1024 threads.
template <class T>
__global__ void __launch_bounds__(1024) k_scan(const T* count, T* start, int m, const int* ctrl) {
  if (skip_ctrl(ctrl)) return;
  __shared__ T part[1024];
  const int t = threadIdx.x;
  const int per = (m + 1023) / 1024;
  const int b = t * per, e = min(m, b + per);
  T s = 0;
  for (int k = b; k < e; ++k) s += count[k];
  part[t] = s;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    T v = (t >= off) ? part[t - off] : 0;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  T run = (t == 0) ? 0 : part[t - 1];
  for (int k = b; k < e; ++k) { start[k] = run; run += count[k]; }
  if (t == 1023) start[m] = part[1023];
}

__global__ void k_cell_fill(CellArgs a, const int* start, int* cellmol) {
  if (skip_ctrl(a.ctrl)) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < a.n) cellmol[start[a.cell[i]] + a.slot[i]] = i;
}

// (fixed-point COM, molecule) of cell-sorted slot k, so that the row scan reads
// one coalesced 16-byte word per candidate instead of an index and a gather.
__device__ __forceinline__ void fill_cellfix(const ListArgs& a, int k) {
  const uint32_t* fix = (a.ctrl != nullptr && (a.ctrl[1] & 1)) ? a.fix1 : a.fix;
  const int j = a.cellmol[k];
  a.cellfix[k] = make_uint4(fix[j], fix[a.n + j], fix[2 * a.n + j], (uint32_t)j);
}

// Residents of one cell in molecule order, sorted by one warp: every lane
// holds up to 8 ids and computes their ranks (ids are distinct); cells larger
// than 256 fall back to an insertion sort by lane 0.
__device__ void sort_cell_warp(int* cellmol, int b, int e, int lane, const ListArgs* fill = nullptr) {
  const int m = e - b;
  if (m <= 1) {
  } else if (m <= 256) {
    int v[8], r[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) { v[c] = (lane + 32 * c < m) ? cellmol[b + lane + 32 * c] : 0x7fffffff; r[c] = 0; }
#pragma unroll
    for (int cc = 0; cc < 8; ++cc) {
      if (32 * cc >= m) break;   // uniform across the warp
      for (int k = 0; k < 32; ++k) {
        const int w = __shfl_sync(0xffffffffu, v[cc], k);
        if (32 * cc + k < m) {
#pragma unroll
          for (int c = 0; c < 8; ++c) r[c] += (w < v[c]) ? 1 : 0;
        }
      }
    }
    __syncwarp();
#pragma unroll
    for (int c = 0; c < 8; ++c)
      if (lane + 32 * c < m) cellmol[b + r[c]] = v[c];
    __syncwarp();
  } else if (lane == 0) {
    for (int k = b + 1; k < e; ++k) {
      const int v = cellmol[k];
      int q = k - 1;
      while (q >= b && cellmol[q] > v) { cellmol[q + 1] = cellmol[q]; --q; }
      cellmol[q + 1] = v;
    }
  }
  if (fill) {   // the cell's (fixed-point COM, molecule) words in sorted order
    __syncwarp();
    for (int k = b + lane; k < e; k += 32) fill_cellfix(*fill, k);
  }
}

__global__ void k_cell_sort(const int* start, int* cellmol, int ncell, const int* ctrl) {
  if (skip_ctrl(ctrl)) return;
  const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (c >= ncell) return;   // whole warp
  sort_cell_warp(cellmol, start[c], start[c + 1], threadIdx.x & 31);
}

cudaError_t launch_cells(const CellArgs& a, int* start, int* cellmol, cudaStream_t s) {
  const int nc = a.g.ncell_total;
  k_cell_clear<<<(nc + 256) / 256, 256, 0, s>>>(a.count, nc, a.ctrl);
  if (a.n > 0) k_cell_assign<<<(a.n + 255) / 256, 256, 0, s>>>(a);
  k_scan<int><<<1, 1024, 0, s>>>(a.count, start, nc, a.ctrl);
  if (a.n > 0) k_cell_fill<<<(a.n + 255) / 256, 256, 0, s>>>(a, start, cellmol);
  k_cell_sort<<<(nc * 32 + 127) / 128, 128, 0, s>>>(start, cellmol, nc, a.ctrl);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Neighbour list.  One warp per molecule.  The list grid has cells of at least
// half the list radius, so the neighbours lie within two cells in every
// dimension: the (at most) 5 x 5 stencil rows of 5 consecutive x-cells, each
// contiguous in the cell-sorted arrays (two ranges where a row wraps); a
// dimension of fewer than 5 cells is taken whole.  Lane r scans row r on its
// own (independent loads, so several are in flight at once): a counting pass,
// a warp prefix sum of the counts, and a writing pass.  The row order of the
// result is stencil row by stencil row, each in cell-sorted order.
__device__ void list_row(const ListArgs& a, int i, int lane) {
  const int n = a.n;
  const int r = a.rep.mol_rep[i];
  const int nx = a.g.nd[3 * r], ny = a.g.nd[3 * r + 1], nz = a.g.nd[3 * r + 2];
  const int loc = a.cell[i] - a.g.cell_off[r];
  const int cx = loc % nx, cy = (loc / nx) % ny, cz = loc / (nx * ny);
  // fixed-point COM of this step's pose buffer (the buffers alternate with the step parity)
  const uint32_t* fix = (a.ctrl != nullptr && (a.ctrl[1] & 1)) ? a.fix1 : a.fix;
  const uint32_t xi = fix[i], yi = fix[n + i], zi = fix[2 * n + i];
  const float sx = a.rep.fscale[3 * r], sy = a.rep.fscale[3 * r + 1], sz = a.rep.fscale[3 * r + 2];
  const int ky = ny >= 5 ? 5 : ny, kz = nz >= 5 ? 5 : nz;   // rows of y and z to visit
  const int y0 = ny >= 5 ? cy - 2 : 0, z0 = nz >= 5 ? cz - 2 : 0;
  // x-ranges of a row: [xa, xb] and, after a wrap, [0, xc]
  int xa, xb, xc = -1;
  if (nx >= 5) {
    xa = cx - 2; xb = cx + 2;
    if (xa < 0) { xc = xb; xa += nx; xb = nx - 1; }
    else if (xb >= nx) { xc = xb - nx; xb = nx - 1; }
  } else {
    xa = 0; xb = nx - 1;
  }
  // this lane's stencil row
  int b0 = 0, e0 = 0, b1 = 0, e1 = 0;
  if (lane < ky * kz) {
    const int yy = (y0 + lane % ky + ny) % ny, zz = (z0 + lane / ky + nz) % nz;
    const int base = a.g.cell_off[r] + (zz * ny + yy) * nx;
    b0 = a.start[base + xa]; e0 = a.start[base + xb + 1];
    if (xc >= 0) { b1 = a.start[base]; e1 = a.start[base + xc + 1]; }
  }
  auto near = [&](const uint4& q) {
    const float dx = (float)(int)(xi - q.x) * sx;
    const float dy = (float)(int)(yi - q.y) * sy;
    const float dz = (float)(int)(zi - q.z) * sz;
    return (int)q.w != i && (!a.half || half_keep(i, (int)q.w)) && dx * dx + dy * dy + dz * dz < a.rlist2;
  };
  int cnt = 0;
#pragma unroll 4
  for (int k = b0; k < e0; ++k) cnt += near(a.cellfix[k]) ? 1 : 0;
#pragma unroll 4
  for (int k = b1; k < e1; ++k) cnt += near(a.cellfix[k]) ? 1 : 0;
  int pre = cnt;   // inclusive warp prefix sum
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, pre, d);
    if (lane >= d) pre += v;
  }
  const int total = __shfl_sync(0xffffffffu, pre, 31);
  int pos = pre - cnt;
  int* row = a.nbr + (size_t)i * a.cap;
  for (int k = b0; k < e0; ++k) {
    const uint4 q = a.cellfix[k];
    if (near(q)) { if (pos < a.cap) row[pos] = (int)q.w; ++pos; }
  }
  for (int k = b1; k < e1; ++k) {
    const uint4 q = a.cellfix[k];
    if (near(q)) { if (pos < a.cap) row[pos] = (int)q.w; ++pos; }
  }
  if (lane == 0) {
    int c = total;
    if (c > a.cap) { atomicExch(a.overflow, 1); c = a.cap; }
    a.nnb[i] = c;
    a.com_build[i] = a.com[i];
    a.com_build[n + i] = a.com[n + i];
    a.com_build[2 * n + i] = a.com[2 * n + i];
    if (a.fix_build) {
      a.fix_build[i] = xi;
      a.fix_build[n + i] = yi;
      a.fix_build[2 * n + i] = zi;
    }
  }
}

__global__ void k_cell_fix(ListArgs a) {
  if (skip_ctrl(a.ctrl)) return;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < a.n) fill_cellfix(a, k);
}

__global__ void __launch_bounds__(128) k_list_build(ListArgs a) {
  if (skip_ctrl(a.ctrl)) return;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (warp >= a.n) return;   // whole warp leaves together
  list_row(a, warp, threadIdx.x & 31);
}

// ---------------------------------------------------------------------------
// The whole neighbour-list rebuild in one cooperative launch: clear, assign
// and count, scan, fill, sort, list, separated by grid-wide barriers.  When
// the rebuild flag is 0 every block returns before the first barrier (the
// flag is written only by the kernel that runs before this one).
// ---------------------------------------------------------------------------
struct RebuildArgs {
  CellArgs c;
  ListArgs l;
  int* start;
  int* cellmol;
  StepArgs s;
  int with_step;   // MD step head: the rebuild decision comes from the previous step
};

__global__ void __launch_bounds__(256) k_rebuild(RebuildArgs a) {
  bool rebuild;
  if (a.with_step) {
    const int* ctrl = a.s.ctrl;
    if (ctrl[4]) {
      // the decision the previous step's last block made from its displacement test
      rebuild = ctrl[0] != 0;
    } else if (ctrl[0] == 2) {
      // first step of a run over a list built earlier: rebuild only if some
      // molecule has moved more than half the skin since that build (the
      // same test as between steps, on the fixed-point COM)
      cg::grid_group grid = cg::this_grid();
      if (!grid.is_valid()) {   // not launched cooperatively: report, never wait
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicExch(a.l.overflow, 2);
        return;
      }
      const int n = a.l.n;
      const uint32_t* fx = (ctrl[1] & 1) ? a.l.fix1 : a.l.fix;
      float dmax = 0.0f;
      for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int r = a.l.rep.mol_rep[i];
        float dd = 0.0f;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          const float e = (float)(int)(fx[(size_t)k * n + i] - a.l.fix_build[(size_t)k * n + i]) * a.l.rep.fscale[3 * r + k];
          dd += e * e;
        }
        dmax = fmaxf(dmax, dd);
      }
#pragma unroll
      for (int m = 16; m >= 1; m >>= 1) dmax = fmaxf(dmax, __shfl_xor_sync(0xffffffffu, dmax, m));
      if ((threadIdx.x & 31) == 0) atomicMax(&a.s.gmax[1], __float_as_uint(dmax));   // the word is 0 at run start
      grid.sync();
      rebuild = (double)__uint_as_float(__ldcg(&a.s.gmax[1])) > a.s.half_skin2;
      if (blockIdx.x == 0 && threadIdx.x == 0) a.s.ctrl[0] = rebuild ? 1 : 0;
    } else if (ctrl[0] == 3) {
      // first step of a host-buffer step: the records-in kernel raised each
      // molecule's displacement since the last build into gmax[1]; a block that
      // reads ctrl[0] after block 0 has written the decision reads the same decision
      rebuild = (double)__uint_as_float(__ldcg(&a.s.gmax[1])) > a.s.half_skin2;
      if (blockIdx.x == 0 && threadIdx.x == 0) a.s.ctrl[0] = rebuild ? 1 : 0;
    } else {
      rebuild = ctrl[0] != 0;   // first step of a run: the flag set by the host
    }
  } else {
    rebuild = !skip_ctrl(a.c.ctrl);
  }
  if (!rebuild) return;
  cg::grid_group grid = cg::this_grid();
  const int gt = blockIdx.x * blockDim.x + threadIdx.x, gs = gridDim.x * blockDim.x;
  if (!grid.is_valid()) {   // not launched cooperatively: report, never wait
    if (gt == 0) atomicExch(a.l.overflow, 2);
    return;
  }
  const int lane = threadIdx.x & 31, gw = gt >> 5, nw = gs >> 5;
  const int nc = a.c.g.ncell_total, n = a.c.n;
  for (int c = gt; c <= nc; c += gs) a.c.count[c] = 0;
  grid.sync();
  for (int base = gt - lane; base < n; base += gs) {   // whole warps, grid-stride
    const int i = base + lane;
    const bool valid = i < n;
    int c = -1;
    if (valid) {
      c = ref_cell(a.c.rep, a.c.g, a.c.rep.mol_rep[i], a.c.com[i], a.c.com[n + i], a.c.com[2 * n + i]);
      a.c.cell[i] = c;
    }
    const unsigned act = __ballot_sync(0xffffffffu, valid);
    if (valid) {
      const unsigned peers = __match_any_sync(act, c);
      const int leader = __ffs(peers) - 1;
      const int rank = __popc(peers & ((1u << lane) - 1u));
      int b0 = 0;
      if (lane == leader) b0 = atomicAdd(&a.c.count[c], __popc(peers));
      b0 = __shfl_sync(peers, b0, leader);
      a.c.slot[i] = b0 + rank;
    }
  }
  grid.sync();
  if (blockIdx.x == 0) {   // exclusive scan of the cell counts by one block
    __shared__ int part[256];
    const int t = threadIdx.x, per = (nc + 255) / 256;
    const int b = t * per, e = min(nc, b + per);
    int s = 0;
    for (int k = b; k < e; ++k) s += a.c.count[k];
    part[t] = s;
    __syncthreads();
    for (int off = 1; off < 256; off <<= 1) {
      const int v = t >= off ? part[t - off] : 0;
      __syncthreads();
      part[t] += v;
      __syncthreads();
    }
    int run = t == 0 ? 0 : part[t - 1];
    for (int k = b; k < e; ++k) { a.start[k] = run; run += a.c.count[k]; }
    if (t == 255) a.start[nc] = part[255];
  }
  grid.sync();
  for (int i = gt; i < n; i += gs) a.cellmol[a.start[a.c.cell[i]] + a.c.slot[i]] = i;
  grid.sync();
  for (int c = gw; c < nc; c += nw) sort_cell_warp(a.cellmol, a.start[c], a.start[c + 1], lane, &a.l);
  grid.sync();
  for (int i = gw; i < n; i += nw) list_row(a.l, i, lane);
}

int rebuild_grid_limit() {
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_rebuild, 256, 0);
  // two blocks per SM: the launch runs every step and mostly returns at once,
  // so its block count is paid every step while a rebuild is rare
  return sms * (per > 2 ? 2 : (per > 0 ? per : 1));
}

cudaError_t launch_rebuild(const CellArgs& c, const ListArgs& l, int* start, int* cellmol, int grid_limit,
                           const StepArgs* step, cudaStream_t s) {
  RebuildArgs a;
  memset(&a, 0, sizeof a);
  a.c = c; a.l = l; a.start = start; a.cellmol = cellmol;
  if (step) { a.s = *step; a.with_step = 1; }
  const int want = (max(c.n, c.g.ncell_total) * 32 + 255) / 256;
  const int blocks = max(1, min(grid_limit, want));
  void* args[] = {&a};
  return cudaLaunchCooperativeKernel((void*)k_rebuild, dim3(blocks), dim3(256), args, 0, s);
}

cudaError_t launch_list(const ListArgs& a, cudaStream_t s) {
  if (a.n == 0) return cudaSuccess;
  const long long threads = (long long)a.n * 32;
  k_cell_fix<<<(a.n + 255) / 256, 256, 0, s>>>(a);
  k_list_build<<<(unsigned)((threads + 127) / 128), 128, 0, s>>>(a);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// K3: exact pair set under the reference grid and stencil.
// ---------------------------------------------------------------------------

__device__ __forceinline__ void exact_switch(double dd, double rin2, double rout2, double rin, double rout, double c1,
                                             double c2, double& hh, double& dh) {
  hh = 0.0; dh = 0.0;
  if (dd < rout2) {
    if (dd > rin2) {
      double dr = __dsqrt_rn(dd);
      double u = xsub(dr, rout), l = xsub(dr, rin), uu = xmul(u, u), ll = xmul(l, l);
      double poly = xadd(xsub(xmul(10.0, ll), xmul(xmul(5.0, u), l)), uu);
      hh = xmul(xmul(xmul(c1, uu), u), poly);
      dh = -__ddiv_rn(xmul(xmul(c2, uu), ll), dr);
    } else {
      hh = 1.0; dh = 0.0;
    }
  }
}

__global__ void k_pairset(PairSetArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const int n = a.n;
  const int r = a.rep.mol_rep[i];
  const int nx = a.g.nd[3 * r], ny = a.g.nd[3 * r + 1], nz = a.g.nd[3 * r + 2];
  const int loc = a.cell[i] - a.g.cell_off[r];
  const int cx = loc % nx, cy = (loc / nx) % ny, cz = loc / (nx * ny);
  double L[3], iL[3], ci[3] = {a.com[i], a.com[n + i], a.com[2 * n + i]};
#pragma unroll
  for (int d = 0; d < 3; ++d) { L[d] = a.rep.L[3 * r + d]; iL[d] = a.rep.invL[3 * r + d]; }
  long long cnt = 0;
  long long w = a.pass ? a.off[i] : 0;
  for (int kind = 0; kind < 2; ++kind) {
    for (int e = a.sten_off[r]; e < a.sten_off[r + 1]; ++e) {
      if (a.sten[4 * e + 3] != kind) continue;
      const int xx = (cx + a.sten[4 * e]) % nx, yy = (cy + a.sten[4 * e + 1]) % ny, zz = (cz + a.sten[4 * e + 2]) % nz;
      const int c = a.g.cell_off[r] + (zz * ny + yy) * nx + xx;
      for (int k = a.start[c]; k < a.start[c + 1]; ++k) {
        const int j = a.cellmol[k];
        if (kind == 1 && !(j > i)) continue;
        double cj[3] = {a.com[j], a.com[n + j], a.com[2 * n + j]}, o[3], d[3];
        double dd = exact_dd(ci, cj, L, iL, o, d);
        if (!(dd < a.rout2)) continue;
        if (a.pass) {
          double h, dh;
          exact_switch(dd, a.rin2, a.rout2, a.rin, a.rout, a.c1, a.c2, h, dh);
          a.pi[w] = i; a.pj[w] = j;
          a.ox[w] = o[0]; a.oy[w] = o[1]; a.oz[w] = o[2];
          a.hh[w] = h; a.dh[w] = dh;
          ++w;
        }
        ++cnt;
      }
    }
  }
  if (!a.pass) a.cnt[i] = cnt;
}

cudaError_t launch_pairset_count(PairSetArgs a, cudaStream_t s) {
  a.pass = 0;
  if (a.n > 0) k_pairset<<<(a.n + 127) / 128, 128, 0, s>>>(a);
  k_scan<long long><<<1, 1024, 0, s>>>(a.cnt, a.cnt + a.n + 1, a.n, nullptr);
  return cudaGetLastError();
}

cudaError_t launch_pairset_write(PairSetArgs a, cudaStream_t s) {
  a.pass = 1;
  if (a.n > 0) k_pairset<<<(a.n + 127) / 128, 128, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace g6
