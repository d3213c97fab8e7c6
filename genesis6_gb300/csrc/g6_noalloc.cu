// g6_noalloc.cu -- the full force evaluation of g6_force for callers that must
// not allocate device memory.
//
// Who needs it: host programs whose device memory is owned by their own arena
// or pool (a Fortran driver that reserves the GPU up front, a code that runs
// next to a framework caching allocator and may not grow the footprint), and
// callers that hand in device buffers they already hold.  They cannot call
// cudaMalloc (or anything that calls it), so the context-based entry points,
// which allocate their tables in g6_system, are closed to them.
//
// What it does: the same kernels as g6_force (site placement, cell build,
// neighbour list, force, collect) on one system of at most
// G6_NOALLOC_MAX_MOL molecules.  All intermediate tables live in one
// file-scope __device__ array (g6_noalloc_scratch, 7,195,392 bytes (6.9 MiB)), which every
// GPU that loads the library holds until the process exits.  Inputs and
// outputs are device pointers owned by the caller.
//
// Rules of use:
//   - the first call on a device (with that device current) looks up the
//     array's device address with cudaGetSymbolAddress; make that first call
//     before any stream capture on that device;
//   - every call on a device shares the one array and it keeps the previous
//     call's contents; the call clears what must start at zero (cell counts,
//     the overflow flag) itself;
//   - calls that overlap on the GPU (different streams or host threads at the
//     same time) race on the array: serialise them;
//   - the call is synchronous: it waits for its stream before returning so
//     that it can report a neighbour-list overflow.
// No cudaMalloc, cudaFree or allocating library routine is called here.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>

#include "g6_internal.cuh"

namespace g6 {
namespace noalloc {

constexpr int MAXN = G6_NOALLOC_MAX_MOL;
constexpr int CAP = 224;          // neighbour-list row capacity: r_out + skin up to ~11.7 A at 1 g/cm^3 water
constexpr int MAXCELL = 32768;    // cells of the list grid
constexpr int W64MAX = 18;        // doubles per molecule in pk64 (5-site models)
constexpr int NPKMAX = 5;         // float4 per molecule in pk32

constexpr size_t al(size_t b) { return (b + 255) / 256 * 256; }

// Byte offsets of the regions inside the scratch array.
constexpr size_t O_ST = 0;                                            // 37 x MAXN doubles (com, q used)
constexpr size_t O_TMAT = O_ST + al(37ull * MAXN * 8);
constexpr size_t O_PK64 = O_TMAT + al(9ull * MAXN * 8);
constexpr size_t O_PK32 = O_PK64 + al((size_t)W64MAX * MAXN * 8);
constexpr size_t O_FIX = O_PK32 + al((size_t)NPKMAX * MAXN * 16);
constexpr size_t O_PKQ = O_FIX + al(3ull * MAXN * 4);                // 2 float4 per molecule
constexpr size_t O_F = O_PKQ + al(2ull * MAXN * 16);
constexpr size_t O_TL = O_F + al(3ull * MAXN * 8);
constexpr size_t O_EMOL = O_TL + al(3ull * MAXN * 8);
constexpr size_t O_WMOL = O_EMOL + al((size_t)MAXN * 8);
constexpr size_t O_NPIN = O_WMOL + al(9ull * MAXN * 8);
constexpr size_t O_OFF = O_NPIN + al((size_t)MAXN * 4);
constexpr size_t O_MOLREP = O_OFF + al(2 * 4);
constexpr size_t O_L = O_MOLREP + al((size_t)MAXN * 4);
constexpr size_t O_INVL = O_L + al(3 * 8);
constexpr size_t O_FSCALE = O_INVL + al(3 * 8);
constexpr size_t O_ND = O_FSCALE + al(3 * 4);
constexpr size_t O_EDGE = O_ND + al(3 * 4);
constexpr size_t O_ICELL = O_EDGE + al(3 * 8);
constexpr size_t O_CELLOFF = O_ICELL + al(3 * 8);
constexpr size_t O_CELL = O_CELLOFF + al(2 * 4);
constexpr size_t O_SLOT = O_CELL + al((size_t)MAXN * 4);
constexpr size_t O_COUNT = O_SLOT + al((size_t)MAXN * 4);
constexpr size_t O_START = O_COUNT + al((size_t)(MAXCELL + 1) * 4);
constexpr size_t O_CELLMOL = O_START + al((size_t)(MAXCELL + 1) * 4);
constexpr size_t O_NBR = O_CELLMOL + al((size_t)MAXN * 4);
constexpr size_t O_NNB = O_NBR + al((size_t)MAXN * CAP * 4);
constexpr size_t O_COMB = O_NNB + al((size_t)MAXN * 4);
constexpr size_t O_CFIX = O_COMB + al(3ull * MAXN * 8);
constexpr size_t O_OVF = O_CFIX + al((size_t)MAXN * 16);
constexpr size_t BYTES = O_OVF + al(4);

}  // namespace noalloc

// The scratch array (see the file comment for its size, sharing and lifetime).
static __device__ __align__(256) unsigned char g6_noalloc_scratch[noalloc::BYTES];

namespace noalloc {

struct Setup {
  int n, ncell;
  double L[3], invL[3];
  float fs[3];
  int nd[3];
  double edge[3], icell[3];
};

// Geometry tables of the single replica and the cleared overflow flag.
__global__ void k_setup(Setup s, unsigned char* base) {
  int* off = (int*)(base + O_OFF);
  int* mol_rep = (int*)(base + O_MOLREP);
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  for (int i = t; i < s.n; i += gridDim.x * blockDim.x) mol_rep[i] = 0;
  if (t == 0) {
    off[0] = 0; off[1] = s.n;
    double* L = (double*)(base + O_L); double* iL = (double*)(base + O_INVL); float* fs = (float*)(base + O_FSCALE);
    int* nd = (int*)(base + O_ND); double* ed = (double*)(base + O_EDGE); double* ic = (double*)(base + O_ICELL);
    int* co = (int*)(base + O_CELLOFF);
    for (int d = 0; d < 3; ++d) {
      L[d] = s.L[d]; iL[d] = s.invL[d]; fs[d] = s.fs[d]; nd[d] = s.nd[d]; ed[d] = s.edge[d]; ic[d] = s.icell[d];
    }
    co[0] = 0; co[1] = s.ncell;
    *(int*)(base + O_OVF) = 0;
  }
}

// Caller's com (n,3) and quat (n,4) into the SoA state used by site placement.
__global__ void k_load(int n, const double* com, const double* quat, unsigned char* base) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double* st = (double*)(base + O_ST);
  for (int k = 0; k < 3; ++k) st[(size_t)k * n + i] = com[3 * i + k];
  for (int k = 0; k < 4; ++k) st[(size_t)(33 + k) * n + i] = quat[4 * i + k];
}

// Outputs in the caller's layout: F (n,3), body torque T^T tau_lab (n,3), and
// the total energy summed in a fixed order by one block.
__global__ void k_finish(int n, unsigned char* base, double* F, double* tau, double* epot) {
  const double* f = (const double*)(base + O_F);
  const double* tl = (const double*)(base + O_TL);
  const double* tm = (const double*)(base + O_TMAT);
  const double* em = (const double*)(base + O_EMOL);
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    for (int k = 0; k < 3; ++k) F[3 * i + k] = f[(size_t)k * n + i];
    double t[9];
    for (int k = 0; k < 9; ++k) t[k] = tm[(size_t)k * n + i];
    const double l0 = tl[i], l1 = tl[n + i], l2 = tl[2 * n + i];
    tau[3 * i] = t[0] * l0 + t[3] * l1 + t[6] * l2;
    tau[3 * i + 1] = t[1] * l0 + t[4] * l1 + t[7] * l2;
    tau[3 * i + 2] = t[2] * l0 + t[5] * l1 + t[8] * l2;
  }
  __shared__ double part[256];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += em[i];
  part[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double e = 0.0;
    for (int k = 0; k < (int)blockDim.x; ++k) e += part[k];
    *epot = e;
  }
}

std::mutex mu;
unsigned char* base_of[64] = {nullptr};

}  // namespace noalloc
}  // namespace g6

using namespace g6;

extern "C" int g6_force_noalloc(int model, int path, int precision, int n, const double* box, double r_in,
                                double r_out, double skin, const double* d_com, const double* d_quat, double* d_F,
                                double* d_tau, double* d_epot, void* stream) {
  using namespace g6::noalloc;
  ModelHost mh;
  if (!make_model(model, mh)) return G6_ERR_ARG;
  if (path != G6_PATH_STD && path != G6_PATH_CUSTOM) return G6_ERR_ARG;
  if (precision != G6_FP64 && precision != G6_MIXED) return G6_ERR_ARG;
  if (n > MAXN) return G6_ERR_CAPACITY;   // beyond the static tables
  if (n < 2 || !box || !d_com || !d_quat || !d_F || !d_tau || !d_epot) return G6_ERR_ARG;
  if (!(r_out > 0.0) || !(r_in >= 0.0) || !(r_in < r_out) || !(skin >= 0.0)) return G6_ERR_ARG;
  for (int d = 0; d < 3; ++d)
    if (!(box[d] > 0.0) || !(r_out <= 0.5 * box[d])) return G6_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return G6_ERR_CUDA;
  unsigned char* base = nullptr;
  {
    std::lock_guard<std::mutex> lock(mu);
    if (!base_of[dev]) {
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g6_noalloc_scratch) != cudaSuccess || !p) return G6_ERR_CUDA;
      base_of[dev] = (unsigned char*)p;
    }
    base = base_of[dev];
  }
  // geometry of the list grid: edge >= (r_out + skin) / 2 (list_row visits two
  // cells each way), at most MAXCELL cells (coarser cells stay correct)
  Setup su;
  std::memset(&su, 0, sizeof su);
  su.n = n;
  double sk = skin;
  for (int d = 0; d < 3; ++d) sk = std::min(sk, 0.5 * box[d] - r_out);
  sk = std::max(0.0, sk);
  const double rlist = r_out + sk;
  for (int d = 0; d < 3; ++d) {
    su.L[d] = box[d]; su.invL[d] = 1.0 / box[d]; su.fs[d] = (float)(box[d] / 4294967296.0);
    su.nd[d] = std::max(1, (int)(box[d] / (0.5 * rlist)));
  }
  while ((long long)su.nd[0] * su.nd[1] * su.nd[2] > MAXCELL) {   // coarser cells stay correct
    int d = (int)(std::max_element(su.nd, su.nd + 3) - su.nd);
    su.nd[d] = std::max(1, su.nd[d] / 2);
  }
  for (int d = 0; d < 3; ++d) { su.edge[d] = box[d] / su.nd[d]; su.icell[d] = 1.0 / su.edge[d]; }
  su.ncell = su.nd[0] * su.nd[1] * su.nd[2];

  RepDev rep;
  rep.nrep = 1; rep.off = (const int*)(base + O_OFF); rep.mol_rep = (const int*)(base + O_MOLREP);
  rep.L = (const double*)(base + O_L); rep.invL = (const double*)(base + O_INVL);
  rep.fscale = (const float*)(base + O_FSCALE);
  GridDev g;
  g.ncell_total = su.ncell; g.nd = (const int*)(base + O_ND); g.cell = (const double*)(base + O_EDGE);
  g.icell = (const double*)(base + O_ICELL); g.cell_off = (const int*)(base + O_CELLOFF);

  PlaceArgs pa;
  pa.n = n; pa.nq = mh.nq; pa.npk = pk32_width(model); pa.w64 = pk64_width(model); pa.rep = rep;
  for (int q = 0; q < MAXSITE; ++q)
    for (int k = 0; k < 3; ++k) { pa.body[q][k] = mh.body[q][k]; pa.fbody[q][k] = (float)mh.body[q][k]; }
  pa.st = (double*)(base + O_ST); pa.tmat = (double*)(base + O_TMAT); pa.pk64 = (double*)(base + O_PK64);
  pa.pk32 = (float4*)(base + O_PK32); pa.pkq = (float4*)(base + O_PKQ); pa.fix = (uint32_t*)(base + O_FIX);

  CellArgs ca;
  ca.n = n; ca.rep = rep; ca.g = g; ca.com = pa.st; ca.cell = (int*)(base + O_CELL); ca.slot = (int*)(base + O_SLOT);
  ca.count = (int*)(base + O_COUNT); ca.ctrl = nullptr;

  ListArgs la;
  std::memset(&la, 0, sizeof la);   // fix_build stays NULL: no displacement bookkeeping here
  la.n = n; la.cap = CAP; la.rep = rep; la.g = g; la.cell = ca.cell; la.start = (const int*)(base + O_START);
  la.cellmol = (const int*)(base + O_CELLMOL); la.fix = pa.fix; la.fix1 = pa.fix; la.com = pa.st; la.com_build = (double*)(base + O_COMB);
  la.rlist2 = (float)(rlist * rlist) + 1e-3f; la.nbr = (int*)(base + O_NBR); la.nnb = (int*)(base + O_NNB);
  la.overflow = (int*)(base + O_OVF); la.ctrl = nullptr; la.cellfix = (uint4*)(base + O_CFIX);

  ForceArgs fa;
  std::memset(&fa, 0, sizeof fa);
  fa.n = n; fa.cap = CAP; fa.stride_pk32 = pa.npk; fa.nbr = la.nbr; fa.nnb = la.nnb; fa.rep = rep; fa.pk64 = pa.pk64;
  fa.pk32 = pa.pk32; fa.pk64_1 = pa.pk64; fa.pk32_1 = pa.pk32; fa.ctrl = nullptr;
  make_pair_const(mh, path, fa.pc);
  make_cut_const(r_in, r_out, fa.cc);
  fa.F = (double*)(base + O_F); fa.tl = (double*)(base + O_TL); fa.emol = (double*)(base + O_EMOL);
  fa.wmol = (double*)(base + O_WMOL); fa.npair_in = (int*)(base + O_NPIN);
  fa.ccap = CAP; fa.overflow = la.overflow;
  fa.pkq = pa.pkq; fa.pkq_1 = pa.pkq;
  for (int q = 0; q < MAXSITE; ++q)
    for (int k = 0; k < 3; ++k) fa.fbody[q][k] = pa.fbody[q][k];
  fa.band = row_test_band(rlist, std::max(box[0], std::max(box[1], box[2])));
  for (int k = 0; k < 3; ++k) fa.fs1[k] = (float)(box[k] / 4294967296.0);

  const int blocks = (n + 255) / 256;
  k_setup<<<blocks, 256, 0, s>>>(su, base);
  k_load<<<blocks, 256, 0, s>>>(n, d_com, d_quat, base);
  if (cudaGetLastError() != cudaSuccess) return G6_ERR_CUDA;
  if (launch_predict_place(pa, 0, nullptr, 0, s) != cudaSuccess) return G6_ERR_CUDA;
  if (launch_cells(ca, (int*)(base + O_START), (int*)(base + O_CELLMOL), s) != cudaSuccess) return G6_ERR_CUDA;
  if (launch_list(la, s) != cudaSuccess) return G6_ERR_CUDA;
  if (launch_force(fa, model, precision == G6_MIXED, 16, s) != cudaSuccess) return G6_ERR_CUDA;
  k_finish<<<1, 256, 0, s>>>(n, base, d_F, d_tau, d_epot);
  if (cudaGetLastError() != cudaSuccess) return G6_ERR_CUDA;
  int ovf = 0;
  if (cudaMemcpyAsync(&ovf, base + O_OVF, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess) return G6_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return G6_ERR_CUDA;
  return ovf ? G6_ERR_CAPACITY : G6_OK;
}
