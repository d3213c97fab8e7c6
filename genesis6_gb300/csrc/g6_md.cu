// g6_md.cu -- placement kernel, replica exchange and state transposes.
//
// k_predict_place: rigid_predict (RigidModule.F90:480-559) and site placement
//   (rigid_setmatrix :62-83, rigid_setsiteposition0 :88-144) for one molecule
//   per thread, writing pose buffer 0, plus the first Nose_Predict of a run.
// The Gear corrector and the per-step reductions run in the epilogue of the
// fused force kernel (g6_force.cu) through the device functions of g6_rigid.cuh.
// k_stf_move / k_begin_mixed: state moves and the first step of a
// mixed-precision run (float SoA for the small Gear terms).
#include <cuda_runtime.h>

#include "g6_internal.cuh"
#include "g6_rigid.cuh"

namespace g6 {

#define ST(c) st[(size_t)(c) * n + i]

__global__ void k_predict_place(PlaceArgs a, int do_predict, ThermoDev* th, int nose_predict) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (nose_predict && blockIdx.x == 0) {
    for (int r = threadIdx.x; r < a.rep.nrep; r += blockDim.x) {
      ThermoDev& T = th[r];
      if (T.kind == G6_NOSE) {   // Nose_Predict
        T.z[0] = T.z[0] + T.z[1] + T.z[2] + T.z[3] + T.z[4];
        T.z[1] = T.z[1] + 2.0 * T.z[2] + 3.0 * T.z[3] + 4.0 * T.z[4];
        T.z[2] = T.z[2] + 3.0 * T.z[3] + 6.0 * T.z[4];
        T.z[3] = T.z[3] + 4.0 * T.z[4];
      }
    }
  }
  if (i >= a.n) return;
  if (do_predict) predict_one(a.st, a.n, i);
  place_to(a, i, a.tmat, a.pk64, a.pk32, a.pkq, a.fix);
}

cudaError_t launch_predict_place(const PlaceArgs& a, int do_predict, ThermoDev* th, int nose_predict,
                                 cudaStream_t s) {
  const int blocks = a.n > 0 ? (a.n + 127) / 128 : 1;
  k_predict_place<<<blocks, 128, 0, s>>>(a, do_predict, th, nose_predict);
  return cudaGetLastError();
}

// Mixed-precision runs: the small Gear terms move from the FP64 state into
// the float SoA at the start of a run (to_float) and back at its end, so the
// FP64 state is the complete rigid record whenever no run is active.
// State column (of the 53-double record) of float column c.
__device__ __forceinline__ int stf_state_col(int c) {
  if (c < STF_W2) return 6 + c;                    // d2..d5
  if (c < STF_Q2) return 21 + (c - STF_W2);        // w2..w5
  return 37 + (c - STF_Q2);                        // q2..q5 stacks
}

__global__ void k_stf_move(double* st, float* stf, int n, int to_float) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)n * STF_COLS) return;
  const int c = (int)(t / n), i = (int)(t % n);
  const int sc = stf_state_col(c);
  if (to_float) stf[t] = (float)st[(size_t)sc * n + i];
  else st[(size_t)sc * n + i] = (double)stf[t];
}

// Float column of state column sc, or -1 for the columns kept in FP64 (com,
// d1, w1, q); the inverse of stf_state_col.
__device__ __forceinline__ int state_float_col(int sc) {
  if (sc < 6) return -1;
  if (sc < 18) return sc - 6;
  if (sc < 21) return -1;
  if (sc < 33) return STF_W2 + (sc - 21);
  if (sc < 37) return -1;
  return STF_Q2 + (sc - 37);
}

// Records move between the AoS layout (n,53) and the column layout through a
// shared-memory tile of REC_TILE molecules: the record block is read or
// written as one contiguous run, the columns as 32-molecule runs, so both
// sides are coalesced.
constexpr int REC_TILE = 32;
constexpr int REC_THREADS = 128;
constexpr int REC_V2 = REC_TILE * REC / 2;                                // double2 per full tile (848)
constexpr int REC_V2_PER = (REC_V2 + REC_THREADS - 1) / REC_THREADS;      // per thread (7)
constexpr int REC_PER = (REC_TILE * REC + REC_THREADS - 1) / REC_THREADS;  // doubles per thread (14)

// One tile of records (m molecules from src) into shared memory and, when
// keep is set, into a device copy.  Every load of the thread is issued before
// the first store (a store to global memory between them would order each
// load after it: one round trip per element, costly when src is host memory
// read over the host link); a full tile on a 16-byte boundary moves as double2.
__device__ __forceinline__ void rec_tile_in(const double* src, int m, double* tile, double* keep) {
  if (m == REC_TILE && (reinterpret_cast<uintptr_t>(src) & 15) == 0) {
    const double2* s2 = reinterpret_cast<const double2*>(src);
    double2 v[REC_V2_PER];
#pragma unroll
    for (int u = 0; u < REC_V2_PER; ++u) {
      const int t = threadIdx.x + u * REC_THREADS;
      if (t < REC_V2) v[u] = s2[t];
    }
    double2* t2 = reinterpret_cast<double2*>(tile);
    double2* k2 = reinterpret_cast<double2*>(keep);   // device copy: 16-byte aligned at a full tile
#pragma unroll
    for (int u = 0; u < REC_V2_PER; ++u) {
      const int t = threadIdx.x + u * REC_THREADS;
      if (t < REC_V2) {
        t2[t] = v[u];
        if (keep) k2[t] = v[u];
      }
    }
  } else {
    double v[REC_PER];
#pragma unroll
    for (int u = 0; u < REC_PER; ++u) {
      const int t = threadIdx.x + u * REC_THREADS;
      if (t < m * REC) v[u] = src[t];
    }
#pragma unroll
    for (int u = 0; u < REC_PER; ++u) {
      const int t = threadIdx.x + u * REC_THREADS;
      if (t < m * REC) {
        tile[t] = v[u];
        if (keep) keep[t] = v[u];
      }
    }
  }
}

// Block 0 of the records-in kernel, after its tile: the control block from
// page-locked memory (when h.ctl_up is set) and the Nose predict of the step.
// The thermostats are read by no other block of this kernel.
__device__ __forceinline__ void host_in_control(const PlaceArgs& a, const HostInArgs& h, ThermoDev* th, double dt) {
  if (h.ctl_up) {
    for (int w = threadIdx.x; w < h.ctl_n16; w += blockDim.x) {
      const uint4 v = h.ctl_up[w];
      if (w != h.gmax16) {
        h.ctl[w] = v;
      } else {
        unsigned int* g = reinterpret_cast<unsigned int*>(h.ctl + w);
        g[0] = v.x; g[2] = v.z; g[3] = v.w;
      }
    }
    __syncthreads();
  }
  for (int r = threadIdx.x; r < a.rep.nrep; r += blockDim.x) {
    ThermoDev& T = th[r];
    if (T.kind == G6_NOSE) {
      T.z[0] = T.z[0] + T.z[1] + T.z[2] + T.z[3] + T.z[4];
      T.z[1] = T.z[1] + 2.0 * T.z[2] + 3.0 * T.z[3] + 4.0 * T.z[4];
      T.z[2] = T.z[2] + 3.0 * T.z[3] + 6.0 * T.z[4];
      T.z[3] = T.z[3] + 4.0 * T.z[4];
      T.fext = (float)(T.z[0] * dt);
    }
  }
}

// One mixed-precision step with the state in the caller's record buffer
// (g6_md_step_host): the records (n,53) become the FP64 state (com, d1, w1,
// q) and the float small terms, followed by the step's first predict and
// placement and the Nose predict -- the work of k_rec_transpose, k_stf_move
// and k_begin_mixed in one pass, with the same arithmetic.  h.rec may be the
// caller's page-locked buffer itself (read over the host link by the tiles);
// h.keep then receives a device copy for a repeat of the step.  With h.gmax,
// each molecule's displacement since the last list build (the step head's
// keep-the-list test, on the new fixed-point COM) is raised into h.gmax[1],
// so the head only compares one word.  With h.ctl_up, block 0 also reads the
// run's control block from page-locked memory after its tile (the upload that
// is otherwise a copy before this kernel).
__global__ void __launch_bounds__(REC_THREADS) k_host_in_mixed(PlaceArgs a, HostInArgs h, float* stf, ThermoDev* th,
                                                               double dt) {
  __shared__ __align__(16) double tile[REC_TILE * REC];
  const int n = a.n;
  const int i0 = blockIdx.x * REC_TILE;
  const int m = min(REC_TILE, n - i0);
  if (m <= 0) {
    if (blockIdx.x == 0) host_in_control(a, h, th, dt);
    return;
  }
  rec_tile_in(h.rec + (size_t)i0 * REC, m, tile, h.keep ? h.keep + (size_t)i0 * REC : nullptr);
  __syncthreads();
  double* st = a.st;
  for (int t = threadIdx.x; t < REC_TILE * REC; t += blockDim.x) {
    const int c = t / REC_TILE, k = t % REC_TILE;
    if (k >= m) continue;
    const double v = tile[k * REC + c];
    const int fc = state_float_col(c);
    if (fc < 0) st[(size_t)c * n + i0 + k] = v;
    else stf[(size_t)fc * n + i0 + k] = (float)v;
  }
  __syncthreads();   // the block's columns are visible to the block
  if (threadIdx.x < 32) {
    float dd = 0.0f;
    if ((int)threadIdx.x < m) {
      const int i = i0 + threadIdx.x;
      double x[3], q[4];
      predict_mixed(st, stf, n, i, x, q);
      if (a.nq == 3) place_mixed<3>(a, i, x, q, a.pk64, a.pk32, a.pkq, a.fix);
      else place_mixed<4>(a, i, x, q, a.pk64, a.pk32, a.pkq, a.fix);
      if (h.gmax) {
        const int r = a.rep.mol_rep[i];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          const float e =
              (float)(int)(a.fix[(size_t)k * n + i] - h.fix_build[(size_t)k * n + i]) * a.rep.fscale[3 * r + k];
          dd += e * e;
        }
      }
    }
    if (h.gmax) {
#pragma unroll
      for (int o = 16; o >= 1; o >>= 1) dd = fmaxf(dd, __shfl_xor_sync(0xffffffffu, dd, o));
      if (threadIdx.x == 0) atomicMax(&h.gmax[1], __float_as_uint(dd));
    }
  }
  if (blockIdx.x == 0) {
    __syncthreads();
    host_in_control(a, h, th, dt);
  }
}

// The end of that step: the replica finish of the step (the first nrep
// blocks) beside the state going back to the FP64 record, both in the device
// state and as records (n,53) in o.rec (the caller's page-locked buffer or a
// device copy) -- the work of k_finish_step, k_stf_move and k_rec_transpose in
// one launch.  With o.th_dn the finish blocks also write the words the host
// reads after the step (thermostats, sums, control words, overflow flag) to
// page-locked memory.
__global__ void __launch_bounds__(REC_THREADS) k_host_out_mixed(StepArgs sa, HostOutArgs o) {
  __shared__ __align__(16) double tile[REC_TILE * REC];
  const int nfin = sa.p.rep.nrep;
  if ((int)blockIdx.x < nfin) {
    const int rr = blockIdx.x;
    finish_pending(sa, rr, 32);
    if (o.th_dn) {
      __syncthreads();   // the replica's thermostat and sums as finish_pending left them
      constexpr int TW = (int)(sizeof(ThermoDev) / sizeof(double));
      static_assert(sizeof(ThermoDev) % sizeof(double) == 0, "ThermoDev is copied as doubles");
      const double* ts = reinterpret_cast<const double*>(sa.th + rr);
      double* td = reinterpret_cast<double*>(o.th_dn + rr);
      for (int w = threadIdx.x; w < TW; w += blockDim.x) td[w] = ts[w];
      for (int k = threadIdx.x; k < NRED; k += blockDim.x) o.red_dn[(size_t)rr * NRED + k] = sa.red[(size_t)rr * NRED + k];
      if (rr == 0) {
        if (threadIdx.x < 8) o.ctrl_dn[threadIdx.x] = sa.ctrl[threadIdx.x];
        if (threadIdx.x == 8) *o.ovf_dn = *o.ovf;
      }
    }
    return;
  }
  double* out = o.rec;
  const int n = sa.p.n;
  const int i0 = (blockIdx.x - nfin) * REC_TILE;
  const int m = min(REC_TILE, n - i0);
  if (m <= 0) return;
  double* st = sa.p.st;
  // all loads of the thread first (the FP64 columns and the float small
  // terms), then the small terms back into the FP64 state and the tile
  double v[REC_PER];
#pragma unroll
  for (int u = 0; u < REC_PER; ++u) {
    const int t = threadIdx.x + u * REC_THREADS;
    const int c = t / REC_TILE, k = t % REC_TILE;
    v[u] = 0.0;
    if (t < REC_TILE * REC && k < m) {
      const int fc = state_float_col(c);
      v[u] = fc < 0 ? st[(size_t)c * n + i0 + k] : (double)sa.stf[(size_t)fc * n + i0 + k];
    }
  }
#pragma unroll
  for (int u = 0; u < REC_PER; ++u) {
    const int t = threadIdx.x + u * REC_THREADS;
    const int c = t / REC_TILE, k = t % REC_TILE;
    if (t < REC_TILE * REC && k < m) {
      if (state_float_col(c) >= 0) st[(size_t)c * n + i0 + k] = v[u];
      tile[k * REC + c] = v[u];
    }
  }
  __syncthreads();
  double* dst = out + (size_t)i0 * REC;
  if (m == REC_TILE && (reinterpret_cast<uintptr_t>(dst) & 15) == 0) {
    double2* d2 = reinterpret_cast<double2*>(dst);
    const double2* t2 = reinterpret_cast<const double2*>(tile);
#pragma unroll
    for (int u = 0; u < REC_V2_PER; ++u) {
      const int t = threadIdx.x + u * REC_THREADS;
      if (t < REC_V2) d2[t] = t2[t];
    }
  } else {
    for (int t = threadIdx.x; t < m * REC; t += blockDim.x) dst[t] = tile[t];
  }
}

// First predict + placement of a mixed run (plus the first Nose_Predict).
__global__ void k_begin_mixed(PlaceArgs a, float* stf, ThermoDev* th, double dt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (blockIdx.x == 0) {
    for (int r = threadIdx.x; r < a.rep.nrep; r += blockDim.x) {
      ThermoDev& T = th[r];
      if (T.kind == G6_NOSE) {
        T.z[0] = T.z[0] + T.z[1] + T.z[2] + T.z[3] + T.z[4];
        T.z[1] = T.z[1] + 2.0 * T.z[2] + 3.0 * T.z[3] + 4.0 * T.z[4];
        T.z[2] = T.z[2] + 3.0 * T.z[3] + 6.0 * T.z[4];
        T.z[3] = T.z[3] + 4.0 * T.z[4];
        T.fext = (float)(T.z[0] * dt);
      }
    }
  }
  if (i >= a.n) return;
  double x[3], q[4];
  predict_mixed(a.st, stf, a.n, i, x, q);
  if (a.nq == 3) place_mixed<3>(a, i, x, q, a.pk64, a.pk32, a.pkq, a.fix);
  else place_mixed<4>(a, i, x, q, a.pk64, a.pk32, a.pkq, a.fix);
}

cudaError_t launch_stf_move(double* st, float* stf, int n, int to_float, cudaStream_t s) {
  const long long total = (long long)n * STF_COLS;
  if (total == 0) return cudaSuccess;
  k_stf_move<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(st, stf, n, to_float);
  return cudaGetLastError();
}

cudaError_t launch_host_in_mixed(const PlaceArgs& a, const HostInArgs& h, float* stf, ThermoDev* th, double dt,
                                 cudaStream_t s) {
  const int blocks = a.n > 0 ? (a.n + REC_TILE - 1) / REC_TILE : 1;
  k_host_in_mixed<<<blocks, REC_THREADS, 0, s>>>(a, h, stf, th, dt);
  return cudaGetLastError();
}

cudaError_t launch_host_out_mixed(const StepArgs& sa, const HostOutArgs& o, cudaStream_t s) {
  const int blocks = sa.p.rep.nrep + (sa.p.n + REC_TILE - 1) / REC_TILE;
  k_host_out_mixed<<<blocks, REC_THREADS, 0, s>>>(sa, o);
  return cudaGetLastError();
}

cudaError_t launch_begin_mixed(const PlaceArgs& a, float* stf, ThermoDev* th, double dt, cudaStream_t s) {
  const int blocks = a.n > 0 ? (a.n + 127) / 128 : 1;
  k_begin_mixed<<<blocks, 128, 0, s>>>(a, stf, th, dt);
  return cudaGetLastError();
}

// Replica exchange for neighbouring temperature pairs (replica_exchange_trial,
// Replica.F90:7-73) with the MD side effects of Mixture.F90:1616-1653: the
// replica that changes temperature has its first derivatives scaled by
// sqrt(T_new/T_old) (Rigid_ScaleVelocity) and its Nose zeta stack zeroed.

__global__ void k_exchange(ExchArgs a) {
  if (threadIdx.x != 0) return;
  for (int r = 0; r < a.nrep; ++r) a.temp[r] = a.th[r].temp;
  ExchangeIO x;
  x.nrep = a.nrep; x.parity = a.parity; x.seed = a.seed; x.counter = a.counter; x.epot = a.epot; x.beta = a.beta;
  x.temp = a.temp; x.numb = a.numb; x.umb = a.umb; x.op = a.op; x.slot = a.slot; x.scale = a.scale;
  x.moved = a.moved; x.accepted = a.accepted;
  exchange_run(x);
  for (int r = 0; r < a.nrep; ++r) {
    if (!a.moved[r]) continue;
    a.th[r].temp = a.temp[r];
    for (int k = 0; k < 5; ++k) a.th[r].z[k] = 0.0;
  }
}

__global__ void k_scale_velocity(double* st, int n, const int* mol_rep, const double* scale) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double f = scale[mol_rep[i]];
  if (f == 1.0) return;
  for (int c = 0; c < 3; ++c) { ST(3 + c) *= f; ST(18 + c) *= f; }
}

cudaError_t launch_scale_velocity(double* st, int n, const int* mol_rep, const double* scale, cudaStream_t s) {
  if (n > 0) k_scale_velocity<<<(n + 127) / 128, 128, 0, s>>>(st, n, mol_rep, scale);
  return cudaGetLastError();
}

cudaError_t launch_exchange(const ExchArgs& a, double* st, int n, const int* mol_rep, cudaStream_t s) {
  k_exchange<<<1, 32, 0, s>>>(a);
  if (n > 0) k_scale_velocity<<<(n + 127) / 128, 128, 0, s>>>(st, n, mol_rep, a.scale);
  return cudaGetLastError();
}

// AoS rigid records (n x 53) <-> SoA device state (53 x n), one tile of
// REC_TILE molecules per block.
__global__ void __launch_bounds__(REC_THREADS) k_rec_transpose(double* aos, double* soa, int n, int to_soa) {
  __shared__ double tile[REC_TILE * REC];
  const int i0 = blockIdx.x * REC_TILE;
  const int m = min(REC_TILE, n - i0);
  double* blk = aos + (size_t)i0 * REC;
  if (to_soa) {
    for (int t = threadIdx.x; t < m * REC; t += blockDim.x) tile[t] = blk[t];
    __syncthreads();
    for (int t = threadIdx.x; t < REC_TILE * REC; t += blockDim.x) {
      const int c = t / REC_TILE, k = t % REC_TILE;
      if (k < m) soa[(size_t)c * n + i0 + k] = tile[k * REC + c];
    }
  } else {
    for (int t = threadIdx.x; t < REC_TILE * REC; t += blockDim.x) {
      const int c = t / REC_TILE, k = t % REC_TILE;
      if (k < m) tile[k * REC + c] = soa[(size_t)c * n + i0 + k];
    }
    __syncthreads();
    for (int t = threadIdx.x; t < m * REC; t += blockDim.x) blk[t] = tile[t];
  }
}

cudaError_t launch_rec_transpose(double* aos, double* soa, int n, int to_soa, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_rec_transpose<<<(n + REC_TILE - 1) / REC_TILE, REC_THREADS, 0, s>>>(aos, soa, n, to_soa);
  return cudaGetLastError();
}

}  // namespace g6
