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
  place_to(a, i, a.tmat, a.pk64, a.pk32, a.fix);
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
__global__ void k_stf_move(double* st, float* stf, int n, int to_float) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)n * STF_COLS) return;
  const int c = (int)(t / n), i = (int)(t % n);
  int sc;   // state column of float column c
  if (c < STF_W2) sc = 6 + c;                      // d2..d5
  else if (c < STF_Q2) sc = 21 + (c - STF_W2);     // w2..w5
  else sc = 37 + (c - STF_Q2);                     // q2..q5 stacks
  if (to_float) stf[t] = (float)st[(size_t)sc * n + i];
  else st[(size_t)sc * n + i] = (double)stf[t];
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
  if (a.nq == 3) place_mixed<3>(a, i, x, q, a.pk64, a.pk32, a.fix);
  else place_mixed<4>(a, i, x, q, a.pk64, a.pk32, a.fix);
}

cudaError_t launch_stf_move(double* st, float* stf, int n, int to_float, cudaStream_t s) {
  const long long total = (long long)n * STF_COLS;
  if (total == 0) return cudaSuccess;
  k_stf_move<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(st, stf, n, to_float);
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

// AoS rigid records (n x 53) <-> SoA device state (53 x n).
__global__ void k_rec_transpose(double* aos, double* soa, int n, int to_soa) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)n * REC) return;
  const int c = (int)(t / n), i = (int)(t % n);
  if (to_soa) soa[t] = aos[(size_t)i * REC + c];
  else aos[(size_t)i * REC + c] = soa[t];
}

cudaError_t launch_rec_transpose(double* aos, double* soa, int n, int to_soa, cudaStream_t s) {
  const long long total = (long long)n * REC;
  if (total == 0) return cudaSuccess;
  k_rec_transpose<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(aos, soa, n, to_soa);
  return cudaGetLastError();
}

}  // namespace g6
