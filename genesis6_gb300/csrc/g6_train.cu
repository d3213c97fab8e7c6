// g6_train.cu -- training of the proposal-width MLP on Monte Carlo records.
//
// A record holds the features of the target at the old and at the proposed
// pose (x, x'), the squared translation |d|^2 and rotation-vector |r|^2 of the
// move, and b = beta * dE (reduced units) -- all from a chain run with the
// plain fixed-width proposal (sigma0).  For widths s(x) = (s_t, s_r) the
// importance-weighted expected squared jump of the Metropolis-Hastings chain
// with the learned proposal is estimated by
//   J = mean_i  exp(min(lf_i, lr_i)) * D_i,
//   lf = log q_s(x'|x) - log q0(x'|x),
//   lr = log q_s(x|x') - b - log q0(x'|x),
//   log q_s(.|x) = -3 log s_t(x) - |d|^2 / (2 s_t(x)^2) - 3 log s_r(x) - |r|^2 / (2 s_r(x)^2),
//   D = w_move (|d|^2 / s0_t^2 + |r|^2 / s0_r^2) + w_energy b^2,
// i.e. the proposal density ratio times the MH acceptance min(1, e^-b q(x|x')/q(x'|x))
// times the jump (in configuration, scaled by the fixed widths, and in energy).
// The loss is -J.  Kernels: forward of both sides of every record (one warp
// per row, activations stored), the loss and dL/dz of the active branch,
// backward through the two tanh layers, weight gradients as reductions over
// rows (one thread per parameter), and Adam.
#include <cuda_runtime.h>

#include "g6_internal.cuh"
#include "g6_mlp.cuh"

namespace g6 {


__device__ __forceinline__ const float* row_feat(const TrainArgs& a, int row) {
  const int b = row >> 1;
  const int r = a.idx ? a.idx[b] : b;
  return a.rec + (size_t)r * MLP_REC + ((row & 1) ? MLP_IN : 0);
}

__global__ void k_mlp_forward(TrainArgs a) {
  const int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (row >= a.nrows) return;
  const float* f = row_feat(a, row);
  float x[MLP_IN];
#pragma unroll
  for (int k = 0; k < MLP_IN; ++k) x[k] = (f[k] - a.mean[k]) * a.istd[k];
  if (lane < MLP_IN) a.X[(size_t)row * MLP_IN + lane] = x[lane];
  const float* w = a.w;
  float h1[2], h2[2];
#pragma unroll
  for (int u = 0; u < 2; ++u) {
    const int o = lane + 32 * u;
    float s = w[MLP_B1 + o];
#pragma unroll
    for (int k = 0; k < MLP_IN; ++k) s += w[MLP_W1 + o * MLP_IN + k] * x[k];
    h1[u] = tanhf(s);
    a.H1[(size_t)row * MLP_H + o] = h1[u];
  }
#pragma unroll
  for (int u = 0; u < 2; ++u) {
    const int o = lane + 32 * u;
    float s = w[MLP_B2 + o];
    for (int k = 0; k < MLP_H; ++k) s += w[MLP_W2 + o * MLP_H + k] * __shfl_sync(0xffffffffu, h1[k >> 5], k & 31);
    h2[u] = tanhf(s);
    a.H2[(size_t)row * MLP_H + o] = h2[u];
  }
#pragma unroll
  for (int q = 0; q < MLP_OUT; ++q) {
    float s = w[MLP_W3 + q * MLP_H + lane] * h2[0] + w[MLP_W3 + q * MLP_H + lane + 32] * h2[1];
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) s += __shfl_xor_sync(0xffffffffu, s, m);
    if (lane == 0) a.Z[(size_t)row * MLP_OUT + q] = s + w[MLP_B3 + q];
  }
}

// Widths of the network for n raw feature rows (one thread per row; a
// diagnostic evaluation, e.g. of the width distribution over a sample).
__global__ void k_mlp_eval(const float* feat, long long n, const float* w, const float* mean, const float* istd,
                           double s0t, double s0r, double* st, double* sr) {
  const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  float x[MLP_IN], h1[MLP_H];
#pragma unroll
  for (int k = 0; k < MLP_IN; ++k) x[k] = (feat[r * MLP_IN + k] - mean[k]) * istd[k];
  for (int o = 0; o < MLP_H; ++o) {
    float t = w[MLP_B1 + o];
#pragma unroll
    for (int k = 0; k < MLP_IN; ++k) t = fmaf(w[MLP_W1 + o * MLP_IN + k], x[k], t);
    h1[o] = tanhf(t);
  }
  float z0 = w[MLP_B3], z1 = w[MLP_B3 + 1];
  for (int o = 0; o < MLP_H; ++o) {
    float t = w[MLP_B2 + o];
    for (int k = 0; k < MLP_H; ++k) t = fmaf(w[MLP_W2 + o * MLP_H + k], h1[k], t);
    const float h2 = tanhf(t);
    z0 = fmaf(w[MLP_W3 + o], h2, z0);
    z1 = fmaf(w[MLP_W3 + MLP_H + o], h2, z1);
  }
  st[r] = s0t * (MLP_SMIN + MLP_SSPAN * (double)mlp_sigmoid(z0));
  sr[r] = s0r * (MLP_SMIN + MLP_SSPAN * (double)mlp_sigmoid(z1));
}

cudaError_t launch_mlp_eval(const float* feat, long long n, const float* w, const float* mean, const float* istd,
                            double s0t, double s0r, double* st, double* sr, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_mlp_eval<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(feat, n, w, mean, istd, s0t, s0r, st, sr);
  return cudaGetLastError();
}

// Loss and dL/dz, one thread per record (both rows).
__global__ void k_mlp_loss(TrainArgs a, float inv_batch) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  double lossv = 0.0;
  if (2 * b < a.nrows) {
    const int r = a.idx ? a.idx[b] : b;
    const float* rc = a.rec + (size_t)r * MLP_REC;
    const double d2 = rc[2 * MLP_IN], r2 = rc[2 * MLP_IN + 1], bde = rc[2 * MLP_IN + 2];
    double s[2][2], sg[2][2];
    for (int side = 0; side < 2; ++side)
      for (int q = 0; q < 2; ++q) {
        const double z = a.Z[(size_t)(2 * b + side) * MLP_OUT + q];
        const double sgm = 1.0 / (1.0 + exp(-z));
        const double s0 = q == 0 ? a.s0t : a.s0r;
        s[side][q] = s0 * (MLP_SMIN + MLP_SSPAN * sgm);
        sg[side][q] = s0 * MLP_SSPAN * sgm * (1.0 - sgm);   // ds/dz
      }
    auto logq = [&](int side) {
      return -3.0 * log(s[side][0]) - d2 / (2.0 * s[side][0] * s[side][0]) - 3.0 * log(s[side][1]) -
             r2 / (2.0 * s[side][1] * s[side][1]);
    };
    const double lq0 = -3.0 * log(a.s0t) - d2 / (2.0 * a.s0t * a.s0t) - 3.0 * log(a.s0r) - r2 / (2.0 * a.s0r * a.s0r);
    const double lf = logq(0) - lq0;
    const double lr = logq(1) - bde - lq0;
    const int side = lf <= lr ? 0 : 1;
    const double l = side == 0 ? lf : lr;
    const double D = a.w_move * (d2 / (a.s0t * a.s0t) + r2 / (a.s0r * a.s0r)) + a.w_energy * bde * bde;
    const double J = exp(fmin(l, 30.0)) * D;
    lossv = -J;
    // d(-J)/dz_q on the active side = -J * dl/ds_q * ds/dz_q
    const double dls[2] = {-3.0 / s[side][0] + d2 / (s[side][0] * s[side][0] * s[side][0]),
                           -3.0 / s[side][1] + r2 / (s[side][1] * s[side][1] * s[side][1])};
    for (int q = 0; q < 2; ++q) {
      a.G3[(size_t)(2 * b + side) * MLP_OUT + q] = (float)(-J * dls[q] * sg[side][q] * inv_batch);
      a.G3[(size_t)(2 * b + 1 - side) * MLP_OUT + q] = 0.0f;
    }
  }
#pragma unroll
  for (int m = 16; m >= 1; m >>= 1) lossv += __shfl_xor_sync(0xffffffffu, lossv, m);
  if ((threadIdx.x & 31) == 0 && lossv != 0.0) atomicAdd(a.loss, lossv);
}

// Backward through the hidden layers, one warp per row.
__global__ void k_mlp_backward(TrainArgs a) {
  const int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (row >= a.nrows) return;
  const float* w = a.w;
  const float g0 = a.G3[(size_t)row * MLP_OUT], g1 = a.G3[(size_t)row * MLP_OUT + 1];
  float d2[2];
#pragma unroll
  for (int u = 0; u < 2; ++u) {
    const int o = lane + 32 * u;
    const float h = a.H2[(size_t)row * MLP_H + o];
    d2[u] = (w[MLP_W3 + o] * g0 + w[MLP_W3 + MLP_H + o] * g1) * (1.0f - h * h);
    a.D2[(size_t)row * MLP_H + o] = d2[u];
  }
#pragma unroll
  for (int u = 0; u < 2; ++u) {
    const int o = lane + 32 * u;   // unit of layer 1
    float s = 0.0f;
    for (int k = 0; k < MLP_H; ++k) s += w[MLP_W2 + k * MLP_H + o] * __shfl_sync(0xffffffffu, d2[k >> 5], k & 31);
    const float h = a.H1[(size_t)row * MLP_H + o];
    a.D1[(size_t)row * MLP_H + o] = s * (1.0f - h * h);
  }
}

// One thread per parameter: reduction over rows in a fixed order.
__global__ void k_mlp_wgrad(TrainArgs a) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= MLP_NPARAM) return;
  const float* A = nullptr;
  const float* B = nullptr;
  int lda = 0, ldb = 0, ia = 0, ib = -1;
  if (p < MLP_B1) { const int o = (p - MLP_W1) / MLP_IN, k = (p - MLP_W1) % MLP_IN; A = a.D1; lda = MLP_H; ia = o; B = a.X; ldb = MLP_IN; ib = k; }
  else if (p < MLP_W2) { A = a.D1; lda = MLP_H; ia = p - MLP_B1; }
  else if (p < MLP_B2) { const int o = (p - MLP_W2) / MLP_H, k = (p - MLP_W2) % MLP_H; A = a.D2; lda = MLP_H; ia = o; B = a.H1; ldb = MLP_H; ib = k; }
  else if (p < MLP_W3) { A = a.D2; lda = MLP_H; ia = p - MLP_B2; }
  else if (p < MLP_B3) { const int q = (p - MLP_W3) / MLP_H, k = (p - MLP_W3) % MLP_H; A = a.G3; lda = MLP_OUT; ia = q; B = a.H2; ldb = MLP_H; ib = k; }
  else { A = a.G3; lda = MLP_OUT; ia = p - MLP_B3; }
  float s = 0.0f;
  if (B) {
    for (int r = 0; r < a.nrows; ++r) s += A[(size_t)r * lda + ia] * B[(size_t)r * ldb + ib];
  } else {
    for (int r = 0; r < a.nrows; ++r) s += A[(size_t)r * lda + ia];
  }
  a.grad[p] = s;
}

__global__ void k_adam(float* w, const float* g, float* m, float* v, int np, float lr, float b1, float b2, float eps,
                       int t) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= np) return;
  const float gg = g[p];
  const float mm = b1 * m[p] + (1.0f - b1) * gg;
  const float vv = b2 * v[p] + (1.0f - b2) * gg * gg;
  m[p] = mm; v[p] = vv;
  const float mh = mm / (1.0f - powf(b1, (float)t)), vh = vv / (1.0f - powf(b2, (float)t));
  w[p] -= lr * mh / (sqrtf(vh) + eps);
}

// Feature statistics over the x side of nrec records: mean and 1/std.
__global__ void k_feat_stats(const float* rec, long long nrec, float* mean, float* istd) {
  const int k = blockIdx.x;
  double s = 0.0, s2 = 0.0;
  for (long long r = threadIdx.x; r < nrec; r += blockDim.x) {
    const double v = rec[(size_t)r * MLP_REC + k];
    s += v; s2 += v * v;
  }
  __shared__ double ps[256], ps2[256];
  ps[threadIdx.x] = s; ps2[threadIdx.x] = s2;
  __syncthreads();
  for (int o = blockDim.x / 2; o >= 1; o >>= 1) {
    if ((int)threadIdx.x < o) { ps[threadIdx.x] += ps[threadIdx.x + o]; ps2[threadIdx.x] += ps2[threadIdx.x + o]; }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double m = nrec ? ps[0] / nrec : 0.0;
    const double var = nrec ? ps2[0] / nrec - m * m : 1.0;
    mean[k] = (float)m;
    istd[k] = (float)(1.0 / sqrt(fmax(var, 1e-6)));
  }
}

cudaError_t launch_mlp_grad(TrainArgs a, float inv_batch, cudaStream_t s) {
  if (a.nrows <= 0) return cudaSuccess;
  const int warps_per_block = 4;
  const int blocks = (a.nrows + warps_per_block - 1) / warps_per_block;
  k_mlp_forward<<<blocks, 32 * warps_per_block, 0, s>>>(a);
  const int nb = a.nrows / 2;
  k_mlp_loss<<<(nb + 127) / 128, 128, 0, s>>>(a, inv_batch);
  k_mlp_backward<<<blocks, 32 * warps_per_block, 0, s>>>(a);
  k_mlp_wgrad<<<(MLP_NPARAM + 127) / 128, 128, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_adam(float* w, const float* g, float* m, float* v, float lr, int t, cudaStream_t s) {
  k_adam<<<(MLP_NPARAM + 255) / 256, 256, 0, s>>>(w, g, m, v, MLP_NPARAM, lr, 0.9f, 0.999f, 1e-8f, t);
  return cudaGetLastError();
}

cudaError_t launch_feat_stats(const float* rec, long long nrec, float* mean, float* istd, cudaStream_t s) {
  k_feat_stats<<<MLP_IN, 256, 0, s>>>(rec, nrec, mean, istd);
  return cudaGetLastError();
}

}  // namespace g6
