// g6_mlp.cuh -- learned Monte Carlo proposal widths: local-environment
// features, the 24-64-64-2 tanh MLP, and the Monte Carlo kernel arguments.
//
// Features of a molecule at a pose (24 floats):
//   [0,16)  radial shells: sum_j exp(-((r_j - c_k)/0.25)^2) for neighbour COMs
//           within 6.5 A, centres c_k = 2.4 + 0.25 k;
//   [16,24) tetrahedral-direction occupancy: for each of (up to) four charged
//           sites s with lab direction u_s, sum_j g(r_j) max(0, u_s . e_j)^4
//           where e_j is the unit vector towards neighbour j and g a first-
//           shell (centre 2.9 A, [16,20)) or second-shell (4.5 A, [20,24)) weight.
// These follow the local-order ideas of Tetrahedrality.F90:4-23 (directions of
// the four nearest neighbours) in a smooth, fixed-length form.
//
// Widths: sigma = sigma0 * (0.5 + 2 sigmoid(z)), so sigma stays inside
// (0.5, 2.5) x sigma0 and the Hastings ratio stays bounded.
#pragma once

#include "g6_internal.cuh"

namespace g6 {

constexpr int MLP_IN = 24, MLP_H = 64, MLP_OUT = 2;
// parameter offsets in one flat float array
constexpr int MLP_W1 = 0;                          // [H][IN]
constexpr int MLP_B1 = MLP_W1 + MLP_H * MLP_IN;    // [H]
constexpr int MLP_W2 = MLP_B1 + MLP_H;             // [H][H]
constexpr int MLP_B2 = MLP_W2 + MLP_H * MLP_H;     // [H]
constexpr int MLP_W3 = MLP_B2 + MLP_H;             // [OUT][H]
constexpr int MLP_B3 = MLP_W3 + MLP_OUT * MLP_H;   // [OUT]
constexpr int MLP_NPARAM = MLP_B3 + MLP_OUT;

struct MlpDev {
  const float* w;         // MLP_NPARAM parameters
  float feat_mean[MLP_IN];
  float feat_inv_std[MLP_IN];
  double sigma0_t, sigma0_r;
};

struct McArgs {
  int n, ntrial, nsamples, sample_every;
  RepDev rep;
  double body[MAXSITE][3];
  double* st;
  double* pk64;
  float* pk32f;           // the float4 packed poses viewed as floats
  uint32_t* fix;
  PairConst pc;
  CutConst cc;
  const double* beta;     // per chain
  const double* sigma_t;  // per chain (fixed widths)
  const double* sigma_r;
  double* energy;         // per chain running total (in/out)
  long long* counts;      // per chain: accepted, attempted (accumulated)
  double* samples;        // optional: per chain nsamples energies
  double* trace;          // optional: per chain per trial (dE, energy, accepted, target)
  float* records;         // optional: per chain per trial training record (MLP_REC floats)
  unsigned long long seed, counter;
  MlpDev mlp;
};

constexpr int MLP_REC = 2 * MLP_IN + 3;   // x_old, x_new, |dx|^2, |rot|^2, beta*dE (reduced units)

__device__ __forceinline__ float mlp_sigmoid(float z) { return 1.0f / (1.0f + __expf(-z)); }

// Forward pass on one warp (all 32 lanes participate): sigma_t, sigma_r.
__device__ __forceinline__ void mlp_widths(const MlpDev& m, const float* feat, double* st, double* sr) {
  const int lane = threadIdx.x & 31;
  const float* w = m.w;
  float x[MLP_IN];
#pragma unroll
  for (int k = 0; k < MLP_IN; ++k) x[k] = (feat[k] - m.feat_mean[k]) * m.feat_inv_std[k];
  float h1[2];
#pragma unroll
  for (int u = 0; u < 2; ++u) {
    const int o = lane + 32 * u;
    float s = w[MLP_B1 + o];
#pragma unroll
    for (int k = 0; k < MLP_IN; ++k) s += w[MLP_W1 + o * MLP_IN + k] * x[k];
    h1[u] = tanhf(s);
  }
  float h2[2];
#pragma unroll
  for (int u = 0; u < 2; ++u) {
    const int o = lane + 32 * u;
    float s = w[MLP_B2 + o];
    for (int k = 0; k < MLP_H; ++k) {
      const float hk = __shfl_sync(0xffffffffu, h1[k >> 5], k & 31);
      s += w[MLP_W2 + o * MLP_H + k] * hk;
    }
    h2[u] = tanhf(s);
  }
  float z[MLP_OUT];
#pragma unroll
  for (int q = 0; q < MLP_OUT; ++q) {
    float s = w[MLP_W3 + q * MLP_H + lane] * h2[0] + w[MLP_W3 + q * MLP_H + lane + 32] * h2[1];
#pragma unroll
    for (int mm = 16; mm >= 1; mm >>= 1) s += __shfl_xor_sync(0xffffffffu, s, mm);
    z[q] = s + w[MLP_B3 + q];
  }
  if (lane == 0) {
    *st = m.sigma0_t * (0.5 + 2.0 * (double)mlp_sigmoid(z[0]));
    *sr = m.sigma0_r * (0.5 + 2.0 * (double)mlp_sigmoid(z[1]));
  }
}

struct TrainArgs {
  int nrows;              // 2 * records in the batch (row 2i = x, row 2i+1 = x')
  const float* rec;       // records (MLP_REC floats each)
  const int* idx;         // optional: record index of batch entry b
  const float* w;         // parameters
  const float* mean;      // feature normalisation
  const float* istd;
  double s0t, s0r;
  float* X;               // [rows][IN] normalised inputs
  float* H1;              // [rows][H]
  float* H2;              // [rows][H]
  float* Z;               // [rows][OUT]
  float* G3;              // [rows][OUT] dL/dz
  float* D2;              // [rows][H]
  float* D1;              // [rows][H]
  float* grad;            // [NPARAM]
  double* loss;           // accumulated sum of -J over the batch
};

cudaError_t launch_mc(const McArgs& a, int model, bool mixed, bool learned, cudaStream_t s);
cudaError_t launch_mlp_grad(TrainArgs a, float inv_batch, cudaStream_t s);

// Block-wide feature accumulation (every thread of the block calls it) for
// molecule tg placed at COM `com` with lab site offsets `off` (index 1..NQ =
// charged sites).  Neighbours are the other molecules i0..i1-1 of its chain.
template <int NQ>
__device__ void mc_features(const McArgs& a, int tg, const double* com, const double (*off)[3], float* out, int i0,
                            int i1, const double L[3], const double iL[3]) {
  __shared__ float red[32][MLP_IN];
  constexpr int W64 = ((6 + 3 * NQ) + 1) / 2 * 2;
  float f[MLP_IN];
#pragma unroll
  for (int k = 0; k < MLP_IN; ++k) f[k] = 0.0f;
  float u[4][3];
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    if (s < NQ) {
      const double x = off[s + 1][0], y = off[s + 1][1], z = off[s + 1][2];
      const double inv = 1.0 / sqrt(x * x + y * y + z * z);
      u[s][0] = (float)(x * inv); u[s][1] = (float)(y * inv); u[s][2] = (float)(z * inv);
    } else {
      u[s][0] = u[s][1] = u[s][2] = 0.0f;
    }
  }
  for (int j = i0 + threadIdx.x; j < i1; j += blockDim.x) {
    if (j == tg) continue;
    const double* pj = a.pk64 + (size_t)j * W64;
    float d[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      double dl = pj[k] - com[k];
      dl -= round(dl * iL[k]) * L[k];
      d[k] = (float)dl;
    }
    const float r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    if (r2 > 6.5f * 6.5f || r2 <= 0.0f) continue;
    const float r = sqrtf(r2), ir = 1.0f / r;
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      const float t = (r - (2.4f + 0.25f * k)) * 4.0f;
      f[k] += __expf(-t * t);
    }
    const float t1 = (r - 2.9f) * (1.0f / 0.35f), t2 = (r - 4.5f) * 2.0f;
    const float g1 = __expf(-t1 * t1), g2 = __expf(-t2 * t2);
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      float c = (u[s][0] * d[0] + u[s][1] * d[1] + u[s][2] * d[2]) * ir;
      c = fmaxf(c, 0.0f);
      const float c4 = (c * c) * (c * c);
      f[16 + s] += g1 * c4;
      f[20 + s] += g2 * c4;
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < MLP_IN; ++k) {
    float v = f[k];
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) v += __shfl_xor_sync(0xffffffffu, v, m);
    if (lane == 0) red[warp][k] = v;
  }
  __syncthreads();
  if (threadIdx.x < MLP_IN) {
    float v = 0.0f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += red[w][threadIdx.x];
    out[threadIdx.x] = v;
  }
  __syncthreads();
}

}  // namespace g6
