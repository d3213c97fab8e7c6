// g6_mlp.cuh -- learned Monte Carlo proposal widths: local-environment
// features, the 24-64-64-2 tanh MLP, and the Monte Carlo kernel arguments.
//
// Features of a molecule at a pose (24 floats):
//   [0,16)  radial shells: sum_j exp(-((r_j - c_k)/0.25)^2) for neighbour COMs
//           within 6 A, centres c_k = 2.4 + 0.225 k;
//   [16,24) tetrahedral-direction occupancy: for each of (up to) four charged
//           sites s with lab direction u_s, sum_j g(r_j) max(0, u_s . e_j)^4
//           where e_j is the unit vector towards neighbour j and g a first-
//           shell (centre 2.9 A, [16,20)) or second-shell (4.5 A, [20,24)) weight.
// These follow the local-order ideas of Tetrahedrality.F90:4-23 (directions of
// the four nearest neighbours) in a smooth, fixed-length form.
// Every pair term is rounded to an integer multiple of 2^-20 before it is
// summed, so a feature vector is an exact integer sum: the Monte Carlo kernel
// keeps the features of all molecules and updates the neighbours of a moved
// molecule by subtracting and adding single terms, and the result is bitwise
// what a fresh summation over the new configuration gives.
//
// Widths: sigma = sigma0 * (0.1 + 2.9 sigmoid(z)), so sigma stays inside
// (0.1, 3.0) x sigma0 and the Hastings ratio stays bounded.
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
// widths: sigma = sigma0 * (MLP_SMIN + MLP_SSPAN * sigmoid(z)), inside (0.1, 3.0) x sigma0
constexpr double MLP_SMIN = 0.1, MLP_SSPAN = 2.9;

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
  float fbody[MAXSITE][3];   // the same in FP32 (mixed trial poses)
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
  int* fcache;            // features of every molecule at its current pose (MLP_IN integers each)
  int* flag;              // set to 1 when a pose has more than MC_POOL feature neighbours
  float* udir;            // unit directions of every molecule's charged sites (12 floats each)
  int ncmax;              // molecules of the largest chain
  int fc_smem;            // set by launch_mc: each chain's feature cache lives in shared memory
  unsigned long long seed, counter;
  MlpDev mlp;
};

constexpr int MLP_REC = 2 * MLP_IN + 3;   // x_old, x_new, |dx|^2, |rot|^2, beta*dE (reduced units)

__device__ __forceinline__ float mlp_sigmoid(float z) { return 1.0f / (1.0f + __expf(-z)); }

struct TrainArgs {
  int nrows;              // 2 * records in the batch (row 2i = x, row 2i+1 = x')
  const float* rec;       // records (MLP_REC floats each)
  const int* idx;         // optional: record index of batch entry b
  const float* w;         // parameters
  const float* mean;      // feature normalisation
  const float* istd;
  double s0t, s0r;
  double w_move, w_energy;   // objective: w_move * scaled |jump|^2 + w_energy * (beta dE)^2
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

cudaError_t launch_mc(const McArgs& a, int model, bool mixed, int mode, cudaStream_t s);
cudaError_t launch_mlp_grad(TrainArgs a, float inv_batch, cudaStream_t s);
cudaError_t launch_mlp_eval(const float* feat, long long n, const float* w, const float* mean, const float* istd,
                            double s0t, double s0r, double* st, double* sr, cudaStream_t s);

}  // namespace g6
