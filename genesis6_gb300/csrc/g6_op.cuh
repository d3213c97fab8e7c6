// g6_op.cuh -- order-parameter state of the umbrella Monte Carlo chains
// (mc2.F90 OP_EP, OP_Q6T, OP_TRIANGLE) and the launchers of g6_opmc.cu.
#pragma once

#include <cuda_runtime.h>

#include "g6_internal.cuh"
#include "g6_mlp.cuh"

namespace g6 {

constexpr int OP_N5 = 48;     // neighbours within 5 A kept per molecule (about 17 in liquid water)
constexpr int OP_NB = 10;     // bonds (pairs within 3 A) per molecule: MAXBOND of Q6Local.F90:32
constexpr int OP_NBIN = 21;   // triangle histogram: 21 bins of 0.1 from -1 (Triangle.F90:64)
constexpr int OP_NM = 13;     // Y_6m, m = -6..6

// Device state, one entry per molecule unless noted.  n5*: the molecules
// within 5 A (label, vector molecule -> neighbour and its squared length, in
// the reference's minimum-image arithmetic); b*: the bonds (within 3 A) with
// the Y_6m of their direction; qs, nb, q6: the local Q6 sums, bond counts and
// values; hist: per chain the triangle counts; op: per chain the current
// order parameter.
struct OpDev {
  int kind;            // G6_OP_EP, G6_OP_Q6 or G6_OP_TRIANGLE
  int logarithmic;     // triangle: op = log(divergence)
  double ref[OP_NBIN]; // triangle reference histogram
  const double* umb;   // per chain: center, coefficient of the umbrella coeff (op - center)^2
  int* n5c;
  int* n5j;            // [n][OP_N5]
  double4* n5v;        // [n][OP_N5]: x, y, z, dd
  int* bc;
  int* bj;             // [n][OP_NB]
  double2* bq;         // [n][OP_NB][OP_NM]
  double2* qs;         // [n][OP_NM]
  int* nb;
  double* q6;
  int* hist;           // [nrep][OP_NBIN]
  double* op;          // [nrep]
  double* opsamp;      // optional: per chain the sampled order parameter
  int* flag;           // set to 1 when a neighbour list, a bond list or a trial's pool overflows
};

cudaError_t launch_op_prepare(const McArgs& a, const OpDev& o, cudaStream_t s);
cudaError_t launch_mc_op(const McArgs& a, const OpDev& o, int model, bool mixed, cudaStream_t s);

}  // namespace g6
