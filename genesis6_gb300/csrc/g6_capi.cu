// g6_capi.cu -- context, model tables and the extern "C" entry points of g6gpu.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "g6_internal.cuh"
#include "g6_mlp.cuh"
#include "g6_op.cuh"

namespace g6 {

// ---------------------------------------------------------------------------
// Model tables (host).  Values and formulas follow the reference:
// TIP4P TIP4PModule.F90:43-97 + TIP4PConst.F90; TIP5P TIP5PModule.F90:38-83 +
// RigidModule.F90:429-477; ST2 ST2Module.F90:10-100 (float literals promoted).
// ---------------------------------------------------------------------------
static void five_site(ModelHost& m, double theta, double phi, double l1, double l2) {
  const double hmass = 1.0, omass = 16.0;
  double x[6] = {0}, y[6] = {0}, z[6] = {0};
  y[1] = l1 * std::sin(0.5 * theta); z[1] = l1 * std::cos(0.5 * theta);
  y[2] = -l1 * std::sin(0.5 * theta); z[2] = l1 * std::cos(0.5 * theta);
  x[3] = l2 * std::sin(0.5 * phi); z[3] = -l2 * std::cos(0.5 * phi);
  x[4] = -l2 * std::sin(0.5 * phi); z[4] = -l2 * std::cos(0.5 * phi);
  const double zshift = z[1] * 2.0 * hmass / (2.0 * hmass + omass);
  for (int i = 0; i < 5; ++i) z[i] = z[i] - zshift;
  for (int s = 0; s < 6; ++s) { m.body[s][0] = x[s]; m.body[s][1] = y[s]; m.body[s][2] = z[s]; }
  m.I[0] = omass * (y[0] * y[0] + z[0] * z[0]) + hmass * (y[1] * y[1] + z[1] * z[1]) * 2.0;
  m.I[1] = omass * (z[0] * z[0] + x[0] * x[0]) + hmass * (z[1] * z[1] + x[1] * x[1]) * 2.0;
  m.I[2] = omass * (x[0] * x[0] + y[0] * y[0]) + hmass * (x[1] * x[1] + y[1] * y[1]) * 2.0;
  m.mass = 2.0 * hmass + omass;
  m.nsite = 6;
  m.nq = 4;
}

static const double ST2_QM = (double)(-0.2357f), ST2_QH = (double)(+0.2357f);
static const double ST2_EPS = (double)(0.52605e-21f) * NA * 1e-3, ST2_SIG = 3.100;

// The kernels' layout is the reference's for TIP4P, TIP5P and ST2 (LJ site,
// charged sites, COM).  SPC/E (SPCEModule.F90:28-71: O carries the LJ site and
// a charge) becomes LJ O, charged O, H, H for the kernels.
static void reference_layout(ModelHost& m) {
  m.nref = m.nsite;
  for (int s = 0; s < MAXSITE; ++s) {
    m.site[s] = s;
    for (int k = 0; k < 3; ++k) { m.rbody[s][k] = m.body[s][k]; m.rparam[s][k] = m.param[s][k]; }
  }
}

static bool make_model_sites(int model, ModelHost& m);

bool make_model(int model, ModelHost& m) {
  if (!make_model_sites(model, m)) return false;
  if (model != G6_SPCE && model != G6_OPLSMEOH) reference_layout(m);
  return true;
}

static bool make_model_sites(int model, ModelHost& m) {
  m = ModelHost();
  m.model = model;
  if (model == G6_OPLSMEOH) {
    // Rigid_OPLSMeOH_Constructor RigidModule.F90:391-426 (Me, O, H, COM; masses
    // 15, 16, 1), oplsmeoh_setinteraction OPLSMeOHModule.F90:82-101.  Two LJ
    // sites: only the site-pair-table kernels (g6_force_sites_hetero) run it.
    const double mass[4] = {15.0, 16.0, 1.0, 0.0};
    const double x[4] = {0.0133, -0.0634, 0.8152, 0.0}, y[4] = {0.7666, -0.6559, -1.0042, 0.0};
    m.nref = 4;
    for (int s = 0; s < 4; ++s) {
      m.rbody[s][0] = x[s]; m.rbody[s][1] = y[s]; m.rbody[s][2] = 0.0;
      m.I[0] = m.I[0] + mass[s] * (y[s] * y[s]);
      m.I[1] = m.I[1] + mass[s] * (x[s] * x[s]);
      m.I[2] = m.I[2] + mass[s] * (x[s] * x[s] + y[s] * y[s]);
      m.mass = m.mass + mass[s];
    }
    m.rparam[0][0] = 0.265; m.rparam[0][1] = 0.207 * CA; m.rparam[0][2] = 3.775;
    m.rparam[1][0] = -0.700; m.rparam[1][1] = 0.170 * CA; m.rparam[1][2] = 3.070;
    m.rparam[2][0] = 0.435;
    m.nsite = 0; m.nq = 0;   // no layout for the LJ-site + charged-site kernels
    return true;
  }
  if (model == G6_SPCE) {
    const double theta = 109.5 * PI / 180.0, l1 = 1.0, hmass = 1.0, omass = 16.0;
    double y[4] = {0.0, l1 * std::sin(0.5 * theta), -l1 * std::sin(0.5 * theta), 0.0};
    double z[4] = {0.0, l1 * std::cos(0.5 * theta), l1 * std::cos(0.5 * theta), 0.0};
    const double zshift = z[1] * 2.0 * hmass / (2.0 * hmass + omass);
    for (int i = 0; i < 3; ++i) z[i] = z[i] - zshift;
    m.nref = 4;
    for (int s = 0; s < 4; ++s) { m.rbody[s][0] = 0.0; m.rbody[s][1] = y[s]; m.rbody[s][2] = z[s]; }
    const double qo = -0.8476, qh = 0.4238, eps = 78.208 / J2K * 1e-3, sig = 3.166;
    m.rparam[0][0] = qo; m.rparam[0][1] = eps; m.rparam[0][2] = sig;
    m.rparam[1][0] = qh; m.rparam[2][0] = qh;
    m.I[0] = omass * (y[0] * y[0] + z[0] * z[0]) + hmass * (y[1] * y[1] + z[1] * z[1]) * 2.0;
    m.I[1] = omass * (z[0] * z[0]) + hmass * (z[1] * z[1]) * 2.0;
    m.I[2] = omass * (y[0] * y[0]) + hmass * (y[1] * y[1]) * 2.0;
    m.mass = 2.0 * hmass + omass;
    // kernel layout: LJ O, charged O, H, H, COM
    const int map[5] = {0, 0, 1, 2, 3};
    m.nsite = 5; m.nq = 3;
    for (int s = 0; s < 5; ++s) {
      m.site[s] = map[s];
      for (int k = 0; k < 3; ++k) m.body[s][k] = m.rbody[map[s]][k];
    }
    m.param[0][1] = eps; m.param[0][2] = sig;
    m.param[1][0] = qo; m.param[2][0] = qh; m.param[3][0] = qh;
    return true;
  }
  if (model == G6_TIP4P) {
    m.nsite = 5; m.nq = 3;
    const double y[5] = {0.0, 0.0, 7.56950327263661182e-01, -7.56950327263661182e-01, 0.0};
    const double z[5] = {-6.50980307353661025e-02, 8.49019692646338919e-02, 5.20784245882928820e-01,
                         5.20784245882928820e-01, 0.0};
    for (int s = 0; s < 5; ++s) { m.body[s][0] = 0; m.body[s][1] = y[s]; m.body[s][2] = z[s]; }
    m.I[0] = 1.75618411509879202e+00; m.I[1] = 6.10236519209664374e-01; m.I[2] = 1.14594759588912742e+00;
    m.mass = 18.0;
    m.param[1][0] = -1.04; m.param[2][0] = 0.52; m.param[3][0] = 0.52;
    m.param[0][1] = 0.15504166666666666666666 * CA; m.param[0][2] = 3.15357794197649532464;
    return true;
  }
  if (model == G6_TIP5P) {
    five_site(m, 104.52 * PI / 180.0, 109.47 * PI / 180.0, 0.9572, 0.70);
    m.param[1][0] = 0.2410; m.param[2][0] = 0.2410; m.param[3][0] = -0.2410; m.param[4][0] = -0.2410;
    m.param[0][1] = 0.6694; m.param[0][2] = 3.12;
    return true;
  }
  if (model == G6_ST2) {
    const double th = 109.47 * PI / 180.0;
    five_site(m, th, th, 1.0, 0.8);
    m.param[1][0] = ST2_QH; m.param[2][0] = ST2_QH; m.param[3][0] = ST2_QM; m.param[4][0] = ST2_QM;
    m.param[0][1] = ST2_EPS; m.param[0][2] = ST2_SIG;
    return true;
  }
  return false;
}

static inline double p6(double x) { double x2 = x * x; return x2 * x2 * x2; }

// Pair constants for the chosen path.  PATH_STD: StdInteraction.F90:201-222
// (q_i q_j COEFF KX2X J2I; LB-mixed aa, bb).  PATH_CUSTOM: the hand kernels'
// precomputed products (TIP4PConst.F90:4-11, ST2Module.F90:123-127).
void make_pair_const(const ModelHost& m, int path, PairConst& pc) {
  std::memset(&pc, 0, sizeof pc);
  const int nq = m.nq;
  const bool custom = path == G6_PATH_CUSTOM;
  if (custom && m.model == G6_TIP4P) {
    const double WM = -1.04, WH = 0.52;
    const double WWMM = WM * WM * COEFF * 100.0, WWMH = WM * WH * COEFF * 100.0, WWHH = WH * WH * COEFF * 100.0;
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) pc.qq[a][b] = (a == 0 && b == 0) ? WWMM : ((a == 0 || b == 0) ? WWMH : WWHH);
    pc.aa = 600000.0 * CA * 100.0;
    pc.bb = -610.0 * CA * 100.0;
  } else if (custom && m.model == G6_ST2) {
    const double QMM = ST2_QM * ST2_QM * COEFF * 100.0, QHM = ST2_QH * ST2_QM * COEFF * 100.0,
                 QHH = ST2_QH * ST2_QH * COEFF * 100.0;
    for (int a = 0; a < 4; ++a)
      for (int b = 0; b < 4; ++b) {
        const bool ah = a < 2, bh = b < 2;
        pc.qq[a][b] = (ah && bh) ? QHH : ((!ah && !bh) ? QMM : QHM);
      }
    const double s6 = p6(ST2_SIG);
    pc.aa = 4.0 * ST2_EPS * (s6 * s6) * 100.0;
    pc.bb = -4.0 * ST2_EPS * s6 * 100.0;
    pc.taper = 1;
    pc.rl = 2.0160; pc.ru = 3.1287;
    pc.w3 = (pc.ru - pc.rl) * (pc.ru - pc.rl) * (pc.ru - pc.rl);
  } else {
    for (int a = 0; a < nq; ++a)
      for (int b = 0; b < nq; ++b) pc.qq[a][b] = m.param[a + 1][0] * m.param[b + 1][0] * COEFF * KX2X * J2I * 1.0;
    const double ljeps = std::sqrt(m.param[0][1] * m.param[0][1]);
    const double ljsig = p6((m.param[0][2] + m.param[0][2]) * 0.5);
    pc.aa = 4.0 * ljeps * ljsig * ljsig * KX2X * J2I * 1.0;
    pc.bb = -4.0 * ljeps * ljsig * KX2X * J2I * 1.0;
  }
  for (int a = 0; a < MAXQ; ++a)
    for (int b = 0; b < MAXQ; ++b) pc.fqq[a][b] = (float)pc.qq[a][b];
  pc.faa = (float)pc.aa; pc.fbb = (float)pc.bb;
  pc.frl = (float)pc.rl; pc.fru = (float)pc.ru; pc.fw3 = (float)pc.w3;
}

// cutoff_initialize CutoffModule.F90:25-36 (x**5 by binary powering).
void make_cut_const(double rin, double rout, CutConst& cc) {
  const double x = rin - rout, x2 = x * x;
  cc.rin = rin; cc.rout = rout;
  cc.c1 = 1.0 / (x * (x2 * x2));
  cc.c2 = cc.c1 * 30.0;
  cc.rin2 = rin * rin; cc.rout2 = rout * rout;
  cc.frin = (float)rin; cc.frout = (float)rout; cc.frin2 = (float)cc.rin2; cc.frout2 = (float)cc.rout2;
  cc.fc1 = (float)cc.c1; cc.fc2 = (float)cc.c2;
}

// NeighborCell_ListHomo GridModule.F90:279-374 (maxradius == 0): half-shell
// offsets (kind 0) and self-mirror offsets (kind 1) as (x,y,z,kind).
static void homo_stencil(const int nd[3], std::vector<int>& out) {
  int nmax[3], nmin[3];
  for (int d = 0; d < 3; ++d) {
    nmax[d] = std::min(1, (nd[d] - 1) / 2);
    nmin[d] = std::max(-1, -(nd[d] / 2));
  }
  std::vector<int> mark((size_t)nd[0] * nd[1] * nd[2], 0);
  auto at = [&](int x, int y, int z) -> int& { return mark[((size_t)z * nd[1] + y) * nd[0] + x]; };
  for (int jz = nmin[2]; jz <= nmax[2]; ++jz) {
    const int pz = jz < 0 ? jz + nd[2] : jz, mz = pz == 0 ? 0 : nd[2] - pz;
    for (int jy = nmin[1]; jy <= nmax[1]; ++jy) {
      const int py = jy < 0 ? jy + nd[1] : jy, my = py == 0 ? 0 : nd[1] - py;
      for (int jx = nmin[0]; jx <= nmax[0]; ++jx) {
        const int px = jx < 0 ? jx + nd[0] : jx, mx = px == 0 ? 0 : nd[0] - px;
        if (at(px, py, pz) == 0) {
          at(mx, my, mz) += 1;
          at(px, py, pz) += 1;
          out.push_back(px); out.push_back(py); out.push_back(pz);
          out.push_back(at(px, py, pz) != 1 ? 1 : 0);
        }
      }
    }
  }
}

}  // namespace g6

using namespace g6;

// ---------------------------------------------------------------------------
// Context
// ---------------------------------------------------------------------------
struct HostGrid {
  std::vector<int> nd, cell_off;
  std::vector<double> cell, icell;
  int ncell = 0;
  int* d_nd = nullptr; double* d_edge = nullptr; double* d_icell = nullptr; int* d_cell_off = nullptr;
  int* d_cell = nullptr; int* d_slot = nullptr; int* d_count = nullptr; int* d_start = nullptr; int* d_cellmol = nullptr;
  uint4* d_cellfix = nullptr;
  bool valid = false;
};

struct g6_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  std::vector<void*> allocs;      // freed on redefinition / destroy
  // system
  bool have_system = false, have_cut = false, have_state = false;
  int model = 0, path = 0, prec = 0, nrep = 0, n = 0, nq = 0, w64 = 0, npk = 0;
  ModelHost mh;
  PairConst pc;
  CutConst cc;
  double req = 0.0, skin = 1.0;
  std::vector<int> off;
  std::vector<double> L;
  int lpi = 0;                    // lanes per molecule in the force kernel (0 = default)
  int step_lpi = 0;               // lanes per molecule of the MD step's force kernel (0 = default)
  int step_mpw = 0;               // mixed MD step: molecules per warp of the integrator kernel (0 = default)
  int step_half = -1;             // mixed MD step: 1 half list, 0 full list, -1 default
  bool half_fixed = false;        // step_half set by g6_set_shape (the tuner keeps it)
  int coop_grid = 0;              // blocks of the cooperative rebuild kernel
  // device arrays
  int* d_off = nullptr; int* d_mol_rep = nullptr; double* d_L = nullptr; double* d_invL = nullptr;
  float* d_fscale = nullptr;
  double* d_st = nullptr; double* d_tmat = nullptr; double* d_pk64 = nullptr; float4* d_pk32 = nullptr;
  uint32_t* d_fix = nullptr;
  double* d_tmat1 = nullptr; double* d_pk64_1 = nullptr; float4* d_pk32_1 = nullptr; uint32_t* d_fix1 = nullptr;
  float4* d_pkq = nullptr; float4* d_pkq_1 = nullptr;   // list-kernel records (fixed COM, float quaternion)
  double *d_F = nullptr, *d_tl = nullptr, *d_emol = nullptr, *d_wmol = nullptr;
  int* d_npin = nullptr;
  float4* d_fres = nullptr;       // mixed MD step: per-molecule float-pair results of the pair kernel
  float4* d_jacc = nullptr;       // mixed MD step, half list: j-side force and torque (zero between steps)
  double* d_jacc64 = nullptr;     // FP64 MD step, half list: the same in FP64, 6 SoA columns
  double* d_save = nullptr;       // state at the start of the current run (row-overflow recovery)
  int cap_request = 0;            // neighbour-list row capacity set by g6_set_shape or raised after an overflow
  bool overflow_recovered = false;   // the last run overflowed a row and was rolled back
  double* d_stage = nullptr;      // AoS staging (53 n)
  // grids
  HostGrid gref, glist;
  bool list_valid = false;   // the device neighbour list matches glist (built since the grid was made)
  bool rows_half = false;    // the device rows hold only the half-list pairs (built by a half-list MD run)
  std::vector<int> sten, sten_off;
  int* d_sten = nullptr; int* d_sten_off = nullptr;
  // neighbour list
  int cap = 0;
  int ccap = 0;   // in-range entries per row held by the mixed list kernel's shared memory
  int* d_nbr = nullptr; int* d_nnb = nullptr; double* d_com_build = nullptr; int* d_overflow = nullptr;
  uint32_t* d_fix_build = nullptr;
  float* d_stf = nullptr;   // mixed precision: small Gear terms during a run
  // reductions and control
  int nblk = 0;
  double* d_part = nullptr; unsigned int* d_gmax = nullptr; double* d_red = nullptr; int* d_repcnt = nullptr;
  char* d_ctl = nullptr;   // the control block (ctl_layout); the pointers around it point into it
  double* d_rfac = nullptr;   // per replica temperature and pressure factors
  double* d_fixs = nullptr;   // per replica and axis 2^32 / L
  unsigned int* d_done = nullptr; int* d_ctrl = nullptr;
  ThermoDev* d_th = nullptr; double* d_scale = nullptr; double* d_beta = nullptr; int* d_acc = nullptr;
  double* d_epot_rep = nullptr;
  double* d_xtemp = nullptr; int* d_slot = nullptr; int* d_moved = nullptr;   // replica-exchange scratch
  // Monte Carlo and the proposal-width MLP
  double *d_sig_t = nullptr, *d_sig_r = nullptr, *d_energy = nullptr;
  long long* d_counts = nullptr;
  double* d_samples = nullptr; size_t samples_cap = 0;
  double* d_trace = nullptr; size_t trace_cap = 0;
  float* d_rec = nullptr; size_t rec_cap = 0; long long nrec = 0;   // training records
  float* d_mlp = nullptr;          // parameters
  int* d_fcache = nullptr;         // per-molecule features at the current pose (Monte Carlo)
  int* d_mcflag = nullptr;         // Monte Carlo: too many feature neighbours
  float* d_udir = nullptr;         // Monte Carlo: charged-site directions per molecule
  OpDev opd{};                     // umbrella Monte Carlo: order-parameter state (allocated on first use)
  bool have_op = false;
  double* d_umb = nullptr;         // per chain: umbrella center, coefficient
  double* d_opsamp = nullptr; size_t opsamp_cap = 0;
  float h_mean[MLP_IN] = {0}, h_istd[MLP_IN] = {0};
  double sig0_t = 0.15, sig0_r = 0.15;
  double obj_move = 1.0, obj_energy = 0.0;   // training objective weights (g6_mlp_objective)
  bool have_mlp = false;
  // pair set
  long long* d_pcnt = nullptr;
  long long npairs = -1;
  size_t pair_capacity = 0;
  int* d_pi = nullptr; int* d_pj = nullptr;
  double *d_ox = nullptr, *d_oy = nullptr, *d_oz = nullptr, *d_hh = nullptr, *d_dh = nullptr;
  // scratch for the pair-list entry points (grow only)
  void* d_scratch = nullptr; size_t scratch_bytes = 0;
  // log buffer
  double* d_log = nullptr; size_t log_cap = 0;
  // pinned host staging for g6_md_step_host
  // pinned host block for the small per-run transfers (thermostats, control
  // words, per-replica factors, read-backs), so that they are asynchronous
  char* h_pinned = nullptr; size_t pinned_bytes = 0;
  char* d_pinned = nullptr;   // the device's address of h_pinned
  cudaEvent_t pin_ev = nullptr;   // the last uploads from the block have been read
  // graph of a block of MD steps
  cudaGraphExec_t graph = nullptr;
  int graph_steps = 0;
  double graph_dt = 0.0;
  int graph_log = -1;
  std::vector<double> last_epot;  // per replica, from the last MD step
  unsigned long long steps_done = 0;
  unsigned long long seed = 0;
  // open g6_md_begin .. g6_md_end run
  bool in_run = false, run_log = false;
  double run_dt = 0.0;
  int run_max = 0, run_done = 0;
  cudaGraphExec_t graph1 = nullptr;   // one step, for step-by-step advancing
  // g6_md_step_host with a pinned host record: the whole call as one graph,
  // for one record pointer, dt, log choice and lane width
  cudaGraphExec_t graph_host = nullptr;
  const double* ghost_rec = nullptr; double ghost_dt = 0.0; bool ghost_log = false; int ghost_lpi = 0;
  int step_timing = 0;                // 1: graph1 carries events around the step; 2: and around the kernel
  cudaEvent_t sev[4] = {nullptr, nullptr, nullptr, nullptr};
};

static int fail(g6_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}
static int cuda_fail(g6_ctx* c, cudaError_t e, const char* what) {
  return fail(c, G6_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
#define CK(call)                                                   \
  do {                                                             \
    cudaError_t e_ = (call);                                       \
    if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call);       \
  } while (0)

template <class T>
static cudaError_t dalloc(g6_ctx* c, T** p, size_t count) {
  void* q = nullptr;
  cudaError_t e = cudaMalloc(&q, std::max<size_t>(count, 1) * sizeof(T));
  if (e != cudaSuccess) return e;
  c->allocs.push_back(q);
  *p = (T*)q;
  return cudaMemset(q, 0, std::max<size_t>(count, 1) * sizeof(T));
}

static void drop_graphs(g6_ctx* c) {
  if (c->graph) { cudaGraphExecDestroy(c->graph); c->graph = nullptr; }
  if (c->graph1) { cudaGraphExecDestroy(c->graph1); c->graph1 = nullptr; }
  if (c->graph_host) { cudaGraphExecDestroy(c->graph_host); c->graph_host = nullptr; }
}

static void free_all(g6_ctx* c) {
  drop_graphs(c);
  for (int k = 0; k < 4; ++k)
    if (c->sev[k]) { cudaEventDestroy(c->sev[k]); c->sev[k] = nullptr; }
  c->step_timing = 0;
  for (void* p : c->allocs) cudaFree(p);
  c->allocs.clear();
  if (c->d_scratch) { cudaFree(c->d_scratch); c->d_scratch = nullptr; c->scratch_bytes = 0; }
  if (c->d_log) { cudaFree(c->d_log); c->d_log = nullptr; c->log_cap = 0; }
  if (c->d_samples) { cudaFree(c->d_samples); c->d_samples = nullptr; c->samples_cap = 0; }
  if (c->d_trace) { cudaFree(c->d_trace); c->d_trace = nullptr; c->trace_cap = 0; }
  if (c->d_opsamp) { cudaFree(c->d_opsamp); c->d_opsamp = nullptr; c->opsamp_cap = 0; }
  if (c->d_rec) { cudaFree(c->d_rec); c->d_rec = nullptr; c->rec_cap = 0; c->nrec = 0; }
  c->have_mlp = false;
  if (c->h_pinned) { cudaFreeHost(c->h_pinned); c->h_pinned = nullptr; c->d_pinned = nullptr; c->pinned_bytes = 0; }
  if (c->pin_ev) { cudaEventDestroy(c->pin_ev); c->pin_ev = nullptr; }
  c->gref = HostGrid(); c->glist = HostGrid();
  c->list_valid = false;
  c->pair_capacity = 0; c->npairs = -1; c->cap = 0;
}

static RepDev rep_dev(const g6_ctx* c) {
  RepDev r;
  r.nrep = c->nrep; r.off = c->d_off; r.mol_rep = c->d_mol_rep; r.L = c->d_L; r.invL = c->d_invL; r.fscale = c->d_fscale;
  return r;
}
static GridDev grid_dev(const HostGrid& g) {
  GridDev d;
  d.ncell_total = g.ncell; d.nd = g.d_nd; d.cell = g.d_edge; d.icell = g.d_icell; d.cell_off = g.d_cell_off;
  return d;
}

// Grid_Update (adaptive), GridModule.F90:95-125 and 473-501, per replica.
static int build_grid(g6_ctx* ctx, HostGrid& g, double edge, bool with_stencil) {
  const int R = ctx->nrep;
  g.nd.assign(3 * R, 1); g.cell.assign(3 * R, 0.0); g.icell.assign(3 * R, 0.0); g.cell_off.assign(R + 1, 0);
  if (with_stencil) { ctx->sten.clear(); ctx->sten_off.assign(R + 1, 0); }
  for (int r = 0; r < R; ++r) {
    for (int d = 0; d < 3; ++d) {
      int nd = (int)(ctx->L[3 * r + d] / edge);
      nd = std::max(1, nd);
      g.nd[3 * r + d] = nd;
      g.cell[3 * r + d] = ctx->L[3 * r + d] / nd;
      g.icell[3 * r + d] = 1.0 / g.cell[3 * r + d];
    }
    g.cell_off[r + 1] = g.cell_off[r] + g.nd[3 * r] * g.nd[3 * r + 1] * g.nd[3 * r + 2];
    if (with_stencil) {
      homo_stencil(&g.nd[3 * r], ctx->sten);
      ctx->sten_off[r + 1] = (int)ctx->sten.size() / 4;
    }
  }
  g.ncell = g.cell_off[R];
  const int n = ctx->n;
  if (!g.d_nd) {
    CK(dalloc(ctx, &g.d_nd, 3 * R)); CK(dalloc(ctx, &g.d_edge, 3 * R)); CK(dalloc(ctx, &g.d_icell, 3 * R));
    CK(dalloc(ctx, &g.d_cell_off, R + 1)); CK(dalloc(ctx, &g.d_cell, n)); CK(dalloc(ctx, &g.d_slot, n));
    CK(dalloc(ctx, &g.d_cellmol, n)); CK(dalloc(ctx, &g.d_cellfix, n));
  }
  // cell-count arrays are sized per grid (re-allocated if the grid grows)
  CK(dalloc(ctx, &g.d_count, g.ncell + 1));
  CK(dalloc(ctx, &g.d_start, g.ncell + 1));
  CK(cudaMemcpy(g.d_nd, g.nd.data(), 3 * R * sizeof(int), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(g.d_edge, g.cell.data(), 3 * R * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(g.d_icell, g.icell.data(), 3 * R * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(g.d_cell_off, g.cell_off.data(), (R + 1) * sizeof(int), cudaMemcpyHostToDevice));
  if (with_stencil) {
    CK(dalloc(ctx, &ctx->d_sten, std::max<size_t>(ctx->sten.size(), 4)));
    CK(dalloc(ctx, &ctx->d_sten_off, R + 1));
    CK(cudaMemcpy(ctx->d_sten, ctx->sten.data(), ctx->sten.size() * sizeof(int), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ctx->d_sten_off, ctx->sten_off.data(), (R + 1) * sizeof(int), cudaMemcpyHostToDevice));
  }
  g.valid = true;
  return G6_OK;
}

static double grid_edge_ref(const g6_ctx* c) { return c->req > 0.0 ? c->req : c->cc.rout; }

// Effective Verlet margin: rc + skin must not exceed half the smallest box edge.
static double effective_skin(const g6_ctx* c) {
  double s = c->skin;
  for (int r = 0; r < c->nrep; ++r)
    for (int d = 0; d < 3; ++d) s = std::min(s, 0.5 * c->L[3 * r + d] - c->cc.rout);
  return std::max(0.0, s);
}

static int check_ready(g6_ctx* ctx, bool need_state) {
  if (!ctx) return G6_ERR_ARG;
  if (!ctx->have_system) return fail(ctx, G6_ERR_STATE, "no system defined (g6_system)");
  if (!ctx->have_cut) return fail(ctx, G6_ERR_STATE, "no cutoff defined (g6_set_cutoff)");
  if (need_state && !ctx->have_state) return fail(ctx, G6_ERR_STATE, "no state uploaded");
  for (int r = 0; r < ctx->nrep; ++r)
    for (int d = 0; d < 3; ++d)
      if (!(ctx->cc.rout <= 0.5 * ctx->L[3 * r + d]))
        return fail(ctx, G6_ERR_ARG, "cutoff exceeds half the box edge (minimum image)");
  CK(cudaSetDevice(ctx->device));
  return G6_OK;
}

// Neighbour-list grid, capacity and buffers for the current box/cutoff/skin.
static int prepare_list(g6_ctx* ctx) {
  if (ctx->glist.valid && ctx->cap > 0) return G6_OK;
  ctx->list_valid = false;
  const double skin = effective_skin(ctx);
  const double rlist = ctx->cc.rout + skin;
  // cells of at least half the list radius (list_row visits two cells each way)
  int rc = build_grid(ctx, ctx->glist, 0.5 * rlist, false);
  if (rc) return rc;
  double rho = 0.0;
  for (int r = 0; r < ctx->nrep; ++r) {
    const double V = ctx->L[3 * r] * ctx->L[3 * r + 1] * ctx->L[3 * r + 2];
    rho = std::max(rho, (ctx->off[r + 1] - ctx->off[r]) / V);
  }
  const double expect = 4.18879020478639 * rlist * rlist * rlist * rho;
  int cap = (int)(2.0 * expect + 64.0);
  int nmax = 0;
  for (int r = 0; r < ctx->nrep; ++r) nmax = std::max(nmax, ctx->off[r + 1] - ctx->off[r]);
  if (ctx->cap_request > 0) cap = ctx->cap_request;
  cap = std::min(cap, std::max(nmax - 1, 1));
  cap = (cap + 31) / 32 * 32;
  if (cap != ctx->cap) {
    CK(dalloc(ctx, &ctx->d_nbr, (size_t)cap * ctx->n));
    ctx->cap = cap;
  }
  // the in-range part of a row (rc, not rc + skin): 1.5x the expected count +
  // 64; a row beyond it is reported as an overflow and the run repeated with
  // the full capacity (cap_request set by the recovery)
  const double rcut = ctx->cc.rout;
  const int want = (int)(1.5 * 4.18879020478639 * rcut * rcut * rcut * rho + 64.0);
  ctx->ccap = ctx->cap_request > 0 ? cap : std::min(cap, (want + 31) / 32 * 32);
  return G6_OK;
}

static int prepare_ref_grid(g6_ctx* ctx) {
  if (ctx->gref.valid) return G6_OK;
  return build_grid(ctx, ctx->gref, grid_edge_ref(ctx), true);
}

static PlaceArgs place_args(g6_ctx* c) {
  PlaceArgs p;
  std::memset(&p, 0, sizeof p);
  p.n = c->n; p.nq = c->nq; p.npk = c->npk; p.w64 = c->w64;
  p.rep = rep_dev(c);
  for (int s = 0; s < MAXSITE; ++s)
    for (int k = 0; k < 3; ++k) { p.body[s][k] = c->mh.body[s][k]; p.fbody[s][k] = (float)c->mh.body[s][k]; }
  p.st = c->d_st; p.tmat = c->d_tmat; p.pk64 = c->d_pk64; p.pk32 = c->d_pk32; p.pkq = c->d_pkq; p.fix = c->d_fix;
  return p;
}

static CellArgs cell_args(g6_ctx* c, HostGrid& g, const int* ctrl) {
  CellArgs a;
  std::memset(&a, 0, sizeof a);
  a.n = c->n; a.rep = rep_dev(c); a.g = grid_dev(g); a.com = c->d_st;
  a.cell = g.d_cell; a.slot = g.d_slot; a.count = g.d_count; a.ctrl = ctrl;
  return a;
}

static ListArgs list_args(g6_ctx* c, const int* ctrl, bool half = false) {
  ListArgs a;
  std::memset(&a, 0, sizeof a);
  a.n = c->n; a.cap = c->cap; a.rep = rep_dev(c); a.g = grid_dev(c->glist); a.cell = c->glist.d_cell;
  a.start = c->glist.d_start; a.cellmol = c->glist.d_cellmol; a.fix = c->d_fix; a.fix1 = c->d_fix1; a.com = c->d_st;
  a.cellfix = c->glist.d_cellfix;
  a.com_build = c->d_com_build;
  a.fix_build = c->d_fix_build;
  const double rl = c->cc.rout + effective_skin(c);
  a.rlist2 = (float)(rl * rl) + 1e-3f;   // superset margin over the fixed-point rounding
  a.nbr = c->d_nbr; a.nnb = c->d_nnb; a.overflow = c->d_overflow; a.ctrl = ctrl;
  a.half = half ? 1 : 0;
  return a;
}

// MD steps of this context evaluate each pair once (mixed precision, half list).
static bool step_uses_half(const g6_ctx* c) { return c->step_half > 0; }

static ForceArgs force_args(g6_ctx* c) {
  ForceArgs a;
  std::memset(&a, 0, sizeof a);
  a.n = c->n; a.cap = c->cap; a.stride_pk32 = c->npk; a.nbr = c->d_nbr; a.nnb = c->d_nnb; a.rep = rep_dev(c);
  a.pk64 = c->d_pk64; a.pk32 = c->d_pk32; a.pk64_1 = c->d_pk64_1; a.pk32_1 = c->d_pk32_1; a.ctrl = nullptr;
  a.pc = c->pc; a.cc = c->cc; a.F = c->d_F; a.tl = c->d_tl;
  a.emol = c->d_emol; a.wmol = c->d_wmol; a.npair_in = c->d_npin; a.fres = c->d_fres;
  a.ccap = c->ccap; a.overflow = c->d_overflow;
  a.pkq = c->d_pkq; a.pkq_1 = c->d_pkq_1;
  a.jacc = c->d_jacc; a.jacc64 = c->d_jacc64; a.half = 0;
  for (int s = 0; s < MAXSITE; ++s)
    for (int k = 0; k < 3; ++k) a.fbody[s][k] = (float)c->mh.body[s][k];
  a.planar = planar_sites(c->nq, a.fbody) ? 1 : 0;
  double lmax = 0.0;
  for (double l : c->L) lmax = std::max(lmax, l);
  a.band = row_test_band(c->cc.rout + effective_skin(c), lmax);
  for (int k = 0; k < 3; ++k) a.fs1[k] = (float)(c->L[k] / 4294967296.0);   // the values of d_fscale
  return a;
}

static int default_lpi(const g6_ctx* c) {
  // enough lanes per molecule to put ~16 warps on each of the 152 SMs
  const long long want = 152LL * 16 * 32;
  int l = 4;
  while (l < 32 && (long long)c->n * l < want) l *= 2;
  return l;
}

// Molecules per warp of the mixed integrator kernel: 8 spreads a small system's
// FP64 corrector work over more schedulers, 32 issues the fewest FP64
// instructions for a large one.
static int default_mpw(const g6_ctx* c) { return c->n <= 8192 ? 4 : (c->n <= 24576 ? 16 : 32); }

// Default list form of the MD step: the half list in mixed precision (each
// pair evaluated once, the other molecule's share added with float atomics:
// sums in a varying order, so runs are not bit-reproducible), the full list in
// FP64 (bit-reproducible; the FP64 half list is there for g6_set_shape and the
// tuner).
static int default_half(const g6_ctx* c) { return c->prec == G6_MIXED ? 1 : 0; }

// The mixed list kernel keeps each molecule's in-range row in shared memory
// (32/lpi rows per warp): widen lpi until the rows of a block fit.
static int fit_lpi(const g6_ctx* c, int lpi) {
  if (c->prec != G6_MIXED) return lpi;
  while (lpi < 32 && c->ccap > pairs_max_cap(lpi)) lpi *= 2;
  return lpi;
}

// Enqueue the neighbour-list rebuild (conditional on ctrl[0] when ctrl != NULL):
// one cooperative launch that exits at once when no rebuild is due.
static int enqueue_rebuild(g6_ctx* ctx, const int* ctrl, const StepArgs* step = nullptr) {
  if (ctx->coop_grid == 0) ctx->coop_grid = rebuild_grid_limit();
  CellArgs ca = cell_args(ctx, ctx->glist, ctrl);
  CK(launch_rebuild(ca, list_args(ctx, ctrl, step != nullptr && step_uses_half(ctx)), ctx->glist.d_start,
                    ctx->glist.d_cellmol, ctx->coop_grid, step, ctx->stream));
  return G6_OK;
}

static void apply_cached_shape(g6_ctx* ctx);
extern "C" {
static StepArgs step_args(g6_ctx* ctx, double dt, double* log);   // defined with the MD entry points
}

static int force_once(g6_ctx* ctx) {
  int rc = prepare_list(ctx);
  if (rc) return rc;
  apply_cached_shape(ctx);
  if (ctx->lpi == 0) ctx->lpi = default_lpi(ctx);
  CK(cudaMemsetAsync(ctx->d_overflow, 0, sizeof(int), ctx->stream));
  CK(launch_predict_place(place_args(ctx), 0, ctx->d_th, 0, ctx->stream));
  rc = enqueue_rebuild(ctx, nullptr);
  if (rc) return rc;
  ctx->rows_half = false;   // the rebuild wrote full rows
  if (ctx->prec == G6_MIXED && ctx->ccap > pairs_max_cap(32))
    return fail(ctx, G6_ERR_CAPACITY, "neighbour-list rows too long for the shared-memory rows (lower the skin)");
  ctx->lpi = fit_lpi(ctx, ctx->lpi);
  CK(launch_force(force_args(ctx), ctx->model, ctx->prec == G6_MIXED, ctx->lpi, ctx->stream));
  int ovf = 0;
  CK(cudaMemcpyAsync(&ovf, ctx->d_overflow, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (ovf == 2) return fail(ctx, G6_ERR_CUDA, "neighbour-list rebuild was not launched cooperatively");
  if (ovf) return fail(ctx, G6_ERR_CAPACITY, "neighbour-list row overflow");
  return G6_OK;
}

extern "C" {

int g6_version(void) { return 10000; }

const char* g6_last_error(const g6_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

const char* g6_status_string(int s) {
  switch (s) {
    case G6_OK: return "ok";
    case G6_ERR_ARG: return "bad argument";
    case G6_ERR_CUDA: return "CUDA error";
    case G6_ERR_CAPACITY: return "capacity exceeded";
    case G6_ERR_NONFINITE: return "non-finite value";
    case G6_ERR_STATE: return "call order";
    default: return "unknown status";
  }
}

int g6_model_info(int model, int* nsite, double* body, double* param, double* mass_inertia) {
  ModelHost m;
  if (!make_model(model, m)) return G6_ERR_ARG;
  if (nsite) *nsite = m.nref;
  for (int s = 0; s < m.nref; ++s)
    for (int k = 0; k < 3; ++k) {
      if (body) body[3 * s + k] = m.rbody[s][k];
      if (param) param[3 * s + k] = m.rparam[s][k];
    }
  if (mass_inertia) { mass_inertia[0] = m.mass; mass_inertia[1] = m.I[0]; mass_inertia[2] = m.I[1]; mass_inertia[3] = m.I[2]; }
  return G6_OK;
}

int g6_ctx_create(int device, g6_ctx** out) {
  if (!out) return G6_ERR_ARG;
  *out = nullptr;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) return G6_ERR_CUDA;
  if (device < 0 || device >= ndev) return G6_ERR_ARG;
  g6_ctx* c = new g6_ctx();
  c->device = device;
  if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return G6_ERR_CUDA;
  }
  *out = c;
  return G6_OK;
}

int g6_ctx_destroy(g6_ctx* ctx) {
  if (!ctx) return G6_OK;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  free_all(ctx);
  cudaStreamDestroy(ctx->stream);
  delete ctx;
  return G6_OK;
}

// Bytes of the pinned host block of a context with nrep replicas (its regions: pinned_runs).
// The control block of a run, one device allocation mirrored by two pinned
// copies (up, down) so that a run uploads its inputs in one copy and reads its
// results back in one copy: thermostats, temperature / pressure factors,
// fixed-point scales, control words, counters the upload zeroes (done flag,
// per-axis maxima, overflow flag, per-replica counts), reductions.
struct CtlLayout {
  size_t th, rf, fx, ctrl, done, gmax, ovf, repcnt, up_bytes, red, bytes;
};
static CtlLayout ctl_layout(int R) {
  auto al = [](size_t x) { return (x + 15) & ~(size_t)15; };
  CtlLayout L;
  size_t o = 0;
  L.th = o; o = al(o + (size_t)R * sizeof(ThermoDev));
  L.rf = o; o = al(o + 2 * (size_t)R * sizeof(double));
  L.fx = o; o = al(o + 3 * (size_t)R * sizeof(double));
  L.ctrl = o; o = al(o + 8 * sizeof(int));
  L.done = o; o += 4 * sizeof(unsigned);
  L.gmax = o; o += 4 * sizeof(unsigned);
  L.ovf = o; o += 4 * sizeof(int);
  L.repcnt = o; o = al(o + (size_t)R * sizeof(int));
  L.up_bytes = o;
  L.red = o; o = al(o + (size_t)R * NRED * sizeof(double));
  L.bytes = o;
  return L;
}

static size_t pinned_runs_bytes(int nrep) {
  return 2 * ctl_layout(nrep).bytes + (size_t)nrep * G6_LOG_WIDTH * sizeof(double);
}

int g6_system(g6_ctx* ctx, int model, int path, int precision, int nrep, const int* nmol, const double* box) {
  if (!ctx) return G6_ERR_ARG;
  if (nrep < 1 || !nmol || !box) return fail(ctx, G6_ERR_ARG, "nrep, nmol and box are required");
  if (path != G6_PATH_STD && path != G6_PATH_CUSTOM) return fail(ctx, G6_ERR_ARG, "unknown path");
  if (precision != G6_FP64 && precision != G6_MIXED) return fail(ctx, G6_ERR_ARG, "unknown precision");
  ModelHost mh;
  if (!make_model(model, mh)) return fail(ctx, G6_ERR_ARG, "unknown model");
  if (mh.nsite == 0) return fail(ctx, G6_ERR_ARG, "this model runs only through the site-pair-table entry points");
  CK(cudaSetDevice(ctx->device));
  CK(cudaStreamSynchronize(ctx->stream));
  free_all(ctx);
  ctx->have_system = false; ctx->have_state = false;
  ctx->model = model; ctx->path = path; ctx->prec = precision; ctx->nrep = nrep; ctx->mh = mh; ctx->nq = mh.nq;
  make_pair_const(mh, path, ctx->pc);
  ctx->w64 = pk64_width(model); ctx->npk = pk32_width(model);
  ctx->off.assign(nrep + 1, 0); ctx->L.assign(3 * (size_t)nrep, 0.0);
  for (int r = 0; r < nrep; ++r) {
    if (nmol[r] < 2) return fail(ctx, G6_ERR_ARG, "every replica needs at least 2 molecules");
    ctx->off[r + 1] = ctx->off[r] + nmol[r];
    for (int d = 0; d < 3; ++d) {
      if (!(box[3 * r + d] > 0.0)) return fail(ctx, G6_ERR_ARG, "box edges must be positive");
      ctx->L[3 * r + d] = box[3 * r + d];
    }
  }
  const int n = ctx->n = ctx->off[nrep];
  // every update block may touch at most MAXREP_PER_BLOCK replicas
  for (int b = 0; b * RED_BLOCK < n; ++b) {
    const int i0 = b * RED_BLOCK, i1 = std::min(n, i0 + RED_BLOCK) - 1;
    int r0 = (int)(std::upper_bound(ctx->off.begin(), ctx->off.end(), i0) - ctx->off.begin()) - 1;
    int r1 = (int)(std::upper_bound(ctx->off.begin(), ctx->off.end(), i1) - ctx->off.begin()) - 1;
    if (r1 - r0 + 1 > MAXREP_PER_BLOCK) return fail(ctx, G6_ERR_ARG, "replicas too small for the update blocks");
  }
  std::vector<int> mol_rep(n);
  for (int r = 0; r < nrep; ++r)
    for (int i = ctx->off[r]; i < ctx->off[r + 1]; ++i) mol_rep[i] = r;
  std::vector<double> invL(3 * nrep);
  std::vector<float> fs(3 * nrep);
  for (int k = 0; k < 3 * nrep; ++k) { invL[k] = 1.0 / ctx->L[k]; fs[k] = (float)(ctx->L[k] / 4294967296.0); }
  CK(dalloc(ctx, &ctx->d_off, nrep + 1)); CK(dalloc(ctx, &ctx->d_mol_rep, n)); CK(dalloc(ctx, &ctx->d_L, 3 * nrep));
  CK(dalloc(ctx, &ctx->d_invL, 3 * nrep)); CK(dalloc(ctx, &ctx->d_fscale, 3 * nrep));
  CK(cudaMemcpy(ctx->d_off, ctx->off.data(), (nrep + 1) * sizeof(int), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->d_mol_rep, mol_rep.data(), n * sizeof(int), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->d_L, ctx->L.data(), 3 * nrep * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->d_invL, invL.data(), 3 * nrep * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->d_fscale, fs.data(), 3 * nrep * sizeof(float), cudaMemcpyHostToDevice));
  CK(dalloc(ctx, &ctx->d_st, (size_t)REC * n)); CK(dalloc(ctx, &ctx->d_tmat, 9 * (size_t)n));
  CK(dalloc(ctx, &ctx->d_pk64, (size_t)ctx->w64 * n)); CK(dalloc(ctx, &ctx->d_pk32, (size_t)ctx->npk * n));
  CK(dalloc(ctx, &ctx->d_fix, 3 * (size_t)n));
  CK(dalloc(ctx, &ctx->d_tmat1, 9 * (size_t)n));
  CK(dalloc(ctx, &ctx->d_pk64_1, (size_t)ctx->w64 * n)); CK(dalloc(ctx, &ctx->d_pk32_1, (size_t)ctx->npk * n));
  CK(dalloc(ctx, &ctx->d_fix1, 3 * (size_t)n));
  CK(dalloc(ctx, &ctx->d_pkq, 2 * (size_t)n)); CK(dalloc(ctx, &ctx->d_pkq_1, 2 * (size_t)n));
  CK(dalloc(ctx, &ctx->d_F, 3 * (size_t)n)); CK(dalloc(ctx, &ctx->d_tl, 3 * (size_t)n));
  CK(dalloc(ctx, &ctx->d_emol, n)); CK(dalloc(ctx, &ctx->d_wmol, 9 * (size_t)n)); CK(dalloc(ctx, &ctx->d_npin, n));
  CK(dalloc(ctx, &ctx->d_fres, 4 * (size_t)n));
  CK(dalloc(ctx, &ctx->d_jacc, 2 * (size_t)n));
  CK(dalloc(ctx, &ctx->d_jacc64, 6 * (size_t)n));
  CK(dalloc(ctx, &ctx->d_save, (size_t)REC * n));
  CK(dalloc(ctx, &ctx->d_stage, (size_t)REC * n));
  CK(dalloc(ctx, &ctx->d_nnb, n)); CK(dalloc(ctx, &ctx->d_com_build, 3 * (size_t)n));
  CK(dalloc(ctx, &ctx->d_fix_build, 3 * (size_t)n)); CK(dalloc(ctx, &ctx->d_stf, (size_t)STF_COLS * n));
  ctx->nblk = (int)(((long long)n * 32 + 127) / 128);   // partial-sum slots: blocks of the FP64 fused step kernel at 32 lanes per molecule (the most blocks of any step kernel)
  CK(dalloc(ctx, &ctx->d_part, (size_t)ctx->nblk * MAXREP_PER_BLOCK * NRED));
  {
    const CtlLayout cl = ctl_layout(nrep);
    char* blk = nullptr;
    CK(dalloc(ctx, &blk, cl.bytes));
    ctx->d_ctl = blk;
    ctx->d_th = (ThermoDev*)(blk + cl.th); ctx->d_rfac = (double*)(blk + cl.rf); ctx->d_fixs = (double*)(blk + cl.fx);
    ctx->d_ctrl = (int*)(blk + cl.ctrl); ctx->d_done = (unsigned int*)(blk + cl.done);
    ctx->d_gmax = (unsigned int*)(blk + cl.gmax); ctx->d_overflow = (int*)(blk + cl.ovf);
    ctx->d_repcnt = (int*)(blk + cl.repcnt); ctx->d_red = (double*)(blk + cl.red);
  }
  CK(dalloc(ctx, &ctx->d_scale, nrep)); CK(dalloc(ctx, &ctx->d_beta, nrep));
  CK(dalloc(ctx, &ctx->d_acc, nrep)); CK(dalloc(ctx, &ctx->d_epot_rep, nrep));
  CK(dalloc(ctx, &ctx->d_xtemp, nrep)); CK(dalloc(ctx, &ctx->d_slot, nrep)); CK(dalloc(ctx, &ctx->d_moved, nrep));
  CK(dalloc(ctx, &ctx->d_pcnt, 2 * (size_t)n + 2));
  CK(dalloc(ctx, &ctx->d_sig_t, nrep)); CK(dalloc(ctx, &ctx->d_sig_r, nrep)); CK(dalloc(ctx, &ctx->d_energy, nrep));
  CK(dalloc(ctx, &ctx->d_counts, 2 * (size_t)nrep));
  CK(dalloc(ctx, &ctx->d_mlp, MLP_NPARAM)); CK(dalloc(ctx, &ctx->d_fcache, (size_t)n * MLP_IN));
  CK(dalloc(ctx, &ctx->d_mcflag, 1)); CK(dalloc(ctx, &ctx->d_udir, (size_t)n * 12));
  ctx->last_epot.assign(nrep, 0.0);
  ctx->pinned_bytes = pinned_runs_bytes(nrep);
  CK(cudaMallocHost((void**)&ctx->h_pinned, ctx->pinned_bytes));
  std::memset(ctx->h_pinned, 0, ctx->pinned_bytes);   // the up block's counters stay zero
  CK(cudaHostGetDevicePointer((void**)&ctx->d_pinned, ctx->h_pinned, 0));
  CK(cudaEventCreateWithFlags(&ctx->pin_ev, cudaEventDisableTiming));
  CK(cudaEventRecord(ctx->pin_ev, ctx->stream));
  ctx->have_system = true;
  return G6_OK;
}

int g6_set_cutoff(g6_ctx* ctx, double r_in, double r_out) {
  if (!ctx) return G6_ERR_ARG;
  if (!(r_out > 0.0) || !(r_in >= 0.0) || !(r_in < r_out))
    return fail(ctx, G6_ERR_ARG, "need 0 <= r_in < r_out");
  make_cut_const(r_in, r_out, ctx->cc);
  ctx->have_cut = true;
  ctx->gref.valid = false; ctx->glist.valid = false; ctx->cap = 0;
  drop_graphs(ctx);
  return G6_OK;
}

int g6_set_grid(g6_ctx* ctx, double edge) {
  if (!ctx) return G6_ERR_ARG;
  if (edge < 0.0) return fail(ctx, G6_ERR_ARG, "cell edge must be >= 0");
  ctx->req = edge;
  ctx->gref.valid = false;
  return G6_OK;
}

int g6_set_skin(g6_ctx* ctx, double skin) {
  if (!ctx) return G6_ERR_ARG;
  if (!(skin >= 0.0)) return fail(ctx, G6_ERR_ARG, "skin must be >= 0");
  ctx->skin = skin;
  ctx->glist.valid = false; ctx->cap = 0;
  drop_graphs(ctx);
  return G6_OK;
}

int g6_set_box(g6_ctx* ctx, int replica, const double* L3) {
  if (!ctx || !ctx->have_system) return fail(ctx, G6_ERR_STATE, "no system");
  if (replica < 0 || replica >= ctx->nrep || !L3) return fail(ctx, G6_ERR_ARG, "bad replica or box");
  for (int d = 0; d < 3; ++d) {
    if (!(L3[d] > 0.0)) return fail(ctx, G6_ERR_ARG, "box edges must be positive");
    ctx->L[3 * replica + d] = L3[d];
  }
  CK(cudaSetDevice(ctx->device));
  std::vector<double> invL(3 * ctx->nrep);
  std::vector<float> fs(3 * ctx->nrep);
  for (int k = 0; k < 3 * ctx->nrep; ++k) { invL[k] = 1.0 / ctx->L[k]; fs[k] = (float)(ctx->L[k] / 4294967296.0); }
  CK(cudaMemcpy(ctx->d_L, ctx->L.data(), 3 * ctx->nrep * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->d_invL, invL.data(), 3 * ctx->nrep * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->d_fscale, fs.data(), 3 * ctx->nrep * sizeof(float), cudaMemcpyHostToDevice));
  ctx->gref.valid = false; ctx->glist.valid = false; ctx->cap = 0;
  drop_graphs(ctx);
  return G6_OK;
}

int g6_upload_state(g6_ctx* ctx, const double* rec) {
  if (!ctx || !ctx->have_system) return fail(ctx, G6_ERR_STATE, "no system");
  if (!rec) return fail(ctx, G6_ERR_ARG, "rec is NULL");
  CK(cudaSetDevice(ctx->device));
  const int n = ctx->n;
  CK(cudaMemcpyAsync(ctx->d_stage, rec, (size_t)REC * n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  CK(launch_rec_transpose(ctx->d_stage, ctx->d_st, n, 1, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->have_state = true;
  return G6_OK;
}

int g6_download_state(g6_ctx* ctx, double* rec) {
  if (!ctx || !ctx->have_system) return fail(ctx, G6_ERR_STATE, "no system");
  if (!rec) return fail(ctx, G6_ERR_ARG, "rec is NULL");
  CK(cudaSetDevice(ctx->device));
  const int n = ctx->n;
  CK(launch_rec_transpose(ctx->d_stage, ctx->d_st, n, 0, ctx->stream));
  CK(cudaMemcpyAsync(rec, ctx->d_stage, (size_t)REC * n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return G6_OK;
}

int g6_upload_poses(g6_ctx* ctx, const double* com, const double* quat) {
  if (!ctx || !ctx->have_system) return fail(ctx, G6_ERR_STATE, "no system");
  if (!com || !quat) return fail(ctx, G6_ERR_ARG, "com and quat are required");
  CK(cudaSetDevice(ctx->device));
  const int n = ctx->n;
  std::vector<double> soa(7 * (size_t)n);
  for (int i = 0; i < n; ++i) {
    for (int k = 0; k < 3; ++k) soa[(size_t)k * n + i] = com[3 * i + k];
    for (int k = 0; k < 4; ++k) soa[(size_t)(3 + k) * n + i] = quat[4 * i + k];
  }
  CK(cudaMemcpy(ctx->d_st, soa.data(), 3 * (size_t)n * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->d_st + 33 * (size_t)n, soa.data() + 3 * (size_t)n, 4 * (size_t)n * sizeof(double),
                cudaMemcpyHostToDevice));
  ctx->have_state = true;
  return G6_OK;
}

int g6_cells(g6_ctx* ctx, int* cell) {
  int rc = check_ready(ctx, true);
  if (rc) return rc;
  if (!cell) return fail(ctx, G6_ERR_ARG, "cell is NULL");
  rc = prepare_ref_grid(ctx);
  if (rc) return rc;
  CellArgs ca = cell_args(ctx, ctx->gref, nullptr);
  CK(launch_cells(ca, ctx->gref.d_start, ctx->gref.d_cellmol, ctx->stream));
  CK(cudaMemcpyAsync(cell, ctx->gref.d_cell, ctx->n * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return G6_OK;
}

int g6_pairsearch(g6_ctx* ctx, int64_t* npair) {
  int rc = check_ready(ctx, true);
  if (rc) return rc;
  rc = prepare_ref_grid(ctx);
  if (rc) return rc;
  CellArgs ca = cell_args(ctx, ctx->gref, nullptr);
  CK(launch_cells(ca, ctx->gref.d_start, ctx->gref.d_cellmol, ctx->stream));
  PairSetArgs pa;
  std::memset(&pa, 0, sizeof pa);
  pa.n = ctx->n; pa.rep = rep_dev(ctx); pa.g = grid_dev(ctx->gref); pa.cell = ctx->gref.d_cell;
  pa.start = ctx->gref.d_start; pa.cellmol = ctx->gref.d_cellmol; pa.sten = ctx->d_sten; pa.sten_off = ctx->d_sten_off;
  pa.com = ctx->d_st; pa.rout2 = ctx->cc.rout2; pa.rin2 = ctx->cc.rin2; pa.rin = ctx->cc.rin; pa.rout = ctx->cc.rout;
  pa.c1 = ctx->cc.c1; pa.c2 = ctx->cc.c2; pa.cnt = ctx->d_pcnt; pa.off = ctx->d_pcnt + ctx->n + 1;
  CK(launch_pairset_count(pa, ctx->stream));
  long long total = 0;
  CK(cudaMemcpyAsync(&total, ctx->d_pcnt + 2 * (size_t)ctx->n + 1, sizeof(long long), cudaMemcpyDeviceToHost,
                     ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if ((size_t)total > ctx->pair_capacity) {
    const size_t cap = (size_t)(total * 1.25) + 1024;
    CK(dalloc(ctx, &ctx->d_pi, cap)); CK(dalloc(ctx, &ctx->d_pj, cap));
    CK(dalloc(ctx, &ctx->d_ox, cap)); CK(dalloc(ctx, &ctx->d_oy, cap)); CK(dalloc(ctx, &ctx->d_oz, cap));
    CK(dalloc(ctx, &ctx->d_hh, cap)); CK(dalloc(ctx, &ctx->d_dh, cap));
    ctx->pair_capacity = cap;
  }
  pa.pi = ctx->d_pi; pa.pj = ctx->d_pj; pa.ox = ctx->d_ox; pa.oy = ctx->d_oy; pa.oz = ctx->d_oz;
  pa.hh = ctx->d_hh; pa.dh = ctx->d_dh;
  CK(launch_pairset_write(pa, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->npairs = total;
  if (npair) *npair = total;
  return G6_OK;
}

int g6_get_pairs(g6_ctx* ctx, int64_t cap, int* pi, int* pj, double* ox, double* oy, double* oz, double* hh,
                 double* dh) {
  if (!ctx) return G6_ERR_ARG;
  if (ctx->npairs < 0) return fail(ctx, G6_ERR_STATE, "no pair set (g6_pairsearch)");
  CK(cudaSetDevice(ctx->device));
  const size_t m = (size_t)std::min<long long>(cap, ctx->npairs);
  if (m == 0) return G6_OK;
  if (pi) CK(cudaMemcpy(pi, ctx->d_pi, m * sizeof(int), cudaMemcpyDeviceToHost));
  if (pj) CK(cudaMemcpy(pj, ctx->d_pj, m * sizeof(int), cudaMemcpyDeviceToHost));
  if (ox) CK(cudaMemcpy(ox, ctx->d_ox, m * sizeof(double), cudaMemcpyDeviceToHost));
  if (oy) CK(cudaMemcpy(oy, ctx->d_oy, m * sizeof(double), cudaMemcpyDeviceToHost));
  if (oz) CK(cudaMemcpy(oz, ctx->d_oz, m * sizeof(double), cudaMemcpyDeviceToHost));
  if (hh) CK(cudaMemcpy(hh, ctx->d_hh, m * sizeof(double), cudaMemcpyDeviceToHost));
  if (dh) CK(cudaMemcpy(dh, ctx->d_dh, m * sizeof(double), cudaMemcpyDeviceToHost));
  return G6_OK;
}

// Per-molecule F and lab torque (d_F, d_tl), rotation (d_tmat), energies
// (d_emol) and virials (d_wmol, when vir is wanted) to the caller's arrays:
// F (n,3), body torque (n,3), epot and vir per replica.
static int copy_forces(g6_ctx* ctx, double* F, double* tau, double* epot, double* vir) {
  const int n = ctx->n;
  std::vector<double> hF(3 * (size_t)n), hT(3 * (size_t)n), hM(9 * (size_t)n), hE(n), hW(9 * (size_t)n);
  CK(cudaMemcpy(hF.data(), ctx->d_F, hF.size() * sizeof(double), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(hT.data(), ctx->d_tl, hT.size() * sizeof(double), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(hM.data(), ctx->d_tmat, hM.size() * sizeof(double), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(hE.data(), ctx->d_emol, hE.size() * sizeof(double), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(hW.data(), ctx->d_wmol, hW.size() * sizeof(double), cudaMemcpyDeviceToHost));
  for (int i = 0; i < n; ++i) {
    if (F)
      for (int k = 0; k < 3; ++k) F[3 * i + k] = hF[(size_t)k * n + i];
    if (tau) {
      double t[9], l[3] = {hT[i], hT[(size_t)n + i], hT[2 * (size_t)n + i]};
      for (int k = 0; k < 9; ++k) t[k] = hM[(size_t)k * n + i];
      // rigid_collectforce RigidModule.F90:305-310: tau_body = T^T tau_lab
      tau[3 * i] = t[0] * l[0] + t[3] * l[1] + t[6] * l[2];
      tau[3 * i + 1] = t[1] * l[0] + t[4] * l[1] + t[7] * l[2];
      tau[3 * i + 2] = t[2] * l[0] + t[5] * l[1] + t[8] * l[2];
    }
  }
  for (int r = 0; r < ctx->nrep; ++r) {
    double e = 0.0, w[9] = {0};
    for (int i = ctx->off[r]; i < ctx->off[r + 1]; ++i) {
      e += hE[i];
      for (int k = 0; k < 9; ++k) w[k] += hW[(size_t)k * n + i];
    }
    if (epot) epot[r] = e;
    if (vir)
      for (int k = 0; k < 9; ++k) vir[9 * r + k] = w[k];
  }
  return G6_OK;
}

int g6_force(g6_ctx* ctx, double* F, double* tau, double* epot, double* vir) {
  int rc = check_ready(ctx, true);
  if (rc) return rc;
  rc = force_once(ctx);
  if (rc) return rc;
  return copy_forces(ctx, F, tau, epot, vir);
}

int g6_step_forces(g6_ctx* ctx, double* F, double* tau, double* epot) {
  int rc = check_ready(ctx, true);
  if (rc) return rc;
  if (ctx->prec != G6_MIXED)
    return fail(ctx, G6_ERR_STATE, "g6_step_forces: mixed precision only (the FP64 step fuses force and corrector)");
  if (ctx->in_run) return fail(ctx, G6_ERR_STATE, "g6_step_forces inside g6_md_begin/g6_md_end");
  if ((rc = prepare_list(ctx))) return rc;
  apply_cached_shape(ctx);
  if (ctx->lpi == 0) ctx->lpi = default_lpi(ctx);
  if (ctx->step_lpi == 0) ctx->step_lpi = default_lpi(ctx);
  if (ctx->step_mpw == 0) ctx->step_mpw = default_mpw(ctx);
  if (ctx->step_half < 0) ctx->step_half = default_half(ctx);
  if (ctx->ccap > pairs_max_cap(32))
    return fail(ctx, G6_ERR_CAPACITY, "neighbour-list rows too long for the shared-memory rows (lower the skin)");
  ctx->step_lpi = fit_lpi(ctx, ctx->step_lpi);
  const bool half = step_uses_half(ctx);
  CK(cudaMemsetAsync(ctx->d_overflow, 0, sizeof(int), ctx->stream));
  // step 0 (pose buffer 0) with no finished step for the pair kernel's first blocks to finish
  CK(cudaMemsetAsync(ctx->d_ctrl, 0, 8 * sizeof(int), ctx->stream));
  CK(launch_predict_place(place_args(ctx), 0, ctx->d_th, 0, ctx->stream));
  if (ctx->coop_grid == 0) ctx->coop_grid = rebuild_grid_limit();
  CellArgs ca = cell_args(ctx, ctx->glist, nullptr);
  CK(launch_rebuild(ca, list_args(ctx, nullptr, half), ctx->glist.d_start, ctx->glist.d_cellmol, ctx->coop_grid,
                    nullptr, ctx->stream));
  ctx->rows_half = half;
  ForceArgs fa = force_args(ctx);
  fa.ctrl = ctx->d_ctrl;
  fa.half = half ? 1 : 0;
  const StepArgs sa = step_args(ctx, 1.0, nullptr);
  CK(launch_step_pair_forces(fa, sa, ctx->model, ctx->step_lpi, ctx->stream));
  int ovf = 0;
  CK(cudaMemcpyAsync(&ovf, ctx->d_overflow, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (ovf == 2) return fail(ctx, G6_ERR_CUDA, "neighbour-list rebuild was not launched cooperatively");
  if (ovf) return fail(ctx, G6_ERR_CAPACITY, "neighbour-list row overflow");
  return copy_forces(ctx, F, tau, epot, nullptr);
}

int g6_molecule_energies(g6_ctx* ctx, double* e) {
  int rc = check_ready(ctx, true);
  if (rc) return rc;
  if (!e) return fail(ctx, G6_ERR_ARG, "e is NULL");
  rc = force_once(ctx);
  if (rc) return rc;
  CK(cudaMemcpy(e, ctx->d_emol, ctx->n * sizeof(double), cudaMemcpyDeviceToHost));
  return G6_OK;
}

static int ensure_scratch(g6_ctx* ctx, size_t bytes) {
  if (bytes <= ctx->scratch_bytes) return G6_OK;
  if (ctx->d_scratch) { cudaFree(ctx->d_scratch); ctx->d_scratch = nullptr; ctx->scratch_bytes = 0; }
  CK(cudaMalloc(&ctx->d_scratch, bytes));
  ctx->scratch_bytes = bytes;
  return G6_OK;
}

// radialdistrib (RDFModule.F90:101-137) on the device pair set of the uploaded
// poses: FP64 site positions, then one shared-memory histogram per block.
int g6_rdf(g6_ctx* ctx, int nbin, double binwidth, double minvalue, int64_t* hist) {
  int rc = check_ready(ctx, true);
  if (rc) return rc;
  if (!hist || nbin <= 0 || !(binwidth > 0.0)) return fail(ctx, G6_ERR_ARG, "hist, nbin > 0 and binwidth > 0 are needed");
  const int ns = ctx->mh.nref;
  const size_t smem = rdf_smem_bytes(ctx->nrep, ns, nbin);
  if (smem > 200 * 1024)
    return fail(ctx, G6_ERR_CAPACITY, "histogram of all replicas exceeds 200 KB of shared memory (nrep x nsite^2 x nbin x 4)");
  int64_t np = 0;
  rc = g6_pairsearch(ctx, &np);
  if (rc) return rc;
  const size_t nh = (size_t)ctx->nrep * ns * ns * nbin;
  const size_t pos_bytes = ((size_t)ctx->n * ns * 3 * sizeof(double) + 255) & ~(size_t)255;
  const size_t off_bytes = ((size_t)ctx->n * 16 * sizeof(float) + 255) & ~(size_t)255;
  const size_t fix_bytes = ((size_t)ctx->n * 4 * sizeof(uint32_t) + 255) & ~(size_t)255;
  rc = ensure_scratch(ctx, pos_bytes + off_bytes + fix_bytes + nh * sizeof(unsigned long long));
  if (rc) return rc;
  double* pos = (double*)ctx->d_scratch;
  float* off = (float*)((char*)ctx->d_scratch + pos_bytes);
  uint32_t* fixc = (uint32_t*)((char*)ctx->d_scratch + pos_bytes + off_bytes);
  unsigned long long* dh = (unsigned long long*)((char*)ctx->d_scratch + pos_bytes + off_bytes + fix_bytes);
  SitePosArgs sp;
  std::memset(&sp, 0, sizeof sp);
  sp.n = ctx->n; sp.nsite = ns; sp.st = ctx->d_st; sp.pos = pos; sp.off = off; sp.fixc = fixc; sp.rep = rep_dev(ctx);
  for (int s = 0; s < ns; ++s)
    for (int k = 0; k < 3; ++k) sp.body[s][k] = ctx->mh.rbody[s][k];
  CK(launch_site_positions(sp, ctx->stream));
  CK(cudaMemsetAsync(dh, 0, nh * sizeof(unsigned long long), ctx->stream));
  RdfArgs ra;
  std::memset(&ra, 0, sizeof ra);
  ra.npair = np; ra.nrep = ctx->nrep; ra.nsite = ns; ra.nbin = nbin; ra.binwidth = binwidth; ra.minvalue = minvalue;
  ra.off_rep = ctx->d_off; ra.pi = ctx->d_pi; ra.pj = ctx->d_pj; ra.ox = ctx->d_ox; ra.oy = ctx->d_oy; ra.oz = ctx->d_oz;
  ra.pos = pos; ra.off = off; ra.fixc = fixc; ra.fscale = ctx->d_fscale; ra.n = ctx->n; ra.hist = dh;
  ra.fp64_only = ctx->cc.rout > 30.0;   // the FP32 distance bound holds for separations below 32 A
  int nsm = 0;
  CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->device));
  CK(launch_rdf(ra, nsm, ctx->stream));
  std::vector<unsigned long long> h(nh);
  CK(cudaMemcpyAsync(h.data(), dh, nh * sizeof(unsigned long long), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  for (size_t k = 0; k < nh; ++k) hist[k] += (int64_t)h[k];
  return G6_OK;
}

// interaction_hb_by_oh_distance (InteractionModule.F90:682-777) on the device
// pair set: the bonds (donor, its hydrogen 1/2, acceptor), compacted.
int g6_hbonds(g6_ctx* ctx, int64_t cap, int* from, int* which, int* to, int64_t* nbond) {
  int rc = check_ready(ctx, true);
  if (rc) return rc;
  if (cap > 0 && (!from || !which || !to)) return fail(ctx, G6_ERR_ARG, "from, which and to are needed");
  const int ns = ctx->mh.nref;
  // the oxygen and the two hydrogens in the reference's site names (TIP4PConst.F90:22,
  // TIP5PModule.F90:51, ST2Module.F90:26, SPCEModule.F90:18)
  const int osite = 0, h1 = ctx->mh.model == G6_TIP4P ? 2 : 1, h2 = h1 + 1;
  int64_t np = 0;
  rc = g6_pairsearch(ctx, &np);
  if (rc) return rc;
  const int64_t capd = std::max<int64_t>(std::min<int64_t>(cap, np), 0);
  const size_t pos_bytes = ((size_t)ctx->n * ns * 3 * sizeof(double) + 255) & ~(size_t)255;
  const size_t off_bytes = ((size_t)ctx->n * 16 * sizeof(float) + 255) & ~(size_t)255;
  const size_t out_bytes = ((size_t)capd * sizeof(int) + 255) & ~(size_t)255;
  const size_t fix_bytes = ((size_t)ctx->n * 4 * sizeof(uint32_t) + 255) & ~(size_t)255;
  rc = ensure_scratch(ctx, pos_bytes + off_bytes + fix_bytes + 3 * out_bytes + 256);
  if (rc) return rc;
  char* base = (char*)ctx->d_scratch;
  SitePosArgs sp;
  std::memset(&sp, 0, sizeof sp);
  sp.n = ctx->n; sp.nsite = ns; sp.st = ctx->d_st; sp.pos = (double*)base; sp.off = (float*)(base + pos_bytes);
  sp.fixc = (uint32_t*)(base + pos_bytes + off_bytes); sp.rep = rep_dev(ctx);
  for (int s = 0; s < ns; ++s)
    for (int k = 0; k < 3; ++k) sp.body[s][k] = ctx->mh.rbody[s][k];
  CK(launch_site_positions(sp, ctx->stream));
  HbArgs ha;
  std::memset(&ha, 0, sizeof ha);
  ha.npair = np; ha.nsite = ns; ha.osite = osite; ha.hsite[0] = h1; ha.hsite[1] = h2;
  ha.pi = ctx->d_pi; ha.pj = ctx->d_pj; ha.ox = ctx->d_ox; ha.oy = ctx->d_oy; ha.oz = ctx->d_oz; ha.pos = sp.pos;
  char* outp = base + pos_bytes + off_bytes + fix_bytes;
  ha.cap = capd;
  ha.from = (int*)outp; ha.which = (int*)(outp + out_bytes); ha.to = (int*)(outp + 2 * out_bytes);
  ha.count = (unsigned long long*)(outp + 3 * out_bytes);
  CK(cudaMemsetAsync(ha.count, 0, sizeof(unsigned long long), ctx->stream));
  CK(launch_hbonds(ha, ctx->stream));
  unsigned long long total = 0;
  CK(cudaMemcpyAsync(&total, ha.count, sizeof total, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (nbond) *nbond = (int64_t)total;
  const size_t m = (size_t)std::min<int64_t>(capd, (int64_t)total);
  if (m > 0) {
    CK(cudaMemcpyAsync(from, ha.from, m * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(which, ha.which, m * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(to, ha.to, m * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
  }
  return G6_OK;
}

static int pairlist_call(g6_ctx* ctx, int nsites, const double* x, const double* y, const double* z, double* fx,
                         double* fy, double* fz, int64_t npair, const int* pi, const int* pj, const double* ox,
                         const double* oy, const double* oz, const double* er, const double* fr, double* ep,
                         double* vrmat, bool with_force) {
  if (!ctx || !ctx->have_system) return fail(ctx, G6_ERR_STATE, "no system");
  if (nsites < 0 || npair < 0) return fail(ctx, G6_ERR_ARG, "negative size");
  if (nsites % ctx->mh.nref != 0) return fail(ctx, G6_ERR_ARG, "nsites is not a multiple of the model's sites");
  if (!x || !y || !z || (npair > 0 && (!pi || !pj || !ox || !oy || !oz || !er || !ep)))
    return fail(ctx, G6_ERR_ARG, "NULL array");
  if (with_force && (!fx || !fy || !fz || !vrmat || (npair > 0 && !fr))) return fail(ctx, G6_ERR_ARG, "NULL array");
  const int nmol = nsites / ctx->mh.nref;
  for (int64_t k = 0; k < npair; ++k)
    if (pi[k] < 0 || pi[k] >= nmol || pj[k] < 0 || pj[k] >= nmol)
      return fail(ctx, G6_ERR_ARG, "pair index out of range");
  CK(cudaSetDevice(ctx->device));
  const size_t S = (size_t)nsites, P = (size_t)npair;
  const size_t bytes = (with_force ? 6 : 3) * S * 8 + P * (2 * 4 + (with_force ? 6 : 5) * 8 + 8) + 9 * 8 + 64 * 16;
  int rc = ensure_scratch(ctx, bytes);
  if (rc) return rc;
  char* p = (char*)ctx->d_scratch;
  auto take = [&](size_t b) { char* q = p; p += (b + 255) / 256 * 256; return (void*)q; };
  double* dx = (double*)take(S * 8); double* dy = (double*)take(S * 8); double* dz = (double*)take(S * 8);
  double *dfx = nullptr, *dfy = nullptr, *dfz = nullptr;
  if (with_force) { dfx = (double*)take(S * 8); dfy = (double*)take(S * 8); dfz = (double*)take(S * 8); }
  int* dpi = (int*)take(P * 4); int* dpj = (int*)take(P * 4);
  double* dox = (double*)take(P * 8); double* doy = (double*)take(P * 8); double* doz = (double*)take(P * 8);
  double* dhh = (double*)take(P * 8); double* ddh = with_force ? (double*)take(P * 8) : nullptr;
  double* dep = (double*)take(P * 8); double* dvir = (double*)take(9 * 8);
  cudaStream_t s = ctx->stream;
  CK(cudaMemcpyAsync(dx, x, S * 8, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(dy, y, S * 8, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(dz, z, S * 8, cudaMemcpyHostToDevice, s));
  if (with_force) {
    CK(cudaMemcpyAsync(dfx, fx, S * 8, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dfy, fy, S * 8, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dfz, fz, S * 8, cudaMemcpyHostToDevice, s));
  }
  if (P) {
    CK(cudaMemcpyAsync(dpi, pi, P * 4, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dpj, pj, P * 4, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dox, ox, P * 8, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(doy, oy, P * 8, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(doz, oz, P * 8, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dhh, er, P * 8, cudaMemcpyHostToDevice, s));
    if (with_force) CK(cudaMemcpyAsync(ddh, fr, P * 8, cudaMemcpyHostToDevice, s));
  }
  CK(cudaMemsetAsync(dvir, 0, 9 * 8, s));
  SitesArgs a;
  std::memset(&a, 0, sizeof a);
  a.nsite = ctx->mh.nref; a.nq = ctx->nq; a.npair = npair; a.x = dx; a.y = dy; a.z = dz;
  for (int s = 0; s < MAXSITE; ++s) a.site[s] = ctx->mh.site[s];
  a.fx = dfx; a.fy = dfy; a.fz = dfz; a.pi = dpi; a.pj = dpj; a.ox = dox; a.oy = doy; a.oz = doz; a.hh = dhh;
  a.dh = ddh; a.ep = dep; a.vir = dvir; a.pc = ctx->pc; a.with_force = with_force ? 1 : 0;
  CK(launch_force_sites(a, ctx->model, s));
  if (P) CK(cudaMemcpyAsync(ep, dep, P * 8, cudaMemcpyDeviceToHost, s));
  if (with_force) {
    CK(cudaMemcpyAsync(fx, dfx, S * 8, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(fy, dfy, S * 8, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(fz, dfz, S * 8, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(vrmat, dvir, 9 * 8, cudaMemcpyDeviceToHost, s));
  }
  CK(cudaStreamSynchronize(s));
  return G6_OK;
}

int g6_force_sites(g6_ctx* ctx, int nsites, const double* x, const double* y, const double* z, double* fx, double* fy,
                   double* fz, int64_t npair, const int* pair_i, const int* pair_j, const double* ox, const double* oy,
                   const double* oz, const double* eratio, const double* fratio, double* ep, double* vrmat) {
  return pairlist_call(ctx, nsites, x, y, z, fx, fy, fz, npair, pair_i, pair_j, ox, oy, oz, eratio, fratio, ep, vrmat,
                       true);
}

int g6_pair_potential(g6_ctx* ctx, int nsites, const double* x, const double* y, const double* z, int64_t npair,
                      const int* pair_i, const int* pair_j, const double* ox, const double* oy, const double* oz,
                      const double* eratio, double* ep) {
  return pairlist_call(ctx, nsites, x, y, z, nullptr, nullptr, nullptr, npair, pair_i, pair_j, ox, oy, oz, eratio,
                       nullptr, ep, nullptr, false);
}

// ---------------------------------------------------------------------------
// Two components: hetero pair search and the site-pair-table force
// ---------------------------------------------------------------------------
int g6_pairsearch_hetero(g6_ctx* ctx, const double* box, int na, const double* com_a, int nb, const double* com_b,
                         int64_t* npair) {
  if (!ctx) return G6_ERR_ARG;
  if (!ctx->have_cut) return fail(ctx, G6_ERR_STATE, "no cutoff defined (g6_set_cutoff)");
  if (!box || na < 0 || nb < 0 || (na > 0 && !com_a) || (nb > 0 && !com_b)) return fail(ctx, G6_ERR_ARG, "bad arrays");
  for (int d = 0; d < 3; ++d)
    if (!(box[d] > 0.0) || !(ctx->cc.rout <= 0.5 * box[d]))
      return fail(ctx, G6_ERR_ARG, "box edges must be positive and at least twice the cutoff");
  CK(cudaSetDevice(ctx->device));
  const double edge = ctx->req > 0.0 ? ctx->req : ctx->cc.rout;
  const double req[3] = {edge, edge, edge};
  const size_t cbytes = ((size_t)3 * na * 8 + 255) / 256 * 256 + ((size_t)3 * nb * 8 + 255) / 256 * 256;
  const size_t sbytes = pairsearch_hetero_scratch(box, req, na, nb);
  int rc = ensure_scratch(ctx, cbytes + sbytes);
  if (rc) return rc;
  double* dca = (double*)ctx->d_scratch;
  double* dcb = dca + ((size_t)3 * na * 8 + 255) / 256 * 32;
  char* work = (char*)ctx->d_scratch + cbytes;
  if (na) CK(cudaMemcpyAsync(dca, com_a, (size_t)3 * na * 8, cudaMemcpyHostToDevice, ctx->stream));
  if (nb) CK(cudaMemcpyAsync(dcb, com_b, (size_t)3 * nb * 8, cudaMemcpyHostToDevice, ctx->stream));
  HetOutputs out;
  std::memset(&out, 0, sizeof out);
  long long total = 0;
  CK(launch_pairsearch_hetero(box, req, ctx->cc, na, dca, nb, dcb, work, sbytes, &total, ctx->stream, out, false));
  if ((size_t)total > ctx->pair_capacity) {
    const size_t cap = (size_t)(total * 1.25) + 1024;
    CK(dalloc(ctx, &ctx->d_pi, cap)); CK(dalloc(ctx, &ctx->d_pj, cap));
    CK(dalloc(ctx, &ctx->d_ox, cap)); CK(dalloc(ctx, &ctx->d_oy, cap)); CK(dalloc(ctx, &ctx->d_oz, cap));
    CK(dalloc(ctx, &ctx->d_hh, cap)); CK(dalloc(ctx, &ctx->d_dh, cap));
    ctx->pair_capacity = cap;
  }
  out.pi = ctx->d_pi; out.pj = ctx->d_pj; out.ox = ctx->d_ox; out.oy = ctx->d_oy; out.oz = ctx->d_oz;
  out.hh = ctx->d_hh; out.dh = ctx->d_dh;
  CK(launch_pairsearch_hetero(box, req, ctx->cc, na, dca, nb, dcb, work, sbytes, &total, ctx->stream, out, true));
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->npairs = total;
  if (npair) *npair = total;
  return G6_OK;
}

int g6_force_sites_hetero(g6_ctx* ctx, int model_i, int model_j, int path, int nsites, const double* x, const double* y,
                          const double* z, double* fx, double* fy, double* fz, int offset_i, int offset_j,
                          int64_t npair, const int* pair_i, const int* pair_j, const double* ox, const double* oy,
                          const double* oz, const double* eratio, const double* fratio, double* ep, double* vrmat) {
  if (!ctx) return G6_ERR_ARG;
  ModelHost mi, mj;
  if (!make_model(model_i, mi) || !make_model(model_j, mj)) return fail(ctx, G6_ERR_ARG, "unknown model");
  if (path != G6_PATH_STD && path != G6_PATH_CUSTOM) return fail(ctx, G6_ERR_ARG, "unknown path");
  if (nsites < 0 || npair < 0 || offset_i < 0 || offset_j < 0) return fail(ctx, G6_ERR_ARG, "negative size");
  const bool with_force = fx != nullptr;
  if (!x || !y || !z || (npair > 0 && (!pair_i || !pair_j || !ox || !oy || !oz || !eratio || !ep)))
    return fail(ctx, G6_ERR_ARG, "NULL array");
  if (with_force && (!fy || !fz || !vrmat || (npair > 0 && !fratio))) return fail(ctx, G6_ERR_ARG, "NULL array");
  for (int64_t k = 0; k < npair; ++k)
    if (pair_i[k] < 0 || pair_j[k] < 0 || (int64_t)offset_i + ((int64_t)pair_i[k] + 1) * mi.nref > nsites ||
        (int64_t)offset_j + ((int64_t)pair_j[k] + 1) * mj.nref > nsites)
      return fail(ctx, G6_ERR_ARG, "pair index outside the site store");
  TableArgs a;
  std::memset(&a, 0, sizeof a);
  if (!pair_table2(mi, mj, path, a)) return fail(ctx, G6_ERR_ARG, "site-pair table too large");
  CK(cudaSetDevice(ctx->device));
  const size_t S = (size_t)nsites, P = (size_t)npair;
  auto al = [](size_t b) { return (b + 255) / 256 * 256; };
  const size_t bytes = (with_force ? 6 : 3) * al(S * 8) + 2 * al(P * 4) + 6 * al(P * 8) + al(9 * 8);
  int rc = ensure_scratch(ctx, bytes);
  if (rc) return rc;
  char* p = (char*)ctx->d_scratch;
  auto take = [&](size_t b) { char* q = p; p += al(b); return (void*)q; };
  double* dx = (double*)take(S * 8); double* dy = (double*)take(S * 8); double* dz = (double*)take(S * 8);
  double *dfx = nullptr, *dfy = nullptr, *dfz = nullptr;
  if (with_force) { dfx = (double*)take(S * 8); dfy = (double*)take(S * 8); dfz = (double*)take(S * 8); }
  int* dpi = (int*)take(P * 4); int* dpj = (int*)take(P * 4);
  double* dox = (double*)take(P * 8); double* doy = (double*)take(P * 8); double* doz = (double*)take(P * 8);
  double* dhh = (double*)take(P * 8); double* ddh = (double*)take(P * 8); double* dep = (double*)take(P * 8);
  double* dvir = (double*)take(9 * 8);
  cudaStream_t s = ctx->stream;
  CK(cudaMemcpyAsync(dx, x, S * 8, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(dy, y, S * 8, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(dz, z, S * 8, cudaMemcpyHostToDevice, s));
  if (with_force) {
    CK(cudaMemcpyAsync(dfx, fx, S * 8, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dfy, fy, S * 8, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dfz, fz, S * 8, cudaMemcpyHostToDevice, s));
  }
  if (P) {
    CK(cudaMemcpyAsync(dpi, pair_i, P * 4, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dpj, pair_j, P * 4, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dox, ox, P * 8, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(doy, oy, P * 8, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(doz, oz, P * 8, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dhh, eratio, P * 8, cudaMemcpyHostToDevice, s));
    if (with_force) CK(cudaMemcpyAsync(ddh, fratio, P * 8, cudaMemcpyHostToDevice, s));
  }
  CK(cudaMemsetAsync(dvir, 0, 9 * 8, s));
  a.nsi = mi.nref; a.nsj = mj.nref; a.offi = offset_i; a.offj = offset_j; a.npair = npair;
  a.x = dx; a.y = dy; a.z = dz; a.fx = dfx; a.fy = dfy; a.fz = dfz; a.pi = dpi; a.pj = dpj;
  a.ox = dox; a.oy = doy; a.oz = doz; a.hh = dhh; a.dh = ddh; a.ep = dep; a.vir = dvir;
  a.with_force = with_force ? 1 : 0;
  CK(launch_table_force(a, s));
  if (P) CK(cudaMemcpyAsync(ep, dep, P * 8, cudaMemcpyDeviceToHost, s));
  if (with_force) {
    CK(cudaMemcpyAsync(fx, dfx, S * 8, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(fy, dfy, S * 8, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(fz, dfz, S * 8, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(vrmat, dvir, 9 * 8, cudaMemcpyDeviceToHost, s));
  }
  CK(cudaStreamSynchronize(s));
  return G6_OK;
}

// ---------------------------------------------------------------------------
// Molecular dynamics
// ---------------------------------------------------------------------------
static StepArgs step_args(g6_ctx* ctx, double dt, double* log) {
  StepArgs a;
  std::memset(&a, 0, sizeof a);
  a.p = place_args(ctx);
  a.tmat1 = ctx->d_tmat1; a.pk64_1 = ctx->d_pk64_1; a.pk32_1 = ctx->d_pk32_1; a.pkq_1 = ctx->d_pkq_1;
  a.fix1 = ctx->d_fix1;
  a.mass = ctx->mh.mass; a.I[0] = ctx->mh.I[0]; a.I[1] = ctx->mh.I[1]; a.I[2] = ctx->mh.I[2]; a.dt = dt;
  a.com_build = ctx->d_com_build;
  a.fix_build = ctx->d_fix_build;
  a.stf = ctx->d_stf;
  const double hs = 0.5 * effective_skin(ctx);
  a.half_skin2 = hs * hs;
  a.th = ctx->d_th; a.part = ctx->d_part; a.gmax = ctx->d_gmax; a.red = ctx->d_red; a.done = ctx->d_done;
  a.repcnt = ctx->d_repcnt;
  a.inv_dt2 = 1.0 / (dt * dt);
  a.fdt = (float)dt; a.fcf = (float)(dt * dt * 0.5 / ctx->mh.mass); a.fmass = (float)ctx->mh.mass;
  for (int k = 0; k < 3; ++k) a.fI[k] = (float)ctx->mh.I[k];
  a.rfac = ctx->d_rfac; a.fixs = ctx->d_fixs;
  a.ctrl = ctx->d_ctrl; a.log = log; a.seed = ctx->seed;
  return a;
}

// One MD step = the (conditional) neighbour-list rebuild + the fused force /
// integrator kernel.  ev (optional, 4 events) brackets the step and the kernel.
static int enqueue_step(g6_ctx* ctx, const StepArgs& sa, cudaEvent_t* ev = nullptr) {
  // external records become event nodes of a captured graph (queryable after launch)
  // the kernel's own events only in mode 2: event nodes between the kernels add
  // their own latency to the step
  const bool kev = ev && ctx->step_timing == 2;
  if (ev) CK(cudaEventRecordWithFlags(ev[0], ctx->stream, cudaEventRecordExternal));
  int rc = enqueue_rebuild(ctx, ctx->d_ctrl, &sa);
  if (rc) return rc;
  ForceArgs fa = force_args(ctx);
  fa.ctrl = ctx->d_ctrl;
  fa.half = ctx->step_half > 0 ? 1 : 0;
  if (kev) CK(cudaEventRecordWithFlags(ev[1], ctx->stream, cudaEventRecordExternal));
  if (ctx->prec == G6_MIXED) {
    // pair kernel, then the integrator kernel; the kernel events bracket the pair kernel
    CK(launch_step_mixed(fa, sa, ctx->model, ctx->step_lpi, ctx->step_mpw, ctx->stream, kev ? ev[2] : nullptr));
  } else if (fa.half) {
    // pair kernel (partner shares by FP64 atomics), then the integrator kernel
    CK(launch_step_fp64_half(fa, sa, ctx->model, ctx->step_lpi, ctx->stream));
    if (kev) CK(cudaEventRecordWithFlags(ev[2], ctx->stream, cudaEventRecordExternal));
  } else {
    CK(launch_step_fp64(fa, sa, ctx->model, ctx->step_lpi, ctx->stream));
    if (kev) CK(cudaEventRecordWithFlags(ev[2], ctx->stream, cudaEventRecordExternal));
  }
  if (ev) CK(cudaEventRecordWithFlags(ev[3], ctx->stream, cudaEventRecordExternal));
  return G6_OK;
}

static const int GRAPH_STEPS = 16;

// First predict + placement of a run.  Mixed runs first move the small Gear
// terms into the float SoA; md_stop moves them back so that the FP64 state is
// the complete record outside a run.
static int md_start(g6_ctx* ctx, double dt) {
  if (ctx->prec == G6_MIXED) {
    CK(launch_stf_move(ctx->d_st, ctx->d_stf, ctx->n, 1, ctx->stream));
    CK(launch_begin_mixed(place_args(ctx), ctx->d_stf, ctx->d_th, dt, ctx->stream));
  } else {
    CK(launch_predict_place(place_args(ctx), 1, ctx->d_th, 1, ctx->stream));
  }
  return G6_OK;
}

// End of a run: the mixed path finishes its last step's replicas here (every
// other step is finished inside the next step's pair kernel).
static int md_stop(g6_ctx* ctx, const StepArgs& sa) {
  if (ctx->prec == G6_MIXED) {
    CK(launch_finish_step(sa, ctx->nrep, ctx->stream));
    CK(launch_stf_move(ctx->d_st, ctx->d_stf, ctx->n, 0, ctx->stream));
  }
  return G6_OK;
}

// Regions of the pinned host block: uploads (thermostats, control words,
// factors) and read-backs kept apart, since an upload may still be pending
// while a read-back is enqueued.
struct PinnedRuns {
  char* up;       // mirror of the device control block: inputs (and zero counters)
  char* dn;       // mirror of the device control block: results
  ThermoDev* th_up;
  ThermoDev* th_dn;
  double* red;
  double* rf;
  double* fx;
  int* ctrl_up;
  int* ctrl_dn;
  int* ovf;
  double* log1;   // one step's log (g6_md_step_host)
};
// The pinned block's parts at host addresses, or at the device's addresses
// when base is d_pinned.
static PinnedRuns pinned_runs(g6_ctx* ctx, char* base = nullptr) {
  const int R = ctx->nrep;
  char* b = base ? base : ctx->h_pinned;
  const CtlLayout cl = ctl_layout(R);
  PinnedRuns p;
  char* up = b;
  char* dn = b + cl.bytes;
  p.up = up; p.dn = dn;
  p.th_up = (ThermoDev*)(up + cl.th); p.rf = (double*)(up + cl.rf); p.fx = (double*)(up + cl.fx);
  p.ctrl_up = (int*)(up + cl.ctrl);
  p.th_dn = (ThermoDev*)(dn + cl.th); p.ctrl_dn = (int*)(dn + cl.ctrl); p.ovf = (int*)(dn + cl.ovf);
  p.red = (double*)(dn + cl.red);
  p.log1 = (double*)(b + 2 * cl.bytes);
  return p;
}

// Host part of a run's set-up: list buffers, lane widths, the log buffer and
// the thermostat / control / factor words written into the pinned block
// (whose previous uploads must have been read: callers wait on pin_ev or the
// stream first).
static int md_fill(g6_ctx* ctx, double dt, int nsteps, g6_thermostat* thermo, bool want_log) {
  int rc = prepare_list(ctx);
  if (rc) return rc;
  apply_cached_shape(ctx);
  if (ctx->lpi == 0) ctx->lpi = default_lpi(ctx);
  if (ctx->step_lpi == 0) {
    const char* env = std::getenv("G6_LPI");
    ctx->step_lpi = env ? std::atoi(env) : default_lpi(ctx);
    if (ctx->step_lpi != 4 && ctx->step_lpi != 8 && ctx->step_lpi != 16 && ctx->step_lpi != 32)
      ctx->step_lpi = default_lpi(ctx);
  }
  if (ctx->prec == G6_MIXED && ctx->ccap > pairs_max_cap(32))
    return fail(ctx, G6_ERR_CAPACITY, "neighbour-list rows too long for the shared-memory rows (lower the skin)");
  ctx->lpi = fit_lpi(ctx, ctx->lpi);
  ctx->step_lpi = fit_lpi(ctx, ctx->step_lpi);
  if (ctx->step_mpw == 0) ctx->step_mpw = default_mpw(ctx);
  if (ctx->step_half < 0) ctx->step_half = default_half(ctx);
  const PinnedRuns pr = pinned_runs(ctx);
  ThermoDev* th = pr.th_up;
  for (int r = 0; r < ctx->nrep; ++r) {
    ThermoDev& t = th[r];
    std::memset(&t, 0, sizeof t);
    if (thermo) {
      t.kind = thermo[r].kind; t.temp = thermo[r].temp; t.q = thermo[r].q; t.dump = thermo[r].dump;
      for (int k = 0; k < 5; ++k) t.z[k] = thermo[r].zeta[k];
      t.zsum = thermo[r].zetasum; t.rate = thermo[r].collision_rate;
      t.inv_q = t.q > 0.0 ? 1.0 / t.q : 0.0;
      t.fext = (float)(t.z[0] * dt);
      t.fkT = (float)(t.temp * RGAS * J2I);
      t.frdt = (float)(t.rate * dt);
      if (t.kind == G6_NOSE && !(t.q > 0.0)) return fail(ctx, G6_ERR_ARG, "Nose q must be > 0");
      if (t.kind < G6_NVE || t.kind > G6_ANDERSEN) return fail(ctx, G6_ERR_ARG, "unknown thermostat");
    }
  }
  const size_t need_log = want_log ? (size_t)nsteps * ctx->nrep * G6_LOG_WIDTH : 0;
  if (need_log > ctx->log_cap) {
    if (ctx->d_log) { cudaFree(ctx->d_log); ctx->d_log = nullptr; ctx->log_cap = 0; }
    CK(cudaMalloc(&ctx->d_log, need_log * sizeof(double)));
    ctx->log_cap = need_log;
    drop_graphs(ctx);
  }
  // first step: rebuild the list (1), or let the step head test the displacements
  // since the last build (2) when a list for this grid exists
  // (a list of the other row form is rebuilt: a full-list step needs every pair)
  const bool keep = ctx->list_valid && ctx->rows_half == step_uses_half(ctx);
  const int ctrl[8] = {keep ? 2 : 1, 0, nsteps, 0, 0, want_log ? nsteps : 0,
                       (int)(ctx->steps_done & 0x3fffffffULL), 0};
  std::memcpy(pr.ctrl_up, ctrl, sizeof ctrl);
  // temperature and pressure factors of each replica (Mixture.F90:2251-2264)
  for (int r = 0; r < ctx->nrep; ++r) {
    const double dof = 6.0 * (ctx->off[r + 1] - ctx->off[r]);
    const double vol = ctx->L[3 * r] * ctx->L[3 * r + 1] * ctx->L[3 * r + 2];
    pr.rf[2 * r] = I2J * 2.0 / (RGAS * dof);
    pr.rf[2 * r + 1] = I2J / (3.0 * A2P * vol * NA * ANG2M * ANG2M * ANG2M);
  }
  for (int k = 0; k < 3 * ctx->nrep; ++k) pr.fx[k] = (1.0 / ctx->L[k]) * 4294967296.0;
  if (thermo && thermo[0].seed != ctx->seed) {
    ctx->seed = thermo[0].seed;
    drop_graphs(ctx);
  }
  return G6_OK;
}

// Device part of a run's set-up: the uploads from the pinned block and the clears.
static int md_upload(g6_ctx* ctx) {
  const PinnedRuns pr = pinned_runs(ctx);
  // thermostats, factors, scales, control words and the zeroed counters in one copy
  CK(cudaMemcpyAsync(ctx->d_ctl, pr.up, ctl_layout(ctx->nrep).up_bytes, cudaMemcpyHostToDevice, ctx->stream));
  return G6_OK;
}

static int md_prepare(g6_ctx* ctx, double dt, int nsteps, g6_thermostat* thermo, bool want_log, uint64_t seed) {
  // the previous uploads from the pinned block have been read before it is refilled
  CK(cudaEventSynchronize(ctx->pin_ev));
  int rc = md_fill(ctx, dt, nsteps, thermo, want_log);
  if (rc) return rc;
  if ((rc = md_upload(ctx))) return rc;
  CK(cudaEventRecord(ctx->pin_ev, ctx->stream));
  (void)seed;
  return G6_OK;
}

// Read-backs of a run into the pinned block (and the log into `log`, host memory).
static int md_readback(g6_ctx* ctx, int nsteps, double* log) {
  const PinnedRuns pr = pinned_runs(ctx);
  // control words, overflow flag, thermostats and reductions in one copy
  CK(cudaMemcpyAsync(pr.dn, ctx->d_ctl, ctl_layout(ctx->nrep).bytes, cudaMemcpyDeviceToHost, ctx->stream));
  if (log && nsteps > 0)
    CK(cudaMemcpyAsync(log, ctx->d_log, (size_t)nsteps * ctx->nrep * G6_LOG_WIDTH * sizeof(double),
                       cudaMemcpyDeviceToHost, ctx->stream));
  return G6_OK;
}

// After the stream has finished: thermostat state back to the caller, errors.
static int md_check(g6_ctx* ctx, int nsteps, g6_thermostat* thermo) {
  const PinnedRuns pr = pinned_runs(ctx);
  const int* ctrl = pr.ctrl_dn;
  const ThermoDev* th = pr.th_dn;
  const double* red = pr.red;
  // errors first: a failed run leaves the caller's thermostats untouched
  const int ovf = *pr.ovf;
  if (ovf == 2) return fail(ctx, G6_ERR_CUDA, "neighbour-list rebuild was not launched cooperatively");
  if (ovf) return fail(ctx, G6_ERR_CAPACITY, "neighbour-list row overflow");
  if (ctrl[3] & 1) return fail(ctx, G6_ERR_NONFINITE, "non-finite force, torque or position");
  if (ctrl[1] != nsteps) return fail(ctx, G6_ERR_STATE, "step counter mismatch");
  for (int r = 0; r < ctx->nrep; ++r) {
    ctx->last_epot[r] = red[(size_t)r * NRED];
    if (thermo) {
      thermo[r].temp = th[r].temp;
      for (int k = 0; k < 5; ++k) thermo[r].zeta[k] = th[r].z[k];
      thermo[r].zetasum = th[r].zsum;
    }
  }
  ctx->steps_done += (unsigned long long)nsteps;
  ctx->list_valid = true;   // every step leaves the list valid for its positions
  ctx->rows_half = step_uses_half(ctx);   // the first step rebuilt the rows unless they had this form
  return G6_OK;
}

// A neighbour-list row overflowed during a run: the steps after it used
// truncated rows, so the state goes back to the run's start (saved at
// g6_md_begin) and the row capacity is raised by half for the next attempt.
static int recover_overflow(g6_ctx* ctx) {
  CK(cudaMemcpyAsync(ctx->d_st, ctx->d_save, (size_t)REC * ctx->n * sizeof(double), cudaMemcpyDeviceToDevice,
                     ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->cap_request = (ctx->cap * 3 / 2 + 31) / 32 * 32;
  ctx->glist.valid = false; ctx->cap = 0; ctx->list_valid = false;
  ctx->overflow_recovered = true;
  drop_graphs(ctx);
  return fail(ctx, G6_ERR_CAPACITY,
              "neighbour-list row overflow: the state is back at the start of the run and the row capacity was "
              "raised; repeat the run");
}

static int md_finish(g6_ctx* ctx, int nsteps, g6_thermostat* thermo, double* log) {
  int rc = md_readback(ctx, nsteps, log);
  if (rc) return rc;
  CK(cudaStreamSynchronize(ctx->stream));
  return md_check(ctx, nsteps, thermo);
}

static int capture_steps(g6_ctx* ctx, const StepArgs& sa, int k, cudaGraphExec_t* out) {
  cudaGraph_t g;
  CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  for (int q = 0; q < k; ++q) {
    int rc = enqueue_step(ctx, sa, (k == 1 && ctx->step_timing) ? ctx->sev : nullptr);
    if (rc) { cudaStreamEndCapture(ctx->stream, &g); return rc; }
  }
  CK(cudaStreamEndCapture(ctx->stream, &g));
  cudaError_t e = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaGraphInstantiate");
  return G6_OK;
}

// Steps run as graph launches: blocks of GRAPH_STEPS, then single steps.
static int md_enqueue_steps(g6_ctx* ctx, int nsteps) {
  StepArgs sa = step_args(ctx, ctx->run_dt, ctx->run_log ? ctx->d_log : nullptr);
  const int want_log = ctx->run_log ? 1 : 0;
  if (ctx->graph_dt != ctx->run_dt || ctx->graph_log != want_log) drop_graphs(ctx);
  ctx->graph_dt = ctx->run_dt; ctx->graph_log = want_log;
  const int full = ctx->step_timing ? 0 : nsteps / GRAPH_STEPS;
  const int rest = nsteps - full * GRAPH_STEPS;
  int rc;
  if (full > 0 && !ctx->graph) { rc = capture_steps(ctx, sa, GRAPH_STEPS, &ctx->graph); if (rc) return rc; }
  if (rest > 0 && !ctx->graph1) { rc = capture_steps(ctx, sa, 1, &ctx->graph1); if (rc) return rc; }
  for (int k = 0; k < full; ++k) CK(cudaGraphLaunch(ctx->graph, ctx->stream));
  for (int k = 0; k < rest; ++k) CK(cudaGraphLaunch(ctx->graph1, ctx->stream));
  return G6_OK;
}

int g6_md_begin(g6_ctx* ctx, double dt, int max_steps, const g6_thermostat* thermo, int want_log) {
  int rc = check_ready(ctx, true);
  if (rc) return rc;
  if (!(dt > 0.0) || max_steps < 1) return fail(ctx, G6_ERR_ARG, "need dt > 0 and max_steps >= 1");
  rc = md_prepare(ctx, dt, max_steps, const_cast<g6_thermostat*>(thermo), want_log != 0, 0);
  if (rc) return rc;
  ctx->run_dt = dt; ctx->run_log = want_log != 0; ctx->run_max = max_steps; ctx->run_done = 0; ctx->in_run = true;
  CK(cudaMemcpyAsync(ctx->d_save, ctx->d_st, (size_t)REC * ctx->n * sizeof(double), cudaMemcpyDeviceToDevice,
                     ctx->stream));
  return md_start(ctx, dt);
}

int g6_md_advance(g6_ctx* ctx, int nsteps) {
  if (!ctx || !ctx->in_run) return fail(ctx, G6_ERR_STATE, "g6_md_advance outside g6_md_begin/g6_md_end");
  if (nsteps < 0 || ctx->run_done + nsteps > ctx->run_max) return fail(ctx, G6_ERR_ARG, "more steps than max_steps");
  CK(cudaSetDevice(ctx->device));
  int rc = md_enqueue_steps(ctx, nsteps);
  if (rc) return rc;
  ctx->run_done += nsteps;
  return G6_OK;
}

int g6_md_end(g6_ctx* ctx, g6_thermostat* thermo, double* log) {
  if (!ctx || !ctx->in_run) return fail(ctx, G6_ERR_STATE, "g6_md_end without g6_md_begin");
  ctx->in_run = false;
  CK(cudaSetDevice(ctx->device));
  int rc = md_stop(ctx, step_args(ctx, ctx->run_dt, ctx->run_log ? ctx->d_log : nullptr));
  if (rc) return rc;
  rc = md_finish(ctx, ctx->run_done, thermo, ctx->run_log ? log : nullptr);
  if (rc == G6_ERR_CAPACITY && *pinned_runs(ctx).ovf == 1) return recover_overflow(ctx);
  if (rc) return rc;
  // every step but the last predicts the next one; the state is a corrected
  // (reference-consistent) state only after exactly max_steps steps
  if (ctx->run_done != ctx->run_max)
    return fail(ctx, G6_ERR_STATE, "g6_md_end after fewer than max_steps steps: state holds a predicted step");
  return G6_OK;
}

int g6_set_step_timing(g6_ctx* ctx, int on) {
  if (!ctx) return G6_ERR_ARG;
  CK(cudaSetDevice(ctx->device));
  for (int k = 0; k < 4; ++k)
    if (!ctx->sev[k]) CK(cudaEventCreate(&ctx->sev[k]));
  if (on < 0 || on > 2) return fail(ctx, G6_ERR_ARG, "step timing mode is 0, 1 or 2");
  ctx->step_timing = on;
  drop_graphs(ctx);
  return G6_OK;
}

int g6_step_times(g6_ctx* ctx, double* step_ms, double* kernel_ms) {
  if (!ctx || !ctx->step_timing) return fail(ctx, G6_ERR_STATE, "step timing is off (g6_set_step_timing)");
  CK(cudaSetDevice(ctx->device));
  CK(cudaEventSynchronize(ctx->sev[3]));
  float a = 0.0f, b = 0.0f;
  CK(cudaEventElapsedTime(&a, ctx->sev[0], ctx->sev[3]));
  if (ctx->step_timing == 2) CK(cudaEventElapsedTime(&b, ctx->sev[1], ctx->sev[2]));
  if (step_ms) *step_ms = a;
  if (kernel_ms) *kernel_ms = b;
  return G6_OK;
}

int g6_time_force(g6_ctx* ctx, double* ms) {
  if (!ctx || !ms) return G6_ERR_ARG;
  if (!ctx->have_system || ctx->cap == 0 || ctx->lpi == 0) return fail(ctx, G6_ERR_STATE, "no neighbour list yet");
  CK(cudaSetDevice(ctx->device));
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  cudaError_t e = cudaEventRecord(e0, ctx->stream);
  if (e == cudaSuccess) e = launch_force(force_args(ctx), ctx->model, ctx->prec == G6_MIXED, ctx->lpi, ctx->stream);
  if (e == cudaSuccess) e = cudaEventRecord(e1, ctx->stream);
  if (e == cudaSuccess) e = cudaEventSynchronize(e1);
  float t = 0.0f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "g6_time_force");
  *ms = t;
  return G6_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Autotuner.  Shapes of the step kernels that change the speed but not the
// set of pairs: lanes per molecule of the force-only and MD-step pair kernels,
// molecules per warp of the mixed integrator kernel and, on request, the
// Verlet skin (with the row capacity that follows from it).  Each candidate
// is timed with CUDA events on the context's stream, on the uploaded state,
// which is restored after every trial run.  Chosen shapes are cached per
// system size, model, path, precision and cutoff, and a context that has not
// been tuned or given a shape starts from the cached one.
// ---------------------------------------------------------------------------
namespace {
struct ShapeKey {
  int model, path, prec, nrep, n;
  long long rc_milli;
  bool operator<(const ShapeKey& o) const {
    return std::tie(model, path, prec, nrep, n, rc_milli) < std::tie(o.model, o.path, o.prec, o.nrep, o.n, o.rc_milli);
  }
};
std::map<ShapeKey, g6_shape>& shape_cache() {
  static std::map<ShapeKey, g6_shape> m;
  return m;
}
std::mutex& shape_mutex() {
  static std::mutex m;
  return m;
}
ShapeKey shape_key(const g6_ctx* c) {
  return ShapeKey{c->model, c->path, c->prec, c->nrep, c->n, (long long)std::llround(c->cc.rout * 1000.0)};
}
}  // namespace

static void fill_shape(const g6_ctx* ctx, g6_shape* out, double step_ms) {
  out->lpi = ctx->lpi; out->step_lpi = ctx->step_lpi; out->step_mpw = ctx->step_mpw;
  out->skin = ctx->skin; out->cap = ctx->cap; out->step_ms = step_ms;
  out->step_half = ctx->step_half < 0 ? default_half(ctx) : ctx->step_half;
}

// A context without a chosen shape takes the cached one for its size.
static void apply_cached_shape(g6_ctx* ctx) {
  if (ctx->lpi || ctx->step_lpi || ctx->step_mpw) return;
  std::lock_guard<std::mutex> lk(shape_mutex());
  auto it = shape_cache().find(shape_key(ctx));
  if (it == shape_cache().end()) return;
  ctx->lpi = it->second.lpi; ctx->step_lpi = it->second.step_lpi; ctx->step_mpw = it->second.step_mpw;
  ctx->step_half = it->second.step_half;
}

// Duration of `timed` NVE steps (after `warm` untimed ones) from the state
// saved in d_stage, which is put back afterwards.
static int time_md_steps(g6_ctx* ctx, int warm, int timed, cudaEvent_t e0, cudaEvent_t e1, float* ms) {
  const size_t bytes = (size_t)REC * ctx->n * sizeof(double);
  drop_graphs(ctx);
  int rc = g6_md_begin(ctx, 0.001, warm + timed, nullptr, 0);
  if (rc == G6_OK) rc = g6_md_advance(ctx, warm);
  if (rc == G6_OK && cudaEventRecord(e0, ctx->stream) != cudaSuccess) rc = fail(ctx, G6_ERR_CUDA, "event");
  if (rc == G6_OK) rc = g6_md_advance(ctx, timed);
  if (rc == G6_OK && cudaEventRecord(e1, ctx->stream) != cudaSuccess) rc = fail(ctx, G6_ERR_CUDA, "event");
  if (ctx->in_run) { int r2 = g6_md_end(ctx, nullptr, nullptr); if (rc == G6_OK) rc = r2; }
  if (rc == G6_OK && (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(ms, e0, e1) != cudaSuccess))
    rc = fail(ctx, G6_ERR_CUDA, "event timing");
  cudaMemcpyAsync(ctx->d_st, ctx->d_stage, bytes, cudaMemcpyDeviceToDevice, ctx->stream);
  ctx->list_valid = false;
  return rc;
}

// Force-only lanes per molecule: each candidate's kernel, best of 3 launches.
static int tune_force_lpi(g6_ctx* ctx) {
  static const int cand[4] = {4, 8, 16, 32};
  int best = ctx->lpi;
  double tbest = 1e30;
  for (int k = 0; k < 4; ++k) {
    if (fit_lpi(ctx, cand[k]) != cand[k]) continue;   // rows do not fit this width's shared memory
    ctx->lpi = cand[k];
    double t = 1e30, m = 0.0;
    for (int rep = 0; rep < 3; ++rep) {
      int rc = g6_time_force(ctx, &m);
      if (rc) return rc;
      t = std::min(t, m);
    }
    if (t < tbest) { tbest = t; best = cand[k]; }
  }
  ctx->lpi = best;
  return G6_OK;
}

// MD-step kernel shape at the current skin: every (lanes, molecules per warp)
// pair on a short run (FP64: lanes only), with the half and the full list;
// returns the best shape's time for `timed` steps.  A context whose list form
// was set (g6_set_shape) keeps it.
static int tune_step_shape(g6_ctx* ctx, cudaEvent_t e0, cudaEvent_t e1, float* best_ms) {
  static const int lcand[4] = {4, 8, 16, 32};
  static const int mcand[4] = {4, 8, 16, 32};   // 4: the component-parallel integrator
  const int nm = ctx->prec == G6_MIXED ? 4 : 1;
  const bool fixed_half = ctx->half_fixed;
  const int h0 = fixed_half ? ctx->step_half : 0;
  const int h1 = fixed_half ? ctx->step_half : 1;
  int bl = ctx->step_lpi, bm = ctx->step_mpw, bh = h0;
  float sb = 1e30f;
  for (int h = h0; h <= h1; ++h)
    for (int k = 0; k < 4; ++k) {
      if (fit_lpi(ctx, lcand[k]) != lcand[k]) continue;
      for (int q = 0; q < nm; ++q) {
        ctx->step_lpi = lcand[k];
        ctx->step_mpw = ctx->prec == G6_MIXED ? mcand[q] : 8;
        ctx->step_half = h;
        float ms = 0.0f;
        int rc = time_md_steps(ctx, 2, 10, e0, e1, &ms);
        if (rc) return rc;
        if (ms < sb) { sb = ms; bl = ctx->step_lpi; bm = ctx->step_mpw; bh = h; }
      }
    }
  ctx->step_lpi = bl; ctx->step_mpw = bm; ctx->step_half = bh;
  *best_ms = sb / 10.0f;
  return G6_OK;
}

static int tune(g6_ctx* ctx, int flags, g6_shape* out) {
  int rc = check_ready(ctx, true);
  if (rc) return rc;
  if (ctx->in_run) return fail(ctx, G6_ERR_STATE, "tuning inside g6_md_begin/g6_md_end");
  if (ctx->lpi == 0) ctx->lpi = default_lpi(ctx);
  if (ctx->step_lpi == 0) ctx->step_lpi = ctx->lpi;
  if (ctx->step_mpw == 0) ctx->step_mpw = default_mpw(ctx);
  const size_t bytes = (size_t)REC * ctx->n * sizeof(double);
  CK(cudaMemcpyAsync(ctx->d_stage, ctx->d_st, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
  const unsigned long long steps0 = ctx->steps_done;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  float step_ms = 0.0f;
  // skin candidates (A); the requested skin alone without G6_TUNE_SKIN
  std::vector<double> skins;
  const double skin0 = ctx->skin;
  if (flags & G6_TUNE_SKIN) {
    for (double sk : {0.5, 0.75, 1.0, 1.5}) skins.push_back(sk);
  } else {
    skins.push_back(skin0);
  }
  double best_skin = skin0;
  float best_long = 1e30f;
  int bl = 0, bs = 0, bm = 0, bh = 0;
  const int half0 = ctx->step_half;
  for (size_t k = 0; k < skins.size() && rc == G6_OK; ++k) {
    ctx->step_half = half0;
    if (skins.size() > 1) {
      ctx->skin = skins[k]; ctx->glist.valid = false; ctx->cap = 0;
    }
    rc = force_once(ctx);   // list for this skin
    if (rc == G6_OK) rc = tune_force_lpi(ctx);
    float short_ms = 0.0f;
    if (rc == G6_OK) rc = tune_step_shape(ctx, e0, e1, &short_ms);
    float long_ms = short_ms;
    if (rc == G6_OK && skins.size() > 1) {
      // the rebuild frequency depends on the skin: a longer run per candidate
      const int timed = 128;
      float ms = 0.0f;
      rc = time_md_steps(ctx, 2, timed, e0, e1, &ms);
      long_ms = ms / timed;
    }
    if (rc == G6_OK && long_ms < best_long) {
      best_long = long_ms; best_skin = ctx->skin; bl = ctx->lpi; bs = ctx->step_lpi; bm = ctx->step_mpw;
      bh = ctx->step_half;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc == G6_OK) {
    if (skins.size() > 1 && best_skin != ctx->skin) { ctx->skin = best_skin; ctx->glist.valid = false; ctx->cap = 0; }
    ctx->lpi = bl; ctx->step_lpi = bs; ctx->step_mpw = bm; ctx->step_half = bh;
    step_ms = best_long;
  } else {
    ctx->step_half = half0;
  }
  if (rc != G6_OK && skins.size() > 1) {
    ctx->skin = skin0; ctx->glist.valid = false; ctx->cap = 0;
  }
  ctx->steps_done = steps0;
  drop_graphs(ctx);
  CK(cudaMemcpyAsync(ctx->d_st, ctx->d_stage, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->list_valid = false;
  if (rc) return rc;
  rc = prepare_list(ctx);   // capacity of the chosen skin
  if (rc) return rc;
  if (out) fill_shape(ctx, out, step_ms);
  g6_shape sh;
  fill_shape(ctx, &sh, step_ms);
  std::lock_guard<std::mutex> lk(shape_mutex());
  shape_cache()[shape_key(ctx)] = sh;
  return G6_OK;
}

extern "C" {

int g6_tune(g6_ctx* ctx, int* lpi_out) {
  int rc = tune(ctx, 0, nullptr);
  if (rc) return rc;
  if (lpi_out) *lpi_out = ctx->step_lpi;
  return G6_OK;
}

int g6_tune_shape(g6_ctx* ctx, int flags, g6_shape* shape) { return tune(ctx, flags, shape); }

int g6_get_shape(g6_ctx* ctx, g6_shape* shape) {
  if (!ctx || !shape) return G6_ERR_ARG;
  if (!ctx->have_system) return fail(ctx, G6_ERR_STATE, "no system defined (g6_system)");
  fill_shape(ctx, shape, 0.0);
  return G6_OK;
}

int g6_set_shape(g6_ctx* ctx, const g6_shape* shape) {
  if (!ctx || !shape) return G6_ERR_ARG;
  auto ok = [](int l) { return l == 4 || l == 8 || l == 16 || l == 32; };
  if (!ok(shape->lpi) || !ok(shape->step_lpi) || !ok(shape->step_mpw))
    return fail(ctx, G6_ERR_ARG, "lanes per molecule must be 4, 8, 16 or 32 and step_mpw 4, 8, 16 or 32");
  if (!(shape->skin >= 0.0)) return fail(ctx, G6_ERR_ARG, "skin must be >= 0");
  if (shape->cap < 0) return fail(ctx, G6_ERR_ARG, "cap must be >= 0 (0: from the skin and density)");
  if (shape->step_half != 0 && shape->step_half != 1)
    return fail(ctx, G6_ERR_ARG, "step_half must be 0 (full list) or 1 (half list)");
  ctx->lpi = shape->lpi; ctx->step_lpi = shape->step_lpi; ctx->step_mpw = shape->step_mpw;
  ctx->step_half = shape->step_half;
  ctx->half_fixed = true;
  if (shape->skin != ctx->skin || shape->cap != ctx->cap_request) {
    ctx->skin = shape->skin; ctx->cap_request = shape->cap;
    ctx->glist.valid = false; ctx->cap = 0; ctx->list_valid = false;
  }
  drop_graphs(ctx);
  return G6_OK;
}

int g6_set_lpi(g6_ctx* ctx, int lpi) {
  if (!ctx || (lpi != 4 && lpi != 8 && lpi != 16 && lpi != 32)) return G6_ERR_ARG;
  ctx->lpi = lpi;
  ctx->step_lpi = lpi;
  if (ctx->step_mpw == 0) ctx->step_mpw = default_mpw(ctx);
  drop_graphs(ctx);
  return G6_OK;
}

int g6_stream(g6_ctx* ctx, void** stream) {
  if (!ctx || !stream) return G6_ERR_ARG;
  *stream = (void*)ctx->stream;
  return G6_OK;
}

int g6_md_run(g6_ctx* ctx, double dt, int nsteps, g6_thermostat* thermo, double* log) {
  if (nsteps == 0 && ctx) return G6_OK;
  if (!ctx) return G6_ERR_ARG;
  // a row overflow is repeated from the run's start with a larger capacity
  for (int attempt = 0;; ++attempt) {
    int rc = g6_md_begin(ctx, dt, nsteps, thermo, log != nullptr);
    if (rc) return rc;
    rc = g6_md_advance(ctx, nsteps);
    if (rc) {
      ctx->in_run = false;
      md_stop(ctx, step_args(ctx, ctx->run_dt, ctx->run_log ? ctx->d_log : nullptr));
      cudaStreamSynchronize(ctx->stream);
      return rc;
    }
    ctx->overflow_recovered = false;
    rc = g6_md_end(ctx, thermo, log);
    if (rc != G6_ERR_CAPACITY || !ctx->overflow_recovered || attempt == 3) return rc;
  }
}

// Enqueue the whole host-buffer step on the context's stream (used directly,
// or captured once into graph_host).  log_dst: host destination of the log.
// upload = false repeats a step from the state kept in d_save (FP64) or the
// records in d_stage (mixed) -- the row-overflow recovery.  dev_rec (mixed):
// the device address of a page-locked rec, which the records-in and
// records-out kernels then read and write over the host link themselves
// instead of two staged copies.
static int enqueue_step_host(g6_ctx* ctx, double dt, double* rec, double* log_dst, bool want_log, bool upload = true,
                             double* dev_rec = nullptr) {
  const int n = ctx->n;
  const size_t bytes = (size_t)REC * n * sizeof(double);
  if (ctx->prec == G6_MIXED) {
    // records -> state + first predict in one kernel, the step, finish + state
    // -> records in one kernel; the input records stay in d_stage (a copy made
    // by the first kernel when it reads rec directly), the output goes to rec
    // directly or through d_save
    HostInArgs h;
    std::memset(&h, 0, sizeof h);
    h.fix_build = ctx->d_fix_build;
    h.gmax = ctx->d_gmax;
    HostOutArgs o;
    std::memset(&o, 0, sizeof o);
    o.rec = dev_rec ? dev_rec : ctx->d_save;
    // with direct record access the control words move through the pinned
    // block's device address as well: no copy-engine transfer in the step
    const bool direct = upload && dev_rec && ctx->d_pinned;
    const PinnedRuns pd = pinned_runs(ctx, ctx->d_pinned);
    if (upload && dev_rec) {
      h.rec = dev_rec;
      h.keep = ctx->d_stage;
    } else {
      if (upload) CK(cudaMemcpyAsync(ctx->d_stage, rec, bytes, cudaMemcpyHostToDevice, ctx->stream));
      h.rec = ctx->d_stage;
    }
    int rc = G6_OK;
    if (direct) {
      const CtlLayout cl = ctl_layout(ctx->nrep);
      h.ctl_up = (const uint4*)pd.up;
      h.ctl = (uint4*)ctx->d_ctl;
      h.ctl_n16 = (int)(cl.up_bytes / 16);
      h.gmax16 = (int)(cl.gmax / 16);
      o.th_dn = pd.th_dn; o.red_dn = pd.red; o.ctrl_dn = pd.ctrl_dn; o.ovf_dn = pd.ovf; o.ovf = ctx->d_overflow;
    } else if ((rc = md_upload(ctx))) {
      return rc;
    }
    // the direct form writes the log row into the pinned log block (log_dst)
    StepArgs sa = step_args(ctx, dt, want_log ? (direct ? pd.log1 : ctx->d_log) : nullptr);
    CK(launch_host_in_mixed(place_args(ctx), h, ctx->d_stf, ctx->d_th, dt, ctx->stream));
    if ((rc = enqueue_step(ctx, sa))) return rc;
    CK(launch_host_out_mixed(sa, o, ctx->stream));
    if (!dev_rec) CK(cudaMemcpyAsync(rec, ctx->d_save, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    return direct ? G6_OK : md_readback(ctx, 1, want_log ? log_dst : nullptr);
  }
  if (upload) {
    CK(cudaMemcpyAsync(ctx->d_stage, rec, bytes, cudaMemcpyHostToDevice, ctx->stream));
    CK(launch_rec_transpose(ctx->d_stage, ctx->d_st, n, 1, ctx->stream));
    CK(cudaMemcpyAsync(ctx->d_save, ctx->d_st, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
  }
  int rc = md_upload(ctx);
  if (rc) return rc;
  StepArgs sa = step_args(ctx, dt, want_log ? ctx->d_log : nullptr);
  if ((rc = md_start(ctx, dt))) return rc;
  if ((rc = enqueue_step(ctx, sa))) return rc;
  if ((rc = md_stop(ctx, sa))) return rc;
  CK(launch_rec_transpose(ctx->d_stage, ctx->d_st, n, 0, ctx->stream));
  CK(cudaMemcpyAsync(rec, ctx->d_stage, bytes, cudaMemcpyDeviceToHost, ctx->stream));
  return md_readback(ctx, 1, want_log ? log_dst : nullptr);
}

// The end of a host-buffer step, which takes tens of microseconds: the
// stream's status polled for up to 2 ms (a blocking synchronisation returns
// several microseconds after the work ends), then the blocking wait.
static cudaError_t wait_spin(cudaStream_t s) {
  const auto t0 = std::chrono::steady_clock::now();
  for (;;) {
    const cudaError_t e = cudaStreamQuery(s);
    if (e != cudaErrorNotReady) return e;
    if (std::chrono::steady_clock::now() - t0 > std::chrono::milliseconds(2)) return cudaStreamSynchronize(s);
  }
}

int g6_md_step_host(g6_ctx* ctx, double dt, g6_thermostat* thermo, double* rec, double* log) {
  int rc = check_ready(ctx, false);
  if (rc) return rc;
  if (!rec) return fail(ctx, G6_ERR_ARG, "rec is NULL");
  // the pinned block is free: every earlier use ended with a stream synchronisation or pin_ev
  // (both recorded on the context's stream: an idle stream answers for both in one query)
  if (cudaStreamQuery(ctx->stream) != cudaSuccess) {
    cudaGetLastError();   // a busy stream's status is not an error
    CK(cudaEventSynchronize(ctx->pin_ev));
    CK(cudaStreamSynchronize(ctx->stream));
  }
  if ((rc = md_fill(ctx, dt, 1, thermo, log != nullptr))) return rc;
  ctx->have_state = true;
  // a page-locked record: the call runs as one cached graph (launch overhead of
  // the dozen copies and kernels paid once); otherwise the same work is enqueued
  // operation by operation
  cudaPointerAttributes at;
  bool pinned = cudaPointerGetAttributes(&at, rec) == cudaSuccess && at.type == cudaMemoryTypeHost;
  if (!pinned) cudaGetLastError();   // clear the lookup's status for a pageable pointer
  // mixed: page-locked records that the device can address are read and written
  // by the step's kernels directly
  double* dev_rec = (pinned && ctx->prec == G6_MIXED) ? (double*)at.devicePointer : nullptr;
  const PinnedRuns pr = pinned_runs(ctx);
  // mixed: the records-in kernel makes the keep-the-list test (ctrl[0] = 3)
  if (ctx->prec == G6_MIXED && pr.ctrl_up[0] == 2) pr.ctrl_up[0] = 3;
  if (pinned) {
    const bool want_log = log != nullptr;
    if (ctx->graph_host && (ctx->ghost_rec != rec || ctx->ghost_dt != dt || ctx->ghost_log != want_log ||
                            ctx->ghost_lpi != ctx->step_lpi)) {
      cudaGraphExecDestroy(ctx->graph_host);
      ctx->graph_host = nullptr;
    }
    if (!ctx->graph_host) {
      cudaGraph_t g;
      CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
      rc = enqueue_step_host(ctx, dt, rec, pr.log1, want_log, true, dev_rec);
      if (rc) { cudaStreamEndCapture(ctx->stream, &g); return rc; }
      CK(cudaStreamEndCapture(ctx->stream, &g));
      cudaError_t e = cudaGraphInstantiate(&ctx->graph_host, g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) { ctx->graph_host = nullptr; return cuda_fail(ctx, e, "cudaGraphInstantiate"); }
      ctx->ghost_rec = rec; ctx->ghost_dt = dt; ctx->ghost_log = want_log; ctx->ghost_lpi = ctx->step_lpi;
    }
    CK(cudaGraphLaunch(ctx->graph_host, ctx->stream));
    CK(wait_spin(ctx->stream));
  } else {
    if ((rc = enqueue_step_host(ctx, dt, rec, log, log != nullptr))) return rc;
    CK(cudaStreamSynchronize(ctx->stream));
  }
  if (pinned && log) std::memcpy(log, pr.log1, (size_t)ctx->nrep * G6_LOG_WIDTH * sizeof(double));
  rc = md_check(ctx, 1, thermo);
  // a row overflow: the step again from the uploaded state with a larger capacity
  for (int attempt = 0; rc == G6_ERR_CAPACITY && *pr.ovf == 1 && attempt < 3; ++attempt) {
    recover_overflow(ctx);
    if ((rc = md_fill(ctx, dt, 1, thermo, log != nullptr))) return rc;
    if ((rc = enqueue_step_host(ctx, dt, rec, log, log != nullptr, false))) return rc;
    CK(cudaStreamSynchronize(ctx->stream));
    rc = md_check(ctx, 1, thermo);
  }
  return rc;
}

static int replica_exchange(g6_ctx* ctx, int parity, uint64_t seed, uint64_t counter, double* beta,
                            g6_thermostat* thermo, int numb, double* umbrella, const double* op, int* accepted) {
  int rc = check_ready(ctx, true);
  if (rc) return rc;
  if (!beta || !thermo) return fail(ctx, G6_ERR_ARG, "beta and thermo are required");
  if (parity != 0 && parity != 1) return fail(ctx, G6_ERR_ARG, "parity must be 0 or 1");
  if (numb < 0 || (numb > 0 && (!umbrella || !op))) return fail(ctx, G6_ERR_ARG, "umbrella and op are required");
  const int R = ctx->nrep;
  double* d_umb = nullptr;
  double* d_op = nullptr;
  if (numb > 0) {
    rc = ensure_scratch(ctx, (size_t)R * numb * 3 * sizeof(double));
    if (rc) return rc;
    d_umb = (double*)ctx->d_scratch;
    d_op = d_umb + (size_t)R * numb * 2;
    CK(cudaMemcpyAsync(d_umb, umbrella, (size_t)R * numb * 2 * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(d_op, op, (size_t)R * numb * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  }
  std::vector<ThermoDev> th(R);
  for (int r = 0; r < R; ++r) {
    std::memset(&th[r], 0, sizeof(ThermoDev));
    th[r].kind = thermo[r].kind; th[r].temp = thermo[r].temp; th[r].q = thermo[r].q; th[r].dump = thermo[r].dump;
    for (int k = 0; k < 5; ++k) th[r].z[k] = thermo[r].zeta[k];
    th[r].zsum = thermo[r].zetasum; th[r].rate = thermo[r].collision_rate;
  }
  CK(cudaMemcpyAsync(ctx->d_th, th.data(), R * sizeof(ThermoDev), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_beta, beta, R * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_epot_rep, ctx->last_epot.data(), R * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemsetAsync(ctx->d_acc, 0, R * sizeof(int), ctx->stream));
  ExchArgs ea;
  ea.nrep = R; ea.parity = parity; ea.seed = seed; ea.counter = counter; ea.epot = ctx->d_epot_rep; ea.beta = ctx->d_beta;
  ea.th = ctx->d_th; ea.accepted = ctx->d_acc; ea.scale = ctx->d_scale;
  ea.numb = numb; ea.umb = d_umb; ea.op = d_op;
  ea.temp = ctx->d_xtemp; ea.slot = ctx->d_slot; ea.moved = ctx->d_moved;
  CK(launch_exchange(ea, ctx->d_st, ctx->n, ctx->d_mol_rep, ctx->stream));
  if (numb > 0)
    CK(cudaMemcpyAsync(umbrella, d_umb, (size_t)R * numb * 2 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  std::vector<int> acc(R);
  CK(cudaMemcpyAsync(beta, ctx->d_beta, R * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(th.data(), ctx->d_th, R * sizeof(ThermoDev), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(acc.data(), ctx->d_acc, R * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  for (int r = 0; r < R; ++r) {
    thermo[r].temp = th[r].temp;
    for (int k = 0; k < 5; ++k) thermo[r].zeta[k] = th[r].z[k];
    if (accepted) accepted[r] = acc[r];
  }
  return G6_OK;
}

int g6_replica_exchange(g6_ctx* ctx, int parity, uint64_t seed, uint64_t counter, double* beta, g6_thermostat* thermo,
                        int* accepted) {
  return replica_exchange(ctx, parity, seed, counter, beta, thermo, 0, nullptr, nullptr, accepted);
}

int g6_replica_exchange_umbrella(g6_ctx* ctx, int parity, uint64_t seed, uint64_t counter, double* beta,
                                 g6_thermostat* thermo, int numbrella, double* umbrella, const double* op,
                                 int* accepted) {
  return replica_exchange(ctx, parity, seed, counter, beta, thermo, numbrella, umbrella, op, accepted);
}

int g6_exchange_plan(int nrep, int parity, uint64_t seed, uint64_t counter, const double* epot, double* beta,
                     double* temp, int numbrella, double* umbrella, const double* op, double* scale, int* accepted) {
  if (nrep < 1 || !epot || !beta || !temp || !scale) return G6_ERR_ARG;
  if (parity != 0 && parity != 1) return G6_ERR_ARG;
  if (numbrella < 0 || (numbrella > 0 && (!umbrella || !op))) return G6_ERR_ARG;
  for (int r = 0; r < nrep; ++r)
    if (!(temp[r] > 0.0) || !std::isfinite(beta[r]) || !std::isfinite(epot[r])) return G6_ERR_ARG;
  std::vector<int> slot(nrep), moved(nrep);
  ExchangeIO x;
  x.nrep = nrep; x.parity = parity; x.seed = seed; x.counter = counter; x.epot = epot; x.beta = beta; x.temp = temp;
  x.numb = numbrella; x.umb = umbrella; x.op = op; x.slot = slot.data(); x.scale = scale; x.moved = moved.data();
  x.accepted = accepted;
  exchange_run(x);
  return G6_OK;
}

int g6_replica_scale(g6_ctx* ctx, const double* scale) {
  int rc = check_ready(ctx, true);
  if (rc) return rc;
  if (!scale) return fail(ctx, G6_ERR_ARG, "scale is required");
  if (ctx->in_run) return fail(ctx, G6_ERR_STATE, "g6_replica_scale inside g6_md_begin/g6_md_end");
  for (int r = 0; r < ctx->nrep; ++r)
    if (!(scale[r] > 0.0) || !std::isfinite(scale[r])) return fail(ctx, G6_ERR_ARG, "scale factors must be positive");
  CK(cudaMemcpyAsync(ctx->d_scale, scale, ctx->nrep * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  CK(launch_scale_velocity(ctx->d_st, ctx->n, ctx->d_mol_rep, ctx->d_scale, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return G6_OK;
}

int g6_last_epot(g6_ctx* ctx, double* epot) {
  if (!ctx || !epot) return G6_ERR_ARG;
  if (!ctx->have_system) return fail(ctx, G6_ERR_STATE, "no system defined (g6_system)");
  for (int r = 0; r < ctx->nrep; ++r) epot[r] = ctx->last_epot[r];
  return G6_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Monte Carlo and the learned proposal widths
// ---------------------------------------------------------------------------
static int grow(g6_ctx* ctx, void** p, size_t* cap, size_t need_bytes, bool keep) {
  if (need_bytes <= *cap) return G6_OK;
  void* q = nullptr;
  CK(cudaMalloc(&q, need_bytes));
  if (keep && *p && *cap) CK(cudaMemcpy(q, *p, *cap, cudaMemcpyDeviceToDevice));
  if (*p) cudaFree(*p);
  *p = q;
  *cap = need_bytes;
  return G6_OK;
}

static MlpDev mlp_dev(g6_ctx* ctx) {
  MlpDev m;
  m.w = ctx->d_mlp;
  for (int k = 0; k < MLP_IN; ++k) { m.feat_mean[k] = ctx->h_mean[k]; m.feat_inv_std[k] = ctx->h_istd[k]; }
  m.sigma0_t = ctx->sig0_t; m.sigma0_r = ctx->sig0_r;
  return m;
}

extern "C" {

// Start of a Monte Carlo call: the energy of every chain from a full force
// evaluation (which also places the poses), and the inverse temperatures,
// widths and energies on the device; etot gets the energies.
static int mc_begin(g6_ctx* ctx, const double* beta, const double* sigma_t, const double* sigma_r,
                    std::vector<double>& etot) {
  const int R = ctx->nrep;
  int rc = force_once(ctx);
  if (rc) return rc;
  std::vector<double> e(ctx->n);
  etot.assign(R, 0.0);
  CK(cudaMemcpy(e.data(), ctx->d_emol, ctx->n * sizeof(double), cudaMemcpyDeviceToHost));
  for (int r = 0; r < R; ++r)
    for (int i = ctx->off[r]; i < ctx->off[r + 1]; ++i) etot[r] += e[i];
  std::vector<double> st(R, ctx->sig0_t), sr(R, ctx->sig0_r);
  if (sigma_t) st.assign(sigma_t, sigma_t + R);
  if (sigma_r) sr.assign(sigma_r, sigma_r + R);
  if (beta) CK(cudaMemcpy(ctx->d_beta, beta, R * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->d_sig_t, st.data(), R * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->d_sig_r, sr.data(), R * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->d_energy, etot.data(), R * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemset(ctx->d_counts, 0, 2 * R * sizeof(long long)));
  return G6_OK;
}

static McArgs mc_args(g6_ctx* ctx, int ntrial, uint64_t seed, uint64_t counter) {
  McArgs a;
  std::memset(&a, 0, sizeof a);
  a.n = ctx->n; a.ntrial = ntrial;
  a.rep = rep_dev(ctx);
  for (int q = 0; q < MAXSITE; ++q)
    for (int k = 0; k < 3; ++k) { a.body[q][k] = ctx->mh.body[q][k]; a.fbody[q][k] = (float)ctx->mh.body[q][k]; }
  a.st = ctx->d_st; a.pk64 = ctx->d_pk64; a.pk32f = (float*)ctx->d_pk32; a.fix = ctx->d_fix;
  a.pc = ctx->pc; a.cc = ctx->cc; a.beta = ctx->d_beta; a.sigma_t = ctx->d_sig_t; a.sigma_r = ctx->d_sig_r;
  a.energy = ctx->d_energy; a.counts = ctx->d_counts; a.seed = seed; a.counter = counter;
  a.fcache = ctx->d_fcache; a.flag = ctx->d_mcflag; a.udir = ctx->d_udir;
  for (int r = 0; r < ctx->nrep; ++r) a.ncmax = std::max(a.ncmax, ctx->off[r + 1] - ctx->off[r]);
  return a;
}

// Order-parameter state (first use) and its kind, reference histogram and
// umbrellas for one call.
static int op_setup(g6_ctx* ctx, int kind, const double* refhist, int logarithmic, const double* umbrella) {
  if (kind < G6_OP_EP || kind > G6_OP_TRIANGLE) return fail(ctx, G6_ERR_ARG, "unknown order parameter");
  if (kind == G6_OP_TRIANGLE) {
    if (!refhist) return fail(ctx, G6_ERR_ARG, "the triangle order parameter needs a reference histogram");
    double sum = 0.0;
    for (int b = 0; b < OP_NBIN; ++b) {
      if (!(refhist[b] >= 0.0) || !std::isfinite(refhist[b]))
        return fail(ctx, G6_ERR_ARG, "reference histogram entries must be finite and >= 0");
      sum += refhist[b];
    }
    if (!(sum > 0.0)) return fail(ctx, G6_ERR_ARG, "reference histogram is empty");
  }
  const int n = ctx->n, R = ctx->nrep;
  OpDev& o = ctx->opd;
  if (!ctx->have_op) {
    CK(dalloc(ctx, &o.n5c, n)); CK(dalloc(ctx, &o.n5j, (size_t)n * OP_N5)); CK(dalloc(ctx, &o.n5v, (size_t)n * OP_N5));
    CK(dalloc(ctx, &o.bc, n)); CK(dalloc(ctx, &o.bj, (size_t)n * OP_NB));
    CK(dalloc(ctx, &o.bq, (size_t)n * OP_NB * OP_NM)); CK(dalloc(ctx, &o.qs, (size_t)n * OP_NM));
    CK(dalloc(ctx, &o.nb, n)); CK(dalloc(ctx, &o.q6, n));
    CK(dalloc(ctx, &o.hist, (size_t)R * OP_NBIN)); CK(dalloc(ctx, &o.op, R)); CK(dalloc(ctx, &o.flag, 1));
    CK(dalloc(ctx, &ctx->d_umb, 2 * (size_t)R));
    ctx->have_op = true;
  }
  o.kind = kind;
  o.logarithmic = logarithmic ? 1 : 0;
  for (int b = 0; b < OP_NBIN; ++b) o.ref[b] = refhist ? refhist[b] : 0.0;
  o.umb = ctx->d_umb;
  o.opsamp = nullptr;
  if (umbrella) CK(cudaMemcpy(ctx->d_umb, umbrella, 2 * (size_t)R * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemsetAsync(o.flag, 0, sizeof(int), ctx->stream));
  return G6_OK;
}

int g6_mc_run(g6_ctx* ctx, int ntrial, uint64_t seed, uint64_t counter, const double* beta, const double* sigma_t,
              const double* sigma_r, int mode, int sample_every, double* samples, int64_t* counts, double* energy,
              double* trace) {
  int rc = check_ready(ctx, true);
  if (rc) return rc;
  if (ntrial < 0 || !beta || (mode != G6_MC_LEARNED && (!sigma_t || !sigma_r)))
    return fail(ctx, G6_ERR_ARG, "ntrial >= 0, beta and widths are required");
  if (mode < G6_MC_PLAIN || mode > G6_MC_COLLECT) return fail(ctx, G6_ERR_ARG, "unknown Monte Carlo mode");
  if (mode == G6_MC_LEARNED && !ctx->have_mlp) return fail(ctx, G6_ERR_STATE, "no trained network (g6_mlp_set / g6_mlp_train)");
  if (sample_every < 0) return fail(ctx, G6_ERR_ARG, "sample_every must be >= 0");
  const int R = ctx->nrep;
  std::vector<double> etot;
  if ((rc = mc_begin(ctx, beta, sigma_t, sigma_r, etot))) return rc;
  const int nsamples = sample_every > 0 ? ntrial / sample_every : 0;
  if (samples && nsamples > 0)
    if ((rc = grow(ctx, (void**)&ctx->d_samples, &ctx->samples_cap, (size_t)R * nsamples * sizeof(double), false))) return rc;
  if (trace && ntrial > 0)
    if ((rc = grow(ctx, (void**)&ctx->d_trace, &ctx->trace_cap, (size_t)R * ntrial * 4 * sizeof(double), false))) return rc;
  float* rec_out = nullptr;
  if (mode == G6_MC_COLLECT && ntrial > 0) {
    const size_t need = (size_t)(ctx->nrec + (long long)R * ntrial) * MLP_REC * sizeof(float);
    if ((rc = grow(ctx, (void**)&ctx->d_rec, &ctx->rec_cap, need, true))) return rc;
    rec_out = ctx->d_rec + (size_t)ctx->nrec * MLP_REC;
  }
  McArgs a = mc_args(ctx, ntrial, seed, counter);
  a.nsamples = nsamples; a.sample_every = samples ? sample_every : 0;
  a.samples = (samples && nsamples) ? ctx->d_samples : nullptr;
  a.trace = trace ? ctx->d_trace : nullptr; a.records = rec_out;
  a.mlp = mlp_dev(ctx);
  CK(cudaMemsetAsync(ctx->d_mcflag, 0, sizeof(int), ctx->stream));
  if (ntrial > 0) CK(launch_mc(a, ctx->model, ctx->prec == G6_MIXED, mode, ctx->stream));
  std::vector<long long> cnt(2 * R);
  int mcflag = 0;
  CK(cudaMemcpyAsync(&mcflag, ctx->d_mcflag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(etot.data(), ctx->d_energy, R * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(cnt.data(), ctx->d_counts, 2 * R * sizeof(long long), cudaMemcpyDeviceToHost, ctx->stream));
  if (a.samples) CK(cudaMemcpyAsync(samples, ctx->d_samples, (size_t)R * nsamples * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  if (a.trace) CK(cudaMemcpyAsync(trace, ctx->d_trace, (size_t)R * ntrial * 4 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (mode == G6_MC_COLLECT) ctx->nrec += (long long)R * ntrial;
  if (energy) for (int r = 0; r < R; ++r) energy[r] = etot[r];
  if (mcflag) return fail(ctx, G6_ERR_CAPACITY, "more than 64 molecules within 6 A of a Monte Carlo pose");
  if (counts) for (int k = 0; k < 2 * R; ++k) counts[k] = cnt[k];
  drop_graphs(ctx);   // poses changed outside the MD state machine
  return G6_OK;
}

int g6_order_parameter(g6_ctx* ctx, int kind, const double* refhist, int logarithmic, double* op) {
  int rc = check_ready(ctx, true);
  if (rc) return rc;
  if (!op) return fail(ctx, G6_ERR_ARG, "op is required");
  if ((rc = op_setup(ctx, kind, refhist, logarithmic, nullptr))) return rc;
  std::vector<double> etot;
  if ((rc = mc_begin(ctx, nullptr, nullptr, nullptr, etot))) return rc;
  McArgs a = mc_args(ctx, 0, 0, 0);
  CK(launch_op_prepare(a, ctx->opd, ctx->stream));
  int flag = 0;
  CK(cudaMemcpyAsync(op, ctx->opd.op, ctx->nrep * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(&flag, ctx->opd.flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (flag) return fail(ctx, G6_ERR_CAPACITY, "more than 48 molecules within 5 A or more than 10 bonds of a molecule");
  return G6_OK;
}

int g6_mc_run_umbrella(g6_ctx* ctx, int ntrial, uint64_t seed, uint64_t counter, const double* beta,
                       const double* sigma_t, const double* sigma_r, int kind, const double* umbrella,
                       const double* refhist, int logarithmic, double* op, int sample_every, double* samples,
                       double* op_samples, int64_t* counts, double* energy, double* trace) {
  int rc = check_ready(ctx, true);
  if (rc) return rc;
  if (ntrial < 0 || !beta || !sigma_t || !sigma_r || !umbrella)
    return fail(ctx, G6_ERR_ARG, "ntrial >= 0, beta, widths and umbrellas are required");
  if (sample_every < 0) return fail(ctx, G6_ERR_ARG, "sample_every must be >= 0");
  const int R = ctx->nrep;
  for (int r = 0; r < 2 * R; ++r)
    if (!std::isfinite(umbrella[r])) return fail(ctx, G6_ERR_ARG, "umbrella parameters must be finite");
  if ((rc = op_setup(ctx, kind, refhist, logarithmic, umbrella))) return rc;
  std::vector<double> etot;
  if ((rc = mc_begin(ctx, beta, sigma_t, sigma_r, etot))) return rc;
  const int nsamples = sample_every > 0 ? ntrial / sample_every : 0;
  if ((samples || op_samples) && nsamples > 0) {
    if ((rc = grow(ctx, (void**)&ctx->d_samples, &ctx->samples_cap, (size_t)R * nsamples * sizeof(double), false))) return rc;
    if ((rc = grow(ctx, (void**)&ctx->d_opsamp, &ctx->opsamp_cap, (size_t)R * nsamples * sizeof(double), false))) return rc;
  }
  if (trace && ntrial > 0)
    if ((rc = grow(ctx, (void**)&ctx->d_trace, &ctx->trace_cap, (size_t)R * ntrial * 5 * sizeof(double), false))) return rc;
  McArgs a = mc_args(ctx, ntrial, seed, counter);
  const bool sampling = (samples || op_samples) && nsamples > 0;
  a.nsamples = nsamples; a.sample_every = sampling ? sample_every : 0;
  a.samples = sampling ? ctx->d_samples : nullptr;
  a.trace = trace ? ctx->d_trace : nullptr;
  OpDev o = ctx->opd;
  o.opsamp = sampling ? ctx->d_opsamp : nullptr;
  CK(cudaMemsetAsync(ctx->d_mcflag, 0, sizeof(int), ctx->stream));
  CK(launch_op_prepare(a, o, ctx->stream));
  if (ntrial > 0) CK(launch_mc_op(a, o, ctx->model, ctx->prec == G6_MIXED, ctx->stream));
  std::vector<long long> cnt(2 * R);
  int flag = 0;
  CK(cudaMemcpyAsync(&flag, o.flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(etot.data(), ctx->d_energy, R * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(cnt.data(), ctx->d_counts, 2 * R * sizeof(long long), cudaMemcpyDeviceToHost, ctx->stream));
  if (op) CK(cudaMemcpyAsync(op, o.op, R * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  if (sampling && samples)
    CK(cudaMemcpyAsync(samples, ctx->d_samples, (size_t)R * nsamples * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  if (sampling && op_samples)
    CK(cudaMemcpyAsync(op_samples, ctx->d_opsamp, (size_t)R * nsamples * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  if (a.trace) CK(cudaMemcpyAsync(trace, ctx->d_trace, (size_t)R * ntrial * 5 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (energy) for (int r = 0; r < R; ++r) energy[r] = etot[r];
  if (counts) for (int k = 0; k < 2 * R; ++k) counts[k] = cnt[k];
  drop_graphs(ctx);   // poses changed outside the MD state machine
  if (flag)
    return fail(ctx, G6_ERR_CAPACITY,
                "order parameter: more than 48 molecules within 5 A, 10 bonds of a molecule or 64 molecules near a trial");
  return G6_OK;
}

int g6_mlp_set(g6_ctx* ctx, const float* params, const float* feat_mean, const float* feat_inv_std, double sigma0_t,
               double sigma0_r) {
  if (!ctx || !ctx->have_system) return fail(ctx, G6_ERR_STATE, "no system");
  if (!params || !feat_mean || !feat_inv_std || !(sigma0_t > 0.0) || !(sigma0_r > 0.0))
    return fail(ctx, G6_ERR_ARG, "parameters, normalisation and positive widths are required");
  CK(cudaSetDevice(ctx->device));
  CK(cudaMemcpy(ctx->d_mlp, params, MLP_NPARAM * sizeof(float), cudaMemcpyHostToDevice));
  std::memcpy(ctx->h_mean, feat_mean, sizeof ctx->h_mean);
  std::memcpy(ctx->h_istd, feat_inv_std, sizeof ctx->h_istd);
  ctx->sig0_t = sigma0_t; ctx->sig0_r = sigma0_r;
  ctx->have_mlp = true;
  return G6_OK;
}

int g6_mlp_widths(g6_ctx* ctx, const float* features, int64_t n, double* sigma_t, double* sigma_r) {
  if (!ctx || !ctx->have_system || !ctx->have_mlp) return fail(ctx, G6_ERR_STATE, "no system or network");
  if (n < 0 || (n > 0 && (!features || !sigma_t || !sigma_r))) return fail(ctx, G6_ERR_ARG, "bad arguments");
  if (n == 0) return G6_OK;
  CK(cudaSetDevice(ctx->device));
  float *df = nullptr, *dm = nullptr;
  double* dw = nullptr;
  cudaError_t e = cudaMalloc(&df, (size_t)n * MLP_IN * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&dm, 2 * MLP_IN * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&dw, 2 * (size_t)n * sizeof(double));
  if (e == cudaSuccess) e = cudaMemcpy(df, features, (size_t)n * MLP_IN * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dm, ctx->h_mean, MLP_IN * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dm + MLP_IN, ctx->h_istd, MLP_IN * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = launch_mlp_eval(df, n, ctx->d_mlp, dm, dm + MLP_IN, ctx->sig0_t, ctx->sig0_r, dw, dw + n, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpy(sigma_t, dw, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(sigma_r, dw + n, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost);
  cudaFree(df); cudaFree(dm); cudaFree(dw);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "g6_mlp_widths");
  return G6_OK;
}

int g6_mlp_objective(g6_ctx* ctx, double w_move, double w_energy) {
  if (!ctx) return G6_ERR_ARG;
  if (!(w_move >= 0.0) || !(w_energy >= 0.0) || !(w_move + w_energy > 0.0))
    return fail(ctx, G6_ERR_ARG, "objective weights must be >= 0 and not both 0");
  ctx->obj_move = w_move;
  ctx->obj_energy = w_energy;
  return G6_OK;
}

int g6_mlp_get(g6_ctx* ctx, float* params, float* feat_mean, float* feat_inv_std) {
  if (!ctx || !ctx->have_system) return fail(ctx, G6_ERR_STATE, "no system");
  CK(cudaSetDevice(ctx->device));
  if (params) CK(cudaMemcpy(params, ctx->d_mlp, MLP_NPARAM * sizeof(float), cudaMemcpyDeviceToHost));
  if (feat_mean) std::memcpy(feat_mean, ctx->h_mean, sizeof ctx->h_mean);
  if (feat_inv_std) std::memcpy(feat_inv_std, ctx->h_istd, sizeof ctx->h_istd);
  return G6_OK;
}

int g6_mlp_records(g6_ctx* ctx, float* host, int64_t cap, int64_t* count) {
  if (!ctx || !ctx->have_system) return fail(ctx, G6_ERR_STATE, "no system");
  CK(cudaSetDevice(ctx->device));
  const long long m = std::min<long long>(cap, ctx->nrec);
  if (host && m > 0) CK(cudaMemcpy(host, ctx->d_rec, (size_t)m * MLP_REC * sizeof(float), cudaMemcpyDeviceToHost));
  if (count) *count = ctx->nrec;
  if (cap < 0) ctx->nrec = 0;   // cap < 0 discards the collected records
  return G6_OK;
}

}  // extern "C"

struct TrainBuffers {
  float *X = nullptr, *H1 = nullptr, *H2 = nullptr, *Z = nullptr, *G3 = nullptr, *D2 = nullptr, *D1 = nullptr;
  float *grad = nullptr, *m = nullptr, *v = nullptr, *mean = nullptr, *istd = nullptr;
  double* loss = nullptr;
  int* idx = nullptr;
  std::vector<void*> all;
  ~TrainBuffers() { for (void* p : all) cudaFree(p); }
  template <class T> cudaError_t get(T** p, size_t count) {
    cudaError_t e = cudaMalloc((void**)p, std::max<size_t>(count, 1) * sizeof(T));
    if (e == cudaSuccess) { all.push_back(*p); e = cudaMemset(*p, 0, std::max<size_t>(count, 1) * sizeof(T)); }
    return e;
  }
};

static int train_buffers(g6_ctx* ctx, TrainBuffers& b, int batch, long long nidx) {
  const size_t rows = 2 * (size_t)batch;
  CK(b.get(&b.X, rows * MLP_IN)); CK(b.get(&b.H1, rows * MLP_H)); CK(b.get(&b.H2, rows * MLP_H));
  CK(b.get(&b.Z, rows * MLP_OUT)); CK(b.get(&b.G3, rows * MLP_OUT)); CK(b.get(&b.D2, rows * MLP_H));
  CK(b.get(&b.D1, rows * MLP_H)); CK(b.get(&b.grad, MLP_NPARAM)); CK(b.get(&b.m, MLP_NPARAM));
  CK(b.get(&b.v, MLP_NPARAM)); CK(b.get(&b.mean, MLP_IN)); CK(b.get(&b.istd, MLP_IN)); CK(b.get(&b.loss, 1));
  CK(b.get(&b.idx, (size_t)std::max<long long>(nidx, batch)));
  return G6_OK;
}

static TrainArgs train_args(g6_ctx* ctx, TrainBuffers& b, const float* rec, int nb, const int* idx) {
  TrainArgs t;
  t.nrows = 2 * nb; t.rec = rec; t.idx = idx; t.w = ctx->d_mlp; t.mean = b.mean; t.istd = b.istd;
  t.s0t = ctx->sig0_t; t.s0r = ctx->sig0_r; t.w_move = ctx->obj_move; t.w_energy = ctx->obj_energy; t.X = b.X; t.H1 = b.H1; t.H2 = b.H2; t.Z = b.Z; t.G3 = b.G3;
  t.D2 = b.D2; t.D1 = b.D1; t.grad = b.grad; t.loss = b.loss;
  return t;
}

extern "C" {

// Gradient of the training loss over caller records (host), with the current
// parameters and normalisation: mean over records of -J (see g6_train.cu).
int g6_mlp_grad(g6_ctx* ctx, const float* records, int64_t nrec, float* grad, double* loss) {
  if (!ctx || !ctx->have_system || !ctx->have_mlp) return fail(ctx, G6_ERR_STATE, "no system or network");
  if (!records || nrec <= 0 || nrec > (1 << 22)) return fail(ctx, G6_ERR_ARG, "1 <= nrec <= 2^22 records required");
  CK(cudaSetDevice(ctx->device));
  TrainBuffers b;
  int rc = train_buffers(ctx, b, (int)nrec, 0);
  if (rc) return rc;
  float* drec = nullptr;
  CK(b.get(&drec, (size_t)nrec * MLP_REC));
  CK(cudaMemcpy(drec, records, (size_t)nrec * MLP_REC * sizeof(float), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(b.mean, ctx->h_mean, sizeof ctx->h_mean, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(b.istd, ctx->h_istd, sizeof ctx->h_istd, cudaMemcpyHostToDevice));
  CK(launch_mlp_grad(train_args(ctx, b, drec, (int)nrec, nullptr), 1.0f / (float)nrec, ctx->stream));
  double l = 0.0;
  CK(cudaMemcpyAsync(&l, b.loss, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  if (grad) CK(cudaMemcpyAsync(grad, b.grad, MLP_NPARAM * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (loss) *loss = l / (double)nrec;
  return G6_OK;
}

// Adam on the records collected by G6_MC_COLLECT runs: feature normalisation
// from the records, seeded initialisation (constant sigma0 at start), shuffled
// mini-batches.  loss (optional, epochs) receives the mean loss per epoch.
int g6_mlp_train(g6_ctx* ctx, int epochs, int batch, double lr, uint64_t seed, double sigma0_t, double sigma0_r,
                 double* loss) {
  if (!ctx || !ctx->have_system) return fail(ctx, G6_ERR_STATE, "no system");
  if (ctx->nrec < 2) return fail(ctx, G6_ERR_STATE, "no records (run g6_mc_run in G6_MC_COLLECT mode)");
  if (epochs < 0 || batch < 2 || !(lr > 0.0) || !(sigma0_t > 0.0) || !(sigma0_r > 0.0))
    return fail(ctx, G6_ERR_ARG, "bad training arguments");
  CK(cudaSetDevice(ctx->device));
  const long long N = ctx->nrec;
  batch = (int)std::min<long long>(batch, N);
  TrainBuffers b;
  int rc = train_buffers(ctx, b, batch, N);
  if (rc) return rc;
  CK(launch_feat_stats(ctx->d_rec, N, b.mean, b.istd, ctx->stream));
  CK(cudaMemcpyAsync(ctx->h_mean, b.mean, sizeof ctx->h_mean, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(ctx->h_istd, b.istd, sizeof ctx->h_istd, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->sig0_t = sigma0_t; ctx->sig0_r = sigma0_r;
  // initialisation: uniform(-a, a) with a = 1/sqrt(fan_in) from the Philox stream; output layer starts at 0
  std::vector<float> w(MLP_NPARAM, 0.0f);
  for (int p = 0; p < MLP_W3; ++p) {
    const int fan = p < MLP_B1 ? MLP_IN : (p < MLP_W2 ? 1 : (p < MLP_B2 ? MLP_H : 1));
    double u[2];
    uniform2(seed, (uint32_t)p, 0x4d4cu, 0u, 0u, u);
    const bool bias = (p >= MLP_B1 && p < MLP_W2) || (p >= MLP_B2 && p < MLP_W3);
    w[p] = bias ? 0.0f : (float)((2.0 * u[0] - 1.0) / std::sqrt((double)fan));
  }
  {   // output bias: sigma = sigma0 before training
    const double p0 = (1.0 - MLP_SMIN) / MLP_SSPAN;
    w[MLP_B3] = w[MLP_B3 + 1] = (float)std::log(p0 / (1.0 - p0));
  }
  CK(cudaMemcpy(ctx->d_mlp, w.data(), w.size() * sizeof(float), cudaMemcpyHostToDevice));
  ctx->have_mlp = true;
  std::vector<int> perm(N);
  int t = 0;
  for (int ep = 0; ep < epochs; ++ep) {
    for (long long k = 0; k < N; ++k) perm[k] = (int)k;
    for (long long k = N - 1; k > 0; --k) {   // Fisher-Yates from the Philox stream
      double u[2];
      uniform2(seed, (uint32_t)k, (uint32_t)ep, 0x5348u, (uint32_t)(k >> 32), u);
      const long long j = std::min<long long>(k, (long long)(u[0] * (double)(k + 1)));
      std::swap(perm[k], perm[j]);
    }
    CK(cudaMemsetAsync(b.loss, 0, sizeof(double), ctx->stream));
    // the epoch's permutation goes up once; the host vector is refilled only
    // after the copy has completed (the loss read-back below synchronises)
    CK(cudaMemcpyAsync(b.idx, perm.data(), N * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    const long long nb = N / batch;
    for (long long q = 0; q < nb; ++q) {
      CK(launch_mlp_grad(train_args(ctx, b, ctx->d_rec, batch, b.idx + q * batch), 1.0f / (float)batch, ctx->stream));
      CK(launch_adam(ctx->d_mlp, b.grad, b.m, b.v, (float)lr, ++t, ctx->stream));
    }
    double l = 0.0;
    CK(cudaMemcpy(&l, b.loss, sizeof(double), cudaMemcpyDeviceToHost));
    if (loss) loss[ep] = nb > 0 ? l / (double)(nb * batch) : 0.0;
  }
  return G6_OK;
}

}  // extern "C"
