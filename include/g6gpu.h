/*
 * g6gpu.h -- C ABI of the GB300 (sm_103a) rigid-water force/energy library.
 *
 * This is the drop-in boundary for Genesis6's rigid-molecule force path.  Each
 * entry point names the Fortran interface it replaces (file:line in the
 * Genesis6 sources).  Conventions:
 *   - every function returns an int status (G6_OK = 0, G6_ERR_* otherwise);
 *     g6_last_error() gives a one-line message for the last failure;
 *   - host pointers are borrowed for the duration of the call, never retained;
 *   - a context owns all device memory of one system (one or more replicas);
 *     use one context per host thread;
 *   - calls are synchronous at return;
 *   - indices are 0-based (the Fortran shim subtracts 1);
 *   - arrays are row-major: com (n,3), quat (n,4), rec (n,53), F/tau (n,3);
 *     a 3x3 virial is vir[3*a+b] = sum over pairs of d00_a * F_b, which is
 *     the reference's vrmat(a,b).
 *   - units are the reference's: Angstrom, ps, amu, energy in 10 J/mol.
 */
#ifndef G6GPU_H
#define G6GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define G6_OK 0
#define G6_ERR_ARG 1        /* bad argument or unsupported combination          */
#define G6_ERR_CUDA 2       /* CUDA runtime error (message in g6_last_error)    */
#define G6_ERR_CAPACITY 3   /* a fixed-capacity device table overflowed          */
#define G6_ERR_NONFINITE 4  /* NaN/Inf coordinates or forces detected            */
/* 5 is unused: no kernel of this library waits on a flag or a peer */
#define G6_ERR_STATE 6      /* call order violated (e.g. no system defined)      */

/* models: site order is the reference's, the centre of mass is the last site */
#define G6_TIP4P 1 /* O, M, H, H, COM      TIP4PModule.F90:43-97               */
#define G6_TIP5P 2 /* O, H, H, L, L, COM   TIP5PModule.F90:57-83, RigidModule.F90:429-477 */
#define G6_ST2 3   /* O, H, H, M, M, COM   ST2Module.F90:10-100                */
#define G6_SPCE 4  /* O, H, H, COM         SPCEModule.F90:8-71 (StdForce path only) */
#define G6_OPLSMEOH 5 /* Me, O, H, COM   OPLSMeOHModule.F90:40-101, RigidModule.F90:391-426
                         (site-pair-table entry points only: g6_force_sites_hetero) */

/* force path, the reference's `custom` flag (@FAST) of Interaction2.F90:19-68 */
#define G6_PATH_STD 0    /* StdForce / StdPairPotential (LB mixing, no ST2 taper)   */
#define G6_PATH_CUSTOM 1 /* hand kernels: interaction_force_tip4p, force_st2 (taper) */

/* arithmetic of the site-site loop */
#define G6_FP64 0  /* plain form: everything in double                              */
#define G6_MIXED 1 /* site-site math in float, per-molecule and global sums in double */

/* thermostats for g6_md_run */
#define G6_NVE 0
#define G6_NOSE 1     /* Nose-Hoover zeta with Gear-4, NoseModule.F90:43-87           */
#define G6_ANDERSEN 2 /* stochastic-collision thermostat (new; the reference's Andersen is a barostat) */

typedef struct g6_ctx g6_ctx;

/* Per-replica thermostat parameters. */
typedef struct g6_thermostat {
  int kind;              /* G6_NVE, G6_NOSE or G6_ANDERSEN                            */
  double temp;           /* target temperature [K]                                    */
  double q;              /* Nose mass as the reference holds it during a run: the @NOS2
                            value times dt (Mixture.F90:1206); @NOSE values are first
                            scaled by 21.8852721616497249235^2 (NoseModule.F90:101) */
  double dump;           /* Nose damping term (@NOS2 dump)                            */
  double zeta[5];        /* Nose zeta0..zeta4                                          */
  double zetasum;        /* running sum of zeta0 (conserved-quantity term)            */
  double collision_rate; /* Andersen: collisions per molecule per ps                  */
  uint64_t seed;         /* Andersen: random stream (first replica's value is used)   */
} g6_thermostat;

/* Per-step log record written by g6_md_run (doubles, 10 per replica per step). */
#define G6_LOG_WIDTH 10
/* [0] Epot  [1] Ekin translational  [2] Ekin rotational  (internal units)
   [3] T [K]  [4] P [atm]  [5] H [J/mol] (Mixture.F90:2431-2453)
   [6] pairs within rc  [7] zeta0  [8] neighbour-list rebuild flag  [9] step   */

int g6_version(void);
const char* g6_last_error(const g6_ctx* ctx);
const char* g6_status_string(int status);

/* Host-only model tables (no device work): body-frame site coordinates
   (nsite,3), site parameters (nsite,3) = (charge, LJ eps [kJ/mol], LJ sigma [A])
   as sStdInt%param (StdInteraction.F90:34-39), and mass, Ixx, Iyy, Izz. */
int g6_model_info(int model, int* nsite, double* body, double* param, double* mass_inertia);

int g6_ctx_create(int device, g6_ctx** out);
int g6_ctx_destroy(g6_ctx* ctx);

/* Define the system: nrep replicas of one model; replica r holds nmol[r]
   molecules in an orthorhombic box box[3r..3r+2].  Replaces the allocation
   done by Mol_allocate / interaction_initialize (MolModule.F90:63-113,
   InteractionModule.F90:199-223). */
int g6_system(g6_ctx* ctx, int model, int path, int precision, int nrep, const int* nmol, const double* box);

/* cutoff_initialize(in, out), CutoffModule.F90:25-36 (@RCOA rc margin gives in = rc - margin). */
int g6_set_cutoff(g6_ctx* ctx, double r_in, double r_out);
/* Requested cell edge of the adaptive grid (@VOXA, GridModule.F90:488-501); 0 selects r_out. */
int g6_set_grid(g6_ctx* ctx, double cell_edge);
/* Verlet margin of the device neighbour list (>= 0).  The set of interacting
   pairs is unchanged: every pair is re-tested against r_out each step. */
int g6_set_skin(g6_ctx* ctx, double skin);
/* Box of replica r (BoxModule @BOX3); invalidates the neighbour list. */
int g6_set_box(g6_ctx* ctx, int replica, const double* L3);

/* State transfer.  rec is the per-molecule rigid record (53 doubles):
   com[3], d[5][3] (dx(1..5): Gear-5 COM stack, dx(1) = v*dt), w[5][3]
   (angular velocity stack, body frame), q[5][4] (quaternion stack), i.e. the
   content of sRigid1 (RigidModule.F90:14-24).  Poses only: com (n,3), quat (n,4). */
int g6_upload_state(g6_ctx* ctx, const double* rec);
int g6_download_state(g6_ctx* ctx, double* rec);
int g6_upload_poses(g6_ctx* ctx, const double* com, const double* quat);

/* Address_Assign (GridModule.F90:503-552): 0-based cell id of every molecule
   under the reference grid (bit-exact with the reference FP64 arithmetic). */
int g6_cells(g6_ctx* ctx, int* cell);
/* Grid_Update + Address_Assign + Grid_NeighborList + Interaction_Compress2 +
   CutOff_Dimmer2 (GridModule.F90:95, 503, 557; InteractionModule.F90:398;
   CutoffModule.F90:220): build the exact within-cutoff pair set on the device. */
int g6_pairsearch(g6_ctx* ctx, int64_t* npair);
/* Copy the pair set of the last g6_pairsearch: pair_i/pair_j, image offsets
   ox/oy/oz (iv%ox..), eratio (hh) and fratio (dh).  cap bounds every array. */
int g6_get_pairs(g6_ctx* ctx, int64_t cap, int* pi, int* pj, double* ox, double* oy, double* oz, double* hh,
                 double* dh);

/* Full force path on the uploaded poses: rigid_setsiteposition
   (RigidModule.F90:146) -> pair search -> switch -> force (Interaction2.F90:19)
   -> rigid_collectforce (RigidModule.F90:159).  Outputs per-molecule COM force
   F (n,3), body-frame torque tau (n,3), per-replica potential energy
   epot[nrep] and virial vir[nrep*9].  Any output pointer may be NULL. */
int g6_force(g6_ctx* ctx, double* F, double* tau, double* epot, double* vir);

/* No counterpart in the reference: the forces exactly as the mixed MD step's
   pair kernel computes them on the uploaded poses (the context's list form
   and lanes: with the half list each pair is evaluated once and the other
   molecule's share added by float atomics), before its integrator uses them.
   F, tau and epot as in g6_force (no virial).  Mixed precision only; returns
   G6_ERR_STATE for an FP64 context, whose step fuses force and corrector. */
int g6_step_forces(g6_ctx* ctx, double* F, double* tau, double* epot);
/* Per-molecule potential energy e_i = 1/2 sum_j e_ij (n) of the uploaded poses. */
int g6_molecule_energies(g6_ctx* ctx, double* e);
/* Site-site distance histograms of the uploaded poses, radialdistrib
   (RDFModule.F90:101-137): over the within-cutoff pair set (g6_pairsearch),
   for each replica r and each pair of reference sites a <= b (nsite of
   g6_model_info, COM included), the molecule pairs with site a of one molecule
   and site b of the other (either order) at distance r go to bin
   nint((r - minvalue) / binwidth) when 0 <= bin < nbin (Histogram_Accumulate,
   DistribModule.F90:149-158).  Counts are ADDED to hist[((r*nsite + a)*nsite
   + b)*nbin + bin]; entries with a > b stay untouched.  Positions and distances
   are FP64.  G6_ERR_CAPACITY when nrep * nsite^2 * nbin * 4 bytes exceeds
   200 KB. */
int g6_rdf(g6_ctx* ctx, int nbin, double binwidth, double minvalue, int64_t* hist);
/* Hydrogen bonds of the uploaded poses by O-H distance,
   interaction_hb_by_oh_distance (InteractionModule.F90:682-777): for every
   pair of the within-cutoff pair set the shortest of the four intermolecular
   O-H distances (FP64, first strict minimum); below 2.5 A the pair is a bond
   with donor from[b] (the molecule that owns the hydrogen), which[b] (1 or 2)
   its hydrogen and acceptor to[b] (0-based molecules).  Only bonds are
   written, at most cap of them, in no particular order (the reference writes
   one entry per pair, zeros for pairs without a bond); nbond gets the number
   of bonds, which may exceed cap. */
int g6_hbonds(g6_ctx* ctx, int64_t cap, int* from, int* which, int* to, int64_t* nbond);

/* The reference `force(iv,mi,mj,site,ep,vrmat,custom,si,sj)` call,
   Interaction2.F90:19-68, for one homogeneous component: caller-owned site
   arrays (site%x/y/z, molecule m site s at m*nsite+s), the compressed pair
   list with image offsets and switch factors.  Site forces are ACCUMULATED
   into fx/fy/fz (the caller zeroes them, site_resetforce); ep[npair] and
   vrmat[9] are outputs.  Model and path come from g6_system. */
int g6_force_sites(g6_ctx* ctx, int nsites, const double* x, const double* y, const double* z, double* fx, double* fy,
                   double* fz, int64_t npair, const int* pair_i, const int* pair_j, const double* ox, const double* oy,
                   const double* oz, const double* eratio, const double* fratio, double* ep, double* vrmat);
/* The reference `PairPotential(iv,mi,mj,site,ep,custom,si,sj)`, Interaction2.F90:71-121. */
int g6_pair_potential(g6_ctx* ctx, int nsites, const double* x, const double* y, const double* z, int64_t npair,
                      const int* pair_i, const int* pair_j, const double* ox, const double* oy, const double* oz,
                      const double* eratio, double* ep);

/* Two components in one box, the reference's mixture path.
   g6_pairsearch_hetero: Grid_Update + Address_Assign of both components +
   Grid_NeighborList over the hetero stencil (NeighborCell_ListHetero,
   GridModule.F90:757-899: the 27 neighbouring cells, clipped to the grid) +
   Interaction_Compress2 + CutOff_Dimmer2 (InteractionModule.F90:398;
   CutoffModule.F90:220): the exact pair set (i in A, j in B) with the
   reference's FP64 arithmetic, for com_a (na,3) and com_b (nb,3) in the box
   box[3]; cutoff and requested cell edge from g6_set_cutoff / g6_set_grid (no
   g6_system needed).  g6_get_pairs returns the list.
   g6_force_sites_hetero: force(iv, mi, mj, site, ep, vrmat, custom, si, sj),
   Interaction2.F90:19-68, for components of models model_i and model_j on one
   global site store (site arrays of nsites entries; molecule m of component i
   at sites offset_i + m*nsite_i + s, the reference's mi%offset; the COM is the
   last site of each model): the TIP4P-OPLS methanol hand kernel
   (interaction_force_tip4p_oplsmeoh, OPLSMeOHModule.F90:1201-1480) on the
   custom path, StdForce (StdInteraction.F90:63-630) otherwise, FP64.  Site
   forces are ACCUMULATED into fx/fy/fz; ep[npair] and vrmat[9] are outputs.
   fx == NULL gives the energies only (PairPotential, Interaction2.F90:71-121;
   fratio and vrmat may then be NULL). */
int g6_pairsearch_hetero(g6_ctx* ctx, const double* box, int na, const double* com_a, int nb, const double* com_b,
                         int64_t* npair);
int g6_force_sites_hetero(g6_ctx* ctx, int model_i, int model_j, int path, int nsites, const double* x, const double* y,
                          const double* z, double* fx, double* fy, double* fz, int offset_i, int offset_j,
                          int64_t npair, const int* pair_i, const int* pair_j, const double* ox, const double* oy,
                          const double* oz, const double* eratio, const double* fratio, double* ep, double* vrmat);

/* Molecular dynamics on the device-resident state: per step rigid_predict,
   Nose_Predict, site placement, pair search, force, rigid_collectforce,
   rigid_correct, Rigid_Ek, Nose_Correct in the order of Mixture.F90:1789-2290.
   dt in ps.  thermo[nrep] is read at the start and written back at the end.
   log (optional) receives nsteps*nrep*G6_LOG_WIDTH doubles, step-major.
   The steps run as CUDA-graph launches with no host synchronisation inside. */
int g6_md_run(g6_ctx* ctx, double dt, int nsteps, g6_thermostat* thermo, double* log);
/* Row overflow: a neighbour-list row longer than the capacity would leave the
   steps after it on truncated rows.  g6_md_run and g6_md_step_host then put
   the state back to where the run started, raise the capacity by half and
   repeat the run (up to three times); g6_md_end returns G6_ERR_CAPACITY with
   the state put back and the capacity raised, so that the caller repeats the
   run from g6_md_begin with the same thermostats (which a failed run leaves
   untouched). */

/* g6_md_run split into its three phases so that a driver can interleave its
   own stream work: g6_md_begin uploads the thermostats and performs the first
   rigid_predict; g6_md_advance enqueues nsteps steps on the context's stream
   and returns without synchronising (at most max_steps in total);
   g6_md_end synchronises, returns thermostats/log and reports device errors. */
int g6_md_begin(g6_ctx* ctx, double dt, int max_steps, const g6_thermostat* thermo, int want_log);
int g6_md_advance(g6_ctx* ctx, int nsteps);
int g6_md_end(g6_ctx* ctx, g6_thermostat* thermo, double* log);
/* The cudaStream_t (as void*) on which the context enqueues its work. */
int g6_stream(g6_ctx* ctx, void** stream);
/* Step timing: with g6_set_step_timing(ctx, 1) every MD step runs as its own
   one-step CUDA graph that records events around the whole step; with mode 2
   also around the fused force/integrator kernel (the extra event nodes add
   their own latency to the step).  g6_step_times waits for the last step and
   returns both durations in ms (kernel_ms = 0 in mode 1); 0 turns it off. */
int g6_set_step_timing(g6_ctx* ctx, int on);
int g6_step_times(g6_ctx* ctx, double* step_ms, double* kernel_ms);
/* Duration (ms, CUDA events on the context's stream) of one launch of the
   force kernel on the current configuration and neighbour list. */
int g6_time_force(g6_ctx* ctx, double* ms);
/* Lanes cooperating on one molecule in the force kernel and in the fused MD
   step kernel (4, 8, 16 or 32).  g6_tune times each choice on the uploaded
   configuration -- the force kernel alone, and the MD step in a short NVE run
   whose state is restored afterwards -- and keeps the fastest of each (lpi
   gets the MD choice); g6_set_lpi fixes both.  Without either, the first
   force evaluation or run picks a value from the system size.  (Per-lane
   partial sums change with it, so results differ at rounding level between
   choices.) */
int g6_tune(g6_ctx* ctx, int* lpi);
int g6_set_lpi(g6_ctx* ctx, int lpi);

/* Kernel shape of a context: the parameters that change the speed of the
   force and MD-step kernels but not the set of interacting pairs (every
   listed pair is re-tested against r_out each step).  No counterpart in the
   reference, whose CPU loops have no launch shape. */
typedef struct g6_shape {
  int lpi;         /* lanes per molecule, force-only kernel (4, 8, 16, 32)           */
  int step_lpi;    /* lanes per molecule, pair kernel of the MD step (4, 8, 16, 32)  */
  int step_mpw;    /* mixed MD integrator: molecules per warp, one lane each (8, 16,
                      32), or 4: four lanes per molecule (component-parallel)      */
  double skin;     /* Verlet margin [A] (g6_set_skin)                                */
  int cap;         /* neighbour-list row capacity (entries); g6_set_shape: 0 derives it
                      from the skin and the density (twice the expected row + 64)    */
  double step_ms;  /* g6_tune_shape: the chosen shape's MD step time in the search   */
  int step_half;   /* MD step: 1 = half list (each pair within rc evaluated once;
                      the other molecule's force and torque added with atomics --
                      float in mixed precision, FP64 in FP64 -- so the order of those
                      sums varies and runs are not bit-reproducible), 0 = full list
                      (every pair from both sides, fixed summation order,
                      bit-reproducible).  Default (no g6_set_shape): half in mixed
                      precision, full in FP64; g6_tune_shape times both unless
                      g6_set_shape chose */
} g6_shape;
#define G6_TUNE_SKIN 1
/* Autotuner: times the candidates on the uploaded state (restored after every
   trial run) with CUDA events -- the force kernel for lpi, short NVE runs for
   every (step_lpi, step_mpw) pair and, with G6_TUNE_SKIN, 128-step runs for
   skins of 0.5, 0.75, 1.0 and 1.5 A (the rebuild frequency depends on the
   skin) -- and keeps the fastest.  The choice is cached per model, path,
   precision, replica count, molecule count and cutoff: a context of the same
   size that has no shape of its own starts from it.  g6_tune is
   g6_tune_shape(ctx, 0, NULL) returning step_lpi. */
int g6_tune_shape(g6_ctx* ctx, int flags, g6_shape* shape);
int g6_get_shape(g6_ctx* ctx, g6_shape* shape);
int g6_set_shape(g6_ctx* ctx, const g6_shape* shape);

/* One MD step with the state in caller-owned host memory: uploads rec,
   advances one step, downloads rec and the step's log record.  This is the
   call a host-side driver makes when it keeps the state itself.  With rec in
   page-locked memory the whole call runs as one CUDA graph, captured on the
   first call for that rec pointer, dt, log choice and lane width (so that
   first call must not come during a stream capture); in mixed precision its
   kernels then read and write rec directly through the buffer's device
   address instead of staging copies, the run's control words (thermostat,
   control, sums, log row) travel through the context's own page-locked block
   the same way, and the call polls the stream for the end of the step.
   Pageable rec works too, operation by operation.  The neighbour list of the
   previous call is kept when no molecule moved more than half the skin since
   it was built. */
int g6_md_step_host(g6_ctx* ctx, double dt, g6_thermostat* thermo, double* rec, double* log);

/* replica_exchange_trial (Replica.F90:7-73) for neighbouring temperatures of
   the replicas of this context, FP64 acceptance.  beta[nrep] is in 1/K and is
   permuted in place on acceptance (with the MD side effects of
   Mixture.F90:1630-1653: velocities scaled by sqrt(T'/T), Nose zeta reset).
   The temperature slots are the replicas ordered by decreasing beta (the
   reference's node_in_charge, Mixture.F90:1589-1611); parity selects the slot
   pairs (j, j+1) with j % 2 == parity.  accepted[nrep] (optional) gets 1 for
   the replica in the lower slot of each accepted pair. */
int g6_replica_exchange(g6_ctx* ctx, int parity, uint64_t seed, uint64_t counter, double* beta,
                        g6_thermostat* thermo, int* accepted);
/* The same with numbrella parabolic umbrellas per replica on order parameters
   the caller computes (Replica.F90:20-62, Umbrella.F90:11-16): each side of the
   test adds coeffi (op - center)^2 for its umbrellas; umbrella[nrep][numbrella][2]
   = (center, coeffi) is swapped between the replicas of an accepted pair
   together with beta; op[nrep][numbrella] is read only. */
int g6_replica_exchange_umbrella(g6_ctx* ctx, int parity, uint64_t seed, uint64_t counter, double* beta,
                                 g6_thermostat* thermo, int numbrella, double* umbrella, const double* op,
                                 int* accepted);

/* The decision step of g6_replica_exchange(_umbrella) on the host, for an
   ensemble whose replicas live in several contexts, processes or GPUs: the
   gather -> replica_exchange_trial -> scatter of mc2.F90:901-1001 and
   Mixture.F90:1583-1653, where every process gathers the (E, beta, T,
   umbrella, op) of all nrep replicas, calls this with the same arguments
   (same seed and counter) and so reaches the same decisions.  Host only, no
   context and no device.  epot[nrep] (internal units), beta[nrep] [1/K] and
   temp[nrep] [K, the thermostat targets] are permuted in place on acceptance
   (umbrella[nrep][numbrella][2] too); scale[nrep] gets the velocity factor
   sqrt(T_new/T_old) (1 when unchanged), accepted[nrep] (optional) as above.
   Decisions and draws are those of g6_replica_exchange_umbrella; apply the
   factors to a context's replicas with g6_replica_scale and reset the Nose
   zeta of each replica whose temperature changed. */
int g6_exchange_plan(int nrep, int parity, uint64_t seed, uint64_t counter, const double* epot, double* beta,
                     double* temp, int numbrella, double* umbrella, const double* op, double* scale, int* accepted);
/* Rigid_ScaleVelocity (Mixture.F90:1631-1637) for every replica of the
   context: the COM and angular-velocity first derivatives of replica r are
   multiplied by scale[r] (> 0). */
int g6_replica_scale(g6_ctx* ctx, const double* scale);
/* Potential energy epot[nrep] of each replica at the last MD step (the
   rep_energy that replica_exchange_trial reads, Mixture.F90:1587). */
int g6_last_epot(g6_ctx* ctx, double* epot);

/* Monte Carlo, mc2.F90:544-832: the replicas of the context are independent
   chains; each advances ntrial single-molecule trials (uniform target,
   Gaussian translation of per-axis width sigma_t [A], rotation vector of
   per-axis width sigma_r [rad] applied with qinfrotator + qadd,
   QuatModule.F90:108-223) under an exact Metropolis-Hastings test at
   beta[r] [1/K] (acceptance exp(-dE*I2J*J2K*beta), mc2.F90:712-722, tested
   as log(u) < -dE*I2J*J2K*beta).  dE sums
   the PairPotential energies of the target at both poses against every other
   molecule of its chain, so no stored pair table is needed and the chain is
   exact; the reference's per-trial width adaptation (mc2.F90:794-810) is not
   applied.  Modes: G6_MC_PLAIN uses sigma_t/sigma_r; G6_MC_LEARNED takes the
   widths from the network (g6_mlp_*) evaluated at the old pose, with the
   reverse density at the new pose in the Hastings ratio; G6_MC_COLLECT runs
   the plain proposal and stores one training record per trial.  Precision
   follows the context: mixed contexts evaluate trial poses and pair energies
   in FP32 and keep the state in FP64.  Draws come
   from Philox4x32-10 (key = seed, counter = chain, trial, draw).
   samples (optional, nrep x ntrial/sample_every) gets the running energy,
   counts (optional, nrep x 2) accepted/attempted, energy (optional, nrep) the
   final energies, trace (optional, nrep x ntrial x 4) per trial dE, energy,
   accepted flag and target index.  G6_MC_LEARNED and G6_MC_COLLECT return
   G6_ERR_CAPACITY when a pose has more than 64 molecules within the 6 A
   feature radius (about 31 in liquid water at 1 g/cm^3). */
#define G6_MC_PLAIN 0
#define G6_MC_LEARNED 1
#define G6_MC_COLLECT 2
int g6_mc_run(g6_ctx* ctx, int ntrial, uint64_t seed, uint64_t counter, const double* beta, const double* sigma_t,
              const double* sigma_r, int mode, int sample_every, double* samples, int64_t* counts, double* energy,
              double* trace);

/* Order parameters of umbrella Monte Carlo (mc2.F90 OP_EP, OP_Q6T,
   OP_TRIANGLE), per chain (replica):
   G6_OP_EP        the chain's potential energy;
   G6_OP_Q6        local Q6 (Q6Local.F90): bonds are pairs within 3 A, the
                   neighbourhood of a molecule is itself and the molecules
                   within 5 A, q6(k) = sqrt(4 pi/13 sum_m |sum Y_6m(b)|^2) /
                   nbond(k) over the directed bonds b with both ends in k's
                   neighbourhood; op = mean of q6 over the chain;
   G6_OP_TRIANGLE  Triangle.F90: the cosines of the angles spanned at every
                   molecule by its (at most) 4 nearest neighbours within 5 A,
                   in G6_OP_NBIN bins of 0.1 on [-1, 1]; op = Kullback
                   divergence of that histogram from refhist (its log when
                   logarithmic != 0).
   Distances use the minimum image of the COMs.  A bond along the z axis
   (x = y = 0) gives 0/0 in e^{i phi} as in the reference. */
#define G6_OP_EP 0
#define G6_OP_Q6 1
#define G6_OP_TRIANGLE 2
#define G6_OP_NBIN 21
/* op[nrep] of the current state (refhist[G6_OP_NBIN] for G6_OP_TRIANGLE). */
int g6_order_parameter(g6_ctx* ctx, int kind, const double* refhist, int logarithmic, double* op);
/* g6_mc_run (G6_MC_PLAIN proposal) with a parabolic umbrella per chain,
   umbrella[nrep][2] = (center, coeff), on the order parameter `kind`: the
   trial's order parameter is evaluated incrementally on the device
   (Differentiate / Integrate / Reject of Q6Local.F90 and Triangle.F90) and
   coeff (op_new - center)^2 - coeff (op - center)^2 is added to dE in the
   Metropolis test (mc2.F90:684-722).  op[nrep] (optional) gets the final
   order parameters, samples/op_samples (optional, nrep x ntrial/sample_every)
   the running energy and order parameter, trace (optional, nrep x ntrial x
   5) dE, energy, accepted, target and op per trial.  Returns
   G6_ERR_CAPACITY when a molecule has more than 48 neighbours within 5 A or
   more than 10 bonds, or a trial more than 64 molecules within 5 A of its
   two poses. */
int g6_mc_run_umbrella(g6_ctx* ctx, int ntrial, uint64_t seed, uint64_t counter, const double* beta,
                       const double* sigma_t, const double* sigma_r, int kind, const double* umbrella,
                       const double* refhist, int logarithmic, double* op, int sample_every, double* samples,
                       double* op_samples, int64_t* counts, double* energy, double* trace);

/* Proposal-width network: 24 local-environment features -> 64 -> 64 (tanh)
   -> 2 widths, sigma = sigma0 * (0.1 + 2.9 sigmoid(z)).  Parameters are one
   float array of G6_MLP_NPARAM values: W1[64][24], b1[64], W2[64][64],
   b2[64], W3[2][64], b3[2]; features are normalised with feat_mean and
   feat_inv_std.  A training record is G6_MLP_RECORD floats: features at the
   old and at the proposed pose, |translation|^2, |rotation vector|^2 and
   beta*dE. */
#define G6_MLP_NPARAM 5890
#define G6_MLP_NFEAT 24
#define G6_MLP_RECORD 51
int g6_mlp_set(g6_ctx* ctx, const float* params, const float* feat_mean, const float* feat_inv_std, double sigma0_t,
               double sigma0_r);
int g6_mlp_get(g6_ctx* ctx, float* params, float* feat_mean, float* feat_inv_std);
/* Copy up to cap collected records to host (count = records held); cap < 0 discards them. */
int g6_mlp_records(g6_ctx* ctx, float* host, int64_t cap, int64_t* count);
/* Mean loss and its gradient over caller records (host) with the current parameters. */
int g6_mlp_grad(g6_ctx* ctx, const float* records, int64_t nrec, float* grad, double* loss);
/* Training objective: the mean over records of
   min(q(x'|x), exp(-beta dE) q(x|x')) / q0(x'|x) * (w_move * D + w_energy * (beta dE)^2),
   the expected jump of an accepted move under the network's proposal q,
   estimated from moves drawn with the fixed widths (q0); D = |dx|^2/sigma0_t^2
   + |rot|^2/sigma0_r^2.  Defaults: w_move = 1, w_energy = 0. */
int g6_mlp_objective(g6_ctx* ctx, double w_move, double w_energy);
/* Widths sigma_t[n], sigma_r[n] the current network gives for n raw feature
   rows (n x G6_MLP_NFEAT floats, e.g. the first half of training records).
   This evaluation uses tanhf; the Monte Carlo kernel of a mixed context uses
   the hardware tanh approximation (relative error below 2^-10), the same
   function for both poses of a trial, so its chains stay exact. */
int g6_mlp_widths(g6_ctx* ctx, const float* features, int64_t n, double* sigma_t, double* sigma_r);
/* Train on the collected records with Adam (hand-written forward/backward
   kernels); loss (optional, epochs) gets the mean loss of each epoch. */
int g6_mlp_train(g6_ctx* ctx, int epochs, int batch, double lr, uint64_t seed, double sigma0_t, double sigma0_r,
                 double* loss);

/* Force evaluation that allocates no device memory.  No counterpart in the
   reference: it exists for callers that may not call cudaMalloc -- programs
   whose device memory is owned by their own arena or pool, or that must not
   grow the process's device footprint -- and that hold their own device
   buffers.  Same computation as g6_force (sites, cell grid, neighbour list,
   force, collect) for ONE system of at most G6_NOALLOC_MAX_MOL molecules;
   larger n returns G6_ERR_CAPACITY, and so does a neighbour-list row of more
   than 224 entries (r_out + skin above about 11.7 A in water at 1 g/cm^3).
   0 <= r_in < r_out <= box/2 and skin >= 0 are required (G6_ERR_ARG
   otherwise).  d_com (n,3), d_quat (n,4) are device
   inputs; d_F (n,3), d_tau (n,3, body frame) and d_epot (1) are device
   outputs; box (3) is host memory; stream is a cudaStream_t (NULL = default).
   Intermediate tables live in one static device array of 7,195,392 bytes (6.9 MiB) that
   every GPU loading the library keeps until exit.  The first call on a device
   looks up that array's address: make it before any stream capture.  All
   calls share the array, so calls that overlap on the GPU race; serialise
   them.  The call waits for its stream before returning. */
#define G6_NOALLOC_MAX_MOL 4096
int g6_force_noalloc(int model, int path, int precision, int n, const double* box, double r_in, double r_out,
                     double skin, const double* d_com, const double* d_quat, double* d_F, double* d_tau,
                     double* d_epot, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* G6GPU_H */
