// g6_oracle.cpp -- FP64 CPU restatement of Genesis6's rigid-water force/energy path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker that the CUDA library
// (libg6gpu.so) is compared against.  Only tests/, __graft_entry__.smoke() and
// the CPU-baseline leg of bench.py load it.  The product path never calls it.
//
// PARITY UNPINNED: Genesis6 ships no test vectors and its Fortran cannot be
// compiled or run here (no Fortran compiler), so no output of the reference
// itself exists to pin this restatement against.  It is checked instead by
//   (1) dimer energies/forces computed independently in closed form
//       (tests/golden/make_golden.py -> tests/golden/*.json),
//   (2) the reference's own in-code self-checks restated as tests
//       (incremental-vs-full MC energy, virial identity, hand-kernel vs
//       StdForce for TIP4P, finite-difference forces/torques).
//
// Build: g++ -O2 -ffp-contract=off -fno-fast-math -fopenmp -shared -fPIC.
// -ffp-contract=off keeps every a*b+c as two IEEE operations so that the cell
// assignment and the `dd < rc^2` pair decision reproduce the reference's FP64
// arithmetic bit for bit.
//
// Every function cites the reference file:line it restates.  Indices are
// 0-based here; the reference is 1-based.

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------------------
// Units and constants: PhysConst.F90:4-62, TIP4PConst.F90:4-22
// ---------------------------------------------------------------------------
const double PI = 3.1415926535897932;          // PItanaka, PhysConst.F90:18-19
const double NA = 6.0225e23;                   // PhysConst.F90:21
const double KB = 1.380066e-23;                // PhysConst.F90:24
const double RGAS = NA * KB;                   // PhysConst.F90:26
const double CA = 4.184;                       // CAtanaka, PhysConst.F90:29-30
const double COEFF = CA * 332.17752;           // COEFFtanaka, PhysConst.F90:43-44
const double X2KX = 1e-3;                      // PhysConst.F90:38
const double KX2X = 1.0 / X2KX;                // PhysConst.F90:40
const double I2J = 10.0;                       // PhysConst.F90:48
const double J2I = 1.0 / I2J;                  // PhysConst.F90:50
const double J2K = 0.120273;                   // PhysConst.F90:56 (literal)
const double A2P = 101326.0;                   // PhysConst.F90:52
const double P2A = 1.0 / A2P;
const double ANG2M = 1e-10;
const double GEAR5_0 = 3.0 / 16.0, GEAR5_1 = 251.0 / 360.0, GEAR5_3 = 11.0 / 18.0,
             GEAR5_4 = 1.0 / 6.0, GEAR5_5 = 1.0 / 60.0;      // PhysConst.F90:7-11
const double GEAR4_0 = 251.0 / 720.0, GEAR4_2 = 11.0 / 12.0, GEAR4_3 = 1.0 / 3.0,
             GEAR4_4 = 1.0 / 24.0;                          // PhysConst.F90:12-15

// TIP4P hand-kernel constants, TIP4PConst.F90:4-18
const double T4_AA = (600000.0 * CA * 100.0);
const double T4_BB = (-610.0 * CA * 100.0);
const double T4_WM = -1.04, T4_WH = 0.52;
const double T4_WWMM = T4_WM * T4_WM * COEFF * 100.0;
const double T4_WWMH = T4_WM * T4_WH * COEFF * 100.0;
const double T4_WWHH = T4_WH * T4_WH * COEFF * 100.0;
const double T4_EPSWO = 0.15504166666666666666666 * CA;
const double T4_SIGWO = 3.15357794197649532464;

// ST2 constants, ST2Module.F90:10-26.  Q and EPS are default-real (float)
// literals promoted to double (quirk kept on purpose).
const double ST2_QM = (double)(-0.2357f);
const double ST2_QH = (double)(+0.2357f);
const double ST2_EPS = (double)(0.52605e-21f) * NA * 1e-3;
const double ST2_SIG = 3.100;
const double ST2_RL = 2.0160, ST2_RU = 3.1287;

inline double pow6(double x) { double x2 = x * x; return x2 * x2 * x2; }
// x**5 evaluated by binary powering, as Fortran integer powers are.
inline double powi5(double x) { double x2 = x * x; return x * (x2 * x2); }
inline double pow12(double x) { double x6 = pow6(x); return x6 * x6; }
// Fortran dnint: round half away from zero.
inline double dnint(double x) { return std::round(x); }

// ---------------------------------------------------------------------------
// Models
// ---------------------------------------------------------------------------
enum { M_TIP4P = 1, M_TIP5P = 2, M_ST2 = 3, M_SPCE = 4, M_OPLSMEOH = 5 };
enum { P_STD = 0, P_CUSTOM = 1 };
const int MAXS = 8;

struct Model {
  int id = 0, nsite = 0;
  double molx[MAXS] = {0}, moly[MAXS] = {0}, molz[MAXS] = {0};
  double q[MAXS] = {0}, eps[MAXS] = {0}, sig[MAXS] = {0};   // sStdInt%param(1:3,:)
  double mass = 0, Ixx = 0, Iyy = 0, Izz = 0;
};

// Rigid_TIP4P_Constructor TIP4PModule.F90:70-97, tip4p_setinteraction :43-68
void model_tip4p(Model& m) {
  m.id = M_TIP4P; m.nsite = 5;
  m.Ixx = 1.75618411509879202e+00; m.Iyy = 6.10236519209664374e-01; m.Izz = 1.14594759588912742e+00;
  m.mass = 18.0;
  const double y[5] = {0.0, 0.0, 7.56950327263661182e-01, -7.56950327263661182e-01, 0.0};
  const double z[5] = {-6.50980307353661025e-02, 8.49019692646338919e-02, 5.20784245882928820e-01,
                       5.20784245882928820e-01, 0.0};
  for (int s = 0; s < 5; ++s) { m.molx[s] = 0; m.moly[s] = y[s]; m.molz[s] = z[s]; }
  m.q[1] = T4_WM; m.q[2] = T4_WH; m.q[3] = T4_WH;
  m.eps[0] = T4_EPSWO; m.sig[0] = T4_SIGWO;
}

// Shared 5+1-site construction of Rigid_TIP5P_Constructor RigidModule.F90:429-477
// and Rigid_ST2_Constructor ST2Module.F90:60-100.
void five_site_geometry(Model& m, double theta, double phi, double l1, double l2) {
  const double hmass = 1.0, omass = 16.0;
  m.nsite = 6;
  m.molx[0] = 0; m.moly[0] = 0; m.molz[0] = 0;
  m.molx[1] = 0; m.moly[1] = l1 * std::sin(0.5 * theta); m.molz[1] = l1 * std::cos(0.5 * theta);
  m.molx[2] = 0; m.moly[2] = -l1 * std::sin(0.5 * theta); m.molz[2] = l1 * std::cos(0.5 * theta);
  m.molx[3] = l2 * std::sin(0.5 * phi); m.moly[3] = 0; m.molz[3] = -l2 * std::cos(0.5 * phi);
  m.molx[4] = -l2 * std::sin(0.5 * phi); m.moly[4] = 0; m.molz[4] = -l2 * std::cos(0.5 * phi);
  double zshift = m.molz[1] * 2.0 * hmass / (2.0 * hmass + omass);
  for (int i = 0; i < 5; ++i) m.molz[i] = m.molz[i] - zshift;
  m.molx[5] = m.moly[5] = m.molz[5] = 0;
  m.Ixx = omass * (m.moly[0] * m.moly[0] + m.molz[0] * m.molz[0]) +
          hmass * (m.moly[1] * m.moly[1] + m.molz[1] * m.molz[1]) * 2.0;
  m.Iyy = omass * (m.molz[0] * m.molz[0] + m.molx[0] * m.molx[0]) +
          hmass * (m.molz[1] * m.molz[1] + m.molx[1] * m.molx[1]) * 2.0;
  m.Izz = omass * (m.molx[0] * m.molx[0] + m.moly[0] * m.moly[0]) +
          hmass * (m.molx[1] * m.molx[1] + m.moly[1] * m.moly[1]) * 2.0;
  m.mass = 2.0 * hmass + omass;
}

// TIP5P: RigidModule.F90:429-477, tip5p_setinteraction TIP5PModule.F90:57-83
void model_tip5p(Model& m) {
  m.id = M_TIP5P;
  five_site_geometry(m, 104.52 * PI / 180.0, 109.47 * PI / 180.0, 0.9572, 0.70);
  const double c = 0.2410;
  m.q[1] = c; m.q[2] = c; m.q[3] = -c; m.q[4] = -c;
  m.eps[0] = 0.6694; m.sig[0] = 3.12;
}

// ST2: ST2Module.F90:10-58 (setinteraction), :60-100 (geometry)
void model_st2(Model& m) {
  m.id = M_ST2;
  const double th = 109.47 * PI / 180.0;
  five_site_geometry(m, th, th, 1.0, 0.8);
  m.q[1] = ST2_QH; m.q[2] = ST2_QH; m.q[3] = ST2_QM; m.q[4] = ST2_QM;
  m.eps[0] = ST2_EPS; m.sig[0] = ST2_SIG;
}

// SPC/E: Rigid_SPCE_Constructor SPCEModule.F90:44-71, spce_setinteraction :24-43
// (the oxygen carries both the charge and the LJ site; StdForce only).
void model_spce(Model& m) {
  m.id = M_SPCE; m.nsite = 4;
  const double theta = 109.5 * PI / 180.0, l1 = 1.0, hmass = 1.0, omass = 16.0;
  m.molx[0] = 0; m.moly[0] = 0; m.molz[0] = 0;
  m.molx[1] = 0; m.moly[1] = l1 * std::sin(0.5 * theta); m.molz[1] = l1 * std::cos(0.5 * theta);
  m.molx[2] = 0; m.moly[2] = -l1 * std::sin(0.5 * theta); m.molz[2] = l1 * std::cos(0.5 * theta);
  double zshift = m.molz[1] * 2.0 * hmass / (2.0 * hmass + omass);
  for (int i = 0; i < 3; ++i) m.molz[i] = m.molz[i] - zshift;
  m.molx[3] = m.moly[3] = m.molz[3] = 0;
  m.Ixx = omass * (m.moly[0] * m.moly[0] + m.molz[0] * m.molz[0]) +
          hmass * (m.moly[1] * m.moly[1] + m.molz[1] * m.molz[1]) * 2.0;
  m.Iyy = omass * (m.molz[0] * m.molz[0] + m.molx[0] * m.molx[0]) +
          hmass * (m.molz[1] * m.molz[1] + m.molx[1] * m.molx[1]) * 2.0;
  m.Izz = omass * (m.molx[0] * m.molx[0] + m.moly[0] * m.moly[0]) +
          hmass * (m.molx[1] * m.molx[1] + m.moly[1] * m.moly[1]) * 2.0;
  m.mass = 2.0 * hmass + omass;
  m.q[0] = -0.8476; m.q[1] = 0.4238; m.q[2] = 0.4238;
  m.eps[0] = 78.208 / J2K * 1e-3; m.sig[0] = 3.166;
}

// OPLS methanol: Rigid_OPLSMeOH_Constructor RigidModule.F90:391-426 (Me, O,
// H, COM; masses 15, 16, 1), oplsmeoh_setinteraction OPLSMeOHModule.F90:82-101
// (charges :44-46, LJ of Me and O :53-56, J. Chem. Phys. 105, 11199 (1996)).
void model_oplsmeoh(Model& m) {
  m.id = M_OPLSMEOH; m.nsite = 4;
  const double mass[4] = {15.0, 16.0, 1.0, 0.0};
  const double x[4] = {0.0133, -0.0634, 0.8152, 0.0}, y[4] = {0.7666, -0.6559, -1.0042, 0.0};
  for (int s = 0; s < 4; ++s) { m.molx[s] = x[s]; m.moly[s] = y[s]; m.molz[s] = 0.0; }
  m.Ixx = m.Iyy = m.Izz = m.mass = 0.0;
  for (int s = 0; s < 4; ++s) {
    m.Ixx = m.Ixx + mass[s] * (m.moly[s] * m.moly[s] + m.molz[s] * m.molz[s]);
    m.Iyy = m.Iyy + mass[s] * (m.molz[s] * m.molz[s] + m.molx[s] * m.molx[s]);
    m.Izz = m.Izz + mass[s] * (m.molx[s] * m.molx[s] + m.moly[s] * m.moly[s]);
    m.mass = m.mass + mass[s];
  }
  m.q[0] = 0.265; m.q[1] = -0.700; m.q[2] = 0.435;
  m.eps[0] = 0.207 * CA; m.sig[0] = 3.775;
  m.eps[1] = 0.170 * CA; m.sig[1] = 3.070;
}

bool make_model(int id, Model& m) {
  m = Model();
  if (id == M_TIP4P) model_tip4p(m);
  else if (id == M_TIP5P) model_tip5p(m);
  else if (id == M_ST2) model_st2(m);
  else if (id == M_SPCE) model_spce(m);
  else if (id == M_OPLSMEOH) model_oplsmeoh(m);
  else return false;
  return true;
}

// ---------------------------------------------------------------------------
// Counter-based RNG: Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11).
// Same stream on the GPU, so Monte Carlo chains can be replayed step by step.
// ---------------------------------------------------------------------------
inline void philox4x32(uint32_t ctr[4], uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)M0 * ctr[0];
    uint64_t p1 = (uint64_t)M1 * ctr[2];
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ ctr[1] ^ k0, n2 = hi0 ^ ctr[3] ^ k1;
    ctr[0] = n0; ctr[1] = lo1; ctr[2] = n2; ctr[3] = lo0;
    k0 += W0; k1 += W1;
  }
}
// Two uniforms in (0,1] from one Philox block.
inline void uniform2(uint64_t seed, uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, double out[2]) {
  uint32_t c[4] = {c0, c1, c2, c3};
  philox4x32(c, (uint32_t)seed, (uint32_t)(seed >> 32));
  for (int k = 0; k < 2; ++k) {
    uint64_t u = ((uint64_t)(c[2 * k] >> 5) << 26) | (uint64_t)(c[2 * k + 1] >> 6);
    out[k] = ((double)u + 1.0) * (1.0 / 9007199254740992.0);
  }
}
// Random_Normal RandomModule.F90:20-28 (Box-Muller, sine branch; var = variance)
inline double random_normal(double avg, double var, double r1, double r2) {
  double r = std::sqrt(-2.0 * std::log(r1));
  double theta = 2.0 * PI * r2;
  return r * std::sin(theta) * std::sqrt(var) + avg;
}

// ---------------------------------------------------------------------------
// Site placement: rigid_setmatrix RigidModule.F90:62-83,
// rigid_setsiteposition0 :88-144 (non-VPOPTIMIZE branch)
// ---------------------------------------------------------------------------
void setmatrix(const double* q, double t[9]) {
  double qa = q[0], qb = q[1], qc = q[2], qd = q[3];
  t[0] = (qa * qa + qb * qb - (qc * qc + qd * qd));
  t[1] = -2.0 * (qa * qd + qb * qc);
  t[2] = 2.0 * (qb * qd - qa * qc);
  t[3] = 2.0 * (qa * qd - qb * qc);
  t[4] = qa * qa + qc * qc - (qb * qb + qd * qd);
  t[5] = -2.0 * (qa * qb + qc * qd);
  t[6] = 2.0 * (qa * qc + qb * qd);
  t[7] = 2.0 * (qa * qb - qc * qd);
  t[8] = qa * qa + qd * qd - (qb * qb + qc * qc);
}

void place_sites(const Model& m, int n, const double* com, const double* quat, double* sx, double* sy,
                 double* sz, double* intra, double* tmat) {
  for (int i = 0; i < n; ++i) {
    double t[9];
    setmatrix(quat + 4 * i, t);
    if (tmat) std::memcpy(tmat + 9 * i, t, sizeof t);
    for (int s = 0; s < m.nsite; ++s) {
      double ix = t[0] * m.molx[s] + t[1] * m.moly[s] + t[2] * m.molz[s];
      double iy = t[3] * m.molx[s] + t[4] * m.moly[s] + t[5] * m.molz[s];
      double iz = t[6] * m.molx[s] + t[7] * m.moly[s] + t[8] * m.molz[s];
      if (intra) { intra[3 * (i * m.nsite + s)] = ix; intra[3 * (i * m.nsite + s) + 1] = iy; intra[3 * (i * m.nsite + s) + 2] = iz; }
      sx[i * m.nsite + s] = com[3 * i] + ix;
      sy[i * m.nsite + s] = com[3 * i + 1] + iy;
      sz[i * m.nsite + s] = com[3 * i + 2] + iz;
    }
  }
}

// ---------------------------------------------------------------------------
// Cell grid and pair search
// ---------------------------------------------------------------------------
struct Grid {
  int nd[3] = {1, 1, 1};
  double cell[3] = {0, 0, 0};
  std::vector<int> n, n0;   // stencil offsets (x,y,z triples), half shell and self-mirror
};

// NeighborCell_ListHomo GridModule.F90:279-374 (maxradius == 0 branch)
void neighborcell_listhomo(Grid& g) {
  int nmax[3], nmin[3];
  for (int d = 0; d < 3; ++d) {
    nmax[d] = 1; nmin[d] = -1;
    if (nmax[d] > (g.nd[d] - 1) / 2) nmax[d] = (g.nd[d] - 1) / 2;
    if (nmin[d] < -(g.nd[d] / 2)) nmin[d] = -(g.nd[d] / 2);
  }
  std::vector<int> mark((size_t)g.nd[0] * g.nd[1] * g.nd[2], 0);
  auto at = [&](int x, int y, int z) -> int& { return mark[((size_t)z * g.nd[1] + y) * g.nd[0] + x]; };
  g.n.clear(); g.n0.clear();
  for (int jz = nmin[2]; jz <= nmax[2]; ++jz) {
    int pz = jz < 0 ? jz + g.nd[2] : jz, mz = pz == 0 ? 0 : g.nd[2] - pz;
    for (int jy = nmin[1]; jy <= nmax[1]; ++jy) {
      int py = jy < 0 ? jy + g.nd[1] : jy, my = py == 0 ? 0 : g.nd[1] - py;
      for (int jx = nmin[0]; jx <= nmax[0]; ++jx) {
        int px = jx < 0 ? jx + g.nd[0] : jx, mx = px == 0 ? 0 : g.nd[0] - px;
        if (at(px, py, pz) == 0) {
          at(mx, my, mz) += 1;
          at(px, py, pz) += 1;
          std::vector<int>& dst = (at(px, py, pz) != 1) ? g.n0 : g.n;
          dst.push_back(px); dst.push_back(py); dst.push_back(pz);
        }
      }
    }
  }
}

// Grid_Update (adaptive) GridModule.F90:95-125 -> Grid_ResetDivision :488-501
// -> Grid_ResetCellSize :473-486.  ndiv = int(L/req) is clamped to >= 1 (the
// reference divides by zero when the box is smaller than the requested cell).
void grid_update(Grid& g, const double L[3], const double req[3]) {
  for (int d = 0; d < 3; ++d) {
    int nd = (int)(L[d] / req[d]);
    g.nd[d] = nd < 1 ? 1 : nd;
    g.cell[d] = L[d] / g.nd[d];
  }
  neighborcell_listhomo(g);
}

// Address_Assign GridModule.F90:503-531 (cell index part), box_renormalize
// BoxModule.F90:58-68.  Returns the 0-based cell id (reference mAddr - 1).
int cell_of(const Grid& g, const double* c, const double L[3], const double invL[3]) {
  double ci[3] = {1.0 / g.cell[0], 1.0 / g.cell[1], 1.0 / g.cell[2]};
  int j[3];
  for (int d = 0; d < 3; ++d) {
    double delta = c[d];
    double cellv = dnint(delta * invL[d]) * L[d];
    delta = delta - cellv;
    int jj = (int)dnint(delta * ci[d]);
    if (jj < 0) jj += g.nd[d];
    if (jj >= g.nd[d]) jj -= g.nd[d];   // only reachable for ndiv == 1 at |delta| == L/2
    j[d] = jj;
  }
  return (j[2] * g.nd[1] + j[1]) * g.nd[0] + j[0];
}

struct Pairs {
  std::vector<int> i, j;
  std::vector<double> ox, oy, oz, hh, dh;
  void clear() { i.clear(); j.clear(); ox.clear(); oy.clear(); oz.clear(); hh.clear(); dh.clear(); }
};

// Interaction_Compress2 InteractionModule.F90:398-470 (fbox, TEST32 inline
// image, TEST31 explicit squares): keep the candidate when dd < rr (strict).
inline bool compress_test(const double* ci, const double* cj, const double L[3], const double invL[3], double rr,
                          double o[3]) {
  double d[3];
  for (int k = 0; k < 3; ++k) {
    double delta = ci[k] - cj[k];
    o[k] = dnint(delta * invL[k]) * L[k];
    d[k] = delta - o[k];
  }
  double dd = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
  return dd < rr;
}

// Grid_NeighborList GridModule.F90:557-752 followed by Interaction_Compress2:
// candidate pairs cell by cell (half-shell list, then the self-mirror list with
// j > i), filtered by the strict cutoff test.  Pairs come out in the
// reference's order: cell, resident i, stencil entry, resident j.
void pairsearch(int n, const double* com, const double L[3], const double req[3], double rc, Grid& g,
                std::vector<int>& cellid, Pairs& P) {
  double invL[3] = {1.0 / L[0], 1.0 / L[1], 1.0 / L[2]};
  grid_update(g, L, req);
  int ng = g.nd[0] * g.nd[1] * g.nd[2];
  cellid.assign(n, 0);
  std::vector<std::vector<int>> resident(ng);
  for (int i = 0; i < n; ++i) {
    cellid[i] = cell_of(g, com + 3 * i, L, invL);
    resident[cellid[i]].push_back(i);        // molecule order (Address_Assign :536-546)
  }
  double rr = rc * rc;
  P.clear();
  auto emit = [&](int i, int j) {
    double o[3];
    if (compress_test(com + 3 * i, com + 3 * j, L, invL, rr, o)) {
      P.i.push_back(i); P.j.push_back(j);
      P.ox.push_back(o[0]); P.oy.push_back(o[1]); P.oz.push_back(o[2]);
      P.hh.push_back(1.0); P.dh.push_back(0.0);   // eratio=1, fratio=0 (:602-603)
    }
  };
  for (int pass = 0; pass < 2; ++pass) {
    const std::vector<int>& st = pass == 0 ? g.n : g.n0;
    int ns = (int)st.size() / 3;
    for (int c = 0; c < ng; ++c) {
      int cx = c % g.nd[0], cy = (c / g.nd[0]) % g.nd[1], cz = c / (g.nd[0] * g.nd[1]);
      for (int i : resident[c]) {
        for (int s = 0; s < ns; ++s) {   // NeighborCell_MakeAcl :941-967
          int nx = (cx + st[3 * s]) % g.nd[0], ny = (cy + st[3 * s + 1]) % g.nd[1], nz = (cz + st[3 * s + 2]) % g.nd[2];
          int cj = (nz * g.nd[1] + ny) * g.nd[0] + nx;
          for (int j : resident[cj]) {
            if (pass == 1 && !(j > i)) continue;   // :722-727
            emit(i, j);
          }
        }
      }
    }
  }
}

// NeighborCell_ListHetero GridModule.F90:757-899 (maxradius == 0, the adaptive
// grid): every offset of -1..1 per axis, clipped to (ndiv-1)/2 and -ndiv/2,
// as a cell offset in [0, ndiv).  No mirror marks: the two components' pairs
// are ordered, so all cells of the stencil are visited.
std::vector<int> neighborcell_listhetero(const Grid& g) {
  int nmax[3], nmin[3];
  for (int d = 0; d < 3; ++d) {
    nmax[d] = 1; nmin[d] = -1;
    if (nmax[d] > (g.nd[d] - 1) / 2) nmax[d] = (g.nd[d] - 1) / 2;
    if (nmin[d] < -(g.nd[d] / 2)) nmin[d] = -(g.nd[d] / 2);
  }
  std::vector<int> st;
  for (int jz = nmin[2]; jz <= nmax[2]; ++jz)
    for (int jy = nmin[1]; jy <= nmax[1]; ++jy)
      for (int jx = nmin[0]; jx <= nmax[0]; ++jx) {
        st.push_back(jx < 0 ? jx + g.nd[0] : jx);
        st.push_back(jy < 0 ? jy + g.nd[1] : jy);
        st.push_back(jz < 0 ? jz + g.nd[2] : jz);
      }
  return st;
}

// Grid_NeighborList(g, g%hetero, iv, ai, aj) + Interaction_Compress2 for two
// components in one box (GridModule.F90:557-752; the same grid, one address
// table per component, InteractionModule.F90:398-470): for every cell, its A
// residents against the B residents of each stencil cell, strict cutoff test.
// Pairs (i in A, j in B) in the reference's order: cell, i, stencil entry, j.
void pairsearch_hetero(int na, const double* ca, int nb, const double* cb, const double L[3], const double req[3],
                       double rc, std::vector<int>& cella, std::vector<int>& cellb, Pairs& P) {
  double invL[3] = {1.0 / L[0], 1.0 / L[1], 1.0 / L[2]};
  Grid g;
  grid_update(g, L, req);
  const std::vector<int> st = neighborcell_listhetero(g);
  const int ng = g.nd[0] * g.nd[1] * g.nd[2], ns = (int)st.size() / 3;
  cella.assign(na, 0); cellb.assign(nb, 0);
  std::vector<std::vector<int>> ra(ng), rb(ng);
  for (int i = 0; i < na; ++i) { cella[i] = cell_of(g, ca + 3 * i, L, invL); ra[cella[i]].push_back(i); }
  for (int j = 0; j < nb; ++j) { cellb[j] = cell_of(g, cb + 3 * j, L, invL); rb[cellb[j]].push_back(j); }
  const double rr = rc * rc;
  P.clear();
  for (int c = 0; c < ng; ++c) {
    const int cx = c % g.nd[0], cy = (c / g.nd[0]) % g.nd[1], cz = c / (g.nd[0] * g.nd[1]);
    for (int i : ra[c])
      for (int s = 0; s < ns; ++s) {
        const int nx = (cx + st[3 * s]) % g.nd[0], ny = (cy + st[3 * s + 1]) % g.nd[1], nz = (cz + st[3 * s + 2]) % g.nd[2];
        for (int j : rb[(nz * g.nd[1] + ny) * g.nd[0] + nx]) {
          double o[3];
          if (compress_test(ca + 3 * i, cb + 3 * j, L, invL, rr, o)) {
            P.i.push_back(i); P.j.push_back(j);
            P.ox.push_back(o[0]); P.oy.push_back(o[1]); P.oz.push_back(o[2]);
            P.hh.push_back(1.0); P.dh.push_back(0.0);
          }
        }
      }
  }
}

// pairsearch split over cells on nthreads host threads (CPU-baseline timing
// only): the same candidates and test, concatenated per cell in cell order.
void pairsearch_threaded(int n, const double* com, const double L[3], const double req[3], double rc, Grid& g,
                         Pairs& P, int nthreads) {
  double invL[3] = {1.0 / L[0], 1.0 / L[1], 1.0 / L[2]};
  grid_update(g, L, req);
  const int ng = g.nd[0] * g.nd[1] * g.nd[2];
  std::vector<std::vector<int>> resident(ng);
  for (int i = 0; i < n; ++i) resident[cell_of(g, com + 3 * i, L, invL)].push_back(i);
  const double rr = rc * rc;
  std::vector<Pairs> part(ng);
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
  for (int c = 0; c < ng; ++c) {
    Pairs& Q = part[c];
    const int cx = c % g.nd[0], cy = (c / g.nd[0]) % g.nd[1], cz = c / (g.nd[0] * g.nd[1]);
    for (int pass = 0; pass < 2; ++pass) {
      const std::vector<int>& st = pass == 0 ? g.n : g.n0;
      const int ns = (int)st.size() / 3;
      for (int i : resident[c])
        for (int s = 0; s < ns; ++s) {
          const int nx = (cx + st[3 * s]) % g.nd[0], ny = (cy + st[3 * s + 1]) % g.nd[1],
                    nz = (cz + st[3 * s + 2]) % g.nd[2];
          for (int j : resident[(nz * g.nd[1] + ny) * g.nd[0] + nx]) {
            if (pass == 1 && !(j > i)) continue;
            double o[3];
            if (compress_test(com + 3 * i, com + 3 * j, L, invL, rr, o)) {
              Q.i.push_back(i); Q.j.push_back(j); Q.ox.push_back(o[0]); Q.oy.push_back(o[1]); Q.oz.push_back(o[2]);
              Q.hh.push_back(1.0); Q.dh.push_back(0.0);
            }
          }
        }
    }
  }
  P.clear();
  for (auto& Q : part) {
    P.i.insert(P.i.end(), Q.i.begin(), Q.i.end()); P.j.insert(P.j.end(), Q.j.begin(), Q.j.end());
    P.ox.insert(P.ox.end(), Q.ox.begin(), Q.ox.end()); P.oy.insert(P.oy.end(), Q.oy.begin(), Q.oy.end());
    P.oz.insert(P.oz.end(), Q.oz.begin(), Q.oz.end()); P.hh.insert(P.hh.end(), Q.hh.begin(), Q.hh.end());
    P.dh.insert(P.dh.end(), Q.dh.begin(), Q.dh.end());
  }
}

// cutoff_func CutoffModule.F90:38-59
inline void cutoff_func(double rin, double rout, double dd, double& hh, double& dh) {
  double c1 = (1.0 / powi5(rin - rout));
  double c2 = (c1 * 30.0);
  hh = 0; dh = 0;
  if (dd < rout * rout) {
    if (dd > rin * rin) {
      double dr = std::sqrt(dd), u = dr - rout, l = dr - rin, uu = u * u, ll = l * l;
      hh = c1 * uu * u * (10.0 * ll - 5.0 * u * l + uu);
      dh = -c2 * uu * ll / dr;
    } else {
      hh = 1.0; dh = 0.0;
    }
  }
}

// CutOff_Dimmer2 CutoffModule.F90:220-278
void cutoff_dimmer2(double rin, double rout, const double* com_i, const double* com_j, Pairs& P) {
  for (size_t k = 0; k < P.i.size(); ++k) {
    const double* a = com_i + 3 * P.i[k];
    const double* b = com_j + 3 * P.j[k];
    double dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
    dx = dx - P.ox[k]; dy = dy - P.oy[k]; dz = dz - P.oz[k];
    cutoff_func(rin, rout, dx * dx + dy * dy + dz * dz, P.hh[k], P.dh[k]);
  }
}

// ---------------------------------------------------------------------------
// Pair forces
// ---------------------------------------------------------------------------
struct SiteArrays { const double *x, *y, *z; double *fx, *fy, *fz; };

// Std site-pair constants, StdInteraction.F90:201-222 (si: sites of the
// i-component, sj: of the j-component; LB mixing of eps and sigma)
struct StdPairConst { int si, sj; double qq, aa, bb; bool lj, coul; };
std::vector<StdPairConst> std_table2(const Model& mi, const Model& mj, double scale) {
  std::vector<StdPairConst> t;
  for (int is = 0; is < mi.nsite; ++is)
    for (int js = 0; js < mj.nsite; ++js) {
      StdPairConst c{is, js, 0, 0, 0, false, false};
      c.qq = mi.q[is] * mj.q[js] * COEFF * KX2X * J2I * scale;
      double aa = mi.eps[is] * mj.eps[js];
      if (c.qq == 0.0 && aa == 0.0) continue;
      c.coul = c.qq != 0.0;
      if (aa != 0.0) {
        double ljeps = std::sqrt(aa);
        double ljsig = pow6((mi.sig[is] + mj.sig[js]) * 0.5);
        c.aa = 4.0 * ljeps * ljsig * ljsig * KX2X * J2I * scale;
        c.bb = -4.0 * ljeps * ljsig * KX2X * J2I * scale;
        c.lj = true;
      }
      t.push_back(c);
    }
  return t;
}
std::vector<StdPairConst> std_table(const Model& m, double scale) { return std_table2(m, m, scale); }

// Constants of the hand kernel interaction_force_tip4p_oplsmeoh
// (OPLSMeOHModule.F90:1-7, 1189-1198, 1201-1480): water O with methyl and
// methanol O by LB mixing of EPSWO/SIGWO (TIP4PConst.F90:17-18), the TIP4P
// charges M, H with Me, O, H.  i: TIP4P sites (O, M, H, H, COM), j: OPLS-MeOH
// sites (Me, O, H, COM).
std::vector<StdPairConst> tip4p_meoh_table() {
  const double EPSM = 0.207 * CA, SIGM = 3.775, EPSO = 0.170 * CA, SIGO = 3.070;
  const double QM = 0.265, QO = -0.700, QH = 0.435;
  auto p12 = [](double x) { return pow12(x); };
  const double AAOMXS = p12((T4_SIGWO + SIGM) * 0.5) * 100.0, BBOMXS = pow6((T4_SIGWO + SIGM) * 0.5) * 100.0;
  const double AAOOXS = p12((T4_SIGWO + SIGO) * 0.5) * 100.0, BBOOXS = pow6((T4_SIGWO + SIGO) * 0.5) * 100.0;
  std::vector<StdPairConst> t;
  t.push_back({0, 0, 0.0, 4.0 * std::sqrt(T4_EPSWO * EPSM) * AAOMXS, -4.0 * std::sqrt(T4_EPSWO * EPSM) * BBOMXS, true, false});
  t.push_back({0, 1, 0.0, 4.0 * std::sqrt(T4_EPSWO * EPSO) * AAOOXS, -4.0 * std::sqrt(T4_EPSWO * EPSO) * BBOOXS, true, false});
  const double qw[4] = {0.0, T4_WM, T4_WH, T4_WH}, qm[3] = {QM, QO, QH};
  for (int a = 1; a <= 3; ++a)
    for (int b = 0; b < 3; ++b) t.push_back({a, b, qw[a] * qm[b] * COEFF * 100.0, 0.0, 0.0, false, true});
  return t;
}

// The site-pair table of force() for components mi, mj (Interaction2.F90:19-68):
// the TIP4P-OPLSMeOH hand kernel on the custom path, StdForce otherwise.
std::vector<StdPairConst> pair_table2(const Model& mi, const Model& mj, int path) {
  if (path == P_CUSTOM && mi.id == M_TIP4P && mj.id == M_OPLSMEOH) return tip4p_meoh_table();
  return std_table2(mi, mj, 1.0);
}

// StdForce StdInteraction.F90:63-630 on a site-pair table, for molecules of
// nsi sites (component at site offset offi) against molecules of nsj sites
// (offset offj); the COM is the last site of each.  Accumulation orders follow
// the reference: per pair and site, j-sites in ascending order for the i
// buffer and i-sites in ascending order for the j buffer; the scatter adds
// every i-side contribution before every j-side one (TEST22 branch :566-581).
void table_force(int nsi, int nsj, const std::vector<StdPairConst>& tab, const SiteArrays& S, int offi, int offj,
                 const Pairs& P, double* ep, double vrmat[9]) {
  const size_t np = P.i.size();
  std::vector<double> fi(np * nsi * 3, 0.0), fj(np * nsj * 3, 0.0);
  for (size_t k = 0; k < np; ++k) {
    int ii = offi + P.i[k] * nsi, jj = offj + P.j[k] * nsj;
    double e = 0;
    for (const auto& c : tab) {
      double dx = S.x[ii + c.si] - S.x[jj + c.sj];
      double dy = S.y[ii + c.si] - S.y[jj + c.sj];
      double dz = S.z[ii + c.si] - S.z[jj + c.sj];
      dx = dx - P.ox[k]; dy = dy - P.oy[k]; dz = dz - P.oz[k];
      double dd = 1.0 / (dx * dx + dy * dy + dz * dz);
      double e0 = 0, f0 = 0;
      if (c.coul) {
        double radiusi = std::sqrt(dd);
        e0 = c.qq * radiusi;
        f0 = c.qq * radiusi * dd;
        if (c.lj) {
          double d6 = dd * dd * dd, d12 = d6 * d6;
          e0 = e0 + c.aa * d12 + c.bb * d6;
          f0 = f0 + dd * (c.aa * 12.0 * d12 + c.bb * 6.0 * d6);
        }
      } else {
        double d6 = dd * dd * dd, d12 = d6 * d6;
        e0 = c.aa * d12 + c.bb * d6;
        f0 = dd * (c.aa * 12.0 * d12 + c.bb * 6.0 * d6);
      }
      double fxv = dx * f0, fyv = dy * f0, fzv = dz * f0;
      double* a = &fi[(k * nsi + c.si) * 3];
      double* b = &fj[(k * nsj + c.sj) * 3];
      a[0] += fxv; a[1] += fyv; a[2] += fzv;
      b[0] += fxv; b[1] += fyv; b[2] += fzv;
      e += e0;
    }
    ep[k] = e;
  }
  const int lasti = nsi - 1, lastj = nsj - 1;
  for (size_t k = 0; k < np; ++k) {
    double hh = P.hh[k];
    for (int l = 0; l < nsi; ++l)
      for (int c = 0; c < 3; ++c) fi[(k * nsi + l) * 3 + c] *= hh;
    for (int l = 0; l < nsj; ++l)
      for (int c = 0; c < 3; ++c) fj[(k * nsj + l) * 3 + c] *= hh;
    int ii = offi + P.i[k] * nsi, jj = offj + P.j[k] * nsj;
    double dx00 = S.x[ii + lasti] - S.x[jj + lastj] - P.ox[k];
    double dy00 = S.y[ii + lasti] - S.y[jj + lastj] - P.oy[k];
    double dz00 = S.z[ii + lasti] - S.z[jj + lastj] - P.oz[k];
    double dh = P.dh[k];
    double dhx = dh * dx00 * ep[k], dhy = dh * dy00 * ep[k], dhz = dh * dz00 * ep[k];
    double* a = &fi[(k * nsi + lasti) * 3];
    double* b = &fj[(k * nsj + lastj) * 3];
    a[0] += dhx; a[1] += dhy; a[2] += dhz;
    b[0] += dhx; b[1] += dhy; b[2] += dhz;
  }
  for (int l = 0; l < nsi; ++l)
    for (size_t k = 0; k < np; ++k) {
      int ii = offi + P.i[k] * nsi + l;
      S.fx[ii] += fi[(k * nsi + l) * 3]; S.fy[ii] += fi[(k * nsi + l) * 3 + 1]; S.fz[ii] += fi[(k * nsi + l) * 3 + 2];
    }
  for (int l = 0; l < nsj; ++l)
    for (size_t k = 0; k < np; ++k) {
      int jj = offj + P.j[k] * nsj + l;
      S.fx[jj] -= fj[(k * nsj + l) * 3]; S.fy[jj] -= fj[(k * nsj + l) * 3 + 1]; S.fz[jj] -= fj[(k * nsj + l) * 3 + 2];
    }
  for (size_t k = 0; k < np; ++k) ep[k] = ep[k] * P.hh[k];
  for (int c = 0; c < 9; ++c) vrmat[c] = 0;
  for (size_t k = 0; k < np; ++k) {
    int ii = offi + P.i[k] * nsi, jj = offj + P.j[k] * nsj;
    double d00[3] = {S.x[ii + lasti] - S.x[jj + lastj] - P.ox[k], S.y[ii + lasti] - S.y[jj + lastj] - P.oy[k],
                     S.z[ii + lasti] - S.z[jj + lastj] - P.oz[k]};
    double vr[3] = {0, 0, 0};
    for (int l = 0; l < nsi; ++l)
      for (int c = 0; c < 3; ++c) vr[c] += fi[(k * nsi + l) * 3 + c];
    // vrmat(a,b) += d00(a) * vr(b); stored row-major [a][b]
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) vrmat[3 * a + b] += d00[a] * vr[b];
  }
}

void std_force(const Model& m, const SiteArrays& S, const Pairs& P, double* ep, double vrmat[9], double scale) {
  table_force(m.nsite, m.nsite, std_table(m, scale), S, 0, 0, P, ep, vrmat);
}

// StdPairPotential StdInteraction.F90:633-762
void std_pairpot(const Model& m, const double* x, const double* y, const double* z, const Pairs& P, double* ep,
                 double scale) {
  const int ns = m.nsite;
  auto tab = std_table(m, scale);
  for (size_t k = 0; k < P.i.size(); ++k) {
    int ii = P.i[k] * ns, jj = P.j[k] * ns;
    double e = 0;
    for (const auto& c : tab) {
      double dx = x[ii + c.si] - x[jj + c.sj], dy = y[ii + c.si] - y[jj + c.sj], dz = z[ii + c.si] - z[jj + c.sj];
      dx = dx - P.ox[k]; dy = dy - P.oy[k]; dz = dz - P.oz[k];
      double dd = 1.0 / (dx * dx + dy * dy + dz * dz);
      double e0 = 0;
      if (c.coul) {
        e0 = c.qq * std::sqrt(dd);
        if (c.lj) { double d6 = dd * dd * dd; e0 = e0 + c.aa * d6 * d6 + c.bb * d6; }
      } else {
        double d6 = dd * dd * dd; e0 = c.aa * d6 * d6 + c.bb * d6;
      }
      e += e0;
    }
    ep[k] = e * P.hh[k];
  }
}

// Hand-unrolled TIP4P kernel, interaction_force_tip4p TIP4PModule.F90:102-785
// (non-TEST12, non-VPOPTIMIZE): site-pair order MM, MH, MH, HM, HM, HH x4, OO.
void tip4p_force(const SiteArrays& S, const Pairs& P, double* ep1, double vrmat[9]) {
  static const int order[10][2] = {{1, 1}, {1, 2}, {1, 3}, {2, 1}, {3, 1}, {2, 2}, {2, 3}, {3, 2}, {3, 3}, {0, 0}};
  const double qq[4][4] = {{0, 0, 0, 0}, {0, T4_WWMM, T4_WWMH, T4_WWMH}, {0, T4_WWMH, T4_WWHH, T4_WWHH},
                           {0, T4_WWMH, T4_WWHH, T4_WWHH}};
  for (int c = 0; c < 9; ++c) vrmat[c] = 0;
  for (size_t k = 0; k < P.i.size(); ++k) {
    int ii = P.i[k] * 5, jj = P.j[k] * 5;
    double dx00 = S.x[ii + 4], dy00 = S.y[ii + 4], dz00 = S.z[ii + 4];
    dx00 = dx00 - S.x[jj + 4]; dy00 = dy00 - S.y[jj + 4]; dz00 = dz00 - S.z[jj + 4];
    double ox = P.ox[k], oy = P.oy[k], oz = P.oz[k];
    dx00 = dx00 - ox; dy00 = dy00 - oy; dz00 = dz00 - oz;
    double hh = P.hh[k], dh = P.dh[k];
    double dhx = dh * dx00, dhy = dh * dy00, dhz = dh * dz00;
    double cx = -ox, cy = -oy, cz = -oz;
    double fi[5][3] = {{0}}, fj[5][3] = {{0}};
    double ep = 0;
    for (int t = 0; t < 10; ++t) {
      int a = order[t][0], b = order[t][1];
      double dx = S.x[ii + a] - S.x[jj + b] + cx, dy = S.y[ii + a] - S.y[jj + b] + cy, dz = S.z[ii + a] - S.z[jj + b] + cz;
      double dd = 1.0 / (dx * dx + dy * dy + dz * dz), e0, f0;
      if (a == 0) {
        double d6 = dd * dd * dd, d12 = d6 * d6;
        e0 = T4_AA * d12 + T4_BB * d6;
        f0 = dd * (T4_AA * 12.0 * d12 + T4_BB * 6.0 * d6);
      } else {
        double radiusi = std::sqrt(dd);
        e0 = qq[a][b] * radiusi;
        f0 = qq[a][b] * radiusi * dd;
      }
      ep = ep + e0;
      double fx = dx * f0, fy = dy * f0, fz = dz * f0;
      fi[a][0] += fx; fi[a][1] += fy; fi[a][2] += fz;
      fj[b][0] += fx; fj[b][1] += fy; fj[b][2] += fz;
    }
    for (int s = 0; s < 5; ++s)
      for (int c = 0; c < 3; ++c) { fi[s][c] *= hh; fj[s][c] *= hh; }
    dhx = dhx * ep; dhy = dhy * ep; dhz = dhz * ep;
    fi[4][0] += dhx; fi[4][1] += dhy; fi[4][2] += dhz;
    fj[4][0] += dhx; fj[4][1] += dhy; fj[4][2] += dhz;
    ep1[k] = ep * hh;
    double vrx = (fi[0][0] + fi[1][0] + fi[2][0] + fi[3][0] + fi[4][0]);
    double vry = (fi[0][1] + fi[1][1] + fi[2][1] + fi[3][1] + fi[4][1]);
    double vrz = (fi[0][2] + fi[1][2] + fi[2][2] + fi[3][2] + fi[4][2]);
    double d[3] = {dx00, dy00, dz00}, v[3] = {vrx, vry, vrz};
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) vrmat[3 * a + b] += d[a] * v[b];
    for (int s = 0; s < 5; ++s) {
      S.fx[ii + s] += fi[s][0]; S.fx[jj + s] -= fj[s][0];
      S.fy[ii + s] += fi[s][1]; S.fy[jj + s] -= fj[s][1];
      S.fz[ii + s] += fi[s][2]; S.fz[jj + s] -= fj[s][2];
    }
  }
}

// ST2 taper s12 and -s12'/r, ST2Module.F90:206-225
inline void st2_taper(double d12, double& s12, double& ds12) {
  const double rl = ST2_RL, ru = ST2_RU;
  if (d12 < ru * ru) {
    if (d12 < rl * rl) { s12 = 0; ds12 = 0; }
    else {
      double r12 = std::sqrt(d12);
      double w3 = (ru - rl) * (ru - rl) * (ru - rl);
      s12 = (r12 - rl) * (r12 - rl) * (3.0 * ru - rl - 2.0 * r12) / w3;
      ds12 = 6.0 * (r12 - rl) * (ru - r12) / w3;
      ds12 = -ds12 / r12;
    }
  } else { s12 = 1; ds12 = 0; }
}

// force_st2 ST2Module.F90:112-897 (non-VPOPTIMIZE).  Site order O,H,H,M,M,COM.
const int ST2_ORDER[17][2] = {{1, 1}, {1, 2}, {2, 1}, {2, 2}, {3, 3}, {3, 4}, {4, 3}, {4, 4}, {1, 3},
                              {1, 4}, {2, 3}, {2, 4}, {3, 1}, {3, 2}, {4, 1}, {4, 2}, {0, 0}};
inline double st2_qq(int a, int b) {
  const double QMM = ST2_QM * ST2_QM * COEFF * 100.0, QHM = ST2_QH * ST2_QM * COEFF * 100.0,
               QHH = ST2_QH * ST2_QH * COEFF * 100.0;
  bool ah = a <= 2, bh = b <= 2;
  return ah && bh ? QHH : (!ah && !bh ? QMM : QHM);
}
const double ST2_AA = 4.0 * ST2_EPS * pow12(ST2_SIG) * 100.0;
const double ST2_BB = -4.0 * ST2_EPS * pow6(ST2_SIG) * 100.0;

void st2_force(const SiteArrays& S, const Pairs& P, double* ep1, double vrmat[9]) {
  for (int c = 0; c < 9; ++c) vrmat[c] = 0;
  for (size_t k = 0; k < P.i.size(); ++k) {
    int ii = P.i[k] * 6, jj = P.j[k] * 6;
    double dx00 = S.x[ii + 5] - S.x[jj + 5], dy00 = S.y[ii + 5] - S.y[jj + 5], dz00 = S.z[ii + 5] - S.z[jj + 5];
    double ox = P.ox[k], oy = P.oy[k], oz = P.oz[k];
    dx00 = dx00 - ox; dy00 = dy00 - oy; dz00 = dz00 - oz;
    double hh = P.hh[k], dh = P.dh[k];
    double d12 = (dx00 * dx00 + dy00 * dy00 + dz00 * dz00), s12, ds12;
    st2_taper(d12, s12, ds12);
    double dhc = dh * s12 + hh * ds12, hhc = hh * s12;
    double dhcx = dhc * dx00, dhcy = dhc * dy00, dhcz = dhc * dz00;
    double dhx = dh * dx00, dhy = dh * dy00, dhz = dh * dz00;
    double cx = -ox, cy = -oy, cz = -oz;
    double fi[6][3] = {{0}}, fj[6][3] = {{0}};
    double ep = 0, eplj = 0;
    for (int t = 0; t < 17; ++t) {
      int a = ST2_ORDER[t][0], b = ST2_ORDER[t][1];
      double dx = S.x[ii + a] - S.x[jj + b] + cx, dy = S.y[ii + a] - S.y[jj + b] + cy, dz = S.z[ii + a] - S.z[jj + b] + cz;
      double dd = 1.0 / (dx * dx + dy * dy + dz * dz), f0;
      if (a == 0) {
        double d6 = dd * dd * dd, dd12 = d6 * d6;
        double e0 = ST2_AA * dd12 + ST2_BB * d6;
        f0 = dd * (ST2_AA * 12.0 * dd12 + ST2_BB * 6.0 * d6);
        eplj = e0;
      } else {
        double radiusi = std::sqrt(dd), q = st2_qq(a, b);
        double e0 = q * radiusi;
        f0 = q * radiusi * dd;
        ep = ep + e0;
      }
      double fx = dx * f0, fy = dy * f0, fz = dz * f0;
      fi[a][0] += fx; fi[a][1] += fy; fi[a][2] += fz;
      fj[b][0] += fx; fj[b][1] += fy; fj[b][2] += fz;
    }
    for (int s = 0; s < 6; ++s) {
      double sc = (s >= 1 && s <= 4) ? hhc : hh;
      for (int c = 0; c < 3; ++c) { fi[s][c] *= sc; fj[s][c] *= sc; }
    }
    dhx = dhx * eplj; dhy = dhy * eplj; dhz = dhz * eplj;
    dhcx = dhcx * ep; dhcy = dhcy * ep; dhcz = dhcz * ep;
    fi[5][0] = fi[5][0] + dhx + dhcx; fi[5][1] = fi[5][1] + dhy + dhcy; fi[5][2] = fi[5][2] + dhz + dhcz;
    fj[5][0] = fj[5][0] + dhx + dhcx; fj[5][1] = fj[5][1] + dhy + dhcy; fj[5][2] = fj[5][2] + dhz + dhcz;
    ep1[k] = ep * hhc + eplj * hh;
    double v[3] = {0, 0, 0};
    for (int c = 0; c < 3; ++c) v[c] = (fi[0][c] + fi[1][c] + fi[2][c] + fi[3][c] + fi[4][c] + fi[5][c]);
    double d[3] = {dx00, dy00, dz00};
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) vrmat[3 * a + b] += d[a] * v[b];
    for (int s = 0; s < 6; ++s) {
      S.fx[ii + s] += fi[s][0]; S.fx[jj + s] -= fj[s][0];
      S.fy[ii + s] += fi[s][1]; S.fy[jj + s] -= fj[s][1];
      S.fz[ii + s] += fi[s][2]; S.fz[jj + s] -= fj[s][2];
    }
  }
}

// pairpotential_st2 ST2Module.F90:900-1212
void st2_pairpot(const double* x, const double* y, const double* z, const Pairs& P, double* ep1) {
  for (size_t k = 0; k < P.i.size(); ++k) {
    int ii = P.i[k] * 6, jj = P.j[k] * 6;
    double dx00 = x[ii + 5] - x[jj + 5] - P.ox[k], dy00 = y[ii + 5] - y[jj + 5] - P.oy[k],
           dz00 = z[ii + 5] - z[jj + 5] - P.oz[k];
    double s12, ds12;
    st2_taper(dx00 * dx00 + dy00 * dy00 + dz00 * dz00, s12, ds12);
    double hh = P.hh[k], hhc = hh * s12, ep = 0, eplj = 0;
    for (int t = 0; t < 17; ++t) {
      int a = ST2_ORDER[t][0], b = ST2_ORDER[t][1];
      double dx = x[ii + a] - x[jj + b] - P.ox[k], dy = y[ii + a] - y[jj + b] - P.oy[k], dz = z[ii + a] - z[jj + b] - P.oz[k];
      double dd = 1.0 / (dx * dx + dy * dy + dz * dz);
      if (a == 0) { double d6 = dd * dd * dd; eplj = ST2_AA * d6 * d6 + ST2_BB * d6; }
      else ep = ep + st2_qq(a, b) * std::sqrt(dd);
    }
    ep1[k] = ep * hhc + eplj * hh;
  }
}

// Dispatcher `force` Interaction2.F90:19-68 restricted to this path: with
// `custom` (the reference's @FAST) TIP4P-TIP4P goes to the hand kernel and
// ST2-ST2 to force_st2; everything else (TIP5P, or custom == false) runs
// StdForce.
void force_dispatch(const Model& m, int path, const SiteArrays& S, const Pairs& P, double* ep, double vr[9]) {
  if (path == P_CUSTOM && m.id == M_TIP4P) tip4p_force(S, P, ep, vr);
  else if (path == P_CUSTOM && m.id == M_ST2) st2_force(S, P, ep, vr);
  else std_force(m, S, P, ep, vr, 1.0);
}

// PairPotential Interaction2.F90:71-121 (TIP4P custom calls the force kernel).
void pairpot_dispatch(const Model& m, int path, const double* x, const double* y, const double* z, const Pairs& P,
                      double* ep) {
  if (path == P_CUSTOM && m.id == M_TIP4P) {
    // Same arithmetic as the force kernel; the side-effect site forces go to scratch.
    int nmax = 0;
    for (size_t k = 0; k < P.i.size(); ++k) nmax = std::max(nmax, std::max(P.i[k], P.j[k]) + 1);
    std::vector<double> fx(5 * (size_t)nmax, 0.0), fy(fx), fz(fx);
    SiteArrays S{x, y, z, fx.data(), fy.data(), fz.data()};
    double vr[9];
    tip4p_force(S, P, ep, vr);
  } else if (path == P_CUSTOM && m.id == M_ST2) {
    st2_pairpot(x, y, z, P, ep);
  } else {
    std_pairpot(m, x, y, z, P, ep, 1.0);
  }
}

// rigid_collectforce RigidModule.F90:275-317 (serial branch)
void collectforce(const Model& m, int n, const double* intra, const double* tmat, const double* fx, const double* fy,
                  const double* fz, double* F, double* tau) {
  for (int i = 0; i < n; ++i) {
    double tx = 0, ty = 0, tz = 0, sx = 0, sy = 0, sz = 0;
    for (int s = 0; s < m.nsite; ++s) {
      int k = i * m.nsite + s;
      const double* r = intra + 3 * k;
      sx = sx + fx[k]; sy = sy + fy[k]; sz = sz + fz[k];
      tx = tx + r[1] * fz[k] - r[2] * fy[k];
      ty = ty + r[2] * fx[k] - r[0] * fz[k];
      tz = tz + r[0] * fy[k] - r[1] * fx[k];
    }
    const double* t = tmat + 9 * i;
    F[3 * i] = sx; F[3 * i + 1] = sy; F[3 * i + 2] = sz;
    tau[3 * i] = t[0] * tx + t[3] * ty + t[6] * tz;
    tau[3 * i + 1] = t[1] * tx + t[4] * ty + t[7] * tz;
    tau[3 * i + 2] = t[2] * tx + t[5] * ty + t[8] * tz;
  }
}

// ---------------------------------------------------------------------------
// Rigid-body state and Gear predictor-corrector
// Per-molecule record (53 doubles): com[3], d[5][3], w[5][3], q[5][4]
//   d[k] = dx(k+1), w[k] = wx(k+1), q[k] = quat(k+1)  (RigidModule.F90:14-24)
// ---------------------------------------------------------------------------
const int REC = 53;
inline double* R_com(double* r) { return r; }
inline double* R_d(double* r, int k) { return r + 3 + 3 * k; }
inline double* R_w(double* r, int k) { return r + 18 + 3 * k; }
inline double* R_q(double* r, int k) { return r + 33 + 4 * k; }

// rigid_predict RigidModule.F90:480-559
void rigid_predict(double* r) {
  double* c = R_com(r);
  for (int a = 0; a < 3; ++a) {
    double d1 = R_d(r, 0)[a], d2 = R_d(r, 1)[a], d3 = R_d(r, 2)[a], d4 = R_d(r, 3)[a], d5 = R_d(r, 4)[a];
    c[a] = c[a] + d1 + d2 + d3 + d4 + d5;
    R_d(r, 0)[a] = d1 + 2.0 * d2 + 3.0 * d3 + 4.0 * d4 + 5.0 * d5;
    R_d(r, 1)[a] = d2 + 3.0 * d3 + 6.0 * d4 + 10.0 * d5;
    R_d(r, 2)[a] = d3 + 4.0 * d4 + 10.0 * d5;
    R_d(r, 3)[a] = d4 + 5.0 * d5;
  }
  for (int a = 0; a < 3; ++a) {
    double w1 = R_w(r, 0)[a], w2 = R_w(r, 1)[a], w3 = R_w(r, 2)[a], w4 = R_w(r, 3)[a], w5 = R_w(r, 4)[a];
    R_w(r, 0)[a] = w1 + w2 + w3 + w4 + w5;
    R_w(r, 1)[a] = w2 + 2.0 * w3 + 3.0 * w4 + 4.0 * w5;
    R_w(r, 2)[a] = w3 + 3.0 * w4 + 6.0 * w5;
    R_w(r, 3)[a] = w4 + 4.0 * w5;
  }
  for (int a = 0; a < 4; ++a) {
    double q1 = R_q(r, 0)[a], q2 = R_q(r, 1)[a], q3 = R_q(r, 2)[a], q4 = R_q(r, 3)[a], q5 = R_q(r, 4)[a];
    R_q(r, 0)[a] = q1 + q2 + q3 + q4 + q5;
    R_q(r, 1)[a] = q2 + 2.0 * q3 + 3.0 * q4 + 4.0 * q5;
  }
  double* q = R_q(r, 0);
  double re = 1.0 / std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  for (int a = 0; a < 4; ++a) q[a] = q[a] * re;
}

// q-derivative (1/2) W(w) q, the common pattern in RigidModule.F90:1337-1348, 1389-1404
inline void qdot(const double* w, const double* q, double out[4]) {
  out[0] = (-w[0] * q[1] + w[1] * q[2] - w[2] * q[3]);
  out[1] = (w[0] * q[0] - w[1] * q[3] - w[2] * q[2]);
  out[2] = (-w[0] * q[3] - w[1] * q[0] + w[2] * q[1]);
  out[3] = (w[0] * q[2] + w[1] * q[1] + w[2] * q[0]);
}

struct Thermo {            // Nose (NoseModule.F90:3-10) plus friction inputs of rigid_correct
  int nose_active = 0;
  double q = 0, dump = 0, temp = 0;
  double z0 = 0, z1 = 0, z2 = 0, z3 = 0, z4 = 0, zsum = 0;
};

// rigid_correct RigidModule.F90:1255-1487 (Nose friction only; the Andersen
// barostat branch :1285-1296 is out of this path).
void rigid_correct(const Model& m, double* r, const double* F, const double* tau, double dt, const Thermo& th) {
  double ext_t = 0, ext_r = 0;
  if (th.nose_active) {
    double nc = th.z0 * dt;
    ext_t = ext_t + nc * 0.5;
    ext_r = ext_r + nc;
  }
  double massi = 1.0 / m.mass;
  double* c = R_com(r);
  for (int a = 0; a < 3; ++a) {
    double nf = F[a] * (dt * dt * 0.5 * massi);
    nf = nf - R_d(r, 0)[a] * ext_t;
    double delta = nf - R_d(r, 1)[a];
    c[a] = c[a] + GEAR5_0 * delta;
    R_d(r, 0)[a] = R_d(r, 0)[a] + GEAR5_1 * delta;
    R_d(r, 1)[a] = nf;
    R_d(r, 2)[a] = R_d(r, 2)[a] + GEAR5_3 * delta;
    R_d(r, 3)[a] = R_d(r, 3)[a] + GEAR5_4 * delta;
    R_d(r, 4)[a] = R_d(r, 4)[a] + GEAR5_5 * delta;
  }
  double* q1 = R_q(r, 0);
  double* w1 = R_w(r, 0);
  double nw[4];
  qdot(w1, q1, nw);
  for (int a = 0; a < 4; ++a) nw[a] = nw[a] * dt * 0.5;
  for (int a = 0; a < 4; ++a) {
    double dw = nw[a] - R_q(r, 1)[a];
    q1[a] = q1[a] + GEAR4_0 * dw;
  }
  double I[3] = {m.Ixx, m.Iyy, m.Izz}, Ii[3] = {1.0 / m.Ixx, 1.0 / m.Iyy, 1.0 / m.Izz};
  double nf[3];
  nf[0] = (tau[0] + (I[1] - I[2]) * w1[1] * w1[2]) * dt * Ii[0];
  nf[1] = (tau[1] + (I[2] - I[0]) * w1[2] * w1[0]) * dt * Ii[1];
  nf[2] = (tau[2] + (I[0] - I[1]) * w1[0] * w1[1]) * dt * Ii[2];
  for (int a = 0; a < 3; ++a) {
    nf[a] = nf[a] - w1[a] * ext_r;
    double delta = nf[a] - R_w(r, 1)[a];
    R_w(r, 0)[a] = R_w(r, 0)[a] + GEAR4_0 * delta;
    R_w(r, 1)[a] = nf[a];
    R_w(r, 2)[a] = R_w(r, 2)[a] + GEAR4_2 * delta;
    R_w(r, 3)[a] = R_w(r, 3)[a] + GEAR4_3 * delta;
    R_w(r, 4)[a] = R_w(r, 4)[a] + GEAR4_4 * delta;
  }
  // quaternion derivative stacks rebuilt from the corrected w stacks (:1389-1486)
  double t[4], u[4];
  qdot(R_w(r, 0), q1, t);
  for (int a = 0; a < 4; ++a) R_q(r, 1)[a] = t[a] * dt * 0.5;
  qdot(R_w(r, 1), q1, t); qdot(R_w(r, 0), R_q(r, 1), u);
  for (int a = 0; a < 4; ++a) R_q(r, 2)[a] = (t[a] + u[a]) * dt * 0.25;
  {
    double v[4];
    qdot(R_w(r, 2), q1, t); qdot(R_w(r, 0), R_q(r, 2), u); qdot(R_w(r, 1), R_q(r, 1), v);
    for (int a = 0; a < 4; ++a) R_q(r, 3)[a] = (t[a] + u[a] + v[a]) * dt * (1.0 / 6.0);
  }
  {
    double v[4], x[4];
    qdot(R_w(r, 3), q1, t); qdot(R_w(r, 2), R_q(r, 1), u); qdot(R_w(r, 1), R_q(r, 2), v); qdot(R_w(r, 0), R_q(r, 3), x);
    for (int a = 0; a < 4; ++a) R_q(r, 4)[a] = (t[a] + u[a] + v[a] + x[a]) * dt * (1.0 / 8.0);
  }
}

// Nose_Predict NoseModule.F90:74-87, Nose_Correct :43-72
void nose_predict(Thermo& n) {
  n.z0 = n.z0 + n.z1 + n.z2 + n.z3 + n.z4;
  n.z1 = n.z1 + 2.0 * n.z2 + 3.0 * n.z3 + 4.0 * n.z4;
  n.z2 = n.z2 + 3.0 * n.z3 + 6.0 * n.z4;
  n.z3 = n.z3 + 4.0 * n.z4;
}
void nose_correct(Thermo& n, double temp) {
  double zetaf = (temp - n.temp) / n.q - n.dump * n.z0;
  double dz2 = zetaf - n.z1;
  n.z0 = n.z0 + GEAR4_0 * dz2;
  n.z1 = zetaf;
  n.z2 = n.z2 + GEAR4_2 * dz2;
  n.z3 = n.z3 + GEAR4_3 * dz2;
  n.z4 = n.z4 + GEAR4_4 * dz2;
  n.zsum = n.zsum + n.z0;
}

// Rigid_Ek RigidModule.F90:576-597; Rigid_PressureTensor :599-619
void rigid_ek(const Model& m, int n, const double* rec, double dt, double& ekt, double& ekr, double pk[9]) {
  double ex = 0, ey = 0, ez = 0;
  ekt = 0;
  for (int c = 0; c < 9; ++c) pk[c] = 0;
  for (int i = 0; i < n; ++i) {
    const double* r = rec + (size_t)REC * i;
    const double* d1 = r + 3;
    const double* w1 = r + 18;
    ekt = ekt + d1[0] * d1[0] + d1[1] * d1[1] + d1[2] * d1[2];
    ex = ex + w1[0] * w1[0]; ey = ey + w1[1] * w1[1]; ez = ez + w1[2] * w1[2];
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) pk[3 * a + b] = pk[3 * a + b] + d1[a] * d1[b];
  }
  ekr = (ex * m.Ixx + ey * m.Iyy + ez * m.Izz) * 0.5;
  ekt = ekt * m.mass * 0.5 * (1.0 / (dt * dt));
  for (int c = 0; c < 9; ++c) pk[c] = pk[c] * m.mass * (1.0 / (dt * dt));
}

// One complete force evaluation as the MD loop performs it (Mixture.F90:1850-2044):
// sites -> grid -> neighbour list -> compress -> switch -> force -> collect.
struct ForceOut {
  double epot = 0, vir[9] = {0};
  long npair = 0;
};
void full_force(const Model& m, int path, int n, const double* com, const double* quat, const double L[3],
                const double req[3], double rin, double rc, double* F, double* tau, ForceOut& out,
                std::vector<int>* cells_out = nullptr, Pairs* pairs_out = nullptr) {
  const size_t ns = m.nsite;
  std::vector<double> sx(n * ns), sy(n * ns), sz(n * ns), intra(n * ns * 3), tmat(9 * (size_t)n);
  place_sites(m, n, com, quat, sx.data(), sy.data(), sz.data(), intra.data(), tmat.data());
  Grid g;
  std::vector<int> cells;
  Pairs P;
  pairsearch(n, com, L, req, rc, g, cells, P);
  cutoff_dimmer2(rin, rc, com, com, P);
  std::vector<double> fx(n * ns, 0.0), fy(n * ns, 0.0), fz(n * ns, 0.0), ep(P.i.size());
  SiteArrays S{sx.data(), sy.data(), sz.data(), fx.data(), fy.data(), fz.data()};
  force_dispatch(m, path, S, P, ep.data(), out.vir);
  out.epot = 0;
  for (double e : ep) out.epot += e;
  out.npair = (long)P.i.size();
  collectforce(m, n, intra.data(), tmat.data(), fx.data(), fy.data(), fz.data(), F, tau);
  if (cells_out) *cells_out = cells;
  if (pairs_out) *pairs_out = P;
}

// ---------------------------------------------------------------------------
// Threaded force for the CPU-baseline timing: same physics as force_dispatch
// (StdForce arithmetic), pairs split across OpenMP threads with private
// site-force buffers.  Used only to time the CPU side.
// ---------------------------------------------------------------------------
void std_force_threaded(const Model& m, const double* x, const double* y, const double* z, const Pairs& P,
                        double* fx, double* fy, double* fz, double& epot, double vir[9], int nthreads, int nsites) {
  auto tab = std_table(m, 1.0);
  const int ns = m.nsite, last = ns - 1;
  const long np = (long)P.i.size();
  double etot = 0, v[9] = {0};
#pragma omp parallel num_threads(nthreads) reduction(+ : etot)
  {
    std::vector<double> lf((size_t)nsites * 3, 0.0);
    double lv[9] = {0};
#pragma omp for schedule(static)
    for (long k = 0; k < np; ++k) {
      int ii = P.i[k] * ns, jj = P.j[k] * ns;
      double fi[MAXS][3] = {{0}}, fj[MAXS][3] = {{0}}, e = 0;
      for (const auto& c : tab) {
        double dx = x[ii + c.si] - x[jj + c.sj] - P.ox[k], dy = y[ii + c.si] - y[jj + c.sj] - P.oy[k],
               dz = z[ii + c.si] - z[jj + c.sj] - P.oz[k];
        double dd = 1.0 / (dx * dx + dy * dy + dz * dz), e0 = 0, f0 = 0;
        if (c.coul) { double ri = std::sqrt(dd); e0 = c.qq * ri; f0 = c.qq * ri * dd; }
        if (c.lj) { double d6 = dd * dd * dd, d12 = d6 * d6; e0 += c.aa * d12 + c.bb * d6; f0 += dd * (c.aa * 12.0 * d12 + c.bb * 6.0 * d6); }
        fi[c.si][0] += dx * f0; fi[c.si][1] += dy * f0; fi[c.si][2] += dz * f0;
        fj[c.sj][0] += dx * f0; fj[c.sj][1] += dy * f0; fj[c.sj][2] += dz * f0;
        e += e0;
      }
      double hh = P.hh[k], dh = P.dh[k];
      double d00[3] = {x[ii + last] - x[jj + last] - P.ox[k], y[ii + last] - y[jj + last] - P.oy[k],
                       z[ii + last] - z[jj + last] - P.oz[k]};
      double vr[3] = {0, 0, 0};
      for (int s = 0; s < ns; ++s)
        for (int c = 0; c < 3; ++c) {
          fi[s][c] *= hh; fj[s][c] *= hh;
          if (s == last) { fi[s][c] += dh * d00[c] * e; fj[s][c] += dh * d00[c] * e; }
          vr[c] += fi[s][c];
          lf[(size_t)(ii + s) * 3 + c] += fi[s][c];
          lf[(size_t)(jj + s) * 3 + c] -= fj[s][c];
        }
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) lv[3 * a + b] += d00[a] * vr[b];
      etot += e * hh;
    }
#pragma omp critical
    {
      for (int s = 0; s < nsites; ++s) { fx[s] += lf[3 * s]; fy[s] += lf[3 * s + 1]; fz[s] += lf[3 * s + 2]; }
      for (int c = 0; c < 9; ++c) v[c] += lv[c];
    }
  }
  epot = etot;
  for (int c = 0; c < 9; ++c) vir[c] = v[c];
}


// ---------------------------------------------------------------------------
// Order parameters of umbrella Monte Carlo (mc2.F90:505-520, 684-705):
// OP_Q6T (Q6Local.F90 sq6system_prepareall :98-223), OP_TRIANGLE
// (Triangle.F90 sTriangle_prepareall :53-100), each computed from scratch
// for a configuration -- the value the reference's incremental
// Differentiate/Integrate must reproduce (its own DEBUG3 check, mc2.F90:745-760).
// ---------------------------------------------------------------------------
// Separation of molecule b seen from a, as neighbors_all2 stores it
// (Neighbor.F90:85-130): dx = ca - cb - o with the Compress2 image o, the
// entry of nei(a) holds -dx; returns dd = dx^2 + dy^2 + dz^2.
inline double nb_vec(const double* a, const double* b, const double L[3], const double iL[3], double v[3]) {
  double d[3];
  for (int k = 0; k < 3; ++k) {
    const double delta = a[k] - b[k];
    const double o = dnint(delta * iL[k]) * L[k];
    d[k] = delta - o;
    v[k] = -d[k];
  }
  return d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
}

struct NbEntry { int j; double v[3]; double dd; };

// Neighbours of every molecule with dd <= radius^2 (the reference's
// `radius**2 < dd` rejection), ordered by label (ORDER_BY_LABEL).
std::vector<std::vector<NbEntry>> neighbours_within(int n, const double* com, const double L[3], double radius) {
  const double iL[3] = {1.0 / L[0], 1.0 / L[1], 1.0 / L[2]};
  std::vector<std::vector<NbEntry>> nb(n);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      if (j == i) continue;
      NbEntry e;
      e.j = j;
      e.dd = nb_vec(com + 3 * i, com + 3 * j, L, iL, e.v);
      if (!(radius * radius < e.dd)) nb[i].push_back(e);
    }
  return nb;
}

// Associated Legendre function P_l^m(x), 0 <= m <= l (the upward recurrence of
// q6.F90 plgndr :69-100).
double legendre_plm(int l, int m, double x) {
  double pmm = 1.0;
  if (m > 0) {
    const double somx2 = std::sqrt((1.0 - x) * (1.0 + x));
    double fact = 1.0;
    for (int i = 1; i <= m; ++i) { pmm = -pmm * fact * somx2; fact = fact + 2.0; }
  }
  if (l == m) return pmm;
  double pmmp1 = x * (2 * m + 1) * pmm;
  if (l == m + 1) return pmmp1;
  double pll = 0.0;
  for (int ll = m + 2; ll <= l; ++ll) {
    pll = (x * (2 * ll - 1) * pmmp1 - (ll + m - 1) * pmm) / (ll - m);
    pmm = pmmp1;
    pmmp1 = pll;
  }
  return pll;
}

struct Cplx { double re, im; };
inline Cplx cmul(Cplx a, Cplx b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }

// q_6m of a bond along (x, y, z), |(x,y,z)| = 1: the spherical harmonic Y_6m
// with cos(theta) = z and e^{i phi} = (x + iy)/sqrt(x^2 + y^2) (q6.F90 qlm,
// ylm2, ylm :24-66), m = -6..6 at index m + 6.
void q6_of_bond(double x, double y, double z, Cplx out[13]) {
  static const double fact[13] = {1.0, 1.0, 2.0, 6.0, 24.0, 120.0, 720.0, 5040.0, 40320.0, 362880.0, 3628800.0,
                                  39916800.0, 479001600.0};
  const double rxy = std::sqrt(x * x + y * y);
  const Cplx w = {x / rxy, y / rxy};
  Cplx wm = {1.0, 0.0};
  for (int m = 0; m <= 6; ++m) {
    if (m > 0) wm = cmul(wm, w);
    const double norm = std::sqrt((2.0 * 6 + 1.0) * fact[6 - m] / (4.0 * PI * fact[6 + m]));
    const double p = norm * legendre_plm(6, m, z);
    const Cplx y6 = {p * wm.re, p * wm.im};
    out[6 + m] = y6;
    if (m > 0) {
      const double sg = (m & 1) ? -1.0 : 1.0;   // Y_{6,-m} = (-1)^m conj(Y_6m)
      out[6 - m] = {sg * y6.re, -sg * y6.im};
    }
  }
}

// Local Q6 (sq6system_prepareall): bonds are pairs within 3 A, the
// neighbourhood of a molecule is itself plus the molecules within 5 A, and
// q6(k) = sqrt(4 pi / 13 sum_m |sum q_6m(b)|^2) / nbond(k) over the directed
// bonds b = (i -> j) with both i and j in k's neighbourhood; the order
// parameter is the mean of q6 over the molecules.
double op_q6(int n, const double* com, const double L[3], double* q6out) {
  auto nei5 = neighbours_within(n, com, L, 5.0);
  auto in5 = [&](int k, int j) {
    if (j == k) return true;
    for (const NbEntry& e : nei5[k]) if (e.j == j) return true;
    return false;
  };
  std::vector<std::array<Cplx, 13>> qsum(n);
  std::vector<int> nbond(n, 0);
  for (auto& q : qsum) for (auto& c : q) c = {0.0, 0.0};
  for (int i = 0; i < n; ++i)
    for (const NbEntry& b : nei5[i]) {
      if (9.0 < b.dd) continue;   // nei3: bonds within 3 A
      const double pp = 1.0 / std::sqrt(b.dd);
      Cplx q[13];
      q6_of_bond(b.v[0] * pp, b.v[1] * pp, b.v[2] * pp, q);
      // neib = neis(i) ^ neis(j): k = i, j and the common neighbours
      std::vector<int> ks = {i};
      for (const NbEntry& e : nei5[i]) if (in5(b.j, e.j)) ks.push_back(e.j);
      for (int k : ks) {
        nbond[k] += 1;
        for (int m = 0; m < 13; ++m) { qsum[k][m].re += q[m].re; qsum[k][m].im += q[m].im; }
      }
    }
  double sum = 0.0;
  for (int k = 0; k < n; ++k) {
    double s2 = 0.0;
    for (int m = 0; m < 13; ++m) {
      const double a = std::hypot(qsum[k][m].re, qsum[k][m].im);
      s2 = s2 + a * a;
    }
    const double q6 = std::sqrt(s2 * 4.0 * PI / (2.0 * 6 + 1.0)) / nbond[k];
    if (q6out) q6out[k] = q6;
    sum = sum + q6;
  }
  return sum / n;
}

// Histogram bin (DistribModule.F90 histogram_accumulate): nint((x - min) /
// width) + 1, kept when 1 <= bin <= nbin; 0-based here, -1 when outside.
inline int tri_bin(double costh) {
  const int bin = (int)dnint((costh - (-1.0)) / 0.1);
  return (bin >= 0 && bin < 21) ? bin : -1;
}

// kullback_div (DistribModule.F90:304-326) of counts h against the reference
// histogram ref (21 bins each).
double kullback(const double* h, const double* ref) {
  double s1 = 0.0, s2 = 0.0;
  for (int i = 0; i < 21; ++i) { s1 = s1 + h[i]; s2 = s2 + ref[i]; }
  double div = 0.0;
  for (int i = 0; i < 21; ++i) {
    const double p = h[i] / s1;
    double q = ref[i] / s2;
    if (q == 0) q = p;
    if (p != 0) div = div + p * std::log(p / q);
  }
  return div;
}

// Triangle order parameter (sTriangle_prepareall): for every molecule its (at
// most) 4 nearest neighbours within 5 A, the cosines of the 6 angles they
// span at the molecule in a 21-bin histogram on [-1, 1], and the Kullback
// divergence of that histogram from ref (its log when logarithmic).  Equal
// distances are ordered by label.
double op_triangle(int n, const double* com, const double L[3], const double* ref, int logarithmic, double* hist) {
  auto nei = neighbours_within(n, com, L, 5.0);
  double h[21] = {0.0};
  for (int i = 0; i < n; ++i) {
    std::vector<NbEntry>& v = nei[i];
    std::stable_sort(v.begin(), v.end(), [](const NbEntry& a, const NbEntry& b) { return a.dd < b.dd; });
    const int m = std::min<int>(4, (int)v.size());
    for (int a = 0; a < m; ++a)
      for (int b = a + 1; b < m; ++b) {
        double c = v[a].v[0] * v[b].v[0] + v[a].v[1] * v[b].v[1] + v[a].v[2] * v[b].v[2];
        c = c / std::sqrt(v[a].dd * v[b].dd);
        const int bin = tri_bin(c);
        if (bin >= 0) h[bin] = h[bin] + 1.0;
      }
  }
  if (hist) for (int i = 0; i < 21; ++i) hist[i] = h[i];
  double op = kullback(h, ref);
  if (logarithmic) op = std::log(op);
  return op;
}

}  // namespace

// ===========================================================================
// C ABI for the Python test harness (ctypes).  Arrays are row-major:
// com (n,3), quat (n,4), rec (n,53), F/tau (n,3), sites (n*nsite).
// ===========================================================================
extern "C" {

int orc_model_info(int model, int* nsite, double* body /*nsite*3*/, double* param /*nsite*3: q,eps,sig*/,
                   double* mass_inertia /*4*/) {
  Model m;
  if (!make_model(model, m)) return 1;
  *nsite = m.nsite;
  for (int s = 0; s < m.nsite; ++s) {
    body[3 * s] = m.molx[s]; body[3 * s + 1] = m.moly[s]; body[3 * s + 2] = m.molz[s];
    param[3 * s] = m.q[s]; param[3 * s + 1] = m.eps[s]; param[3 * s + 2] = m.sig[s];
  }
  mass_inertia[0] = m.mass; mass_inertia[1] = m.Ixx; mass_inertia[2] = m.Iyy; mass_inertia[3] = m.Izz;
  return 0;
}

// Physical constants used by the harness (same values as above).
void orc_constants(double* out /*12*/) {
  out[0] = PI; out[1] = NA; out[2] = KB; out[3] = RGAS; out[4] = COEFF; out[5] = I2J;
  out[6] = J2I; out[7] = J2K; out[8] = KX2X; out[9] = P2A; out[10] = ANG2M; out[11] = X2KX;
}

void orc_place_sites(int model, int n, const double* com, const double* quat, double* sx, double* sy, double* sz,
                     double* intra, double* tmat) {
  Model m;
  make_model(model, m);
  place_sites(m, n, com, quat, sx, sy, sz, intra, tmat);
}

int orc_grid(const double* L, const double* req, int* ndiv, double* cell, int* nn, int* nn0, int* stencil /*27*3*/) {
  Grid g;
  grid_update(g, L, req);
  for (int d = 0; d < 3; ++d) { ndiv[d] = g.nd[d]; cell[d] = g.cell[d]; }
  *nn = (int)g.n.size() / 3; *nn0 = (int)g.n0.size() / 3;
  int k = 0;
  for (int v : g.n) stencil[k++] = v;
  for (int v : g.n0) stencil[k++] = v;
  return 0;
}

// Cell assignment (0-based ids) and the exact within-cutoff pair set.
// Returns the pair count; when it exceeds cap nothing beyond cap is written.
long orc_pairsearch(int n, const double* com, const double* L, const double* req, double rin, double rc, int* cell,
                    long cap, int* pi, int* pj, double* ox, double* oy, double* oz, double* hh, double* dh) {
  Grid g;
  std::vector<int> cells;
  Pairs P;
  pairsearch(n, com, L, req, rc, g, cells, P);
  cutoff_dimmer2(rin, rc, com, com, P);
  if (cell) for (int i = 0; i < n; ++i) cell[i] = cells[i];
  long np = (long)P.i.size();
  for (long k = 0; k < np && k < cap; ++k) {
    pi[k] = P.i[k]; pj[k] = P.j[k]; ox[k] = P.ox[k]; oy[k] = P.oy[k]; oz[k] = P.oz[k]; hh[k] = P.hh[k]; dh[k] = P.dh[k];
  }
  return np;
}

// The reference `force` call on an explicit pair list (Interaction2.F90:19):
// site forces are ACCUMULATED into fx/fy/fz, ep (per pair) and vrmat are outputs.
int orc_force_sites(int model, int path, int nsites_total, const double* x, const double* y, const double* z,
                    double* fx, double* fy, double* fz, long npair, const int* pi, const int* pj, const double* ox,
                    const double* oy, const double* oz, const double* eratio, const double* fratio, double* ep,
                    double* vrmat) {
  Model m;
  if (!make_model(model, m)) return 1;
  (void)nsites_total;
  Pairs P;
  P.i.assign(pi, pi + npair); P.j.assign(pj, pj + npair);
  P.ox.assign(ox, ox + npair); P.oy.assign(oy, oy + npair); P.oz.assign(oz, oz + npair);
  P.hh.assign(eratio, eratio + npair); P.dh.assign(fratio, fratio + npair);
  SiteArrays S{x, y, z, fx, fy, fz};
  force_dispatch(m, path, S, P, ep, vrmat);
  return 0;
}

// Grid_NeighborList with the hetero stencil + Interaction_Compress2 +
// CutOff_Dimmer2 for components A (na COMs) and B (nb COMs) in one box:
// cell ids of both and the pairs (i in A, j in B).
long orc_pairsearch_hetero(int na, const double* ca, int nb, const double* cb, const double* L, const double* req,
                           double rin, double rc, int* cella, int* cellb, long cap, int* pi, int* pj, double* ox,
                           double* oy, double* oz, double* hh, double* dh) {
  std::vector<int> ia, ib;
  Pairs P;
  pairsearch_hetero(na, ca, nb, cb, L, req, rc, ia, ib, P);
  cutoff_dimmer2(rin, rc, ca, cb, P);
  if (cella) for (int i = 0; i < na; ++i) cella[i] = ia[i];
  if (cellb) for (int j = 0; j < nb; ++j) cellb[j] = ib[j];
  long np = (long)P.i.size();
  for (long k = 0; k < np && k < cap; ++k) {
    pi[k] = P.i[k]; pj[k] = P.j[k]; ox[k] = P.ox[k]; oy[k] = P.oy[k]; oz[k] = P.oz[k]; hh[k] = P.hh[k]; dh[k] = P.dh[k];
  }
  return np;
}

// The reference `force(iv, mi, mj, site, ...)` for two components (mi != mj,
// or a model with no hand kernel): one global site store, component i at site
// offset offi and j at offj (mi%offset, mj%offset); site forces ACCUMULATED.
int orc_force_sites_hetero(int model_i, int model_j, int path, const double* x, const double* y, const double* z,
                           double* fx, double* fy, double* fz, int offi, int offj, long npair, const int* pi,
                           const int* pj, const double* ox, const double* oy, const double* oz, const double* eratio,
                           const double* fratio, double* ep, double* vrmat) {
  Model mi, mj;
  if (!make_model(model_i, mi) || !make_model(model_j, mj)) return 1;
  Pairs P;
  P.i.assign(pi, pi + npair); P.j.assign(pj, pj + npair);
  P.ox.assign(ox, ox + npair); P.oy.assign(oy, oy + npair); P.oz.assign(oz, oz + npair);
  P.hh.assign(eratio, eratio + npair); P.dh.assign(fratio, fratio + npair);
  SiteArrays S{x, y, z, fx, fy, fz};
  table_force(mi.nsite, mj.nsite, pair_table2(mi, mj, path), S, offi, offj, P, ep, vrmat);
  return 0;
}

int orc_pair_potential(int model, int path, const double* x, const double* y, const double* z, long npair,
                       const int* pi, const int* pj, const double* ox, const double* oy, const double* oz,
                       const double* eratio, double* ep) {
  Model m;
  if (!make_model(model, m)) return 1;
  Pairs P;
  P.i.assign(pi, pi + npair); P.j.assign(pj, pj + npair);
  P.ox.assign(ox, ox + npair); P.oy.assign(oy, oy + npair); P.oz.assign(oz, oz + npair);
  P.hh.assign(eratio, eratio + npair); P.dh.assign(npair, 0.0);
  pairpot_dispatch(m, path, x, y, z, P, ep);
  return 0;
}

// Whole force path for one configuration: per-molecule F and body torque,
// total potential energy, 3x3 molecular virial (row a, column b = sum d00_a F_b).
long orc_compute(int model, int path, int n, const double* com, const double* quat, const double* L, const double* req,
                 double rin, double rc, double* F, double* tau, double* epot, double* vir) {
  Model m;
  if (!make_model(model, m)) return -1;
  ForceOut o;
  full_force(m, path, n, com, quat, L, req, rin, rc, F, tau, o);
  *epot = o.epot;
  for (int c = 0; c < 9; ++c) vir[c] = o.vir[c];
  return o.npair;
}

// Molecular dynamics, Mixture.F90:1789-2290 order.  rec is (n,53), updated in
// place.  thermo[10] = {nose_active, q_internal, dump, T0, z0, z1, z2, z3, z4, zsum}
// in/out.  log (nsteps, 8) per step: epot, ekt, ekr, T, P_kin+vir trace/3
// (internal), H (J/mol), npair, zeta0.
int orc_md_run(int model, int path, int n, double* rec, const double* L, const double* req, double rin, double rc,
               double dt, int nsteps, double* thermo, double* log) {
  Model m;
  if (!make_model(model, m)) return 1;
  Thermo th;
  th.nose_active = (int)thermo[0]; th.q = thermo[1]; th.dump = thermo[2]; th.temp = thermo[3];
  th.z0 = thermo[4]; th.z1 = thermo[5]; th.z2 = thermo[6]; th.z3 = thermo[7]; th.z4 = thermo[8]; th.zsum = thermo[9];
  const double dof = 6.0 * n;
  std::vector<double> com(3 * (size_t)n), quat(4 * (size_t)n), F(3 * (size_t)n), tau(3 * (size_t)n);
  double vol = L[0] * L[1] * L[2];
  for (int step = 0; step < nsteps; ++step) {
    for (int i = 0; i < n; ++i) rigid_predict(rec + (size_t)REC * i);
    if (th.nose_active) nose_predict(th);
    for (int i = 0; i < n; ++i) {
      std::memcpy(&com[3 * i], rec + (size_t)REC * i, 3 * sizeof(double));
      std::memcpy(&quat[4 * i], rec + (size_t)REC * i + 33, 4 * sizeof(double));
    }
    ForceOut o;
    full_force(m, path, n, com.data(), quat.data(), L, req, rin, rc, F.data(), tau.data(), o);
    for (int i = 0; i < n; ++i) rigid_correct(m, rec + (size_t)REC * i, &F[3 * i], &tau[3 * i], dt, th);
    double ekt, ekr, pk[9];
    rigid_ek(m, n, rec, dt, ekt, ekr, pk);
    double temperature = I2J * 2.0 * (ekt + ekr) / (RGAS * dof);
    double vp = pk[0] + pk[4] + pk[8] + o.vir[0] + o.vir[4] + o.vir[8];
    double pressure = (vp / 3.0) * I2J * P2A / (vol * NA * ANG2M * ANG2M * ANG2M);
    if (th.nose_active) nose_correct(th, temperature);
    // conserved quantity, Mixture.F90:2431-2453
    double nose_ek = 0, nose_ep = 0;
    if (th.nose_active) {
      nose_ek = (th.z0 * th.z0 * th.q * dt * dof * 0.5) * RGAS;
      nose_ep = (dof * th.temp * (th.zsum - 0.5 * th.z0) * dt) * RGAS;
    }
    double H = (o.epot + ekt + ekr) * I2J + nose_ep + nose_ek;
    if (log) {
      double* lg = log + 8 * (size_t)step;
      lg[0] = o.epot; lg[1] = ekt; lg[2] = ekr; lg[3] = temperature; lg[4] = pressure; lg[5] = H;
      lg[6] = (double)o.npair; lg[7] = th.z0;
    }
  }
  thermo[4] = th.z0; thermo[5] = th.z1; thermo[6] = th.z2; thermo[7] = th.z3; thermo[8] = th.z4; thermo[9] = th.zsum;
  return 0;
}

// Kinetic part only (for checks of the state upload/download path).
void orc_kinetic(int model, int n, const double* rec, double dt, double* out /*ekt, ekr*/) {
  Model m;
  make_model(model, m);
  double pk[9];
  rigid_ek(m, n, rec, dt, out[0], out[1], pk);
}

// Philox uniforms for cross-checking the device generator.
void orc_philox_uniform2(uint64_t seed, uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, double* out) {
  uniform2(seed, c0, c1, c2, c3, out);
}

// Energy of molecule `t` placed at (com_t, quat_t) against every other
// molecule (minimum image, strict rc test, COM switch) -- the per-molecule
// trial energy of mc2.F90:621-668 computed without the N x N pair table.
double orc_molecule_energy(int model, int path, int n, const double* com, const double* quat, int t,
                           const double* com_t, const double* quat_t, const double* L, double rin, double rc) {
  Model m;
  make_model(model, m);
  const int ns = m.nsite;
  double invL[3] = {1.0 / L[0], 1.0 / L[1], 1.0 / L[2]};
  std::vector<double> sx((size_t)(n + 1) * ns), sy(sx.size()), sz(sx.size());
  place_sites(m, n, com, quat, sx.data(), sy.data(), sz.data(), nullptr, nullptr);
  place_sites(m, 1, com_t, quat_t, sx.data() + (size_t)n * ns, sy.data() + (size_t)n * ns, sz.data() + (size_t)n * ns,
              nullptr, nullptr);
  std::vector<double> allcom(com, com + 3 * (size_t)n);
  allcom.insert(allcom.end(), com_t, com_t + 3);
  Pairs P;
  for (int i = 0; i < n; ++i) {
    if (i == t) continue;
    double o[3];
    if (compress_test(com + 3 * i, com_t, L, invL, rc * rc, o)) {
      P.i.push_back(i); P.j.push_back(n); P.ox.push_back(o[0]); P.oy.push_back(o[1]); P.oz.push_back(o[2]);
      P.hh.push_back(1.0); P.dh.push_back(0.0);
    }
  }
  cutoff_dimmer2(rin, rc, allcom.data(), allcom.data(), P);
  std::vector<double> ep(P.i.size());
  pairpot_dispatch(m, path, sx.data(), sy.data(), sz.data(), P, ep.data());
  double e = 0;
  for (double v : ep) e += v;
  return e;
}

// Threaded CPU force path for the baseline timing: sites, cell search,
// switch, StdForce arithmetic on nthreads threads, collect.  Returns npair.
long orc_compute_threaded(int model, int n, const double* com, const double* quat, const double* L, const double* req,
                          double rin, double rc, int nthreads, double* F, double* tau, double* epot, double* vir) {
  Model m;
  if (!make_model(model, m)) return -1;
  const size_t ns = m.nsite;
  std::vector<double> sx(n * ns), sy(n * ns), sz(n * ns), intra(n * ns * 3), tmat(9 * (size_t)n);
  place_sites(m, n, com, quat, sx.data(), sy.data(), sz.data(), intra.data(), tmat.data());
  Grid g;
  Pairs P;
  pairsearch_threaded(n, com, L, req, rc, g, P, nthreads);
  cutoff_dimmer2(rin, rc, com, com, P);
  std::vector<double> fx(n * ns, 0.0), fy(n * ns, 0.0), fz(n * ns, 0.0);
  std_force_threaded(m, sx.data(), sy.data(), sz.data(), P, fx.data(), fy.data(), fz.data(), *epot, vir, nthreads,
                     (int)(n * ns));
  collectforce(m, n, intra.data(), tmat.data(), fx.data(), fy.data(), fz.data(), F, tau);
  return (long)P.i.size();
}

// Gear MD like orc_md_run, with the force evaluated by the threaded StdForce
// arithmetic on nthreads host threads (CPU-baseline timing).  Same log layout.
int orc_md_run_threaded(int model, int n, double* rec, const double* L, const double* req, double rin, double rc,
                        double dt, int nsteps, double* thermo, double* log, int nthreads) {
  Model m;
  if (!make_model(model, m)) return 1;
  Thermo th;
  th.nose_active = (int)thermo[0]; th.q = thermo[1]; th.dump = thermo[2]; th.temp = thermo[3];
  th.z0 = thermo[4]; th.z1 = thermo[5]; th.z2 = thermo[6]; th.z3 = thermo[7]; th.z4 = thermo[8]; th.zsum = thermo[9];
  const double dof = 6.0 * n;
  std::vector<double> com(3 * (size_t)n), quat(4 * (size_t)n), F(3 * (size_t)n), tau(3 * (size_t)n);
  for (int step = 0; step < nsteps; ++step) {
    for (int i = 0; i < n; ++i) rigid_predict(rec + (size_t)REC * i);
    if (th.nose_active) nose_predict(th);
    for (int i = 0; i < n; ++i) {
      std::memcpy(&com[3 * i], rec + (size_t)REC * i, 3 * sizeof(double));
      std::memcpy(&quat[4 * i], rec + (size_t)REC * i + 33, 4 * sizeof(double));
    }
    double epot = 0, vir[9];
    long npair = orc_compute_threaded(model, n, com.data(), quat.data(), L, req, rin, rc, nthreads, F.data(),
                                      tau.data(), &epot, vir);
    for (int i = 0; i < n; ++i) rigid_correct(m, rec + (size_t)REC * i, &F[3 * i], &tau[3 * i], dt, th);
    double ekt, ekr, pk[9];
    rigid_ek(m, n, rec, dt, ekt, ekr, pk);
    double temperature = I2J * 2.0 * (ekt + ekr) / (RGAS * dof);
    if (th.nose_active) nose_correct(th, temperature);
    if (log) {
      double* lg = log + 8 * (size_t)step;
      lg[0] = epot; lg[1] = ekt; lg[2] = ekr; lg[3] = temperature; lg[4] = 0; lg[5] = (epot + ekt + ekr) * I2J;
      lg[6] = (double)npair; lg[7] = th.z0;
    }
  }
  thermo[4] = th.z0; thermo[5] = th.z1; thermo[6] = th.z2; thermo[7] = th.z3; thermo[8] = th.z4; thermo[9] = th.zsum;
  return 0;
}

// Monte Carlo chain, the trial/accept algorithm of mc2.F90:544-832 with the
// device's conventions: Philox draws (counter = chain, trial, draw), fixed
// widths, dE = E(target at new pose) - E(target at old pose) over every other
// molecule.  com (n,3) and quat (n,4) are updated in place; energy (1) is the
// running total; trace (ntrial,4) gets dE, energy, accepted, target.
int orc_mc_run(int model, int path, int n, double* com, double* quat, const double* L, double rin, double rc,
               double beta, double sig_t, double sig_r, int ntrial, uint64_t seed, uint32_t chain, uint64_t counter,
               double* energy, double* trace) {
  Model m;
  if (!make_model(model, m)) return 1;
  double e = *energy;
  for (int t = 0; t < ntrial; ++t) {
    const uint64_t trial = counter + (uint64_t)t;
    const uint32_t lo = (uint32_t)trial, hi = (uint32_t)(trial >> 32);
    double u0[2];
    uniform2(seed, chain, lo, hi, 0u, u0);
    int tg = (int)(u0[0] * n);
    if (tg >= n) tg = n - 1;   // mc2.F90:551 could select n+1 (1-based) when the uniform is 1
    double rot[3], dx[3];
    for (int k = 0; k < 3; ++k) {
      double u[2];
      uniform2(seed, chain, lo, hi, 1u + k, u);
      rot[k] = random_normal(0.0, sig_r * sig_r, u[0], u[1]);
    }
    for (int k = 0; k < 3; ++k) {
      double u[2];
      uniform2(seed, chain, lo, hi, 4u + k, u);
      dx[k] = random_normal(0.0, sig_t * sig_t, u[0], u[1]);
    }
    // qinfrotator (QuatModule.F90:203-211) then qadd (:108-133)
    double a = 1.0, b = rot[0], c = rot[1], d = rot[2];
    const double r = 1.0 / std::sqrt(a * a + b * b + c * c + d * d);
    a *= r; b *= r; c *= r; d *= r;
    const double* qo = quat + 4 * tg;
    double qn[4] = {a * qo[0] - b * qo[1] - c * qo[2] - d * qo[3], a * qo[1] + b * qo[0] + c * qo[3] - d * qo[2],
                    a * qo[2] + c * qo[0] - b * qo[3] + d * qo[1], a * qo[3] + d * qo[0] + b * qo[2] - c * qo[1]};
    if (qn[0] < 0) for (int k = 0; k < 4; ++k) qn[k] = -qn[k];
    double cn[3] = {com[3 * tg] + dx[0], com[3 * tg + 1] + dx[1], com[3 * tg + 2] + dx[2]};
    const double eo = orc_molecule_energy(model, path, n, com, quat, tg, com + 3 * tg, quat + 4 * tg, L, rin, rc);
    const double en = orc_molecule_energy(model, path, n, com, quat, tg, cn, qn, L, rin, rc);
    const double dE = en - eo;
    const double x = -(dE * I2J * J2K) * beta;
    const bool acc = x >= 0.0 || u0[1] < std::exp(x);
    if (acc) {
      for (int k = 0; k < 3; ++k) com[3 * tg + k] = cn[k];
      for (int k = 0; k < 4; ++k) quat[4 * tg + k] = qn[k];
      e += dE;
    }
    if (trace) { trace[4 * t] = dE; trace[4 * t + 1] = e; trace[4 * t + 2] = acc ? 1.0 : 0.0; trace[4 * t + 3] = tg; }
  }
  *energy = e;
  return 0;
}

// rigid_vreset2 (RigidModule.F90:1016-1053): per molecule, in this order,
// dx(1), dy(1), dz(1) = Random_Normal(0, temp*rgas*J2I/mass, r1, r2) * dt and
// wx(1), wy(1), wz(1) = Random_Normal(0, temp*rgas*J2I/I_k, r1, r2), each
// from the next two numbers of the stream u (the caller's Random_GetNext
// values, 12 per molecule).  Random_Normal is RandomModule.F90:28-36.
void orc_vreset2(int model, int n, double temp, double dt, const double* u, double* d1 /*n,3*/, double* w1 /*n,3*/) {
  Model m;
  if (!make_model(model, m)) return;
  const double kT = temp * RGAS * J2I;
  const double var[6] = {kT / m.mass, kT / m.mass, kT / m.mass, kT / m.Ixx, kT / m.Iyy, kT / m.Izz};
  for (int i = 0; i < n; ++i) {
    const double* ui = u + 12 * (size_t)i;
    for (int k = 0; k < 3; ++k) d1[3 * i + k] = random_normal(0.0, var[k], ui[2 * k], ui[2 * k + 1]) * dt;
    for (int k = 0; k < 3; ++k) w1[3 * i + k] = random_normal(0.0, var[3 + k], ui[6 + 2 * k], ui[7 + 2 * k]);
  }
}

// replica_exchange_trial (Replica.F90:7-73) for temperature slots j, jj
// (0-based): node_in_charge[slot] is the replica holding that slot; u is the
// random_getnext value for the Metropolis test; umbrella (nrep, numbrella, 2)
// holds (center, coeffi), op (nrep, numbrella) the order parameters
// (umbrella_potential = coeffi (op - center)^2, Umbrella.F90:11-16).  On
// acceptance beta, the umbrellas and node_in_charge are swapped.  Returns 1
// when accepted.
int orc_replica_exchange_trial(int j, int jj, int* node_in_charge, double u, const double* rep_energy,
                               double* rep_beta, int numbrella, double* rep_umbrella, const double* rep_op) {
  const int n0 = node_in_charge[j], n1 = node_in_charge[jj];
  auto up = [&](int owner, int at) {   // umbrella of replica `owner` on the order parameter of replica `at`
    double a = 0.0;
    for (int k = 0; k < numbrella; ++k) {
      const double* uu = rep_umbrella + ((size_t)owner * numbrella + k) * 2;
      const double o = rep_op[(size_t)at * numbrella + k];
      a = a + uu[1] * ((o - uu[0]) * (o - uu[0]));
    }
    return a;
  };
  double a0 = rep_energy[n0], a1 = rep_energy[n1];
  if (numbrella > 0) { a0 = a0 + up(n0, n0); a1 = a1 + up(n1, n1); }
  const double acceptance0 = -(a0 * rep_beta[n0] + a1 * rep_beta[n1]) * I2J * J2K;
  a0 = rep_energy[n0]; a1 = rep_energy[n1];
  if (numbrella > 0) { a0 = a0 + up(n1, n0); a1 = a1 + up(n0, n1); }
  const double acceptance1 = -(a0 * rep_beta[n1] + a1 * rep_beta[n0]) * I2J * J2K;
  bool accept = false;
  if (acceptance0 < acceptance1) accept = true;
  else if (u < std::exp(acceptance1 - acceptance0)) accept = true;
  if (accept) {
    for (int k = 0; k < 2 * numbrella; ++k)
      std::swap(rep_umbrella[(size_t)n0 * numbrella * 2 + k], rep_umbrella[(size_t)n1 * numbrella * 2 + k]);
    std::swap(rep_beta[n0], rep_beta[n1]);
    node_in_charge[j] = n1;
    node_in_charge[jj] = n0;
  }
  return accept ? 1 : 0;
}

// Order parameter `kind` (0: potential energy, given; 1: local Q6; 2:
// triangle histogram divergence) of one configuration com (n,3).  q6 (n,
// optional) gets the per-molecule Q6, hist (21, optional) the triangle counts.
double orc_order_parameter(int kind, int n, const double* com, const double* L, const double* ref, int logarithmic,
                           double energy, double* q6, double* hist) {
  if (kind == 1) return op_q6(n, com, L, q6);
  if (kind == 2) return op_triangle(n, com, L, ref, logarithmic, hist);
  return energy;
}

// Umbrella Monte Carlo chain: orc_mc_run's trials with the order parameter of
// the trial configuration (mc2.F90:684-697; computed from scratch here) and
// the umbrella term coeff (op - center)^2 (Umbrella.F90:11-16) added to dE in
// the Metropolis test (mc2.F90:700-722).  op (1) is the current order
// parameter (in/out); trace (ntrial,5) gets dE, energy, accepted, target, op.
int orc_mc_umbrella_run(int model, int path, int n, double* com, double* quat, const double* L, double rin, double rc,
                        double beta, double sig_t, double sig_r, int ntrial, uint64_t seed, uint32_t chain,
                        uint64_t counter, int kind, double center, double coeff, const double* ref, int logarithmic,
                        double* energy, double* op, double* trace) {
  Model m;
  if (!make_model(model, m)) return 1;
  double e = *energy, o = *op;
  std::vector<double> trial_com(com, com + 3 * (size_t)n);
  for (int t = 0; t < ntrial; ++t) {
    const uint64_t trial = counter + (uint64_t)t;
    const uint32_t lo = (uint32_t)trial, hi = (uint32_t)(trial >> 32);
    double u0[2];
    uniform2(seed, chain, lo, hi, 0u, u0);
    int tg = (int)(u0[0] * n);
    if (tg >= n) tg = n - 1;
    double rot[3], dx[3];
    for (int k = 0; k < 3; ++k) {
      double u[2];
      uniform2(seed, chain, lo, hi, 1u + k, u);
      rot[k] = random_normal(0.0, sig_r * sig_r, u[0], u[1]);
    }
    for (int k = 0; k < 3; ++k) {
      double u[2];
      uniform2(seed, chain, lo, hi, 4u + k, u);
      dx[k] = random_normal(0.0, sig_t * sig_t, u[0], u[1]);
    }
    double a = 1.0, b = rot[0], c = rot[1], d = rot[2];
    const double r = 1.0 / std::sqrt(a * a + b * b + c * c + d * d);
    a *= r; b *= r; c *= r; d *= r;
    const double* qo = quat + 4 * tg;
    double qn[4] = {a * qo[0] - b * qo[1] - c * qo[2] - d * qo[3], a * qo[1] + b * qo[0] + c * qo[3] - d * qo[2],
                    a * qo[2] + c * qo[0] - b * qo[3] + d * qo[1], a * qo[3] + d * qo[0] + b * qo[2] - c * qo[1]};
    if (qn[0] < 0) for (int k = 0; k < 4; ++k) qn[k] = -qn[k];
    double cn[3] = {com[3 * tg] + dx[0], com[3 * tg + 1] + dx[1], com[3 * tg + 2] + dx[2]};
    const double eo = orc_molecule_energy(model, path, n, com, quat, tg, com + 3 * tg, quat + 4 * tg, L, rin, rc);
    const double en = orc_molecule_energy(model, path, n, com, quat, tg, cn, qn, L, rin, rc);
    const double dE = en - eo;
    double newop;
    if (kind == 0) {
      newop = e + dE;
    } else {
      for (int k = 0; k < 3; ++k) trial_com[3 * tg + k] = cn[k];
      newop = orc_order_parameter(kind, n, trial_com.data(), L, ref, logarithmic, 0.0, nullptr, nullptr);
      for (int k = 0; k < 3; ++k) trial_com[3 * tg + k] = com[3 * tg + k];
    }
    const double dU = coeff * ((newop - center) * (newop - center)) - coeff * ((o - center) * (o - center));
    const double x = -((dE + dU) * I2J * J2K) * beta;
    const bool acc = x >= 0.0 || u0[1] < std::exp(x);
    if (acc) {
      for (int k = 0; k < 3; ++k) { com[3 * tg + k] = cn[k]; trial_com[3 * tg + k] = cn[k]; }
      for (int k = 0; k < 4; ++k) quat[4 * tg + k] = qn[k];
      e += dE;
      o = newop;
    }
    if (trace) {
      double* tr = trace + 5 * (size_t)t;
      tr[0] = dE; tr[1] = e; tr[2] = acc ? 1.0 : 0.0; tr[3] = tg; tr[4] = o;
    }
  }
  *energy = e;
  *op = o;
  return 0;
}

int orc_max_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"
