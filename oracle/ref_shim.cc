// ref_shim.cc -- TEST INFRASTRUCTURE ONLY.
//
// Glue that turns the reference's own C++ sources (compiled unchanged from
// the reference tree by oracle/ref_build.sh) into a shared library the tests
// can drive through ctypes:
//  * replay versions of the reference's random generators rnd1..rnd7,
//    gauss, nrnd1..4 (mc_randg.cc:90-174) and runif (omprng.cc:34-38), so
//    moves can be fed the same proposals and uniforms as the GB300 kernels;
//  * the Fortran leaf symbols the C++ calls (rotden_, vcord_, rsrot_,
//    rsline_, vspher_, caleng_, ...; extern "C" declarations at
//    mc_piqmc.cc:31-48), bound to the oracle's C restatements because no
//    Fortran compiler is available;
//  * setup/state/move/estimator entry points over the reference globals.
// Nothing here is part of the GB300 library.

#include "mc_input.h"
#include "mc_confg.h"
#include "mc_const.h"
#include "mc_setup.h"
#include "mc_randg.h"
#include "mc_utils.h"
#include "mc_poten.h"
#include "mc_piqmc.h"
#include "mc_qworm.h"
#include "mc_estim.h"
#include "rngstream.h"

#include <cmath>
#include <cstring>
#include <unistd.h>

extern "C" {
#include "pimc_oracle.h"
}

// ------------------------------------------------------------ replay RNG
struct ReplayStream { const double *v = nullptr; long n = 0, pos = 0; };
static ReplayStream g_u[8];       // 1..7 = rnd1..rnd7
static ReplayStream g_n[5];       // 1..4 = nrnd1..nrnd4
static ReplayStream g_gauss;      // x1 values of gauss()
static ReplayStream g_runif;      // runif()
static int g_overrun = 0;

static double take(ReplayStream &s)
{
  if (s.pos >= s.n) { g_overrun = 1; return 0.5; }
  return s.v[s.pos++];
}

double rnd(void) { return take(g_u[0]); }
double rnd1(void) { return take(g_u[1]); }
double rnd2(void) { return take(g_u[2]); }
double rnd3(void) { return take(g_u[3]); }
double rnd4(void) { return take(g_u[4]); }
double rnd5(void) { return take(g_u[5]); }
double rnd6(void) { return take(g_u[6]); }
double rnd7(void) { return take(g_u[7]); }
int nrnd1(int n) { return (int)floor(n * take(g_n[1])); }   // mc_randg.cc:159-178, own streams
int nrnd2(int n) { return (int)floor(n * take(g_n[2])); }
int nrnd3(int n) { return (int)floor(n * take(g_n[3])); }
int nrnd4(int n) { return (int)floor(n * take(g_n[4])); }
double gauss(double alpha) { double x1 = take(g_gauss); return (x1 / sqrt(alpha)); }   // mc_randg.cc:149
void RandomInit(int, int) {}
void RandomFree(void) {}
void RandomIO(int, const char[]) {}
double runif(RngStream *) { return take(g_runif); }
void randomseed() {}

// ------------------------------------------------ Fortran leaf bindings
static int g_rot_nth = 181, g_rot_nph = 361, g_rot_nch = 361;   // rotpro grid (rotpro_sub.f:26)
static int g_chfold = 0;                                          // 0: infer from CHgrd
static const double *g_sph = nullptr;
static int g_nsph = 0;
static double g_sph_r0 = 3.0, g_sph_rmax = 26.0, g_sph_rstep = 0.046;

extern "C" void rotden_(double *Eulan1, double *Eulan2, double *Eulrel, double *rho, double *erot, double *esq,
                        double *rhoprp_, double *erotpr_, double *erotsq_, int *istop)
{
  orc_deleul(Eulan1, Eulan2, Eulrel);
  double phi = Eulrel[0] * 180.0 / M_PI, theta = Eulrel[1] * 180.0 / M_PI, chi = Eulrel[2] * 180.0 / M_PI;
  int jstop = orc_rotpro_raw(chi, phi, theta, rhoprp_, erotpr_, erotsq_, g_rot_nth, g_rot_nph, g_rot_nch, rho, erot, esq);
  if (jstop) *istop = 1;
  *erot = *erot / 0.6950356;
  *esq = *esq / (0.6950356 * 0.6950356);
}

extern "C" void vcord_(double *Eulang, double *RCOM, double *Rpt, double *vtable_, int *Rgrd_, int *THgrd_, int *CHgrd_,
                       double *Rvmax_, double *Rvmin_, double *Rvstep_, double *vpot3d, double *radret, double *theret,
                       double *chiret, double *hatx, double *haty, double *hatz, int *ivcord)
{
  // hat x, y, z are the columns of matpre's rotation matrix (vcord.f:30-34);
  // ivcord = 1 returns right after them (vcord.f:42)
  double m[9];
  orc_matpre(Eulang, m);
  for (int i = 0; i < 3; i++) { hatx[i] = m[i * 3 + 0]; haty[i] = m[i * 3 + 1]; hatz[i] = m[i * 3 + 2]; }
  if (*ivcord == 1) return;
  int fold = g_chfold;
  if (fold == 0) fold = (*CHgrd_ == 181) ? 180 : (*CHgrd_ == 361 ? 360 : 90);
  *vpot3d = orc_vcord_raw(Eulang, RCOM, Rpt, vtable_, *Rgrd_, *THgrd_, *CHgrd_, fold, *Rvmax_, *Rvmin_, *Rvstep_,
                          radret, theret, chiret);
}

extern "C" void rsrot_(double *Eulan1, double *Eulan2, double *X, double *Y, double *Z, double *tau, int *iodevn,
                       double *eoff, double *rho, double *erot)
{
  orc_rsrot(Eulan1, Eulan2, *X, *Y, *Z, *tau, *iodevn, *eoff, rho, erot);
}

extern "C" void rsline_(double *X, double *p0, double *tau, double *rho, double *erot)
{
  orc_rsline(*X, *p0, *tau, rho, erot);
}

extern "C" void vspher_(double *r, double *vpot)
{
  *vpot = g_sph ? orc_vspher_raw(*r, g_sph, g_nsph, g_sph_r0, g_sph_rmax, g_sph_rstep) : 0.0;
}

extern "C" void caleng_(double *com_1, double *com_2, double *E_2H2O, double *Eulang_1, double *Eulang_2)
{
  *E_2H2O = orc_caleng(com_1, com_2, Eulang_1, Eulang_2);
}

// reflections (vcord.f:190-546) are estimator-time symmetrisation moves that
// the sampling path never calls; bound to a loud failure
extern "C" void initconf_(double *, double *, int *, int *, int *, int *) { nrerror("ref_shim", "initconf_ not bound"); }
extern "C" void reflec_(double *, double *, double *, double *, double *) { nrerror("ref_shim", "reflec_ not bound"); }
extern "C" void rflmfx_(double *, double *, double *, double *, double *) { nrerror("ref_shim", "rflmfx_ not bound"); }
extern "C" void rflmfy_(double *, double *, double *, double *, double *) { nrerror("ref_shim", "rflmfy_ not bound"); }
extern "C" void rflmfz_(double *, double *, double *, double *, double *) { nrerror("ref_shim", "rflmfz_ not bound"); }

// estimator state of mc_estim.cc (file scope, not declared in its header)
extern double **_gr1D_sum, ***_gr2D_sum, **_gr3D_sum, *_ploops;
extern double _areas[2], _area2[2], _inert[2];
extern double _areas3DMFF[6], _inert3DMFF[9], _areas3DSFF[6], _inert3DSFF[9];
extern int NUMB_DENS1D, NUMB_DENS2D, NUMB_DENS3D;
extern double **_rcf, **_rcf_sum;
extern double *_relthe_sum, *_relphi_sum, *_relchi_sum;
// block averages of mc_main.cc (file scope there)
extern double avergCount, _bkin, _bpot, _brot, _brotsq, _bCv, _bCv_trans, _bCv_rot;
void MCResetBlockAverage(void);
void MCGetAverage(void);
void SaveEnergy(const char[], double, long int);
extern double totalCount, _kin_total, _pot_total, _rot_total, _rotsq_total, _Cv_total, _Cv_trans_total, _Cv_rot_total;
void InitTotalAverage(void);
void DoneTotalAverage(void);
void SaveSumEnergy(double, double);
void densities_reset(int);
void super_reset(void);
void rcf_reset(int);
// histogram sizes of mc_estim.cc:25-27 (file-scope constants there)
static const int MC_BINSR_REF = PIMC_BINSR, MC_BINST_REF = PIMC_BINST, MC_BINSC_REF = PIMC_BINSC;

// table readers of mc_poten.cc (file scope, not declared in its header)
void init_pot1D(int atype);
void init_pot2D(int atype);
void init_rotdens(int type);

// --------------------------------------------------------- entry points
extern "C" {

// qmc.input in workdir; 1D/2D potentials and .rot files are read by the
// reference's own readers (mc_poten.cc:305-438,508-546).  The 3D potential
// and the nonlinear density tables are handed over in memory (ref_load_3d,
// ref_load_rho) instead of through their 23.6M-line text files.
int ref_setup(const char *workdir)
{
  if (chdir(workdir) != 0) return 1;
  int restart = 0;
  IOReadParams(FINPUT, restart);          // mc_main.cc:105
  MCInitParams();                         // mc_main.cc:112
  MCSetUnits();
  MCMemAlloc();
  MemAllocMCCounts();
  MemAllocQWCounts();
  MCInit();                               // mc_main.cc:124
  if (WORM) MCWormInit();
  // InitPotentials (mc_poten.cc:93-119) type by type; the 3D table of a
  // nonlinear rotor comes from ref_load_3d instead of init_pot3D
  for (int atype = 0; atype < NumbTypes; atype++) {
    if (MCAtom[atype].molecule == 1) init_pot2D(atype);
    else if (MCAtom[atype].molecule == 0) init_pot1D(atype);
  }
  if (ROTATION && MCAtom[IMTYPE].molecule == 1 && RotDenType == 0) init_rotdens(IMTYPE);   // InitRotDensity
  if (BOSONS) InitMCEstims();
  ResetMCCounts();
  ResetQWCounts();                        // mc_main.cc resets them per block (MCResetBlockAverage)
  return 0;
}

void ref_load_3d(const double *vt, int rgrd, int thgrd, int chgrd, double rvmin, double rvmax, int chfold)
{
  long n = (long)rgrd * thgrd * chgrd;
  vtable = new double[n];
  memcpy(vtable, vt, sizeof(double) * n);
  Rgrd = rgrd; THgrd = thgrd; CHgrd = chgrd; Rvmin = rvmin; Rvmax = rvmax;
  Rvstep = (Rvmax - Rvmin) / (double)(Rgrd - 1);     // mc_poten.cc:288
  g_chfold = chfold;
}

void ref_load_rho(const double *rho, const double *eng, const double *esq, int nth, int nph, int nch)
{
  long n = (long)nth * nph * nch;
  memcpy(rhoprp, rho, sizeof(double) * n);
  memcpy(erotpr, eng, sizeof(double) * n);
  memcpy(erotsq, esq, sizeof(double) * n);
  g_rot_nth = nth; g_rot_nph = nph; g_rot_nch = nch;
}

void ref_load_sph(const double *t, int n, double r0, double rmax, double rstep)
{
  g_sph = t; g_nsph = n; g_sph_r0 = r0; g_sph_rmax = rmax; g_sph_rstep = rstep;
}

int ref_natoms(void) { return NumbAtoms; }
int ref_nslices(void) { return NumbTimes; }
double ref_tau(void) { return MCTau; }
double ref_lambda(int type) { return MCAtom[type].lambda; }
int ref_offset(int type) { return MCAtom[type].offset; }

// coordinates and angles in the layout of MCCoords/MCAngles; cosines
// derived like mc_main.cc:184-200
void ref_set_state(const double *coords, const double *angles, const int *pindex)
{
  long nb = (long)NumbAtoms * NumbTimes;
  for (long i = 0; i < nb; i++)
    for (int d = 0; d < 3; d++) {
      MCCoords[d][i] = coords[d * nb + i];
      MCAngles[d][i] = angles[d * nb + i];
    }
  for (long i = 0; i < nb; i++) {
    double phi = MCAngles[PHI][i], cost = MCAngles[CTH][i];
    double sint = sqrt(1.0 - cost * cost);
    MCCosine[AXIS_X][i] = sint * cos(phi);
    MCCosine[AXIS_Y][i] = sint * sin(phi);
    MCCosine[AXIS_Z][i] = cost;
  }
  if (pindex)
    for (int a = 0; a < NumbAtoms; a++) { PIndex[a] = pindex[a]; RIndex[pindex[a]] = a; }
}

void ref_get_state(double *coords, double *angles, double *cosine)
{
  long nb = (long)NumbAtoms * NumbTimes;
  for (long i = 0; i < nb; i++)
    for (int d = 0; d < 3; d++) {
      if (coords) coords[d * nb + i] = MCCoords[d][i];
      if (angles) angles[d * nb + i] = MCAngles[d][i];
      if (cosine) cosine[d * nb + i] = MCCosine[d][i];
    }
}

void ref_set_replay(const double *u1, long n1, const double *u2, long n2, const double *u3, long n3,
                    const double *g, long ng, const double *ur, long nr)
{
  g_u[1] = {u1, n1, 0};
  g_u[2] = {u2, n2, 0};
  g_u[3] = {u3, n3, 0};
  g_gauss = {g, ng, 0};
  g_runif = {ur, nr, 0};
  g_overrun = 0;
}

// worm-move streams: nrnd1..3, rnd1..5, gauss (the other streams are left as set)
void ref_set_wreplay(const double *n1, long nn1, const double *n2, long nn2, const double *n3, long nn3,
                     const double *u1, long m1, const double *u2, long m2, const double *u3, long m3,
                     const double *u4, long m4, const double *u5, long m5, const double *g, long ng)
{
  g_n[1] = {n1, nn1, 0}; g_n[2] = {n2, nn2, 0}; g_n[3] = {n3, nn3, 0};
  g_u[1] = {u1, m1, 0}; g_u[2] = {u2, m2, 0}; g_u[3] = {u3, m3, 0}; g_u[4] = {u4, m4, 0}; g_u[5] = {u5, m5, 0};
  g_gauss = {g, ng, 0};
  g_overrun = 0;
}

void ref_wreplay_pos(long *pos)   // n1 n2 n3 u1..u5 gauss overrun
{
  pos[0] = g_n[1].pos; pos[1] = g_n[2].pos; pos[2] = g_n[3].pos;
  for (int k = 1; k <= 5; k++) pos[2 + k] = g_u[k].pos;
  pos[8] = g_gauss.pos; pos[9] = g_overrun;
}

void ref_replay_pos(long *pos)   // consumed counts: rnd1, rnd2, rnd3, gauss, runif, overrun
{
  pos[0] = g_u[1].pos; pos[1] = g_u[2].pos; pos[2] = g_u[3].pos; pos[3] = g_gauss.pos; pos[4] = g_runif.pos;
  pos[5] = g_overrun;
}

// energies (mc_piqmc.cc:1201-1383, 1796-2151); pos in [3][natoms*P] layout
static double **wrap3(const double *pos, double **rows)
{
  long nb = (long)NumbAtoms * NumbTimes;
  for (int d = 0; d < 3; d++) rows[d] = const_cast<double *>(pos) + d * nb;
  return rows;
}
double ref_pot_energy_slice(int atom0, const double *pos, int it) { double *r[3]; return PotEnergy(atom0, wrap3(pos, r), it); }
double ref_pot_energy_path(int atom0, const double *pos) { double *r[3]; return PotEnergy(atom0, wrap3(pos, r)); }
double ref_pot_rot_energy(int atom0, const double *cosine, int it) { double *r[3]; return PotRotEnergy(atom0, wrap3(cosine, r), it); }
double ref_pot_rot_e3d(int atom0, double *eul, int it) { return PotRotE3D(atom0, eul, it); }
double ref_spot1d(double r, int type) { return SPot1D(r, type); }
double ref_lpot2d(double r, double c, int type) { return LPot2D(r, c, type); }
double ref_srotdens(double g, int type, int which)
{
  return which == 0 ? SRotDens(g, type) : (which == 1 ? SRotDensDeriv(g, type) : SRotDensEsqrt(g, type));
}

// moves (mc_piqmc.cc:54-1199) driven by the replay streams
void ref_molecular_move(int type) { MCMolecularMove(type); }
void ref_molecular_move_exchange(int type) { MCMolecularMoveExchange(type); }
void ref_bisection_move(int type, int time) { MCBisectionMove(type, time); }
void ref_bisection_move_exchange(int type, int time) { MCBisectionMoveExchange(type, time); }
void ref_rotations_move(int type) { MCRotationsMove(type); }
void ref_rotations_3d(int type) { MCRotations3D(type); }
void ref_rot_lin_step(int it1, int rotor, const double *u, double *tot, double *acp)
{
  int type = IMTYPE;
  int offset = MCAtom[type].offset + NumbTimes * rotor;
  MCRotLinStep(it1, offset, offset / NumbTimes, type, MCAtom[type].rtstep, u[0], u[1], u[2], *tot, *acp);
}
void ref_rot_3d_step(int it1, int rotor, const double *u, double *tot, double *acp)
{
  int type = IMTYPE;
  int offset = MCAtom[type].offset + NumbTimes * rotor;
  MCRot3Dstep(it1, offset, offset / NumbTimes, type, MCAtom[type].rtstep, u[0], u[1], u[2], u[3], IROTSYM, NFOLD_ROT,
              *tot, *acp);
}
void ref_counters(double *total, double *accep)
{
  for (int t = 0; t < NumbTypes; t++)
    for (int k = 0; k < MCMAXMOVES; k++) { total[t * 3 + k] = MCTotal[t][k]; accep[t * 3 + k] = MCAccep[t][k]; }
}
void ref_reset_counters(void) { ResetMCCounts(); }

// estimators (mc_estim.cc:500-1096)
double ref_kin_energy(void) { return GetKinEnergy(); }
double ref_pot_energy_est(void) { return GetPotEnergy_Densities(); }
double ref_rot_energy(double *esq, double *ets) { double s = GetRotEnergy(); *esq = ErotSQ; *ets = Erot_termSQ; return s; }
double ref_rot_e3d(double *esq, double *ets) { double s = GetRotE3D(); *esq = ErotSQ; *ets = Erot_termSQ; return s; }

double ref_mass(int type) { return MCAtom[type].mass; }

// the worm algorithm (mc_qworm.cc); MCWormInit ran in ref_setup from the WORM line
void ref_worm_move(void) { MCWormMove(); }
void ref_worm_state(int *st) { st[0] = Worm.exists; st[1] = Worm.ira; st[2] = Worm.masha; st[3] = Worm.atom_i; st[4] = Worm.atom_m; }
void ref_worm_set_state(const int *st)
{
  Worm.exists = st[0]; Worm.ira = st[1]; Worm.masha = st[2]; Worm.atom_i = st[3]; Worm.atom_m = st[4];
}
void ref_worm_counters(double *total, double *accep)
{
  for (int k = 0; k < QWMAXMOVES; k++) { total[k] = QWTotal[0][k]; accep[k] = QWAccep[0][k]; }
}
void ref_pindex(int *p, int *r)
{
  for (int a = 0; a < NumbAtoms; a++) { p[a] = PIndex[a]; if (r) r[a] = RIndex[a]; }
}
void ref_set_pindex(const int *pindex)
{
  for (int a = 0; a < NumbAtoms; a++) { PIndex[a] = pindex[a]; RIndex[pindex[a]] = a; }
}

// GetPotEnergy_Densities (mc_estim.cc:500-687) from cleared histograms; the
// accumulated ones (_gr?D_sum) are copied out as [dtype][bins]
double ref_densities(double *gr1d, double *gr2d, double *gr3d)
{
  densities_reset(MC_TOTAL);
  densities_reset(MC_BLOCK);
  double v = GetPotEnergy_Densities();
  for (int d = 0; d < NUMB_DENS1D; d++)
    for (int i = 0; i < MC_BINSR_REF; i++) gr1d[d * MC_BINSR_REF + i] = _gr1D_sum[d][i];
  if (IMPURITY && MCAtom[IMTYPE].molecule == 1)
    for (int d = 0; d < NUMB_DENS2D; d++)
      for (int i = 0; i < MC_BINSR_REF; i++)
        for (int j = 0; j < MC_BINST_REF; j++) gr2d[(d * MC_BINSR_REF + i) * MC_BINST_REF + j] = _gr2D_sum[d][i][j];
  if (IMPURITY && MCAtom[IMTYPE].molecule == 2)
    for (int d = 0; d < NUMB_DENS3D; d++)
      for (long i = 0; i < (long)MC_BINSR_REF * MC_BINST_REF * MC_BINSC_REF; i++)
        gr3d[d * (long)MC_BINSR_REF * MC_BINST_REF * MC_BINSC_REF + i] = _gr3D_sum[d][i];
  return v;
}

// GetExchangeLength (mc_estim.cc:1997-2019) into cleared _ploops
void ref_exchange_lengths(double *ploops)
{
  for (int a = 0; a < MCAtom[BSTYPE].numb; a++) _ploops[a] = 0.0;
  GetExchangeLength();
  for (int a = 0; a < MCAtom[BSTYPE].numb; a++) ploops[a] = _ploops[a];
}

// GetAreaEstimators (mc_estim.cc:2087-2250) from cleared sums:
// out = _areas[2], _area2[2], _inert[2]
void ref_area_estimators(double *out)
{
  super_reset();
  GetAreaEstimators();
  out[0] = _areas[0]; out[1] = _areas[1];       // PERP = 0, PARL = 1 (mc_estim.cc:80-81)
  out[2] = _area2[0]; out[3] = _area2[1];
  out[4] = _inert[0]; out[5] = _inert[1];
}

// GetAreaEstim3D (mc_estim.cc:2252-2594) from cleared sums:
// out = _areas3D[6], _inert3D[9] of the frame
void ref_area_estim3d(int iframe, double *out)
{
  super_reset();
  GetAreaEstim3D(iframe);
  const double *a = iframe ? _areas3DMFF : _areas3DSFF, *in = iframe ? _inert3DMFF : _inert3DSFF;
  for (int i = 0; i < 6; i++) out[i] = a[i];
  for (int i = 0; i < 9; i++) out[6 + i] = in[i];
}

// BoxSize (mc_setup.cc:361-366)
void ref_box_size(double *b)
{
  for (int d = 0; d < NDIM; d++) b[d] = BoxSize[d];
}

// the reference's block writers on the accumulators the calls above filled:
// SaveDensities1D/2D/3D and SaveRho1D (mc_estim.cc:1327-1800, block mode
// only for SaveRho1D: its total mode also writes relative-Euler-angle
// histograms), SaveExchangeLength, SaveAreaEstimators, SaveAreaEstim3D
// (mc_estim.cc:2021-2085, 2596-2720)
void ref_save_densities(const char *fname, double acount, int mode)
{
  SaveDensities1D(fname, acount);
  if (mode == MC_TOTAL) SaveGraSum(fname, acount);
  if (IMPURITY && MCAtom[IMTYPE].molecule == 1) SaveDensities2D(fname, acount, mode);
  if (IMPURITY && MCAtom[IMTYPE].molecule == 2) {
    SaveDensities3D(fname, acount, mode);
    if (mode == MC_BLOCK) {
      SaveRho1D(fname, acount, mode);
      SaveRhoThetaChi(fname, acount, mode);
    }
  }
}
void ref_save_exchange_length(const char *fname, double acount, long blocknumb)
{
  SaveExchangeLength(fname, acount, blocknumb);
}
void ref_save_area_estimators(const char *fname, double acount, long blocknumb)
{
  SaveAreaEstimators(fname, acount, blocknumb);
}
void ref_save_area_estim3d(const char *fname, double acount, long blocknumb, int iframe)
{
  SaveAreaEstim3D(fname, acount, blocknumb, iframe);
}

// one MCGetAverage (mc_main.cc:551-694) on a cleared block, then SaveEnergy
// (mc_main.cc:764-795); sums = _bkin, _bpot, _brot, _brotsq, _bCv,
// _bCv_trans, _bCv_rot.  Run in workdir: with bosons MCGetAverage appends to
// permutation.tab in the working directory.
int ref_energy_block(const char *workdir, const char *fname, long blocknumb, double *sums)
{
  char cwd[4096];
  if (!getcwd(cwd, sizeof cwd) || chdir(workdir) != 0) return 1;
  MCResetBlockAverage();
  MCGetAverage();
  const double v[7] = {_bkin, _bpot, _brot, _brotsq, _bCv, _bCv_trans, _bCv_rot};
  for (int k = 0; k < 7; k++) sums[k] = v[k];
  SaveEnergy(fname, avergCount, blocknumb);
  return chdir(cwd) != 0;
}

// the run totals after one MCGetAverage and their SaveSumEnergy line
// (InitTotalAverage opens <file prefix>_sum.eng in workdir); totals as the
// seven sums of ref_energy_block
int ref_sum_energy(const char *workdir, double numb, double *totals)
{
  char cwd[4096];
  if (!getcwd(cwd, sizeof cwd) || chdir(workdir) != 0) return 1;
  InitTotalAverage();
  MCResetBlockAverage();
  MCGetAverage();
  const double v[7] = {_kin_total, _pot_total, _rot_total, _rotsq_total, _Cv_total, _Cv_trans_total, _Cv_rot_total};
  for (int k = 0; k < 7; k++) totals[k] = v[k];
  SaveSumEnergy(totalCount, numb);
  DoneTotalAverage();
  return chdir(cwd) != 0;
}

// the densities and GetRotE3D's relative-angle histograms of the path from
// cleared accumulators, then SaveRho1D's run-total files; the histograms out
void ref_rel_euler(const char *fname, double acount, double *the, double *phi, double *chi)
{
  densities_reset(MC_TOTAL);
  densities_reset(MC_BLOCK);
  GetPotEnergy_Densities();
  GetRotE3D();
  for (int i = 0; i < MC_BINST_REF; i++) the[i] = _relthe_sum[i];
  for (int i = 0; i < MC_BINSC_REF; i++) { phi[i] = _relphi_sum[i]; chi[i] = _relchi_sum[i]; }
  SaveRho1D(fname, acount, MC_TOTAL);
}

// GetRCF once into cleared accumulators, then SaveRCF; rcf[10][Q] = the
// accumulator the file was written from (block or total)
void ref_rcf_save(const char *fname, double acount, int mode, double *rcf)
{
  rcf_reset(MC_BLOCK);
  rcf_reset(MC_TOTAL);
  GetRCF();
  double **src = mode == MC_TOTAL ? _rcf_sum : _rcf;
  for (int ip = 0; ip < NUMB_RCF; ip++)
    for (int it = 0; it < NumbRotTimes; it++) rcf[ip * NumbRotTimes + it] = src[ip][it];
  SaveRCF(fname, acount, mode);
}

}  // extern "C"

// IOxyz (mc_input.cc:690-794) writing the current path to `file`
extern "C" void ref_write_xyz(const char *file)
{
  IOxyz(IOWrite, file);
}
