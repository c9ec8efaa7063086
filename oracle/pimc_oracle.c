/*
 * pimc_oracle.c -- CPU oracle (TEST INFRASTRUCTURE ONLY) for the MoRiBS-PIMC
 * sampling path.  Every function restates one reference routine; the file and
 * lines are cited above each.  See pimc_oracle.h for the contract.
 *
 * Deliberate, documented departures from the reference:
 *  - rotpro leaves delch2/delch3/delph2/... undefined at the upper grid edges
 *    (rotpro_sub.f:35-55); here they are 0, like delchi/delphi/delthe.
 *  - MCBisectionMoveExchange evaluates the midpoint energy of the atom owning
 *    slice pt0 instead of pt1 (mc_piqmc.cc:373-376), which reads stale
 *    newcoords when a segment crosses a permutation; here the owner of each
 *    slice is used.  With the identity permutation both are identical.
 *  - GetRotE3D advances the rotor offset cumulatively (mc_estim.cc:1000-1003),
 *    which is correct for <= 2 rotors only; here rotor a uses offset a*P.
 *  - GetRotE3D with the rattle-and-shake density converts the running sum of
 *    all rotors' link sums to an energy once per rotor (mc_estim.cc:1084-1090),
 *    so with two or more rotors the earlier rotors are converted again; here
 *    each rotor's sum is converted once and the energies are added (the same
 *    for one rotor).
 *  - the grids of vcalc and rotpro are generalised to n points over the same
 *    angular ranges; at the reference's 1-degree sizes the arithmetic is the
 *    reference's (the step is exactly 1.0).
 */
#include "pimc_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define NDIM 3
#define PHI 0
#define CTH 1
#define CHI 2
#define RZERO 1.0e-10                                  /* mc_confg.h:59 */
#define WNO2K 0.6950356                                /* mc_const.h:16 */
#define MC_PI 3.14159265358979323846

enum { MCMOLEC = 0, MCMULTI = 1, MCROTAT = 2 };          /* mc_setup.h:165-168 */

struct orc_ctx {
  pimc_system sys;
  int na;                 /* NumbAtoms */
  int P, Q, R;            /* NumbTimes, NumbRotTimes, RotRatio */
  int imtype;             /* IMTYPE or -1 */
  int offset[PIMC_MAX_TYPES + 1]; /* MCAtom[type].offset (slice units) */
  int mlsegm[PIMC_MAX_TYPES];
  double tau, rot_tau, beta;
  int *mctype;
  int *pindex;
  int *rindex;            /* RIndex: the inverse of pindex */
  /* worm state (TPathWorm, mc_qworm.h:32-48) and its derived constants
   * (MCWormInit, mc_qworm.cc:49-82) */
  int worm_on, wtype, wexists, ira, masha, atom_i, atom_m, wm;
  double wc, qw_norm, wcut2;
  double *dr2_list, *ptable;
  int *atm_list;
  double qwtot[7], qwacc[7];
  uint64_t wctr[9];       /* internal-generator counters of the worm draws */
  double *coords, *cosine, *angles, *newc;  /* [3][na*P] */
  int *pflags, *atom_list;
  /* 1D spline */
  int n1d; double *g1d, *p1d, *y2_1d; double alpha1d, unode1d, c6_1d;
  /* 2D */
  int nr2d, nc2d; double dr2d, dc2d; double *rg2d, *cg2d, *pot2d;
  /* 3D */
  int rgrd, thgrd, chgrd, chfold; double rvmin, rvmax, rvstep, dth3, dch3; double *vtab;
  /* linear density */
  int nrot; double *rg, *rd, *rdv, *rde, *rd_y2, *rdv_y2, *rde_y2;
  /* nonlinear density */
  int nth, nph, nch; double dthd, dphd, dchd; double *rhoprp, *erotpr, *erotsq;
  /* spherical */
  int nsph; double sph_r0, sph_rmax, sph_rstep; double *sph;
  double total[PIMC_MAX_TYPES * 3], accep[PIMC_MAX_TYPES * 3];
  /* internal generator state for orc_run_steps */
  uint64_t seed; uint64_t ctr[8];
};

/* ------------------------------------------------------------------ utils */

static double *dup_array(const double *src, long n)
{
  if (!src || n <= 0) return NULL;
  double *d = (double *)malloc(sizeof(double) * (size_t)n);
  memcpy(d, src, sizeof(double) * (size_t)n);
  return d;
}

/* spline() -- mc_utils.cc:112-154 (Numerical Recipes cubic spline) */
static void nr_spline(const double *x, const double *y, int n, double yp1, double ypn, double *y2)
{
  double p, qn, sig, un;
  double *u = (double *)malloc(sizeof(double) * (size_t)n);
  if (yp1 > 0.99e30)
    y2[0] = u[0] = .0;
  else {
    y2[0] = -.5;
    u[0] = (3. / (x[1] - x[0])) * ((y[1] - y[0]) / (x[1] - x[0]) - yp1);
  }
  for (int i = 1; i < (n - 1); i++) {
    sig = (x[i] - x[i - 1]) / (x[i + 1] - x[i - 1]);
    p = sig * y2[i - 1] + 2.;
    y2[i] = (sig - 1.) / p;
    u[i] = (y[i + 1] - y[i]) / (x[i + 1] - x[i]) - (y[i] - y[i - 1]) / (x[i] - x[i - 1]);
    u[i] = (6. * u[i] / (x[i + 1] - x[i - 1]) - sig * u[i - 1]) / p;
  }
  if (ypn > 0.99e30)
    qn = un = 0.;
  else {
    qn = .5;
    un = (3. / (x[n - 1] - x[n - 2])) * (ypn - (y[n - 1] - y[n - 2]) / (x[n - 1] - x[n - 2]));
  }
  y2[n - 1] = (un - qn * u[n - 2]) / (qn * y2[n - 2] + 1.);
  for (int k = n - 2; k >= 0; k--) y2[k] = y2[k] * y2[k + 1] + u[k];
  free(u);
}

/* splint() -- mc_utils.cc:156-186 (bisection lookup, cubic evaluation) */
static double nr_splint(const double *xa, const double *ya, const double *y2a, int n, double x)
{
  int klo = 0, khi = n - 1, k;
  while (khi - klo > 1) {
    k = (khi + klo) >> 1;
    if (xa[k] > x) khi = k;
    else klo = k;
  }
  double h = xa[khi] - xa[klo];
  double a = (xa[khi] - x) / h;
  double b = (x - xa[klo]) / h;
  return a * ya[klo] + b * ya[khi] + ((a * a * a - a) * y2a[klo] + (b * b * b - b) * y2a[khi]) * (h * h) / 6.;
}

/* init_spline() -- mc_utils.cc:188-201 (end slopes from the first/last pair) */
static void nr_init_spline(const double *grid, const double *data, double *sdata, int n)
{
  double drl = (grid[1] - grid[0]);
  double dpl = (data[1] - data[0]) / drl;
  double drr = (grid[n - 1] - grid[n - 2]);
  double dpr = (data[n - 1] - data[n - 2]) / drr;
  nr_spline(grid, data, n, dpl, dpr, sdata);
}

/* ------------------------------------------------------------- life cycle */

static int type_of_molecule(const pimc_system *s, int t) { return s->type[t].molecule; }

orc_ctx *orc_create(const pimc_system *sys, const pimc_tables *tab, int *status)
{
  *status = PIMC_ERR_BAD_ARG;
  if (!sys || !tab || sys->ntypes < 1 || sys->ntypes > PIMC_MAX_TYPES || sys->nslices < 2) return NULL;
  orc_ctx *c = (orc_ctx *)calloc(1, sizeof(orc_ctx));
  c->sys = *sys;
  c->P = sys->nslices;
  c->Q = sys->rotation ? sys->nrotslices : 0;
  c->R = 1;
  c->imtype = -1;
  c->na = 0;
  for (int t = 0; t < sys->ntypes; t++) {
    c->offset[t] = c->na * c->P;               /* mc_input.cc:352-359 */
    c->na += sys->type[t].numb;
    c->mlsegm[t] = 1 << sys->type[t].levels;   /* mc_setup.cc:395 */
    if (type_of_molecule(sys, t) != PIMC_ATOM) c->imtype = t;
  }
  c->offset[sys->ntypes] = c->na * c->P;
  c->beta = 1.0 / sys->temperature;            /* mc_setup.cc:373-374 */
  c->tau = c->beta / (double)c->P;
  if (sys->rotation) {
    if (c->Q <= 0 || c->P % c->Q) { free(c); return NULL; }
    c->rot_tau = c->beta / (double)c->Q;       /* mc_setup.cc:376-377 */
    c->R = c->P / c->Q;                        /* mc_setup.cc:382-389 */
  }
  size_t nb = (size_t)c->na * (size_t)c->P;
  c->mctype = (int *)malloc(sizeof(int) * (size_t)c->na);
  c->pindex = (int *)malloc(sizeof(int) * (size_t)c->na);
  c->rindex = (int *)malloc(sizeof(int) * (size_t)c->na);
  c->pflags = (int *)malloc(sizeof(int) * (size_t)c->na);
  c->atom_list = (int *)malloc(sizeof(int) * (size_t)c->na);
  int g = 0;
  for (int t = 0; t < sys->ntypes; t++)
    for (int a = 0; a < sys->type[t].numb; a++) c->mctype[g++] = t;   /* mc_setup.cc:327-333 */
  for (int a = 0; a < c->na; a++) c->pindex[a] = c->rindex[a] = a;
  c->coords = (double *)calloc(3 * nb, sizeof(double));
  c->cosine = (double *)calloc(3 * nb, sizeof(double));
  c->angles = (double *)calloc(3 * nb, sizeof(double));
  c->newc = (double *)calloc(3 * nb, sizeof(double));

  *status = PIMC_ERR_BAD_TABLE;
  /* 1D: init_pot1D mc_poten.cc:379-438 */
  if (tab->n1d > 0) {
    int n = tab->n1d;
    if (n < 2) { orc_destroy(c); return NULL; }
    c->n1d = n;
    c->g1d = dup_array(tab->grid1d, n);
    c->p1d = dup_array(tab->pot1d, n);
    c->y2_1d = (double *)malloc(sizeof(double) * (size_t)n);
    nr_init_spline(c->g1d, c->p1d, c->y2_1d, n);
    double fr = c->p1d[0] / c->p1d[1];
    double dr = c->g1d[1] - c->g1d[0];
    c->alpha1d = log(fr) / dr;
    c->unode1d = c->p1d[0] * exp(c->alpha1d * c->g1d[0]);
    double r0 = pow(c->g1d[n - 2], 6.0);
    double r1 = pow(c->g1d[n - 1], 6.0);
    fr = c->p1d[n - 1] - c->p1d[n - 2];
    c->c6_1d = fr / (1.0 / r0 - 1.0 / r1);
  }
  /* 2D: init_pot2D mc_poten.cc:305-377 */
  if (tab->nr2d > 0) {
    if (tab->nr2d < 2 || tab->nc2d < 2) { orc_destroy(c); return NULL; }
    c->nr2d = tab->nr2d; c->nc2d = tab->nc2d;
    c->dr2d = tab->dr2d; c->dc2d = tab->dc2d;
    c->rg2d = dup_array(tab->rgrid2d, c->nr2d);
    c->cg2d = dup_array(tab->cgrid2d, c->nc2d);
    c->pot2d = dup_array(tab->pot2d, (long)c->nr2d * c->nc2d);
  }
  /* 3D: init_pot3D mc_poten.cc:254-303 */
  if (tab->rgrd > 0) {
    if (tab->rgrd < 2 || tab->thgrd < 2 || tab->chgrd < 2) { orc_destroy(c); return NULL; }
    c->rgrd = tab->rgrd; c->thgrd = tab->thgrd; c->chgrd = tab->chgrd;
    c->rvmin = tab->rvmin; c->rvmax = tab->rvmax;
    c->rvstep = (c->rvmax - c->rvmin) / (double)(c->rgrd - 1);
    int fold = tab->chi_fold_deg;
    if (fold == 0) fold = (c->chgrd == 181) ? 180 : (c->chgrd == 361 ? 360 : 90);
    c->chfold = fold;
    c->dth3 = 180.0 / (double)(c->thgrd - 1);
    c->dch3 = (double)fold / (double)(c->chgrd - 1);
    c->vtab = dup_array(tab->vtable, (long)c->rgrd * c->thgrd * c->chgrd);
  }
  /* linear density: init_rotdens mc_poten.cc:508-546 */
  if (tab->nrot > 0) {
    int n = tab->nrot;
    if (n < 2) { orc_destroy(c); return NULL; }
    c->nrot = n;
    c->rg = dup_array(tab->rotgrid, n);
    c->rd = dup_array(tab->rotdens, n);
    c->rdv = dup_array(tab->rotderv, n);
    c->rde = dup_array(tab->rotesqr, n);
    c->rd_y2 = (double *)malloc(sizeof(double) * (size_t)n);
    c->rdv_y2 = (double *)malloc(sizeof(double) * (size_t)n);
    c->rde_y2 = (double *)malloc(sizeof(double) * (size_t)n);
    nr_init_spline(c->rg, c->rd, c->rd_y2, n);
    nr_init_spline(c->rg, c->rdv, c->rdv_y2, n);
    nr_init_spline(c->rg, c->rde, c->rde_y2, n);
  }
  /* nonlinear density: init_rot3D mc_poten.cc:440-506 */
  if (tab->nth > 0) {
    if (tab->nth < 2 || tab->nph < 2 || tab->nch < 2) { orc_destroy(c); return NULL; }
    c->nth = tab->nth; c->nph = tab->nph; c->nch = tab->nch;
    c->dthd = 180.0 / (double)(c->nth - 1);
    c->dphd = 360.0 / (double)(c->nph - 1);
    c->dchd = 360.0 / (double)(c->nch - 1);
    long n = (long)c->nth * c->nph * c->nch;
    c->rhoprp = dup_array(tab->rhoprp, n);
    c->erotpr = dup_array(tab->erotpr, n);
    c->erotsq = dup_array(tab->erotsq, n);
  }
  if (tab->nsph > 0) {
    c->nsph = tab->nsph;
    c->sph_r0 = tab->sph_r0; c->sph_rmax = tab->sph_rmax; c->sph_rstep = tab->sph_rstep;
    c->sph = dup_array(tab->sph_table, tab->nsph);
  }
  *status = PIMC_OK;
  return c;
}

void orc_destroy(orc_ctx *c)
{
  if (!c) return;
  free(c->mctype); free(c->pindex); free(c->rindex); free(c->pflags); free(c->atom_list);
  free(c->dr2_list); free(c->ptable); free(c->atm_list);
  free(c->coords); free(c->cosine); free(c->angles); free(c->newc);
  free(c->g1d); free(c->p1d); free(c->y2_1d);
  free(c->rg2d); free(c->cg2d); free(c->pot2d);
  free(c->vtab);
  free(c->rg); free(c->rd); free(c->rdv); free(c->rde); free(c->rd_y2); free(c->rdv_y2); free(c->rde_y2);
  free(c->rhoprp); free(c->erotpr); free(c->erotsq);
  free(c->sph);
  free(c);
}

int orc_natoms(const orc_ctx *c) { return c->na; }

/* coordinates and angles as read in mc_main.cc:184-200; cosines from angles */
int orc_set_state(orc_ctx *c, const double *coords, const double *angles, const int *pindex)
{
  size_t nb = (size_t)c->na * (size_t)c->P;
  if (coords) memcpy(c->coords, coords, sizeof(double) * 3 * nb);
  if (angles) {
    memcpy(c->angles, angles, sizeof(double) * 3 * nb);
    for (size_t i = 0; i < nb; i++) {
      double phi = c->angles[PHI * nb + i];
      double cost = c->angles[CTH * nb + i];
      double sint = sqrt(1.0 - cost * cost);
      c->cosine[0 * nb + i] = sint * cos(phi);
      c->cosine[1 * nb + i] = sint * sin(phi);
      c->cosine[2 * nb + i] = cost;
    }
  }
  if (pindex) {
    memcpy(c->pindex, pindex, sizeof(int) * (size_t)c->na);
    for (int a = 0; a < c->na; a++) c->rindex[c->pindex[a]] = a;
  }
  return PIMC_OK;
}

int orc_get_state(const orc_ctx *c, double *coords, double *angles, double *cosine, int *pindex)
{
  size_t nb = (size_t)c->na * (size_t)c->P;
  if (coords) memcpy(coords, c->coords, sizeof(double) * 3 * nb);
  if (angles) memcpy(angles, c->angles, sizeof(double) * 3 * nb);
  if (cosine) memcpy(cosine, c->cosine, sizeof(double) * 3 * nb);
  if (pindex) memcpy(pindex, c->pindex, sizeof(int) * (size_t)c->na);
  return PIMC_OK;
}

void orc_get_counters(const orc_ctx *c, double *total, double *accep)
{
  for (int i = 0; i < PIMC_MAX_TYPES * 3; i++) { total[i] = c->total[i]; accep[i] = c->accep[i]; }
}

void orc_reset_counters(orc_ctx *c)
{
  memset(c->total, 0, sizeof(c->total));
  memset(c->accep, 0, sizeof(c->accep));
}

/* ------------------------------------------------------------ table leaves */

/* SPot1D -- mc_poten.cc:624-639 */
double orc_spot1d(const orc_ctx *c, double r)
{
  int size = c->n1d;
  if (r >= c->g1d[size - 1]) return (-c->c6_1d / pow(r, 6.0));
  if (r <= c->g1d[0]) return (c->unode1d * exp(-c->alpha1d * r));
  return nr_splint(c->g1d, c->p1d, c->y2_1d, size, r);
}

/* LPot2D -- mc_poten.cc:688-729 (index clamped, fraction not: linear extrapolation) */
double orc_lpot2d(const orc_ctx *c, double r, double cost)
{
  double rmin = c->rg2d[0];
  double cmin = c->cg2d[0];
  int rsize = c->nr2d, csize = c->nc2d;
  int ir = (int)floor((r - rmin) / c->dr2d);
  int ic = (int)floor((cost - cmin) / c->dc2d);
  if (ir < 0) ir = 0;
  else if (ir >= (rsize - 1)) ir = (rsize - 2);
  if (ic < 0) ic = 0;
  else if (ic >= (csize - 1)) ic = (csize - 2);
  const double *pot = c->pot2d;
  double y1 = pot[(long)ir * csize + ic];
  double y2 = pot[(long)(ir + 1) * csize + ic];
  double y3 = pot[(long)(ir + 1) * csize + ic + 1];
  double y4 = pot[(long)ir * csize + ic + 1];
  double r1 = c->rg2d[ir], r2 = c->rg2d[ir + 1];
  double c1 = c->cg2d[ic], c2 = c->cg2d[ic + 1];
  double dr = (r - r1) / (r2 - r1);
  double dc = (cost - c1) / (c2 - c1);
  return (1.0 - dr) * (1.0 - dc) * y1 + dr * (1.0 - dc) * y2 + dr * dc * y3 + (1.0 - dr) * dc * y4;
}

/* SRotDens / SRotDensDeriv / SRotDensEsqrt -- mc_poten.cc:548-622 */
double orc_srotdens(const orc_ctx *c, double gamma, int which)
{
  int size = c->nrot;
  const double *d = which == 0 ? c->rd : (which == 1 ? c->rdv : c->rde);
  const double *y2 = which == 0 ? c->rd_y2 : (which == 1 ? c->rdv_y2 : c->rde_y2);
  if (gamma > c->rg[size - 1]) return which == 0 ? d[size - 1] : 0.0;
  if (gamma < c->rg[0]) {
    double rl = c->rg[0], rr = c->rg[1];
    double salpha = (d[1] - d[0]) / (rr - rl);
    double sbeta = (d[0] * rr - d[1] * rl) / (rr - rl);
    return (salpha * gamma + sbeta);
  }
  return nr_splint(c->rg, d, y2, size, gamma);
}

/* matpre -- rotden.f:136-163 (ZYZ Euler rotation matrix); m[(i-1)*3+(j-1)] = rotmat(i,j) */
void orc_matpre(const double eul[3], double m[9])
{
  double phi = eul[0], theta = eul[1], chi = eul[2];
  double cp = cos(phi), sp = sin(phi);
  double ct = cos(theta), st = sin(theta);
  double ck = cos(chi), sk = sin(chi);
  m[0] = cp * ct * ck - sp * sk;
  m[1] = -cp * ct * sk - sp * ck;
  m[2] = cp * st;
  m[3] = sp * ct * ck + cp * sk;
  m[4] = -sp * ct * sk + cp * ck;
  m[5] = sp * st;
  m[6] = -st * ck;
  m[7] = st * sk;
  m[8] = ct;
}

/* within -- rotden.f:208-216 */
static double within(double v)
{
  if (v > 1.0) v = 1.0;
  if (v < -1.0) v = -1.0;
  return v;
}

/* deleul -- rotden.f:32-134: relative Euler angles of R1^T R2 */
void orc_deleul(const double e1[3], const double e2[3], double rel[3])
{
  const double small = 1.e-08, zero = 0.0, pi = MC_PI;
  double rotmat[9], rotma1[9], m2[9];
  orc_matpre(e2, rotmat);
  orc_matpre(e1, rotma1);
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      double s = 0.0;
      for (int k = 0; k < 3; k++) s = s + rotma1[k * 3 + i] * rotmat[k * 3 + j];
      m2[i * 3 + j] = s;
    }
  double cost = within(m2[8]);
  double theta2 = acos(cost);
  double sint = sin(theta2);
  double phi2, chi2, cphi, sphi, cchi, schi;
  if (fabs(1.0 - cost) < small) {
    phi2 = 0.0;
    cchi = within(m2[0]);   /* rotma2(1,1) */
    schi = within(m2[3]);   /* rotma2(2,1) */
    chi2 = (schi > zero) ? acos(cchi) : 2.0 * pi - acos(cchi);
  } else if (fabs(1.0 + cost) < small) {
    phi2 = 0.0;
    cchi = within(m2[4]);   /* rotma2(2,2) */
    schi = within(m2[1]);   /* rotma2(1,2) */
    chi2 = (schi > zero) ? acos(cchi) : 2.0 * pi - acos(cchi);
  } else {
    cphi = within(m2[2] / sint);    /* rotma2(1,3) */
    sphi = within(m2[5] / sint);    /* rotma2(2,3) */
    cchi = within(-m2[6] / sint);   /* -rotma2(3,1) */
    schi = within(m2[7] / sint);    /* rotma2(3,2) */
    phi2 = (sphi > zero) ? acos(cphi) : 2.0 * pi - acos(cphi);
    chi2 = (schi > zero) ? acos(cchi) : 2.0 * pi - acos(cchi);
  }
  rel[0] = phi2;
  rel[1] = theta2;
  rel[2] = chi2;
}

/* rotpro -- rotpro_sub.f:1-64, on a grid of nth x nph x nch points spanning
 * theta 0..180, phi 0..360, chi 0..360 degrees (181x361x361 = 1 degree). */
int orc_rotpro_raw(double chi, double phi, double theta, const double *rhoprp, const double *erotpr,
                   const double *erotsq, int nth, int nph, int nch, double *rho, double *erot, double *esq)
{
  int jstop = 0;
  double dth = 180.0 / (double)(nth - 1), dph = 360.0 / (double)(nph - 1), dch = 360.0 / (double)(nch - 1);
  double xc = chi / dch, xp = phi / dph, xt = theta / dth;
  int ichi = (int)xc, iphi = (int)xp, itheta = (int)xt;
  if (ichi > nch - 1 || ichi < 0) { ichi = 0; jstop = 1; }
  if (iphi > nph - 1 || iphi < 0) { iphi = 0; jstop = 1; }
  if (itheta > nth - 1 || itheta < 0) { itheta = 0; jstop = 1; }
  long ind = ((long)itheta * nph + iphi) * nch + ichi;
  double rho0 = rhoprp[ind], erot0 = erotpr[ind], esq0 = erotsq[ind];
  double delchi = 0, delphi = 0, delthe = 0;
  double delch2 = 0, delch3 = 0, delph2 = 0, delph3 = 0, delth2 = 0, delth3 = 0;
  if (ichi != nch - 1) {
    ind = ((long)itheta * nph + iphi) * nch + ichi + 1;
    delchi = rhoprp[ind] - rho0; delch2 = erotpr[ind] - erot0; delch3 = erotsq[ind] - esq0;
  }
  if (iphi != nph - 1) {
    ind = ((long)itheta * nph + iphi + 1) * nch + ichi;
    delphi = rhoprp[ind] - rho0; delph2 = erotpr[ind] - erot0; delph3 = erotsq[ind] - esq0;
  }
  if (itheta != nth - 1) {
    ind = ((long)(itheta + 1) * nph + iphi) * nch + ichi;
    delthe = rhoprp[ind] - rho0; delth2 = erotpr[ind] - erot0; delth3 = erotsq[ind] - esq0;
  }
  double fc = xc - (double)ichi, fp = xp - (double)iphi, ft = xt - (double)itheta;
  *rho = rho0 + delchi * fc + delphi * fp + delthe * ft;
  *erot = erot0 + delch2 * fc + delph2 * fp + delth2 * ft;
  *esq = esq0 + delch3 * fc + delph3 * fp + delth3 * ft;
  return jstop;
}

static int rotpro_g(const orc_ctx *c, double chi, double phi, double theta,
                    double *rho, double *erot, double *esq)
{
  return orc_rotpro_raw(chi, phi, theta, c->rhoprp, c->erotpr, c->erotsq, c->nth, c->nph, c->nch, rho, erot, esq);
}

/* rotden -- rotden.f:1-31; returns 1 where the reference sets istop */
int orc_rotden(const orc_ctx *c, const double e1[3], const double e2[3], double rel[3],
               double *rho, double *erot, double *esq)
{
  const double pi = MC_PI, wno2k = WNO2K;
  orc_deleul(e1, e2, rel);
  double phi = rel[0] * 180.0 / pi;
  double theta = rel[1] * 180.0 / pi;
  double chi = rel[2] * 180.0 / pi;
  int jstop = rotpro_g(c, chi, phi, theta, rho, erot, esq);
  *erot = *erot / wno2k;
  *esq = *esq / (wno2k * wno2k);
  return jstop;
}

static double dotprd(const double *a, const double *b)
{
  double d = 0.0;
  for (int i = 0; i < 3; i++) d = d + a[i] * b[i];
  return d;
}
static double dnorm(const double *a) { return sqrt(dotprd(a, a)); }

/* vcalc -- vcalc.f:1-65: v0 plus three one-sided first-order gradients;
 * theta/chi given here in grid units of the generalised grid. */
static double vcalc_raw(double r, double xth, double xch, double r0, double rmax, double rstep,
                        int nrgrd, int nthgrd, int nchgrd, const double *vtab)
{
  int maxrpt = nrgrd - 1, mxthpt = nthgrd - 1, mxchpt = nchgrd - 1;
  if (r < r0) r = r0;
  if (r > rmax) r = rmax;
  int ir = (int)((r - r0) / rstep);
  int ith = (int)xth;
  int ich = (int)xch;
  if (ich > mxchpt) ich = mxchpt;
  if (ich < 0) ich = 0;
  if (ith > mxthpt) ith = mxthpt;
  if (ith < 0) ith = 0;
  long nth = nthgrd, nch = nchgrd;
  double v0 = vtab[((long)ir * nth + ith) * nch + ich];
  double gradr, delr, gradth, delth, gradch, delch;
  if (ir == maxrpt) { gradr = 0.0; delr = 0.0; }
  else {
    gradr = (vtab[((long)(ir + 1) * nth + ith) * nch + ich] - v0) / rstep;
    delr = r - (r0 + ir * rstep);
  }
  if (ith == mxthpt) { gradth = 0.0; delth = 0.0; }
  else {
    gradth = (vtab[((long)ir * nth + (ith + 1)) * nch + ich] - v0);
    delth = xth - (double)ith;
  }
  if (ich == mxchpt) { gradch = 0.0; delch = 0.0; }
  else {
    gradch = (vtab[((long)ir * nth + ith) * nch + ich + 1] - v0);
    delch = xch - (double)ich;
  }
  return v0 + gradr * delr + gradth * delth + gradch * delch;
}

/* vcord -- vcord.f:1-98: body-frame (r, theta, chi) of the atom, chi folded by
 * the symmetry of the chi grid (chfold 90/180/360 degrees), r converted to
 * bohr, then vcalc on a grid of nthgrd x nchgrd angular points */
double orc_vcord_raw(const double eul[3], const double rcom[3], const double rpt[3], const double *vtab,
                     int nrgrd, int nthgrd, int nchgrd, int chfold, double rvmax, double rvmin, double rvstep,
                     double *radret, double *theret, double *chiret)
{
  const double pi = MC_PI, small = 1.e-08, bo2ang = 0.529177249;
  double m[9], hatx[3], haty[3], hatz[3], R[3];
  orc_matpre(eul, m);
  for (int i = 0; i < 3; i++) {        /* rottrn with unit vectors: columns of rotmat */
    hatx[i] = m[i * 3 + 0];
    haty[i] = m[i * 3 + 1];
    hatz[i] = m[i * 3 + 2];
  }
  for (int i = 0; i < 3; i++) R[i] = rpt[i] - rcom[i];
  /* dotang vcord.f:176-188 */
  double da = dotprd(hatz, R) / (dnorm(hatz) * dnorm(R));
  if (da > 1.0) da = 1.0;
  if (da < -1.0) da = -1.0;
  double thewff = acos(da);
  double chiwff;
  if (fabs(dotprd(R, hatx)) < small) chiwff = pi / 2.0;
  else {
    double tanchi = dotprd(R, haty) / dotprd(R, hatx);
    chiwff = atan(fabs(tanchi));
  }
  double radwff = dnorm(R);
  double rdotx = dotprd(R, hatx), rdoty = dotprd(R, haty);
  double chir;
  if (rdotx >= 0.0 && rdoty >= 0.0) chir = chiwff;
  else if (rdotx < 0.0 && rdoty >= 0.0) chir = pi - chiwff;
  else if (rdotx < 0.0 && rdoty < 0.0) chir = pi + chiwff;
  else chir = 2 * pi - chiwff;
  if (chfold == 180) {
    chiwff = chir;
    if (chir > pi) chiwff = 2 * pi - chir;
  } else if (chfold == 360) {
    chiwff = chir;
  }
  if (radret) *radret = radwff;
  if (theret) *theret = thewff;
  if (chiret) *chiret = chir;
  radwff = radwff / bo2ang;
  thewff = thewff * 180.0 / pi;
  chiwff = chiwff * 180.0 / pi;
  double dth = 180.0 / (double)(nthgrd - 1), dch = (double)chfold / (double)(nchgrd - 1);
  return vcalc_raw(radwff, thewff / dth, chiwff / dch, rvmin, rvmax, rvstep, nrgrd, nthgrd, nchgrd, vtab);
}

double orc_vcord(const orc_ctx *c, const double eul[3], const double rcom[3], const double rpt[3],
                 double *radret, double *theret, double *chiret)
{
  return orc_vcord_raw(eul, rcom, rpt, c->vtab, c->rgrd, c->thgrd, c->chgrd, c->chfold, c->rvmax, c->rvmin,
                       c->rvstep, radret, theret, chiret);
}

/* rsrot -- rotden.f:218-286 (the reachable part: outputs written only for
 * iodevn == -1; for other values the routine returns without setting them) */
void orc_rsrot(const double e1[3], const double e2[3], double xrot, double yrot, double zrot,
               double tauC, int iodevn, double eoff, double *rho, double *erot)
{
  (void)eoff;
  const double wno2k = WNO2K;
  double tau = tauC / wno2k;
  double blist[3] = {1.0 / xrot, 1.0 / yrot, 1.0 / zrot};
  double m1[9], m2[9], dig[3];
  orc_matpre(e1, m1);
  orc_matpre(e2, m2);
  for (int i = 0; i < 3; i++) {
    double s = 0.0;
    for (int j = 0; j < 3; j++) s = s + m1[j * 3 + i] * m2[j * 3 + i];
    dig[i] = s;
  }
  double sumaxs = (blist[0] - blist[1] - blist[2]) * (1.0 - dig[0]) +
                  (blist[1] - blist[2] - blist[0]) * (1.0 - dig[1]) +
                  (blist[2] - blist[0] - blist[1]) * (1.0 - dig[2]);
  if (iodevn == -1) {
    *rho = sumaxs;
    double e = sumaxs / (4.0 * tau * tau);
    e = e + 1.5 / tau + 0.25 * (xrot + yrot + zrot);
    *erot = e / wno2k;
  }
}

/* rsline -- rotden.f:356-375 */
void orc_rsline(double brot, double dprd, double tauC, double *rho, double *erot)
{
  const double wno2k = WNO2K;
  double tau = tauC / wno2k;
  double r = (1.0 - dprd) / (2.0 * brot * tau);
  double e = (1.0 - r) / tau;
  *rho = -r;
  *erot = e / wno2k;
}

/* rottrn -- rotden.f:165-177 */
static void rottrn(const double m[9], const double rwf[3], double rsf[3], const double rcom[3])
{
  for (int i = 0; i < 3; i++) {
    double s = rcom[i];
    for (int j = 0; j < 3; j++) s = s + m[i * 3 + j] * rwf[j];
    rsf[i] = s;
  }
}

static double dist3(const double *a, const double *b)
{
  double s = 0.0;
  for (int i = 0; i < 3; i++) s = s + (a[i] - b[i]) * (a[i] - b[i]);
  return s;
}

/* caleng -- caleng_tip4p_gg.f:2-186: TIP4P-like water dimer energy in K.
 * kcal2k is an implicitly INTEGER parameter in the Fortran source (its name
 * starts with k), so the LJ term is scaled by 503, not 503.2189...; the
 * Coulomb terms are M-H, M-M and H-H only (caleng_tip4p_gg.f:179-181). */
double orc_caleng(const double com1[3], const double com2[3], const double e1[3], const double e2[3])
{
  const double qm = -1.04, qh = 0.520;
  const double br2ang = 0.52917721092, hr2k = 3.1577465e5;
  const double kcal2k = 503.0;
  const double ROwf[3] = {0.0, 0.0, 0.06562};
  const double RH1wf[3] = {0.7557, 0.0, -0.5223};
  const double RH2wf[3] = {-0.7557, 0.0, -0.5223};
  const double RMwf[3] = {0.0, 0.0, -0.08438};
  double m1[9], m2[9];
  double O1[3], M1[3], H11[3], H21[3], O2[3], M2[3], H12[3], H22[3];
  orc_matpre(e1, m1);
  rottrn(m1, ROwf, O1, com1);
  rottrn(m1, RMwf, M1, com1);
  rottrn(m1, RH1wf, H11, com1);
  rottrn(m1, RH2wf, H21, com1);
  orc_matpre(e2, m2);
  rottrn(m2, ROwf, O2, com2);
  rottrn(m2, RMwf, M2, com2);
  rottrn(m2, RH1wf, H12, com2);
  rottrn(m2, RH2wf, H22, com2);
  double roo = 0.0, rmm = 0.0;
  for (int i = 0; i < 3; i++) {
    roo = roo + (O1[i] - O2[i]) * (O1[i] - O2[i]);
    rmm = rmm + (M1[i] - M2[i]) * (M1[i] - M2[i]);
  }
  rmm = sqrt(rmm);
  double roo4 = roo * roo;
  double roo6 = roo4 * roo;
  double roo12 = roo6 * roo6;
  roo = sqrt(roo);
  const double A = 6.e5, B = 610.0;
  double v_o2lj = A / roo12 - B / roo6;
  double rhm1 = sqrt(dist3(M1, H12)), rhm2 = sqrt(dist3(M1, H22));
  double rhm3 = sqrt(dist3(M2, H11)), rhm4 = sqrt(dist3(M2, H21));
  double rhh1 = sqrt(dist3(H11, H12)), rhh2 = sqrt(dist3(H11, H22));
  double rhh3 = sqrt(dist3(H21, H12)), rhh4 = sqrt(dist3(H21, H22));
  double v_mh = qm * qh * (1.0 / rhm1 + 1.0 / rhm2 + 1.0 / rhm3 + 1.0 / rhm4);
  double v_hh = qh * qh * (1.0 / rhh1 + 1.0 / rhh2 + 1.0 / rhh3 + 1.0 / rhh4);
  double v_mm = qm * qm * (1.0 / rmm);
  return v_o2lj * kcal2k + (v_mh + v_mm + v_hh) * hr2k * br2ang;
}

/* vspher -- vspher.f:12-544: r (A) -> bohr with a single-precision
 * conversion constant, clamp, linear interpolation on the supplied table */
double orc_vspher_raw(double r, const double *tab, int n, double r0, double rmax, double rstep)
{
  const double ang2bo = (double)0.5291772f;
  int maxrpt = n - 1;
  r = r / ang2bo;
  if (r < r0) r = r0;
  if (r > rmax) r = rmax;
  int ir = (int)((r - r0) / rstep);
  if (ir > maxrpt) ir = maxrpt;
  double v0 = tab[ir];
  double gradr, delr;
  if (ir == maxrpt) { gradr = 0.0; delr = 0.0; }
  else {
    gradr = (tab[ir + 1] - v0) / rstep;
    delr = r - (r0 + ir * rstep);
  }
  return v0 + gradr * delr;
}

double orc_vspher(const orc_ctx *c, double r)
{
  return orc_vspher_raw(r, c->sph, c->nsph, c->sph_r0, c->sph_rmax, c->sph_rstep);
}

/* --------------------------------------------------------------- energies */

static inline double crd(const double *a, long nb, int d, long i) { return a[(long)d * nb + i]; }

static void euler_at(const orc_ctx *c, const double *ang, long nb, long tm, double e[3])
{
  e[PHI] = ang[PHI * nb + tm];
  e[CTH] = acos(ang[CTH * nb + tm]);
  e[CHI] = ang[CHI * nb + tm];
  (void)c;
}

/* WorldLine -- mc_qworm.cc:553-575: whether bead pt of the worm type's atom
 * (index within the type) lies on a world line, not in the gap between
 * masha and ira */
static int world_line(const orc_ctx *c, int atom, int pt)
{
  int wline = 1;
  if (atom == c->atom_m || atom == c->atom_i) {
    if (c->atom_i != c->atom_m || c->ira > c->masha) {
      if ((atom == c->atom_m && pt < c->masha) || (atom == c->atom_i && pt > c->ira)) wline = 0;
    } else {
      if (pt > c->ira && pt < c->masha) wline = 0;
    }
  }
  return wline;
}

/* the partner test of PotEnergy / PotRotEnergy / PotRotE3D with an open
 * worm (mc_piqmc.cc:1226-1227, 1816-1817, 2000-2001, 2082-2083) */
static int partner_on_line(const orc_ctx *c, int atom1, int it)
{
  int type1 = c->mctype[atom1];
  if (c->worm_on && c->wexists && c->wtype == type1) return world_line(c, atom1 - c->offset[type1] / c->P, it);
  return 1;
}

/* one (atom0, atom1, it) term of PotEnergy -- mc_piqmc.cc:1824-1958 */
static double pair_term(const orc_ctx *c, int atom0, int atom1, const double *pos, int it)
{
  if (!partner_on_line(c, atom1, it)) return 0.0;
  const pimc_system *s = &c->sys;
  long nb = (long)c->na * c->P;
  int P = c->P, R = c->R;
  int type0 = c->mctype[atom0], type1 = c->mctype[atom1];
  int mol0 = s->type[type0].molecule, mol1 = s->type[type1].molecule;
  long offset0 = (long)P * atom0, offset1 = (long)P * atom1;
  long t0 = offset0 + it, t1 = offset1 + it;
  double dr[3], dr2 = 0.0;
  for (int id = 0; id < NDIM; id++) {
    dr[id] = (crd(pos, nb, id, t0) - crd(c->coords, nb, id, t1));
    if (s->minimage) dr[id] -= (s->box[id] * rint(dr[id] / s->box[id]));
    dr2 += (dr[id] * dr[id]);
  }
  double r = sqrt(dr2);
  if (mol0 == PIMC_LINEAR || mol1 == PIMC_LINEAR) {
    int sgn = 1;
    long tm = offset1 + it / R;
    if (mol0 == PIMC_LINEAR) { sgn = -1; tm = offset0 + it / R; }
    double cost = 0.0;
    for (int id = 0; id < NDIM; id++) cost += (c->cosine[id * nb + tm] * dr[id]);
    cost /= r;
    cost *= sgn;
    return orc_lpot2d(c, r, cost);
  } else if ((mol0 == PIMC_NONLINEAR || mol1 == PIMC_NONLINEAR) && s->ispher == 0 && mol0 != mol1) {
    double RCOM[3], Rpt[3], E[3];
    long tm;
    if (mol0 == PIMC_NONLINEAR) {
      tm = offset0 + it / R;
      for (int id = 0; id < 3; id++) { RCOM[id] = crd(pos, nb, id, t0); Rpt[id] = crd(c->coords, nb, id, t1); }
    } else {
      tm = offset1 + it / R;
      for (int id = 0; id < 3; id++) { Rpt[id] = crd(pos, nb, id, t0); RCOM[id] = crd(c->coords, nb, id, t1); }
    }
    euler_at(c, c->angles, nb, tm, E);
    return orc_vcord(c, E, RCOM, Rpt, NULL, NULL, NULL);
  } else if ((mol0 == PIMC_NONLINEAR || mol1 == PIMC_NONLINEAR) && s->ispher == 1 && mol0 != mol1) {
    return orc_vspher(c, r);
  } else if (mol0 == PIMC_NONLINEAR && mol1 == PIMC_NONLINEAR && s->type[c->imtype].numb > 1) {
    double com1[3], com2[3], E1[3], E2[3];
    for (int id = 0; id < 3; id++) { com1[id] = crd(pos, nb, id, t0); com2[id] = crd(c->coords, nb, id, t1); }
    euler_at(c, c->angles, nb, offset0 + it / R, E1);
    euler_at(c, c->angles, nb, offset1 + it / R, E2);
    return orc_caleng(com1, com2, E1, E2);
  }
  return orc_spot1d(c, r);
}

/* PotEnergy(atom0, pos, it) -- mc_piqmc.cc:1796-1965 */
double orc_pot_energy_slice(const orc_ctx *c, int atom0, const double *pos, int it)
{
  double spot = 0.0;
  for (int atom1 = 0; atom1 < c->na; atom1++)
    if (atom1 != atom0) spot += pair_term(c, atom0, atom1, pos, it);
  return spot;
}

/* PotEnergy(atom0, pos) -- mc_piqmc.cc:1201-1383 (per partner, sum over slices) */
static double pot_energy_path_nt(const orc_ctx *c, int atom0, const double *pos, int nthreads)
{
  double spot = 0.0;
  for (int atom1 = 0; atom1 < c->na; atom1++)
    if (atom1 != atom0) {
      double spot_pair = 0.0;
#pragma omp parallel for reduction(+ : spot_pair) num_threads(nthreads) if (nthreads > 1)
      for (int it = 0; it < c->P; it++) spot_pair += pair_term(c, atom0, atom1, pos, it);
      spot += spot_pair;
    }
  return spot;
}

double orc_pot_energy_path(const orc_ctx *c, int atom0, const double *pos)
{
  return pot_energy_path_nt(c, atom0, pos, 1);
}

/* PotRotEnergy -- mc_piqmc.cc:1967-2044 */
double orc_pot_rot_energy(const orc_ctx *c, int atom0, const double *cosine, int it)
{
  long nb = (long)c->na * c->P;
  int type0 = c->mctype[atom0];
  long offset0 = (long)atom0 * c->P;
  double spot = 0.0;
  for (int atom1 = 0; atom1 < c->na; atom1++)
    if (atom1 != atom0 && partner_on_line(c, atom1, it)) {
      long offset1 = (long)atom1 * c->P;
      long t0 = offset0 + it, t1 = offset1 + it;
      double dr[3], dr2 = 0.0;
      for (int id = 0; id < NDIM; id++) {
        dr[id] = (crd(c->coords, nb, id, t0) - crd(c->coords, nb, id, t1));
        dr2 += (dr[id] * dr[id]);
      }
      double r = sqrt(dr2);
      int sgn = -1;
      long tm = offset0 + it / c->R;
      double cost = 0.0;
      for (int id = 0; id < NDIM; id++) cost += (cosine[id * nb + tm] * dr[id]);
      cost /= r;
      cost *= sgn;
      spot += orc_lpot2d(c, r, cost);
      (void)type0;
    }
  return spot;
}

/* PotRotE3D -- mc_piqmc.cc:2046-2151 (vcord for atoms regardless of ISPHER,
 * caleng for the other rotors with their current angles) */
double orc_pot_rot_e3d(const orc_ctx *c, int atom0, const double eul[3], int it)
{
  long nb = (long)c->na * c->P;
  long offset0 = (long)atom0 * c->P;
  double spot = 0.0;
  for (int atom1 = 0; atom1 < c->na; atom1++)
    if (atom1 != atom0 && partner_on_line(c, atom1, it)) {
      long offset1 = (long)atom1 * c->P;
      int type1 = c->mctype[atom1];
      long t0 = offset0 + it, t1 = offset1 + it;
      if (type1 != c->imtype) {
        double RCOM[3], Rpt[3];
        for (int id = 0; id < 3; id++) { RCOM[id] = crd(c->coords, nb, id, t0); Rpt[id] = crd(c->coords, nb, id, t1); }
        spot += orc_vcord(c, eul, RCOM, Rpt, NULL, NULL, NULL);
      } else {
        double com1[3], com2[3], E2[3];
        for (int id = 0; id < 3; id++) { com1[id] = crd(c->coords, nb, id, t0); com2[id] = crd(c->coords, nb, id, t1); }
        euler_at(c, c->angles, nb, offset1 + it / c->R, E2);
        spot += orc_caleng(com1, com2, eul, E2);
      }
    }
  return spot;
}

/* ------------------------------------------------------------------ moves */

static double take(orc_stream *s, int *overrun)
{
  if (s->pos >= s->n) { *overrun = 1; return 0.5; }
  return s->v[s->pos++];
}

/* internal generator: splitmix64 of (seed, stream, counter) -> [0,1) */
static uint64_t mix64(uint64_t z)
{
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
static double u01_key(uint64_t seed, uint64_t stream, uint64_t ctr)
{
  uint64_t z = mix64(seed ^ mix64(stream * 0x632BE59BD9B4E019ull + ctr));
  return ((double)(z >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}

/* a random source: replay streams or the internal generator */
typedef struct {
  orc_replay *rp;
  orc_ctx *c;
} src_t;

static double s_u(src_t *s, int which)  /* which: 1 rnd1, 2 rnd2, 3 rnd3, 4 runif */
{
  if (s->rp) {
    orc_stream *st = which == 1 ? &s->rp->u1 : which == 2 ? &s->rp->u2 : which == 3 ? &s->rp->u3 : &s->rp->urot;
    return take(st, &s->rp->overrun);
  }
  return u01_key(s->c->seed, (uint64_t)which, s->c->ctr[which]++);
}

static double s_gauss_x1(src_t *s)
{
  if (s->rp) return take(&s->rp->gauss, &s->rp->overrun);
  double r1 = u01_key(s->c->seed, 8, s->c->ctr[5]++);
  double r2 = u01_key(s->c->seed, 9, s->c->ctr[6]++);
  return sqrt(-log(r1)) * cos(2.0 * M_PI * r2);     /* mc_randg.cc:144 */
}

/* MCMolecularMove -- mc_piqmc.cc:54-102 */
static int molecular_move(orc_ctx *c, int type, src_t *src, double *dv_out, int *acc_out, int nthreads)
{
  long nb = (long)c->na * c->P;
  int numb = c->sys.type[type].numb;
  double disp[3];
  for (int atom = 0; atom < numb; atom++) {
    long offset = c->offset[type] + (long)c->P * atom;
    int gatom = (int)(offset / c->P);
    for (int id = 0; id < NDIM; id++) disp[id] = c->sys.type[type].mcstep * (s_u(src, 1) - 0.5);
    for (int id = 0; id < NDIM; id++)
      for (int it = 0; it < c->P; it++) {
        c->newc[id * nb + offset + it] = c->coords[id * nb + offset + it];
        c->newc[id * nb + offset + it] += disp[id];
      }
    double deltav = 0.0;
    deltav += (pot_energy_path_nt(c, gatom, c->newc, nthreads) - pot_energy_path_nt(c, gatom, c->coords, nthreads));
    int acc = 0;
    if (deltav < 0.0) acc = 1;
    else if (exp(-deltav * c->tau) > s_u(src, 2)) acc = 1;
    c->total[type * 3 + MCMOLEC] += 1.0;
    if (dv_out) dv_out[atom] = deltav;
    if (acc_out) acc_out[atom] = acc;
    if (acc) {
      c->accep[type * 3 + MCMOLEC] += 1.0;
      for (int id = 0; id < NDIM; id++)
        for (int it = 0; it < c->P; it++) c->coords[id * nb + offset + it] = c->newc[id * nb + offset + it];
    }
  }
  return PIMC_OK;
}

int orc_molecular_move(orc_ctx *c, int type, orc_replay *rp, double *dv_out, int *acc_out)
{
  src_t s = {rp, c};
  return molecular_move(c, type, &s, dv_out, acc_out, 1);
}

/* MCMolecularMoveExchange -- mc_piqmc.cc:104-192 (one displacement per
 * permutation cycle, members tested in cycle order; dv_out/acc_out per cycle
 * leader atom) */
int orc_molecular_move_exchange(orc_ctx *c, int type, orc_replay *rp, double *dv_out, int *acc_out)
{
  src_t src = {rp, c};
  long nb = (long)c->na * c->P;
  int numb = c->sys.type[type].numb;
  double disp[3];
  int acc = 0;
  for (int atom = 0; atom < numb; atom++) c->pflags[atom] = 0;
  for (int atom = 0; atom < numb; atom++) {
    if (dv_out) dv_out[atom] = 0.0;
    if (acc_out) acc_out[atom] = -1;
  }
  for (int atom = 0; atom < numb; atom++)
    if (c->pflags[atom] == 0) {
      int amax = 0;
      c->atom_list[amax++] = atom;
      int patom = c->pindex[atom];
      while (patom != atom) {
        c->atom_list[amax++] = patom;
        c->pflags[patom] = 1;
        patom = c->pindex[patom];
      }
      for (int id = 0; id < NDIM; id++) disp[id] = c->sys.type[type].mcstep * (s_u(&src, 1) - 0.5);
      double dvsum = 0.0;
      for (int ia = 0; ia < amax; ia++) {
        long offset = c->offset[type] + (long)c->P * c->atom_list[ia];
        int gatom = (int)(offset / c->P);
        for (int id = 0; id < NDIM; id++)
          for (int it = 0; it < c->P; it++) {
            c->newc[id * nb + offset + it] = c->coords[id * nb + offset + it];
            c->newc[id * nb + offset + it] += disp[id];
          }
        double deltav = 0.0;
        deltav += (orc_pot_energy_path(c, gatom, c->newc) - orc_pot_energy_path(c, gatom, c->coords));
        dvsum = deltav;
        acc = 0;
        if (deltav < 0.0) acc = 1;
        else if (exp(-deltav * c->tau) > s_u(&src, 2)) acc = 1;
        if (!acc) break;
      }
      c->total[type * 3 + MCMOLEC] += 1.0;
      if (dv_out) dv_out[atom] = dvsum;
      if (acc_out) acc_out[atom] = acc;
      if (acc) {
        c->accep[type * 3 + MCMOLEC] += 1.0;
        for (int ia = 0; ia < amax; ia++) {
          long offset = c->offset[type] + (long)c->P * c->atom_list[ia];
          for (int id = 0; id < NDIM; id++)
            for (int it = 0; it < c->P; it++) c->coords[id * nb + offset + it] = c->newc[id * nb + offset + it];
        }
      }
    }
  return (rp && rp->overrun) ? PIMC_ERR_BAD_ARG : PIMC_OK;
}

/* MCBisectionMove / MCBisectionMoveExchange -- mc_piqmc.cc:194-294, 296-419.
 * With exch == 0 the offsets never switch (identity permutation path). */
static int bisection_move(orc_ctx *c, int type, int time0, src_t *src, double *ds_out, int *lvl_out, int exch)
{
  long nb = (long)c->na * c->P;
  int P = c->P;
  int numb = c->sys.type[type].numb;
  double mclambda = c->sys.type[type].lambda;
  int mclevels = c->sys.type[type].levels;
  int seg_size = c->mlsegm[type];
  for (int atom = 0; atom < numb; atom++) {
    long offset0 = c->offset[type] + (long)P * atom;
    long offset1 = offset0;
    int time1 = time0 + seg_size;
    int timep = time1 % P;
    if (exch && timep != time1) offset1 = c->offset[type] + (long)P * c->pindex[atom];
    for (int id = 0; id < NDIM; id++) {
      c->newc[id * nb + offset0 + time0] = c->coords[id * nb + offset0 + time0];
      c->newc[id * nb + offset1 + timep] = c->coords[id * nb + offset1 + timep];
    }
    double bnorm = 1.0 / (mclambda * c->tau);
    int acc = 0, passed = 0;
    double pot0 = 0.0, pot1 = 0.0;
    for (int level = 0; level < mclevels; level++) {
      int level_seg_size = (int)pow(2.0, (mclevels - level));
      double bkin_norm = bnorm / (double)level_seg_size;
      double bpot_norm = c->tau * (double)(level_seg_size / 2);
      pot1 = pot0;
      pot0 = 0.0;
      int t0, t1, t2 = 0;
      do {
        t0 = t2;
        t2 = t0 + level_seg_size;
        t1 = (t0 + t2) / 2;
        int pt0 = (time0 + t0) % P, pt1 = (time0 + t1) % P, pt2 = (time0 + t2) % P;
        long off0 = offset0, off1 = offset0, off2 = offset0;
        if (pt0 != (time0 + t0)) off0 = offset1;
        if (pt1 != (time0 + t1)) off1 = offset1;
        if (pt2 != (time0 + t2)) off2 = offset1;
        for (int id = 0; id < NDIM; id++) {
          c->newc[id * nb + off1 + pt1] = 0.5 * (c->newc[id * nb + off0 + pt0] + c->newc[id * nb + off2 + pt2]);
          double x1 = s_gauss_x1(src);
          c->newc[id * nb + off1 + pt1] += x1 / sqrt(bkin_norm);     /* gauss() mc_randg.cc:149 */
        }
        int g0 = (int)(off0 / P), g1 = (int)(off1 / P);
        pot0 += (orc_pot_energy_slice(c, g1, c->newc, pt1) - orc_pot_energy_slice(c, g1, c->coords, pt1));
        if (t0 != 0)
          pot0 += (orc_pot_energy_slice(c, g0, c->newc, pt0) - orc_pot_energy_slice(c, g0, c->coords, pt0));
      } while (t2 < seg_size);
      double deltav = (pot0 - 2.0 * pot1);
      deltav *= bpot_norm;
      if (ds_out) ds_out[atom * mclevels + level] = deltav;
      acc = 0;
      if (deltav < 0.0) acc = 1;
      else if (exp(-deltav) > s_u(src, 3)) acc = 1;
      if (!acc) break;
      passed++;
    }
    if (lvl_out) lvl_out[atom] = passed;
    c->total[type * 3 + MCMULTI] += 1.0;
    if (acc) {
      c->accep[type * 3 + MCMULTI] += 1.0;
      for (int id = 0; id < NDIM; id++)
        for (int it = time0; it <= time1; it++) {
          int pit = it % P;
          long offset = offset0;
          if (pit != it) offset = offset1;
          c->coords[id * nb + offset + pit] = c->newc[id * nb + offset + pit];
        }
    }
  }
  return PIMC_OK;
}

int orc_bisection_move(orc_ctx *c, int type, int time, orc_replay *rp, double *ds_out, int *lvl_out)
{
  src_t s = {rp, c};
  int st = bisection_move(c, type, time, &s, ds_out, lvl_out, 0);
  return (rp && rp->overrun) ? PIMC_ERR_BAD_ARG : st;
}

int orc_bisection_move_exchange(orc_ctx *c, int type, int time0, orc_replay *rp, double *ds_out, int *lvl_out)
{
  src_t s = {rp, c};
  int st = bisection_move(c, type, time0, &s, ds_out, lvl_out, 1);
  return (rp && rp->overrun) ? PIMC_ERR_BAD_ARG : st;
}

/* MCRotLinStep -- mc_piqmc.cc:781-936 (uses c->newc rows as the proposal
 * buffer like the reference's newcoords) */
static int rot_lin_step(orc_ctx *c, int it1, long offset, int gatom, const double u[3],
                        double *rd_out, int *acc_out, double *newc, double *chunk_tot, double *chunk_acp)
{
  long nb = (long)c->na * c->P;
  int Q = c->Q;
  double step = c->sys.rtstep;
  int it0 = it1 - 1, it2 = it1 + 1;
  if (it0 < 0) it0 += Q;
  if (it2 >= Q) it2 -= Q;
  long t0 = offset + it0, t1 = offset + it1, t2 = offset + it2;
  double cost = c->angles[CTH * nb + t1];
  double phi = c->angles[PHI * nb + t1];
  cost += (step * (u[0] - 0.5));
  phi += (step * (u[1] - 0.5));
  if (cost > 1.0) cost = 2.0 - cost;
  if (cost < -1.0) cost = -2.0 - cost;
  double sint = sqrt(1.0 - cost * cost);
  newc[0 * nb + t1] = sint * cos(phi);
  newc[1 * nb + t1] = sint * sin(phi);
  newc[2 * nb + t1] = cost;
  double p0 = 0.0, p1 = 0.0;
  for (int id = 0; id < NDIM; id++) {
    p0 += (c->cosine[id * nb + t0] * c->cosine[id * nb + t1]);
    p1 += (c->cosine[id * nb + t1] * c->cosine[id * nb + t2]);
  }
  int rdt = c->sys.rot_den_type;
  double dens_old = 0.0, rho1, rho2, erot;
  if (rdt == 0) dens_old = orc_srotdens(c, p0, 0) * orc_srotdens(c, p1, 0);
  else {
    orc_rsline(c->sys.rot_abc[0], p0, c->rot_tau, &rho1, &erot);
    orc_rsline(c->sys.rot_abc[0], p1, c->rot_tau, &rho2, &erot);
    dens_old = rho1 + rho2;
  }
  if (fabs(dens_old) < RZERO) dens_old = 0.0;
  if (dens_old < 0.0 && rdt == 0) return PIMC_ERR_NEG_DENSITY;
  double pot_old = 0.0;
  int itr0 = it1 * c->R, itr1 = itr0 + c->R;
  for (int it = itr0; it < itr1; it++) pot_old += orc_pot_rot_energy(c, gatom, c->cosine, it);
  p0 = 0.0; p1 = 0.0;
  for (int id = 0; id < NDIM; id++) {
    p0 += (c->cosine[id * nb + t0] * newc[id * nb + t1]);
    p1 += (newc[id * nb + t1] * c->cosine[id * nb + t2]);
  }
  double dens_new = 0.0;
  if (rdt == 0) dens_new = orc_srotdens(c, p0, 0) * orc_srotdens(c, p1, 0);
  else {
    orc_rsline(c->sys.rot_abc[0], p0, c->rot_tau, &rho1, &erot);
    orc_rsline(c->sys.rot_abc[0], p1, c->rot_tau, &rho2, &erot);
    dens_new = rho1 + rho2;
  }
  if (fabs(dens_new) < RZERO) dens_new = 0.0;
  if (dens_new < 0.0 && rdt == 0) return PIMC_ERR_NEG_DENSITY;
  double pot_new = 0.0;
  for (int it = itr0; it < itr1; it++) pot_new += orc_pot_rot_energy(c, gatom, newc, it);
  double rd;
  if (rdt == 0) {
    if (dens_old > RZERO) rd = dens_new / dens_old;
    else rd = 1.0;
    rd *= exp(-c->tau * (pot_new - pot_old));
  } else {
    rd = dens_new - dens_old - c->tau * (pot_new - pot_old);
  }
  int acc = 0;
  if (rdt == 0) {
    if (rd > 1.0) acc = 1;
    else if (rd > u[2]) acc = 1;
  } else {
    if (rd > 0.0) acc = 1;
    else if (rd > log(u[2])) acc = 1;
  }
  *chunk_tot += 1.0;
  if (rd_out) *rd_out = rd;
  if (acc_out) *acc_out = acc;
  if (acc) {
    *chunk_acp += 1.0;
    c->angles[CTH * nb + t1] = cost;
    c->angles[PHI * nb + t1] = phi;
    for (int id = 0; id < NDIM; id++) c->cosine[id * nb + t1] = newc[id * nb + t1];
  }
  return PIMC_OK;
}

/* MCRot3Dstep -- mc_piqmc.cc:938-1199 */
static int rot_3d_step(orc_ctx *c, int it1, long offset, int gatom, const double u[4],
                       double *rd_out, int *acc_out, double *newc, double *chunk_tot, double *chunk_acp)
{
  long nb = (long)c->na * c->P;
  int Q = c->Q;
  double step = c->sys.rtstep;
  const double pi2 = 2.0 * M_PI;
  int it0 = it1 - 1, it2 = it1 + 1;
  if (it0 < 0) it0 += Q;
  if (it2 >= Q) it2 -= Q;
  long t0 = offset + it0, t1 = offset + it1, t2 = offset + it2;
  double cost = c->angles[CTH * nb + t1];
  double phi = c->angles[PHI * nb + t1];
  double chi = c->angles[CHI * nb + t1];
  cost += (step * (u[0] - 0.5));
  phi += 2.0 * M_PI * (step * (u[1] - 0.5));
  chi += 2.0 * M_PI * (step * (u[2] - 0.5));
  if (phi < 0.0) phi = pi2 + phi;
  if (chi < 0.0) chi = pi2 + chi;
  phi = fmod(phi, pi2);
  chi = fmod(chi, pi2);
  if (cost > 1.0) cost = 2.0 - cost;
  if (cost < -1.0) cost = -2.0 - cost;
  newc[PHI * nb + t1] = phi;
  newc[CHI * nb + t1] = chi;
  newc[CTH * nb + t1] = cost;
  int rdt = c->sys.rot_den_type;
  double rho = 0.0, erot = 0.0, esq = 0.0, rel[3];
  double E1[3], E2[3];
  const double *ang = c->angles;
  const double *X = c->sys.rot_abc;
#define EUL(dst, arr, t) do { dst[0] = (arr)[PHI * nb + (t)]; dst[1] = acos((arr)[CTH * nb + (t)]); dst[2] = (arr)[CHI * nb + (t)]; } while (0)
  EUL(E1, ang, t0);
  EUL(E2, ang, t1);
  if (rdt == 0) { if (orc_rotden(c, E1, E2, rel, &rho, &erot, &esq)) return PIMC_ERR_GRID_RANGE; }
  else orc_rsrot(E1, E2, X[0], X[1], X[2], c->rot_tau, c->sys.rot_odevn, c->sys.rot_eoff, &rho, &erot);
  double dens_old = rho, rhoold = rho;
  EUL(E1, ang, t1);
  EUL(E2, ang, t2);
  if (rdt == 0) { if (orc_rotden(c, E1, E2, rel, &rho, &erot, &esq)) return PIMC_ERR_GRID_RANGE; }
  else orc_rsrot(E1, E2, X[0], X[1], X[2], c->rot_tau, c->sys.rot_odevn, c->sys.rot_eoff, &rho, &erot);
  dens_old = dens_old * rho;
  rhoold = rhoold + rho;
  if (fabs(dens_old) < RZERO) dens_old = 0.0;
  if (dens_old < 0.0) dens_old = fabs(dens_old);
  double pot_old = 0.0;
  int itr0 = it1 * c->R, itr1 = itr0 + c->R;
  for (int it = itr0; it < itr1; it++) pot_old += orc_pot_rot_e3d(c, gatom, E1, it);
  EUL(E1, ang, t0);
  EUL(E2, newc, t1);
  if (rdt == 0) { if (orc_rotden(c, E1, E2, rel, &rho, &erot, &esq)) return PIMC_ERR_GRID_RANGE; }
  else orc_rsrot(E1, E2, X[0], X[1], X[2], c->rot_tau, c->sys.rot_odevn, c->sys.rot_eoff, &rho, &erot);
  double dens_new = rho, rhonew = rho;
  EUL(E1, newc, t1);
  EUL(E2, ang, t2);
  if (rdt == 0) { if (orc_rotden(c, E1, E2, rel, &rho, &erot, &esq)) return PIMC_ERR_GRID_RANGE; }
  else orc_rsrot(E1, E2, X[0], X[1], X[2], c->rot_tau, c->sys.rot_odevn, c->sys.rot_eoff, &rho, &erot);
#undef EUL
  dens_new = dens_new * rho;
  rhonew = rhonew + rho;
  if (fabs(dens_new) < RZERO) dens_new = 0.0;
  if (dens_new < 0.0) dens_new = fabs(dens_new);
  double pot_new = 0.0;
  for (int it = itr0; it < itr1; it++) pot_new += orc_pot_rot_e3d(c, gatom, E1, it);
  double rd;
  if (rdt == 0) {
    if (dens_old > RZERO) rd = dens_new / dens_old;
    else rd = 1.0;
    rd *= exp(-c->tau * (pot_new - pot_old));
  } else {
    rd = (rhonew - rhoold) / (4.0 * (c->rot_tau / WNO2K));
    rd -= c->tau * (pot_new - pot_old);
  }
  int acc = 0;
  if (rdt == 0) {
    if (rd > 1.0) acc = 1;
    else if (rd > u[3]) acc = 1;
  } else {
    if (rd > 0.0) acc = 1;
    else if (rd > log(u[3])) acc = 1;
  }
  *chunk_tot += 1.0;
  if (rd_out) *rd_out = rd;
  if (acc_out) *acc_out = acc;
  if (acc) {
    *chunk_acp += 1.0;
    c->angles[CTH * nb + t1] = cost;
    c->angles[PHI * nb + t1] = phi;
    c->angles[CHI * nb + t1] = chi;
    double sint = sqrt(1.0 - cost * cost);
    c->cosine[0 * nb + t1] = sint * cos(phi);
    c->cosine[1 * nb + t1] = sint * sin(phi);
    c->cosine[2 * nb + t1] = cost;
  }
  return PIMC_OK;
}

int orc_rot_lin_step(orc_ctx *c, int it1, int rotor, const double u[3], double *rd, int *acc)
{
  int type = c->imtype;
  long offset = c->offset[type] + (long)c->P * rotor;
  double tot = 0, acp = 0;
  int st = rot_lin_step(c, it1, offset, (int)(offset / c->P), u, rd, acc, c->newc, &tot, &acp);
  c->total[type * 3 + MCROTAT] += tot;
  c->accep[type * 3 + MCROTAT] += acp;
  return st;
}

int orc_rot_3d_step(orc_ctx *c, int it1, int rotor, const double u[4], double *rd, int *acc)
{
  int type = c->imtype;
  long offset = c->offset[type] + (long)c->P * rotor;
  double tot = 0, acp = 0;
  int st = rot_3d_step(c, it1, offset, (int)(offset / c->P), u, rd, acc, c->newc, &tot, &acp);
  c->total[type * 3 + MCROTAT] += tot;
  c->accep[type * 3 + MCROTAT] += acp;
  return st;
}

/* MCRotationsMove -- mc_piqmc.cc:421-517: even slices, then odd slices; the
 * uniforms are consumed in serial slice order (3 per slice) */
int orc_rotations_move(orc_ctx *c, int type, orc_replay *rp, double *rd_out, int *acc_out)
{
  src_t src = {rp, c};
  long offset = c->offset[type];
  int gatom = (int)(offset / c->P);
  double tot = 0, acp = 0;
  for (int ph = 0; ph < 2; ph++)
    for (int it = ph; it < c->Q; it += 2) {
      double u[3] = {s_u(&src, 4), s_u(&src, 4), s_u(&src, 4)};
      int st = rot_lin_step(c, it, offset, gatom, u, rd_out ? &rd_out[it] : NULL, acc_out ? &acc_out[it] : NULL,
                            c->newc, &tot, &acp);
      if (st) return st;
    }
  c->total[type * 3 + MCROTAT] += tot;
  c->accep[type * 3 + MCROTAT] += acp;
  return (rp && rp->overrun) ? PIMC_ERR_BAD_ARG : PIMC_OK;
}

/* MCRotations3D -- mc_piqmc.cc:692-779: even slices then odd; rotors in
 * order inside a slice; 4 uniforms per (slice, rotor) in serial order */
int orc_rotations_3d(orc_ctx *c, int type, orc_replay *rp, double *rd_out, int *acc_out)
{
  src_t src = {rp, c};
  int nrot = c->sys.type[type].numb;
  double tot = 0, acp = 0;
  for (int ph = 0; ph < 2; ph++)
    for (int it = ph; it < c->Q; it += 2)
      for (int a = 0; a < nrot; a++) {
        long offset = c->offset[type] + (long)c->P * a;
        double u[4] = {s_u(&src, 4), s_u(&src, 4), s_u(&src, 4), s_u(&src, 4)};
        long k = (long)it * nrot + a;
        int st = rot_3d_step(c, it, offset, (int)(offset / c->P), u, rd_out ? &rd_out[k] : NULL,
                             acc_out ? &acc_out[k] : NULL, c->newc, &tot, &acp);
        if (st) return st;
      }
  c->total[type * 3 + MCROTAT] += tot;
  c->accep[type * 3 + MCROTAT] += acp;
  return (rp && rp->overrun) ? PIMC_ERR_BAD_ARG : PIMC_OK;
}

/* ------------------------------------------------------------- estimators */

/* GetKinEnergy -- mc_estim.cc:876-937 (primitive estimator, boson wrap) */
double orc_kin_energy(const orc_ctx *c)
{
  long nb = (long)c->na * c->P;
  int P = c->P, numb = 0;
  double r2avr = 0.0;
  for (int atom = 0; atom < c->na; atom++) {
    numb++;
    int type = c->mctype[atom];
    long offset0 = (long)P * atom;
    int gatom = c->offset[type] / P;
    double sum = 0.0;
    for (int it = 0; it < P; it++) {
      long t0 = offset0 + it;
      long offset1 = offset0;
      if (c->sys.type[type].stat == PIMC_BOSE && (it + 1) == P) offset1 = (long)P * (gatom + c->pindex[atom - gatom]);
      long t1 = offset1 + (it + 1) % P;
      for (int d = 0; d < NDIM; d++) {
        double dr = c->coords[d * nb + t0] - c->coords[d * nb + t1];
        if (c->sys.minimage) dr -= (c->sys.box[d] * rint(dr / c->sys.box[d]));
        sum += (dr * dr);
      }
    }
    r2avr += (sum / (4.0 * c->beta * c->sys.type[type].lambda));
  }
  return (double)P * c->sys.temperature * (0.5 * (double)(NDIM * numb) - r2avr);
}

/* bin_1Ddensity / bin_2Ddensity / bin_3Ddensity -- mc_estim.cc:1233-1286,
 * with the grids of densities_init (mc_estim.cc:223-255): MC_BINSR radial
 * bins on [MIN_RADIUS, MAX_RADIUS), theta bins of pi/(MC_BINST-1), chi bins
 * of 2 pi/(MC_BINSC-1) (mc_estim.cc:25-30) */
static void bin_density(double *gr1d, double *gr2d, double *gr3d, int kind, int dtype, double r, double a, double b)
{
  const double drad = (PIMC_DENS_MAX_RADIUS - PIMC_DENS_MIN_RADIUS) / (double)PIMC_BINSR;
  const double dth = M_PI / (double)(PIMC_BINST - 1), dch = 2.0 * M_PI / (double)(PIMC_BINSC - 1);
  int br = (int)floor((r - PIMC_DENS_MIN_RADIUS) / drad);
  if (br >= PIMC_BINSR || br < 0) return;
  if (kind == 1) {
    if (gr1d) gr1d[(long)dtype * PIMC_BINSR + br] += 1.0;
  } else if (kind == 2) {
    double theta = acos(a);
    int bt = (int)floor(theta / dth);
    if (bt < PIMC_BINST && bt >= 0 && gr2d) gr2d[((long)dtype * PIMC_BINSR + br) * PIMC_BINST + bt] += 1.0;
  } else {
    int bt = (int)floor(a / dth);
    if (bt < PIMC_BINST && bt >= 0) {
      int bc = (int)floor(b / dch);
      if (bc < PIMC_BINSC && bc >= 0 && gr3d)
        gr3d[(long)dtype * PIMC_BINSR * PIMC_BINST * PIMC_BINSC + ((long)br * PIMC_BINST + bt) * PIMC_BINSC + bc] += 1.0;
    }
  }
}

/* GetPotEnergy_Densities -- mc_estim.cc:500-687: the potential energy of the
 * path and, with non-NULL histograms, the pair densities it bins */
double orc_pot_energy_est(const orc_ctx *c) { return orc_pot_energy_densities(c, NULL, NULL, NULL); }

double orc_pot_energy_densities(const orc_ctx *c, double *gr1d, double *gr2d, double *gr3d)
{
  const int bin = (gr1d || gr2d || gr3d);
  const pimc_system *s = &c->sys;
  long nb = (long)c->na * c->P;
  int P = c->P, R = c->R;
  double spot = 0.0;
  for (int atom0 = 0; atom0 < c->na - 1; atom0++)
    for (int atom1 = atom0 + 1; atom1 < c->na; atom1++) {
      int type0 = c->mctype[atom0], type1 = c->mctype[atom1];
      int mol0 = s->type[type0].molecule, mol1 = s->type[type1].molecule;
      long offset0 = (long)P * atom0, offset1 = (long)P * atom1;
      double spot_pair = 0.0;
      for (int it = 0; it < P; it++) {
        long t0 = offset0 + it, t1 = offset1 + it;
        double dr[3], dr2 = 0.0;
        for (int id = 0; id < NDIM; id++) {
          dr[id] = (c->coords[id * nb + t0] - c->coords[id * nb + t1]);
          if (s->minimage) dr[id] -= (s->box[id] * rint(dr[id] / s->box[id]));
          dr2 += (dr[id] * dr[id]);
        }
        double r = sqrt(dr2);
        if (mol0 == PIMC_LINEAR || mol1 == PIMC_LINEAR) {
          int sgn = 1;
          long tm = offset1 + it / R;
          if (mol0 == PIMC_LINEAR) { sgn = -1; tm = offset0 + it / R; }
          double cost = 0.0;
          for (int id = 0; id < NDIM; id++) cost += (c->cosine[id * nb + tm] * dr[id]);
          cost /= r;
          cost *= sgn;
          if (bin) bin_density(gr1d, gr2d, gr3d, 2, mol0 == PIMC_LINEAR ? type1 : type0, r, cost, 0.0);
          spot_pair += orc_lpot2d(c, r, cost);
        } else if ((mol0 == PIMC_NONLINEAR || mol1 == PIMC_NONLINEAR) && mol0 != mol1) {
          double RCOM[3], Rpt[3], E[3];
          long tm;
          int typed;
          if (mol0 == PIMC_NONLINEAR) {
            typed = type1;
            tm = offset0 + it / R;
            for (int id = 0; id < 3; id++) { RCOM[id] = c->coords[id * nb + t0]; Rpt[id] = c->coords[id * nb + t1]; }
          } else {
            typed = type0;
            tm = offset1 + it / R;
            for (int id = 0; id < 3; id++) { Rpt[id] = c->coords[id * nb + t0]; RCOM[id] = c->coords[id * nb + t1]; }
          }
          euler_at(c, c->angles, nb, tm, E);
          double radret, theret, chiret;
          if (s->ispher == 0) spot_pair += orc_vcord(c, E, RCOM, Rpt, &radret, &theret, &chiret);
          else {
            radret = r;
            spot_pair += orc_vspher(c, r);
            theret = 0.0;
            chiret = 0.0;
          }
          if (bin) bin_density(gr1d, gr2d, gr3d, 3, typed, radret, theret, chiret);
        } else if (mol0 == PIMC_NONLINEAR && mol1 == PIMC_NONLINEAR && s->type[c->imtype].numb > 1) {
          double com1[3], com2[3], E1[3], E2[3];
          for (int id = 0; id < 3; id++) { com1[id] = c->coords[id * nb + t0]; com2[id] = c->coords[id * nb + t1]; }
          euler_at(c, c->angles, nb, offset0 + it / R, E1);
          euler_at(c, c->angles, nb, offset1 + it / R, E2);
          spot_pair += orc_caleng(com1, com2, E1, E2);
        } else if (type0 == type1 && mol0 == PIMC_ATOM) {
          if (bin) bin_density(gr1d, gr2d, gr3d, 1, type1, r, 0.0, 0.0);
          spot_pair += orc_spot1d(c, r);
        }
      }
      spot += spot_pair;
    }
  return (spot / (double)P);
}

/* GetExchangeLength -- mc_estim.cc:1997-2019: ploops[length] += 1 for every
 * exchange cycle of the boson type, length counted as the reference does
 * (a cycle of k atoms has length k-1) */
void orc_exchange_lengths(const orc_ctx *c, double *ploops)
{
  int bt = -1;
  for (int t = 0; t < c->sys.ntypes; t++)
    if (c->sys.type[t].stat == PIMC_BOSE) bt = t;
  if (bt < 0) return;
  int n = c->sys.type[bt].numb;
  int *flags = (int *)calloc((size_t)n, sizeof(int));
  for (int atom = 0; atom < n; atom++)
    if (flags[atom] == 0) {
      int len = 0, p = c->pindex[atom];
      while (p != atom) {
        flags[p] = 1;
        p = c->pindex[p];
        len++;
      }
      ploops[len] += 1.0;
    }
  free(flags);
}

static int boson_type(const orc_ctx *c)
{
  int bt = -1;
  for (int t = 0; t < c->sys.ntypes; t++)
    if (c->sys.type[t].stat == PIMC_BOSE) bt = t;
  return bt;
}

/* GetAreaEstimators -- mc_estim.cc:2087-2250: projected areas and
 * moments of inertia of the boson paths about the (first) dopant's path,
 * parallel and perpendicular to the linear dopant's axis.  out[6] are the
 * increments the reference adds to _areas[PERP,PARL], _area2[PERP,PARL],
 * _inert[PERP,PARL] (mc_estim.cc:2242-2249) */
int orc_area_estimators(const orc_ctx *c, double *out)
{
  int bt = boson_type(c);
  if (bt < 0 || c->imtype < 0) return PIMC_ERR_STATE;
  long nb = (long)c->na * c->P;
  int P = c->P, R = c->R;
  long imoff = c->offset[c->imtype], off = c->offset[bt];
  double area_perp = 0.0, area_parl = 0.0, inert_perp = 0.0, inert_parl = 0.0;
  for (int atom = 0; atom < c->sys.type[bt].numb; atom++)
    for (int it0 = 0; it0 < P; it0++) {
      int it1 = (it0 + 1) % P;
      long pt0 = off + (long)P * atom, pt1 = pt0;
      if (it1 != it0 + 1) pt1 = off + (long)P * c->pindex[atom];
      pt0 += it0;
      pt1 += it1;
      double dr0[3], dr1[3], np[3], nl[3], area[3], rn0[3], rn1[3];
      for (int d = 0; d < 3; d++) {
        dr0[d] = c->coords[d * nb + pt0] - c->coords[d * nb + imoff + it0];
        dr1[d] = c->coords[d * nb + pt1] - c->coords[d * nb + imoff + it1];
      }
      int itr = it0 / R;
      for (int d = 0; d < 3; d++) nl[d] = c->cosine[d * nb + imoff + itr];
      const double zero = 10e-4;
      double tg = 0.0, st = 1.0;
      if (fabs(nl[0]) > zero) {
        tg = nl[1] / nl[0];
        st = sqrt(1.0 + tg * tg);
      }
      np[0] = tg / st;
      np[1] = -1.0 / st;
      np[2] = 0.0;
      area[0] = 0.5 * (dr0[1] * dr1[2] - dr0[2] * dr1[1]);
      area[1] = 0.5 * (dr0[2] * dr1[0] - dr0[0] * dr1[2]);
      area[2] = 0.5 * (dr0[0] * dr1[1] - dr0[1] * dr1[0]);
      for (int d = 0; d < 3; d++) {
        area_perp += (np[d] * area[d]);
        area_parl += (nl[d] * area[d]);
      }
      const double *nv[2] = {np, nl};
      double *acc[2] = {&inert_perp, &inert_parl};
      for (int k = 0; k < 2; k++) {
        const double *n = nv[k];
        rn0[0] = n[1] * dr0[2] - n[2] * dr0[1];
        rn0[1] = n[2] * dr0[0] - n[0] * dr0[2];
        rn0[2] = n[0] * dr0[1] - n[1] * dr0[0];
        rn1[0] = n[1] * dr1[2] - n[2] * dr1[1];
        rn1[1] = n[2] * dr1[0] - n[0] * dr1[2];
        rn1[2] = n[0] * dr1[1] - n[1] * dr1[0];
        for (int d = 0; d < 3; d++) *acc[k] += (rn0[d] * rn1[d]);
      }
    }
  out[0] = area_perp;
  out[1] = area_parl;
  out[2] = area_perp * area_perp;
  out[3] = area_parl * area_parl;
  out[4] = inert_perp / (double)P;
  out[5] = inert_parl / (double)P;
  return PIMC_OK;
}

/* GetAreaEstim3D -- mc_estim.cc:2252-2594.  iframe 0: about the
 * instantaneous centre of mass of all atoms (mass[type] in amu), projected
 * on the space-fixed axes; iframe 1: about the (first) dopant, projected on
 * its body axes hat x, y, z (the columns of matpre's rotation matrix, as
 * vcord.f:30-34 builds them).  out[18] = area_proj[3], the increments of
 * _areas3D (area_proj[i]*area_proj[j], j <= i, mc_estim.cc:2578-2592) and
 * of _inert3D (inert3D[9]/P, mc_estim.cc:2566-2575) */
int orc_area_estim3d(const orc_ctx *c, int iframe, const double *mass, double *out)
{
  int bt = boson_type(c);
  if (bt < 0 || (iframe == 1 && c->imtype < 0) || !mass) return PIMC_ERR_STATE;
  long nb = (long)c->na * c->P;
  int P = c->P, R = c->R;
  long off = c->offset[bt];
  double *com = (double *)malloc(sizeof(double) * 3 * (size_t)P);
  for (int d = 0; d < 3; d++)
    for (int it = 0; it < P; it++) {
      if (iframe == 0) {
        double tmass = 0.0, v = 0.0;
        for (int atom = 0; atom < c->na; atom++) {
          double m = mass[c->mctype[atom]];
          v += (m * c->coords[d * nb + (long)atom * P + it]);
          tmass += m;
        }
        com[d * P + it] = v / tmass;
      } else {
        com[d * P + it] = c->coords[d * nb + c->offset[c->imtype] + it];
      }
    }
  double bmass = mass[bt];
  double ap[3] = {0, 0, 0}, ic[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int it0 = 0; it0 < P; it0++) {
    double hat[3][3];
    if (iframe == 0) {
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) hat[i][j] = (i == j) ? 1.0 : 0.0;
    } else {
      double E[3], m[9];
      euler_at(c, c->angles, nb, c->offset[c->imtype] + it0 / R, E);
      orc_matpre(E, m);
      for (int i = 0; i < 3; i++)
        for (int d = 0; d < 3; d++) hat[i][d] = m[d * 3 + i];
    }
    for (int atom = 0; atom < c->sys.type[bt].numb; atom++) {
      int it1 = (it0 + 1) % P;
      long pt0 = off + (long)P * atom, pt1 = pt0;
      if (it1 != it0 + 1) pt1 = off + (long)P * c->pindex[atom];
      pt0 += it0;
      pt1 += it1;
      double dr0[3], dr1[3], area[3], rn0[3], rn1[3];
      for (int d = 0; d < 3; d++) {
        dr0[d] = c->coords[d * nb + pt0] - com[d * P + it0];
        dr1[d] = c->coords[d * nb + pt1] - com[d * P + it1];
      }
      area[0] = 0.5 * (dr0[1] * dr1[2] - dr0[2] * dr1[1]);
      area[1] = 0.5 * (dr0[2] * dr1[0] - dr0[0] * dr1[2]);
      area[2] = 0.5 * (dr0[0] * dr1[1] - dr0[1] * dr1[0]);
      for (int i = 0; i < 3; i++)
        for (int d = 0; d < 3; d++) ap[i] += area[d] * hat[i][d];
      for (int i = 0; i < 3; i++) {
        const double *h = hat[i];
        rn0[0] = dr0[1] * h[2] - dr0[2] * h[1];
        rn0[1] = dr0[2] * h[0] - dr0[0] * h[2];
        rn0[2] = dr0[0] * h[1] - dr0[1] * h[0];
        rn1[0] = dr1[1] * h[2] - dr1[2] * h[1];
        rn1[1] = dr1[2] * h[0] - dr1[0] * h[2];
        rn1[2] = dr1[0] * h[1] - dr1[1] * h[0];
        double sum = 0.0;
        for (int d = 0; d < 3; d++) sum += rn0[d] * rn1[d] * bmass;
        ic[i * 3 + i] += sum;
        double d0 = 0.0;
        for (int d = 0; d < 3; d++) d0 += h[d] * dr0[d];
        for (int j = 0; j < 3; j++)
          if (j != i) {
            double d1 = 0.0;
            for (int d = 0; d < 3; d++) d1 += hat[j][d] * dr1[d];
            ic[i * 3 + j] += -bmass * d0 * d1;
          }
      }
    }
  }
  free(com);
  for (int i = 0; i < 3; i++) out[i] = ap[i];
  int ind = 3;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j <= i; j++) out[ind++] = ap[i] * ap[j];
  for (int k = 0; k < 9; k++) out[9 + k] = ic[k] / (double)P;
  return PIMC_OK;
}

/* GetRotEnergy -- mc_estim.cc:939-987 (single linear rotor) */
double orc_rot_energy(const orc_ctx *c, double *erotsq, double *erot_termsq)
{
  long nb = (long)c->na * c->P;
  int type = c->imtype;
  long offset = c->offset[type];
  double srot = 0.0, esq = 0.0, ets = 0.0;
  int Q = c->Q;
  for (int it0 = 0; it0 < Q; it0++) {
    long t0 = offset + it0, t1 = offset + (it0 + 1) % Q;
    double p0 = 0.0;
    for (int id = 0; id < NDIM; id++) p0 += (c->cosine[id * nb + t0] * c->cosine[id * nb + t1]);
    if (c->sys.rot_den_type == 0) {
      double rdens = orc_srotdens(c, p0, 0);
      if (fabs(rdens) > RZERO) srot += (orc_srotdens(c, p0, 1) / rdens);
      ets += (orc_srotdens(c, p0, 1) / rdens) * (orc_srotdens(c, p0, 1) / rdens);
      esq += orc_srotdens(c, p0, 2) / rdens;
    } else {
      double rho, erot;
      orc_rsline(c->sys.rot_abc[0], p0, c->rot_tau, &rho, &erot);
      srot += rho;
    }
  }
  if (c->sys.rot_den_type == 1) {
    srot = srot / (double)Q;
    srot = srot / c->rot_tau + 1.0 / c->rot_tau;
  }
  if (erotsq) *erotsq = esq;
  if (erot_termsq) *erot_termsq = ets;
  return srot;
}

/* GetRotE3D -- mc_estim.cc:989-1096 (rotor a at offset a*P, see header) */
double orc_rot_e3d(const orc_ctx *c, double *erotsq, double *erot_termsq)
{
  long nb = (long)c->na * c->P;
  int type = c->imtype, Q = c->Q;
  double ERot3D = 0.0, ErotSQ = 0.0, EtermSQ = 0.0;
  for (int atom = 0; atom < c->sys.type[type].numb; atom++) {
    long offset = c->offset[type] + (long)c->P * atom;
    double srot = 0.0, sesq = 0.0, se_termsq = 0.0;
    int RNskip = (c->sys.rot_den_type == 0) ? 1 : c->sys.rn_ratio;
    for (int it0 = 0; it0 < Q; it0 = it0 + RNskip) {
      long t0 = offset + it0, t1 = offset + (it0 + RNskip) % Q;
      double rho = 0.0, erot = 0.0, esq = 0.0, rel[3], E1[3], E2[3];
      E1[0] = c->angles[PHI * nb + t0]; E1[1] = acos(c->angles[CTH * nb + t0]); E1[2] = c->angles[CHI * nb + t0];
      E2[0] = c->angles[PHI * nb + t1]; E2[1] = acos(c->angles[CTH * nb + t1]); E2[2] = c->angles[CHI * nb + t1];
      orc_rotden(c, E1, E2, rel, &rho, &erot, &esq);
      if (c->sys.rot_den_type == 1 && c->sys.rn_ratio == 1)
        orc_rsrot(E1, E2, c->sys.rot_abc[0], c->sys.rot_abc[1], c->sys.rot_abc[2], c->rot_tau,
                  c->sys.rot_odevn, c->sys.rot_eoff, &rho, &erot);
      if (c->sys.rot_den_type == 1 && c->sys.rn_ratio == 1) srot += rho;
      else srot += erot;
      sesq += esq;
      se_termsq += erot * erot;
    }
    double nq = (double)(Q / RNskip);
    srot = srot / nq;
    sesq = sesq / (nq * nq);
    se_termsq = se_termsq / (nq * nq);
    ErotSQ += sesq;
    EtermSQ += se_termsq;
    if (c->sys.rot_den_type == 1 && c->sys.rn_ratio == 1) {      /* per rotor, see header */
      srot = srot / (4.0 * (c->rot_tau / WNO2K) * (c->rot_tau / WNO2K));
      srot += 0.25 * (c->sys.rot_abc[0] + c->sys.rot_abc[1] + c->sys.rot_abc[2]) + 1.5 / (c->rot_tau / WNO2K);
      srot = srot / WNO2K;
    }
    ERot3D += srot;
  }
  if (erotsq) *erotsq = ErotSQ;
  if (erot_termsq) *erot_termsq = EtermSQ;
  return ERot3D;
}

/* GetRCF -- mc_estim.cc:1099-1139, the meaningful rcf[0] row */
void orc_rcf(const orc_ctx *c, double *rcf)
{
  long nb = (long)c->na * c->P;
  long offset = c->offset[c->imtype];
  int Q = c->Q;
  for (int it0 = 0; it0 < Q; it0++) {
    long t0 = offset + it0;
    for (int itc = 0; itc < Q; itc++) {
      long tc = offset + (it0 + itc) % Q;
      double p0 = 0.0;
      for (int id = 0; id < NDIM; id++) p0 += (c->cosine[id * nb + t0] * c->cosine[id * nb + tc]);
      rcf[itc] += p0;
    }
  }
}

/* ------------------------------------------------------------------ worm */

/* MCWormInit -- mc_qworm.cc:49-82 */
int orc_worm_init(orc_ctx *c, int type, double wc, int m, double density)
{
  if (type < 0 || type >= c->sys.ntypes || m < 1 || m >= c->P) return PIMC_ERR_BAD_ARG;
  int numb = c->sys.type[type].numb;
  c->worm_on = 1;
  c->wtype = type;
  c->wexists = 0;
  c->ira = c->masha = c->atom_i = c->atom_m = 0;
  c->wm = m;
  c->wc = wc * (density / (double)(numb * c->P * m));
  c->qw_norm = c->wc * numb * c->P * m;
  double twave2 = 4.0 * c->sys.type[type].lambda * c->tau;      /* mc_setup.cc:394 */
  (void)twave2;
  double termal2 = (double)m * 4.0 * c->sys.type[type].lambda * c->tau;
  c->wcut2 = 100.0 * 100.0 * termal2;
  free(c->dr2_list); free(c->ptable); free(c->atm_list);
  c->dr2_list = (double *)calloc((size_t)numb + 1, sizeof(double));
  c->ptable = (double *)calloc((size_t)numb + 1, sizeof(double));
  c->atm_list = (int *)calloc((size_t)numb + 1, sizeof(int));
  for (int k = 0; k < 7; k++) c->qwtot[k] = c->qwacc[k] = 0.0;
  return PIMC_OK;
}

void orc_worm_state(const orc_ctx *c, int *st)
{
  st[0] = c->wexists; st[1] = c->ira; st[2] = c->masha; st[3] = c->atom_i; st[4] = c->atom_m;
}

void orc_worm_set_state(orc_ctx *c, const int *st)
{
  c->wexists = st[0]; c->ira = st[1]; c->masha = st[2]; c->atom_i = st[3]; c->atom_m = st[4];
}

void orc_worm_counters(const orc_ctx *c, double *total, double *accep)
{
  for (int k = 0; k < 7; k++) { total[k] = c->qwtot[k]; accep[k] = c->qwacc[k]; }
}

static double twave2_of(const orc_ctx *c) { return 4.0 * c->sys.type[c->wtype].lambda * c->tau; }

/* a worm draw: replay stream k of rp, or the internal generator (rp NULL);
 * k = 0..2 nrnd1..3, 3..7 rnd1..5, 8 gauss's x1 (mc_randg.cc:90-174) */
static double wt(orc_ctx *c, orc_wreplay *rp, int k)
{
  if (rp) {
    orc_stream *st[9] = {&rp->n1, &rp->n2, &rp->n3, &rp->u1, &rp->u2, &rp->u3, &rp->u4, &rp->u5, &rp->gauss};
    return take(st[k], &rp->overrun);
  }
  if (k == 8) {
    double r1 = u01_key(c->seed, 40, c->wctr[8]++);
    double r2 = u01_key(c->seed, 41, c->wctr[8]++);
    return sqrt(-log(r1)) * cos(2.0 * M_PI * r2);
  }
  return u01_key(c->seed, 30 + (uint64_t)k, c->wctr[k]++);
}

static int nrnd(orc_ctx *c, orc_wreplay *rp, int k, int n) { return (int)floor(n * wt(c, rp, k)); }

/* get_potential -- mc_qworm.cc:402-422 */
static double worm_potential(const orc_ctx *c, int it0, int it1, int atom0, int atom1, const double *coords)
{
  int aoff = c->offset[c->wtype] / c->P;
  int pit0 = it0 % c->P;
  double pot = 0.0;
  int atom = atom0;
  for (int it = it0 + 1; it < it1; it++) {
    int pit = it % c->P;
    if (pit != it && pit0 == it0) atom = atom1;
    pot += orc_pot_energy_slice(c, aoff + atom, coords, pit);
  }
  return pot;
}

/* qw_open_prob -- mc_qworm.cc:127-153 */
static double qw_open_prob(orc_ctx *c, int segm)
{
  long nb = (long)c->na * c->P;
  long offset = c->offset[c->wtype];
  double kin = 0.0;
  long pt0 = offset + (long)c->atom_i * c->P + c->ira;
  long pt1 = offset + (long)c->atom_m * c->P + c->masha;
  for (int id = 0; id < NDIM; id++) {
    double dr = c->coords[id * nb + pt0] - c->coords[id * nb + pt1];
    if (c->sys.minimage) dr -= (c->sys.box[id] * rint(dr / c->sys.box[id]));
    kin += (dr * dr);
  }
  kin /= (twave2_of(c) * (double)segm);
  double pot = worm_potential(c, c->ira, c->ira + segm, c->atom_i, c->atom_m, c->coords);
  pot *= c->tau;
  return (c->qw_norm * pow((double)segm, 0.5 * (double)NDIM) * exp(kin + pot));
}

/* sample_middle -- mc_qworm.cc:238-283 */
static void sample_middle(orc_ctx *c, int it0, int it2, int atom0, int atom2, double *coords, orc_wreplay *rp)
{
  if ((it2 - it0) < 2) return;
  long nb = (long)c->na * c->P;
  int P = c->P;
  int it1 = (int)rint(0.5 * (double)(it0 + it2));
  int pt0 = it0 % P, pt1 = it1 % P, pt2 = it2 % P;
  int atom1 = atom0;
  if ((pt1 != it1) && (pt0 == it0)) atom1 = atom2;
  long offset = c->offset[c->wtype];
  long q0 = pt0 + offset + (long)atom0 * P, q1 = pt1 + offset + (long)atom1 * P, q2 = pt2 + offset + (long)atom2 * P;
  double s0 = (double)(it1 - it0), s2 = (double)(it2 - it1);
  double gkin = (s0 + s2) / (twave2_of(c) * s0 * s2);
  for (int id = 0; id < NDIM; id++) {
    coords[id * nb + q1] = (s2 * coords[id * nb + q0] + s0 * coords[id * nb + q2]) / (s0 + s2);
    coords[id * nb + q1] += wt(c, rp, 8) / sqrt(gkin);     /* gauss(gkin), mc_randg.cc:149 */
  }
  sample_middle(c, it0, it1, atom0, atom1, coords, rp);
  sample_middle(c, it1, it2, atom1, atom2, coords, rp);
}



/* qworm_open -- mc_qworm.cc:155-180 */
static void qworm_open(orc_ctx *c, orc_wreplay *rp)
{
  c->qwtot[0] += 1.0;
  int numb = c->sys.type[c->wtype].numb;
  c->atom_i = nrnd(c, rp, 0, numb);
  c->ira = nrnd(c, rp, 1, c->P);
  int segm = nrnd(c, rp, 2, c->wm) + 1;
  c->masha = (c->ira + segm) % c->P;
  c->atom_m = c->atom_i;
  if (c->masha != (c->ira + segm)) c->atom_m = c->pindex[c->atom_i];
  double prob = qw_open_prob(c, segm);
  int acc = 0;
  if (prob >= 1.0) acc = 1;
  else if (prob > wt(c, rp, 3)) acc = 1;
  if (acc) {
    c->wexists = 1;
    c->qwacc[0] += 1.0;
  }
}

/* qworm_close -- mc_qworm.cc:182-236 */
static void qworm_close(orc_ctx *c, orc_wreplay *rp)
{
  c->qwtot[1] += 1.0;
  int segm = c->masha - c->ira;
  if (segm < 0) segm += c->P;
  if (segm > c->wm) return;
  int it0 = c->ira, it2 = c->ira + segm;
  sample_middle(c, it0, it2, c->atom_i, c->atom_m, c->coords, rp);
  double prob = 1.0 / qw_open_prob(c, segm);
  int acc = 0;
  if (prob >= 1.0) acc = 1;
  else if (prob > wt(c, rp, 3)) acc = 1;
  if (acc) {
    c->wexists = 0;
    c->qwacc[1] += 1.0;
  }
}

/* qworm_advance -- mc_qworm.cc:295-355 */
static void qworm_advance(orc_ctx *c, orc_wreplay *rp)
{
  c->qwtot[4] += 1.0;
  long nb = (long)c->na * c->P;
  int P = c->P;
  int segm = c->masha - c->ira;
  if (segm < 0) segm += P;
  int advance = nrnd(c, rp, 2, c->wm) + 1;
  if (segm - advance <= 0) return;
  long offset = c->offset[c->wtype];
  int it0 = c->ira, it2 = c->ira + advance;
  int ira_new = it2 % P, atom_i_new = c->atom_i;
  if (ira_new != it2) atom_i_new = c->atom_m;
  double gvar = 1.0 / ((double)advance * twave2_of(c));
  long pt0 = offset + (long)c->atom_i * P + it0 % P;
  long pt2 = offset + (long)atom_i_new * P + it2 % P;
  for (int id = 0; id < NDIM; id++)
    c->coords[id * nb + pt2] = c->coords[id * nb + pt0] + wt(c, rp, 8) / sqrt(gvar);
  sample_middle(c, it0, it2, c->atom_i, atom_i_new, c->coords, rp);
  double pot = worm_potential(c, it0, it2 + 1, c->atom_i, atom_i_new, c->coords);
  int acc = 0;
  if (pot < 0.0) acc = 1;
  else if (exp(-pot * c->tau) > wt(c, rp, 4)) acc = 1;
  if (acc) {
    c->qwacc[4] += 1.0;
    c->ira = ira_new;
    c->atom_i = atom_i_new;
  }
}

/* qworm_recede -- mc_qworm.cc:357-400 */
static void qworm_recede(orc_ctx *c, orc_wreplay *rp)
{
  c->qwtot[5] += 1.0;
  int segm = c->ira - c->masha;
  if (segm < 0) segm += c->P;
  int recede = nrnd(c, rp, 2, c->wm) + 1;
  if ((segm - recede) < 1) return;
  int it0 = c->ira - recede, it1 = c->ira;
  int atom0 = c->atom_i, atom1 = c->atom_i;
  if (it0 < 0) {
    it0 += c->P;
    it1 += c->P;
    atom0 = c->rindex[atom1];
  }
  double pot = worm_potential(c, it0, it1 + 1, atom0, atom1, c->coords);
  int acc = 0;
  if (pot > 0.0) acc = 1;
  else if (exp(pot * c->tau) > wt(c, rp, 4)) acc = 1;
  if (acc) {
    c->ira = it0 % c->P;
    c->atom_i = atom0;
    c->qwacc[5] += 1.0;
  }
}

/* get_ptable -- mc_qworm.cc:577-642 (mmsort: mc_utils.cc:206-230) */
static int get_ptable(orc_ctx *c, int atomw, int pt0, int pt1, int segm, int t1)
{
  long nb = (long)c->na * c->P;
  int P = c->P, numb = c->sys.type[c->wtype].numb;
  long offset = c->offset[c->wtype];
  long itw = offset + (long)atomw * P + pt0;
  int count = 0;
  for (int atom1 = 0; atom1 < numb; atom1++)
    if (world_line(c, atom1, pt1)) {
      int atom0 = atom1;
      if (t1 != pt1) atom0 = c->rindex[atom1];
      if (atom0 != c->atom_i) {
        long it1 = offset + (long)atom1 * P + pt1;
        double dr2 = 0.0;
        for (int id = 0; id < NDIM; id++) {
          double dx = c->coords[id * nb + itw] - c->coords[id * nb + it1];
          if (c->sys.minimage) dx -= (c->sys.box[id] * rint(dx / c->sys.box[id]));
          dr2 += (dx * dx);
        }
        if (dr2 < c->wcut2) {
          count++;
          c->dr2_list[count] = dr2;
          c->atm_list[count] = atom1;
        }
      }
    }
  for (int j = 2; j <= count; j++) {
    double dtmp = c->dr2_list[j];
    int itmp = c->atm_list[j];
    int i = j - 1;
    while ((i > 0) && (c->dr2_list[i] > dtmp)) {
      c->dr2_list[i + 1] = c->dr2_list[i];
      c->atm_list[i + 1] = c->atm_list[i];
      i--;
    }
    c->dr2_list[i + 1] = dtmp;
    c->atm_list[i + 1] = itmp;
  }
  if (count > 100) count = 100;     /* MAXNEIGHBORS, mc_qworm.cc:12 */
  double norm = 1.0 / ((double)segm * twave2_of(c));
  for (int ic = 1; ic <= count; ic++) c->ptable[ic] = exp(-norm * c->dr2_list[ic]);
  return count;
}

/* atom2swap -- mc_qworm.cc:644-667 */
static int atom2swap(orc_ctx *c, int count, double *pnorm, orc_wreplay *rp)
{
  *pnorm = 0.0;
  for (int ic = 1; ic <= count; ic++) *pnorm += c->ptable[ic];
  double prand = *pnorm * wt(c, rp, 5);
  double sum = 0.0;
  int ic = 1;
  while ((ic <= count) && (sum < prand)) {
    sum += c->ptable[ic];
    ic++;
  }
  ic--;
  return c->atm_list[ic];
}

/* qworm_swap -- mc_qworm.cc:424-551 */
static void qworm_swap(orc_ctx *c, orc_wreplay *rp)
{
  c->qwtot[6] += 1.0;
  long nb = (long)c->na * c->P;
  int P = c->P;
  int segm = c->wm;
  int it0 = c->ira, it1 = it0 + segm;
  int pit0 = it0, pit1 = it1 % P;
  int atomw = c->atom_i;
  int count = get_ptable(c, atomw, pit0, pit1, segm, it1);
  if (count <= 0) return;
  double pnorm_old, pnorm_new;
  int atom1 = atom2swap(c, count, &pnorm_old, rp);
  if (atom1 < 0) return;
  int atom0 = atom1;
  if (pit1 != it1) atom0 = c->rindex[atom1];
  long offset0 = c->offset[c->wtype] + (long)atom0 * P;
  long offset1 = c->offset[c->wtype] + (long)atom1 * P;
  long offsetw = c->offset[c->wtype] + (long)atomw * P;
  for (int id = 0; id < NDIM; id++) {
    c->newc[id * nb + offset0 + pit0] = c->coords[id * nb + offsetw + pit0];
    c->newc[id * nb + offset1 + pit1] = c->coords[id * nb + offset1 + pit1];
  }
  sample_middle(c, it0, it1, atom0, atom1, c->newc, rp);
  int gatom0 = (int)(offset0 / P), gatom1 = (int)(offset1 / P);
  double pot = 0.0;
  int gatom = gatom0;
  for (int it = it0 + 1; it < it1; it++) {
    int pit = it % P;
    if (pit != it) gatom = gatom1;
    pot += orc_pot_energy_slice(c, gatom, c->newc, pit);
    pot -= orc_pot_energy_slice(c, gatom, c->coords, pit);
  }
  double prob = exp(-pot * c->tau);
  count = get_ptable(c, atom0, pit0, pit1, segm, it1);
  pnorm_new = 0.0;
  for (int ic = 1; ic <= count; ic++) pnorm_new += c->ptable[ic];
  prob *= (pnorm_old / pnorm_new);
  int acc = 0;
  if (prob >= 1.0) acc = 1;
  else if (prob > wt(c, rp, 6)) acc = 1;
  if (acc) {
    c->qwacc[6] += 1.0;
    for (int id = 0; id < NDIM; id++) {
      long offset = offset0;
      for (int it = it0 + 1; it < it1; it++) {
        int pit = it % P;
        if (pit != it) offset = offset1;
        c->coords[id * nb + offset + pit] = c->newc[id * nb + offset + pit];
      }
    }
    for (int id = 0; id < NDIM; id++)
      for (int it = 0; it <= it0; it++) {
        c->newc[id * nb + offset0 + it] = c->coords[id * nb + offset0 + it];
        c->coords[id * nb + offset0 + it] = c->coords[id * nb + offsetw + it];
        c->coords[id * nb + offsetw + it] = c->newc[id * nb + offset0 + it];
      }
    int ratomw = c->rindex[atomw], ratom0 = c->rindex[atom0];
    c->pindex[ratomw] = atom0;
    c->rindex[atom0] = ratomw;
    c->pindex[ratom0] = atomw;
    c->rindex[atomw] = ratom0;
    if (c->ira > c->masha) {
      if (atom0 == c->atom_m) c->atom_m = c->atom_i;
      else if (c->atom_i == c->atom_m) c->atom_m = atom0;
    }
  }
}

/* MCWormMove -- mc_qworm.cc:93-125: one try per atom of the worm type */
int orc_worm_move(orc_ctx *c, orc_wreplay *rp)
{
  if (!c->worm_on) return PIMC_ERR_STATE;
  int numb = c->sys.type[c->wtype].numb;
  int bose = c->sys.type[c->wtype].stat == PIMC_BOSE;
  for (int atom = 0; atom < numb; atom++) {
    if (c->wexists) qworm_close(c, rp);
    else qworm_open(c, rp);
    if (c->wexists) {
      double r = wt(c, rp, 7);
      if (r > 0.5) qworm_advance(c, rp);
      else qworm_recede(c, rp);
    }
    if (bose && c->wexists) qworm_swap(c, rp);
  }
  return (rp && rp->overrun) ? PIMC_ERR_BAD_ARG : PIMC_OK;
}

/* the worm branch of the pass loop (mc_main.cc:348-381) with the internal
 * generator: per time slice, for the worm type MCWormMove and, with the worm
 * closed, MCBisectionMoveExchange at a drawn slice (MCBisectionMove for
 * Boltzmann statistics) and at slice 0 the exchange centroid move; for the
 * other types PIMCPass (mc_main.cc:510-522).  *bead_moves counts the
 * scheduled bead moves of the non-worm moves and P per worm-type atom and
 * slice for the worm tries. */
static int sweep_parallel(orc_ctx *c, int type, uint64_t sweep_id, int nthreads);

int orc_worm_run(orc_ctx *c, int t_begin, int t_count, uint64_t seed, int nthreads, double *bead_moves)
{
  if (!c->worm_on) return PIMC_ERR_STATE;
  src_t src = {NULL, c};
  c->seed = seed;
  double bm = 0.0;
  if (nthreads < 1) nthreads = 1;
  for (int time = t_begin; time < t_begin + t_count; time++) {
    int t = time % c->P;
    for (int type = 0; type < c->sys.ntypes; type++) {
      int numb = c->sys.type[type].numb;
      if (numb <= 0) continue;
      if (type == c->wtype) {
        int st = orc_worm_move(c, NULL);
        if (st) return st;
        bm += (double)numb;
        if (!c->wexists) {
          int rt = (int)floor(c->P * u01_key(c->seed, 50, c->wctr[0]++));   /* nrnd2(NumbTimes) */
          int bose = c->sys.type[type].stat == PIMC_BOSE;
          bisection_move(c, type, rt, &src, NULL, NULL, bose);
          bm += (double)numb * (double)(c->mlsegm[type] - 1);
          if (t == 0) {
            if (bose) orc_molecular_move_exchange(c, type, NULL, NULL, NULL);
            else molecular_move(c, type, &src, NULL, NULL, nthreads);
            bm += (double)numb * c->P;
          }
        }
        continue;
      }
      if (t == 0) {
        molecular_move(c, type, &src, NULL, NULL, nthreads);
        bm += (double)numb * c->P;
      }
      bisection_move(c, type, t, &src, NULL, NULL, 0);
      bm += (double)numb * (double)(c->mlsegm[type] - 1);
      if (type == c->imtype && c->sys.rotation) {
        int st = sweep_parallel(c, type, (uint64_t)time, nthreads);
        if (st) return st;
        bm += (double)c->Q * numb;
      }
    }
  }
  if (bead_moves) *bead_moves = bm;
  return PIMC_OK;
}

/* -------------------------------------------------------- timed schedule */

/* rotational sweep with the internal generator, even/odd phases in
 * parallel like mc_piqmc.cc:490-512 and 737-771; each (sweep, slice, rotor)
 * draws from its own counter so the result does not depend on threads */
static int sweep_parallel(orc_ctx *c, int type, uint64_t sweep_id, int nthreads)
{
  int mol = c->sys.type[type].molecule;
  int nrot = c->sys.type[type].numb;
  long nb = (long)c->na * c->P;
  double tot = 0, acp = 0;
  int err = 0;
  for (int ph = 0; ph < 2; ph++) {
#pragma omp parallel num_threads(nthreads) if (nthreads > 1) reduction(+ : tot, acp)
    {
      /* thread-private proposal rows so threads do not share the buffer */
      double *nbuf = (double *)malloc(sizeof(double) * 3 * (size_t)nb);
#pragma omp for schedule(static)
      for (int it = ph; it < c->Q; it += 2) {
        for (int a = 0; a < nrot; a++) {
          long offset = c->offset[type] + (long)c->P * a;
          uint64_t key = (sweep_id * (uint64_t)c->Q + (uint64_t)it) * 16u + (uint64_t)a;
          double u[4];
          for (int k = 0; k < 4; k++) u[k] = u01_key(c->seed, 100 + k, key);
          int st = (mol == PIMC_LINEAR)
                       ? rot_lin_step(c, it, offset, (int)(offset / c->P), u, NULL, NULL, nbuf, &tot, &acp)
                       : rot_3d_step(c, it, offset, (int)(offset / c->P), u, NULL, NULL, nbuf, &tot, &acp);
          if (st) err = st;
        }
      }
      free(nbuf);
    }
  }
  c->total[type * 3 + MCROTAT] += tot;
  c->accep[type * 3 + MCROTAT] += acp;
  return err;
}

int orc_run_steps(orc_ctx *c, int t_begin, int t_count, uint64_t seed, int nthreads, double *bead_moves)
{
  src_t src = {NULL, c};
  c->seed = seed;
  double bm = 0.0;
  if (nthreads < 1) nthreads = 1;
  for (int time = t_begin; time < t_begin + t_count; time++) {
    int t = time % c->P;
    for (int type = 0; type < c->sys.ntypes; type++) {
      int numb = c->sys.type[type].numb;
      if (numb <= 0) continue;
      /* PIMCPass -- mc_main.cc:510-522 */
      if (t == 0) {
        molecular_move(c, type, &src, NULL, NULL, nthreads);
        bm += (double)numb * c->P;
      }
      bisection_move(c, type, t, &src, NULL, NULL, 0);
      bm += (double)numb * (double)(c->mlsegm[type] - 1);
      if (type == c->imtype && c->sys.rotation) {
        int st = sweep_parallel(c, type, (uint64_t)time, nthreads);
        if (st) return st;
        bm += (double)c->Q * numb;
      }
    }
  }
  if (bead_moves) *bead_moves = bm;
  return PIMC_OK;
}
