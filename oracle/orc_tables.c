/*
 * orc_tables.c -- TEST INFRASTRUCTURE ONLY.  CPU restatements of the
 * reference's propagator-table generators, used as the checker of the GB300
 * generators (pimc_linden / pimc_asymrho):
 *   linear_prop/linden.f   -- exact linear-rotor propagator (exarho, lgnd);
 *   nmv_prop/asymrho.f     -- exact asymmetric-top propagator: rotational
 *                             matrix (rotmat, cplus, cminus), TRED2 + TQL
 *                             diagonalisation, quad-precision Wigner d
 *                             (wigd, calfac) and the per-grid-point state sums.
 * The quad-precision type is __float128 (libquadmath) on x86-64 and the IEEE
 * binary128 long double of aarch64 Linux elsewhere, as the reference's
 * real*16.
 */
#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "pimc_oracle.h"

#if defined(__x86_64__) || defined(__i386__)
#include <quadmath.h>
typedef __float128 qreal;
#define QSQRT sqrtq
#define QCOS cosq
#define QSIN sinq
#else
typedef long double qreal;
_Static_assert(LDBL_MANT_DIG == 113, "long double must be IEEE binary128 here");
#define QSQRT sqrtl
#define QCOS cosl
#define QSIN sinl
#endif

/* ------------------------------------------------------------- linden.f */

/* lgnd -- linden.f:182-198: P_0..P_lmax at x by the upward recurrence;
 * (2.0*L+1) is a default-real product in the Fortran, exact for these L */
static void lgnd(int lmax, double x, double *p)
{
  p[0] = 1.0;
  if (lmax >= 1) p[1] = x;
  for (int l = 1; l <= lmax - 1; l++) p[l + 1] = ((2.0 * l + 1) * x * p[l] - l * p[l - 1]) / (l + 1);
}

/* linden.f:21-37 -- tau = taunit/(T*nslice) and the largest l kept */
int orc_linden_lmax(double temprt, int nslice, double bconst, double *tau_out)
{
  const double taunit = 1.4387752224, eps = 1.e-16;
  const int maxl = 500;
  double tau = taunit / (temprt * nslice);
  if (tau_out) *tau_out = tau;
  for (int l = 0; l <= maxl; l++)
    if (exp(-tau * bconst * l * (l + 1)) < eps) return l;
  return maxl;
}

/* linden.f:39-68 + exarho linden.f:88-122: npt rows (cost, rho, erot, erotsq)
 * written to cost/rho/erot/erotsq */
int orc_linden(double temprt, int nslice, double bconst, int npt, int iodevn, double *cost, double *rho,
               double *erot, double *erotsq)
{
  const double pi = 3.14159265358979323846, boltz = 0.69503476;
  if (npt < 2 || nslice < 1 || !(temprt > 0.0)) return PIMC_ERR_BAD_ARG;
  double tau;
  int lmax = orc_linden_lmax(temprt, nslice, bconst, &tau);
  double *pl = (double *)malloc(sizeof(double) * (size_t)(lmax + 2));
  double cstep = 2.0 / (double)(npt - 1);
  for (int ic = 1; ic <= npt; ic++) {
    double x = (ic - 1) * cstep - 1.0;
    lgnd(lmax, x, pl);
    double r = 0.0, e = 0.0, s = 0.0;
    for (int l = 0; l <= lmax; l++) {
      if ((l % 2) == iodevn || iodevn == -1) {
        double tmp = (double)(2 * l + 1) * pl[l];
        tmp = tmp * exp(-tau * bconst * (double)(l * (l + 1)));
        r = r + tmp;
        e = e + tmp * l * (l + 1) * bconst;
        s = s + tmp * l * (l + 1) * bconst * l * (l + 1) * bconst;
      }
    }
    e = e / (nslice * boltz);
    s = s / ((nslice * boltz) * (nslice * boltz));
    cost[ic - 1] = x;
    rho[ic - 1] = r / (4.0 * pi);
    erot[ic - 1] = e / (4.0 * pi);
    erotsq[ic - 1] = s / (4.0 * pi);
  }
  free(pl);
  return PIMC_OK;
}

/* ------------------------------------------------------------ asymrho.f */

/* cplus / cminus -- asymrho.f:752-790 */
static double cplus(int j, int k)
{
  if (k >= j || k < -j) return 0.0;
  double dj = j, dk = k;
  return sqrt(dj * (dj + 1.0) - dk * (dk + 1.0));
}

static double cminus(int j, int k)
{
  if (k <= -j || k > j) return 0.0;
  double dj = j, dk = k;
  return sqrt(dj * (dj + 1.0) - dk * (dk - 1.0));
}

/* rotmat -- asymrho.f:792-813: <j k|H|j kp> of the rigid asymmetric top */
double orc_rotmat(int j, int k, int kp, double A, double B, double C)
{
  if (abs(k - kp) != 0 && abs(k - kp) != 2) return 0.0;
  if (k == kp) return 0.5 * (A + C) * (double)(j * (j + 1)) + (B - 0.5 * (A + C)) * (double)(k * k);
  if (k == kp + 2) return 0.25 * (A - C) * cplus(j, kp) * cplus(j, kp + 1);
  return 0.25 * (A - C) * cminus(j, kp) * cminus(j, kp - 1);
}

/* TRED2 -- asymrho.f:922-1004: Householder reduction of the symmetric z
 * (column-major md x md, leading n x n used) to tridiagonal form; d the
 * diagonal, e the sub-diagonal, z the accumulated transformation */
#define Z(i, j) z[((j) - 1) * md + ((i) - 1)]
static void tred2(int md, int n, double *z, double *d, double *e)
{
  const double beta = 1e-20;
  for (int nmip2 = 2; nmip2 <= n; nmip2++) {
    int i = n + 2 - nmip2, im1 = i - 1, im2 = i - 2, l = im2;
    double f = Z(i, im1), g = 0.0, h;
    if (l > 0)
      for (int k = 1; k <= l; k++) g = g + Z(i, k) * Z(i, k);
    h = g + f * f;
    if (g - beta <= 0) {
      e[i - 1] = f;
      h = 0.0;
    } else {
      l = l + 1;
      if (f < 0) e[i - 1] = sqrt(h);
      else e[i - 1] = -sqrt(h);
      g = e[i - 1];
      h = h - f * g;
      Z(i, im1) = f - g;
      f = 0.0;
      for (int j = 1; j <= l; j++) {
        Z(j, i) = Z(i, j) / h;
        g = 0.0;
        for (int k = 1; k <= j; k++) g = g + Z(j, k) * Z(i, k);
        int jp1 = j + 1;
        if (jp1 - l <= 0)
          for (int k = jp1; k <= l; k++) g = g + Z(k, j) * Z(i, k);
        e[j - 1] = g / h;
        f = f + g * Z(j, i);
      }
      double hh = f / (h + h);
      for (int j = 1; j <= l; j++) {
        f = Z(i, j);
        e[j - 1] = e[j - 1] - hh * f;
        g = e[j - 1];
        for (int k = 1; k <= j; k++) Z(j, k) = Z(j, k) - f * e[k - 1] - g * Z(i, k);
      }
    }
    d[i - 1] = h;
  }
  d[0] = 0.0;
  e[0] = 0.0;
  for (int i = 1; i <= n; i++) {
    int l = i - 1;
    if (d[i - 1] != 0 && l > 0) {
      for (int j = 1; j <= l; j++) {
        double g = 0.0;
        for (int k = 1; k <= l; k++) g = g + Z(i, k) * Z(k, j);
        for (int k = 1; k <= l; k++) Z(k, j) = Z(k, j) - g * Z(k, i);
      }
    }
    d[i - 1] = Z(i, i);
    Z(i, i) = 1.0;
    if (l > 0)
      for (int j = 1; j <= l; j++) {
        Z(i, j) = 0.0;
        Z(j, i) = 0.0;
      }
  }
}

/* TQL -- asymrho.f:855-921: QL iterations on the tridiagonal form, then
 * eigenvalues sorted ascending with their vectors (columns of z); returns
 * nonzero where the reference stops with 'FAIL' */
static int tql(int md, int n, double *z, double *d, double *e)
{
  const double eps = 1e-12;
  const int niter = 50;
  tred2(md, n, z, d, e);
  for (int i = 2; i <= n; i++) e[i - 2] = e[i - 1];
  double f = 0.0, b = 0.0;
  e[n - 1] = 0.0;
  for (int l = 1; l <= n; l++) {
    int j = 0;
    double h = eps * (fabs(d[l - 1]) + fabs(e[l - 1]));
    int lp1 = l + 1;
    if (b - h < 0) b = h;
    int m;
    for (m = l; m <= n; m++)
      if (fabs(e[m - 1]) - b <= 0) break;
    if (m > n) m = n;   /* e(n) = 0 ends the search there */
    if (m != l) {
      for (;;) {
        if (j == niter) return 1;
        j = j + 1;
        double p = (d[lp1 - 1] - d[l - 1]) / (2 * e[l - 1]);
        double r = sqrt(p * p + 1);
        if (p < 0) h = d[l - 1] - e[l - 1] / (p - r);
        else h = d[l - 1] - e[l - 1] / (p + r);
        for (int i = l; i <= n; i++) d[i - 1] = d[i - 1] - h;
        f = f + h;
        p = d[m - 1];
        double c = 1.0, s = 0.0;
        int mm1 = m - 1;
        if (mm1 - l >= 0) {
          for (int lmip = l; lmip <= mm1; lmip++) {
            int i = l + mm1 - lmip, ip1 = i + 1;
            double g = c * e[i - 1];
            h = c * p;
            if (fabs(p) - fabs(e[i - 1]) >= 0) {
              c = e[i - 1] / p;
              r = sqrt(c * c + 1.0);
              e[ip1 - 1] = s * p * r;
              s = c / r;
              c = 1.0 / r;
            } else {
              c = p / e[i - 1];
              r = sqrt(c * c + 1);
              e[ip1 - 1] = s * e[i - 1] * r;
              s = 1 / r;
              c = c / r;
            }
            p = c * d[i - 1] - s * g;
            d[ip1 - 1] = h + s * (c * g + s * d[i - 1]);
            for (int k = 1; k <= n; k++) {
              h = Z(k, ip1);
              Z(k, ip1) = s * Z(k, i) + c * h;
              Z(k, i) = c * Z(k, i) - s * h;
            }
          }
        }
        e[l - 1] = s * p;
        d[l - 1] = c * p;
        if (fabs(e[l - 1]) - b <= 0) break;
      }
    }
    d[l - 1] = d[l - 1] + f;
  }
  for (int i = 1; i <= n; i++) {
    int ip1 = i + 1, k = i;
    double p = d[i - 1];
    if (n - i > 0)
      for (int jj = ip1; jj <= n; jj++)
        if (d[jj - 1] - p < 0) {
          k = jj;
          p = d[jj - 1];
        }
    if (k != i) {
      d[k - 1] = d[i - 1];
      d[i - 1] = p;
      for (int jj = 1; jj <= n; jj++) {
        p = Z(jj, i);
        Z(jj, i) = Z(jj, k);
        Z(jj, k) = p;
      }
    }
  }
  return 0;
}
#undef Z

/* wigd + calfac -- asymrho.f:1006-1053: d^j_{mk}(theta) as the factorial
 * sum in quad precision */
static qreal *g_fact = NULL;
static int g_maxfac = -1;

static void calfac(int maxfac)
{
  if (g_maxfac >= maxfac) return;
  free(g_fact);
  g_fact = (qreal *)malloc(sizeof(qreal) * (size_t)(maxfac + 1));
  g_fact[0] = 1.0;
  for (int i = 1; i <= maxfac; i++) g_fact[i] = g_fact[i - 1] * (qreal)(double)i;
  g_maxfac = maxfac;
}

/* x**n for an integer n >= 0, by binary exponentiation as the Fortran
 * runtime's integer power does */
static qreal qpowi(qreal x, int n)
{
  qreal r = 1.0;
  while (n > 0) {
    if (n & 1) r *= x;
    x *= x;
    n >>= 1;
  }
  return r;
}

double orc_wigd(int j, int m, int k, double theta)
{
  calfac(2 * j + 2 > 1754 ? 2 * j + 2 : 1754);
  const qreal *fact = g_fact;
  qreal pre1 = QSQRT(fact[j + k]) * QSQRT(fact[j - k]) * QSQRT(fact[j + m]) * QSQRT(fact[j - m]);
  int nulow = k - m > 0 ? k - m : 0;
  int nuup = (j + k) < (j - m) ? (j + k) : (j - m);
  qreal thehlf = (qreal)0.5 * (qreal)theta;
  qreal sum = 0.0;
  const qreal ch = QCOS(thehlf), sh = -QSIN(thehlf);
  for (int nu = nulow; nu <= nuup; nu++) {
    qreal denorm = fact[j - m - nu] * fact[j + k - nu] * fact[nu + m - k] * fact[nu] * (qreal)((nu % 2) ? -1 : 1);
    qreal pre2 = pre1 / denorm;
    qreal cosfac = ch, sinfac = sh;
    cosfac = qpowi(cosfac, 2 * j + k - m - 2 * nu);
    sinfac = qpowi(sinfac, m - k + 2 * nu);
    sum = sum + pre2 * cosfac * sinfac;
  }
  return (double)sum;
}

/* The eigen-decomposition of asymrho.f:114-279: for every j the even-k and
 * odd-k blocks of the rotational matrix diagonalised by TQL; energies in
 * engevn/engodd, coefficient vectors stacked in eigevn/eigodd in the
 * reference's order. */
struct orc_asym {
  int jmax;
  double *engevn, *engodd, *eigevn, *eigodd;
  int nstev, nstod;
};

static struct orc_asym *asym_build(int maxj, double A, double B, double C, int *status)
{
  struct orc_asym *a = (struct orc_asym *)calloc(1, sizeof(struct orc_asym));
  int maxd = 2 * maxj + 1;
  size_t nst = (size_t)(maxj + 1) * (maxj + 1);
  size_t ncf = (size_t)(4L * maxj * maxj * maxj + 12L * maxj * maxj + 11L * maxj + 3) / 3;
  a->jmax = maxj;
  a->engevn = (double *)calloc(nst, sizeof(double));
  a->engodd = (double *)calloc(nst, sizeof(double));
  a->eigevn = (double *)calloc(ncf, sizeof(double));
  a->eigodd = (double *)calloc(ncf, sizeof(double));
  double *H = (double *)calloc((size_t)maxd * maxd, sizeof(double));
  double *ev = (double *)calloc((size_t)maxd, sizeof(double)), *wk = (double *)calloc((size_t)maxd, sizeof(double));
  int ivec = 0, jvec = 0;
  *status = PIMC_OK;
  for (int j = 0; j <= maxj; j++) {
    int kevnst, koddst, ndimev, ndimod;
    if (j % 2 == 0) { kevnst = -j; koddst = -j + 1; ndimev = j + 1; ndimod = j; }
    else { kevnst = -j + 1; koddst = -j; ndimev = j; ndimod = j + 1; }
    for (int par = 0; par < 2; par++) {
      int kst = par ? koddst : kevnst, nd = par ? ndimod : ndimev;
      if (nd == 0) continue;
      memset(H, 0, sizeof(double) * (size_t)maxd * maxd);
      int irow = 0;
      for (int k = kst; k <= j; k += 2) {
        irow++;
        int jcol = 0;
        for (int kp = kst; kp <= k; kp += 2) {
          jcol++;
          double el = orc_rotmat(j, k, kp, A, B, C);
          H[(jcol - 1) * maxd + (irow - 1)] = el;
          H[(irow - 1) * maxd + (jcol - 1)] = el;
        }
      }
      if (tql(maxd, nd, H, ev, wk)) *status = PIMC_ERR_BAD_ARG;
      for (int ist = 1; ist <= nd; ist++) {
        if (par) a->engodd[a->nstod++] = ev[ist - 1];
        else a->engevn[a->nstev++] = ev[ist - 1];
        for (int ibs = 1; ibs <= nd; ibs++) {
          double v = H[(ist - 1) * maxd + (ibs - 1)];
          if (par) a->eigodd[jvec++] = v;
          else a->eigevn[ivec++] = v;
        }
      }
    }
  }
  free(H); free(ev); free(wk);
  return a;
}

static void asym_free(struct orc_asym *a)
{
  if (!a) return;
  free(a->engevn); free(a->engodd); free(a->eigevn); free(a->eigodd);
  free(a);
}

/* the "AT BETA" and "AT TAU" partition functions of asymrho.f:299-423:
 * info[0..8] = Z, E (cm^-1), Cv (kB) for even k, odd k and all states at
 * beta; info[9..14] = Z, E for even, odd, all at tau */
static void asym_info(const struct orc_asym *a, double beta, double tau, double temprt, double *info)
{
  const double boltz = 0.6950356;
  for (int pass = 0; pass < 2; pass++) {
    double bt = pass ? tau : beta;
    double zp[2] = {0, 0}, ea[2] = {0, 0}, es[2] = {0, 0};
    int ist[2] = {0, 0};
    for (int j = 0; j <= a->jmax; j++) {
      int nd[2] = {j % 2 == 0 ? j + 1 : j, j % 2 == 0 ? j : j + 1};
      int ndegen = 2 * j + 1;
      for (int par = 0; par < 2; par++) {
        const double *eng = par ? a->engodd : a->engevn;
        double s = 0, se = 0, sq = 0;
        for (int i = 1; i <= nd[par]; i++) {
          double energy = eng[ist[par] + i - 1];
          s = s + exp(-bt * energy);
          se = se + energy * exp(-bt * energy);
          sq = sq + energy * energy * exp(-bt * energy);
        }
        zp[par] = zp[par] + ndegen * s;
        ea[par] = ea[par] + ndegen * se;
        es[par] = es[par] + ndegen * sq;
        ist[par] += nd[par];
      }
    }
    double eacl = ea[0] + ea[1], escl = es[0] + es[1], zcl = zp[0] + zp[1];
    double e0 = ea[0] / zp[0], e1 = ea[1] / zp[1];
    if (pass == 0) {
      double s0 = es[0] / zp[0], s1 = es[1] / zp[1];
      double kt2 = boltz * boltz * temprt * temprt;
      info[0] = zp[0]; info[1] = e0; info[2] = (s0 - e0 * e0) / kt2;
      info[3] = zp[1]; info[4] = e1; info[5] = (s1 - e1 * e1) / kt2;
      double ec = eacl / zcl, sc = escl / zcl;
      info[6] = zcl; info[7] = ec; info[8] = (sc - ec * ec) / kt2;
    } else {
      info[9] = zp[0]; info[10] = e0; info[11] = zp[1]; info[12] = e1; info[13] = zcl; info[14] = eacl / zcl;
    }
  }
}

/* asymrho.f:34-735 at a list of grid points (ith, iphi, ichi in degrees,
 * each taken as computed, not as a symmetric copy): rho, erot (cm^-1),
 * erotsq per point; info[15] as asym_info.  Returns PIMC_ERR_BAD_ARG where
 * the reference stops (iodevn out of range, too large a contribution from
 * the highest state, TQL failure). */
int orc_asymrho_points(double temprt, int nslice, int iodevn, double A, double B, double C, int maxj, int npts,
                       const int *ith, const int *iphi, const int *ichi, double *rho, double *erot, double *esq,
                       double *info)
{
  const double pi = 3.14159265358979323846, eps = 1.e-16, boltz = 0.6950356;
  if (iodevn > 1 || iodevn < -1 || maxj < 0 || maxj > 876) return PIMC_ERR_BAD_ARG;
  double beta = 1.0 / (boltz * temprt), tau = beta / (double)nslice;
  int st;
  struct orc_asym *a = asym_build(maxj, A, B, C, &st);
  if (st) { asym_free(a); return st; }
  double emax = -1e300;
  for (int i = 0; i < a->nstev; i++) emax = a->engevn[i] > emax ? a->engevn[i] : emax;
  for (int i = 0; i < a->nstod; i++) emax = a->engodd[i] > emax ? a->engodd[i] : emax;
  if (exp(-beta * emax) > 1.e-8 || exp(-tau * emax) > 1.e-8) { asym_free(a); return PIMC_ERR_BAD_ARG; }
  if (info) asym_info(a, beta, tau, temprt, info);
  /* dlist(j, m, k, ith) of asymrho.f:102-112 for the theta in use */
  const int w = 2 * maxj + 1;
  double *dl = (double *)malloc(sizeof(double) * (size_t)(maxj + 1) * w * w);
  int dl_ith = -1;
  for (int p = 0; p < npts; p++) {
    double theta = (double)ith[p] * pi / 180.0, phi = (double)iphi[p] * pi / 180.0, chi = (double)ichi[p] * pi / 180.0;
    if (ith[p] != dl_ith) {
      for (int j = 0; j <= maxj; j++)
        for (int m = -j; m <= j; m++)
          for (int k = -j; k <= j; k++) dl[((size_t)j * w + (m + maxj)) * w + (k + maxj)] = orc_wigd(j, m, k, theta);
      dl_ith = ith[p];
    }
    double r[2] = {0, 0}, e[2] = {0, 0}, s[2] = {0, 0};
    for (int par = 0; par < 2; par++) {
      if ((par == 0 && iodevn == 1) || (par == 1 && iodevn == 0)) continue;
      const double *eng = par ? a->engodd : a->engevn, *eig = par ? a->eigodd : a->eigevn;
      int ist = 0, ivec = 0;
      for (int j = 0; j <= maxj; j++) {
        int kst, nd;
        if (j % 2 == 0) { kst = par ? -j + 1 : -j; nd = par ? j : j + 1; }
        else { kst = par ? -j : -j + 1; nd = par ? j + 1 : j; }
        double pre = (double)(2 * j + 1) / (8.0 * pi * pi);
        double rho1 = 0, erot1 = 0, esq1 = 0;
        for (int is = 1; is <= nd; is++) {
          double energy = eng[ist++];
          double expo = exp(-tau * energy);
          if (!(expo * pre < eps)) {
            int im = 0;
            double rho2 = 0.0;
            for (int m = kst; m <= j; m += 2) {
              im++;
              double coef1 = eig[im + ivec - 1];
              int ik = 0;
              double rho3 = 0.0;
              for (int k = kst; k <= j; k += 2) {
                ik++;
                double coef2 = eig[ik + ivec - 1];
                rho3 = rho3 + coef2 * dl[((size_t)j * w + (m + maxj)) * w + (k + maxj)] *
                                  cos((double)m * phi + (double)k * chi);
              }
              rho2 = rho2 + coef1 * rho3;
            }
            rho1 = rho1 + rho2 * expo;
            erot1 = erot1 + expo * rho2 * energy;
            esq1 = esq1 + expo * rho2 * energy * energy;
          }
          ivec += nd;
        }
        r[par] = r[par] + pre * rho1;
        e[par] = e[par] + pre * erot1;
        s[par] = s[par] + pre * esq1;
      }
      if (fabs(r[par]) > 1.0e-16) {
        e[par] = e[par] / r[par];
        s[par] = s[par] / r[par];
      } else {
        e[par] = 0.0;
        s[par] = 0.0;
      }
    }
    if (iodevn == 0) { rho[p] = r[0]; erot[p] = e[0]; esq[p] = s[0]; }
    else if (iodevn == 1) { rho[p] = r[1]; erot[p] = e[1]; esq[p] = s[1]; }
    else {
      double rc = r[1] + r[0];
      rho[p] = r[0] + r[1];
      erot[p] = (e[1] * r[1] + e[0] * r[0]) / (r[0] + r[1]);
      esq[p] = (s[1] * r[1] + s[0] * r[0]) / (r[0] + r[1]);
      if (fabs(rc) < 1.e-16) { erot[p] = 0.0; esq[p] = 0.0; }
    }
  }
  free(dl);
  asym_free(a);
  return PIMC_OK;
}

/* the energies of the eigen-decomposition (for known-answer checks):
 * eng[0..nstev) even-k block, then the odd-k block; returns nstev+nstod */
int orc_asymrho_energies(int maxj, double A, double B, double C, double *eng)
{
  int st;
  struct orc_asym *a = asym_build(maxj, A, B, C, &st);
  int n = a->nstev + a->nstod;
  if (eng) {
    memcpy(eng, a->engevn, sizeof(double) * (size_t)a->nstev);
    memcpy(eng + a->nstev, a->engodd, sizeof(double) * (size_t)a->nstod);
  }
  asym_free(a);
  return st ? -1 : n;
}
