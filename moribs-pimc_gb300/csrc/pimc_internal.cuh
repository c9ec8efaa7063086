// pimc_internal.cuh -- device-side data layout and leaf routines of the GB300
// sampling path.  Each leaf names the reference routine whose arithmetic it
// follows; the double-precision versions keep the reference's operation
// order so that results agree with it to rounding.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#define PIMC_PI 3.14159265358979323846
#define PIMC_WNO2K 0.6950356          /* mc_const.h:16 */
#define PIMC_RZERO 1.0e-10            /* mc_confg.h:59 */
#define PIMC_BLOCK 256                /* threads per move CTA */
#define PIMC_BIS_THREADS 512          /* bisection CTA: 2(M-1) slots x partners over 16 warps */
#define PIMC_ROT_THREADS 320          /* rotational move CTA: 8 pair warps, a density warp, a commit warp */
#define PIMC_RED_BUF 4096             /* doubles in a CTA's reduction buffer */
#define PIMC_MAX_SEG 64               /* largest bisection segment (levels <= 6) */
#define PIMC_MAX_ROTORS 16            /* NumbRotLim (mc_setup.cc:63) */

// error bits raised on the device and read back by the host
enum { DERR_GRID_RANGE = 1, DERR_NEG_DENSITY = 2, DERR_STREAM = 4, DERR_TIMEOUT = 8, DERR_PERM = 16 };

struct DevTables {
  // 1D spline, SPot1D (mc_poten.cc:379-438,624-639); float copies for the FP32 path
  int n1d;
  const double *g1d, *p1d, *y21d;
  const float *g1d32, *p1d32, *y21d32;
  double alpha1d, unode1d, c61d;
  int uni1d;                    // grid uniform: direct index (see splint)
  double x01d, ih1d;
  // 2D bilinear, LPot2D (mc_poten.cc:688-729)
  int nr2d, nc2d;
  double dr2d, dc2d;
  const double *rg2d, *cg2d, *pot2d;
  const float *rg2d32, *cg2d32, *pot2d32;
  // 3D, vcord/vcalc (vcord.f, vcalc.f) on a generalised angular grid
  int rgrd, thgrd, chgrd, chfold;
  double rvmin, rvmax, rvstep, dth3, dch3;
  const double *vtab;
  const float *vtab32;
  // linear rotor density, SRotDens (mc_poten.cc:548-622)
  int nrot;
  const double *rg, *rd, *rdv, *rde, *rd_y2, *rdv_y2, *rde_y2;
  int unirot;
  double x0rot, ihrot;
  // nonlinear rotor density, rotden/rotpro (rotden.f, rotpro_sub.f)
  int nth, nph, nch;
  double dthd, dphd, dchd;
  const double *rho, *erot, *esq;
  const float *rho32;
  // spherical rotor-atom table, vspher (vspher.f)
  int nsph;
  double sph_r0, sph_rmax, sph_rstep;
  const double *sph;
  // float constants of the FP32 leaves, converted once on the host so that
  // those leaves execute no double-precision instruction
  float f_x01d, f_ih1d, f_c61d, f_unode1d, f_alpha1d, f_dr2d, f_dc2d;
  float f_thscale, f_chscale, f_rvmin, f_rvmax, f_rvstep;     // vcord32: degrees per grid step folded in
  float f_dscale[3];                                            // rotden32: theta, phi, chi grid steps per radian
  // packed float tables of the FP32 path: one 16-byte load per evaluation
  const float4 *sp1d4;          // 1D spline interval k: (y_k, y2_k, y_k+1, y2_k+1); uniform grids only
  float f_h1d, f_h2_6;          // step and step^2 / 6
  const float4 *pot2d4;         // 2D cell (ir, ic): corners (ir,ic), (ir+1,ic), (ir+1,ic+1), (ir,ic+1)
  float f_rmin2d, f_cmin2d;
  const float4 *vtab4;          // 3D point: value and its one-sided differences along r, theta, chi
  float f_irstep;
  const float4 *rho4;           // top density point: value and differences along chi, phi, theta
  const float4 *rd4;            // linear-rotor density spline interval k: (y_k, y2_k, y_k+1, y2_k+1), uniform grid
  float f_ihrot, f_hrot2_6;
  // reciprocals of grid steps for the double-precision leaves: a division by
  // a grid constant becomes a multiplication (within an ulp of the quotient)
  double d_thscale, d_chscale, d_irstep, d_idr2d, d_idc2d, d_dscale[3];
};

struct DevSys {
  int na, nap;                 // atoms, padded row length of the slice-major arrays
  int P, Q, R;                 // NumbTimes, NumbRotTimes, RotRatio
  int ntypes, imtype, nrotors, rot_first;   // rotor type, its count, its first global atom
  int numb[2], molecule[2], stat[2], levels[2], first[2];
  double lambda[2], mcstep[2];
  double bis_sq[2][8];         // sqrt(1 / (lambda tau 2^(L-l))): gauss()'s sqrt(alpha) at level l (mc_randg.cc:149)
  double bis_isq[2][8];        // its inverse (the bisection midpoints, both precisions)
  double tau, rot_tau, beta, temperature, rtstep;
  int ispher, rot_den_type, rot_odevn, rn_ratio;
  double rot_eoff, abc[3];
  float rs_coef[3];            // FP32 rattle-and-shake density: 1/A - 1/B - 1/C and its cyclic forms (rotden.f:218-286)
  float rs_scale;              // 1 / (4 tau_rot) in cm: the log-density difference's factor in the accept (mc_piqmc.cc:1145-1178)
  int minimage;
  double box[3];
  int mixed;                   // 1: FP32 table interpolation with FP64 sums
  unsigned long long wait_ns;  // limit of a persistent sweep's wait for its neighbours
};

// path state on the device
//   x/y/z[t*nap + a]: bead of global atom a at slice t (slice-major so a
//   partner sweep at one slice is a unit-stride read);
//   ang[k*nrotors*Q + r*Q + q], k = {phi, cos theta, chi}: rotor r at rotational slice q;
//   cosv[k*nrotors*Q + r*Q + q]: its unit vector (MCCosine).
//   b4: float copies of the beads, one 16-byte word each, read by the FP32 path;
//   rp_cache/rp_ok[r*Q + q]: the rotor's potential summed over the R
//   translational slices of rotational slice q with its current orientation,
//   valid while no bead of those slices and no orientation at q has changed;
//   rl_cache/rl_ok[r*Q + q]: the current link density rho(q, q+1).
//   Both caches hold exactly the value a fresh evaluation would return.
// TPathWorm (mc_qworm.h:32-48) with MCWormInit's constants (mc_qworm.cc:49-82)
// and the QWTotal/QWAccep counters (mc_qworm.h:52-53) of the worm type
struct DevWorm {
  int exists, ira, masha, atom_i, atom_m;
  int type, m, numb, first;
  double qw_norm, cut2, twave2;
  double qwtot[7], qwacc[7];
};

struct DevState {
  double *x, *y, *z;
  float4 *b4;                   // float copy of the beads (x, y, z, 0) for the FP32 path
  double *ang, *cosv;
  float *cosvf;
  int *pindex;
  int *mctype;
  unsigned int *err;
  double *rp_cache, *rl_cache;
  int *rp_ok, *rl_ok;
  const DevWorm *worm;          // the worm, when the worm algorithm is on (else null)
};

struct Ctx {
  DevSys s;
  DevTables t;
  DevState st;
};

// pair-density histograms (counts), [dtype][bins] as _gr1D/_gr2D/_gr3D
// (mc_estim.cc:257-287); g3 is null without a nonlinear rotor
#ifndef PIMC_BINSR                 /* the same values as pimc_types.h */
#define PIMC_BINSR 300
#define PIMC_BINST 50
#define PIMC_BINSC 100
#define PIMC_DENS_MIN_RADIUS 0.0
#define PIMC_DENS_MAX_RADIUS 15.0
#endif
struct DensHist {
  unsigned long long *g1, *g2, *g3;
  // relative Euler angles of adjacent rotational slices of a nonlinear rotor
  // (GetRotE3D's _relthe_sum[BINST], _relphi_sum[BINSC], _relchi_sum[BINSC],
  // mc_estim.cc:1044-1057), in that order; null otherwise
  unsigned long long *rel;
};

// ------------------------------------------------------------------ frames
// Body frame of a nonlinear rotor: the columns of matpre(phi, acos(cost), chi)
// (rotden.f:136-163, vcord.f:31-36) plus |hatz| as dnorm computes it.
struct Frame {
  double e[3];          // phi, cos theta, chi
  double m[9];          // rotmat(i,j) at m[i*3+j]
  double hz_norm;
  float mf[9];          // float copy for the FP32 path
  float hzf;
};

__device__ __forceinline__ void matpre(const double e[3], double m[9])
{
  double sp, cp, st, ct, sk, ck;
  sincos(e[0], &sp, &cp);
  sincos(e[1], &st, &ct);
  sincos(e[2], &sk, &ck);
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

// cos and sin of theta = acos(cost) are cost and sqrt((1-cost)(1+cost)): the
// same matrix as matpre(phi, acos(cost), chi) without the acos/sincos chain
// the float frame of the FP32 path, from the float-rounded angles
__device__ __forceinline__ void make_frame32(float phi, float cost, float chi, float mf[9], float *hzf)
{
  float sp, cp, sk, ck;
  sincosf(phi, &sp, &cp);
  sincosf(chi, &sk, &ck);
  float ct = cost, st = sqrtf(fmaxf((1.0f - cost) * (1.0f + cost), 0.0f));
  mf[0] = cp * ct * ck - sp * sk;
  mf[1] = -cp * ct * sk - sp * ck;
  mf[2] = cp * st;
  mf[3] = sp * ct * ck + cp * sk;
  mf[4] = -sp * ct * sk + cp * ck;
  mf[5] = sp * st;
  mf[6] = -st * ck;
  mf[7] = st * sk;
  mf[8] = ct;
  *hzf = sqrtf(mf[2] * mf[2] + mf[5] * mf[5] + mf[8] * mf[8]);
}

// the float unit vector of (phi, cos theta) on the FP32 path
__device__ __forceinline__ void unit_vector32(float phi, float cost, float v[3])
{
  float sp, cp;
  sincosf(phi, &sp, &cp);
  float st = sqrtf(fmaxf(1.0f - cost * cost, 0.0f));
  v[0] = st * cp;
  v[1] = st * sp;
  v[2] = cost;
}

// the double-precision frame (m, hz_norm) from the angles and the sines and
// cosines of phi and chi
__device__ __forceinline__ void frame_from_sincos(double phi, double cost, double chi, double sp, double cp,
                                                  double sk, double ck, Frame &f)
{
  double ct = cost, st = sqrt((1.0 - cost) * (1.0 + cost));
  f.e[0] = phi;
  f.e[1] = cost;
  f.e[2] = chi;
  f.m[0] = cp * ct * ck - sp * sk;
  f.m[1] = -cp * ct * sk - sp * ck;
  f.m[2] = cp * st;
  f.m[3] = sp * ct * ck + cp * sk;
  f.m[4] = -sp * ct * sk + cp * ck;
  f.m[5] = sp * st;
  f.m[6] = -st * ck;
  f.m[7] = st * sk;
  f.m[8] = ct;
  double s = 0.0;
  s = s + f.m[2] * f.m[2];
  s = s + f.m[5] * f.m[5];
  s = s + f.m[8] * f.m[8];
  f.hz_norm = sqrt(s);
}

// the double-precision frame (m, hz_norm) only
__device__ __forceinline__ void make_frame64(double phi, double cost, double chi, Frame &f)
{
  double sp, cp, sk, ck;
  sincos(phi, &sp, &cp);
  sincos(chi, &sk, &ck);
  frame_from_sincos(phi, cost, chi, sp, cp, sk, ck, f);
}

__device__ __forceinline__ void make_frame(double phi, double cost, double chi, Frame &f)
{
  make_frame64(phi, cost, chi, f);
  make_frame32((float)phi, (float)cost, (float)chi, f.mf, &f.hzf);
}

// ------------------------------------------------------------------ leaves

// klo of splint's bisection (mc_utils.cc:170-176): the largest k <= n-2 with
// xa[k] <= x.  On a uniform grid (uni != 0) the index is computed and then
// corrected by whole steps until that condition holds, which returns the
// bisection's klo exactly.
__device__ __forceinline__ int spline_klo(const double *__restrict__ xa, int n, double x, int uni, double x0, double ih)
{
  if (uni && x == x) {
    double g = (x - x0) * ih;
    int k = g < 0.0 ? 0 : (g > (double)(n - 2) ? n - 2 : (int)g);
    while (k < n - 2 && __ldg(xa + k + 1) <= x) k++;
    while (k > 0 && __ldg(xa + k) > x) k--;
    return k;
  }
  int klo = 0, khi = n - 1;
  while (khi - klo > 1) {
    int k = (khi + klo) >> 1;
    if (__ldg(xa + k) > x) khi = k;
    else klo = k;
  }
  return klo;
}

// splint (mc_utils.cc:156-186): bisection for klo, then the cubic
__device__ __forceinline__ double splint(const double *__restrict__ xa, const double *__restrict__ ya,
                                         const double *__restrict__ y2a, int n, double x, int uni = 0,
                                         double x0 = 0.0, double ih = 0.0)
{
  int klo = spline_klo(xa, n, x, uni, x0, ih), khi = klo + 1;
  double xk = __ldg(xa + khi), xl = __ldg(xa + klo);
  double h = xk - xl;
  double a, b;
  if (uni) {
    // uniform grid: the step's reciprocal instead of two divisions
    a = (xk - x) * ih;
    b = (x - xl) * ih;
  } else {
    a = (xk - x) / h;
    b = (x - xl) / h;
  }
  return a * __ldg(ya + klo) + b * __ldg(ya + khi) +
         ((a * a * a - a) * __ldg(y2a + klo) + (b * b * b - b) * __ldg(y2a + khi)) * (h * h) * (1.0 / 6.0);
}

// SPot1D (mc_poten.cc:624-639)
__device__ __forceinline__ double spot1d(const DevTables &t, double r)
{
  if (r >= __ldg(t.g1d + t.n1d - 1)) return -t.c61d / pow(r, 6.0);
  if (r <= __ldg(t.g1d)) return t.unode1d * exp(-t.alpha1d * r);
  return splint(t.g1d, t.p1d, t.y21d, t.n1d, r, t.uni1d, t.x01d, t.ih1d);
}

// LPot2D (mc_poten.cc:688-729): clamped index, unclamped fraction
__device__ __forceinline__ double lpot2d(const DevTables &t, double r, double cost)
{
  double rmin = __ldg(t.rg2d), cmin = __ldg(t.cg2d);
  int ir = (int)floor((r - rmin) * t.d_idr2d);
  int ic = (int)floor((cost - cmin) * t.d_idc2d);
  if (ir < 0) ir = 0;
  else if (ir >= t.nr2d - 1) ir = t.nr2d - 2;
  if (ic < 0) ic = 0;
  else if (ic >= t.nc2d - 1) ic = t.nc2d - 2;
  const double *p = t.pot2d + (size_t)ir * t.nc2d + ic;
  double y1 = __ldg(p), y4 = __ldg(p + 1);
  double y2 = __ldg(p + t.nc2d), y3 = __ldg(p + t.nc2d + 1);
  double r1 = __ldg(t.rg2d + ir), r2 = __ldg(t.rg2d + ir + 1);
  double c1 = __ldg(t.cg2d + ic), c2 = __ldg(t.cg2d + ic + 1);
  (void)r2;
  (void)c2;
  double dr = (r - r1) * t.d_idr2d;          // (r - r1) / (r2 - r1) on the uniform grid
  double dc = (cost - c1) * t.d_idc2d;
  return (1.0 - dr) * (1.0 - dc) * y1 + dr * (1.0 - dc) * y2 + dr * dc * y3 + (1.0 - dr) * dc * y4;
}

// SRotDens / SRotDensDeriv / SRotDensEsqrt (mc_poten.cc:548-622)
__device__ __forceinline__ double srotdens(const DevTables &t, double g, int which)
{
  const double *d = which == 0 ? t.rd : (which == 1 ? t.rdv : t.rde);
  const double *y2 = which == 0 ? t.rd_y2 : (which == 1 ? t.rdv_y2 : t.rde_y2);
  int n = t.nrot;
  if (g > __ldg(t.rg + n - 1)) return which == 0 ? __ldg(d + n - 1) : 0.0;
  if (g < __ldg(t.rg)) {
    double rl = __ldg(t.rg), rr = __ldg(t.rg + 1);
    double salpha = (__ldg(d + 1) - __ldg(d)) / (rr - rl);
    double sbeta = (__ldg(d) * rr - __ldg(d + 1) * rl) / (rr - rl);
    return salpha * g + sbeta;
  }
  return splint(t.rg, d, y2, n, g, t.unirot, t.x0rot, t.ihrot);
}

// SRotDens on the FP32 path from dc = 1 - cos(gamma) >= 0 (computed as
// |n - n'|^2 / 2, which keeps its relative precision for small angles): the
// spline interval is counted down from the top node cos(gamma) = 1 of the
// uniform grid, so the weights do not lose the digits that cos(gamma) itself
// would
__device__ __forceinline__ float srotdens32(const DevTables &t, float dc)
{
  const int n = t.nrot;
  float tt = fmaxf(dc, 0.0f) * t.f_ihrot;           // grid steps below the top node
  int kk = min((int)tt, n - 2);
  float b = 1.0f - (tt - (float)kk);                // weight of node n-1-kk
  if (b < 0.0f) b = 0.0f;
  float a = 1.0f - b;
  float4 w = __ldg(t.rd4 + (n - 2 - kk));
  return a * w.x + b * w.z + ((a * a * a - a) * w.y + (b * b * b - b) * w.w) * t.f_hrot2_6;
}

// 1 - n.n' of two unit vectors, stable for small angles
__device__ __forceinline__ float one_minus_dot32(const float *na, const float *nb)
{
  float dx = na[0] - nb[0], dy = na[1] - nb[1], dz = na[2] - nb[2];
  return 0.5f * (dx * dx + dy * dy + dz * dz);
}

__device__ __forceinline__ double within1(double v)
{
  if (v > 1.0) v = 1.0;
  if (v < -1.0) v = -1.0;
  return v;
}

// deleul (rotden.f:32-134): Euler angles of rotma1^T rotmat
__device__ __forceinline__ void deleul(const double m1[9], const double m2in[9], double rel[3])
{
  double m2[9];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      double s = 0.0;
      for (int k = 0; k < 3; k++) s = s + m1[k * 3 + i] * m2in[k * 3 + j];
      m2[i * 3 + j] = s;
    }
  const double small = 1.e-08, pi = PIMC_PI;
  double cost = within1(m2[8]);
  double theta2 = acos(cost);
  double sint = sqrt((1.0 - cost) * (1.0 + cost));   // sin(acos(cost)), independent of the acos
  double phi2, chi2, cchi, schi;
  if (fabs(1.0 - cost) < small) {
    phi2 = 0.0;
    cchi = within1(m2[0]);
    schi = within1(m2[3]);
    chi2 = (schi > 0.0) ? acos(cchi) : 2.0 * pi - acos(cchi);
  } else if (fabs(1.0 + cost) < small) {
    phi2 = 0.0;
    cchi = within1(m2[4]);
    schi = within1(m2[1]);
    chi2 = (schi > 0.0) ? acos(cchi) : 2.0 * pi - acos(cchi);
  } else {
    double isint = 1.0 / sint;
    double cphi = within1(m2[2] * isint);
    double sphi = within1(m2[5] * isint);
    cchi = within1(-m2[6] * isint);
    schi = within1(m2[7] * isint);
    phi2 = (sphi > 0.0) ? acos(cphi) : 2.0 * pi - acos(cphi);
    chi2 = (schi > 0.0) ? acos(cchi) : 2.0 * pi - acos(cchi);
  }
  rel[0] = phi2;
  rel[1] = theta2;
  rel[2] = chi2;
}

// Note on the edge guards below (rotpro, vcalc, vspher): the reference tests
// "index != last" after clamping the index to <= last.  Written that way,
// ptxas 13.0 at its default optimisation level drops the guarded terms for
// sm_103a (the same source is correct at -O0); "index < last" is the same
// condition for a clamped index and compiles correctly.
//
// Grid coordinates of the FP64 leaves are products with precomputed
// reciprocal steps, which lie within a few ulps of the reference's quotients.
// Only at a grid node can that choose the neighbouring cell, and vcalc's and
// rotpro's one-sided differences are not continuous across a node; there the
// coordinate is recomputed with the reference's own divisions.
// f: the coordinate's distance above its cell's lower node, x - (int)x
__device__ __forceinline__ bool near_node(double f) { return f < 1e-9 || f > 1.0 - 1e-9; }

// rotden (rotden.f:1-31) -> rotpro (rotpro_sub.f:1-64) on the generalised
// (theta, phi, chi) grid; returns the rho value, sets *bad on an index out
// of range (the reference's istop).  which_mask bit0: rho, bit1: erot+esq.
__device__ __forceinline__ double rotden_rho(const DevTables &t, const Frame &f1, const Frame &f2, int *bad,
                                            double *erot_out, double *esq_out)
{
  double rel[3];
  deleul(f1.m, f2.m, rel);
  double xt = rel[1] * t.d_dscale[0], xp = rel[0] * t.d_dscale[1], xc = rel[2] * t.d_dscale[2];
  int ichi = (int)xc, iphi = (int)xp, ith = (int)xt;
  double fc = xc - (double)ichi, fp = xp - (double)iphi, ft = xt - (double)ith;
  if (near_node(ft)) {                                               // rotden.f:22-24
    xt = (rel[1] * 180.0 / PIMC_PI) / t.dthd;
    ith = (int)xt;
    ft = xt - (double)ith;
  }
  if (near_node(fp)) {
    xp = (rel[0] * 180.0 / PIMC_PI) / t.dphd;
    iphi = (int)xp;
    fp = xp - (double)iphi;
  }
  if (near_node(fc)) {
    xc = (rel[2] * 180.0 / PIMC_PI) / t.dchd;
    ichi = (int)xc;
    fc = xc - (double)ichi;
  }
  if (ichi > t.nch - 1 || ichi < 0) { ichi = 0; fc = xc; *bad = 1; }
  if (iphi > t.nph - 1 || iphi < 0) { iphi = 0; fp = xp; *bad = 1; }
  if (ith > t.nth - 1 || ith < 0) { ith = 0; ft = xt; *bad = 1; }
  size_t nph = t.nph, nch = t.nch;
  size_t i0 = ((size_t)ith * nph + iphi) * nch + ichi;
  double r0 = __ldg(t.rho + i0);
  double dc = 0.0, dp = 0.0, dt = 0.0;
  size_t ic = i0 + 1, ip = i0 + nch, itt = i0 + nph * nch;
  if (ichi < t.nch - 1) dc = __ldg(t.rho + ic) - r0;
  if (iphi < t.nph - 1) dp = __ldg(t.rho + ip) - r0;
  if (ith < t.nth - 1) dt = __ldg(t.rho + itt) - r0;
  double rho = r0 + dc * fc + dp * fp + dt * ft;
  if (erot_out) {
    double e0 = __ldg(t.erot + i0), s0 = __ldg(t.esq + i0);
    double ec = 0, ep = 0, et = 0, sc = 0, sp = 0, st = 0;
    if (ichi < t.nch - 1) { ec = __ldg(t.erot + ic) - e0; sc = __ldg(t.esq + ic) - s0; }
    if (iphi < t.nph - 1) { ep = __ldg(t.erot + ip) - e0; sp = __ldg(t.esq + ip) - s0; }
    if (ith < t.nth - 1) { et = __ldg(t.erot + itt) - e0; st = __ldg(t.esq + itt) - s0; }
    *erot_out = (e0 + ec * fc + ep * fp + et * ft) / PIMC_WNO2K;
    *esq_out = (s0 + sc * fc + sp * fp + st * ft) / (PIMC_WNO2K * PIMC_WNO2K);
  }
  return rho;
}

// rotden_rho's rho (no energies) with deleul's three acos on three lanes:
// lanes 3d, 3d+1, 3d+2 of the calling warp evaluate the density of frames
// (m1, m2in) given to them (the same on the three lanes), lane 3d+k taking
// theta, phi or chi; every lane of the warp calls it (lanes past the last
// full group compute on whatever frames they are given and their result is
// not used).  The same operations as deleul + rotden_rho, so the same value.
__device__ __forceinline__ double rotden_rho_lanes(const DevTables &t, const double *m1, const double *m2in,
                                                   int lane, int *bad)
{
  const int sub = lane % 3, base = lane - sub;
  double m2[9];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      double s = 0.0;
      for (int k = 0; k < 3; k++) s = s + m1[k * 3 + i] * m2in[k * 3 + j];
      m2[i * 3 + j] = s;
    }
  const double small = 1.e-08, pi = PIMC_PI;
  double cost = within1(m2[8]);
  double sint = sqrt((1.0 - cost) * (1.0 + cost));
  double cphi = 0.0, sphi = 0.0, cchi, schi;
  const bool pole0 = fabs(1.0 - cost) < small, pole1 = !pole0 && fabs(1.0 + cost) < small;
  if (pole0) {
    cchi = within1(m2[0]);
    schi = within1(m2[3]);
  } else if (pole1) {
    cchi = within1(m2[4]);
    schi = within1(m2[1]);
  } else {
    double isint = 1.0 / sint;
    cphi = within1(m2[2] * isint);
    sphi = within1(m2[5] * isint);
    cchi = within1(-m2[6] * isint);
    schi = within1(m2[7] * isint);
  }
  const double a = acos(sub == 0 ? cost : (sub == 1 ? cphi : cchi));
  const double theta2 = __shfl_sync(0xffffffffu, a, base & 31);
  const double acphi = __shfl_sync(0xffffffffu, a, (base + 1) & 31);
  const double acchi = __shfl_sync(0xffffffffu, a, (base + 2) & 31);
  double rel[3];
  rel[0] = (pole0 || pole1) ? 0.0 : ((sphi > 0.0) ? acphi : 2.0 * pi - acphi);
  rel[1] = theta2;
  rel[2] = (schi > 0.0) ? acchi : 2.0 * pi - acchi;
  double xt = rel[1] * t.d_dscale[0], xp = rel[0] * t.d_dscale[1], xc = rel[2] * t.d_dscale[2];
  int ichi = (int)xc, iphi = (int)xp, ith = (int)xt;
  double fc = xc - (double)ichi, fp = xp - (double)iphi, ft = xt - (double)ith;
  if (near_node(ft)) {                                               // rotden.f:22-24
    xt = (rel[1] * 180.0 / PIMC_PI) / t.dthd;
    ith = (int)xt;
    ft = xt - (double)ith;
  }
  if (near_node(fp)) {
    xp = (rel[0] * 180.0 / PIMC_PI) / t.dphd;
    iphi = (int)xp;
    fp = xp - (double)iphi;
  }
  if (near_node(fc)) {
    xc = (rel[2] * 180.0 / PIMC_PI) / t.dchd;
    ichi = (int)xc;
    fc = xc - (double)ichi;
  }
  if (ichi > t.nch - 1 || ichi < 0) { ichi = 0; fc = xc; *bad = 1; }
  if (iphi > t.nph - 1 || iphi < 0) { iphi = 0; fp = xp; *bad = 1; }
  if (ith > t.nth - 1 || ith < 0) { ith = 0; ft = xt; *bad = 1; }
  size_t nph = t.nph, nch = t.nch;
  size_t i0 = ((size_t)ith * nph + iphi) * nch + ichi;
  double r0 = __ldg(t.rho + i0);
  double dc = 0.0, dp = 0.0, dt = 0.0;
  if (ichi < t.nch - 1) dc = __ldg(t.rho + i0 + 1) - r0;
  if (iphi < t.nph - 1) dp = __ldg(t.rho + i0 + nch) - r0;
  if (ith < t.nth - 1) dt = __ldg(t.rho + i0 + nph * nch) - r0;
  return r0 + dc * fc + dp * fp + dt * ft;
}

// rsrot (rotden.f:218-286): outputs written only for iodevn == -1
__device__ __forceinline__ void rsrot(const Frame &f1, const Frame &f2, const double abc[3], double tauC, int iodevn,
                                      double *rho, double *erot)
{
  double tau = tauC / PIMC_WNO2K;
  double b0 = 1.0 / abc[0], b1 = 1.0 / abc[1], b2 = 1.0 / abc[2];
  double dig[3];
  for (int i = 0; i < 3; i++) {
    double s = 0.0;
    for (int j = 0; j < 3; j++) s = s + f1.m[j * 3 + i] * f2.m[j * 3 + i];
    dig[i] = s;
  }
  double sumaxs = (b0 - b1 - b2) * (1.0 - dig[0]) + (b1 - b2 - b0) * (1.0 - dig[1]) + (b2 - b0 - b1) * (1.0 - dig[2]);
  if (iodevn == -1) {
    *rho = sumaxs;
    double e = sumaxs / (4.0 * tau * tau);
    e = e + 1.5 / tau + 0.25 * (abc[0] + abc[1] + abc[2]);
    *erot = e / PIMC_WNO2K;
  }
}

// rsrot's log-density on the FP32 path, from the float frames: each
// 1 - (column i of m1).(column i of m2) taken as half the squared distance
// of the two unit columns, which keeps its precision for nearby frames
// (adjacent rotational slices) where 1 - dot in float does not
__device__ __forceinline__ float rsrot32(const float *m1, const float *m2, const float coef[3])
{
  float sumaxs = 0.0f;
#pragma unroll
  for (int i = 0; i < 3; i++) {
    float dx = m1[i] - m2[i], dy = m1[3 + i] - m2[3 + i], dz = m1[6 + i] - m2[6 + i];
    sumaxs += coef[i] * (0.5f * (dx * dx + dy * dy + dz * dz));
  }
  return sumaxs;
}

// rsline (rotden.f:356-375)
__device__ __forceinline__ void rsline(double brot, double dprd, double tauC, double *rho, double *erot)
{
  double tau = tauC / PIMC_WNO2K;
  double r = (1.0 - dprd) / (2.0 * brot * tau);
  double e = (1.0 - r) / tau;
  *rho = -r;
  *erot = e / PIMC_WNO2K;
}

__device__ __forceinline__ double dot3(const double *a, const double *b)
{
  double d = 0.0;
  d = d + a[0] * b[0];
  d = d + a[1] * b[1];
  d = d + a[2] * b[2];
  return d;
}

// vcord (vcord.f:1-98) + vcalc (vcalc.f:1-65) for an atom at rpt around a
// rotor at rcom with body frame f; optional (r, theta, chi) returns
__device__ __forceinline__ double vcord(const DevTables &t, const Frame &f, double rcx, double rcy, double rcz,
                                       double rpx, double rpy, double rpz, double *rr = nullptr,
                                       double *th = nullptr, double *chr = nullptr)
{
  const double pi = PIMC_PI, small = 1.e-08, bo2ang = 0.529177249;
  double R[3] = {rpx - rcx, rpy - rcy, rpz - rcz};
  double hx[3] = {f.m[0], f.m[3], f.m[6]};
  double hy[3] = {f.m[1], f.m[4], f.m[7]};
  double hz[3] = {f.m[2], f.m[5], f.m[8]};
  double rn = sqrt(dot3(R, R));
  double da = dot3(hz, R) / (f.hz_norm * rn);
  if (da > 1.0) da = 1.0;
  if (da < -1.0) da = -1.0;
  double thewff = acos(da);
  double rdotx = dot3(R, hx), rdoty = dot3(R, hy);
  double chiwff;
  if (fabs(rdotx) < small) chiwff = pi / 2.0;
  else chiwff = atan(fabs(rdoty / rdotx));
  double chir;
  if (rdotx >= 0.0 && rdoty >= 0.0) chir = chiwff;
  else if (rdotx < 0.0 && rdoty >= 0.0) chir = pi - chiwff;
  else if (rdotx < 0.0 && rdoty < 0.0) chir = pi + chiwff;
  else chir = 2 * pi - chiwff;
  if (t.chfold == 180) {
    chiwff = chir;
    if (chir > pi) chiwff = 2 * pi - chir;
  } else if (t.chfold == 360) {
    chiwff = chir;
  }
  if (rr) { *rr = rn; *th = thewff; *chr = chir; }
  double r = rn * (1.0 / bo2ang);
  // grid coordinates, their cells and offsets in the cells (one conversion
  // each, reused below unless an index is clamped)
  double xth = thewff * t.d_thscale;           // (theta * 180 / pi) / dth
  double xch = chiwff * t.d_chscale;
  int ith = (int)xth, ich = (int)xch;
  double fth = xth - (double)ith, fch = xch - (double)ich;
  if (near_node(fth)) {                                              // vcord.f:90-91
    xth = ((thewff * 180.0) / pi) / t.dth3;
    ith = (int)xth;
    fth = xth - (double)ith;
  }
  if (near_node(fch)) {
    xch = ((chiwff * 180.0) / pi) / t.dch3;
    ich = (int)xch;
    fch = xch - (double)ich;
  }
  // vcalc
  int maxrpt = t.rgrd - 1, mxthpt = t.thgrd - 1, mxchpt = t.chgrd - 1;
  if (r < t.rvmin) r = t.rvmin;
  if (r > t.rvmax) r = t.rvmax;
  double xr = (r - t.rvmin) * t.d_irstep;
  int ir = (int)xr;
  if (near_node(xr - (double)ir)) {                                  // vcord.f:88, vcalc.f:21
    r = rn / bo2ang;
    if (r < t.rvmin) r = t.rvmin;
    if (r > t.rvmax) r = t.rvmax;
    xr = (r - t.rvmin) / t.rvstep;
    ir = (int)xr;
  }
  if (ir > maxrpt) ir = maxrpt;
  const int ith0 = ith, ich0 = ich;
  if (ich > mxchpt) ich = mxchpt;
  if (ich < 0) ich = 0;
  if (ith > mxthpt) ith = mxthpt;
  if (ith < 0) ith = 0;
  size_t nth = t.thgrd, nch = t.chgrd;
  size_t i0 = ((size_t)ir * nth + ith) * nch + ich;
  double v0 = __ldg(t.vtab + i0);
  double gradr = 0.0, delr = 0.0, gradth = 0.0, delth = 0.0, gradch = 0.0, delch = 0.0;
  if (ir < maxrpt) {
    gradr = (__ldg(t.vtab + i0 + nth * nch) - v0) * t.d_irstep;
    delr = r - (t.rvmin + ir * t.rvstep);
  }
  if (ith < mxthpt) {
    gradth = (__ldg(t.vtab + i0 + nch) - v0);
    delth = (ith == ith0) ? fth : xth - (double)ith;
  }
  if (ich < mxchpt) {
    gradch = (__ldg(t.vtab + i0 + 1) - v0);
    delch = (ich == ich0) ? fch : xch - (double)ich;
  }
  return v0 + gradr * delr + gradth * delth + gradch * delch;
}

// ---------------------------------------------------------- FP32 table path
// The FP32 forms follow the same grids and interpolation as the FP64 leaves;
// angles are taken from atan2 of a cross and a dot product, which is the same
// angle as the reference's acos/atan but keeps full float precision near 0
// and pi.

__device__ __forceinline__ float splint32(const float *__restrict__ xa, const float *__restrict__ ya,
                                          const float *__restrict__ y2a, int n, float x, int uni, float x0, float ih)
{
  int klo;
  if (uni && x == x) {
    float g = (x - x0) * ih;
    int k = g < 0.0f ? 0 : (g > (float)(n - 2) ? n - 2 : (int)g);
    while (k < n - 2 && __ldg(xa + k + 1) <= x) k++;
    while (k > 0 && __ldg(xa + k) > x) k--;
    klo = k;
  } else {
    klo = 0;
    int khi = n - 1;
    while (khi - klo > 1) {
      int k = (khi + klo) >> 1;
      if (__ldg(xa + k) > x) khi = k;
      else klo = k;
    }
  }
  int khi = klo + 1;
  float xk = __ldg(xa + khi), xl = __ldg(xa + klo);
  float h = xk - xl;
  float a = (xk - x) / h, b = (x - xl) / h;
  return a * __ldg(ya + klo) + b * __ldg(ya + khi) +
         ((a * a * a - a) * __ldg(y2a + klo) + (b * b * b - b) * __ldg(y2a + khi)) * (h * h) * (1.0f / 6.0f);
}

__device__ __forceinline__ float spot1d32(const DevTables &t, float r)
{
  if (r >= __ldg(t.g1d32 + t.n1d - 1)) {
    float r2 = r * r;
    return -t.f_c61d / (r2 * r2 * r2);
  }
  if (r <= __ldg(t.g1d32)) return t.f_unode1d * expf(-t.f_alpha1d * r);
  if (t.sp1d4) {
    // uniform grid: the interval from the index formula, its four spline
    // words in one load, the node positions from the grid formula
    float g = (r - t.f_x01d) * t.f_ih1d;
    int k = min(max((int)g, 0), t.n1d - 2);
    float4 w = __ldg(t.sp1d4 + k);
    float b = g - (float)k, a = 1.0f - b;
    return a * w.x + b * w.z + ((a * a * a - a) * w.y + (b * b * b - b) * w.w) * t.f_h2_6;
  }
  return splint32(t.g1d32, t.p1d32, t.y21d32, t.n1d, r, t.uni1d, t.f_x01d, t.f_ih1d);
}

__device__ __forceinline__ float lpot2d32(const DevTables &t, float r, float cost)
{
  // LPot2D's cell from its index formula on the uniform grid, the four
  // corners in one load
  float gr = (r - t.f_rmin2d) / t.f_dr2d, gc = (cost - t.f_cmin2d) / t.f_dc2d;
  int ir = min(max((int)floorf(gr), 0), t.nr2d - 2);
  int ic = min(max((int)floorf(gc), 0), t.nc2d - 2);
  float4 y = __ldg(t.pot2d4 + (size_t)ir * (t.nc2d - 1) + ic);
  float dr = gr - (float)ir, dc = gc - (float)ic;
  return (1.0f - dr) * (1.0f - dc) * y.x + dr * (1.0f - dc) * y.y + dr * dc * y.z + (1.0f - dr) * dc * y.w;
}

// vcord + vcalc in float: R = atom - rotor centre in the space frame
__device__ __forceinline__ float vcord32(const DevTables &t, const Frame &f, float Rx, float Ry, float Rz)
{
  const float pi = 3.14159265358979f;
  const float *m = f.mf;
  float rdotx = m[0] * Rx + m[3] * Ry + m[6] * Rz;
  float rdoty = m[1] * Rx + m[4] * Ry + m[7] * Rz;
  float rdotz = m[2] * Rx + m[5] * Ry + m[8] * Rz;
  float rn2 = Rx * Rx + Ry * Ry + Rz * Rz;
  float rn = rn2 * rsqrtf(rn2);       // a partner on the centre gives NaN, which the clamp below sends to rvmin
  const float rho2 = rdotx * rdotx + rdoty * rdoty;
  float thewff = atan2f(rho2 > 0.0f ? rho2 * rsqrtf(rho2) : 0.0f, rdotz);
  float chiwff = atan2f(fabsf(rdoty), fabsf(rdotx));
  float chir;
  if (rdotx >= 0.0f && rdoty >= 0.0f) chir = chiwff;
  else if (rdotx < 0.0f && rdoty >= 0.0f) chir = pi - chiwff;
  else if (rdotx < 0.0f && rdoty < 0.0f) chir = pi + chiwff;
  else chir = 2.0f * pi - chiwff;
  if (t.chfold == 180) chiwff = (chir > pi) ? 2.0f * pi - chir : chir;
  else if (t.chfold == 360) chiwff = chir;
  float r = rn * 1.88972614f;          // 1 / 0.529177249 (bohr per angstrom)
  float xth = thewff * t.f_thscale;
  float xch = chiwff * t.f_chscale;
  float rvmin = t.f_rvmin, rvmax = t.f_rvmax;
  r = fminf(fmaxf(r, rvmin), rvmax);
  int maxrpt = t.rgrd - 1, mxthpt = t.thgrd - 1, mxchpt = t.chgrd - 1;
  float gr = (r - rvmin) * t.f_irstep;
  int ir = min((int)gr, maxrpt);
  int ith = min(max((int)xth, 0), mxthpt), ich = min(max((int)xch, 0), mxchpt);
  size_t nth = t.thgrd, nch = t.chgrd;
  // value and the one-sided differences of vcalc (zero at the last node)
  float4 w = __ldg(t.vtab4 + ((size_t)ir * nth + ith) * nch + ich);
  return w.x + w.y * (gr - (float)ir) + w.z * (xth - (float)ith) + w.w * (xch - (float)ich);
}

// rotden's rho on the FP32 path: relative rotation m1^T m2 as deleul
// (rotden.f:32-134) with its Euler angles from atan2 (stable where acos of
// a rounded cosine is not), then rotpro's first-order interpolation
// (rotpro_sub.f:1-64) on the float table
__device__ __forceinline__ float rotden_rho32(const DevTables &t, const float *m1, const float *m2in, int *bad)
{
  const float pi2 = 6.28318530717959f;
  float m2[9];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) m2[i * 3 + j] = m1[i] * m2in[j] + m1[3 + i] * m2in[3 + j] + m1[6 + i] * m2in[6 + j];
  float s2 = m2[6] * m2[6] + m2[7] * m2[7];
  float theta = atan2f(sqrtf(s2), m2[8]);
  float phi, chi;
  if (s2 < 2.0e-8f) {                 // |1 -+ cos theta| < 1e-8: phi = 0 (rotden.f:73-86)
    phi = 0.0f;
    chi = (m2[8] > 0.0f) ? atan2f(m2[3], m2[0]) : atan2f(m2[1], m2[4]);
  } else {
    phi = atan2f(m2[5], m2[2]);
    chi = atan2f(m2[7], -m2[6]);
  }
  if (phi < 0.0f) phi += pi2;
  if (chi < 0.0f) chi += pi2;
  float xt = theta * t.f_dscale[0], xp = phi * t.f_dscale[1], xc = chi * t.f_dscale[2];
  int ichi = (int)xc, iphi = (int)xp, ith = (int)xt;
  if (ichi > t.nch - 1 || ichi < 0) { ichi = 0; *bad = 1; }
  if (iphi > t.nph - 1 || iphi < 0) { iphi = 0; *bad = 1; }
  if (ith > t.nth - 1 || ith < 0) { ith = 0; *bad = 1; }
  size_t nph = t.nph, nch = t.nch;
  float4 w = __ldg(t.rho4 + ((size_t)ith * nph + iphi) * nch + ichi);
  return w.x + w.y * (xc - (float)ichi) + w.z * (xp - (float)iphi) + w.w * (xt - (float)ith);
}

// caleng (caleng_tip4p_gg.f:2-186).  kcal2k is an INTEGER parameter in the
// Fortran source (implicit typing), so the LJ term is scaled by 503.
__device__ __forceinline__ double caleng(const Frame &f1, const Frame &f2, double c1x, double c1y, double c1z,
                                         double c2x, double c2y, double c2z)
{
  const double qm = -1.04, qh = 0.520, br2ang = 0.52917721092, hr2k = 3.1577465e5, kcal2k = 503.0;
  const double site[4][3] = {{0.0, 0.0, 0.06562}, {0.0, 0.0, -0.08438}, {0.7557, 0.0, -0.5223}, {-0.7557, 0.0, -0.5223}};
  double a[4][3], b[4][3];   // O, M, H1, H2 in the space frame
  const double c1[3] = {c1x, c1y, c1z}, c2[3] = {c2x, c2y, c2z};
  for (int s = 0; s < 4; s++)
    for (int i = 0; i < 3; i++) {
      double u = c1[i], v = c2[i];
      for (int j = 0; j < 3; j++) {
        u = u + f1.m[i * 3 + j] * site[s][j];
        v = v + f2.m[i * 3 + j] * site[s][j];
      }
      a[s][i] = u;
      b[s][i] = v;
    }
  double roo = 0.0, rmm = 0.0;
  for (int i = 0; i < 3; i++) {
    roo = roo + (a[0][i] - b[0][i]) * (a[0][i] - b[0][i]);
    rmm = rmm + (a[1][i] - b[1][i]) * (a[1][i] - b[1][i]);
  }
  rmm = sqrt(rmm);
  double roo4 = roo * roo, roo6 = roo4 * roo, roo12 = roo6 * roo6;
  double vlj = 6.e5 / roo12 - 610.0 / roo6;
  auto d = [](const double *p, const double *q) {
    double s = 0.0;
    for (int i = 0; i < 3; i++) s = s + (p[i] - q[i]) * (p[i] - q[i]);
    return sqrt(s);
  };
  double vmh = qm * qh * (1.0 / d(a[1], b[2]) + 1.0 / d(a[1], b[3]) + 1.0 / d(b[1], a[2]) + 1.0 / d(b[1], a[3]));
  double vhh = qh * qh * (1.0 / d(a[2], b[2]) + 1.0 / d(a[2], b[3]) + 1.0 / d(a[3], b[2]) + 1.0 / d(a[3], b[3]));
  double vmm = qm * qm * (1.0 / rmm);
  return vlj * kcal2k + (vmh + vmm + vhh) * hr2k * br2ang;
}

// caleng on the FP32 path: the same sites, charges and terms as caleng
// above, from the float frames and float centres, summed in float (the
// Coulomb terms of the four sites cancel to about 1/50 of their size, so
// the result keeps about six digits)
__device__ __forceinline__ float caleng32(const float *ma, const float *mb, float c1x, float c1y, float c1z, float c2x,
                                          float c2y, float c2z)
{
  const float qm = -1.04f, qh = 0.520f, kcal2k = 503.0f;
  const float coul = (float)(3.1577465e5 * 0.52917721092);
  const float site[4][3] = {{0.0f, 0.0f, 0.06562f}, {0.0f, 0.0f, -0.08438f}, {0.7557f, 0.0f, -0.5223f},
                            {-0.7557f, 0.0f, -0.5223f}};
  float a[4][3], b[4][3];
  const float c1[3] = {c1x, c1y, c1z}, c2[3] = {c2x, c2y, c2z};
#pragma unroll
  for (int s = 0; s < 4; s++)
#pragma unroll
    for (int i = 0; i < 3; i++) {
      float u = c1[i], v = c2[i];
#pragma unroll
      for (int j = 0; j < 3; j++) {
        u = fmaf(ma[i * 3 + j], site[s][j], u);
        v = fmaf(mb[i * 3 + j], site[s][j], v);
      }
      a[s][i] = u;
      b[s][i] = v;
    }
  auto d2 = [](const float *p, const float *q) {
    float x = p[0] - q[0], y = p[1] - q[1], z = p[2] - q[2];
    return x * x + y * y + z * z;
  };
  // the FP32 path's reciprocal distances and powers from the hardware
  // reciprocal square root and reciprocal (within a few ulp of float, far
  // inside the path's 1e-5 tolerance)
  const float roo = d2(a[0], b[0]);
  const float iroo = __frcp_rn(roo);
  const float iroo6 = iroo * iroo * iroo;
  const float vlj = 6.e5f * iroo6 * iroo6 - 610.0f * iroo6;
  auto inv = [&](const float *p, const float *q) { return rsqrtf(d2(p, q)); };
  const float vmh = qm * qh * (inv(a[1], b[2]) + inv(a[1], b[3]) + inv(b[1], a[2]) + inv(b[1], a[3]));
  const float vhh = qh * qh * (inv(a[2], b[2]) + inv(a[2], b[3]) + inv(a[3], b[2]) + inv(a[3], b[3]));
  const float vmm = qm * qm * inv(a[1], b[1]);
  return vlj * kcal2k + (vmh + vmm + vhh) * coul;
}

// vspher (vspher.f:12-544) on the supplied table
__device__ __forceinline__ double vspher(const DevTables &t, double r)
{
  const double ang2bo = (double)0.5291772f;
  int maxrpt = t.nsph - 1;
  r = r / ang2bo;
  if (r < t.sph_r0) r = t.sph_r0;
  if (r > t.sph_rmax) r = t.sph_rmax;
  int ir = (int)((r - t.sph_r0) / t.sph_rstep);
  if (ir > maxrpt) ir = maxrpt;
  double v0 = __ldg(t.sph + ir);
  if (ir >= maxrpt) return v0;
  return v0 + (__ldg(t.sph + ir + 1) - v0) / t.sph_rstep * (r - (t.sph_r0 + ir * t.sph_rstep));
}

// ---------------------------------------------------------- Philox 4x32-10
// Counter-based generator of Salmon et al., "Parallel random numbers: as
// easy as 1, 2, 3" (SC'11): ten rounds of two 32x32->64 multiplies with the
// published multipliers and Weyl key increments.
struct U4 { uint32_t x, y, z, w; };

__device__ __forceinline__ U4 philox4x32(U4 c, uint32_t k0, uint32_t k1)
{
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int i = 0; i < 10; i++) {
    uint32_t hi0 = __umulhi(M0, c.x), lo0 = M0 * c.x;
    uint32_t hi1 = __umulhi(M1, c.z), lo1 = M1 * c.z;
    U4 n = {hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
    c = n;
    k0 += W0;
    k1 += W1;
  }
  return c;
}

// two uniforms in (0,1) with 32-bit resolution from one Philox block, in
// float (the FP32 path: no double conversion)
__device__ __forceinline__ void philox_u2f(uint64_t seed, uint64_t a, uint32_t b, uint32_t c, float *u0, float *u1)
{
  U4 ctr = {(uint32_t)a, (uint32_t)(a >> 32), b, c};
  U4 r = philox4x32(ctr, (uint32_t)seed, (uint32_t)(seed >> 32));
  *u0 = ((float)r.x + 0.5f) * 2.3283064365386963e-10f;
  *u1 = ((float)r.z + 0.5f) * 2.3283064365386963e-10f;
}

// two uniforms in (0,1) with 53-bit resolution from one Philox block
__device__ __forceinline__ void philox_u2(uint64_t seed, uint64_t a, uint32_t b, uint32_t c, double *u0, double *u1)
{
  U4 ctr = {(uint32_t)a, (uint32_t)(a >> 32), b, c};
  U4 r = philox4x32(ctr, (uint32_t)seed, (uint32_t)(seed >> 32));
  uint64_t v0 = ((uint64_t)r.x << 21) ^ (uint64_t)r.y;
  uint64_t v1 = ((uint64_t)r.z << 21) ^ (uint64_t)r.w;
  *u0 = ((double)(v0 & ((1ull << 53) - 1)) + 0.5) * (1.0 / 9007199254740992.0);
  *u1 = ((double)(v1 & ((1ull << 53) - 1)) + 0.5) * (1.0 / 9007199254740992.0);
}
