/*
 * pimc_oracle.h -- CPU oracle for the MoRiBS-PIMC sampling path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference's
 * move, energy and estimator routines (mc_piqmc.cc, mc_poten.cc, mc_utils.cc,
 * mc_estim.cc) and of its Fortran leaves (rotden.f, rotpro_sub.f, vcord.f,
 * vcalc.f, caleng_tip4p_gg.f, vspher.f), used as the checker by the tests,
 * by __graft_entry__.smoke() and by bench.py's CPU-baseline leg.  The GB300
 * library never links, loads or calls it.
 *
 * Parity pinning: the C++ parts are pinned against the reference compiled
 * from its own sources (oracle/ref_build.sh -> oracle/_ref) and against the
 * committed fixtures in tests/golden.  The Fortran leaves cannot be compiled
 * here (no Fortran compiler); they are pinned by known-answer tests derived
 * from the formulas in the .f files (tests/test_oracle_leaves.py).
 *
 * State layout is the reference's: coords/angles/cosine are [3][natoms*P].
 * Random numbers come from an orc_rng: either replay streams (one per
 * reference generator: rnd1, rnd2, rnd3, gauss, runif) consumed exactly in
 * the order the reference consumes them, or an internal counter-based
 * generator for the timed CPU baseline.
 */
#ifndef PIMC_ORACLE_H
#define PIMC_ORACLE_H

#include <stdint.h>
#include "../include/pimc_types.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_ctx orc_ctx;

/* replay stream: v[pos++]; running past n sets the overrun flag */
typedef struct {
  const double *v;
  long n;
  long pos;
} orc_stream;

typedef struct {
  orc_stream u1;     /* rnd1(): centroid displacement (mc_randg.cc:96-100)      */
  orc_stream u2;     /* rnd2(): centroid accept (mc_piqmc.cc:86)                */
  orc_stream u3;     /* rnd3(): bisection level accept (mc_piqmc.cc:271)        */
  orc_stream gauss;  /* x1 = sqrt(-log r1) cos(2 pi r2) of gauss() (mc_randg.cc:138-150) */
  orc_stream urot;   /* runif(): rotational proposals/accepts (omprng.cc:34-38) */
  int overrun;
} orc_replay;

/* worm-move replay streams: nrnd1..nrnd3 (mc_randg.cc:159-171), rnd1..rnd5
 * and the x1 values of gauss(), each consumed where mc_qworm.cc draws it */
typedef struct {
  orc_stream n1, n2, n3, u1, u2, u3, u4, u5, gauss;
  int overrun;
} orc_wreplay;

/* life cycle */
orc_ctx *orc_create(const pimc_system *sys, const pimc_tables *tab, int *status);
void     orc_destroy(orc_ctx *c);
int      orc_set_state(orc_ctx *c, const double *coords, const double *angles, const int *pindex);
int      orc_get_state(const orc_ctx *c, double *coords, double *angles, double *cosine, int *pindex);
int      orc_natoms(const orc_ctx *c);

/* table leaves */
double orc_spot1d(const orc_ctx *c, double r);
double orc_lpot2d(const orc_ctx *c, double r, double cost);
double orc_srotdens(const orc_ctx *c, double gamma, int which); /* 0 rho, 1 deriv, 2 esq */
void   orc_matpre(const double eul[3], double m[9]);            /* m[i*3+j] = rotmat(i+1,j+1) */
void   orc_deleul(const double e1[3], const double e2[3], double rel[3]);
int    orc_rotden(const orc_ctx *c, const double e1[3], const double e2[3], double rel[3],
                  double *rho, double *erot, double *esq);
double orc_vcord(const orc_ctx *c, const double eul[3], const double rcom[3], const double rpt[3],
                 double *radret, double *theret, double *chiret);
void   orc_rsrot(const double e1[3], const double e2[3], double xrot, double yrot, double zrot,
                 double tauC, int iodevn, double eoff, double *rho, double *erot);
void   orc_rsline(double brot, double dprd, double tauC, double *rho, double *erot);
double orc_caleng(const double com1[3], const double com2[3], const double e1[3], const double e2[3]);
double orc_vspher(const orc_ctx *c, double r);

/* raw-argument forms of the table leaves (explicit grids), used to bind the
 * reference's Fortran symbols when the reference is compiled here */
int    orc_rotpro_raw(double chi, double phi, double theta, const double *rhoprp, const double *erotpr,
                      const double *erotsq, int nth, int nph, int nch, double *rho, double *erot, double *esq);
double orc_vcord_raw(const double eul[3], const double rcom[3], const double rpt[3], const double *vtab,
                     int nrgrd, int nthgrd, int nchgrd, int chfold, double rvmax, double rvmin, double rvstep,
                     double *radret, double *theret, double *chiret);
double orc_vspher_raw(double r, const double *tab, int n, double r0, double rmax, double rstep);

/* energies; pos is a [3][natoms*P] array like coords */
double orc_pot_energy_slice(const orc_ctx *c, int atom0, const double *pos, int it);
double orc_pot_energy_path(const orc_ctx *c, int atom0, const double *pos);
double orc_pot_rot_energy(const orc_ctx *c, int atom0, const double *cosine, int it);
double orc_pot_rot_e3d(const orc_ctx *c, int atom0, const double eul[3], int it);

/* moves with replayed randoms (per-move records are optional, may be NULL) */
int orc_molecular_move(orc_ctx *c, int type, orc_replay *rp, double *dv_out, int *acc_out);
int orc_molecular_move_exchange(orc_ctx *c, int type, orc_replay *rp, double *dv_out, int *acc_out);
/* ds_out[atom*levels + level] = level action difference; lvl_out[atom] = levels passed */
int orc_bisection_move(orc_ctx *c, int type, int time, orc_replay *rp, double *ds_out, int *lvl_out);
int orc_bisection_move_exchange(orc_ctx *c, int type, int time0, orc_replay *rp, double *ds_out, int *lvl_out);
/* one full even/odd sweep; rd_out[slice*nrot+rotor] acceptance ratio, acc_out same index */
int orc_rotations_move(orc_ctx *c, int type, orc_replay *rp, double *rd_out, int *acc_out);
int orc_rotations_3d(orc_ctx *c, int type, orc_replay *rp, double *rd_out, int *acc_out);
/* single slice steps with explicit uniforms (MCRotLinStep / MCRot3Dstep) */
int orc_rot_lin_step(orc_ctx *c, int it1, int rotor, const double u[3], double *rd, int *acc);
int orc_rot_3d_step(orc_ctx *c, int it1, int rotor, const double u[4], double *rd, int *acc);

/* counters MCTotal/MCAccep (mc_piqmc.h:25-26): [type*3 + kind] */
void orc_get_counters(const orc_ctx *c, double *total, double *accep);
void orc_reset_counters(orc_ctx *c);

/* estimators (one MCGetAverage sample) */
double orc_kin_energy(const orc_ctx *c);
double orc_pot_energy_est(const orc_ctx *c);
double orc_rot_energy(const orc_ctx *c, double *erotsq, double *erot_termsq);
double orc_rot_e3d(const orc_ctx *c, double *erotsq, double *erot_termsq);
void   orc_rcf(const orc_ctx *c, double *rcf);   /* adds this sample's <n(t0).n(t0+dt)> sums into rcf[Q] */
/* GetPotEnergy_Densities with its histograms: counts are added to
 * gr1d[type][BINSR], gr2d[type][BINSR][BINST], gr3d[type][BINSR*BINST*BINSC]
 * (any may be NULL), indexed by the density type as the reference's are */
double orc_pot_energy_densities(const orc_ctx *c, double *gr1d, double *gr2d, double *gr3d);
void   orc_exchange_lengths(const orc_ctx *c, double *ploops);           /* ploops[numb of the boson type] += */
int    orc_area_estimators(const orc_ctx *c, double *out);               /* out[6]  */
int    orc_area_estim3d(const orc_ctx *c, int iframe, const double *mass, double *out);   /* out[18] */

/* worm algorithm (mc_qworm.cc): MCWormInit with the WORM line's c and m and
 * the input density; one MCWormMove call; the worm state {exists, ira,
 * masha, atom_i, atom_m} and the QWTotal/QWAccep counters [QWMAXMOVES=7] */
int  orc_worm_init(orc_ctx *c, int type, double wc, int m, double density);
int  orc_worm_move(orc_ctx *c, orc_wreplay *rp);
void orc_worm_state(const orc_ctx *c, int *st);
void orc_worm_set_state(orc_ctx *c, const int *st);
void orc_worm_counters(const orc_ctx *c, double *total, double *accep);
/* the worm branch of the pass loop for slices [t_begin, t_begin+t_count)
 * with the internal generator (timed CPU baseline) */
int  orc_worm_run(orc_ctx *c, int t_begin, int t_count, uint64_t seed, int nthreads, double *bead_moves);

/* propagator-table generators (orc_tables.c): linear_prop/linden.f and
 * nmv_prop/asymrho.f restated */
int    orc_linden_lmax(double temprt, int nslice, double bconst, double *tau_out);
int    orc_linden(double temprt, int nslice, double bconst, int npt, int iodevn, double *cost, double *rho,
                  double *erot, double *erotsq);
double orc_rotmat(int j, int k, int kp, double A, double B, double C);
double orc_wigd(int j, int m, int k, double theta);
int    orc_asymrho_energies(int maxj, double A, double B, double C, double *eng);
int    orc_asymrho_points(double temprt, int nslice, int iodevn, double A, double B, double C, int maxj, int npts,
                          const int *ith, const int *iphi, const int *ichi, double *rho, double *erot, double *esq,
                          double *info);

/* reference schedule (mc_main.cc:348-381 + PIMCPass mc_main.cc:510-522) for
 * time slices [t_begin, t_begin+t_count), with the internal generator.
 * nthreads > 1 parallelises the even/odd rotational phases and the
 * whole-path energy sums over slices, as the reference's OpenMP loops do.
 * Returns the number of scheduled bead-moves in *bead_moves. */
int orc_run_steps(orc_ctx *c, int t_begin, int t_count, uint64_t seed, int nthreads, double *bead_moves);

#ifdef __cplusplus
}
#endif
#endif
