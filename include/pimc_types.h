/*
 * pimc_types.h -- plain-C description of a MoRiBS-PIMC system, its tables and
 * its path-integral state.  Shared by the GB300 library (pimc_gb300.h) and by
 * the CPU oracle used in the tests; no CUDA or torch types appear here.
 *
 * Units follow the reference after MCSetUnits (mc_setup.cc:194-217): Kelvin,
 * Angstrom, amu.  Layouts follow the reference globals:
 *   coords/cosine/angles are row-major [3][natoms*nslices] with the bead of
 *   global atom a at imaginary-time slice t stored at a*nslices + t
 *   (MCCoords/MCCosine/MCAngles, mc_setup.h:176-178, mc_setup.cc:139-148);
 *   angles rows are {phi, cos(theta), chi} (PHI=0, CTH=1, CHI=2,
 *   mc_confg.h:53-55) and only the first nrotslices entries of a rotor's
 *   block are used (mc_piqmc.cc:790-792).
 */
#ifndef PIMC_TYPES_H
#define PIMC_TYPES_H

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes returned by every entry point.  They replace the reference's
 * exit() paths: nrerror (mc_utils.cc:99-108), _io_error (mc_input.h:35-42),
 * rotden's istop -> exit(0) (mc_piqmc.cc:1025-1029) and the negative linear
 * density check (mc_piqmc.cc:850). */
typedef enum {
  PIMC_OK = 0,
  PIMC_ERR_BAD_ARG = 1,      /* malformed system / pointer / size */
  PIMC_ERR_BAD_TABLE = 2,    /* table missing or inconsistent */
  PIMC_ERR_GRID_RANGE = 3,   /* rotpro index out of range (rotpro_sub.f:10-24) */
  PIMC_ERR_NEG_DENSITY = 4,  /* negative linear rotational density (mc_piqmc.cc:850,886) */
  PIMC_ERR_TIMEOUT = 5,      /* a bounded device wait gave up */
  PIMC_ERR_CUDA = 6,         /* CUDA runtime error */
  PIMC_ERR_NO_DEVICE = 7,    /* no CUDA device */
  PIMC_ERR_SIZE = 8,         /* size beyond a compiled limit */
  PIMC_ERR_STATE = 9         /* call out of order (e.g. no tables loaded) */
} pimc_status;

/* MCAtom[].molecule (mc_setup.h:78) */
enum { PIMC_ATOM = 0, PIMC_LINEAR = 1, PIMC_NONLINEAR = 2 };
/* MCAtom[].stat (mc_confg.h:13-15) */
enum { PIMC_BOLTZMANN = 0, PIMC_BOSE = 1 };
/* RotDenType (mc_setup.cc:55) */
enum { PIMC_ROTDEN_TABLE = 0, PIMC_ROTDEN_RS = 1 };

#define PIMC_MAX_TYPES 2

/* Density histogram grids of densities_init (mc_estim.cc:25-30, 223-255):
 * radial bins of (MAX-MIN)/BINSR Angstrom from MIN_RADIUS, theta bins of
 * pi/(BINST-1), chi bins of 2 pi/(BINSC-1). */
#define PIMC_BINSR 300
#define PIMC_BINST 50
#define PIMC_BINSC 100
#define PIMC_DENS_MIN_RADIUS 0.0
#define PIMC_DENS_MAX_RADIUS 15.0

/* One particle type: the fields of TParticle (mc_setup.h:66-91) that the
 * sampling path reads.  lambda is hbar^2/2m in K*A^2 (mc_setup.cc:207-215). */
typedef struct {
  int    numb;      /* number of particles of this type           */
  int    molecule;  /* PIMC_ATOM / PIMC_LINEAR / PIMC_NONLINEAR    */
  int    stat;      /* PIMC_BOLTZMANN / PIMC_BOSE                  */
  int    levels;    /* bisection levels, segment = 2^levels        */
  double mcstep;    /* centroid (whole-path) displacement step, A  */
  double lambda;    /* hbar^2/(2m), K*A^2                          */
} pimc_type;

/* The run parameters of qmc.input that the sampling path reads
 * (mc_input.cc:114-343) plus the derived ones of MCInit (mc_setup.cc:321-453).
 * Atom types come first, then at most one molecule type
 * (mc_input.cc:194, 395-396). */
typedef struct {
  int       ntypes;        /* 1 or 2                                    */
  pimc_type type[PIMC_MAX_TYPES];
  int       nslices;       /* P  = NUMBEROFSLICES                       */
  int       nrotslices;    /* Q  = ROTATION ... <Q>; 0 without rotation */
  int       rotation;      /* ROTATION keyword present                  */
  double    temperature;   /* K                                         */
  double    rtstep;        /* rotational MC step                        */
  int       ispher;        /* spherical rotor treatment (mc_input.cc:152-156) */
  int       rot_den_type;  /* ROTDENSI [1]: 0 tables, 1 rattle-and-shake */
  int       rot_odevn;     /* ROTDENSI [2]                              */
  double    rot_eoff;      /* ROTDENSI [3], cm^-1                       */
  double    rot_abc[3];    /* ROTDENSI [4..6]: X_Rot,Y_Rot,Z_Rot, cm^-1 */
  int       rn_ratio;      /* ROTDENSI [7]                              */
  int       minimage;      /* MINIMAGE                                  */
  double    box[3];        /* BoxSize (used with minimage)              */
} pimc_system;

/* Interaction and propagator tables.  Pointers are borrowed for the
 * duration of the load call only.
 *  - 1D atom-atom potential, SPot1D (mc_poten.cc:379-438,624-639): n1d
 *    points (grid1d[i], pot1d[i]); the cubic spline and the short/long range
 *    extrapolation constants are derived from them exactly as init_pot1D does.
 *  - 2D linear-rotor--atom potential, LPot2D (mc_poten.cc:305-377,688-729):
 *    pot2d[ir*nc2d+ic] on grids rgrid2d[nr2d], cgrid2d[nc2d], steps dr2d,dc2d.
 *  - 3D nonlinear-rotor--atom potential, vcord/vcalc (vcord.f:1-98,
 *    vcalc.f:1-65): vtable[(ir*thgrd+ith)*chgrd+ich], r in bohr on
 *    [rvmin,rvmax].  theta covers 0..180 deg in thgrd points; chi covers
 *    0..chi_fold_deg deg in chgrd points.  chi_fold_deg = 0 means "as the
 *    reference": 91->90, 181->180, 361->360 (vcord.f:78-85).  With thgrd=181
 *    and chgrd in {91,181,361} the lookup is the reference's 1-degree one.
 *  - linear rotor density .rot file, SRotDens (mc_poten.cc:508-622): nrot
 *    rows of (cos gamma, rho, E-derivative, E^2).
 *  - nonlinear rotor density .rho/.eng/.esq, rotden/rotpro (rotden.f:1-31,
 *    rotpro_sub.f:1-64): [(ith*nph+iph)*nch+ich] on theta 0..180, phi 0..360,
 *    chi 0..360 deg.  nth=181,nph=361,nch=361 is the reference's grid.
 *  - spherical rotor--atom table for ISPHER=1, vspher (vspher.f:12-544):
 *    nsph points from sph_r0 (bohr) with step sph_rstep, clamped at sph_rmax. */
typedef struct {
  int           n1d;
  const double *grid1d, *pot1d;

  int           nr2d, nc2d;
  double        dr2d, dc2d;
  const double *rgrid2d, *cgrid2d, *pot2d;

  int           rgrd, thgrd, chgrd, chi_fold_deg;
  double        rvmin, rvmax;
  const double *vtable;

  int           nrot;
  const double *rotgrid, *rotdens, *rotderv, *rotesqr;

  int           nth, nph, nch;
  const double *rhoprp, *erotpr, *erotsq;

  int           nsph;
  double        sph_r0, sph_rmax, sph_rstep;
  const double *sph_table;
} pimc_tables;

#ifdef __cplusplus
}
#endif
#endif /* PIMC_TYPES_H */
