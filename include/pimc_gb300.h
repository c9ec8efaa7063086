/*
 * pimc_gb300.h -- C ABI of the GB300 (sm_103a) MoRiBS-PIMC sampling path.
 *
 * Plain pointers and sizes only.  A handle owns its device buffers and one
 * CUDA stream; calls on one handle are ordered on that stream and return a
 * pimc_status.  Host buffers passed in are only read or written during the
 * call.  Layouts and units are those of pimc_types.h (the reference's
 * MCCoords / MCAngles / MCCosine arrays, Kelvin and Angstrom).
 *
 * Each entry point names the reference interface it replaces.  The replay
 * entry points run exactly one reference call on the GPU with the random
 * numbers supplied by the caller, consumed in the reference's order
 * (conditional draws included), so that their results can be compared move
 * by move with the reference.  pimc_run_passes is the production sampler.
 */
#ifndef PIMC_GB300_H
#define PIMC_GB300_H

#include <stdint.h>
#include "pimc_types.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct pimc_handle pimc_handle;

/* MCMemAlloc + MCInit (mc_setup.cc:135-163, 321-453): validate the system
 * (segment 2^levels < P, P divisible by Q, <= 1024 particles, one molecule
 * type with at most 16 rotors) and allocate the path on `device`. */
pimc_status pimc_create(const pimc_system *sys, int device, pimc_handle **out);
pimc_status pimc_destroy(pimc_handle *h);

/* InitPotentials / InitRotDensity (mc_poten.cc:93-164, 254-546): upload the
 * tables and derive the spline second derivatives and the 1D extrapolation
 * constants exactly as init_pot1D / init_rotdens do. */
pimc_status pimc_load_tables(pimc_handle *h, const pimc_tables *tab);

/* The path: coords/angles in the reference's [3][natoms*P] layout
 * (MCCoords, MCAngles; mc_main.cc:184-200 derives MCCosine from the
 * angles), pindex = PIndex.  Any pointer may be NULL to keep that part. */
pimc_status pimc_set_state(pimc_handle *h, const double *coords, const double *angles, const int *pindex);
pimc_status pimc_get_state(pimc_handle *h, double *coords, double *angles, double *cosine, int *pindex);

/* ---- replay entry points (one reference call each) ---------------------- */

/* MCMolecularMove(type) (mc_piqmc.cc:54-102): u1 = rnd1() draws (3 per
 * atom), u2 = rnd2() draws (one per atom whose dV >= 0).  consumed[0..1]
 * returns the counts drawn; dv_out[atom], acc_out[atom] per atom. */
pimc_status pimc_molecular_move(pimc_handle *h, int type, const double *u1, long n1, const double *u2, long n2,
                                long *consumed, double *dv_out, int *acc_out);

/* MCMolecularMoveExchange(type) (mc_piqmc.cc:104-192) for the boson type:
 * every exchange cycle of the permutation moved rigidly, u1 = rnd1() draws
 * (3 per cycle), u2 = rnd2() draws (one per tested atom whose dV >= 0). */
pimc_status pimc_molecular_move_exchange(pimc_handle *h, int type, const double *u1, long n1, const double *u2,
                                         long n2, long *consumed);

/* MCBisectionMove(type, time) (mc_piqmc.cc:194-294) and, with exchange = 1,
 * MCBisectionMoveExchange(type, time) (mc_piqmc.cc:296-419): gauss holds the
 * x1 = sqrt(-log r1) cos(2 pi r2) values of gauss() (mc_randg.cc:138-150),
 * three per midpoint in level order; u3 the rnd3() draws.  ds_out[atom*levels
 * + level] = level action difference, lvl_out[atom] = levels accepted. */
pimc_status pimc_bisection_move(pimc_handle *h, int type, int time, int exchange, const double *gauss, long ng,
                                const double *u3, long n3, long *consumed, double *ds_out, int *lvl_out);

/* MCRotationsMove / MCRotations3D (mc_piqmc.cc:421-517, 692-779): one
 * even/odd sweep of all rotational slices; urot = runif() draws, 3 (linear)
 * or 4 (nonlinear) per (slice, rotor) in serial order: even slices, then odd,
 * rotors in order inside a slice.  rd_out/acc_out[slice*nrotors + rotor]. */
pimc_status pimc_rotations_move(pimc_handle *h, const double *urot, long nrot, double *rd_out, int *acc_out);

/* ---- energies ----------------------------------------------------------- */

/* PotEnergy(atom0, pos, it) (mc_piqmc.cc:1796-1965) for n queries: atom0 at
 * xyz[3k..3k+2] against all other atoms' current beads at slice it[k]. */
pimc_status pimc_pot_energy(pimc_handle *h, int n, const int *atom0, const int *it, const double *xyz, double *out);

/* No counterpart in the reference.  pimc_pot_energy for callers that must not
 * have device memory allocated for them after set-up (an application that owns
 * all device memory through its own pool, or runs under a fixed budget): the
 * queries and results are staged in a fixed array inside the library, so the
 * call makes no cudaMalloc/cudaFree.  n <= 4096 (PIMC_ERR_SIZE otherwise).
 * All calls on a device share the array: calls that overlap on the GPU race
 * and must be ordered by the caller.  The first call on each device looks up
 * the array's address; make it before any stream capture.  The address is
 * kept for the life of the process: after a cudaDeviceReset the library's
 * module may load elsewhere, so this entry point must not be used after one. */
pimc_status pimc_pot_energy_noalloc(pimc_handle *h, int n, const int *atom0, const int *it, const double *xyz,
                                    double *out);

/* PotRotE3D(rotor, Eulang, it) (mc_piqmc.cc:2046-2151) with v3 = (phi,
 * theta, chi) for a nonlinear rotor, or PotRotEnergy (mc_piqmc.cc:1967-2044)
 * with v3 = the unit vector for the linear rotor; rotor = global atom index. */
pimc_status pimc_pot_rot_energy(pimc_handle *h, int n, const int *rotor, const int *it, const double *v3, double *out);

/* ---- estimators (one MCGetAverage sample, mc_main.cc:551-616) ---------- */

/* out = {GetKinEnergy, GetPotEnergy_Densities, GetRotEnergy|GetRotE3D,
 *        ErotSQ, Erot_termSQ} (mc_estim.cc:500-1096) */
pimc_status pimc_estimators(pimc_handle *h, double *out);
/* GetRCF row 0 of one sample (mc_estim.cc:1099-1139): rcf[Q] */
pimc_status pimc_rcf(pimc_handle *h, double *rcf);

/* Pair densities of GetPotEnergy_Densities (mc_estim.cc:500-687 with
 * bin_1Ddensity/bin_2Ddensity/bin_3Ddensity :1233-1286).  With
 * PIMC_OPT_DENSITIES = 1 every pimc_estimators call also bins its
 * configuration into histograms kept on the device, as the reference's
 * _gr?D_sum accumulate: atom-atom pairs of one type by r, linear rotor-atom
 * pairs by (r, theta), nonlinear rotor-atom pairs by vcord's (r, theta, chi).
 * pimc_densities_accumulate bins the current configuration alone.
 * pimc_densities_read copies the counts out as doubles:
 * gr1d[PIMC_MAX_TYPES][PIMC_BINSR], gr2d[PIMC_MAX_TYPES][PIMC_BINSR][PIMC_BINST],
 * gr3d[PIMC_MAX_TYPES][PIMC_BINSR*PIMC_BINST*PIMC_BINSC] indexed by the
 * density type (the atom type) like _gr1D/_gr2D/_gr3D; any may be NULL. */
#define PIMC_OPT_DENSITIES 2
pimc_status pimc_densities_accumulate(pimc_handle *h);
pimc_status pimc_densities_read(pimc_handle *h, double *gr1d, double *gr2d, double *gr3d);
pimc_status pimc_densities_reset(pimc_handle *h);
/* With a nonlinear rotor the same binning also counts the relative Euler
 * angles (theta, phi, chi) of rotational slices it0 and it0 + skip, as
 * GetRotE3D fills _relthe_sum, _relphi_sum, _relchi_sum (mc_estim.cc:1023-1057);
 * pimc_rel_euler_read copies the[PIMC_BINST], phi[PIMC_BINSC], chi[PIMC_BINSC]
 * (zeros without a nonlinear rotor); pimc_densities_reset clears them too.
 * The reference keeps these counts for the whole run (_relthe_sum & co. are
 * reset only with the run totals, mc_estim.cc:361-372): a caller that resets
 * the densities per block reads pimc_rel_euler_read before each reset and
 * adds the counts to its own run totals. */
pimc_status pimc_rel_euler_read(pimc_handle *h, double *the, double *phi, double *chi);

/* GetExchangeLength (mc_estim.cc:1997-2019): ploops[k] += 1 for every
 * exchange cycle of k+1 bosons in the current permutation; ploops has one
 * entry per boson. */
pimc_status pimc_exchange_lengths(pimc_handle *h, double *ploops);

/* GetAreaEstimators (mc_estim.cc:2087-2250): the superfluid area estimators
 * of the boson paths about the linear dopant.  out[6] are the increments
 * the reference adds to _areas[PERP,PARL], _area2[PERP,PARL] and
 * _inert[PERP,PARL] (mc_estim.cc:2242-2249). */
pimc_status pimc_area_estimators(pimc_handle *h, double *out);

/* GetAreaEstim3D(iframe) (mc_estim.cc:2252-2594): iframe 0 about the
 * instantaneous centre of mass of all atoms on the space-fixed axes, 1 about
 * the dopant on its body axes.  mass[type] in amu (MCAtom[].mass,
 * mc_setup.cc:244-319).  out[18] = area_proj[3], then the increments of
 * _areas3D (area_proj[i]*area_proj[j], j <= i) and of _inert3D (inert3D/P,
 * row-major 3x3). */
pimc_status pimc_area_estim3d(pimc_handle *h, int iframe, const double *mass, double *out);

/* The estimators' block files (host only, no handle): the reference's
 * writers with the same file names, columns, normalisations and number
 * format (scientific, 6 digits, width 14, three-blank separators), from the
 * arrays the entry points above return, summed over the block by the
 * caller.  fname is the file stem; mode 0 is a block file (MC_BLOCK), 1 the
 * accumulated one ("_sum" before the extension, MC_TOTAL); acount is the
 * number of samples summed.  sys->box must hold the reference's BoxSize
 * (mc_setup.cc:361-366) for the .gra normalisation.  bstype is the boson
 * type (BSTYPE) and mass its mass in amu.
 *  pimc_save_densities_1d   SaveDensities1D (mc_estim.cc:1327-1443): .gra;
 *                           with a linear impurity also .gri and .grt from gr2d
 *  pimc_save_gra_sum        SaveGraSum (mc_estim.cc:1288-1325): _sum.gra
 *  pimc_save_densities_2d   SaveDensities2D (mc_estim.cc:1666-1726): .g2d
 *  pimc_save_densities_3d   SaveDensities3D (mc_estim.cc:1728-1800): .g3d
 *  pimc_save_rho_1d         SaveRho1D's .gri, .grt, .grc (mc_estim.cc:1445-1590)
 *  pimc_save_rho_theta_chi  SaveRhoThetaChi (mc_estim.cc:1930-1996): .gtc
 *  pimc_save_rel_euler      the run-total files of SaveRho1D (mc_estim.cc:1590-1660):
 *                           _sum.eulphi, _sum.eulchi, _sum.eulthe from pimc_rel_euler_read
 *  pimc_save_exchange_length  SaveExchangeLength (mc_estim.cc:2021-2085): .prl, appended
 *  pimc_save_area_estimators  SaveAreaEstimators (mc_estim.cc:2596-2641): .sup, appended;
 *                           sums[6] as pimc_area_estimators' out
 *  pimc_save_area_estim3d   SaveAreaEstim3D (mc_estim.cc:2670-2720): .sffs3d / .mffs3d,
 *                           appended; areas[6], inert[9] as pimc_area_estim3d's out[3..17]
 *  pimc_save_rcf            SaveRCF (mc_estim.cc:1141-1189): .rcf from rcf[10][Q], GetRCF's
 *                           ten rows summed (row 0 = pimc_rcf's output; rows 1..9 count the
 *                           (origin, lag) pairs, in block mode those with n.n < 0.9999999)
 * gr1d/gr2d/gr3d are laid out as pimc_densities_read writes them. */
pimc_status pimc_save_densities_1d(const pimc_system *sys, const char *fname, double acount, const double *gr1d,
                                   const double *gr2d);
pimc_status pimc_save_gra_sum(const pimc_system *sys, const char *fname, double acount, const double *gr1d);
pimc_status pimc_save_densities_2d(const pimc_system *sys, const char *fname, double acount, int mode,
                                   const double *gr2d);
pimc_status pimc_save_densities_3d(const pimc_system *sys, const char *fname, double acount, int mode,
                                   const double *gr3d);
pimc_status pimc_save_rho_1d(const pimc_system *sys, const char *fname, double acount, int mode,
                             const double *gr3d);
pimc_status pimc_save_rho_theta_chi(const pimc_system *sys, const char *fname, double acount, int mode,
                                    const double *gr3d);
pimc_status pimc_save_rel_euler(const pimc_system *sys, const char *fname, double acount, const double *the,
                                const double *phi, const double *chi);
pimc_status pimc_save_exchange_length(const pimc_system *sys, const char *fname, double acount, long blocknumb,
                                      int bstype, const double *ploops, const int *pindex, int print_xyz_prl);
pimc_status pimc_save_area_estimators(const pimc_system *sys, const char *fname, double acount, long blocknumb,
                                      int bstype, const double *sums, double mass);
pimc_status pimc_save_area_estim3d(const pimc_system *sys, const char *fname, double acount, long blocknumb,
                                   int iframe, int bstype, const double *areas, const double *inert, double mass);
pimc_status pimc_save_rcf(const pimc_system *sys, const char *fname, double acount, int mode, const double *rcf);
/* The energy block of MCGetAverage / SaveEnergy (mc_main.cc:551-616, 764-795):
 * pimc_energy_accumulate adds one sample's terms (from pimc_estimators' out[5])
 * to sums[7] = {E_kin, E_pot, E_rot, ErotSQ, Cv, Cv_trans, Cv_rot} block sums;
 * pimc_save_energy appends the block's .eng line (values over acount). */
pimc_status pimc_energy_accumulate(const pimc_system *sys, const double *est, double *sums);
pimc_status pimc_save_energy(const pimc_system *sys, const char *fname, double acount, long blocknumb,
                             const double *sums);
/* SaveSumEnergy (mc_main.cc:797-836): a line of the run's _sum.eng from the
 * run sums of pimc_energy_accumulate (append = 0 starts the file). */
pimc_status pimc_save_sum_energy(const pimc_system *sys, const char *fname, double acount, double numb,
                                 const double *sums, int append);

/* Standard error of the mean of a correlated series (host only, no handle):
 * the reference writes one .eng row of block averages per block
 * (SaveEnergy, mc_main.cc:764-795) and leaves their error analysis to the
 * user; this is that analysis.  Blocking (Flyvbjerg and Petersen 1989) of
 * the last 2^d of the n >= 16 values, the level chosen automatically
 * (Jonsson 2018: the first level whose lag-one autocorrelations pass a
 * chi-squared test at 99 %).  out[8] = mean, sample sd, naive SE, blocked
 * SE, statistical inefficiency g = (blocked / naive SE)^2 (= 2 tau_int in
 * samples), block size chosen, 1 if the test passed at some level (0: the
 * top level is used), values used (2^d). */
pimc_status pimc_blocking_se(const double *x, long n, double *out);

/* The FP64 rate the part sustains on independent fused multiply-adds
 * (GFLOP/s, an FMA counted as two), measured with CUDA events on `device`:
 * the denominator of the FP64 roofline fractions.  No reference counterpart. */
pimc_status pimc_fp64_peak(int device, double *gflops);

/* The FP64 pipe's occupancy rule: one CTA per SM of `warps` warps (1-32),
 * `lanes` active lanes per warp (1-32), each active lane running 8
 * independent FMA chains of `iters` steps (1-2^24); *ms is the launch's
 * device time (CUDA events, after a warm-up launch).  The time per warp
 * instruction per SM follows: ms / (warps * iters * 8).  Measures how the
 * rotational kernels' low-lane-count FP64 stages load the pipe. */
pimc_status pimc_fp64_probe(int device, int warps, int lanes, int iters, double *ms);

/* ---- worm algorithm (mc_qworm.cc) ------------------------------------------ */

/* MCWormInit (mc_qworm.cc:49-82) for the atom type `type` with the WORM
 * line's c and m (mc_input.cc:286-295) and the input DENSITY; m < P and
 * m <= 64.  The worm starts closed. */
pimc_status pimc_worm_init(pimc_handle *h, int type, double c, int m, double density);
/* One MCWormMove call (mc_qworm.cc:93-125): for each atom of the worm type
 * an open or close try, an advance or recede try and, for bosons, a swap
 * try, with the random numbers replayed from nine streams in the order
 * mc_qworm.cc draws them: streams[0..2] the uniforms behind nrnd1, nrnd2,
 * nrnd3 (mc_randg.cc:159-171), streams[3..7] rnd1..rnd5, streams[8] the x1
 * values of gauss() (mc_randg.cc:138-150).  consumed[9] (optional): draws
 * taken from each.  Potential sums leave out partner beads in the worm's
 * gap as PotEnergy does (WorldLine, mc_qworm.cc:553-575).  FP64 only. */
pimc_status pimc_worm_move(pimc_handle *h, const double *const *streams, const long *lengths, long *consumed);
/* npasses passes of the worm branch of the pass loop (mc_main.cc:348-381)
 * with counter-based draws keyed by (seed, pass, slice): per time slice the
 * worm type's MCWormMove and, while the worm is closed, its exchange
 * bisection at a drawn slice and (slice 0) its exchange-cycle centroid move,
 * then the other types' PIMCPass (centroid at slice 0, bisection, the
 * rotational sweep).  Partner sums leave out the worm's gap throughout. */
pimc_status pimc_worm_run(pimc_handle *h, int npasses, uint64_t seed);
/* the worm {exists, ira, masha, atom_i, atom_m} (TPathWorm, mc_qworm.h:32-48) */
pimc_status pimc_worm_state(pimc_handle *h, int *state);
pimc_status pimc_worm_set_state(pimc_handle *h, const int *state);
/* QWTotal / QWAccep (mc_qworm.h:52-53): [QW_OPEN, CLOSE, INSERT, REMOVE,
 * ADVANCE, RECEDE, SWAP] */
pimc_status pimc_worm_counters(pimc_handle *h, double *total, double *accep);

/* ---- rotor-rotor surrogate for delayed acceptance ----------------------- */

/* An MLP 6 -> 256 -> 256 -> 256 -> 1 with SiLU activations: FP32 first and
 * last layers, BF16 weights and FP32 accumulation in the two 256 x 256
 * layers, which run on the tensor cores (tcgen05).  Weights are row-major
 * [in][out]: w1[6*256], w2/w3[256*256], w4[256]. */
typedef struct pimc_mlp pimc_mlp;
pimc_status pimc_mlp_create(int device, pimc_mlp **out);
pimc_status pimc_mlp_destroy(pimc_mlp *m);
pimc_status pimc_mlp_set_weights(pimc_mlp *m, const float *w1, const float *b1, const float *w2, const float *b2,
                                 const float *w3, const float *b3, const float *w4, float b4);
/* y[i] = MLP(x[i*6 .. i*6+5]) for n inputs (host buffers) */
pimc_status pimc_mlp_forward(pimc_mlp *m, int n, const float *x, float *y);
/* the forward kernel again on the n rows the last pimc_mlp_forward uploaded
 * (outputs stay on the device), on the stream pimc_mlp_stream returns */
pimc_status pimc_mlp_forward_resident(pimc_mlp *m, int n);
void       *pimc_mlp_stream(const pimc_mlp *m);
/* The parameter vector: w1[6*256], b1[256], w2[256*256], b2[256],
 * w3[256*256], b3[256], w4[256], b4 (pimc_mlp_param_count() floats). */
int         pimc_mlp_param_count(void);
pimc_status pimc_mlp_get_params(pimc_mlp *m, float *params);
/* Gradient of mean((y - e)^2) over n samples (the tensor-core training
 * kernels), in parameter-vector order; *loss = that mean (optional). */
pimc_status pimc_mlp_gradients(pimc_mlp *m, int n, const float *x, const float *e, float *grad, double *loss);
/* epochs of Adam over n samples in a seeded order, minibatches of `batch`
 * (a multiple of 128); loss_out[epoch] = the epoch's mean minibatch loss.
 * PIMC_ERR_TIMEOUT when a training kernel gave up a wait: a step may then
 * have applied an incomplete gradient, so the surrogate refuses every later
 * forward, training and delayed-acceptance call (PIMC_ERR_TIMEOUT) until
 * pimc_mlp_set_weights loads weights again. */
pimc_status pimc_mlp_train(pimc_mlp *m, int n, const float *x, const float *e, int epochs, int batch, float lr,
                           uint64_t seed, double *loss_out);

/* Delayed-acceptance rotational sweeps of a water dimer (two nonlinear
 * rotors, no atoms, tabulated densities, even Q) screened by the surrogate.
 * pimc_da_samples: the training data the sampler emits -- for each of the
 * P translational slices the six dimer features (distance, the unit
 * centre-to-centre vector on rotor 0's body axes, its component on rotor
 * 1's z axis, the cosine between the z axes) and the exact caleng energy
 * (caleng_tip4p_gg.f, K).  pimc_da_sweeps: nsweeps sweeps of MCRot3Dstep
 * moves (mc_piqmc.cc:938-1199) in four independent sub-phases per sweep;
 * with use_surrogate the first stage accepts with
 * min(1, rho'/rho exp(-tau dV_sur)), dV_sur = escale * (MLP(new) - MLP(old))
 * summed over the rotor's slices, and the second with
 * min(1, exp(-tau (dV - dV_sur))) from the exact caleng difference, so the
 * sampled distribution is the exact one; without it the plain Metropolis
 * move.  On the FP32 path (pimc_set_precision(h, 1)) the moves use the float
 * proposal, frames, densities, features and caleng terms of that path, the
 * differences and tests in double.  stats[4] = moves, passed the first
 * stage, accepted, exact differences evaluated. */
pimc_status pimc_da_samples(pimc_handle *h, float *feat, float *energy);
pimc_status pimc_da_sweeps(pimc_handle *h, pimc_mlp *m, int nsweeps, uint64_t seed, float escale, int use_surrogate,
                           double *stats);

/* ---- propagator tables ---------------------------------------------------- */

/* The exact linear-rotor propagator of linear_prop/linden.f (tau and the l
 * cut-off linden.f:21-37, exarho linden.f:88-122) for n (temperature K,
 * rotational slices) pairs at once: out[(t*4 + c)*npt + i], columns c =
 * cos gamma, rho, erot, erotsq of the .rot file rows linden.f:48-68.  bconst
 * in cm^-1; iodevn -1 (all l), 0 (even l), 1 (odd l). */
pimc_status pimc_linden(int device, int n, const double *temperature, const int *nslice, double bconst, int npt,
                        int iodevn, double *out);

/* The exact asymmetric-top propagator of nmv_prop/asymrho.f:34-735 on its
 * 1-degree grid for theta = ith0..ith1 (degrees): rho, erot and esq
 * [(ith - ith0)*361*361 + iphi*361 + ichi] as the rho.denXXX_{rho,eng,esq}
 * slabs, energies in cm^-1; abc = A, B, C in cm^-1, J <= maxj.  info[15]
 * (optional): Z, E, Cv of the even-K, odd-K and all states at beta, then Z, E
 * of the three at tau (the "AT BETA" / "AT TAU" lines, asymrho.f:299-423).
 * PIMC_ERR_BAD_ARG where the reference stops (maxj too small for the
 * temperature: exp(-tau E_max) > 1e-8). */
#define PIMC_ASYMRHO_MAXJ 300
pimc_status pimc_asymrho(int device, double temperature, int nslice, int iodevn, int ith0, int ith1,
                         const double *abc, int maxj, double *rho, double *erot, double *esq, double *info);

/* ---- production sampler -------------------------------------------------- */

/* npasses passes of the reference schedule's moves (mc_main.cc:348-381,
 * PIMCPass mc_main.cc:510-522): per pass and type, one centroid move per
 * atom, one bisection per (atom, start slice), and P sweeps of all
 * rotational slices, executed as independent-set phases (disjoint bisection
 * windows; even/odd rotational slices) with a counter-based generator keyed
 * by seed.  Requires P divisible by every type's 2^levels.  Asynchronous on
 * the handle's stream; errors are reported by the next synchronising call. */
pimc_status pimc_run_passes(pimc_handle *h, int npasses, uint64_t seed);
/* Time one pass's launches grouped by move kind (0 centroid, 1 bisection,
 * 2 rotation), outside the graph, with CUDA events on the handle's stream:
 * ms[k] = device time of the group, launches[k] = its kernel launches.  The
 * moves are real moves (the path advances one pass). */
pimc_status pimc_profile_pass(pimc_handle *h, uint64_t seed, double *ms, long long *launches);
/* MCTotal / MCAccep (mc_piqmc.h:25-26): total[type*3+kind], kind = molecule,
 * multilevel, rotation */
pimc_status pimc_counters(pimc_handle *h, double *total, double *accep);
pimc_status pimc_reset_counters(pimc_handle *h);
pimc_status pimc_synchronize(pimc_handle *h);
/* 1: the FP32 path -- pair terms, table interpolation, rotational frames and
 * link densities in float from float copies of the beads, frames and tables;
 * sums, action differences and the Metropolis tests in FP64; the path (and
 * the double frames, derived from the angles before anything reads them) in
 * FP64.  0 (default): every operation in FP64 as the reference. */
pimc_status pimc_set_precision(pimc_handle *h, int mixed);
/* Production-schedule options (no reference counterpart; the reference has
 * one schedule).  PIMC_OPT_FUSED = 1 (default): one launch per bisection
 * block of numb phases and persistent rotational sweeps; 0: one launch per
 * phase.  Both give identical paths for the same seed. */
#define PIMC_OPT_FUSED 1
/* PIMC_OPT_WAIT_NS: how long (ns of %globaltimer, default 2e9) a persistent
 * rotational sweep's slice waits for its neighbours before it gives up, sets
 * the abort word and ends the sweep; the next synchronising call reports
 * PIMC_ERR_TIMEOUT, clears the abort word, and the handle is usable again
 * (the moves of the aborted sweep that had committed stay in the path).
 * Values 0 .. 6e10. */
#define PIMC_OPT_WAIT_NS 3
pimc_status pimc_set_option(pimc_handle *h, int option, long long value);
/* MCAtom[type].numb and .levels (mc_setup.h:66-93) of the handle's system */
pimc_status pimc_type_info(const pimc_handle *h, int type, int *numb, int *levels);
/* scheduled bead-moves per pass: per type N*P*(2^L-1) + N*P, plus P*Q per rotor */
double      pimc_bead_moves_per_pass(const pimc_handle *h);
/* kernels launched on the handle's stream so far */
long long   pimc_launch_count(const pimc_handle *h);
/* the handle's cudaStream_t, for event timing by the caller */
void       *pimc_stream(const pimc_handle *h);
const char *pimc_status_string(pimc_status s);

/* ---- restart files and configurations ------------------------------------
 * pimc_save_checkpoint / pimc_load_checkpoint: the whole path, PIndex, the
 * pass counter and the move counters (the reference's ConfigIO,
 * mc_input.cc:560-600, keeps the first row of MCCoords and MCCosine only);
 * loading checks the system's sizes and temperature, and a continued run with
 * the same seed repeats the uninterrupted one.  pimc_write_xyz /
 * pimc_read_xyz: IOxyz's text format (mc_input.cc:690-794), labels from
 * type_names (may be NULL); reading sets the rotor angles from the unit
 * vectors with chi = 0, as the format keeps no third angle. */
pimc_status pimc_save_checkpoint(pimc_handle *h, const char *path);
pimc_status pimc_load_checkpoint(pimc_handle *h, const char *path);
pimc_status pimc_write_xyz(pimc_handle *h, const char *path, const char *const *type_names);
pimc_status pimc_read_xyz(pimc_handle *h, const char *path);

/* ---- replica batches (no reference counterpart) --------------------------
 * Many independent systems of one species family -- the same types,
 * molecules, masses, levels (<= 4) and steps, each with its own particle
 * counts, slices, rotational slices and temperature -- sampled in one
 * persistent launch: the reference's run of one system repeated for each
 * replica.  Shared potentials come from tables[0]; each replica's rotational
 * density (a .rot or top density at its own tau) from tables[r].  A replica's
 * moves and uniforms are those of a single handle of the same system run
 * with seed pimc_batch_replica_seed(seed, r). */
typedef struct pimc_batch pimc_batch;
pimc_status pimc_batch_create(int n, const pimc_system *systems, int device, pimc_batch **out);
pimc_status pimc_batch_destroy(pimc_batch *b);
pimc_status pimc_batch_load_tables(pimc_batch *b, const pimc_tables *tables);
pimc_status pimc_batch_set_state(pimc_batch *b, int replica, const double *coords, const double *angles,
                                 const int *pindex);
pimc_status pimc_batch_get_state(pimc_batch *b, int replica, double *coords, double *angles, double *cosine,
                                 int *pindex);
pimc_status pimc_batch_set_precision(pimc_batch *b, int mixed);
/* launch shape: warps per CTA (2, 4 or 8) and the resident CTAs per SM the
 * kernels' registers are bounded for (2, 3, or 4: the half-sweep launches of
 * rotation mode 1 take 4, the persistent pass then 3).  pimc_batch_autotune times one
 * pass of each of six shapes (the passes run: the replicas move on), keeps
 * the fastest and returns it in shape_out[2] and the six times in ms_out[6] */
pimc_status pimc_batch_set_shape(pimc_batch *b, int warps, int min_blocks);
/* where the rotational half-sweeps run: 0 (default) inside the persistent
 * pass, each CTA sweeping its own replica's slices; 1 one launch per
 * half-sweep over all replicas, one warp per (replica, slice pair) -- for
 * replicas with many rotational slices, whose sweeps would otherwise keep
 * one CTA busy long after the others finished.  Both make the same moves
 * with the same draws in the same order per replica (identical paths); 1
 * needs an even Q in every replica. */
pimc_status pimc_batch_set_rotation_mode(pimc_batch *b, int mode);
pimc_status pimc_batch_autotune(pimc_batch *b, uint64_t seed, int *shape_out, double *ms_out);
pimc_status pimc_batch_run_passes(pimc_batch *b, int npasses, uint64_t seed);
/* per replica 4 values: E_kin, E_pot, E_rot (as pimc_estimators out[0..2])
 * and the mean z component of the rotor axis over the rotational slices */
pimc_status pimc_batch_estimators(pimc_batch *b, double *out);
/* MCTotal / MCAccep summed over the replicas (layout of pimc_counters) */
pimc_status pimc_batch_counters(pimc_batch *b, double *total, double *accep);
pimc_status pimc_batch_synchronize(pimc_batch *b);
double      pimc_batch_bead_moves_per_pass(const pimc_batch *b);
/* Delayed-acceptance rotational moves of a batch of water dimers (every
 * replica two nonlinear rotors, no atoms, tabulated densities, one P, Q and
 * R): pimc_da_sweeps of every replica at once -- per sub-phase one proposal
 * launch over all replicas' moves, one surrogate launch over all their
 * feature rows, one decision launch -- with replica r's moves and draws
 * those of a single handle run with pimc_batch_replica_seed(seed, r).
 * pimc_batch_da_passes: npasses passes, each the translational moves of
 * the production pass (pimc_batch_run_passes without its rotational
 * sweeps) followed by P delayed-acceptance sweeps, the pass's rotational
 * moves.  stats[4] summed over the replicas as pimc_da_sweeps'. */
pimc_status pimc_batch_da_sweeps(pimc_batch *b, pimc_mlp *m, int nsweeps, uint64_t seed, float escale,
                                 int use_surrogate, double *stats);
pimc_status pimc_batch_da_passes(pimc_batch *b, pimc_mlp *m, int npasses, uint64_t seed, float escale,
                                 int use_surrogate, double *stats);
uint64_t    pimc_batch_replica_seed(uint64_t seed, int replica);
void       *pimc_batch_stream(const pimc_batch *b);

#ifdef __cplusplus
}
#endif
#endif /* PIMC_GB300_H */
