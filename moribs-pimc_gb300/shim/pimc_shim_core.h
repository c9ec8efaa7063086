/*
 * pimc_shim_core.h -- the reference's move calls on the GB300 library with
 * the reference's own random-number streams (host code, C ABI).
 *
 * A replay entry point of the library consumes a number of draws that
 * depends on its decisions (gauss() only for the bisection levels reached,
 * rnd2() / rnd3() only where the action difference is not negative).  The
 * reference draws lazily, one value when its code reaches the call.  The
 * core keeps a look-ahead queue per stream: it fills each queue with the
 * most a call can use, hands the queued values to the GPU, drops the count
 * the GPU reports consumed and keeps the rest for the next call.  Each
 * stream therefore gives the same values to the same decisions as in the
 * reference, provided nothing else draws from these streams in between
 * (in the reference's pass loop without the worm nothing does).
 *
 * The reference-facing functions (MCBisectionMove(int,int) and the others
 * of mc_piqmc.h:4-23 over the reference's globals) are in
 * pimc_gpu_shim.cc, which is compiled into the reference's program.
 */
#ifndef PIMC_SHIM_CORE_H
#define PIMC_SHIM_CORE_H

#include "../../include/pimc_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* one draw from a reference stream */
typedef double (*pimc_shim_draw)(void *ctx);

typedef struct pimc_shim pimc_shim;

/* rnd1, rnd2, rnd3 (mc_randg.cc:95-112) and the x1 of gauss()
 * (mc_randg.cc:138-150; gauss(1.0) returns it exactly) */
pimc_shim *pimc_shim_create(pimc_handle *h, pimc_shim_draw rnd1, pimc_shim_draw rnd2, pimc_shim_draw rnd3,
                            pimc_shim_draw gauss_x1, void *ctx);
void pimc_shim_destroy(pimc_shim *s);

/* MCBisectionMove(type, time) (mc_piqmc.cc:194-294); *total / *accep get
 * the increments of MCTotal / MCAccep[type][MCMULTI] (one per atom, one per
 * atom whose levels were all accepted) */
pimc_status pimc_shim_bisection(pimc_shim *s, int type, int time, double *total, double *accep);
/* MCMolecularMove(type) (mc_piqmc.cc:54-102): increments of [type][MCMOLEC] */
pimc_status pimc_shim_molecular(pimc_shim *s, int type, double *total, double *accep);
/* MCRotationsMove / MCRotations3D (mc_piqmc.cc:421-517, 692-779) with the
 * call's runif() draws (3 per slice of the linear rotor, 4 per slice and
 * rotor of the tops, in the reference's order): increments of [type][MCROTAT] */
pimc_status pimc_shim_rotations(pimc_shim *s, const double *urot, long n, double *total, double *accep);
/* values drawn from each stream and not yet used: rnd1, rnd2, rnd3, gauss */
void pimc_shim_pending(const pimc_shim *s, long *pending);

#ifdef __cplusplus
}
#endif
#endif
