// pimc_gpu_shim.cc -- the reference's move functions on the GB300 library.
//
// Compiled into the reference's own program (with the reference's headers
// on the include path) in place of the move functions of mc_piqmc.cc:
//   void MCMolecularMove(int type)             mc_piqmc.h:4, mc_piqmc.cc:54-102
//   void MCBisectionMove(int type, int time)   mc_piqmc.h:5, mc_piqmc.cc:194-294
//   void MCRotationsMove(int type)             mc_piqmc.h:6, mc_piqmc.cc:421-517
//   void MCRotations3D(int type)               mc_piqmc.h:8, mc_piqmc.cc:692-779
// with the same signatures, over the reference's globals: each call copies
// MCCoords / MCAngles / PIndex to the GPU, makes the reference's move there
// with the reference's own random streams (rnd1, rnd2, rnd3 and gauss
// through the look-ahead queues of pimc_shim_core; runif from a fresh
// RngStream per rotational call, as the reference draws them), copies the
// path and MCCosine back, and adds the move's counts to MCTotal / MCAccep
// (mc_piqmc.h:25-26).  The rest of the program (PIMCPass, mc_main.cc:510-522,
// the estimators, the IO) is the reference's, unchanged.
//
// The build leaves the four definitions of mc_piqmc.cc out by renaming them
// when that file is compiled (-DMCMolecularMove=MCMolecularMove_cpu and the
// others); calls from every other file then reach these.  Before the first
// pass the program calls GpuShimInit with the tables it read
// (InitPotentials / InitRotDensity, mc_poten.cc:93-164).
#include <omp.h>

#include <cmath>
#include <vector>

#include "mc_confg.h"
#include "mc_piqmc.h"
#include "mc_randg.h"
#include "mc_setup.h"
#include "mc_utils.h"
#include "rngstream.h"
#include "omprng.h"

#include "pimc_shim_core.h"

static pimc_handle *g_handle = nullptr;
static pimc_shim *g_shim = nullptr;

static double draw_rnd1(void *) { return rnd1(); }
static double draw_rnd2(void *) { return rnd2(); }
static double draw_rnd3(void *) { return rnd3(); }
static double draw_gauss(void *) { return gauss(1.0); }     // x1 exactly (mc_randg.cc:138-150)

// the reference's system as the library's: MCAtom[] (mc_setup.h:66-93) and
// the run parameters of mc_setup.h:9-64
void GpuShimInit(const pimc_tables *tables, int device)
{
  pimc_system s = {};
  s.ntypes = NumbTypes;
  for (int t = 0; t < NumbTypes && t < PIMC_MAX_TYPES; t++) {
    s.type[t].numb = MCAtom[t].numb;
    s.type[t].molecule = MCAtom[t].molecule;
    s.type[t].stat = MCAtom[t].stat;
    s.type[t].levels = MCAtom[t].levels;
    s.type[t].mcstep = MCAtom[t].mcstep;
    s.type[t].lambda = MCAtom[t].lambda;
  }
  s.nslices = NumbTimes;
  s.rotation = ROTATION ? 1 : 0;
  s.nrotslices = ROTATION ? NumbRotTimes : 0;
  s.temperature = Temperature;
  s.rtstep = (ROTATION && IMTYPE >= 0) ? MCAtom[IMTYPE].rtstep : 0.0;
  s.ispher = ISPHER;
  s.rot_den_type = RotDenType;
  s.rot_odevn = RotOdEvn;
  s.rot_eoff = RotEoff;
  s.rot_abc[0] = X_Rot;
  s.rot_abc[1] = Y_Rot;
  s.rot_abc[2] = Z_Rot;
  s.rn_ratio = RNratio;
  s.minimage = MINIMAGE ? 1 : 0;
  for (int d = 0; d < 3; d++) s.box[d] = BoxSize ? BoxSize[d] : 0.0;
  if (pimc_create(&s, device, &g_handle) != PIMC_OK || pimc_load_tables(g_handle, tables) != PIMC_OK)
    nrerror("GpuShimInit", "the GB300 library rejected the system or its tables");
  g_shim = pimc_shim_create(g_handle, draw_rnd1, draw_rnd2, draw_rnd3, draw_gauss, nullptr);
  if (!g_shim) nrerror("GpuShimInit", "shim");
}

void GpuShimFree(void)
{
  pimc_shim_destroy(g_shim);
  pimc_destroy(g_handle);
  g_shim = nullptr;
  g_handle = nullptr;
}

static std::vector<double> flat3(double **a)
{
  const size_t n = (size_t)NumbAtoms * NumbTimes;
  std::vector<double> v(3 * n);
  for (int d = 0; d < 3; d++)
    for (size_t i = 0; i < n; i++) v[d * n + i] = a[d][i];
  return v;
}

static void unflat3(const std::vector<double> &v, double **a)
{
  const size_t n = (size_t)NumbAtoms * NumbTimes;
  for (int d = 0; d < 3; d++)
    for (size_t i = 0; i < n; i++) a[d][i] = v[d * n + i];
}

static void push(void)
{
  std::vector<double> c = flat3(MCCoords), a = flat3(MCAngles);
  if (pimc_set_state(g_handle, c.data(), a.data(), PIndex) != PIMC_OK) nrerror("GpuShim", "pimc_set_state");
}

static void pull(void)
{
  const size_t n = 3 * (size_t)NumbAtoms * NumbTimes;
  std::vector<double> c(n), a(n), o(n);
  if (pimc_get_state(g_handle, c.data(), a.data(), o.data(), PIndex) != PIMC_OK) nrerror("GpuShim", "pimc_get_state");
  unflat3(c, MCCoords);
  unflat3(o, MCCosine);
  // only the rotors' first NumbRotTimes angles are the sampled ones
  // (mc_main.cc:193-199); the library returns the others as they were set
  unflat3(a, MCAngles);
}

static void check(pimc_status e, const char *what)
{
  if (e != PIMC_OK) nrerror(what, pimc_status_string(e));
}

void MCBisectionMove(int type, int time)
{
  double tot = 0.0, acc = 0.0;
  push();
  check(pimc_shim_bisection(g_shim, type, time, &tot, &acc), "MCBisectionMove");
  pull();
  MCTotal[type][MCMULTI] += tot;
  MCAccep[type][MCMULTI] += acc;
}

void MCMolecularMove(int type)
{
  double tot = 0.0, acc = 0.0;
  push();
  check(pimc_shim_molecular(g_shim, type, &tot, &acc), "MCMolecularMove");
  pull();
  MCTotal[type][MCMOLEC] += tot;
  MCAccep[type][MCMOLEC] += acc;
}

// runif() draws of one rotational call in the reference's order: even
// slices then odd slices, per slice `per` draws for each rotor in turn
static std::vector<double> rot_draws(int nrotors, int per)
{
  RngStream Rng[omp_get_num_procs()];
  std::vector<double> u;
  u.reserve((size_t)NumbRotTimes * nrotors * per);
  for (int parity = 0; parity < 2; parity++)
    for (int it = parity; it < NumbRotTimes; it += 2)
      for (int r = 0; r < nrotors; r++)
        for (int k = 0; k < per; k++) u.push_back(runif(Rng));
  return u;
}

void MCRotationsMove(int type)
{
  std::vector<double> u = rot_draws(1, 3);            // mc_piqmc.cc:490-512
  double tot = 0.0, acc = 0.0;
  push();
  check(pimc_shim_rotations(g_shim, u.data(), (long)u.size(), &tot, &acc), "MCRotationsMove");
  pull();
  MCTotal[type][MCROTAT] += tot;
  MCAccep[type][MCROTAT] += acc;
}

void MCRotations3D(int type)
{
  std::vector<double> u = rot_draws(MCAtom[type].numb, 4);   // mc_piqmc.cc:737-771
  double tot = 0.0, acc = 0.0;
  push();
  check(pimc_shim_rotations(g_shim, u.data(), (long)u.size(), &tot, &acc), "MCRotations3D");
  pull();
  MCTotal[type][MCROTAT] += tot;
  MCAccep[type][MCROTAT] += acc;
}
