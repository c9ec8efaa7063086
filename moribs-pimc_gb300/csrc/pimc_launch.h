// pimc_launch.h -- host-callable launchers of the kernels in pimc_kernels.cu
#pragma once
#include "pimc_internal.cuh"

struct ReplaySrc;
struct MolScratch;

void launch_derive_state(const Ctx &c, Frame *frames, cudaStream_t s);
void launch_invalidate_caches(const Ctx &c, cudaStream_t s);
void launch_refresh_frames(const Ctx &c, Frame *frames, cudaStream_t s);
void launch_bisect_replay(const Ctx &c, Frame *f, int type, int time0, int exch, ReplaySrc src, double *ds, int *lvl,
                          unsigned long long *cnt, cudaStream_t s);
void launch_bisect_phase(const Ctx &c, Frame *f, int type, int s0, int j, unsigned phase, uint64_t seed,
                         const unsigned *pass, unsigned long long *cnt, cudaStream_t s);
void launch_rot_replay(const Ctx &c, Frame *f, int parity, const double *urot, long nurot, double *rd, int *acc,
                       unsigned long long *cnt, cudaStream_t s);
int launch_rot_phase(const Ctx &c, Frame *f, int parity, unsigned phase, uint64_t seed, const unsigned *pass,
                     unsigned long long *cnt, cudaStream_t s);
int rot_sweeps_max_ctas(int mixed);
int rot_slices_max_ctas(int mixed);
cudaError_t launch_rot_slices(const Ctx &c, Frame *f, int nhalf, unsigned phase0, unsigned group, uint64_t seed,
                              const unsigned *pass, unsigned long long *prog, unsigned *abort_word,
                              unsigned long long *cnt, cudaStream_t s);
cudaError_t launch_rot_sweeps(const Ctx &c, Frame *f, int nctas, int nhalf, unsigned phase0, unsigned group,
                              uint64_t seed, const unsigned *pass, unsigned long long *prog, unsigned *abort_word,
                              unsigned long long *cnt, cudaStream_t s);
void launch_bisect_block(const Ctx &c, Frame *f, int type, int s0, unsigned phase0, uint64_t seed,
                         const unsigned *pass, unsigned long long *cnt, cudaStream_t s);
int launch_mol(const Ctx &c, Frame *f, int type, int atom, bool replay, ReplaySrc src, uint64_t seed,
               const unsigned *pass, unsigned phase, MolScratch *ms, double *dv, int *acc, unsigned long long *cnt,
               cudaStream_t s);
void launch_q_slice(const Ctx &c, Frame *f, int n, const int *a0, const int *it, const double *xyz, double *out,
                    cudaStream_t s);
void launch_q_rot(const Ctx &c, Frame *f, int n, const int *rot, const int *it, const double *v3, int linear,
                  double *out, cudaStream_t s);
void launch_est(const Ctx &c, Frame *f, double *kin, double *pot, double *rot, double *rcf, cudaStream_t s);
void launch_pass_begin(unsigned *pass, cudaStream_t s);
int launch_est_dens(const Ctx &c, Frame *f, DensHist hs, cudaStream_t s);

// ------------------------------------------------------------ worm algorithm
#define PIMC_WORM_MAXM 64             /* the worm's m (Worm.m, mc_qworm.h:46) at most */
size_t worm_scratch_bytes(int numb);
int launch_mol_exchange(const Ctx &c, Frame *f, int type, bool replay, ReplaySrc src, uint64_t seed,
                        const unsigned *pass, unsigned phase, void *scratch, unsigned long long *cnt, cudaStream_t s,
                        const DevWorm *gate = nullptr);
int launch_bisect_slice(const Ctx &c, Frame *f, int type, int time0, int exch, const DevWorm *gate, uint64_t seed,
                        const unsigned *pass, unsigned phase, unsigned long long *cnt, cudaStream_t s);
void launch_worm_prod(const Ctx &c, Frame *f, DevWorm *wk, int *rindex, uint64_t seed, const unsigned *pass,
                      unsigned phase, void *scratch, int numb, cudaStream_t s);
void launch_worm_move(const Ctx &c, Frame *f, DevWorm *wk, int *rindex, const double *const *streams,
                      const long *lengths, long *cursors, void *scratch, int numb, cudaStream_t s);
int est_area_ctas(const Ctx &c, int btype);
int launch_est_area(const Ctx &c, int mode, int btype, const double *mass, double *out, cudaStream_t s);
size_t mol_scratch_bytes();

// ------------------------------------------------------------ delayed acceptance
struct DaMove {
  double prop[3];        // the proposal (phi, cos theta, chi)
  double rn, ro;         // rho(q-1, q) rho(q, q+1) with the new and the old orientation
  double ln[2], lo[2];   // the two link densities, new and old (the link cache's values)
  Frame fn;              // the proposal's frame
  int bad;
};
int launch_da_samples(const Ctx &c, const Frame *f, float *feat, float *energy, cudaStream_t s);
int launch_da_propose(const Ctx &c, const Frame *f, int r, int parity, unsigned phase, uint64_t seed,
                      const unsigned *pass, float *feat, DaMove *mv, cudaStream_t s);
int launch_da_decide(const Ctx &c, Frame *f, int r, int parity, unsigned phase, uint64_t seed, const unsigned *pass,
                     const float *y, int use_sur, float escale, const DaMove *mv, unsigned long long *stats,
                     unsigned long long *cnt, cudaStream_t s);
struct pimc_mlp;
// the surrogate on device-resident rows, on stream s (pimc_mlp.cu)
int mlp_forward_device(pimc_mlp *m, const float *x, int n, float *y, cudaStream_t s);
bool mlp_take_error(pimc_mlp *m);
bool mlp_poisoned(const pimc_mlp *m);
unsigned long long mlp_uid(const pimc_mlp *m);   // 0 for none; unique per created surrogate

// ------------------------------------------------------------ replica batches
#define PIMC_BATCH_MAX_SEG 16         /* bisection segment of batched replicas (levels <= 4) */

// one replica of a batch, as the batch kernels read it
struct BatchRep {
  Ctx c;
  Frame *frames;
  unsigned *pass;                    // the replica's pass counter
  unsigned long long *cnt;           // its MCTotal / MCAccep counters [type][kind][total, accepted]
  uint64_t seed_mix;                 // xor-ed into the run's seed
  int rotation;
};
#define PIMC_BATCH_CTX_BYTES (((sizeof(Ctx) + 15) / 16) * 16)

size_t batch_smem_bytes(int warps);
int launch_da_propose_b(const BatchRep *reps, int nm, int nrep, int r, int parity, unsigned phase, uint64_t seed,
                        float *feat, DaMove *mv, int mixed, cudaStream_t s);
int launch_da_decide_b(const BatchRep *reps, int nm, int nrep, int r, int parity, unsigned phase, uint64_t seed,
                       const float *y, int use_sur, float escale, const DaMove *mv, unsigned long long *stats, int mixed,
                       cudaStream_t s);
int launch_da_pass_b(const BatchRep *reps, int nrep, cudaStream_t s);
int batch_max_ctas(int mixed, int warps, int minb);
void launch_batch_pass(const BatchRep *reps, const int *order, int n, uint64_t seed, unsigned *work, int mixed,
                       int warps, int minb, int nctas, cudaStream_t s, int rot_on = 1, int blk_lo = 0,
                       int blk_hi = 1 << 30);
void launch_batch_rot_flat(const BatchRep *reps, const int *sorted, const int *pre, int nact, int units, int blk,
                           int j, int parity, int nbk, uint64_t seed, int mixed, int warps, int minb,
                           cudaStream_t s, long long phase0 = -1);
int batch_flat_setup(int warps);
void launch_batch_rot_changed(const BatchRep *reps, int n, cudaStream_t s);
void launch_batch_est(const BatchRep *reps, int n, double *out, cudaStream_t s);
void launch_batch_refresh(const BatchRep *reps, int n, int derive, cudaStream_t s);
