// pimc_da.cu -- two-stage delayed-acceptance rotational moves for a pair of
// rigid asymmetric tops (the water dimer of caleng_tip4p_gg.f) screened by
// the surrogate MLP.
//
// A rotational sweep runs in four sub-phases (even slices of rotor 0, of
// rotor 1, then the odd slices), each an independent set: every move of a
// sub-phase reads only orientations the sub-phase does not change.  Per
// sub-phase: k_da_propose draws each move's proposal (the reference's
// MCRot3Dstep proposal, mc_piqmc.cc:955-1001), its density ratio from the
// rotden table (mc_piqmc.cc:1021-1127) and the dimer features of the new
// and the old orientation at the rotor's R translational slices; the MLP
// evaluates all rows in one tensor-core launch; k_da_decide runs the first
// stage with the surrogate's potential difference and, for the moves that
// pass it, the second stage with the exact caleng difference
// (acceptance min(1, exp(-tau (dV - dV_sur)))), which keeps the exact
// stationary distribution (Christen and Fox, J. Comput. Graph. Stat. 14,
// 795 (2005)).  With the surrogate off the same kernels make the plain
// Metropolis move with the exact difference.
#include "pimc_kernels.cuh"
#include "pimc_launch.h"

namespace {

// Six features of a rigid-top dimer seen from rotor a (frame fa, centre ca)
// towards rotor b: the distance (shifted and scaled), the unit vector a->b
// on a's three body axes, its component on b's z axis and the cosine
// between the two z axes.
__device__ __forceinline__ void dimer_features(const Frame &fa, const double ca[3], const Frame &fb,
                                               const double cb[3], float *f)
{
  double R[3] = {cb[0] - ca[0], cb[1] - ca[1], cb[2] - ca[2]};
  double r = sqrt(R[0] * R[0] + R[1] * R[1] + R[2] * R[2]);
  double u[3] = {R[0] / r, R[1] / r, R[2] / r};
  const double *m = fa.m, *n = fb.m;
  f[0] = (float)((r - 3.0) * 2.0);
  f[1] = (float)(u[0] * m[0] + u[1] * m[3] + u[2] * m[6]);
  f[2] = (float)(u[0] * m[1] + u[1] * m[4] + u[2] * m[7]);
  f[3] = (float)(u[0] * m[2] + u[1] * m[5] + u[2] * m[8]);
  f[4] = (float)(u[0] * n[2] + u[1] * n[5] + u[2] * n[8]);
  f[5] = (float)(m[2] * n[2] + m[5] * n[5] + m[8] * n[8]);
}

// the same six features from the float frames (FP32 path)
__device__ __forceinline__ void dimer_features32(const float *m, const double ca[3], const float *nm,
                                                 const double cb[3], float *f)
{
  const float R0 = (float)(cb[0] - ca[0]), R1 = (float)(cb[1] - ca[1]), R2 = (float)(cb[2] - ca[2]);
  const float r = sqrtf(R0 * R0 + R1 * R1 + R2 * R2);
  const float u0 = R0 / r, u1 = R1 / r, u2 = R2 / r;
  f[0] = (r - 3.0f) * 2.0f;
  f[1] = u0 * m[0] + u1 * m[3] + u2 * m[6];
  f[2] = u0 * m[1] + u1 * m[4] + u2 * m[7];
  f[3] = u0 * m[2] + u1 * m[5] + u2 * m[8];
  f[4] = u0 * nm[2] + u1 * nm[5] + u2 * nm[8];
  f[5] = m[2] * nm[2] + m[5] * nm[5] + m[8] * nm[8];
}

__device__ __forceinline__ void centre(const Ctx &c, int g, int it, double v[3])
{
  size_t i = sidx(c.s, it, g);
  v[0] = c.st.x[i];
  v[1] = c.st.y[i];
  v[2] = c.st.z[i];
}

// the features and the exact caleng energy of rotor 0 against rotor 1 at
// every translational slice of the current path
__global__ void k_da_samples(Ctx c, const Frame *frames, float *feat, float *energy)
{
  const DevSys &s = c.s;
  int it = blockIdx.x * blockDim.x + threadIdx.x;
  if (it >= s.P) return;
  const int g0 = s.rot_first, g1 = s.rot_first + 1, q = it / s.R;
  const Frame &f0 = frames[rot_index(s, g0, q)], &f1 = frames[rot_index(s, g1, q)];
  double c0[3], c1[3];
  centre(c, g0, it, c0);
  centre(c, g1, it, c1);
  dimer_features(f0, c0, f1, c1, feat + (size_t)it * 6);
  energy[it] = (float)caleng(f0, f1, c0[0], c0[1], c0[2], c1[0], c1[1], c1[2]);
}

// the link density of two frames in the move's precision: rotden in double,
// or rotden_rho32 from the float frames on the FP32 path
template <bool MIX>
__device__ __forceinline__ double da_link(const Ctx &c, const Frame &a, const Frame &b, int *bad)
{
  if (MIX) return (double)rotden_rho32(c.t, a.mf, b.mf, bad);
  return rotden_rho(c.t, a, b, bad, nullptr, nullptr);
}

// move k of the sub-phase (rotor r, slices of parity `parity`) of one system.
// FP32 path: the float uniforms and proposal increments, the float frame,
// densities and features (as the FP32 rotational moves make them)
template <bool MIX>
__device__ __forceinline__ void da_propose_move(const Ctx &c, const Frame *frames, int k, int r, int parity,
                                                unsigned phase, uint64_t seed, unsigned ps, float *feat, DaMove &d)
{
  const DevSys &s = c.s;
  const int q = 2 * k + parity;
  const int Q = s.Q, R = s.R, g = s.rot_first + r, o = s.rot_first + 1 - r;
  const size_t n = (size_t)s.nrotors * Q;
  const int ri = rot_index(s, g, q);
  double u[4], prop[3];
  rot_uniforms_t<MIX>(seed, ps, phase, q, r, false, u);
  rot_propose_t<MIX>(s, false, c.st.ang[ri], c.st.ang[n + ri], c.st.ang[2 * n + ri], u, prop);
  Frame &fn = d.fn;
  if (MIX) make_frame32((float)prop[0], (float)prop[1], (float)prop[2], fn.mf, &fn.hzf);
  else make_frame(prop[0], prop[1], prop[2], fn);
  const Frame &fo = frames[ri];
  const int im = rot_index(s, g, (q - 1 + Q) % Q);
  const Frame &fm = frames[im], &fp = frames[rot_index(s, g, (q + 1) % Q)];
  // the old links from the link cache where it holds them (it holds exactly
  // what the move's precision evaluates; link (q-1, q) at q-1's entry)
  const bool links = Q >= 3;
  int bad = 0;
  const double l0n = da_link<MIX>(c, fm, fn, &bad), l1n = da_link<MIX>(c, fn, fp, &bad);
  const double l0o = (links && c.st.rl_ok[im]) ? c.st.rl_cache[im] : da_link<MIX>(c, fm, fo, &bad);
  const double l1o = (links && c.st.rl_ok[ri]) ? c.st.rl_cache[ri] : da_link<MIX>(c, fo, fp, &bad);
  double rn = l0n * l1n;
  double ro = l0o * l1o;
  if (MIX) {
    // the float density ratio's terms as rot_decide forms them
    rn = (double)((float)l0n * (float)l1n);
    ro = (double)((float)l0o * (float)l1o);
  }
  const Frame &fb = frames[rot_index(s, o, q)];
  for (int j = 0; j < R; j++) {
    double ca[3], cb[3];
    centre(c, g, q * R + j, ca);
    centre(c, o, q * R + j, cb);
    if (MIX) {
      dimer_features32(fn.mf, ca, fb.mf, cb, feat + (2 * j) * 6);
      dimer_features32(fo.mf, ca, fb.mf, cb, feat + (2 * j + 1) * 6);
    } else {
      dimer_features(fn, ca, fb, cb, feat + (2 * j) * 6);
      dimer_features(fo, ca, fb, cb, feat + (2 * j + 1) * 6);
    }
  }
  d.prop[0] = prop[0]; d.prop[1] = prop[1]; d.prop[2] = prop[2];
  d.rn = rn;
  d.ro = ro;
  d.ln[0] = l0n; d.ln[1] = l1n;
  d.lo[0] = l0o; d.lo[1] = l1o;
  d.bad = bad;
}

template <bool MIX>
__global__ void k_da_propose(Ctx c, const Frame *frames, int r, int parity, unsigned phase, uint64_t seed,
                             const unsigned *pass, float *feat, DaMove *mv)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (2 * k + parity >= c.s.Q) return;
  da_propose_move<MIX>(c, frames, k, r, parity, phase, seed, *pass, feat + (size_t)k * 2 * c.s.R * 6, mv[k]);
}

// the same sub-phase of every replica of a batch: move j is replica j / nm's
// move j % nm (replicas of one shape: the same Q and R)
template <bool MIX>
__global__ void k_da_propose_b(const BatchRep *reps, int nm, int nrep, int r, int parity, unsigned phase,
                               uint64_t seed, float *feat, DaMove *mv)
{
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nm * nrep) return;
  const int rep = j / nm, k = j - rep * nm;
  const BatchRep &b = reps[rep];
  da_propose_move<MIX>(b.c, b.frames, k, r, parity, phase, seed ^ b.seed_mix, *b.pass,
                  feat + (size_t)j * 2 * b.c.s.R * 6, mv[j]);
}

// stats[0] moves, [1] passed the first stage (all, without the surrogate),
// [2] accepted, [3] exact potential differences evaluated
// returns bit 0: passed the first stage, bit 1: accepted, bit 2: exact
// difference evaluated
template <bool MIX>
__device__ __forceinline__ unsigned da_decide_move(const Ctx &c, Frame *frames, int k, int r, int parity,
                                                   unsigned phase, uint64_t seed, unsigned ps, const float *y,
                                                   int use_sur, float escale, const DaMove &d)
{
  const DevSys &s = c.s;
  const int q = 2 * k + parity;
  const int Q = s.Q, R = s.R, g = s.rot_first + r, o = s.rot_first + 1 - r;
  const size_t n = (size_t)s.nrotors * Q;
  const int ri = rot_index(s, g, q);
  if (d.bad) atomicOr(c.st.err, (unsigned)DERR_GRID_RANGE);
  double u1, u2;
  philox_u2(seed, ((uint64_t)ps << 32) | ((uint64_t)phase << 12) | (uint64_t)q, 0x600000u | (uint32_t)r, 0u, &u1,
            &u2);
  const double lr = log(d.rn / d.ro);
  double dvs = 0.0;
  bool pass1 = true;
  if (use_sur) {
    for (int j = 0; j < R; j++) dvs += (double)y[2 * j] - (double)y[2 * j + 1];
    dvs *= (double)escale;
    pass1 = lr - s.tau * dvs > log(u1);
  }
  bool acc = false;
  if (pass1) {
    const Frame &fn = d.fn;
    const Frame &fo = frames[ri], &fb = frames[rot_index(s, o, q)];
    double dv = 0.0;
    for (int j = 0; j < R; j++) {
      if (MIX) {
        // the float pair terms from the float beads, their difference added in double
        const float4 pa = c.st.b4[sidx(s, q * R + j, g)], pb = c.st.b4[sidx(s, q * R + j, o)];
        dv += (double)(caleng32(fn.mf, fb.mf, pa.x, pa.y, pa.z, pb.x, pb.y, pb.z) -
                       caleng32(fo.mf, fb.mf, pa.x, pa.y, pa.z, pb.x, pb.y, pb.z));
      } else {
        double ca[3], cb[3];
        centre(c, g, q * R + j, ca);
        centre(c, o, q * R + j, cb);
        dv += caleng(fn, fb, ca[0], ca[1], ca[2], cb[0], cb[1], cb[2]) -
              caleng(fo, fb, ca[0], ca[1], ca[2], cb[0], cb[1], cb[2]);
      }
    }
    if (use_sur) acc = -s.tau * (dv - dvs) > log(u2);
    else acc = lr - s.tau * dv > log(u1);
    if (acc) {
      c.st.ang[ri] = d.prop[0];
      c.st.ang[n + ri] = d.prop[1];
      c.st.ang[2 * n + ri] = d.prop[2];
      if (MIX) {                        // the double frame is derived from the angles later
        for (int e = 0; e < 9; e++) frames[ri].mf[e] = fn.mf[e];
        frames[ri].hzf = fn.hzf;
      } else {
        frames[ri] = fn;
      }
    }
  }
  // the link cache after the move (its two links belong to this move alone
  // within the sub-phase)
  if (Q >= 3 && !d.bad) {
    const int im = rot_index(s, g, (q - 1 + Q) % Q);
    c.st.rl_cache[im] = acc ? d.ln[0] : d.lo[0];
    c.st.rl_cache[ri] = acc ? d.ln[1] : d.lo[1];
    c.st.rl_ok[im] = 1;
    c.st.rl_ok[ri] = 1;
  }
  return (pass1 ? 1u : 0u) | (acc ? 2u : 0u) | (pass1 ? 4u : 0u);
}

// the counts of a warp's moves added once per warp: stats[0..3] (moves,
// first stage passed, accepted, exact differences) and the rotation
// counters of MCTotal / MCAccep; cnt may differ between the lanes
__device__ __forceinline__ void da_count(bool live, unsigned f, unsigned long long *stats, unsigned long long *cnt)
{
  const unsigned m = __ballot_sync(0xffffffffu, live);
  const unsigned p1 = __ballot_sync(0xffffffffu, live && (f & 1u));
  const unsigned ac = __ballot_sync(0xffffffffu, live && (f & 2u));
  const unsigned ex = __ballot_sync(0xffffffffu, live && (f & 4u));
  const int lane = threadIdx.x & 31;
  if (lane == 0 && m) {
    atomicAdd(stats, (unsigned long long)__popc(m));
    atomicAdd(stats + 1, (unsigned long long)__popc(p1));
    atomicAdd(stats + 2, (unsigned long long)__popc(ac));
    atomicAdd(stats + 3, (unsigned long long)__popc(ex));
  }
  // lanes with the same counter array add together
  const unsigned long long key = live ? (unsigned long long)cnt : 0ull;
  const unsigned grp = __match_any_sync(0xffffffffu, key);
  if (live && lane == __ffs(grp) - 1) {
    atomicAdd(cnt, (unsigned long long)__popc(grp));
    atomicAdd(cnt + 1, (unsigned long long)__popc(grp & ac));
  }
}

// stats[0] moves, [1] passed the first stage (all, without the surrogate),
// [2] accepted, [3] exact potential differences evaluated
template <bool MIX>
__global__ void k_da_decide(Ctx c, Frame *frames, int r, int parity, unsigned phase, uint64_t seed,
                            const unsigned *pass, const float *y, int use_sur, float escale, const DaMove *mv,
                            unsigned long long *stats, unsigned long long *cnt)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const bool live = 2 * k + parity < c.s.Q;
  unsigned f = 0;
  if (live) f = da_decide_move<MIX>(c, frames, k, r, parity, phase, seed, *pass, y + (size_t)k * 2 * c.s.R, use_sur, escale,
                               mv[k]);
  da_count(live, f, stats, cnt + (c.s.imtype * 3 + 2) * 2);
}

template <bool MIX>
__global__ void k_da_decide_b(const BatchRep *reps, int nm, int nrep, int r, int parity, unsigned phase,
                              uint64_t seed, const float *y, int use_sur, float escale, const DaMove *mv,
                              unsigned long long *stats)
{
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const bool live = j < nm * nrep;
  const int rep = live ? j / nm : 0, k = j - rep * nm;
  const BatchRep &b = reps[rep];
  unsigned f = 0;
  if (live)
    f = da_decide_move<MIX>(b.c, b.frames, k, r, parity, phase, seed ^ b.seed_mix, *b.pass, y + (size_t)j * 2 * b.c.s.R,
                       use_sur, escale, mv[j]);
  da_count(live, f, stats, b.cnt + (b.c.s.imtype * 3 + 2) * 2);
}

// one more pass on every replica's counter (the keys of the call's draws)
__global__ void k_da_pass_b(const BatchRep *reps, int nrep)
{
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < nrep) ++(*reps[j].pass);
}

}  // namespace

int launch_da_samples(const Ctx &c, const Frame *f, float *feat, float *energy, cudaStream_t s)
{
  k_da_samples<<<(c.s.P + 127) / 128, 128, 0, s>>>(c, f, feat, energy);
  return 1;
}

int launch_da_propose(const Ctx &c, const Frame *f, int r, int parity, unsigned phase, uint64_t seed,
                      const unsigned *pass, float *feat, DaMove *mv, cudaStream_t s)
{
  int nm = (c.s.Q + 1 - parity) / 2;
  if (c.s.mixed) k_da_propose<true><<<(nm + 127) / 128, 128, 0, s>>>(c, f, r, parity, phase, seed, pass, feat, mv);
  else k_da_propose<false><<<(nm + 127) / 128, 128, 0, s>>>(c, f, r, parity, phase, seed, pass, feat, mv);
  return 1;
}

int launch_da_decide(const Ctx &c, Frame *f, int r, int parity, unsigned phase, uint64_t seed, const unsigned *pass,
                     const float *y, int use_sur, float escale, const DaMove *mv, unsigned long long *stats,
                     unsigned long long *cnt, cudaStream_t s)
{
  int nm = (c.s.Q + 1 - parity) / 2;
  if (c.s.mixed)
    k_da_decide<true><<<(nm + 127) / 128, 128, 0, s>>>(c, f, r, parity, phase, seed, pass, y, use_sur, escale, mv, stats,
                                                       cnt);
  else
    k_da_decide<false><<<(nm + 127) / 128, 128, 0, s>>>(c, f, r, parity, phase, seed, pass, y, use_sur, escale, mv,
                                                        stats, cnt);
  return 1;
}

int launch_da_propose_b(const BatchRep *reps, int nm, int nrep, int r, int parity, unsigned phase, uint64_t seed,
                        float *feat, DaMove *mv, int mixed, cudaStream_t s)
{
  const int n = nm * nrep;
  if (mixed) k_da_propose_b<true><<<(n + 127) / 128, 128, 0, s>>>(reps, nm, nrep, r, parity, phase, seed, feat, mv);
  else k_da_propose_b<false><<<(n + 127) / 128, 128, 0, s>>>(reps, nm, nrep, r, parity, phase, seed, feat, mv);
  return 1;
}

int launch_da_decide_b(const BatchRep *reps, int nm, int nrep, int r, int parity, unsigned phase, uint64_t seed,
                       const float *y, int use_sur, float escale, const DaMove *mv, unsigned long long *stats,
                       int mixed, cudaStream_t s)
{
  const int n = nm * nrep;
  if (mixed)
    k_da_decide_b<true><<<(n + 127) / 128, 128, 0, s>>>(reps, nm, nrep, r, parity, phase, seed, y, use_sur, escale, mv,
                                                        stats);
  else
    k_da_decide_b<false><<<(n + 127) / 128, 128, 0, s>>>(reps, nm, nrep, r, parity, phase, seed, y, use_sur, escale,
                                                         mv, stats);
  return 1;
}

int launch_da_pass_b(const BatchRep *reps, int nrep, cudaStream_t s)
{
  k_da_pass_b<<<(nrep + 127) / 128, 128, 0, s>>>(reps, nrep);
  return 1;
}
