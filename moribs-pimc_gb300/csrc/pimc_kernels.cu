// pimc_kernels.cu -- sm_103a kernels of the sampling path.
//   k_*_replay : one reference call with replayed random streams (parity)
//   k_*_phase  : one independent-set phase of the production schedule
//   k_q_*      : batched energy queries (PotEnergy / PotRotE3D / PotRotEnergy)
//   k_est_*    : estimator sums (mc_estim.cc)
#include "pimc_kernels.cuh"
#include "pimc_launch.h"

// ------------------------------------------------------------ derived state
// after a path upload: float copies of beads and unit vectors, rotor frames,
// and both caches marked stale
__global__ void k_derive_state(Ctx c, Frame *frames)
{
  size_t nb = (size_t)c.s.P * c.s.nap;
  size_t n = (size_t)c.s.nrotors * c.s.Q;
  size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < nb; i += stride) {
    c.st.b4[i] = make_float4((float)c.st.x[i], (float)c.st.y[i], (float)c.st.z[i], 0.0f);
  }
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    make_frame(c.st.ang[i], c.st.ang[n + i], c.st.ang[2 * n + i], frames[i]);
    if (c.s.nrotors > 0 && c.s.molecule[c.s.imtype] == 1 && lazy_linear(c, c.s.mixed != 0)) {
      // as the FP32 moves write it
      float v[3];
      unit_vector32((float)c.st.ang[i], (float)c.st.ang[n + i], v);
      for (int d = 0; d < 3; d++) c.st.cosvf[d * n + i] = v[d];
    } else {
      for (int d = 0; d < 3; d++) c.st.cosvf[d * n + i] = (float)c.st.cosv[d * n + i];
    }
    c.st.rp_ok[i] = 0;
    c.st.rl_ok[i] = 0;
  }
}

__global__ void k_invalidate_caches(Ctx c)
{
  size_t n = (size_t)c.s.nrotors * c.s.Q;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    c.st.rp_ok[i] = 0;
    c.st.rl_ok[i] = 0;
  }
}

// ------------------------------------------------------------ bisection
// MCBisectionMove(type, time) / MCBisectionMoveExchange: all atoms of the
// type in order, each consuming the replayed gauss()/rnd3() streams
template <bool MIX>
__global__ void __launch_bounds__(PIMC_BIS_THREADS) k_bisect_replay(Ctx c, Frame *frames, int type, int time0, int exch,
                                                               ReplaySrc src, double *ds_out, int *lvl_out,
                                                               unsigned long long *cnt)
{
  __shared__ BisectShared sh;
  int L = c.s.levels[type];
  for (int atom = 0; atom < c.s.numb[type]; atom++) {
    int acc = bisect_move<MIX>(c, frames, type, atom, time0, exch, src, sh, ds_out + (size_t)atom * L);
    if (threadIdx.x == 0) {
      lvl_out[atom] = sh.passed;
      cnt[(type * 3 + 1) * 2 + 0] += 1;
      if (acc) cnt[(type * 3 + 1) * 2 + 1] += 1;
    }
    __syncthreads();
  }
}

// one phase of the production schedule: window k starts at s0 + k*M and
// moves atom (k + j) mod numb; interiors of all windows are disjoint
template <bool MIX>
__global__ void __launch_bounds__(PIMC_BIS_THREADS) k_bisect_phase(Ctx c, Frame *frames, int type, int s0, int j,
                                                              unsigned phase, uint64_t seed, const unsigned *pass,
                                                              unsigned long long *cnt)
{
  __shared__ BisectShared sh;
  int M = 1 << c.s.levels[type];
  int k = blockIdx.x;
  int atom = (k + j) % c.s.numb[type];
  int time0 = s0 + k * M;
  PhiloxSrc src{seed, ((uint64_t)(*pass) << 32) | ((uint64_t)phase << 12) | (uint64_t)k};
  int acc = bisect_move<MIX>(c, frames, type, atom, time0, 0, src, sh, nullptr);
  if (threadIdx.x == 0) {
    atomicAdd(&cnt[(type * 3 + 1) * 2 + 0], 1ull);
    if (acc) atomicAdd(&cnt[(type * 3 + 1) * 2 + 1], 1ull);
  }
}

// one bisection block of the production schedule: all phases j < numb of
// one (type, s0).  Window k = [s0 + kM, s0 + (k+1)M] moves atoms (k + j) mod
// numb for j = 0, 1, ...; the beads a window's moves read and write lie in
// its own interior or on its fixed end points, so CTA k runs its phases one
// after the other with no other CTA involved, and the result equals the
// phase-by-phase launches with the same phase numbers.
template <bool MIX>
__global__ void __launch_bounds__(PIMC_BIS_THREADS) k_bisect_block(Ctx c, Frame *frames, int type, int s0, unsigned phase0,
                                                              uint64_t seed, const unsigned *pass,
                                                              unsigned long long *cnt)
{
  __shared__ BisectShared sh;
  const int M = 1 << c.s.levels[type], N = c.s.numb[type];
  const int k = blockIdx.x;
  const int time0 = s0 + k * M;
  const unsigned ps = *pass;
  unsigned long long tot = 0, nacc = 0;
  for (int j = 0; j < N; j++) {
    PhiloxSrc src{seed, ((uint64_t)ps << 32) | ((uint64_t)(phase0 + (unsigned)j) << 12) | (uint64_t)k};
    int acc = bisect_move<MIX>(c, frames, type, (k + j) % N, time0, 0, src, sh, nullptr);
    tot++;
    nacc += acc;
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    atomicAdd(&cnt[(type * 3 + 1) * 2 + 0], tot);
    atomicAdd(&cnt[(type * 3 + 1) * 2 + 1], nacc);
  }
}

// ------------------------------------------------------------ rotations
__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long *p)
{
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_u64(unsigned long long *p, unsigned long long v)
{
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long global_ns()
{
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// waits, progress and look-ahead of a one-slice-per-CTA persistent launch
struct RotSliceHooks {
  const unsigned long long *wl, *wr;    // progress words of the neighbouring slices
  unsigned long long *mine;
  unsigned long long id;
  unsigned *abort_word, *err;
  const DevSys *sys;
  uint64_t seed;
  unsigned pass, phase_next;
  int h, pair, linear, has_next, mixed;
  // all lanes of the finishing warp: lane 0 polls until both neighbours have
  // finished half-sweep h-1, then every lane acquires the two progress words
  // itself, so that its own loads of the neighbours' state come after them
  __device__ bool wait(int lane)
  {
    int ok = 1;
    if (lane == 0) {
      if (*(volatile unsigned *)abort_word) ok = 0;
      const unsigned long long t0 = global_ns();
      for (int side = 0; ok && h > 0 && side < 2; side++) {
        const unsigned long long *w = side ? wr : wl;
        for (;;) {
          unsigned long long v = ld_acquire_u64(w);
          if ((v >> 24) == id && (long long)(v & 0xFFFFFFull) >= h) break;
          if (*(volatile unsigned *)abort_word) { ok = 0; break; }
          if (global_ns() - t0 > sys->wait_ns) {
            atomicExch(abort_word, 1u);
            ok = 0;
            break;
          }
        }
      }
      if (!ok) atomicOr(err, (unsigned)DERR_TIMEOUT);
    }
    ok = __shfl_sync(0xffffffffu, ok, 0);
    if (ok && h > 0) {
      (void)ld_acquire_u64(wl);
      (void)ld_acquire_u64(wr);
    }
    return ok != 0;
  }
  __device__ void published() { st_release_u64(mine, (id << 24) | (unsigned long long)(h + 1)); }
  // the slice's next move, for both outcomes of this one, on all lanes of a
  // warp: lane k < 2 proposes from the current (k = 0) or the proposed
  // (k = 1) angles; on the FP64 path lanes 0-3 then take the sines and
  // cosines of the two proposals' phi and chi, and lanes 0 and 2 build
  // their frames (a top) or unit vectors (a linear rotor), so that the next
  // rot_prepare starts its partner sums at once
  __device__ void ahead(RotShared &sh, int lane)
  {
    if (!has_next) return;
    double u[4], prop[3] = {0.0, 0.0, 0.0};
    const int k = lane & 1;
    const double *a = k ? sh.ang_new : sh.ang_old;
    if (mixed) {
      rot_uniforms_t<true>(seed, pass, phase_next, pair, 0, linear, u);
      if (lane < 2) rot_propose_t<true>(*sys, linear, a[0], a[1], a[2], u, prop);
    } else {
      rot_uniforms(seed, pass, phase_next, pair, 0, linear, u);
      if (lane < 2) rot_propose(*sys, linear, a[0], a[1], a[2], u, prop);
    }
    if (lane < 2)
      for (int d = 0; d < 3; d++) sh.nxt_prop[k][d] = prop[d];
    if (lane == 0)
      for (int d = 0; d < 4; d++) sh.nxt_u[d] = u[d];
    if (mixed) return;
    __syncwarp();
    // lane 2o + j: proposal o, angle phi (j = 0) or chi (j = 1)
    const int o = (lane >> 1) & 1, j = lane & 1;
    if (linear) {
      if (lane < 4 && j == 0) unit_vector(sh.nxt_prop[o][0], sh.nxt_prop[o][1], sh.nxt_nv[o]);
      return;
    }
    double sn = 0.0, cs = 1.0;
    if (lane < 4) sincos(sh.nxt_prop[o][j ? 2 : 0], &sn, &cs);
    const double sk = __shfl_down_sync(0xffffffffu, sn, 1), ck = __shfl_down_sync(0xffffffffu, cs, 1);
    if (lane < 4 && j == 0) {
      const double *p = sh.nxt_prop[o];
      Frame &f = sh.nxt_fn[o];
      frame_from_sincos(p[0], p[1], p[2], sn, cs, sk, ck, f);      // = make_frame(p[0], p[1], p[2], f)
      make_frame32((float)p[0], (float)p[1], (float)p[2], f.mf, &f.hzf);
    }
  }
};

// serial position of slice q in MCRotationsMove's loops: even slices, then odd
__device__ __forceinline__ long rot_serial(int Q, int q) { return (q & 1) ? (Q + 1) / 2 + q / 2 : q / 2; }

// one independent set of slices of MCRotationsMove / MCRotations3D: CTA b
// handles slice q = q0 + 2b and all rotors of the type in order
template <bool REPLAY, bool MIX>
__global__ void __launch_bounds__(PIMC_ROT_THREADS) k_rot(Ctx c, Frame *frames, int q0, int nq, const double *urot,
                                                          long nurot, unsigned phase, uint64_t seed,
                                                          const unsigned *pass, double *rd_out, int *acc_out,
                                                          unsigned long long *cnt)
{
  __shared__ RotShared sh;
  if ((int)blockIdx.x >= nq) return;
  const int q = q0 + 2 * (int)blockIdx.x;
  const int nr = c.s.nrotors;
  const bool linear = c.s.molecule[c.s.imtype] == 1;
  const int per = linear ? 3 : 4;
  const size_t n = (size_t)nr * c.s.Q;
  for (int r = 0; r < nr; r++) {
    double u[4] = {0.5, 0.5, 0.5, 0.5}, prop[3] = {0.0, 0.0, 0.0};
    if (threadIdx.x == 0) {
      if (REPLAY) {
        // serial consumption order: even slices then odd, rotors inside a slice
        long idx = rot_serial(c.s.Q, q) * (long)nr + r;
        for (int k = 0; k < per; k++) {
          long p = idx * per + k;
          u[k] = (p < nurot) ? urot[p] : 0.5;
          if (p >= nurot) atomicOr(c.st.err, (unsigned)DERR_STREAM);
        }
      } else {
        rot_uniforms_t<MIX>(seed, *pass, phase, q >> 1, r, linear, u);
      }
      size_t i1 = (size_t)r * c.s.Q + q;
      if (REPLAY) rot_propose(c.s, linear, c.st.ang[i1], c.st.ang[n + i1], c.st.ang[2 * n + i1], u, prop);
      else rot_propose_t<MIX>(c.s, linear, c.st.ang[i1], c.st.ang[n + i1], c.st.ang[2 * n + i1], u, prop);
    }
    int g0 = c.s.rot_first + r;
    int acc = rot_step<MIX, false>(c, frames, g0, q, u, prop, linear, sh, nullptr, REPLAY);
    double rd = sh.rd;          // written by the finishing warp
    if (threadIdx.x == 0) {
      if (REPLAY) {
        rd_out[(size_t)q * nr + r] = rd;
        acc_out[(size_t)q * nr + r] = acc;
      }
      int ty = c.s.imtype;
      atomicAdd(&cnt[(ty * 3 + 2) * 2 + 0], 1ull);
      if (acc) atomicAdd(&cnt[(ty * 3 + 2) * 2 + 1], 1ull);
    }
  }
}

// nhalf half-sweeps (even slices, odd slices, even, ...) of the rotational
// moves in one cooperative launch, Q even.  CTA b owns the slice pairs
// (2p, 2p+1), p in [p0, p1).  Its even slices read the odd slice of the CTA
// on the left and its odd slices the even slice of the CTA on the right, so
// half-sweep h waits only for that neighbour to have finished h-1; the
// neighbour in turn waits for this CTA's h before it writes the slice read
// here again.  Every move therefore sees exactly the state it sees in the
// launch-per-half-sweep schedule, with the same uniforms, and the results
// are identical.  Progress words hold (launch id << 24) | half-sweeps done;
// the wait gives up after wait_ns (two seconds unless set), sets the abort word and the timeout
// error bit, and every CTA then leaves.
template <bool MIX>
__global__ void __launch_bounds__(PIMC_ROT_THREADS) k_rot_sweeps(Ctx c, Frame *frames, int nhalf, unsigned phase0,
                                                                 unsigned group, uint64_t seed, const unsigned *pass,
                                                                 unsigned long long *prog, unsigned *abort_word,
                                                                 unsigned long long *cnt)
{
  __shared__ RotShared sh;
  __shared__ int stop;
  const int nc = gridDim.x, b = blockIdx.x;
  const int npairs = c.s.Q >> 1;
  const int p0 = (int)((long)b * npairs / nc), p1 = (int)((long)(b + 1) * npairs / nc);
  const int nr = c.s.nrotors;
  const bool linear = c.s.molecule[c.s.imtype] == 1;
  const unsigned ps = *pass;
  const unsigned long long id = ((unsigned long long)ps << 8) | (group & 255u);
  const int left = (b + nc - 1) % nc, right = (b + 1) % nc;
  const size_t n = (size_t)nr * c.s.Q;
  unsigned long long tot = 0, nacc = 0;
  double u[4] = {0.5, 0.5, 0.5, 0.5}, prop[3] = {0.0, 0.0, 0.0};
  for (int h = 0; h < nhalf; h++) {
    const int parity = h & 1;
    const unsigned phase = phase0 + (unsigned)h;
    if (threadIdx.x == 0) {
      // the first move's uniforms and proposal read only this CTA's own slice
      // and are ready before the neighbour is
      size_t i1 = (size_t)(2 * p0 + parity);
      rot_uniforms_t<MIX>(seed, ps, phase, p0, 0, linear, u);
      rot_propose_t<MIX>(c.s, linear, c.st.ang[i1], c.st.ang[n + i1], c.st.ang[2 * n + i1], u, prop);
      int st = 0;
      if (*(volatile unsigned *)abort_word) {
        atomicOr(c.st.err, (unsigned)DERR_TIMEOUT);
        st = 1;
      } else if (nc > 1 && h > 0) {
        const unsigned long long *w = prog + (parity ? right : left);
        const unsigned long long t0 = global_ns();
        for (;;) {
          unsigned long long v = ld_acquire_u64(w);
          if ((v >> 24) == id && (long long)(v & 0xFFFFFFull) >= h) break;
          if (*(volatile unsigned *)abort_word) {
            atomicOr(c.st.err, (unsigned)DERR_TIMEOUT);
            st = 1;
            break;
          }
          if (global_ns() - t0 > c.s.wait_ns) {
            atomicExch(abort_word, 1u);
            atomicOr(c.st.err, (unsigned)DERR_TIMEOUT);
            st = 1;
            break;
          }
        }
        __threadfence();
      }
      stop = st;
    }
    __syncthreads();
    if (stop) break;
    for (int p = p0; p < p1; p++) {
      const int q = 2 * p + parity;
      for (int r = 0; r < nr; r++) {
        if (threadIdx.x == 0 && (p != p0 || r != 0)) {
          size_t i1 = (size_t)r * c.s.Q + q;
          rot_uniforms_t<MIX>(seed, ps, phase, p, r, linear, u);
          rot_propose_t<MIX>(c.s, linear, c.st.ang[i1], c.st.ang[n + i1], c.st.ang[2 * n + i1], u, prop);
        }
        int acc = rot_step<MIX, true>(c, frames, c.s.rot_first + r, q, u, prop, linear, sh, nullptr);
        tot++;
        nacc += acc;
      }
    }
    // the commits (warp 8) precede the barrier that ended the last move
    if (threadIdx.x == 0) {
      __threadfence();
      st_release_u64(prog + b, (id << 24) | (unsigned long long)(h + 1));
    }
  }
  if (threadIdx.x == 0) {
    int ty = c.s.imtype;
    atomicAdd(&cnt[(ty * 3 + 2) * 2 + 0], tot);
    atomicAdd(&cnt[(ty * 3 + 2) * 2 + 1], nacc);
  }
}

// ------------------------------------------------------------ centroid move
// MCMolecularMove (mc_piqmc.cc:54-102): replay as propose (the three rnd1()
// displacements), partner sums over all slices, accept/commit; production
// as partner sums (each CTA draws the displacement itself) and accept/commit
// on several CTAs (each takes the same decision from the same sums and
// commits its share of the slices).
template <bool REPLAY>
__global__ void k_mol_propose(Ctx c, int type, ReplaySrc src, uint64_t seed, const unsigned *pass, unsigned phase,
                              int atom, MolScratch *ms)
{
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (REPLAY) {
    for (int d = 0; d < 3; d++) ms->disp[d] = c.s.mcstep[type] * (src.disp_u(d) - 0.5);
  } else {
    mol_disp(c.s, type, seed, *pass, phase, atom, ms->disp);
  }
}

// CTA (partner atom1, slice chunk); threads over the chunk's slices; new =
// old + disp; both whole-path partial sums reduced in a fixed order
template <bool MIX, bool PROD>
__global__ void __launch_bounds__(PIMC_BLOCK) k_mol_pairs(Ctx c, Frame *frames, int type, int atom, int gatom,
                                                          MolScratch *ms, int nchunk, uint64_t seed,
                                                          const unsigned *pass, unsigned phase)
{
  __shared__ double part[2][PIMC_BLOCK / 32];
  __shared__ double dd[3];
  const int a1 = blockIdx.x, ch = blockIdx.y;
  const int tid = threadIdx.x;
  const int t0 = (int)((long)ch * c.s.P / nchunk), t1 = (int)((long)(ch + 1) * c.s.P / nchunk);
  if (tid == 0) {
    if (PROD) mol_disp(c.s, type, seed, *pass, phase, atom, dd);
    else { dd[0] = ms->disp[0]; dd[1] = ms->disp[1]; dd[2] = ms->disp[2]; }
  }
  __syncthreads();
  double an = 0.0, ao = 0.0;
  if (a1 != gatom) {
    const double d0 = dd[0], d1 = dd[1], d2 = dd[2];
    for (int it = t0 + tid; it < t1; it += blockDim.x) {
      size_t i = sidx(c.s, it, gatom);
      if (MIX) {
        const float4 p4 = c.st.b4[i];
        ao += (double)pair_term32(c, frames, gatom, a1, it, p4.x, p4.y, p4.z);
        an += (double)pair_term32(c, frames, gatom, a1, it, (float)(c.st.x[i] + d0), (float)(c.st.y[i] + d1),
                                  (float)(c.st.z[i] + d2));
      } else {
        double x = c.st.x[i], y = c.st.y[i], z = c.st.z[i];
        ao += pair_term64(c, frames, gatom, a1, it, x, y, z);
        an += pair_term64(c, frames, gatom, a1, it, x + d0, y + d1, z + d2);
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    an += __shfl_xor_sync(0xffffffffu, an, o);
    ao += __shfl_xor_sync(0xffffffffu, ao, o);
  }
  if ((tid & 31) == 0) { part[0][tid >> 5] = an; part[1][tid >> 5] = ao; }
  __syncthreads();
  if (tid < 2) {
    double s = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) s += part[tid][k];
    ms->pair[tid][a1 * nchunk + ch] = s;
  }
}

template <bool REPLAY>
__global__ void __launch_bounds__(PIMC_BLOCK) k_mol_finish(Ctx c, int type, int gatom, ReplaySrc src, uint64_t seed,
                                                            const unsigned *pass, unsigned phase, int atom,
                                                            MolScratch *ms, int nchunk, double *dv_out, int *acc_out,
                                                            unsigned long long *cnt)
{
  __shared__ int acc;
  __shared__ double sd[3];
  __shared__ double wpart[2][PIMC_BLOCK / 32];
  {
    // the partials in a fixed tree: thread strides, warp shuffles, warps in order
    const int np = c.s.na * nchunk;
    double en = 0.0, eo = 0.0;
    for (int i = threadIdx.x; i < np; i += blockDim.x)
      if (i / nchunk != gatom) { en += ms->pair[0][i]; eo += ms->pair[1][i]; }
    for (int o = 16; o > 0; o >>= 1) {
      en += __shfl_xor_sync(0xffffffffu, en, o);
      eo += __shfl_xor_sync(0xffffffffu, eo, o);
    }
    if ((threadIdx.x & 31) == 0) { wpart[0][threadIdx.x >> 5] = en; wpart[1][threadIdx.x >> 5] = eo; }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double en = 0.0, eo = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) { en += wpart[0][k]; eo += wpart[1][k]; }
    double deltav = 0.0;
    deltav += (en - eo);
    int a = 0;
    if (deltav < 0.0) a = 1;
    else {
      double u;
      if (REPLAY) u = src.accept_u(0);
      else {
        PhiloxSrc ps{seed, ((uint64_t)(*pass) << 32) | ((uint64_t)phase << 12) | (uint64_t)atom};
        u = ps.accept_u(7);
      }
      if (exp(-deltav * c.s.tau) > u) a = 1;
    }
    acc = a;
    if (REPLAY) { sd[0] = ms->disp[0]; sd[1] = ms->disp[1]; sd[2] = ms->disp[2]; }
    else mol_disp(c.s, type, seed, *pass, phase, atom, sd);
    if (blockIdx.x == 0) {
      if (dv_out) { dv_out[atom] = deltav; acc_out[atom] = a; }
      cnt[(type * 3 + 0) * 2 + 0] += 1;
      if (a) cnt[(type * 3 + 0) * 2 + 1] += 1;
    }
  }
  __syncthreads();
  if (acc) {
    const double d0 = sd[0], d1 = sd[1], d2 = sd[2];
    const int t0 = (int)((long)blockIdx.x * c.s.P / gridDim.x), t1 = (int)((long)(blockIdx.x + 1) * c.s.P / gridDim.x);
    for (int it = t0 + threadIdx.x; it < t1; it += blockDim.x) {
      size_t i = sidx(c.s, it, gatom);
      store_bead(c, i, c.st.x[i] + d0, c.st.y[i] + d1, c.st.z[i] + d2);
    }
    // the whole path moved: every cached rotor potential is stale
    if (blockIdx.x == 0)
      for (int i = threadIdx.x; i < c.s.nrotors * c.s.Q; i += blockDim.x) c.st.rp_ok[i] = 0;
  }
}

// ------------------------------------------------------------ energy queries
// PotEnergy(atom0, pos, it) for a batch of (atom0, it, position) queries
__global__ void __launch_bounds__(PIMC_BLOCK) k_q_slice(Ctx c, Frame *frames, int n, const int *a0, const int *it,
                                                         const double *xyz, double *out)
{
  __shared__ double buf[PIMC_RED_BUF];
  __shared__ int sa;
  __shared__ double so;
  int q = blockIdx.x;
  if (q >= n) return;
  if (threadIdx.x == 0) sa = a0[q];
  __syncthreads();
  int t = it[q];
  double px = xyz[3 * q], py = xyz[3 * q + 1], pz = xyz[3 * q + 2];
  slot_sums(1, c.s.na, &sa, [&](int, int p) -> double { return pair_term64(c, frames, sa, p, t, px, py, pz); }, &so,
            buf);
  if (threadIdx.x == 0) out[q] = so;
}

// PotRotE3D(rotor, Eulang, it) (theta given, not cos theta) or
// PotRotEnergy(rotor, n, it) for a batch
__global__ void __launch_bounds__(PIMC_BLOCK) k_q_rot(Ctx c, Frame *frames, int n, const int *rot, const int *it,
                                                       const double *v3, int linear, double *out)
{
  __shared__ double buf[PIMC_RED_BUF];
  __shared__ Frame f;
  __shared__ int sg;
  __shared__ double so;
  int q = blockIdx.x;
  if (q >= n) return;
  int t = it[q];
  if (threadIdx.x == 0) {
    sg = rot[q];
    if (!linear) {
      f.e[0] = v3[3 * q]; f.e[1] = v3[3 * q + 1]; f.e[2] = v3[3 * q + 2];
      matpre(f.e, f.m);
      double s = 0.0;
      s = s + f.m[2] * f.m[2];
      s = s + f.m[5] * f.m[5];
      s = s + f.m[8] * f.m[8];
      f.hz_norm = sqrt(s);
    }
  }
  __syncthreads();
  double nv[3] = {v3[3 * q], v3[3 * q + 1], v3[3 * q + 2]};
  int g0 = sg;
  slot_sums(1, c.s.na, &sg,
            [&](int, int p) -> double {
              return linear ? rotlin_term64(c, nv, g0, p, t) : rot3d_term64(c, frames, f, g0, p, t);
            },
            &so, buf);
  if (threadIdx.x == 0) out[q] = so;
}

// ------------------------------------------------------------ estimators
// GetKinEnergy (mc_estim.cc:876-937): per-atom sum of |r_t - r_t+1|^2 with
// the boson wrap through pindex; one CTA per atom, out[atom] = sum / (4 beta lambda)
__global__ void __launch_bounds__(PIMC_BLOCK) k_est_kin(Ctx c, double *out)
{
  __shared__ double part[PIMC_BLOCK];
  int a = blockIdx.x, P = c.s.P;
  int type = atom_type(c.s, a);
  double acc = 0.0;
  for (int it = threadIdx.x; it < P; it += blockDim.x) acc += est_spring(c, a, it);
  part[threadIdx.x] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int k = 0; k < (int)blockDim.x; k++) s += part[k];
    out[a] = s / (4.0 * c.s.beta * c.s.lambda[type]);
  }
}

// GetPotEnergy_Densities (mc_estim.cc:500-687) value: CTA per pair (a0 < a1),
// threads over slices; out[pair]
__global__ void __launch_bounds__(PIMC_BLOCK) k_est_pot(Ctx c, Frame *frames, double *out)
{
  __shared__ double part[PIMC_BLOCK];
  int na = c.s.na;
  int pidx = blockIdx.x;
  // unrank pidx -> (a0, a1) in the reference's double-loop order
  int a0 = 0, rem = pidx;
  while (rem >= na - 1 - a0) { rem -= na - 1 - a0; a0++; }
  int a1 = a0 + 1 + rem;
  double acc = 0.0;
  if (est_pair_counted(c, a0, a1))
    for (int it = threadIdx.x; it < c.s.P; it += blockDim.x) {
      size_t i = sidx(c.s, it, a0);
      acc += pair_term64(c, frames, a0, a1, it, c.st.x[i], c.st.y[i], c.st.z[i]);
    }
  part[threadIdx.x] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int k = 0; k < (int)blockDim.x; k++) s += part[k];
    out[pidx] = s;
  }
}

// per (rotor, it0) link terms: out[4*k + {srot, sesq, se_termsq, valid}]
__global__ void k_est_rot(Ctx c, Frame *frames, double *out)
{
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= c.s.nrotors * c.s.Q) return;
  est_link(c, frames, k, out + 4 * (size_t)k);
}

// GetRCF (mc_estim.cc:1099-1139) row 0: rcf[itc] = sum_it0 n(it0).n(it0+itc)
__global__ void k_est_rcf(Ctx c, double *rcf)
{
  int Q = c.s.Q;
  int itc = blockIdx.x * blockDim.x + threadIdx.x;
  if (itc >= Q) return;
  size_t n = (size_t)c.s.nrotors * Q;
  double s = 0.0;
  for (int it0 = 0; it0 < Q; it0++) {
    int t0 = it0, tc = (it0 + itc) % Q;
    double p0 = 0.0;
    for (int d = 0; d < 3; d++) p0 += (c.st.cosv[d * n + t0] * c.st.cosv[d * n + tc]);
    s += p0;
  }
  rcf[itc] = s;
}

// ------------------------------------------------------------ densities
// bin_1Ddensity / bin_2Ddensity / bin_3Ddensity (mc_estim.cc:1233-1286) on
// the grids of densities_init (mc_estim.cc:223-255): the same divisions and
// floors as the reference, counts kept as 64-bit integers indexed
// [dtype][bins] like _gr1D/_gr2D/_gr3D
__device__ __forceinline__ void dens_bin(const DensHist &hs, int kind, int dtype, double r, double a, double b)
{
  const double drad = (PIMC_DENS_MAX_RADIUS - PIMC_DENS_MIN_RADIUS) / (double)PIMC_BINSR;
  const double dth = PIMC_PI / (double)(PIMC_BINST - 1), dch = 2.0 * PIMC_PI / (double)(PIMC_BINSC - 1);
  int br = (int)floor((r - PIMC_DENS_MIN_RADIUS) / drad);
  if (!(br < PIMC_BINSR && br >= 0)) return;
  if (kind == 1) {
    atomicAdd(hs.g1 + (size_t)dtype * PIMC_BINSR + br, 1ull);
  } else if (kind == 2) {
    int bt = (int)floor(acos(a) / dth);
    if (bt < PIMC_BINST && bt >= 0) atomicAdd(hs.g2 + ((size_t)dtype * PIMC_BINSR + br) * PIMC_BINST + bt, 1ull);
  } else if (hs.g3) {
    int bt = (int)floor(a / dth);
    if (bt < PIMC_BINST && bt >= 0) {
      int bc = (int)floor(b / dch);
      if (bc < PIMC_BINSC && bc >= 0)
        atomicAdd(hs.g3 + (size_t)dtype * PIMC_BINSR * PIMC_BINST * PIMC_BINSC +
                      ((size_t)br * PIMC_BINST + bt) * PIMC_BINSC + bc,
                  1ull);
    }
  }
}

// the geometry GetPotEnergy_Densities (mc_estim.cc:520-662) bins for the
// pair (a0 < a1) at slice it: r for atoms of one type, (r, n.dr/r) for a
// linear rotor and an atom, vcord's (r, theta, chi) (or vspher's r) for a
// nonlinear rotor and an atom; rotor pairs are not binned
__device__ void est_pair_bin(const Ctx &c, const Frame *frames, const DensHist &hs, int a0, int a1, int it)
{
  const DevSys &s = c.s;
  int ty0 = atom_type(s, a0), ty1 = atom_type(s, a1);
  int m0 = s.molecule[ty0], m1 = s.molecule[ty1];
  size_t i0 = sidx(s, it, a0), i1 = sidx(s, it, a1);
  double px = c.st.x[i0], py = c.st.y[i0], pz = c.st.z[i0];
  double qx = c.st.x[i1], qy = c.st.y[i1], qz = c.st.z[i1];
  double dx = px - qx, dy = py - qy, dz = pz - qz;
  if (s.minimage) {
    dx -= s.box[0] * rint(dx / s.box[0]);
    dy -= s.box[1] * rint(dy / s.box[1]);
    dz -= s.box[2] * rint(dz / s.box[2]);
  }
  double dr2 = 0.0;
  dr2 += dx * dx;
  dr2 += dy * dy;
  dr2 += dz * dz;
  double r = sqrt(dr2);
  if (m0 == 1 || m1 == 1) {
    int rot = (m0 == 1) ? a0 : a1;
    size_t n = (size_t)s.nrotors * s.Q;
    int ri = rot_index(s, rot, it / s.R);
    double cost = 0.0;
    cost += c.st.cosv[ri] * dx;
    cost += c.st.cosv[n + ri] * dy;
    cost += c.st.cosv[2 * n + ri] * dz;
    cost /= r;
    if (m0 == 1) cost *= -1.0;
    dens_bin(hs, 2, m0 == 1 ? ty1 : ty0, r, cost, 0.0);
  } else if ((m0 == 2 || m1 == 2) && m0 != m1) {
    double rr = r, th = 0.0, ch = 0.0;
    if (!s.ispher) {
      if (m0 == 2) vcord(c.t, frames[rot_index(s, a0, it / s.R)], px, py, pz, qx, qy, qz, &rr, &th, &ch);
      else vcord(c.t, frames[rot_index(s, a1, it / s.R)], qx, qy, qz, px, py, pz, &rr, &th, &ch);
    }
    dens_bin(hs, 3, m0 == 2 ? ty1 : ty0, rr, th, ch);
  } else if (!(m0 == 2 && m1 == 2) && ty0 == ty1 && m0 == 0) {
    dens_bin(hs, 1, ty1, r, 0.0, 0.0);
  }
}

// all pairs x slices of one configuration, one thread per (pair, slice)
__global__ void k_est_dens(Ctx c, Frame *frames, DensHist hs)
{
  int na = c.s.na, P = c.s.P;
  long npairs = (long)na * (na - 1) / 2;
  for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < npairs * P; k += (long)gridDim.x * blockDim.x) {
    int pidx = (int)(k / P), it = (int)(k % P);
    int a0 = 0, rem = pidx;
    while (rem >= na - 1 - a0) { rem -= na - 1 - a0; a0++; }
    est_pair_bin(c, frames, hs, a0, a0 + 1 + rem, it);
  }
}

// GetRotE3D's binning of the relative Euler angles of slices it0 and
// it0 + skip (mc_estim.cc:1023-1057): floor(angle / bin width), each in-range
// bin counted skip times (RNskip: 1, or RNratio for rattle-and-shake)
__global__ void k_est_releuler(Ctx c, const Frame *frames, unsigned long long *rel)
{
  const int Q = c.s.Q, skip = (c.s.rot_den_type == 0) ? 1 : c.s.rn_ratio;
  const double dth = PIMC_PI / (double)(PIMC_BINST - 1), dch = 2.0 * PIMC_PI / (double)(PIMC_BINSC - 1);
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < c.s.nrotors * Q; k += gridDim.x * blockDim.x) {
    const int r = k / Q, it0 = k % Q;
    if (it0 % skip) continue;
    double e[3];
    deleul(frames[r * Q + it0].m, frames[r * Q + (it0 + skip) % Q].m, e);
    const int bt = (int)floor(e[1] / dth), bp = (int)floor(e[0] / dch), bc = (int)floor(e[2] / dch);
    if (bt < PIMC_BINST && bt >= 0) atomicAdd(rel + bt, (unsigned long long)skip);
    if (bp < PIMC_BINSC && bp >= 0) atomicAdd(rel + PIMC_BINST + bp, (unsigned long long)skip);
    if (bc < PIMC_BINSC && bc >= 0) atomicAdd(rel + PIMC_BINST + PIMC_BINSC + bc, (unsigned long long)skip);
  }
}

// ------------------------------------------------------ area estimators
// GetAreaEstimators (mc_estim.cc:2087-2250, mode 0) and GetAreaEstim3D
// (mc_estim.cc:2252-2594; mode 1 space-fixed frame about the mass-weighted
// centre of all atoms, mode 2 dopant-fixed frame about the first rotor).
// Items (it0, boson) are summed per CTA in a fixed tree; out[blockIdx*12 +
// k] are the CTA's partial sums: mode 0 {area_perp, area_parl, inert_perp,
// inert_parl}, modes 1/2 {area_proj[3], inert3D[9]} (unscaled).
template <int MODE>
__global__ void __launch_bounds__(PIMC_BLOCK) k_est_area(Ctx c, int btype, double m0, double m1, double *out)
{
  __shared__ double red[PIMC_BLOCK];
  const DevSys &s = c.s;
  const int P = s.P, nbos = s.numb[btype], g = s.first[btype];
  const long nitem = (long)nbos * P;
  const double bmass = btype == 0 ? m0 : m1;
  double acc[12];
#pragma unroll
  for (int k = 0; k < 12; k++) acc[k] = 0.0;
  auto com = [&](int it, double v[3]) {
    if (MODE == 1) {
      double tmass = 0.0, sx = 0.0, sy = 0.0, sz = 0.0;
      for (int a = 0; a < s.na; a++) {
        double m = atom_type(s, a) == 0 ? m0 : m1;
        size_t i = sidx(s, it, a);
        sx += (m * c.st.x[i]);
        sy += (m * c.st.y[i]);
        sz += (m * c.st.z[i]);
        tmass += m;
      }
      v[0] = sx / tmass; v[1] = sy / tmass; v[2] = sz / tmass;
    } else {
      size_t i = sidx(s, it, s.rot_first);
      v[0] = c.st.x[i]; v[1] = c.st.y[i]; v[2] = c.st.z[i];
    }
  };
  for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < nitem; k += (long)gridDim.x * blockDim.x) {
    int it0 = (int)(k / nbos), atom = (int)(k % nbos);
    int it1 = (it0 + 1) % P;
    int a1 = (it1 != it0 + 1) ? g + c.st.pindex[atom] : g + atom;
    double c0[3], c1[3];
    com(it0, c0);
    com(it1, c1);
    size_t i0 = sidx(s, it0, g + atom), i1 = sidx(s, it1, a1);
    double dr0[3] = {c.st.x[i0] - c0[0], c.st.y[i0] - c0[1], c.st.z[i0] - c0[2]};
    double dr1[3] = {c.st.x[i1] - c1[0], c.st.y[i1] - c1[1], c.st.z[i1] - c1[2]};
    double area[3];
    area[0] = 0.5 * (dr0[1] * dr1[2] - dr0[2] * dr1[1]);
    area[1] = 0.5 * (dr0[2] * dr1[0] - dr0[0] * dr1[2]);
    area[2] = 0.5 * (dr0[0] * dr1[1] - dr0[1] * dr1[0]);
    if (MODE == 0) {
      size_t n = (size_t)s.nrotors * s.Q;
      int ri = rot_index(s, s.rot_first, it0 / s.R);
      double nl[3] = {c.st.cosv[ri], c.st.cosv[n + ri], c.st.cosv[2 * n + ri]};
      double tg = 0.0, st = 1.0;
      if (fabs(nl[0]) > 10e-4) {
        tg = nl[1] / nl[0];
        st = sqrt(1.0 + tg * tg);
      }
      double np[3] = {tg / st, -1.0 / st, 0.0};
      acc[0] += np[0] * area[0] + np[1] * area[1] + np[2] * area[2];
      acc[1] += nl[0] * area[0] + nl[1] * area[1] + nl[2] * area[2];
      const double *nv[2] = {np, nl};
#pragma unroll
      for (int w = 0; w < 2; w++) {
        const double *u = nv[w];
        double r0[3] = {u[1] * dr0[2] - u[2] * dr0[1], u[2] * dr0[0] - u[0] * dr0[2], u[0] * dr0[1] - u[1] * dr0[0]};
        double r1[3] = {u[1] * dr1[2] - u[2] * dr1[1], u[2] * dr1[0] - u[0] * dr1[2], u[0] * dr1[1] - u[1] * dr1[0]};
        acc[2 + w] += r0[0] * r1[0] + r0[1] * r1[1] + r0[2] * r1[2];
      }
    } else {
      double hat[3][3];
      if (MODE == 1) {
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
          for (int j = 0; j < 3; j++) hat[i][j] = (i == j) ? 1.0 : 0.0;
      } else {
        int ri = rot_index(s, s.rot_first, it0 / s.R);
        size_t n = (size_t)s.nrotors * s.Q;
        Frame f;
        make_frame64(c.st.ang[ri], c.st.ang[n + ri], c.st.ang[2 * n + ri], f);
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
          for (int d = 0; d < 3; d++) hat[i][d] = f.m[d * 3 + i];
      }
      double pr0[3], pr1[3];
#pragma unroll
      for (int i = 0; i < 3; i++) {
        acc[i] += area[0] * hat[i][0] + area[1] * hat[i][1] + area[2] * hat[i][2];
        pr0[i] = hat[i][0] * dr0[0] + hat[i][1] * dr0[1] + hat[i][2] * dr0[2];
        pr1[i] = hat[i][0] * dr1[0] + hat[i][1] * dr1[1] + hat[i][2] * dr1[2];
      }
#pragma unroll
      for (int i = 0; i < 3; i++) {
        const double *h = hat[i];
        double r0[3] = {dr0[1] * h[2] - dr0[2] * h[1], dr0[2] * h[0] - dr0[0] * h[2], dr0[0] * h[1] - dr0[1] * h[0]};
        double r1[3] = {dr1[1] * h[2] - dr1[2] * h[1], dr1[2] * h[0] - dr1[0] * h[2], dr1[0] * h[1] - dr1[1] * h[0]};
        acc[3 + 3 * i + i] += (r0[0] * r1[0] + r0[1] * r1[1] + r0[2] * r1[2]) * bmass;
#pragma unroll
        for (int j = 0; j < 3; j++)
          if (j != i) acc[3 + 3 * i + j] += -bmass * pr0[i] * pr1[j];
      }
    }
  }
  const int nv = MODE == 0 ? 4 : 12;
  for (int k = 0; k < nv; k++) {
    red[threadIdx.x] = acc[k];
    __syncthreads();
    for (int w = PIMC_BLOCK / 2; w > 0; w >>= 1) {
      if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
      __syncthreads();
    }
    if (threadIdx.x == 0) out[(size_t)blockIdx.x * 12 + k] = red[0];
    __syncthreads();
  }
}

// ------------------------------------------------------------ bookkeeping
__global__ void k_pass_begin(unsigned *pass) { *pass += 1; }

// ------------------------------------------------------------ launchers
// the double-precision frames and MCCosine of nonlinear rotors from their
// angles (what the rotational commits leave to be derived, see rot_step);
// the float frames are kept as the moves evaluated them
__global__ void k_refresh_frames(Ctx c, Frame *frames, int frames64)
{
  if (c.s.nrotors <= 0) return;
  size_t n = (size_t)c.s.nrotors * c.s.Q;
  if (c.s.molecule[c.s.imtype] == 1) {
    // a linear rotor on the FP32 path: the double MCCosine from the angles
    if (!lazy_linear(c, c.s.mixed != 0)) return;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
      double v[3];
      unit_vector(c.st.ang[i], c.st.ang[n + i], v);
      for (int d = 0; d < 3; d++) c.st.cosv[d * n + i] = v[d];
    }
    return;
  }
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    double phi = c.st.ang[i], cost = c.st.ang[n + i], chi = c.st.ang[2 * n + i];
    if (frames64) make_frame64(phi, cost, chi, frames[i]);
    double v[3];
    unit_vector(phi, cost, v);
    for (int d = 0; d < 3; d++) {
      c.st.cosv[d * n + i] = v[d];
      c.st.cosvf[d * n + i] = (float)v[d];
    }
  }
}

void launch_refresh_frames(const Ctx &c, Frame *frames, cudaStream_t s)
{
  size_t n = (size_t)c.s.nrotors * c.s.Q;
  int nb = (int)((n + 255) / 256);
  if (nb < 1) nb = 1;
  if (nb > 152) nb = 152;
  k_refresh_frames<<<nb, 256, 0, s>>>(c, frames, c.s.mixed);
}

void launch_derive_state(const Ctx &c, Frame *frames, cudaStream_t s)
{
  k_derive_state<<<152, 256, 0, s>>>(c, frames);
}

void launch_invalidate_caches(const Ctx &c, cudaStream_t s)
{
  int n = c.s.nrotors * c.s.Q;
  if (n > 0) k_invalidate_caches<<<(n + 255) / 256, 256, 0, s>>>(c);
}

void launch_bisect_replay(const Ctx &c, Frame *f, int type, int time0, int exch, ReplaySrc src, double *ds,
                          int *lvl, unsigned long long *cnt, cudaStream_t s)
{
  if (c.s.mixed) k_bisect_replay<true><<<1, PIMC_BIS_THREADS, 0, s>>>(c, f, type, time0, exch, src, ds, lvl, cnt);
  else k_bisect_replay<false><<<1, PIMC_BIS_THREADS, 0, s>>>(c, f, type, time0, exch, src, ds, lvl, cnt);
}

void launch_bisect_phase(const Ctx &c, Frame *f, int type, int s0, int j, unsigned phase, uint64_t seed,
                         const unsigned *pass, unsigned long long *cnt, cudaStream_t s)
{
  int M = 1 << c.s.levels[type];
  if (c.s.mixed) k_bisect_phase<true><<<c.s.P / M, PIMC_BIS_THREADS, 0, s>>>(c, f, type, s0, j, phase, seed, pass, cnt);
  else k_bisect_phase<false><<<c.s.P / M, PIMC_BIS_THREADS, 0, s>>>(c, f, type, s0, j, phase, seed, pass, cnt);
}

// nhalf half-sweeps with one CTA per rotational slice (one rotor, Q even,
// all Q CTAs resident).  Slice q moves in the half-sweeps of its parity;
// its move at h waits for both neighbours to have finished h-1, and its
// next move is prepared (proposal, frame, partner sums: nothing a
// neighbour writes) while they move.  The same uniforms and the same
// states as the launch-per-half-sweep schedule: identical results.
template <bool MIX>
__global__ void __launch_bounds__(PIMC_ROT_THREADS) k_rot_slices(Ctx c, Frame *frames, int nhalf, unsigned phase0,
                                                                 unsigned group, uint64_t seed, const unsigned *pass,
                                                                 unsigned long long *prog, unsigned *abort_word,
                                                                 unsigned long long *cnt)
{
  __shared__ RotShared sh;
  // CTAs [0, Q/2) take the even slices and [Q/2, Q) the odd ones, so that
  // two CTAs sharing an SM (blocks b and b + #SMs) mostly have opposite
  // parity: one prepares while the other finishes
  const int Q = c.s.Q, half = Q >> 1, b = blockIdx.x;
  const int q = (b < half) ? 2 * b : 2 * (b - half) + 1;
  const bool linear = c.s.molecule[c.s.imtype] == 1;
  const unsigned ps = *pass;
  const size_t n = (size_t)Q;
  const int g0 = c.s.rot_first;
  RotSliceHooks hk;
  hk.wl = prog + (q + Q - 1) % Q;
  hk.wr = prog + (q + 1) % Q;
  hk.mine = prog + q;
  hk.id = ((unsigned long long)ps << 8) | (group & 255u);
  hk.abort_word = abort_word;
  hk.err = c.st.err;
  hk.sys = &c.s;
  hk.seed = seed;
  hk.pass = ps;
  hk.pair = q >> 1;
  hk.linear = linear;
  hk.mixed = MIX;
  unsigned long long tot = 0, nacc = 0;
  double u[4] = {0.5, 0.5, 0.5, 0.5}, prop[3] = {0.0, 0.0, 0.0};
  int h = q & 1;
  if (h < nhalf) {
    if (threadIdx.x == 0) {
      rot_uniforms_t<MIX>(seed, ps, phase0 + (unsigned)h, q >> 1, 0, linear, u);
      rot_propose_t<MIX>(c.s, linear, c.st.ang[q], c.st.ang[n + q], c.st.ang[2 * n + q], u, prop);
    }
    rot_prepare<MIX>(c, frames, g0, q, u, prop, linear, sh);
  }
  for (; h < nhalf; h += 2) {
    hk.h = h;
    hk.has_next = h + 2 < nhalf;
    hk.phase_next = phase0 + (unsigned)(h + 2);
    int acc = rot_finish<MIX, true>(c, frames, g0, q, linear, sh, nullptr, hk);
    if (sh.stop) break;
    tot++;
    nacc += acc;
    if (h + 2 < nhalf) {
      if (threadIdx.x == 0) {
        for (int k = 0; k < 4; k++) u[k] = sh.nxt_u[k];
        for (int k = 0; k < 3; k++) prop[k] = sh.nxt_prop[acc ? 1 : 0][k];
      }
      rot_prepare<MIX>(c, frames, g0, q, u, prop, linear, sh, MIX ? -1 : (acc ? 1 : 0));
    }
  }
  if (threadIdx.x == 0) {
    int ty = c.s.imtype;
    atomicAdd(&cnt[(ty * 3 + 2) * 2 + 0], tot);
    atomicAdd(&cnt[(ty * 3 + 2) * 2 + 1], nacc);
  }
}

// the slices of one half of a sweep as independent sets: with Q odd the
// last even slice neighbours slice 0 and runs after the other even slices,
// as in the serial loop
template <class F>
static void rot_sets(int Q, int parity, F launch)
{
  if (parity == 0) {
    if (Q % 2 == 1 && Q >= 3) {
      launch(0, (Q - 1) / 2);
      launch(Q - 1, 1);
    } else {
      launch(0, (Q + 1) / 2);
    }
  } else {
    if (Q / 2 > 0) launch(1, Q / 2);
  }
}

void launch_rot_replay(const Ctx &c, Frame *f, int parity, const double *urot, long nurot, double *rd, int *acc,
                       unsigned long long *cnt, cudaStream_t s)
{
  rot_sets(c.s.Q, parity, [&](int q0, int nq) {
    if (c.s.mixed)
      k_rot<true, true><<<nq, PIMC_ROT_THREADS, 0, s>>>(c, f, q0, nq, urot, nurot, 0, 0, nullptr, rd, acc, cnt);
    else
      k_rot<true, false><<<nq, PIMC_ROT_THREADS, 0, s>>>(c, f, q0, nq, urot, nurot, 0, 0, nullptr, rd, acc, cnt);
  });
}

int launch_rot_phase(const Ctx &c, Frame *f, int parity, unsigned phase, uint64_t seed, const unsigned *pass,
                     unsigned long long *cnt, cudaStream_t s)
{
  int n = 0;
  rot_sets(c.s.Q, parity, [&](int q0, int nq) {
    if (c.s.mixed)
      k_rot<false, true><<<nq, PIMC_ROT_THREADS, 0, s>>>(c, f, q0, nq, nullptr, 0, phase, seed, pass, nullptr, nullptr,
                                                         cnt);
    else
      k_rot<false, false><<<nq, PIMC_ROT_THREADS, 0, s>>>(c, f, q0, nq, nullptr, 0, phase, seed, pass, nullptr,
                                                          nullptr, cnt);
    n++;
  });
  return n;
}

int rot_slices_max_ctas(int mixed)
{
  int dev = 0, nsm = 0, per = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
  cudaError_t e = mixed ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_rot_slices<true>, PIMC_ROT_THREADS, 0)
                        : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_rot_slices<false>, PIMC_ROT_THREADS, 0);
  if (e != cudaSuccess) return 0;
  return nsm * per;
}

cudaError_t launch_rot_slices(const Ctx &c, Frame *f, int nhalf, unsigned phase0, unsigned group, uint64_t seed,
                              const unsigned *pass, unsigned long long *prog, unsigned *abort_word,
                              unsigned long long *cnt, cudaStream_t s)
{
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(c.s.Q);
  cfg.blockDim = dim3(PIMC_ROT_THREADS);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (c.s.mixed)
    return cudaLaunchKernelEx(&cfg, k_rot_slices<true>, c, f, nhalf, phase0, group, seed, pass, prog, abort_word, cnt);
  return cudaLaunchKernelEx(&cfg, k_rot_slices<false>, c, f, nhalf, phase0, group, seed, pass, prog, abort_word, cnt);
}

int rot_sweeps_max_ctas(int mixed)
{
  int dev = 0, nsm = 0, per = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
  cudaError_t e = mixed ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_rot_sweeps<true>, PIMC_ROT_THREADS, 0)
                        : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_rot_sweeps<false>, PIMC_ROT_THREADS, 0);
  if (e != cudaSuccess) return 0;
  return nsm * per;
}

cudaError_t launch_rot_sweeps(const Ctx &c, Frame *f, int nctas, int nhalf, unsigned phase0, unsigned group,
                              uint64_t seed, const unsigned *pass, unsigned long long *prog, unsigned *abort_word,
                              unsigned long long *cnt, cudaStream_t s)
{
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(nctas);
  cfg.blockDim = dim3(PIMC_ROT_THREADS);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (c.s.mixed)
    return cudaLaunchKernelEx(&cfg, k_rot_sweeps<true>, c, f, nhalf, phase0, group, seed, pass, prog, abort_word, cnt);
  return cudaLaunchKernelEx(&cfg, k_rot_sweeps<false>, c, f, nhalf, phase0, group, seed, pass, prog, abort_word, cnt);
}

void launch_bisect_block(const Ctx &c, Frame *f, int type, int s0, unsigned phase0, uint64_t seed,
                         const unsigned *pass, unsigned long long *cnt, cudaStream_t s)
{
  int M = 1 << c.s.levels[type];
  int nwin = c.s.P / M;
  if (c.s.mixed) k_bisect_block<true><<<nwin, PIMC_BIS_THREADS, 0, s>>>(c, f, type, s0, phase0, seed, pass, cnt);
  else k_bisect_block<false><<<nwin, PIMC_BIS_THREADS, 0, s>>>(c, f, type, s0, phase0, seed, pass, cnt);
}

int launch_mol(const Ctx &c, Frame *f, int type, int atom, bool replay, ReplaySrc src, uint64_t seed,
               const unsigned *pass, unsigned phase, MolScratch *ms, double *dv, int *acc, unsigned long long *cnt,
               cudaStream_t s)
{
  int g = c.s.first[type] + atom;
  // slice chunks per partner: about two CTAs per SM over all partners
  int nchunk = (2 * 152 + c.s.na - 1) / c.s.na;
  if (nchunk > PIMC_MOL_MAXCHUNK) nchunk = PIMC_MOL_MAXCHUNK;
  if (nchunk > c.s.P / 32) nchunk = c.s.P / 32;
  if (nchunk < 1) nchunk = 1;
  dim3 grid(c.s.na, nchunk);
  if (replay) {
    k_mol_propose<true><<<1, 32, 0, s>>>(c, type, src, seed, pass, phase, atom, ms);
    if (c.s.mixed) k_mol_pairs<true, false><<<grid, PIMC_BLOCK, 0, s>>>(c, f, type, atom, g, ms, nchunk, seed, pass, phase);
    else k_mol_pairs<false, false><<<grid, PIMC_BLOCK, 0, s>>>(c, f, type, atom, g, ms, nchunk, seed, pass, phase);
    k_mol_finish<true><<<1, PIMC_BLOCK, 0, s>>>(c, type, g, src, seed, pass, phase, atom, ms, nchunk, dv, acc, cnt);
    return 3;
  }
  if (c.s.mixed) k_mol_pairs<true, true><<<grid, PIMC_BLOCK, 0, s>>>(c, f, type, atom, g, ms, nchunk, seed, pass, phase);
  else k_mol_pairs<false, true><<<grid, PIMC_BLOCK, 0, s>>>(c, f, type, atom, g, ms, nchunk, seed, pass, phase);
  int nfin = c.s.P / 256;
  if (nfin < 1) nfin = 1;
  if (nfin > 8) nfin = 8;
  k_mol_finish<false><<<nfin, PIMC_BLOCK, 0, s>>>(c, type, g, src, seed, pass, phase, atom, ms, nchunk, dv, acc, cnt);
  return 2;
}

void launch_q_slice(const Ctx &c, Frame *f, int n, const int *a0, const int *it, const double *xyz, double *out,
                    cudaStream_t s)
{
  if (n > 0) k_q_slice<<<n, PIMC_BLOCK, 0, s>>>(c, f, n, a0, it, xyz, out);
}

void launch_q_rot(const Ctx &c, Frame *f, int n, const int *rot, const int *it, const double *v3, int linear,
                  double *out, cudaStream_t s)
{
  if (n > 0) k_q_rot<<<n, PIMC_BLOCK, 0, s>>>(c, f, n, rot, it, v3, linear, out);
}

void launch_est(const Ctx &c, Frame *f, double *kin, double *pot, double *rot, double *rcf, cudaStream_t s)
{
  k_est_kin<<<c.s.na, PIMC_BLOCK, 0, s>>>(c, kin);
  int npairs = c.s.na * (c.s.na - 1) / 2;
  if (npairs > 0) k_est_pot<<<npairs, PIMC_BLOCK, 0, s>>>(c, f, pot);
  int nk = c.s.nrotors * c.s.Q;
  if (nk > 0) {
    k_est_rot<<<(nk + 127) / 128, 128, 0, s>>>(c, f, rot);
    k_est_rcf<<<(c.s.Q + 127) / 128, 128, 0, s>>>(c, rcf);
  }
}

void launch_pass_begin(unsigned *pass, cudaStream_t s) { k_pass_begin<<<1, 1, 0, s>>>(pass); }

int launch_est_dens(const Ctx &c, Frame *f, DensHist hs, cudaStream_t s)
{
  long work = (long)c.s.na * (c.s.na - 1) / 2 * c.s.P;
  if (work <= 0) return 0;
  long nb = (work + 255) / 256;
  k_est_dens<<<(int)(nb < 4096 ? nb : 4096), 256, 0, s>>>(c, f, hs);
  if (hs.rel) {
    k_est_releuler<<<(c.s.nrotors * c.s.Q + 127) / 128, 128, 0, s>>>(c, f, hs.rel);
    return 2;
  }
  return 1;
}

int est_area_ctas(const Ctx &c, int btype)
{
  long items = (long)c.s.numb[btype] * c.s.P;
  long nb = (items + PIMC_BLOCK - 1) / PIMC_BLOCK;
  return (int)(nb < 304 ? (nb > 0 ? nb : 1) : 304);
}

int launch_est_area(const Ctx &c, int mode, int btype, const double *mass, double *out, cudaStream_t s)
{
  int nb = est_area_ctas(c, btype);
  double m0 = mass ? mass[0] : 1.0, m1 = mass ? mass[1] : 1.0;
  if (mode == 0) k_est_area<0><<<nb, PIMC_BLOCK, 0, s>>>(c, btype, m0, m1, out);
  else if (mode == 1) k_est_area<1><<<nb, PIMC_BLOCK, 0, s>>>(c, btype, m0, m1, out);
  else k_est_area<2><<<nb, PIMC_BLOCK, 0, s>>>(c, btype, m0, m1, out);
  return nb;
}

size_t mol_scratch_bytes() { return sizeof(MolScratch); }
