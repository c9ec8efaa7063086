// pimc_batch.cu -- many independent small systems ("replicas") sampled in one
// persistent launch.  A CTA takes replicas from a work queue (largest first)
// and runs the production pass of each in the same order, with the same
// uniforms, as the single-system sampler: the centroid moves on the whole
// CTA, then per bisection block one warp per window (a window's N moves in
// turn, no CTA barrier inside a block), then the block's rotational sweeps
// with one warp per slice of a half-sweep.  The warps' partner sums use a
// per-warp item buffer; each slot is summed by one lane in item order.
#include "pimc_kernels.cuh"
#include "pimc_launch.h"

#define PIMC_BATCH_BUF 256            /* doubles in a warp's item buffer */

struct WarpBis {
  double gz[3 * PIMC_BATCH_MAX_SEG];
  double ua[4], lu[4], dv[4];
  double ob[3][PIMC_BATCH_MAX_SEG + 1], nb[3][PIMC_BATCH_MAX_SEG + 1];
  float4 bf[2][PIMC_BATCH_MAX_SEG + 1];
  double se[2 * PIMC_BATCH_MAX_SEG];
  int slice[PIMC_BATCH_MAX_SEG + 1];
};

struct WarpRot {
  Frame fo[3], fn;
  double ang_new[3], nv[3][3], nnew[3];
  float nvf[3], nnewf[3], nvf0[3], nvf2[3];
  double vals[2 * 16];
  double rho[4], pot_c;
  int bad, pot_cached, link_ok[2];
};

struct __align__(16) WarpMem {
  union {
    WarpBis b;
    WarpRot r;
  } u;
  double buf[PIMC_BATCH_BUF];
};

// out[s] = sum over partners p != skip of f(s, p), s < nslots, on one warp:
// the items in the warp's buffer, then lane s sums slot s in item order
template <class F>
__device__ __forceinline__ void warp_slot_sums(int lane, int nslots, int npart, int skip, F f, double *out,
                                               double *bufd)
{
  using T = decltype(f(0, 0));
  T *buf = reinterpret_cast<T *>(bufd);
  const int cap = PIMC_BATCH_BUF * (int)(sizeof(double) / sizeof(T));
  if (npart <= 0) {
    for (int s = lane; s < nslots; s += 32) out[s] = 0.0;
    __syncwarp();
    return;
  }
  const int total = nslots * npart;
  const int chunk = (npart <= cap) ? (cap / npart) * npart : cap;
  for (int base = 0; base < total; base += chunk) {
    const int cnt = min(chunk, total - base);
    for (int i = lane; i < cnt; i += 32) {
      int g = base + i;
      int s = g / npart, pi = g - s * npart;
      buf[i] = f(s, pi < skip ? pi : pi + 1);
    }
    __syncwarp();
    const int sfirst = base / npart, slast = (base + cnt - 1) / npart;
    for (int sl = sfirst + lane; sl <= slast; sl += 32) {
      int lo = max(sl * npart, base) - base, hi = min((sl + 1) * npart, base + cnt) - base;
      T acc = T(0);
      for (int k = lo; k < hi; k++) acc += buf[k];
      if (sl * npart >= base) out[sl] = (double)acc;
      else out[sl] += (double)acc;
    }
    __syncwarp();
  }
}

// bisect_move (production form) on one warp
template <bool MIX>
__device__ int warp_bisect(const Ctx &c, const Frame *frames, int type, int atom, int time0, PhiloxSrc &src,
                           WarpBis &w, double *buf, int lane)
{
  const DevSys &s = c.s;
  const int P = s.P, L = s.levels[type], M = 1 << L;
  const int g0 = s.first[type] + atom;
  for (int k = lane; k <= M; k += 32) {
    int pt = (time0 + k) % P;
    w.slice[k] = pt;
    size_t i = sidx(s, pt, g0);
    double x = c.st.x[i], y = c.st.y[i], z = c.st.z[i];
    w.nb[0][k] = x; w.nb[1][k] = y; w.nb[2][k] = z;
    w.ob[0][k] = x; w.ob[1][k] = y; w.ob[2][k] = z;
    if (MIX) w.bf[1][k] = c.st.b4[i];
  }
  for (int i = lane; i < 3 * (M - 1); i += 32) {
    int l = 31 - __clz(i / 3 + 1);
    int off = i - 3 * ((1 << l) - 1);
    if (MIX) w.gz[i] = src.gauss_at32(l, off / 3, off - 3 * (off / 3));
    else w.gz[i] = src.gauss_pre(0, i, l, off / 3, off - 3 * (off / 3));
  }
  if (lane < L) {
    if (MIX) {
      w.lu[lane] = (double)logf(src.accept_uf(lane));
    } else {
      double u = src.accept_u(lane);
      w.ua[lane] = u;
      w.lu[lane] = log(u);
    }
  }
  __syncwarp();
  for (int level = 0; level < L; level++) {
    int seg = 1 << (L - level), half = seg >> 1, nmid = M / seg;
    const double isq = s.bis_isq[type][level];
    const double *gz = w.gz + 3 * (nmid - 1);
    for (int j = lane; j < nmid; j += 32) {
      int k0 = j * seg, k1 = k0 + half, k2 = k0 + seg;
      for (int d = 0; d < 3; d++) {
        double v = 0.5 * (w.nb[d][k0] + w.nb[d][k2]);
        v = fma(gz[3 * j + d], isq, v);                // as bisect_move: the reciprocal, fused
        w.nb[d][k1] = v;
      }
      if (MIX) w.bf[0][k1] = make_float4((float)w.nb[0][k1], (float)w.nb[1][k1], (float)w.nb[2][k1], 0.0f);
    }
    __syncwarp();
  }
  if (MIX)
    warp_slot_sums(lane, 2 * (M - 1), s.na - 1, g0,
                   [&](int sl, int p) -> float {
                     int k = (sl >> 1) + 1;
                     const float4 b = w.bf[sl & 1][k];
                     return pair_term32(c, frames, g0, p, w.slice[k], b.x, b.y, b.z);
                   },
                   w.se, buf);
  else
    warp_slot_sums(lane, 2 * (M - 1), s.na - 1, g0,
                   [&](int sl, int p) -> double {
                     int k = (sl >> 1) + 1;
                     const double(*b)[PIMC_BATCH_MAX_SEG + 1] = (sl & 1) ? w.ob : w.nb;
                     return pair_term64(c, frames, g0, p, w.slice[k], b[0][k], b[1][k], b[2][k]);
                   },
                   w.se, buf);
  // the action difference of every level (mc_piqmc.cc:256-266), one lane each
  if (lane < L) {
    const int level = lane;
    double pot[2] = {0.0, 0.0};
    for (int l = (level > 0 ? level - 1 : level), wi = (level > 0 ? 0 : 1); l <= level; l++, wi++) {
      int seg = 1 << (L - l), half = seg >> 1, nmid = M / seg;
      double pot0 = 0.0;
      for (int j = 0; j < nmid; j++) {
        int k0 = j * seg, k1 = k0 + half;
        pot0 += (w.se[2 * (k1 - 1)] - w.se[2 * (k1 - 1) + 1]);
        if (k0 != 0) pot0 += (w.se[2 * (k0 - 1)] - w.se[2 * (k0 - 1) + 1]);
      }
      pot[wi] = pot0;
    }
    int seg = 1 << (L - level);
    double deltav = (pot[1] - 2.0 * pot[0]);
    deltav *= s.tau * (double)(seg / 2);
    w.dv[level] = deltav;
  }
  __syncwarp();
  int a = 0;
  if (lane == 0) {
    for (int level = 0; level < L; level++) {
      double deltav = w.dv[level];
      a = (deltav < 0.0) || (-deltav > w.lu[level]);
      if (!a) break;
    }
  }
  a = __shfl_sync(0xffffffffu, a, 0);
  if (a)
    for (int k = 1 + lane; k < M; k += 32) {
      store_bead(c, sidx(s, w.slice[k], g0), w.nb[0][k], w.nb[1][k], w.nb[2][k]);
      invalidate_rotpot(c, w.slice[k]);
    }
  __syncwarp();
  return a;
}

// rot_prepare + rot_finish on one warp, without the rotor caches
template <bool MIX>
__device__ int warp_rot(const Ctx &c, Frame *frames, int g0, int q, const double u[4], const double prop[3],
                        bool linear, WarpRot &w, double *buf, int lane)
{
  const DevSys &s = c.s;
  const int Q = s.Q, R = s.R;
  const size_t n = (size_t)s.nrotors * Q;
  int q0 = q - 1, q2 = q + 1;
  if (q0 < 0) q0 += Q;
  if (q2 >= Q) q2 -= Q;
  const int r = g0 - s.rot_first;
  const int i0 = r * Q + q0, i1 = r * Q + q, i2 = r * Q + q2;
  const bool need64 = !MIX;                     // on the FP32 path the evaluation reads the float frames only
  const bool use_links = Q >= 3;                // link cache (with Q < 3 both links join the same two slices)
  if (lane == 0) {
    w.bad = 0;
    w.pot_cached = c.st.rp_ok[i1];
    if (w.pot_cached) w.pot_c = c.st.rp_cache[i1];
    w.link_ok[0] = use_links && c.st.rl_ok[i0];
    w.link_ok[1] = use_links && c.st.rl_ok[i1];
    if (w.link_ok[0]) w.rho[0] = c.st.rl_cache[i0];
    if (w.link_ok[1]) w.rho[1] = c.st.rl_cache[i1];
    w.ang_new[0] = prop[0]; w.ang_new[1] = prop[1]; w.ang_new[2] = prop[2];
    if (linear) {
      if (MIX) {
        unit_vector32((float)prop[0], (float)prop[1], w.nnewf);
      } else {
        unit_vector(prop[0], prop[1], w.nnew);
      }
    } else if (need64) {
      make_frame(prop[0], prop[1], prop[2], w.fn);
    } else {
      make_frame32((float)prop[0], (float)prop[1], (float)prop[2], w.fn.mf, &w.fn.hzf);
    }
  }
  const bool lazy = linear && lazy_linear(c, MIX);
  if (linear) {
    if (lane < 9) {
      int k = lane / 3, d = lane - 3 * (lane / 3);
      int ii = (k == 0) ? i0 : (k == 1 ? i1 : i2);
      if (lazy) {
        float v = c.st.cosvf[d * n + ii];
        if (k == 0) w.nvf0[d] = v;
        else if (k == 1) w.nvf[d] = v;
        else w.nvf2[d] = v;
      } else {
        w.nv[k][d] = c.st.cosv[d * n + ii];
        if (k == 1) w.nvf[d] = c.st.cosvf[d * n + ii];
      }
    }
  } else {
    copy_frame<false>(w.fo[0], frames + i0, lane);
    copy_frame<false>(w.fo[1], frames + i1, lane);
    copy_frame<false>(w.fo[2], frames + i2, lane);
  }
  __syncwarp();
  // partner sums: the R old slots unless the rotor-potential cache holds them, then the R new ones
  const int first = w.pot_cached ? R : 0;
  const int nsl = 2 * R - first;
  if (linear) {
    if (MIX)
      warp_slot_sums(lane, nsl, s.na - 1, g0,
                     [&](int sl, int p) -> float {
                       int k = sl + first;
                       return rotlin_term32(c, k < R ? w.nvf : w.nnewf, g0, p, q * R + (k % R));
                     },
                     w.vals, buf);
    else
      warp_slot_sums(lane, nsl, s.na - 1, g0,
                     [&](int sl, int p) -> double {
                       int k = sl + first;
                       return rotlin_term64(c, k < R ? w.nv[1] : w.nnew, g0, p, q * R + (k % R));
                     },
                     w.vals, buf);
  } else {
    if (MIX)
      warp_slot_sums(lane, nsl, s.na - 1, g0,
                     [&](int sl, int p) -> float {
                       int k = sl + first;
                       return rot3d_term32(c, frames, k < R ? w.fo[1] : w.fn, g0, p, q * R + (k % R));
                     },
                     w.vals, buf);
    else
      warp_slot_sums(lane, nsl, s.na - 1, g0,
                     [&](int sl, int p) -> double {
                       int k = sl + first;
                       return rot3d_term64(c, frames, k < R ? w.fo[1] : w.fn, g0, p, q * R + (k % R));
                     },
                     w.vals, buf);
  }
  // 0: (q-1, q) old, 1: (q, q+1) old, 2: (q-1, q) new, 3: (q, q+1) new
  if (lane < 4 && !(lane < 2 && w.link_ok[lane])) {
    int bad = 0;
    double rho;
    if (linear) {
      if (MIX && c.t.rd4 && s.rot_den_type == 0) {
        // FP32 path: 1 - cos(gamma) from the float unit vectors, stable for small angles
        const float *fa = (lane == 0 || lane == 2) ? w.nvf0 : (lane == 1 ? w.nvf : w.nnewf);
        const float *fb = (lane == 0) ? w.nvf : (lane == 2 ? w.nnewf : w.nvf2);
        rho = (double)srotdens32(c.t, one_minus_dot32(fa, fb));
      } else {
        double nn[3];
        if (MIX) unit_vector(w.ang_new[0], w.ang_new[1], nn);
        else for (int d = 0; d < 3; d++) nn[d] = w.nnew[d];
        const double *na = (lane == 0 || lane == 2) ? w.nv[0] : (lane == 1 ? w.nv[1] : nn);
        const double *nb = (lane == 0) ? w.nv[1] : (lane == 2 ? nn : w.nv[2]);
        rho = link_density(c, true, w.fo[0], w.fo[0], na, nb, &bad);
      }
    } else {
      const Frame &fa = (lane == 0 || lane == 2) ? w.fo[0] : (lane == 1 ? w.fo[1] : w.fn);
      const Frame &fb = (lane == 0) ? w.fo[1] : (lane == 2 ? w.fn : w.fo[2]);
      if (MIX && s.rot_den_type == 0) {
        rho = (double)rotden_rho32(c.t, fa.mf, fb.mf, &bad);
      } else if (MIX) {
        rho = s.rot_odevn == -1 ? (double)rsrot32(fa.mf, fb.mf, s.rs_coef) : 0.0;
      } else {
        rho = link_density(c, false, fa, fb, nullptr, nullptr, &bad);
      }
    }
    w.rho[lane] = rho;
    if (bad) atomicOr(&w.bad, 1);
  }
  __syncwarp();
  int acc = 0;
  if (lane == 0) {
    double pot_old = 0.0, pot_new = 0.0;
    if (w.pot_cached) pot_old = w.pot_c;
    else
      for (int k = 0; k < R; k++) pot_old += w.vals[k];
    for (int k = 0; k < R; k++) pot_new += w.vals[R - first + k];
    double boltz = rot_boltz<MIX>(s, pot_old, pot_new);
    double logu = rot_logu<MIX>(s, u[linear ? 2 : 3]);
    double rd;
    int neg = 0;
    acc = rot_decide<MIX>(s, linear, w.rho, pot_old, pot_new, boltz, logu, u, &rd, &neg, false);
    if (neg) { atomicOr(c.st.err, (unsigned)DERR_NEG_DENSITY); acc = 0; }
    if (w.bad) { atomicOr(c.st.err, (unsigned)DERR_GRID_RANGE); acc = 0; }
    if (acc) {
      c.st.ang[i1] = w.ang_new[0];
      c.st.ang[n + i1] = w.ang_new[1];
      if (linear) {
        if (lazy) {
          for (int d = 0; d < 3; d++) c.st.cosvf[d * n + i1] = w.nnewf[d];
        } else {
          double cv[3];
          if (MIX) unit_vector(w.ang_new[0], w.ang_new[1], cv);
          else for (int d = 0; d < 3; d++) cv[d] = w.nnew[d];
          for (int d = 0; d < 3; d++) {
            c.st.cosv[d * n + i1] = cv[d];
            c.st.cosvf[d * n + i1] = (float)cv[d];
          }
        }
      } else {
        c.st.ang[2 * n + i1] = w.ang_new[2];
        if (need64) {
          frames[i1] = w.fn;
        } else {
          for (int k = 0; k < 9; k++) frames[i1].mf[k] = w.fn.mf[k];
          frames[i1].hzf = w.fn.hzf;
        }
        // the other rotors' potentials at slice q depend on this orientation:
        // FP64 path, recomputed at their next move; FP32 path, updated below
        if (!MIX)
          for (int rr = 0; rr < s.nrotors; rr++)
            if (rr != r) c.st.rp_ok[rr * Q + q] = 0;
      }
    }
    c.st.rp_cache[i1] = acc ? pot_new : pot_old;
    c.st.rp_ok[i1] = 1;
    if (use_links && !w.bad) {
      c.st.rl_cache[i0] = acc ? w.rho[2] : w.rho[0];
      c.st.rl_cache[i1] = acc ? w.rho[3] : w.rho[1];
      c.st.rl_ok[i0] = 1;
      c.st.rl_ok[i1] = 1;
    }
  }
  acc = __shfl_sync(0xffffffffu, acc, 0);
  if (MIX && acc && !linear && s.nrotors > 1) {
    // FP32 path: each other rotor's cached potential at slice q takes the
    // change of its term with this rotor, slot by slot, instead of being
    // recomputed over all its partners at its next move (caleng32 pairs
    // (other rotor, slot) one per lane, summed per rotor in double)
    const int npair = (s.nrotors - 1) * R;          // <= 15 x 16, within the warp's 256-double buffer
    __syncwarp();
    for (int l = lane; l < npair; l += 32) {
      const int o = l / R, k = l - o * R, it = q * R + k;
      const int grr = s.rot_first + (o < r ? o : o + 1);
      const float4 pa = c.st.b4[sidx(s, it, grr)], pb = c.st.b4[sidx(s, it, g0)];
      const float *mrr = frames[rot_index(s, grr, q)].mf;
      buf[l] = (double)(caleng32(mrr, w.fn.mf, pa.x, pa.y, pa.z, pb.x, pb.y, pb.z) -
                        caleng32(mrr, w.fo[1].mf, pa.x, pa.y, pa.z, pb.x, pb.y, pb.z));
    }
    __syncwarp();
    if (lane < s.nrotors - 1) {
      const int rr = lane < r ? lane : lane + 1;
      double dsum = 0.0;
      for (int k = 0; k < R; k++) dsum += buf[lane * R + k];
      if (c.st.rp_ok[rr * Q + q]) c.st.rp_cache[rr * Q + q] += dsum;
    }
  }
  __syncwarp();
  return acc;
}

// MCMolecularMove (production form) on the whole CTA
template <bool MIX>
__device__ int cta_mol(const Ctx &c, const Frame *frames, int type, int atom, uint64_t seed, unsigned pass,
                       unsigned phase, double *sd, double *red, int *sacc)
{
  const DevSys &s = c.s;
  const int g = s.first[type] + atom, tid = threadIdx.x;
  if (tid == 0) mol_disp(s, type, seed, pass, phase, atom, sd);
  __syncthreads();
  const double d0 = sd[0], d1 = sd[1], d2 = sd[2];
  double an = 0.0, ao = 0.0;
  for (int it = tid; it < s.P; it += blockDim.x) {
    size_t i = sidx(s, it, g);
    double x = c.st.x[i], y = c.st.y[i], z = c.st.z[i];
    if (MIX) {
      // the slice's partner sums in float, one double add per slice
      const float4 p4 = c.st.b4[i];
      const float nx = (float)(x + d0), ny = (float)(y + d1), nz = (float)(z + d2);
      float fo = 0.0f, fn = 0.0f;
      for (int a1 = 0; a1 < s.na; a1++) {
        if (a1 == g) continue;
        fo += pair_term32(c, frames, g, a1, it, p4.x, p4.y, p4.z);
        fn += pair_term32(c, frames, g, a1, it, nx, ny, nz);
      }
      ao += (double)fo;
      an += (double)fn;
    } else {
      for (int a1 = 0; a1 < s.na; a1++) {
        if (a1 == g) continue;
        ao += pair_term64(c, frames, g, a1, it, x, y, z);
        an += pair_term64(c, frames, g, a1, it, x + d0, y + d1, z + d2);
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    an += __shfl_xor_sync(0xffffffffu, an, o);
    ao += __shfl_xor_sync(0xffffffffu, ao, o);
  }
  if ((tid & 31) == 0) { red[tid >> 5] = an; red[32 + (tid >> 5)] = ao; }
  __syncthreads();
  if (tid == 0) {
    double en = 0.0, eo = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) { en += red[k]; eo += red[32 + k]; }
    double deltav = 0.0;
    deltav += (en - eo);
    int a = 0;
    if (deltav < 0.0) a = 1;
    else {
      PhiloxSrc ps{seed, ((uint64_t)pass << 32) | ((uint64_t)phase << 12) | (uint64_t)atom};
      if (exp(-deltav * s.tau) > ps.accept_u(7)) a = 1;
    }
    *sacc = a;
  }
  __syncthreads();
  const int a = *sacc;
  if (a) {
    for (int it = tid; it < s.P; it += blockDim.x) {
      size_t i = sidx(s, it, g);
      store_bead(c, i, c.st.x[i] + d0, c.st.y[i] + d1, c.st.z[i] + d2);
    }
    // the whole path moved: every cached rotor potential is stale
    for (int i = tid; i < s.nrotors * s.Q; i += blockDim.x) c.st.rp_ok[i] = 0;
  }
  __syncthreads();
  return a;
}

__global__ void k_batch_reset(unsigned *work) { *work = 0u; }

// one production pass of every replica; MINB: resident CTAs per SM the
// register allocation is bounded for (a shape the autotuner tries).
// A launch may cover only the bisection blocks [blk_lo, blk_hi) of the pass;
// the one with blk_lo = 0 opens the pass (pass counter, centroid moves).
template <bool MIX, int MINB>
__global__ void __launch_bounds__(256, MINB) k_batch_pass(const BatchRep *reps, const int *order, int n,
                                                          uint64_t seed, unsigned *work, int rot_on, int blk_lo,
                                                          int blk_hi)
{
  extern __shared__ __align__(16) unsigned char smem[];
  Ctx &c = *reinterpret_cast<Ctx *>(smem);
  WarpMem *wm = reinterpret_cast<WarpMem *>(smem + PIMC_BATCH_CTX_BYTES);
  __shared__ int srep;
  __shared__ unsigned sps;
  __shared__ double sd[3], red[64];
  __shared__ int sacc;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, nw = blockDim.x >> 5;
  for (;;) {
    if (tid == 0) srep = (int)atomicAdd(work, 1u);
    __syncthreads();
    const int k = srep;
    if (k >= n) break;
    const int r = order[k];
    {
      const unsigned *src = reinterpret_cast<const unsigned *>(&reps[r].c);
      unsigned *dst = reinterpret_cast<unsigned *>(&c);
      for (int i = tid; i < (int)(sizeof(Ctx) / 4); i += blockDim.x) dst[i] = src[i];
    }
    Frame *frames = reps[r].frames;
    if (tid == 0) sps = blk_lo == 0 ? ++(*reps[r].pass) : *reps[r].pass;
    __syncthreads();
    const unsigned ps = sps;
    const uint64_t sr = seed ^ reps[r].seed_mix;
    const DevSys &s = c.s;
    const bool rot = s.nrotors > 0 && reps[r].rotation && rot_on;
    const bool linear = rot && s.molecule[s.imtype] == 1;
    unsigned long long cnt[12];
    for (int i = 0; i < 12; i++) cnt[i] = 0;
    unsigned B = 0;
    for (int t = 0; t < s.ntypes; t++) B += (unsigned)((1 << s.levels[t]) * s.numb[t]);
    // centroid moves (mc_main.cc:512-513)
    for (int t = 0; t < s.ntypes && blk_lo == 0; t++)
      for (int a = 0; a < s.numb[t]; a++) {
        int acc = cta_mol<MIX>(c, frames, t, a, sr, ps, B + 2u * (unsigned)s.P + (unsigned)t, sd, red, &sacc);
        if (tid == 0) {
          cnt[(t * 3 + 0) * 2 + 0]++;
          cnt[(t * 3 + 0) * 2 + 1] += acc;
        }
      }
    // bisection blocks, each followed by its share of the rotational sweeps
    int nbk = 0;
    for (int t = 0; t < s.ntypes; t++) nbk += 1 << s.levels[t];
    unsigned b0 = 0;
    int blk = 0;
    for (int t = 0; t < s.ntypes; t++) {
      const int M = 1 << s.levels[t], N = s.numb[t];
      for (int s0 = 0; s0 < M; s0++, blk++) {
        if (blk < blk_lo || blk >= blk_hi) {
          b0 += (unsigned)N;
          continue;
        }
        for (int kw = warp; kw < s.P / M; kw += nw)
          for (int j = 0; j < N; j++) {
            PhiloxSrc src{sr, ((uint64_t)ps << 32) | ((uint64_t)(b0 + (unsigned)j) << 12) | (uint64_t)kw};
            int acc = warp_bisect<MIX>(c, frames, t, (kw + j) % N, s0 + kw * M, src, wm[warp].u.b, wm[warp].buf, lane);
            cnt[(t * 3 + 1) * 2 + 0]++;
            cnt[(t * 3 + 1) * 2 + 1] += acc;
          }
        b0 += (unsigned)N;
        __syncthreads();
        if (!rot) continue;
        const int it0 = (int)((long long)blk * s.P / nbk), it1 = (int)((long long)(blk + 1) * s.P / nbk);
        const size_t nq = (size_t)s.nrotors * s.Q;
        for (int it = it0; it < it1; it++)
          for (int parity = 0; parity < 2; parity++) {
            const unsigned phase = B + 2u * (unsigned)it + (unsigned)parity;
            // the independent sets of the half-sweep (odd Q: the last even slice alone)
            int sets[2][2], nsets = 0;
            if (parity == 0) {
              if (s.Q % 2 == 1 && s.Q >= 3) {
                sets[0][0] = 0; sets[0][1] = (s.Q - 1) / 2;
                sets[1][0] = s.Q - 1; sets[1][1] = 1;
                nsets = 2;
              } else {
                sets[0][0] = 0; sets[0][1] = (s.Q + 1) / 2;
                nsets = 1;
              }
            } else if (s.Q / 2 > 0) {
              sets[0][0] = 1; sets[0][1] = s.Q / 2;
              nsets = 1;
            }
            for (int si = 0; si < nsets; si++) {
              for (int kk = warp; kk < sets[si][1]; kk += nw) {
                const int q = sets[si][0] + 2 * kk;
                for (int rr = 0; rr < s.nrotors; rr++) {
                  double u[4] = {0.5, 0.5, 0.5, 0.5}, prop[3] = {0.0, 0.0, 0.0};
                  if (lane == 0) {
                    size_t i1 = (size_t)rr * s.Q + q;
                    rot_uniforms_t<MIX>(sr, ps, phase, q >> 1, rr, linear, u);
                    rot_propose_t<MIX>(s, linear, c.st.ang[i1], c.st.ang[nq + i1], c.st.ang[2 * nq + i1], u, prop);
                  }
                  int acc = warp_rot<MIX>(c, frames, s.rot_first + rr, q, u, prop, linear, wm[warp].u.r, wm[warp].buf,
                                          lane);
                  cnt[(s.imtype * 3 + 2) * 2 + 0]++;
                  cnt[(s.imtype * 3 + 2) * 2 + 1] += acc;
                }
              }
              __syncthreads();
            }
          }
      }
    }
    // the replica's counters: warp leaders add theirs (thread 0's include the centroid moves)
    if (lane == 0)
      for (int i = 0; i < 12; i++)
        if (cnt[i]) atomicAdd(&reps[r].cnt[i], cnt[i]);
    __syncthreads();
  }
}

// per replica: {E_kin spring sum r2avr, E_pot pair sum, the rotational link
// sums (srot, sesq, sts), sum of the rotor axis z component}
__global__ void __launch_bounds__(256) k_batch_est(const BatchRep *reps, int n, double *out)
{
  __shared__ Ctx c;
  __shared__ double red[8][8];
  const int r = blockIdx.x, tid = threadIdx.x;
  if (r >= n) return;
  {
    const unsigned *src = reinterpret_cast<const unsigned *>(&reps[r].c);
    unsigned *dst = reinterpret_cast<unsigned *>(&c);
    for (int i = tid; i < (int)(sizeof(Ctx) / 4); i += blockDim.x) dst[i] = src[i];
  }
  __syncthreads();
  const Frame *frames = reps[r].frames;
  const DevSys &s = c.s;
  double v[6] = {0, 0, 0, 0, 0, 0};
  for (int i = tid; i < s.na * s.P; i += blockDim.x) {
    int a = i / s.P, it = i - a * s.P;
    v[0] += est_spring(c, a, it) / (4.0 * s.beta * s.lambda[atom_type(s, a)]);
  }
  const int npairs = s.na * (s.na - 1) / 2;
  for (int i = tid; i < npairs * s.P; i += blockDim.x) {
    int pidx = i / s.P, it = i - pidx * s.P;
    int a0 = 0, rem = pidx;
    while (rem >= s.na - 1 - a0) { rem -= s.na - 1 - a0; a0++; }
    int a1 = a0 + 1 + rem;
    if (est_pair_counted(c, a0, a1)) {
      size_t k = sidx(s, it, a0);
      v[1] += pair_term64(c, frames, a0, a1, it, c.st.x[k], c.st.y[k], c.st.z[k]);
    }
  }
  if (s.nrotors > 0 && reps[r].rotation) {
    const size_t nq = (size_t)s.nrotors * s.Q;
    for (int k = tid; k < (int)nq; k += blockDim.x) {
      double o[4];
      est_link(c, frames, k, o);
      v[2] += o[0]; v[3] += o[1]; v[4] += o[2];
      v[5] += c.st.cosv[2 * nq + k];
    }
  }
  for (int j = 0; j < 6; j++)
    for (int o = 16; o > 0; o >>= 1) v[j] += __shfl_xor_sync(0xffffffffu, v[j], o);
  if ((tid & 31) == 0)
    for (int j = 0; j < 6; j++) red[tid >> 5][j] = v[j];
  __syncthreads();
  if (tid < 6) {
    double sum = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) sum += red[w][tid];
    out[6 * (size_t)r + tid] = sum;
  }
}

// float beads, frames and caches of every replica after a path upload
__global__ void k_batch_refresh(const BatchRep *reps, int n, int derive)
{
  const int r = blockIdx.x;
  if (r >= n) return;
  const Ctx &c = reps[r].c;
  Frame *frames = reps[r].frames;
  const size_t nq = (size_t)c.s.nrotors * c.s.Q;
  const bool top = c.s.nrotors > 0 && c.s.molecule[c.s.imtype] == 2;
  for (size_t i = threadIdx.x; i < nq; i += blockDim.x) {
    double phi = c.st.ang[i], cost = c.st.ang[nq + i], chi = c.st.ang[2 * nq + i];
    if (top) {
      if (derive) make_frame(phi, cost, chi, frames[i]);
      else make_frame64(phi, cost, chi, frames[i]);
      double v[3];
      unit_vector(phi, cost, v);
      for (int d = 0; d < 3; d++) {
        c.st.cosv[d * nq + i] = v[d];
        c.st.cosvf[d * nq + i] = (float)v[d];
      }
    } else if (derive) {
      if (c.s.nrotors > 0 && lazy_linear(c, c.s.mixed != 0)) {
        float v[3];
        unit_vector32((float)phi, (float)cost, v);          // as the FP32 moves write it
        for (int d = 0; d < 3; d++) c.st.cosvf[d * nq + i] = v[d];
      } else {
        for (int d = 0; d < 3; d++) c.st.cosvf[d * nq + i] = (float)c.st.cosv[d * nq + i];
      }
      c.st.rp_ok[i] = 0;
      c.st.rl_ok[i] = 0;
    } else if (c.s.nrotors > 0 && lazy_linear(c, c.s.mixed != 0)) {
      double v[3];
      unit_vector(phi, cost, v);
      for (int d = 0; d < 3; d++) c.st.cosv[d * nq + i] = v[d];
    }
  }
  if (derive) {
    size_t nb = (size_t)c.s.P * c.s.nap;
    for (size_t i = threadIdx.x; i < nb; i += blockDim.x)
      c.st.b4[i] = make_float4((float)c.st.x[i], (float)c.st.y[i], (float)c.st.z[i], 0.0f);
  }
}

// ------------------------------------------------------------ launchers
size_t batch_smem_bytes(int warps) { return PIMC_BATCH_CTX_BYTES + (size_t)warps * sizeof(WarpMem); }

template <bool MIX, int MINB>
static int batch_occupancy(int warps, size_t sm)
{
  int per = 0;
  cudaFuncSetAttribute(k_batch_pass<MIX, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  cudaFuncSetAttribute(k_batch_pass<MIX, MINB>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_batch_pass<MIX, MINB>, 32 * warps, sm) != cudaSuccess)
    return 0;
  return per;
}

int batch_max_ctas(int mixed, int warps, int minb)
{
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
  size_t sm = batch_smem_bytes(warps);
  int per;
  if (mixed) per = (minb >= 3) ? batch_occupancy<true, 3>(warps, sm) : batch_occupancy<true, 2>(warps, sm);
  else per = (minb >= 3) ? batch_occupancy<false, 3>(warps, sm) : batch_occupancy<false, 2>(warps, sm);
  return nsm * per;
}

void launch_batch_pass(const BatchRep *reps, const int *order, int n, uint64_t seed, unsigned *work, int mixed,
                       int warps, int minb, int nctas, cudaStream_t s, int rot_on, int blk_lo, int blk_hi)
{
  size_t sm = batch_smem_bytes(warps);
  k_batch_reset<<<1, 1, 0, s>>>(work);
  if (mixed) {
    if (minb >= 3)
      k_batch_pass<true, 3><<<nctas, 32 * warps, sm, s>>>(reps, order, n, seed, work, rot_on, blk_lo, blk_hi);
    else k_batch_pass<true, 2><<<nctas, 32 * warps, sm, s>>>(reps, order, n, seed, work, rot_on, blk_lo, blk_hi);
  } else {
    if (minb >= 3)
      k_batch_pass<false, 3><<<nctas, 32 * warps, sm, s>>>(reps, order, n, seed, work, rot_on, blk_lo, blk_hi);
    else k_batch_pass<false, 2><<<nctas, 32 * warps, sm, s>>>(reps, order, n, seed, work, rot_on, blk_lo, blk_hi);
  }
}

// One half-sweep of the rotational slices of many replicas at once, for
// replicas whose own passes interleave their sweeps with their bisection
// blocks: the launch for (block blk, sweep j of the block, parity) moves, in
// every replica with more than j sweeps in that block, the slices of that
// parity -- one warp per (replica, slice), its rotors in order, exactly the
// moves, draws and order of the persistent pass.  Replicas are taken in the
// order `sorted` (most sweeps per block first) and unit u of the launch is
// slice pair u - pre[k] of replica sorted[k], pre the prefix sums of Q/2.
template <bool MIX, int MINB>
__global__ void __launch_bounds__(256, MINB) k_batch_rot_flat(const BatchRep *reps, const int *sorted, const int *pre,
                                                        int nact, int blk, int j, int parity, int nbk,
                                                        uint64_t seed, long long phase0)
{
  extern __shared__ __align__(16) unsigned char smem[];
  WarpMem *wm = reinterpret_cast<WarpMem *>(smem);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int u = blockIdx.x * (blockDim.x >> 5) + warp;
  if (u >= pre[nact]) return;                           // warp-uniform
  int lo = 0, hi = nact;                                // pre[lo] <= u < pre[hi]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (pre[mid] <= u) lo = mid;
    else hi = mid;
  }
  const BatchRep &rp = reps[sorted[lo]];
  const Ctx &c = rp.c;
  const DevSys &s = c.s;
  Frame *frames = rp.frames;
  const unsigned ps = *rp.pass;
  const uint64_t sr = seed ^ rp.seed_mix;
  const bool linear = s.molecule[s.imtype] == 1;
  unsigned B = 0;
  for (int t = 0; t < s.ntypes; t++) B += (unsigned)((1 << s.levels[t]) * s.numb[t]);
  const int it = (int)((long long)blk * s.P / nbk) + j;
  // the pass's phase of this half-sweep, or phase0 + parity where the caller keys it (the worm loop)
  const unsigned phase = phase0 >= 0 ? (unsigned)phase0 + (unsigned)parity : B + 2u * (unsigned)it + (unsigned)parity;
  const int kk = u - pre[lo], q = parity + 2 * kk;
  const size_t nq = (size_t)s.nrotors * s.Q;
  unsigned long long tot = 0, nacc = 0;
  for (int rr = 0; rr < s.nrotors; rr++) {
    double uu[4] = {0.5, 0.5, 0.5, 0.5}, prop[3] = {0.0, 0.0, 0.0};
    if (lane == 0) {
      size_t i1 = (size_t)rr * s.Q + q;
      rot_uniforms_t<MIX>(sr, ps, phase, q >> 1, rr, linear, uu);
      rot_propose_t<MIX>(s, linear, c.st.ang[i1], c.st.ang[nq + i1], c.st.ang[2 * nq + i1], uu, prop);
    }
    int acc = warp_rot<MIX>(c, frames, s.rot_first + rr, q, uu, prop, linear, wm[warp].u.r, wm[warp].buf, lane);
    tot++;
    nacc += acc;
  }
  if (lane == 0) {
    atomicAdd(&rp.cnt[(s.imtype * 3 + 2) * 2 + 0], tot);
    atomicAdd(&rp.cnt[(s.imtype * 3 + 2) * 2 + 1], nacc);
  }
}

size_t batch_flat_smem_bytes(int warps) { return (size_t)warps * sizeof(WarpMem); }

// minb: resident CTAs per SM the registers are bounded for (2, 3 or 4)
void launch_batch_rot_flat(const BatchRep *reps, const int *sorted, const int *pre, int nact, int units, int blk,
                           int j, int parity, int nbk, uint64_t seed, int mixed, int warps, int minb, cudaStream_t s,
                           long long phase0)
{
  if (units <= 0) return;
  const size_t sm = batch_flat_smem_bytes(warps);
  const int nctas = (units + warps - 1) / warps;
#define PIMC_FLAT(M, B) \
  k_batch_rot_flat<M, B><<<nctas, 32 * warps, sm, s>>>(reps, sorted, pre, nact, blk, j, parity, nbk, seed, phase0)
  if (mixed) {
    if (minb >= 4) PIMC_FLAT(true, 4);
    else if (minb == 3) PIMC_FLAT(true, 3);
    else PIMC_FLAT(true, 2);
  } else {
    if (minb >= 4) PIMC_FLAT(false, 4);
    else if (minb == 3) PIMC_FLAT(false, 3);
    else PIMC_FLAT(false, 2);
  }
#undef PIMC_FLAT
}

template <bool MIX, int MINB>
static bool flat_attr(size_t sm)
{
  return cudaFuncSetAttribute(k_batch_rot_flat<MIX, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) ==
         cudaSuccess;
}

int batch_flat_setup(int warps)
{
  const size_t sm = batch_flat_smem_bytes(warps);
  return flat_attr<true, 2>(sm) && flat_attr<true, 3>(sm) && flat_attr<true, 4>(sm) && flat_attr<false, 2>(sm) &&
         flat_attr<false, 3>(sm) && flat_attr<false, 4>(sm);
}

// after rotational moves made outside k_batch_pass: each replica's MCCosine
// from its angles and its rotor caches stale
__global__ void k_batch_rot_changed(const BatchRep *reps, int n)
{
  const int r = blockIdx.x;
  if (r >= n) return;
  const Ctx &c = reps[r].c;
  const size_t nq = (size_t)c.s.nrotors * c.s.Q;
  for (size_t i = threadIdx.x; i < nq; i += blockDim.x) {
    double v[3];
    unit_vector(c.st.ang[i], c.st.ang[nq + i], v);
    for (int d = 0; d < 3; d++) {
      c.st.cosv[d * nq + i] = v[d];
      c.st.cosvf[d * nq + i] = (float)v[d];
    }
    c.st.rp_ok[i] = 0;
    c.st.rl_ok[i] = 0;
  }
}

void launch_batch_rot_changed(const BatchRep *reps, int n, cudaStream_t s)
{
  if (n > 0) k_batch_rot_changed<<<n, 256, 0, s>>>(reps, n);
}

void launch_batch_est(const BatchRep *reps, int n, double *out, cudaStream_t s)
{
  if (n > 0) k_batch_est<<<n, 256, 0, s>>>(reps, n, out);
}

void launch_batch_refresh(const BatchRep *reps, int n, int derive, cudaStream_t s)
{
  if (n > 0) k_batch_refresh<<<n, 256, 0, s>>>(reps, n, derive);
}
