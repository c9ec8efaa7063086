// pimc_kernels.cuh -- move and energy routines executed by one CTA of
// PIMC_BLOCK threads, shared by the replay (parity) kernels and the
// production phase kernels.
//
// A move's work is a set of (slot, partner) items -- a slot is one slice
// energy PotEnergy(atom, pos, it) or PotRotE3D/PotRotEnergy(rotor, ., it)
// and the partners are all other atoms -- flattened over all threads of the
// CTA; each slot's sum is then reduced by one warp in a fixed order, so the
// result does not depend on scheduling.  MIX selects the FP32 table path:
// pair terms from the float copies of beads and tables, sums and everything
// after them in FP64.
#pragma once
#include "pimc_internal.cuh"

__device__ __forceinline__ size_t sidx(const DevSys &s, int t, int a) { return (size_t)t * s.nap + a; }

__device__ __forceinline__ int rot_index(const DevSys &s, int gatom, int q) { return (gatom - s.rot_first) * s.Q + q; }

// MCType of a global atom: types occupy consecutive ranges (mc_setup.cc:327-333)
__device__ __forceinline__ int atom_type(const DevSys &s, int a) { return (s.ntypes > 1 && a >= s.first[1]) ? 1 : 0; }

// one term of PotEnergy(atom0, pos, it) (mc_piqmc.cc:1824-1958): atom0 at
// (px,py,pz), partner atom1 at its current bead, rotor frames from the cache
// With an open worm, PotEnergy, PotRotEnergy and PotRotE3D leave out the
// partner beads of the worm type that lie in the gap between masha and ira
// (WorldLine, mc_qworm.cc:553-575; mc_piqmc.cc:1226-1227, 1816-1817,
// 2000-2001, 2082-2083).
__device__ __forceinline__ bool worm_gap(const Ctx &c, int a1, int it)
{
  const DevWorm *w = c.st.worm;
  if (w == nullptr || !w->exists || atom_type(c.s, a1) != w->type) return false;
  const int a = a1 - w->first, ai = w->atom_i, am = w->atom_m, ira = w->ira, masha = w->masha;
  if (a != am && a != ai) return false;
  if (ai != am || ira > masha) return (a == am && it < masha) || (a == ai && it > ira);
  return it > ira && it < masha;
}

__device__ __forceinline__ double pair_term64(const Ctx &c, const Frame *frames, int a0, int a1, int it,
                                              double px, double py, double pz)
{
  const DevSys &s = c.s;
  if (worm_gap(c, a1, it)) return 0.0;
  int m0 = s.molecule[atom_type(s, a0)], m1 = s.molecule[atom_type(s, a1)];
  size_t i1 = sidx(s, it, a1);
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
    return lpot2d(c.t, r, cost);
  } else if ((m0 == 2 || m1 == 2) && m0 != m1) {
    if (s.ispher) return vspher(c.t, r);
    if (m0 == 2) return vcord(c.t, frames[rot_index(s, a0, it / s.R)], px, py, pz, qx, qy, qz);
    return vcord(c.t, frames[rot_index(s, a1, it / s.R)], qx, qy, qz, px, py, pz);
  } else if (m0 == 2 && m1 == 2 && s.numb[s.imtype] > 1) {
    return caleng(frames[rot_index(s, a0, it / s.R)], frames[rot_index(s, a1, it / s.R)], px, py, pz, qx, qy, qz);
  }
  return spot1d(c.t, r);
}

// the same term on the FP32 table path
__device__ __forceinline__ float pair_term32(const Ctx &c, const Frame *frames, int a0, int a1, int it,
                                             float px, float py, float pz)
{
  const DevSys &s = c.s;
  if (worm_gap(c, a1, it)) return 0.0f;
  int m0 = s.molecule[atom_type(s, a0)], m1 = s.molecule[atom_type(s, a1)];
  size_t i1 = sidx(s, it, a1);
  const float4 q4 = c.st.b4[i1];
  float qx = q4.x, qy = q4.y, qz = q4.z;
  float dx = px - qx, dy = py - qy, dz = pz - qz;
  if (s.minimage) {
    dx -= (float)s.box[0] * rintf(dx / (float)s.box[0]);
    dy -= (float)s.box[1] * rintf(dy / (float)s.box[1]);
    dz -= (float)s.box[2] * rintf(dz / (float)s.box[2]);
  }
  float r = sqrtf(dx * dx + dy * dy + dz * dz);
  if (m0 == 1 || m1 == 1) {
    int rot = (m0 == 1) ? a0 : a1;
    size_t n = (size_t)s.nrotors * s.Q;
    int ri = rot_index(s, rot, it / s.R);
    float cost = (c.st.cosvf[ri] * dx + c.st.cosvf[n + ri] * dy + c.st.cosvf[2 * n + ri] * dz) / r;
    if (m0 == 1) cost = -cost;
    return lpot2d32(c.t, r, cost);
  } else if ((m0 == 2 || m1 == 2) && m0 != m1) {
    if (s.ispher) return (float)vspher(c.t, (double)r);
    if (m0 == 2) return vcord32(c.t, frames[rot_index(s, a0, it / s.R)], -dx, -dy, -dz);
    return vcord32(c.t, frames[rot_index(s, a1, it / s.R)], dx, dy, dz);
  } else if (m0 == 2 && m1 == 2 && s.numb[s.imtype] > 1) {
    return caleng32(frames[rot_index(s, a0, it / s.R)].mf, frames[rot_index(s, a1, it / s.R)].mf, px, py, pz, qx, qy,
                    qz);
  }
  return spot1d32(c.t, r);
}

// out[s] = sum over partners p != skip[s] of f(s, p), s < nslots.  buf holds
// PIMC_RED_BUF doubles of shared memory; slots are processed in chunks that
// fit.  Each slot is reduced by one warp: lane l adds items l, l+32, ... in
// order, then a fixed xor-shuffle tree; deterministic.  The items and the
// sum have f's type: double on the FP64 path, float on the FP32 path (one
// float round per add instead of a serial chain of double adds, which on
// this part costs about sixty cycles per add).
template <class F, class O>
__device__ __forceinline__ void slot_sums(int nslots, int na, const int *skip, F f, O *out, double *bufd)
{
  using T = decltype(f(0, 0));
  T *buf = reinterpret_cast<T *>(bufd);
  const int npart = na - 1;
  if (npart <= 0) {
    for (int s = threadIdx.x; s < nslots; s += blockDim.x) out[s] = O(0);
    __syncthreads();
    return;
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const int total = nslots * npart;
  // chunks of whole slots when a slot fits the buffer, else of PIMC_RED_BUF items
  const int chunk = (npart <= PIMC_RED_BUF) ? (PIMC_RED_BUF / npart) * npart : PIMC_RED_BUF;
  const int nt = blockDim.x;
  for (int base = 0; base < total; base += chunk) {
    int cnt = min(chunk, total - base);
    // two items per step so that their loads overlap
    for (int i = threadIdx.x; i < cnt; i += 2 * nt) {
      int g = base + i;
      int s = g / npart, pi = g - s * npart;
      int p = pi < skip[s] ? pi : pi + 1;
      int i2 = i + nt;
      T v0 = f(s, p), v1 = T(0);
      if (i2 < cnt) {
        int g2 = base + i2;
        int s2 = g2 / npart, pi2 = g2 - s2 * npart;
        int p2 = pi2 < skip[s2] ? pi2 : pi2 + 1;
        v1 = f(s2, p2);
        buf[i2] = v1;
      }
      buf[i] = v0;
    }
    __syncthreads();
    int sfirst = base / npart, slast = (base + cnt - 1) / npart;
    for (int sl = sfirst + warp; sl <= slast; sl += nw) {
      int lo = max(sl * npart, base) - base, hi = min((sl + 1) * npart, base + cnt) - base;
      T acc = T(0);
      for (int k = lo + lane; k < hi; k += 32) acc += buf[k];
      for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
      if (lane == 0) {
        if (sl * npart >= base) out[sl] = (O)acc;     // the slot starts in this chunk
        else out[sl] += (O)acc;                       // continuation of a slot split across chunks
      }
    }
    __syncthreads();
  }
}

// ------------------------------------------------------ random sources

// replay of the reference's sequential generator streams (parity mode);
// cursors live in global memory.  Gaussian draws of one bisection level are
// consumed unconditionally (3 per midpoint, mc_piqmc.cc:249-253), so they are
// indexed from the level's base; accept draws are taken one at a time.
struct ReplaySrc {
  static constexpr bool kPrefetchU = false;  // rnd3() is drawn only where the reference draws it
  const double *g; long ng; long *gpos;      // gauss() x1 values
  const double *u; long nu; long *upos;      // rnd2()/rnd3() uniforms
  const double *d; long nd; long *dpos;      // rnd1() displacements
  unsigned int *err;
  __device__ double take(const double *v, long n, long *pos)
  {
    long p = *pos;
    if (p >= n) { atomicOr(err, (unsigned)DERR_STREAM); return 0.5; }
    *pos = p + 1;
    return v[p];
  }
  __device__ long gauss_base() { return *gpos; }
  __device__ double gauss_at(long base, int, int j, int dim)
  {
    long p = base + 3 * j + dim;
    if (p >= ng) { atomicOr(err, (unsigned)DERR_STREAM); return 0.0; }
    return g[p];
  }
  __device__ void gauss_advance(long n)
  {
    *gpos += n;
    if (*gpos > ng) atomicOr(err, (unsigned)DERR_STREAM);
  }
  // prefetch of draw i of the move (levels not reached are never consumed)
  __device__ double gauss_pre(long base, int i, int, int, int) { return (base + i < ng) ? g[base + i] : 0.0; }
  __device__ double accept_u(int) { return take(u, nu, upos); }
  __device__ double disp_u(int) { return take(d, nd, dpos); }
  __device__ double gauss_at32(int, int, int) { return 0.0; }
  __device__ float accept_uf(int) { return 0.5f; }
};

// counter-based source for production moves: one Philox block per draw
struct PhiloxSrc {
  static constexpr bool kPrefetchU = true;
  uint64_t seed, move;
  __device__ long gauss_base() { return 0; }
  __device__ double gauss_at(long, int level, int k, int dim)
  {
    double r1, r2;
    philox_u2(seed, move, 0x100000u | ((uint32_t)level << 12) | (uint32_t)k, (uint32_t)dim, &r1, &r2);
    return sqrt(-log(r1)) * cos(2.0 * PIMC_PI * r2);        // Box-Muller as gauss() (mc_randg.cc:144)
  }
  // a draw with float uniforms, logarithm and cosine (FP32 path); the
  // 32-bit uniform keeps the tail out to 6.6 standard deviations
  __device__ double gauss_at32(int level, int k, int dim)
  {
    float r1, r2;
    philox_u2f(seed, move, 0x100000u | ((uint32_t)level << 12) | (uint32_t)k, (uint32_t)dim, &r1, &r2);
    return (double)(sqrtf(-logf(r1)) * cospif(2.0f * r2));
  }
  __device__ void gauss_advance(long) {}
  __device__ double gauss_pre(long, int, int level, int k, int dim) { return gauss_at(0, level, k, dim); }
  __device__ double accept_u(int level)
  {
    double u0, u1;
    philox_u2(seed, move, 0x200000u | (uint32_t)level, 0u, &u0, &u1);
    return u0;
  }
  __device__ float accept_uf(int level)
  {
    float u0, u1;
    philox_u2f(seed, move, 0x200000u | (uint32_t)level, 0u, &u0, &u1);
    return u0;
  }
  __device__ double disp_u(int dim)
  {
    double u0, u1;
    philox_u2(seed, move, 0x300000u, (uint32_t)dim, &u0, &u1);
    return u0;
  }
};

// a translational commit at slice t invalidates the cached rotor potential
// of the rotational slice t/R for every rotor
__device__ __forceinline__ void invalidate_rotpot(const Ctx &c, int t)
{
  for (int r = 0; r < c.s.nrotors; r++) c.st.rp_ok[r * c.s.Q + t / c.s.R] = 0;
}

__device__ __forceinline__ void store_bead(const Ctx &c, size_t i, double x, double y, double z)
{
  c.st.x[i] = x;
  c.st.y[i] = y;
  c.st.z[i] = z;
  c.st.b4[i] = make_float4((float)x, (float)y, (float)z, 0.0f);
}

// ------------------------------------------------------ bisection move
// MCBisectionMove / MCBisectionMoveExchange (mc_piqmc.cc:194-419) for the
// local atom `atom` of `type` over the window [time0, time0 + 2^levels].
// exch switches the owner of slices past P to pindex[atom] (the permutation
// the path closes through); the midpoint energy is that of the slice's owner.
// Returns 1 when accepted; records per-level action differences.
struct BisectShared {
  double gz[3 * PIMC_MAX_SEG];        // all Gaussian draws of the move, level by level
  double ua[8];                       // accept uniforms per level (counter-based source)
  double ob[3][PIMC_MAX_SEG + 1];     // the current beads of the window
  double nb[3][PIMC_MAX_SEG + 1];     // the proposed beads
  double se[2 * PIMC_MAX_SEG];        // slice energies: (bead k, new) at 2(k-1), (bead k, old) at 2(k-1)+1
  float sef[2 * PIMC_MAX_SEG];        // the same on the FP32 path
  double dv[8], ex[8];                // per level: action difference, exp(-difference) (replay)
  double lu[8];                       // log of the accept uniforms (counter-based source)
  float4 bf[2][PIMC_MAX_SEG + 1];     // float copies of the proposed [0] and current [1] beads
  int sa[2 * PIMC_MAX_SEG];           // owner of the slot's bead (the partner sums skip it)
  int owner[PIMC_MAX_SEG + 1], slice[PIMC_MAX_SEG + 1];
  int acc, passed;
  long gbase;
  double buf[PIMC_RED_BUF];
};

// The proposal of all levels is fixed by the Gaussian draws alone (a
// level's midpoints are built from the previous level's new beads whether
// or not it is then accepted), and a bead's slice energy does not change
// once it is placed.  So all 2(M-1) slice energies are summed in one pass
// over (slot, partner) items, and the level-by-level accept of the
// reference (mc_piqmc.cc:243-281) then runs on thread 0 from those sums:
// level l's pot0 is the new-minus-old energy of the beads at multiples of
// 2^(L-l-1) (mc_piqmc.cc:256-263), its action difference
// (pot0 - 2 pot1) tau 2^(L-l-1) (mc_piqmc.cc:265-266).  Only the levels the
// reference reaches consume their draws.
template <bool MIX, class Src>
__device__ int bisect_move(const Ctx &c, const Frame *frames, int type, int atom, int time0, int exch, Src &src,
                           BisectShared &sh, double *ds_out)
{
  const DevSys &s = c.s;
  int tid = threadIdx.x;
  int P = s.P, L = s.levels[type], M = 1 << L;
  int g0 = s.first[type] + atom;
  // PIndex holds the local index of the atom the path continues into
  // (mc_piqmc.cc:312-313)
  int gx = exch ? s.first[type] + c.st.pindex[atom] : g0;
  if (gx < s.first[type] || gx >= s.first[type] + s.numb[type]) gx = g0;
  for (int k = tid; k <= M; k += blockDim.x) {
    int t = time0 + k;
    int own = (exch && t >= P) ? gx : g0;
    int pt = t % P;
    sh.owner[k] = own;
    sh.slice[k] = pt;
    size_t i = sidx(s, pt, own);
    double x = c.st.x[i], y = c.st.y[i], z = c.st.z[i];
    sh.nb[0][k] = x; sh.nb[1][k] = y; sh.nb[2][k] = z;
    sh.ob[0][k] = x; sh.ob[1][k] = y; sh.ob[2][k] = z;
    if (MIX) sh.bf[1][k] = c.st.b4[i];
  }
  if (tid == 0) { sh.acc = 0; sh.passed = 0; sh.gbase = src.gauss_base(); }
  __syncthreads();
  // the move's Gaussian draws, all levels at once: level l's midpoint j,
  // dimension d is draw 3(2^l - 1) + 3j + d (the reference's order)
  for (int i = tid; i < 3 * (M - 1); i += blockDim.x) {
    int l = 31 - __clz(i / 3 + 1);
    int off = i - 3 * ((1 << l) - 1);
    if (MIX && Src::kPrefetchU) sh.gz[i] = src.gauss_at32(l, off / 3, off - 3 * (off / 3));
    else sh.gz[i] = src.gauss_pre(sh.gbase, i, l, off / 3, off - 3 * (off / 3));
  }
  if (Src::kPrefetchU)
    for (int l = tid - 64; l >= 0 && l < L; l += blockDim.x) {
      if (MIX) {
        sh.lu[l] = (double)logf(src.accept_uf(l));          // a float uniform; the test itself in double
      } else {
        double u = src.accept_u(l);
        sh.ua[l] = u;
        sh.lu[l] = log(u);
      }
    }
  __syncthreads();
  // the proposed beads, level by level (mc_piqmc.cc:243-254)
  for (int level = 0; level < L; level++) {
    int seg = 1 << (L - level), half = seg >> 1, nmid = M / seg;
    const double isq = s.bis_isq[type][level];
    const double *gz = sh.gz + 3 * (nmid - 1);
    for (int j = tid; j < nmid; j += blockDim.x) {
      int k0 = j * seg, k1 = k0 + half, k2 = k0 + seg;
      for (int d = 0; d < 3; d++) {
        // mid + x / sqrt(alpha) (mc_piqmc.cc:243-254, mc_randg.cc:149) as one
        // fused multiply-add with the reciprocal: within an ulp of the
        // reference's division and sum, without an FP64 division chain on the
        // few lanes that make the midpoints (both precisions)
        double v = 0.5 * (sh.nb[d][k0] + sh.nb[d][k2]);
        v = fma(gz[3 * j + d], isq, v);
        sh.nb[d][k1] = v;
      }
      if (MIX) sh.bf[0][k1] = make_float4((float)sh.nb[0][k1], (float)sh.nb[1][k1], (float)sh.nb[2][k1], 0.0f);
      sh.sa[2 * (k1 - 1)] = sh.owner[k1];
      sh.sa[2 * (k1 - 1) + 1] = sh.owner[k1];
    }
    __syncthreads();
  }
  // slice energies of every interior bead, new and old
  if (MIX)
    slot_sums(2 * (M - 1), s.na, sh.sa,
              [&](int sl, int p) -> float {
                int k = (sl >> 1) + 1;
                const float4 b = sh.bf[sl & 1][k];
                return pair_term32(c, frames, sh.owner[k], p, sh.slice[k], b.x, b.y, b.z);
              },
              sh.sef, sh.buf);
  else
    slot_sums(2 * (M - 1), s.na, sh.sa,
              [&](int sl, int p) -> double {
                int k = (sl >> 1) + 1;
                const double(*b)[PIMC_MAX_SEG + 1] = (sl & 1) ? sh.ob : sh.nb;
                return pair_term64(c, frames, sh.owner[k], p, sh.slice[k], b[0][k], b[1][k], b[2][k]);
              },
              sh.se, sh.buf);
  // the action difference of every level in double precision on both paths
  // (the energies of the FP32 path are float sums), one level per warp
  // summing the bead differences in the reference's order
  // (mc_piqmc.cc:256-266); thread 0 then takes the level decisions in the
  // reference's order.  Replay draws rnd3() only where the reference does
  // and tests exp(-dS) > u as it does; the counter-based source tests the
  // same inequality as -dS > log u with log u computed up front.
  if ((tid & 31) == 0 && (tid >> 5) < L) {
    const int level = tid >> 5;                 // one warp per level: the chains issue side by side
    auto de = [&](int k) -> double {
      double en = MIX ? (double)sh.sef[2 * (k - 1)] : sh.se[2 * (k - 1)];
      double eo = MIX ? (double)sh.sef[2 * (k - 1) + 1] : sh.se[2 * (k - 1) + 1];
      return en - eo;
    };
    double pot[2] = {0.0, 0.0};                 // pot0 of level-1 and of level
    for (int l = (level > 0 ? level - 1 : level), w = (level > 0 ? 0 : 1); l <= level; l++, w++) {
      int seg = 1 << (L - l), half = seg >> 1, nmid = M / seg;
      double pot0 = 0.0;
      for (int j = 0; j < nmid; j++) {
        int k0 = j * seg, k1 = k0 + half;
        pot0 += de(k1);
        if (k0 != 0) pot0 += de(k0);
      }
      pot[w] = pot0;
    }
    int seg = 1 << (L - level);
    double deltav = (pot[1] - 2.0 * pot[0]);
    deltav *= s.tau * (double)(seg / 2);
    sh.dv[level] = deltav;
    if (!Src::kPrefetchU) sh.ex[level] = exp(-deltav);
  }
  __syncthreads();
  if (tid == 0) {
    int a = 0;
    for (int level = 0; level < L; level++) {
      int seg = 1 << (L - level), nmid = M / seg;
      src.gauss_advance(3 * nmid);
      double deltav = sh.dv[level];
      if (ds_out) ds_out[level] = deltav;
      a = 0;
      if (deltav < 0.0) a = 1;
      else if (Src::kPrefetchU ? (-deltav > sh.lu[level]) : (sh.ex[level] > src.accept_u(level))) a = 1;
      if (!a) break;
      sh.passed = level + 1;
    }
    sh.acc = a;
  }
  __syncthreads();
  int accepted = sh.acc;
  if (accepted) {
    for (int k = 1 + tid; k < M; k += blockDim.x) {
      size_t i = sidx(s, sh.slice[k], sh.owner[k]);
      store_bead(c, i, sh.nb[0][k], sh.nb[1][k], sh.nb[2][k]);
      invalidate_rotpot(c, sh.slice[k]);
    }
  }
  __syncthreads();
  return accepted;
}

// scratch of one centroid move: the displacement and per-partner whole-path
// sums for the displaced and the current path
#define PIMC_MAX_ATOMS 1024
#define PIMC_MOL_MAXCHUNK 8           /* slice chunks per partner in a centroid move */
struct MolScratch {
  double disp[3];
  double pair[2][PIMC_MAX_ATOMS * PIMC_MOL_MAXCHUNK];   // [new/old][partner * nchunk + chunk]
};

// the displacement of a production centroid move (every CTA draws the same)
__device__ __forceinline__ void mol_disp(const DevSys &s, int type, uint64_t seed, unsigned pass, unsigned phase,
                                         int atom, double d[3])
{
  PhiloxSrc ps{seed, ((uint64_t)pass << 32) | ((uint64_t)phase << 12) | (uint64_t)atom};
  for (int k = 0; k < 3; k++) d[k] = s.mcstep[type] * (ps.disp_u(k) - 0.5);
}

// ------------------------------------------------------ rotational moves
// A rotational move runs on PIMC_ROT_THREADS threads in two stages.
// rot_prepare reads only the moved slice: the proposal's frame, the
// (slot, partner) sums over its R translational slices (warps 0-7, named
// barrier 2 inside the sums) and, for a linear rotor on the FP32 path, the
// proposal's unit vector in double precision (warp 9).  rot_finish reads the
// neighbouring slices and runs on warp 8 alone: their frames and the link
// cache, the link densities rho(q-1, q) and rho(q, q+1) old and new (lanes
// 0-3), the accept and the commit (lane 0).  A persistent launch that owns
// one slice per CTA prepares the slice's next move while the neighbours
// move, so only rot_finish lies on the chain between neighbouring slices.
//
// For a nonlinear rotor the commit writes the angles and the frame the
// evaluation used (on the FP32 path only its float part);
// the double-precision frame and MCCosine are then derived from the angles
// by k_refresh_frames before anything reads them (estimators, state
// download, queries), which gives the same values as writing them here.
#define PIMC_ROT_PAIR_THREADS 256

template <int ID, int NT>
__device__ __forceinline__ void group_sync()
{
  asm volatile("bar.sync %0, %1;" ::"n"(ID), "n"(NT) : "memory");
}

// slot_sums over threads [0, NT) of the CTA, synchronised by named barrier ID
template <int NT, int ID, class F, class O>
__device__ __forceinline__ void slot_sums_group(int nslots, int na, const int *skip, F f, O *out, double *bufd)
{
  using T = decltype(f(0, 0));
  T *buf = reinterpret_cast<T *>(bufd);
  const int npart = na - 1;
  if (npart <= 0) {
    for (int s = threadIdx.x; s < nslots; s += NT) out[s] = O(0);
    group_sync<ID, NT>();
    return;
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = NT >> 5;
  const int total = nslots * npart;
  const int chunk = (npart <= PIMC_RED_BUF) ? (PIMC_RED_BUF / npart) * npart : PIMC_RED_BUF;
  for (int base = 0; base < total; base += chunk) {
    int cnt = min(chunk, total - base);
    for (int i = threadIdx.x; i < cnt; i += NT) {
      int g = base + i;
      int s = g / npart, pi = g - s * npart;
      int p = pi < skip[s] ? pi : pi + 1;
      buf[i] = f(s, p);
    }
    group_sync<ID, NT>();
    int sfirst = base / npart, slast = (base + cnt - 1) / npart;
    for (int sl = sfirst + warp; sl <= slast; sl += nw) {
      int lo = max(sl * npart, base) - base, hi = min((sl + 1) * npart, base + cnt) - base;
      T acc = T(0);
      for (int k = lo + lane; k < hi; k += 32) acc += buf[k];
      for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
      if (lane == 0) {
        if (sl * npart >= base) out[sl] = (O)acc;
        else out[sl] += (O)acc;
      }
    }
    group_sync<ID, NT>();
  }
}

// loads of state that other CTAs of a persistent launch write: through L2
template <bool COH>
__device__ __forceinline__ double ld_state(const double *p)
{
  return COH ? __ldcg(p) : *p;
}
template <bool COH>
__device__ __forceinline__ int ld_state(const int *p)
{
  return COH ? __ldcg(p) : *p;
}
template <bool COH>
__device__ __forceinline__ void copy_frame(Frame &dst, const Frame *src, int lane)
{
  const unsigned *a = reinterpret_cast<const unsigned *>(src);
  unsigned *b = reinterpret_cast<unsigned *>(&dst);
  for (int w = lane; w < (int)(sizeof(Frame) / 4); w += 32) b[w] = COH ? __ldcg(a + w) : a[w];
}

struct RotShared {
  Frame fo[3];              // current frames at q-1, q, q+1
  Frame fn;                 // the proposal as evaluated (mf; m too where needed)
  double rho[4], vals[2 * 16];
  double ang_new[3];
  double nv[3][3];          // linear rotor: current unit vectors at q-1, q, q+1
  double nnew[3];           // linear rotor: proposal unit vector (double path)
  double cv[3];             // linear rotor: MCCosine of the proposal
  float nvf[3], nnewf[3];   // linear rotor: current and proposal unit vectors for the FP32 path
  float nvf0[3], nvf2[3];   // linear rotor: the neighbours' float unit vectors
  int bad, acc, pot_cached, link_ok[2], stop;
  int skip[2 * 16];
  double pot_c, rd;
  double u[4], pot_old, pot_new;
  double boltz;             // exp(-tau (pot_new - pot_old)) (Noya densities) or -tau (pot_new - pot_old) (RS)
  double logu;              // log of the accept uniform (RS densities)
  float valsf[2 * 16];      // partner sums on the FP32 path
  double ang_old[3];        // the slice's current angles
  double nxt_u[4], nxt_prop[2][3];   // the slice's next move: uniforms, proposal if this one is rejected / accepted
  Frame nxt_fn[2];          // FP64 path, top: the frames of the two next proposals
  double nxt_nv[2][3];      // FP64 path, linear rotor: their unit vectors
  double buf[PIMC_RED_BUF];
};

// PotRotE3D term (mc_piqmc.cc:2078-2146) for rotor g0 with body frame f at
// slice it against partner a1
__device__ __forceinline__ double rot3d_term64(const Ctx &c, const Frame *frames, const Frame &f, int g0, int a1, int it)
{
  const DevSys &s = c.s;
  if (worm_gap(c, a1, it)) return 0.0;
  size_t i0 = sidx(s, it, g0), i1 = sidx(s, it, a1);
  if (atom_type(s, a1) != s.imtype)
    return vcord(c.t, f, c.st.x[i0], c.st.y[i0], c.st.z[i0], c.st.x[i1], c.st.y[i1], c.st.z[i1]);
  return caleng(f, frames[rot_index(s, a1, it / s.R)], c.st.x[i0], c.st.y[i0], c.st.z[i0], c.st.x[i1], c.st.y[i1],
                c.st.z[i1]);
}

__device__ __forceinline__ float rot3d_term32(const Ctx &c, const Frame *frames, const Frame &f, int g0, int a1, int it)
{
  const DevSys &s = c.s;
  if (worm_gap(c, a1, it)) return 0.0f;
  size_t i0 = sidx(s, it, g0), i1 = sidx(s, it, a1);
  if (atom_type(s, a1) != s.imtype) {
    const float4 p0 = c.st.b4[i0], p1 = c.st.b4[i1];
    return vcord32(c.t, f, p1.x - p0.x, p1.y - p0.y, p1.z - p0.z);
  }
  const float4 p0 = c.st.b4[i0], p1 = c.st.b4[i1];
  return caleng32(f.mf, frames[rot_index(s, a1, it / s.R)].mf, p0.x, p0.y, p0.z, p1.x, p1.y, p1.z);
}

// PotRotEnergy term (mc_piqmc.cc:1987-2040) for the linear rotor g0 with unit
// vector n at slice it against partner a1
__device__ __forceinline__ double rotlin_term64(const Ctx &c, const double n[3], int g0, int a1, int it)
{
  const DevSys &s = c.s;
  if (worm_gap(c, a1, it)) return 0.0;
  size_t i0 = sidx(s, it, g0), i1 = sidx(s, it, a1);
  double dx = c.st.x[i0] - c.st.x[i1], dy = c.st.y[i0] - c.st.y[i1], dz = c.st.z[i0] - c.st.z[i1];
  double dr2 = 0.0;
  dr2 += dx * dx;
  dr2 += dy * dy;
  dr2 += dz * dz;
  double r = sqrt(dr2);
  double cost = 0.0;
  cost += n[0] * dx;
  cost += n[1] * dy;
  cost += n[2] * dz;
  cost /= r;
  cost *= -1.0;
  return lpot2d(c.t, r, cost);
}

__device__ __forceinline__ float rotlin_term32(const Ctx &c, const float n[3], int g0, int a1, int it)
{
  const DevSys &s = c.s;
  if (worm_gap(c, a1, it)) return 0.0f;
  size_t i0 = sidx(s, it, g0), i1 = sidx(s, it, a1);
  const float4 p0 = c.st.b4[i0], p1 = c.st.b4[i1];
  float dx = p0.x - p1.x, dy = p0.y - p1.y, dz = p0.z - p1.z;
  float r = sqrtf(dx * dx + dy * dy + dz * dz);
  float cost = -(n[0] * dx + n[1] * dy + n[2] * dz) / r;
  return lpot2d32(c.t, r, cost);
}

// link density of two neighbouring rotational slices: rotden's rho
// (rotden.f:1-31) or rsrot's log-density for a top, SRotDens(n.n') or
// rsline's for a linear rotor (mc_piqmc.cc:838-847, 1021-1035)
__device__ __forceinline__ double link_density(const Ctx &c, bool linear, const Frame &a, const Frame &b,
                                               const double *na, const double *nb, int *bad)
{
  const DevSys &s = c.s;
  double rho = 0.0, erot = 0.0;
  if (linear) {
    double p = 0.0;
    for (int d = 0; d < 3; d++) p += (na[d] * nb[d]);
    if (s.rot_den_type == 0) rho = srotdens(c.t, p, 0);
    else rsline(s.abc[0], p, s.rot_tau, &rho, &erot);
  } else {
    if (s.rot_den_type == 0) rho = rotden_rho(c.t, a, b, bad, nullptr, nullptr);
    else rsrot(a, b, s.abc, s.rot_tau, s.rot_odevn, &rho, &erot);
  }
  return rho;
}

// fmod(x, 2 pi) for the proposal's angles: on [2 pi, 4 pi) the remainder
// x - 2 pi is exact (Sterbenz), so the subtraction equals the library call
__device__ __forceinline__ double fmod_2pi(double x, double pi2)
{
  if (x >= 0.0 && x < pi2) return x;
  if (x >= pi2 && x < 2.0 * pi2) return x - pi2;
  return fmod(x, pi2);
}

// the proposal of MCRotLinStep (mc_piqmc.cc:801-820) / MCRot3Dstep
// (mc_piqmc.cc:955-1001): out = (phi, cos theta, chi).  Each product and sum
// rounded on its own (no fused multiply-add), as the reference's source
// states them, so that every kernel that inlines this makes the same
// proposal to the last bit.
__device__ __forceinline__ void rot_propose(const DevSys &s, bool linear, double phi, double cost, double chi,
                                            const double u[4], double out[3])
{
  if (linear) {
    cost = __dadd_rn(cost, __dmul_rn(s.rtstep, __dsub_rn(u[0], 0.5)));
    phi = __dadd_rn(phi, __dmul_rn(s.rtstep, __dsub_rn(u[1], 0.5)));
    if (cost > 1.0) cost = 2.0 - cost;
    if (cost < -1.0) cost = -2.0 - cost;
  } else {
    const double pi2 = 2.0 * PIMC_PI;
    cost = __dadd_rn(cost, __dmul_rn(s.rtstep, __dsub_rn(u[0], 0.5)));
    phi = __dadd_rn(phi, __dmul_rn(2.0 * PIMC_PI, __dmul_rn(s.rtstep, __dsub_rn(u[1], 0.5))));
    chi = __dadd_rn(chi, __dmul_rn(2.0 * PIMC_PI, __dmul_rn(s.rtstep, __dsub_rn(u[2], 0.5))));
    if (phi < 0.0) phi = pi2 + phi;
    if (chi < 0.0) chi = pi2 + chi;
    phi = fmod_2pi(phi, pi2);
    chi = fmod_2pi(chi, pi2);
    if (cost > 1.0) cost = 2.0 - cost;
    if (cost < -1.0) cost = -2.0 - cost;
  }
  out[0] = phi;
  out[1] = cost;
  out[2] = chi;
}

// the unit vector of (phi, cos theta) as the accept blocks write MCCosine
__device__ __forceinline__ void unit_vector(double phi, double cost, double v[3])
{
  double sint = sqrt(1.0 - cost * cost);
  v[0] = sint * cos(phi);
  v[1] = sint * sin(phi);
  v[2] = cost;
}

// uniforms of a production rotational move: pair index p = q / 2
__device__ __forceinline__ void rot_uniforms(uint64_t seed, unsigned pass, unsigned phase, int p, int r, bool linear,
                                             double u[4])
{
  uint64_t mv = ((uint64_t)pass << 32) | ((uint64_t)phase << 12) | (uint64_t)p;
  double a, b;
  philox_u2(seed, mv, 0x400000u | (uint32_t)r, 0u, &a, &b);
  u[0] = a; u[1] = b;
  philox_u2(seed, mv, 0x400000u | (uint32_t)r, 1u, &a, &b);
  u[2] = a; u[3] = b;
  if (linear) u[2] = u[3];
}

// Production draws.  FP64 path: rot_uniforms + rot_propose.  FP32 path: the
// uniforms at float resolution (philox_u2f) and the proposal's increments
// in float, added to the double angles (the path stays double); the
// reference's reflection and wrap on the double angles.
template <bool MIX>
__device__ __forceinline__ void rot_uniforms_t(uint64_t seed, unsigned pass, unsigned phase, int p, int r,
                                               bool linear, double u[4])
{
  if (!MIX) {
    rot_uniforms(seed, pass, phase, p, r, linear, u);
    return;
  }
  uint64_t mv = ((uint64_t)pass << 32) | ((uint64_t)phase << 12) | (uint64_t)p;
  float a, b;
  philox_u2f(seed, mv, 0x400000u | (uint32_t)r, 0u, &a, &b);
  u[0] = (double)a; u[1] = (double)b;
  philox_u2f(seed, mv, 0x400000u | (uint32_t)r, 1u, &a, &b);
  u[2] = (double)a; u[3] = (double)b;
  if (linear) u[2] = u[3];
}

template <bool MIX>
__device__ __forceinline__ void rot_propose_t(const DevSys &s, bool linear, double phi, double cost, double chi,
                                              const double u[4], double out[3])
{
  if (!MIX) {
    rot_propose(s, linear, phi, cost, chi, u, out);
    return;
  }
  const float st = (float)s.rtstep;
  if (linear) {
    cost += (double)(st * ((float)u[0] - 0.5f));
    phi += (double)(st * ((float)u[1] - 0.5f));
    if (cost > 1.0) cost = 2.0 - cost;
    if (cost < -1.0) cost = -2.0 - cost;
  } else {
    const double pi2 = 2.0 * PIMC_PI;
    const float tp = 6.28318530717959f * st;
    cost += (double)(st * ((float)u[0] - 0.5f));
    phi += (double)(tp * ((float)u[1] - 0.5f));
    chi += (double)(tp * ((float)u[2] - 0.5f));
    if (phi < 0.0) phi = pi2 + phi;
    if (chi < 0.0) chi = pi2 + chi;
    phi = fmod_2pi(phi, pi2);
    chi = fmod_2pi(chi, pi2);
    if (cost > 1.0) cost = 2.0 - cost;
    if (cost < -1.0) cost = -2.0 - cost;
  }
  out[0] = phi;
  out[1] = cost;
  out[2] = chi;
}

// The acceptance of a rotational move from its four link densities (old
// (q-1,q), old (q,q+1), new, new), the potentials, the Boltzmann factor
// boltz = exp(-tau (pot_new - pot_old)) (Noya densities) or its exponent
// (RS densities) and log u (RS): MCRotLinStep mc_piqmc.cc:838-921,
// MCRot3Dstep mc_piqmc.cc:1021-1178.  Returns 1 if accepted; *neg is set for a
// negative linear-rotor density (the reference's nrerror).
template <bool MIX>
__device__ __forceinline__ int rot_decide(const DevSys &s, bool linear, const double rho[4], double pot_old,
                                          double pot_new, double boltz, double logu, const double u[4], double *rd_out,
                                          int *neg_out, bool need_rd = true)
{
  double rd;
  int acc = 0, neg = 0;
  if (MIX && s.rot_den_type == 0) {
    // the FP32 path: the table densities and their ratio in float
    float dens_old = (float)rho[0] * (float)rho[1], dens_new = (float)rho[2] * (float)rho[3];
    if (fabsf(dens_old) < (float)PIMC_RZERO) dens_old = 0.0f;
    if (fabsf(dens_new) < (float)PIMC_RZERO) dens_new = 0.0f;
    if (linear) {
      if (dens_old < 0.0f || dens_new < 0.0f) neg = 1;
    } else {
      dens_old = fabsf(dens_old);
      dens_new = fabsf(dens_new);
    }
    float rf = (dens_old > (float)PIMC_RZERO) ? dens_new / dens_old : 1.0f;
    // boltz holds the exponent -tau (pot_new - pot_old) here: the test in
    // double as log(ratio) + exponent against 0 and log u
    double lr = (rf > 0.0f) ? (double)logf(rf) + boltz : -1.0e300;
    acc = (lr > 0.0) || (lr > logu);
    rd = need_rd ? (double)rf * exp(boltz) : 0.0;
  } else if (MIX && !linear) {
    // the FP32 path with rattle-and-shake densities (float log-densities):
    // their difference in float, the test in double against 0 and log u
    float rhoold = (float)rho[0] + (float)rho[1], rhonew = (float)rho[2] + (float)rho[3];
    rd = (double)((rhonew - rhoold) * s.rs_scale) + boltz;    // boltz: - tau (pot_new - pot_old)
    acc = (rd > 0.0) || (rd > logu);
  } else if (s.rot_den_type == 0) {
    double dens_old = rho[0] * rho[1], dens_new = rho[2] * rho[3];
    if (fabs(dens_old) < PIMC_RZERO) dens_old = 0.0;
    if (fabs(dens_new) < PIMC_RZERO) dens_new = 0.0;
    if (linear) {
      if (dens_old < 0.0 || dens_new < 0.0) neg = 1;          // mc_piqmc.cc:850,886
    } else {
      if (dens_old < 0.0) dens_old = fabs(dens_old);          // mc_piqmc.cc:1067,1133
      if (dens_new < 0.0) dens_new = fabs(dens_new);
    }
    rd = (dens_old > PIMC_RZERO) ? dens_new / dens_old : 1.0;
    rd *= boltz;                                              // exp(-tau (pot_new - pot_old))
    acc = (rd > 1.0) || (rd > u[linear ? 2 : 3]);
  } else if (linear) {
    double dens_old = rho[0] + rho[1], dens_new = rho[2] + rho[3];
    if (fabs(dens_old) < PIMC_RZERO) dens_old = 0.0;
    if (fabs(dens_new) < PIMC_RZERO) dens_new = 0.0;
    rd = dens_new - dens_old + boltz;                         // - tau (pot_new - pot_old)
    acc = (rd > 0.0) || (rd > logu);
  } else {
    double rhoold = rho[0] + rho[1], rhonew = rho[2] + rho[3];
    rd = (rhonew - rhoold) / (4.0 * (s.rot_tau / PIMC_WNO2K));
    rd += boltz;                                              // - tau (pot_new - pot_old)
    acc = (rd > 0.0) || (rd > logu);
  }
  (void)pot_old;
  (void)pot_new;
  *rd_out = rd;
  *neg_out = neg;
  return acc;
}

// Boltzmann factor (FP64 path, Noya densities) or its exponent (FP32 path,
// or RS densities) of a move, and log u of its accept uniform
template <bool MIX>
__device__ __forceinline__ double rot_boltz(const DevSys &s, double pot_old, double pot_new)
{
  return (!MIX && s.rot_den_type == 0) ? exp(-s.tau * (pot_new - pot_old)) : -(s.tau * (pot_new - pot_old));
}
template <bool MIX>
__device__ __forceinline__ double rot_logu(const DevSys &s, double u)
{
  if (MIX) return (double)logf((float)u);
  return (s.rot_den_type != 0) ? log(u) : 0.0;
}

// A linear rotor on the FP32 path with the float density spline keeps its
// orientation as the angles plus the float unit vector (MCCosine in float);
// the double MCCosine is derived from the angles afterwards
// (k_refresh_frames), like a top's double frame.
__device__ __forceinline__ bool lazy_linear(const Ctx &c, bool mix)
{
  return mix && c.s.rot_den_type == 0 && c.t.rd4 != nullptr;
}

// MCRotLinStep (mc_piqmc.cc:781-936) / MCRot3Dstep (mc_piqmc.cc:938-1199),
// first stage, for rotor g0 at rotational slice q with uniforms u (3 for a
// linear rotor, 4 for a top) and the proposal prop = rot_propose(current
// angles, u); u and prop are read on thread 0 only.  Leaves in sh the
// proposal, its frame, and pot_old / pot_new (the old potential from the
// cache when it is valid; the cache holds exactly what a fresh evaluation
// gives).  All PIMC_ROT_THREADS threads call it.
template <bool MIX>
__device__ void rot_prepare(const Ctx &c, const Frame *frames, int g0, int q, const double u[4], const double prop[3],
                            bool linear, RotShared &sh, int pre = -1)
{
  const DevSys &s = c.s;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int Q = s.Q, R = s.R;
  const size_t n = (size_t)s.nrotors * Q;
  const int i1 = (g0 - s.rot_first) * Q + q;
  const bool need64 = !MIX;                     // proposal frame in double during the evaluation
  if (warp == 0) {
    // pre >= 0: the look-ahead of the previous move (FP64 path) built the
    // proposal's frame or unit vector in sh.nxt_fn / sh.nxt_nv[pre]
    if (lane == 0) {
      for (int k = 0; k < 4; k++) sh.u[k] = u[k];
      const double a[3] = {prop[0], prop[1], prop[2]};
      sh.ang_new[0] = a[0]; sh.ang_new[1] = a[1]; sh.ang_new[2] = a[2];
      if (linear) {
        if (MIX) {
          unit_vector32((float)a[0], (float)a[1], sh.nnewf);
        } else if (pre >= 0) {
          for (int d = 0; d < 3; d++) sh.nnew[d] = sh.nxt_nv[pre][d];
        } else {
          unit_vector(a[0], a[1], sh.nnew);
        }
      } else if (need64) {
        if (pre < 0) make_frame(a[0], a[1], a[2], sh.fn);
      } else {
        make_frame32((float)a[0], (float)a[1], (float)a[2], sh.fn.mf, &sh.fn.hzf);
      }
    }
    if (!linear && need64 && pre >= 0) copy_frame<false>(sh.fn, &sh.nxt_fn[pre], lane);
  } else if (warp == 1) {
    if (linear) {
      if (lane < 3) {
        sh.nv[1][lane] = c.st.cosv[lane * n + i1];
        sh.nvf[lane] = c.st.cosvf[lane * n + i1];
      }
    } else {
      copy_frame<false>(sh.fo[1], frames + i1, lane);
    }
  } else if (warp == 2) {
    if (lane == 0) {
      sh.pot_cached = c.st.rp_ok[i1];
      if (sh.pot_cached) sh.pot_c = c.st.rp_cache[i1];
    }
    if (lane < 2 * R) sh.skip[lane] = g0;
  } else if (warp == 3) {
    if (lane < 3) sh.ang_old[lane] = c.st.ang[lane * n + i1];
  }
  __syncthreads();
  if (warp < 8) {
    const int first = sh.pot_cached ? R : 0;
    const int nsl = 2 * R - first;
    if (linear) {
      if (MIX)
        slot_sums_group<PIMC_ROT_PAIR_THREADS, 2>(
            nsl, s.na, sh.skip,
            [&](int sl, int p) -> float {
              int k = sl + first;
              return rotlin_term32(c, k < R ? sh.nvf : sh.nnewf, g0, p, q * R + (k % R));
            },
            sh.valsf, sh.buf);
      else
        slot_sums_group<PIMC_ROT_PAIR_THREADS, 2>(
            nsl, s.na, sh.skip,
            [&](int sl, int p) -> double {
              int k = sl + first;
              return rotlin_term64(c, k < R ? sh.nv[1] : sh.nnew, g0, p, q * R + (k % R));
            },
            sh.vals, sh.buf);
    } else {
      if (MIX)
        slot_sums_group<PIMC_ROT_PAIR_THREADS, 2>(
            nsl, s.na, sh.skip,
            [&](int sl, int p) -> float {
              int k = sl + first;
              return rot3d_term32(c, frames, k < R ? sh.fo[1] : sh.fn, g0, p, q * R + (k % R));
            },
            sh.valsf, sh.buf);
      else
        slot_sums_group<PIMC_ROT_PAIR_THREADS, 2>(
            nsl, s.na, sh.skip,
            [&](int sl, int p) -> double {
              int k = sl + first;
              return rot3d_term64(c, frames, k < R ? sh.fo[1] : sh.fn, g0, p, q * R + (k % R));
            },
            sh.vals, sh.buf);
    }
    if (tid == 96) {
      // sums and the Boltzmann factor here, off the neighbour chain (on warp
      // 3: warps 0 and 8, which share an SM sub-partition, carry the other
      // serial stages)
      if (MIX) {
        float po = 0.0f, pn = 0.0f;
        if (sh.pot_cached) po = (float)sh.pot_c;
        else
          for (int k = 0; k < R; k++) po += sh.valsf[k];
        for (int k = 0; k < R; k++) pn += sh.valsf[R - first + k];
        sh.pot_old = sh.pot_cached ? sh.pot_c : (double)po;
        sh.pot_new = (double)pn;
        // the action difference in double precision; the test compares it in
        // the log domain (rot_decide)
        sh.boltz = rot_boltz<true>(s, sh.pot_old, sh.pot_new);
        sh.logu = rot_logu<true>(s, sh.u[linear ? 2 : 3]);
      } else {
        double pot_old = 0.0, pot_new = 0.0;
        if (sh.pot_cached) pot_old = sh.pot_c;
        else
          for (int k = 0; k < R; k++) pot_old += sh.vals[k];
        for (int k = 0; k < R; k++) pot_new += sh.vals[R - first + k];
        sh.pot_old = pot_old;
        sh.pot_new = pot_new;
        sh.boltz = (s.rot_den_type == 0) ? exp(-s.tau * (pot_new - pot_old)) : -(s.tau * (pot_new - pot_old));
        if (s.rot_den_type != 0) sh.logu = log(sh.u[linear ? 2 : 3]);
      }
    }
  } else if (warp == 9) {
    if (lane == 0 && linear && !lazy_linear(c, MIX)) {
      if (MIX) unit_vector(sh.ang_new[0], sh.ang_new[1], sh.cv);
      else for (int d = 0; d < 3; d++) sh.cv[d] = sh.nnew[d];
    }
  }
  __syncthreads();
}

// hooks of rot_finish for launches without neighbour waits
struct RotNoHooks {
  __device__ bool wait(int) { return true; }
  __device__ void published() {}
  __device__ void ahead(RotShared &, int) {}
};

// second stage of the move prepared in sh, on warp 8: hooks.wait(lane) on
// all lanes before the neighbours' state is read (false: leave the move
// undone and set sh.stop), hooks.published() on lane 0 after the commit;
// meanwhile warp 9 runs hooks.ahead(sh, lane) (the slice's next proposal).  COH
// reads the neighbours through L2 (persistent launches, where other CTAs
// write them).  All PIMC_ROT_THREADS threads call it; returns 1 if accepted.
template <bool MIX, bool COH, class Hooks>
__device__ int rot_finish(const Ctx &c, Frame *frames, int g0, int q, bool linear, RotShared &sh, double *rd_out,
                          Hooks &hooks, bool need_rd = false)
{
  const DevSys &s = c.s;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int Q = s.Q;
  const size_t n = (size_t)s.nrotors * Q;
  int q0 = q - 1, q2 = q + 1;
  if (q0 < 0) q0 += Q;
  if (q2 >= Q) q2 -= Q;
  const int r = g0 - s.rot_first;
  const int i0 = r * Q + q0, i1 = r * Q + q, i2 = r * Q + q2;
  const bool use_links = Q >= 3;                // link cache (with Q < 3 both links join the same two slices)
  const bool need64 = !MIX;
  const bool mf_only = MIX && !linear;          // densities read the float frames only
  if (warp == 8) {
    bool go = hooks.wait(lane);
    if (lane == 0) sh.stop = !go;
    if (go) {
      // the neighbours' orientations and the link cache, all loads issued together
      if (linear) {
        if (lane < 6) {
          int k = (lane < 3) ? 0 : 2, d = lane - (lane < 3 ? 0 : 3);
          size_t ii = d * n + (k == 0 ? i0 : i2);
          if (lazy_linear(c, MIX)) {
            float v = COH ? __ldcg(c.st.cosvf + ii) : c.st.cosvf[ii];
            if (k == 0) sh.nvf0[d] = v;
            else sh.nvf2[d] = v;
          } else {
            sh.nv[k][d] = ld_state<COH>(c.st.cosv + ii);
          }
        }
      } else if (mf_only) {
        // words of Frame::mf and Frame::hzf
        const int w0 = (int)(offsetof(Frame, mf) / 4), nw = 10;
        if (lane < 2 * nw) {
          const Frame *src = frames + (lane < nw ? i0 : i2);
          Frame &dst = sh.fo[lane < nw ? 0 : 2];
          int w = w0 + (lane < nw ? lane : lane - nw);
          reinterpret_cast<unsigned *>(&dst)[w] =
              COH ? __ldcg(reinterpret_cast<const unsigned *>(src) + w) : reinterpret_cast<const unsigned *>(src)[w];
        }
      } else {
        copy_frame<COH>(sh.fo[0], frames + i0, lane);
        copy_frame<COH>(sh.fo[2], frames + i2, lane);
      }
      if (lane >= 24 && lane < 28) {
        int k = lane - 24;                              // rl_ok i0, rl_ok i1, rl_cache i0, rl_cache i1
        int ii = (k & 1) ? i1 : i0;
        if (k < 2) sh.link_ok[k] = use_links && ld_state<COH>(c.st.rl_ok + ii);
        else sh.rho[k - 2] = use_links ? ld_state<COH>(c.st.rl_cache + ii) : 0.0;
      }
      if (lane == 0) sh.bad = 0;
      __syncwarp();
      // 0: (q-1, q) old, 1: (q, q+1) old, 2: (q-1, q) new, 3: (q, q+1) new
      if (!MIX && !linear && s.rot_den_type == 0) {
        // FP64 top, tabulated densities: density d on lanes 3d..3d+2
        const int d = lane / 3;
        const bool act = d < 4 && !(d < 2 && sh.link_ok[d]);
        const int dd = d < 4 ? d : 0;
        const Frame &fa = (dd == 0 || dd == 2) ? sh.fo[0] : (dd == 1 ? sh.fo[1] : sh.fn);
        const Frame &fb = (dd == 0) ? sh.fo[1] : (dd == 2 ? sh.fn : sh.fo[2]);
        int bad = 0;
        double rho = rotden_rho_lanes(c.t, fa.m, fb.m, lane, &bad);
        if (act && lane % 3 == 0) {
          sh.rho[d] = rho;
          if (bad) atomicOr(&sh.bad, 1);
        }
      } else if (lane < 4 && !(lane < 2 && sh.link_ok[lane])) {
        int bad = 0;
        double rho;
        if (linear) {
          if (MIX && c.t.rd4 && s.rot_den_type == 0) {
            // FP32 path: 1 - cos(gamma) from the float unit vectors, stable for small angles
            const float *fa = (lane == 0 || lane == 2) ? sh.nvf0 : (lane == 1 ? sh.nvf : sh.nnewf);
            const float *fb = (lane == 0) ? sh.nvf : (lane == 2 ? sh.nnewf : sh.nvf2);
            rho = (double)srotdens32(c.t, one_minus_dot32(fa, fb));
          } else {
            double nn[3];
            if (MIX) unit_vector(sh.ang_new[0], sh.ang_new[1], nn);
            else for (int d = 0; d < 3; d++) nn[d] = sh.nnew[d];
            const double *na = (lane == 0 || lane == 2) ? sh.nv[0] : (lane == 1 ? sh.nv[1] : nn);
            const double *nb = (lane == 0) ? sh.nv[1] : (lane == 2 ? nn : sh.nv[2]);
            rho = link_density(c, true, sh.fo[0], sh.fo[0], na, nb, &bad);
          }
        } else {
          const Frame &fa = (lane == 0 || lane == 2) ? sh.fo[0] : (lane == 1 ? sh.fo[1] : sh.fn);
          const Frame &fb = (lane == 0) ? sh.fo[1] : (lane == 2 ? sh.fn : sh.fo[2]);
          if (MIX && s.rot_den_type == 0) {
            rho = (double)rotden_rho32(c.t, fa.mf, fb.mf, &bad);
          } else if (MIX) {
            rho = s.rot_odevn == -1 ? (double)rsrot32(fa.mf, fb.mf, s.rs_coef) : 0.0;
          } else {
            rho = link_density(c, false, fa, fb, nullptr, nullptr, &bad);
          }
        }
        sh.rho[lane] = rho;
        if (bad) atomicOr(&sh.bad, 1);
      }
      __syncwarp();
      if (lane == 0) {
        const double pot_old = sh.pot_old, pot_new = sh.pot_new;
        double rd;
        int neg = 0;
        int acc = rot_decide<MIX>(s, linear, sh.rho, pot_old, pot_new, sh.boltz, sh.logu, sh.u, &rd, &neg,
                                  need_rd || rd_out != nullptr);
        if (neg) { atomicOr(c.st.err, (unsigned)DERR_NEG_DENSITY); acc = 0; }
        if (sh.bad) { atomicOr(c.st.err, (unsigned)DERR_GRID_RANGE); acc = 0; }
        sh.rd = rd;
        sh.acc = acc;
        if (rd_out) *rd_out = rd;
        if (acc) {
          c.st.ang[i1] = sh.ang_new[0];
          c.st.ang[n + i1] = sh.ang_new[1];
          if (linear) {
            if (lazy_linear(c, MIX)) {
              for (int d = 0; d < 3; d++) c.st.cosvf[d * n + i1] = sh.nnewf[d];
            } else {
              for (int d = 0; d < 3; d++) {
                c.st.cosv[d * n + i1] = sh.cv[d];
                c.st.cosvf[d * n + i1] = (float)sh.cv[d];
              }
            }
          } else {
            c.st.ang[2 * n + i1] = sh.ang_new[2];
            if (need64) {
              frames[i1] = sh.fn;
            } else {
              for (int k = 0; k < 9; k++) frames[i1].mf[k] = sh.fn.mf[k];
              frames[i1].hzf = sh.fn.hzf;
            }
            // the other rotors' potentials at slice q depend on this orientation
            for (int rr = 0; rr < s.nrotors; rr++)
              if (rr != r) c.st.rp_ok[rr * Q + q] = 0;
          }
        }
        c.st.rp_cache[i1] = acc ? pot_new : pot_old;
        c.st.rp_ok[i1] = 1;
        if (use_links && !sh.bad) {
          c.st.rl_cache[i0] = acc ? sh.rho[2] : sh.rho[0];
          c.st.rl_cache[i1] = acc ? sh.rho[3] : sh.rho[1];
          c.st.rl_ok[i0] = 1;
          c.st.rl_ok[i1] = 1;
        }
        hooks.published();
      }
    }
  } else if (warp == 9) {
    hooks.ahead(sh, lane);
  }
  __syncthreads();
  return sh.acc;
}

// the whole move: rot_prepare then rot_finish
template <bool MIX, bool COH>
__device__ int rot_step(const Ctx &c, Frame *frames, int g0, int q, const double u[4], const double prop[3],
                        bool linear, RotShared &sh, double *rd_out, bool need_rd = false)
{
  rot_prepare<MIX>(c, frames, g0, q, u, prop, linear, sh);
  RotNoHooks hk;
  return rot_finish<MIX, COH>(c, frames, g0, q, linear, sh, rd_out, hk, need_rd);
}

// ------------------------------------------------------ estimator terms
// GetKinEnergy (mc_estim.cc:876-937): |r(it) - r(it+1)|^2 of atom a, the
// last slice of a boson joined to the atom PIndex names
__device__ __forceinline__ double est_spring(const Ctx &c, int a, int it)
{
  const int P = c.s.P;
  const int type = atom_type(c.s, a), g = c.s.first[type];
  int a1 = a;
  if (c.s.stat[type] == 1 && it + 1 == P) a1 = g + c.st.pindex[a - g];
  size_t i0 = sidx(c.s, it, a), i1 = sidx(c.s, (it + 1) % P, a1);
  double d[3] = {c.st.x[i0] - c.st.x[i1], c.st.y[i0] - c.st.y[i1], c.st.z[i0] - c.st.z[i1]};
  double acc = 0.0;
  for (int k = 0; k < 3; k++) {
    if (c.s.minimage) d[k] -= c.s.box[k] * rint(d[k] / c.s.box[k]);
    acc += d[k] * d[k];
  }
  return acc;
}

// the pairs GetPotEnergy_Densities (mc_estim.cc:500-687) adds to the potential
__device__ __forceinline__ bool est_pair_counted(const Ctx &c, int a0, int a1)
{
  int ty0 = atom_type(c.s, a0), ty1 = atom_type(c.s, a1);
  int m0 = c.s.molecule[ty0], m1 = c.s.molecule[ty1];
  return (m0 == 1 || m1 == 1) || (m0 != m1) || (m0 == 2 && m1 == 2 && c.s.numb[c.s.imtype] > 1) ||
         (ty0 == ty1 && m0 == 0);
}

// GetRotE3D (mc_estim.cc:989-1096) link terms of (rotor, it0) = k and
// GetRotEnergy (mc_estim.cc:939-987) for the linear rotor:
// out = {srot, sesq, se_termsq, valid}
__device__ __forceinline__ void est_link(const Ctx &c, const Frame *frames, int k, double out[4])
{
  const int Q = c.s.Q, nr = c.s.nrotors;
  const int r = k / Q, it0 = k % Q;
  const bool linear = c.s.molecule[c.s.imtype] == 1;
  double srot = 0.0, sesq = 0.0, sts = 0.0;
  if (linear) {
    size_t n = (size_t)nr * Q;
    int t0 = r * Q + it0, t1 = r * Q + (it0 + 1) % Q;
    double p0 = 0.0;
    for (int d = 0; d < 3; d++) p0 += (c.st.cosv[d * n + t0] * c.st.cosv[d * n + t1]);
    if (c.s.rot_den_type == 0) {
      double rdens = srotdens(c.t, p0, 0);
      double dv = srotdens(c.t, p0, 1);
      if (fabs(rdens) > PIMC_RZERO) srot = dv / rdens;
      sts = (dv / rdens) * (dv / rdens);
      sesq = srotdens(c.t, p0, 2) / rdens;
    } else {
      double rho, erot;
      rsline(c.s.abc[0], p0, c.s.rot_tau, &rho, &erot);
      srot = rho;
    }
  } else {
    int skip = (c.s.rot_den_type == 0) ? 1 : c.s.rn_ratio;
    if (it0 % skip == 0) {
      const Frame &f1 = frames[r * Q + it0];
      const Frame &f2 = frames[r * Q + (it0 + skip) % Q];
      double rho = 0.0, erot = 0.0, esq = 0.0;
      int bad = 0;
      // the tabulated E and E^2 (rotden.f:28-29); a rattle-and-shake run
      // may have loaded no table, and then contributes 0 to ErotSQ
      if (c.t.rho) rho = rotden_rho(c.t, f1, f2, &bad, &erot, &esq);
      if (c.s.rot_den_type == 1 && c.s.rn_ratio == 1) {
        rsrot(f1, f2, c.s.abc, c.s.rot_tau, c.s.rot_odevn, &rho, &erot);
        srot = rho;
      } else
        srot = erot;
      sesq = esq;
      sts = erot * erot;
    }
  }
  out[0] = srot;
  out[1] = sesq;
  out[2] = sts;
  out[3] = 1.0;
}
