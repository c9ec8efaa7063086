// pimc_worm.cu -- the worm algorithm of mc_qworm.cc on one CTA
//
// MCWormMove (mc_qworm.cc:93-125) is a chain: for every atom of the worm
// type an open or close try, then an advance or recede try, then (bosons) a
// swap try, each depending on the last.  One CTA runs the whole call: thread
// 0 draws the random numbers in the reference's order and takes every
// decision; the Gaussian bridges (sample_middle, mc_qworm.cc:238-283) are
// built level by level by the whole CTA, each bead placed by its index in
// the reference's recursion order; and the potential sums over a segment --
// the slices of get_potential (mc_qworm.cc:402-422) or the new/old pairs of
// the swap (mc_qworm.cc:470-486) -- spread their (slice, partner) terms over
// the CTA, with the partner beads that lie in the worm's gap left out as
// PotEnergy leaves them out (WorldLine, mc_qworm.cc:553-575;
// mc_piqmc.cc:1816-1817).
#include "pimc_kernels.cuh"
#include "pimc_launch.h"

namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kMaxQ = 2 * (PIMC_WORM_MAXM + 1);   // the swap's new and old slices
#define PIMC_MAXNEIGHBORS 100                     // MAXNEIGHBORS (mc_qworm.cc:12)
constexpr int kTermCap = 2560;                    // (query, partner) terms held in shared memory
constexpr int kDrawCap = 32;                      // draws of each uniform stream held in shared memory
constexpr int kGaussCap = 640;                    // gauss() draws held in shared memory
constexpr int kPdCap = 512;                       // neighbour-table distances held in shared memory

struct WormShared {
  int exists, ira, masha, atom_i, atom_m;   // the worm (TPathWorm)
  int flag;                                  // a decision every thread reads
  int nq;                                    // potential queries of the current sum
  double qtot;                               // their total (query_sums)
  int qa[kMaxQ], qpit[kMaxQ];                // global atom and slice of each
  double qx[kMaxQ], qy[kMaxQ], qz[kMaxQ];    // the bead the atom sits on
  double qsum[kMaxQ];
  int stack[4];                              // the swap's accepted segment (it0, atomw, a0)
  int b_it0, b_len, b_a0, b_a2;              // the bridge bridge_block builds
  int adv, advance;                          // the advance/recede branch and its length
  long gbase;                                // first gauss() draw of the current bridge
  int gneed;                                 // its number of draws
  double gz[3 * (PIMC_WORM_MAXM + 1)];       // the draws, generated by all threads
  // bridge coefficients by segment length and split (s0 = len/2 or len - len/2):
  // the midpoint is bca r0 + bcb r2 + bcs g, i.e. (s2 r0 + s0 r2)/(s0 + s2)
  // + g / sqrt(gkin) of sample_middle (mc_qworm.cc:268-276)
  double bca[2][PIMC_WORM_MAXM + 2], bcb[2][PIMC_WORM_MAXM + 2], bcs[2][PIMC_WORM_MAXM + 2];
  double sqadv[PIMC_WORM_MAXM + 1];          // 1/sqrt(gvar) of qworm_advance (mc_qworm.cc:324-330)
  double pw15[PIMC_WORM_MAXM + 1];           // segm^(NDIM/2) of qw_open_prob (mc_qworm.cc:152)
  double sg3[3 * (PIMC_WORM_MAXM + 1)];      // a bridge's beads it0..it2 (newcoords)
  int qmode, qt0, qt1, qa0, qa1;             // the queries fill_queries builds
  int pw_atom, pw_pt0, pw_pt1, pw_segm, pw_t1; // the arguments of get_ptable
  int pcount;                                // candidates of the neighbour table
  double ptd[PIMC_MAXNEIGHBORS + 1], ptab[PIMC_MAXNEIGHBORS + 1];
  int pta[PIMC_MAXNEIGHBORS + 1];
  double qwtot[7], qwacc[7];                 // the worm's try/accept counters
  double term[kTermCap];                     // the (query, partner) terms of query_sums
  double dc[8 * kDrawCap];                   // the first draws of the uniform streams
  double gc[kGaussCap];                      // the first gauss() draws of the call
  double pd[kPdCap];                         // get_ptable's distances while numb <= kPdCap
};

struct WormSrc {
  const double *v[9];
  long n[9];
  long *pos;
  unsigned *err;
  // one draw of stream k: 0..2 nrnd1..3, 3..7 rnd1..5, 8 gauss's x1
  __device__ void init() {}
  __device__ void fill(double *, double *) const {}
  __device__ long gbase() const { return pos[8]; }
  __device__ double gauss_at(long i) const
  {
    if (i >= n[8]) {
      atomicOr(err, (unsigned)DERR_STREAM);
      return 0.0;
    }
    return v[8][i];
  }
  __device__ void gskip(long k) { pos[8] += k; }
  __device__ double take(int k)
  {
    long p = pos[k];
    if (p >= n[k]) {
      atomicOr(err, (unsigned)DERR_STREAM);
      return 0.5;
    }
    pos[k] = p + 1;
    return v[k][p];
  }
};

// the production draws: Philox keyed by (seed, pass, phase, stream k, count).
// The first kDrawCap draws of streams 0..7 and the first kGaussCap gauss()
// draws are generated by all threads at the start of the call (a call of N
// tries takes at most 2N from any one uniform stream; config 0 takes about
// 560 gauss() draws per call), so that the decision chain and the bridges
// read them from shared memory.
struct WormPhilox {
  uint64_t seed;
  const unsigned *pass;
  unsigned phase;
  uint64_t move;
  unsigned cnt[9];
  const double *cache, *gcache;
  __device__ void init()
  {
    move = ((uint64_t)(*pass) << 32) | ((uint64_t)phase << 12) | 0xFFFu;
    for (int k = 0; k < 9; k++) cnt[k] = 0;
  }
  __device__ void fill(double *buf, double *gbuf)
  {
    for (int i = threadIdx.x; i < 8 * kDrawCap + kGaussCap; i += blockDim.x) {
      if (i < 8 * kDrawCap) buf[i] = draw(i / kDrawCap, (unsigned)(i % kDrawCap));
      else gbuf[i - 8 * kDrawCap] = draw(8, (unsigned)(i - 8 * kDrawCap));
    }
    cache = buf;
    gcache = gbuf;
  }
  __device__ double draw(int k, unsigned n) const
  {
    double u0, u1;
    philox_u2(seed, move, 0x500000u | ((uint32_t)k << 16) | (n & 0xFFFFu), n >> 16, &u0, &u1);
    if (k == 8) return sqrt(-log(u0)) * cos(2.0 * PIMC_PI * u1);   // gauss()'s x1 (mc_randg.cc:144)
    return u0;
  }
  __device__ double take(int k)
  {
    const unsigned n = cnt[k]++;
    return n < (unsigned)kDrawCap ? cache[k * kDrawCap + n] : draw(k, n);
  }
  __device__ long gbase() const { return cnt[8]; }
  __device__ double gauss_at(long i) const { return i < kGaussCap ? gcache[i] : draw(8, (unsigned)i); }
  __device__ void gskip(long k) { cnt[8] += (unsigned)k; }
};

template <class Src>
__device__ __forceinline__ int nrnd(Src &src, int k, int n) { return (int)floor(n * src.take(k)); }

// WorldLine (mc_qworm.cc:553-575) for atom index a of the worm type
__device__ __forceinline__ bool world_line(const WormShared &sh, int a, int pt)
{
  bool wline = true;
  if (a == sh.atom_m || a == sh.atom_i) {
    if (sh.atom_i != sh.atom_m || sh.ira > sh.masha) {
      if ((a == sh.atom_m && pt < sh.masha) || (a == sh.atom_i && pt > sh.ira)) wline = false;
    } else {
      if (pt > sh.ira && pt < sh.masha) wline = false;
    }
  }
  return wline;
}

// PotEnergy(qa[q], bead q, qpit[q]) for every query (mc_piqmc.cc:1201-1383).
// When the (query, partner) terms fit the shared buffer they are spread
// one per thread over the whole CTA (a warp per query would leave most
// lanes idle: a slice has few partners) and each query's terms are then
// summed in the partners' order; otherwise one warp per query, partners
// in a fixed per-lane order and a fixed shuffle tree.
__device__ __noinline__ double query_term(const Ctx &c, const Frame *frames, const DevWorm &wk,
                                             const WormShared &sh, int q, int a1)
{
  const int a0 = sh.qa[q], it = sh.qpit[q];
  if (a1 == a0) return 0.0;
  if (sh.exists && atom_type(c.s, a1) == wk.type && !world_line(sh, a1 - wk.first, it)) return 0.0;
  return pair_term64(c, frames, a0, a1, it, sh.qx[q], sh.qy[q], sh.qz[q]);
}

__device__ void query_sums(const Ctx &c, const Frame *frames, const DevWorm &wk, WormShared &sh)
{
  const int na = c.s.na, nq = sh.nq;
  if (nq * na <= kTermCap) {
    for (int k = threadIdx.x; k < nq * na; k += kThreads) sh.term[k] = query_term(c, frames, wk, sh, k / na, k % na);
    __syncthreads();
    for (int q = threadIdx.x; q < nq; q += kThreads) {
      double acc = 0.0;
      for (int a1 = 0; a1 < na; a1++) acc += sh.term[q * na + a1];
      sh.qsum[q] = acc;
    }
  } else {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int q = warp; q < nq; q += kWarps) {
      double acc = 0.0;
      for (int a1 = lane; a1 < na; a1 += 32) acc += query_term(c, frames, wk, sh, q, a1);
      for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
      if (lane == 0) sh.qsum[q] = acc;
    }
  }
  // the sum's total -- for the swap (mode 2) the new minus the old energies --
  // by warp 0 in a fixed lane order and shuffle tree
  __syncthreads();
  if (threadIdx.x < 32) {
    double acc = 0.0;
    for (int q = threadIdx.x; q < nq; q += 32) acc += (sh.qmode == 2 && (q & 1)) ? -sh.qsum[q] : sh.qsum[q];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (threadIdx.x == 0) sh.qtot = acc;
  }
}

__device__ __forceinline__ size_t bead(const Ctx &c, int gatom, int pit) { return sidx(c.s, pit, gatom); }

// The queries of a potential sum, filled by all threads from the
// description thread 0 left in sh.qmode/qt0/qt1/qa0/qa1.  Mode 0 and 1:
// get_potential(it0, it1, atom0, atom1, coords) (mc_qworm.cc:402-422), one
// query per inner slice, the bead on atom1 past the ring's end; mode 0 reads
// the path, mode 1 the bridge just built in sh.sg3 (based at it0).  Mode 2:
// the swap's new and old bead of every inner slice, in that order
// (mc_qworm.cc:470-486).
__device__ void fill_queries(const Ctx &c, const DevWorm &wk, WormShared &sh)
{
  const int P = c.s.P, it0 = sh.qt0, mode = sh.qmode;
  const int n = max(0, sh.qt1 - it0 - 1);
  const bool w0 = (it0 % P) == it0;
  for (int j = threadIdx.x; j < n; j += kThreads) {
    const int it = it0 + 1 + j, pit = it % P;
    const int g = wk.first + (((pit != it) && w0) ? sh.qa1 : sh.qa0);
    const size_t i = bead(c, g, pit);
    const double *b = sh.sg3 + 3 * (it - it0);
    if (mode == 2) {
      sh.qa[2 * j] = g; sh.qpit[2 * j] = pit;
      sh.qx[2 * j] = b[0]; sh.qy[2 * j] = b[1]; sh.qz[2 * j] = b[2];
      sh.qa[2 * j + 1] = g; sh.qpit[2 * j + 1] = pit;
      sh.qx[2 * j + 1] = c.st.x[i]; sh.qy[2 * j + 1] = c.st.y[i]; sh.qz[2 * j + 1] = c.st.z[i];
    } else {
      sh.qa[j] = g; sh.qpit[j] = pit;
      if (mode == 1) { sh.qx[j] = b[0]; sh.qy[j] = b[1]; sh.qz[j] = b[2]; }
      else { sh.qx[j] = c.st.x[i]; sh.qy[j] = c.st.y[i]; sh.qz[j] = c.st.z[i]; }
    }
  }
  if (threadIdx.x == 0) sh.nq = mode == 2 ? 2 * n : n;
}

__device__ __forceinline__ void set_queries(WormShared &sh, int mode, int it0, int it1, int atom0, int atom1)
{
  sh.qmode = mode; sh.qt0 = it0; sh.qt1 = it1; sh.qa0 = atom0; sh.qa1 = atom1;
}

// rint(0.5 (t0 + t2)) of sample_middle (mc_qworm.cc:245) in integers:
// a half rounds to the even neighbour
__device__ __forceinline__ int bridge_split(int t0, int t2)
{
  const int sum = t0 + t2, h = sum >> 1;
  return (sum & 1) && (h & 1) ? h + 1 : h;
}

// sample_middle(it0, it2, atom0, atom2, coords) (mc_qworm.cc:238-283) by all
// threads, for the bridge thread 0 left in sh.b_* with its end beads in
// sh.sg3[0] and sh.sg3[3 len].  The reference's recursion takes the middle
// bead, then the left half, then the right half, drawing three gauss()
// values per middle bead; the bead that is the middle of the sub-interval
// (lo, hi) is therefore the k-th drawn, k its pre-order index (the left
// child of node k is k + 1, the right one k + mid - lo).  Each thread takes
// one coordinate of one inner bead, finds its sub-interval by descending
// from (0, len), and the beads are built level by level:
// (s2 r_lo + s0 r_hi)/(s0 + s2) + g sqrt(twave2 s0 s2/(s0 + s2)), s0 = mid - lo,
// s2 = hi - mid, from the per-length coefficient table.  The draws start at
// sh.gz[goff].  to_path writes the inner beads to the path, the ones past the
// ring's end on atom2.
__device__ void bridge_block(const Ctx &c, const DevWorm &wk, WormShared &sh, int goff, bool to_path)
{
  const int it0 = sh.b_it0, len = sh.b_len;
  const int j = threadIdx.x, t = 1 + j / 3, d = j % 3;
  const bool mine = j < 3 * (len - 1);
  int lo = 0, hi = len, mid = 0, k = 0, depth = 0;
  if (mine) {
    for (;;) {
      mid = bridge_split(it0 + lo, it0 + hi) - it0;
      if (t == mid) break;
      if (t < mid) { hi = mid; k += 1; }
      else { k += mid - lo; lo = mid; }
      depth++;
    }
  }
  for (int lev = 0;; lev++) {
    if (mine && depth == lev) {
      const int ln = hi - lo, w = (mid - lo == (ln >> 1)) ? 0 : 1;
      sh.sg3[3 * t + d] = fma(sh.bcs[w][ln], sh.gz[goff + 3 * k + d],
                              sh.bca[w][ln] * sh.sg3[3 * lo + d] + sh.bcb[w][ln] * sh.sg3[3 * hi + d]);
    }
    if (!__syncthreads_or(mine && depth > lev)) break;
  }
  if (to_path) {
    const int P = c.s.P;
    const bool w0 = (it0 % P) == it0;
    for (int b = 1 + threadIdx.x; b < len; b += kThreads) {
      const int it = it0 + b, pit = it % P, a = ((pit != it) && w0) ? sh.b_a2 : sh.b_a0;
      const double *r = sh.sg3 + 3 * b;
      store_bead(c, bead(c, wk.first + a, pit), r[0], r[1], r[2]);
    }
  }
}

// thread 0: the end beads of a bridge of the path from (atom0, it0) to
// (atom2, it2), the far one copied from the path unless the caller set it
__device__ void bridge_ends(const Ctx &c, const DevWorm &wk, WormShared &sh, int it0, int it2, int atom0, int atom2,
                            bool have_end)
{
  const int P = c.s.P, len = it2 - it0;
  const size_t i0 = bead(c, wk.first + atom0, it0 % P);
  sh.sg3[0] = c.st.x[i0]; sh.sg3[1] = c.st.y[i0]; sh.sg3[2] = c.st.z[i0];
  if (!have_end) {
    const size_t i2 = bead(c, wk.first + atom2, it2 % P);
    sh.sg3[3 * len] = c.st.x[i2]; sh.sg3[3 * len + 1] = c.st.y[i2]; sh.sg3[3 * len + 2] = c.st.z[i2];
  }
  sh.b_it0 = it0; sh.b_len = len; sh.b_a0 = atom0; sh.b_a2 = atom2;
}

// the kinetic part of qw_open_prob (mc_qworm.cc:131-144) on thread 0
__device__ double open_kin(const Ctx &c, const DevWorm &wk, const WormShared &sh, int segm)
{
  size_t i0 = bead(c, wk.first + sh.atom_i, sh.ira), i1 = bead(c, wk.first + sh.atom_m, sh.masha);
  double r0[3] = {c.st.x[i0], c.st.y[i0], c.st.z[i0]}, r1[3] = {c.st.x[i1], c.st.y[i1], c.st.z[i1]};
  double kin = 0.0;
  for (int d = 0; d < 3; d++) {
    double dr = r0[d] - r1[d];
    if (c.s.minimage) dr -= (c.s.box[d] * rint(dr / c.s.box[d]));
    kin += (dr * dr);
  }
  return kin / (wk.twave2 * (double)segm);
}

// GetPTable (mc_qworm.cc:577-617) by all threads, with the arguments thread
// 0 left in sh.pw_*: every atom's squared distance to the worm bead in
// parallel (dall[a], -1 when the atom is no candidate), then each
// candidate's place in the stable order by distance -- the order mmsort's
// insertion sort gives (mc_utils.cc:206-230) -- as its rank; the first
// MAXNEIGHBORS go to sh.ptd/pta/ptab[1..] and sh.pcount holds the number of
// candidates.
__device__ void get_ptable(const Ctx &c, const DevWorm &wk, WormShared &sh, const int *rindex, double *gdall)
{
  double *dall = wk.numb <= kPdCap ? sh.pd : gdall;   // every rank reads all numb of them
  const int atomw = sh.pw_atom, pt0 = sh.pw_pt0, pt1 = sh.pw_pt1, segm = sh.pw_segm, t1 = sh.pw_t1;
  const size_t iw = bead(c, wk.first + atomw, pt0);
  const double rw[3] = {c.st.x[iw], c.st.y[iw], c.st.z[iw]};
  for (int a1 = threadIdx.x; a1 < wk.numb; a1 += kThreads) {
    double v = -1.0;
    if (world_line(sh, a1, pt1)) {
      int a0 = a1;
      if (t1 != pt1) a0 = rindex[a1];
      if (a0 != sh.atom_i) {
        const size_t i1 = bead(c, wk.first + a1, pt1);
        const double r1[3] = {c.st.x[i1], c.st.y[i1], c.st.z[i1]};
        double dr2 = 0.0;
        for (int d = 0; d < 3; d++) {
          double dx = rw[d] - r1[d];
          if (c.s.minimage) dx -= (c.s.box[d] * rint(dx / c.s.box[d]));
          dr2 += (dx * dx);
        }
        if (dr2 < wk.cut2) v = dr2;
      }
    }
    dall[a1] = v;
  }
  __syncthreads();
  // non-negative doubles order as their bit patterns do, so the ranks are
  // taken with integer compares (the FP64 pipe is the scarce one); -1 marks
  // a non-candidate and is negative as an integer too
  for (int a = threadIdx.x; a < wk.numb; a += kThreads) {
    const long long d = __double_as_longlong(dall[a]);
    if (d < 0) continue;
    atomicAdd(&sh.pcount, 1);
    int r = 0;
    for (int b = 0; b < wk.numb; b++) {
      const long long e = __double_as_longlong(dall[b]);
      r += (e >= 0) && (e < d || (e == d && b < a));
    }
    if (r < PIMC_MAXNEIGHBORS) { sh.ptd[r + 1] = __longlong_as_double(d); sh.pta[r + 1] = a; }
  }
  __syncthreads();
  const int count = min(sh.pcount, PIMC_MAXNEIGHBORS);
  const double norm = 1.0 / ((double)segm * wk.twave2);
  for (int ic = 1 + threadIdx.x; ic <= count; ic += kThreads) sh.ptab[ic] = exp(-norm * sh.ptd[ic]);
  __syncthreads();
}

// gauss() draws gbase .. gbase+gneed-1 of the next bridge, one per thread
// (thread 0 set gbase and gneed before the barrier)
template <class Src>
__device__ __forceinline__ void prefetch_gauss(const Src &src, WormShared &sh)
{
  __syncthreads();
  for (int j = threadIdx.x; j < sh.gneed; j += kThreads) sh.gz[j] = src.gauss_at(sh.gbase + j);
  __syncthreads();
}

template <class Src>
__global__ void __launch_bounds__(kThreads) k_worm_move(Ctx c, Frame *frames, DevWorm *wkp, int *rindex,
                                                       Src src, double *dall)
{
  __shared__ WormShared sh;
  __shared__ double pnorm_old;
  const DevWorm wk = *wkp;
  const int P = c.s.P;
  const bool t0 = threadIdx.x == 0;
  src.init();
  src.fill(sh.dc, sh.gc);
  for (int i = threadIdx.x; i < 2 * (PIMC_WORM_MAXM + 2); i += kThreads) {
    const int w = i / (PIMC_WORM_MAXM + 2), len = i % (PIMC_WORM_MAXM + 2);
    if (len >= 2) {
      const double s0 = (double)(w ? len - (len >> 1) : (len >> 1)), s2 = (double)len - s0;
      const double gkin = (s0 + s2) / (wk.twave2 * s0 * s2);
      sh.bca[w][len] = s2 / (s0 + s2);
      sh.bcb[w][len] = s0 / (s0 + s2);
      sh.bcs[w][len] = 1.0 / sqrt(gkin);
    }
  }
  for (int i = threadIdx.x; i <= PIMC_WORM_MAXM; i += kThreads) {
    sh.sqadv[i] = i > 0 ? 1.0 / sqrt(1.0 / ((double)i * wk.twave2)) : 0.0;
    sh.pw15[i] = (double)i * sqrt((double)i);
  }
  if (threadIdx.x < 7) {
    sh.qwtot[threadIdx.x] = wk.qwtot[threadIdx.x];
    sh.qwacc[threadIdx.x] = wk.qwacc[threadIdx.x];
  }
  if (t0) {
    sh.exists = wk.exists; sh.ira = wk.ira; sh.masha = wk.masha;
    sh.atom_i = wk.atom_i; sh.atom_m = wk.atom_m;
  }
  __syncthreads();
  const bool bose = c.s.stat[wk.type] == 1;      // PIMC_BOSE (pimc_types.h)
  for (int atom = 0; atom < wk.numb; atom++) {
    // ---------------- open (mc_qworm.cc:155-180) / close (:182-236)
    int segm = 0;
    if (t0) {
      sh.gneed = 0;
      if (sh.exists) {
        sh.qwtot[1] += 1.0;
        segm = sh.masha - sh.ira;
        if (segm < 0) segm += P;
        sh.flag = segm > wk.m ? 0 : 1;
        if (sh.flag && segm >= 2) sh.gneed = 3 * (segm - 1);
        sh.gbase = src.gbase();
      }
    }
    prefetch_gauss(src, sh);
    if (sh.exists && sh.flag) {          // close: the gap is bridged
      if (t0) {
        src.gskip(sh.gneed);
        bridge_ends(c, wk, sh, sh.ira, sh.ira + segm, sh.atom_i, sh.atom_m, false);
        set_queries(sh, 1, sh.ira, sh.ira + segm, sh.atom_i, sh.atom_m);
      }
      __syncthreads();
      bridge_block(c, wk, sh, 0, true);
    } else if (t0) {
      if (!sh.exists) {
        sh.qwtot[0] += 1.0;
        sh.atom_i = nrnd(src, 0, wk.numb);
        sh.ira = nrnd(src, 1, P);
        segm = nrnd(src, 2, wk.m) + 1;
        sh.masha = (sh.ira + segm) % P;
        sh.atom_m = sh.atom_i;
        if (sh.masha != (sh.ira + segm)) sh.atom_m = c.st.pindex[sh.atom_i];
        sh.flag = 2;
        set_queries(sh, 0, sh.ira, sh.ira + segm, sh.atom_i, sh.atom_m);
      }
    }
    __syncthreads();
    if (sh.flag) {
      fill_queries(c, wk, sh);
      __syncthreads();
      query_sums(c, frames, wk, sh);
      __syncthreads();
      if (t0) {
        double prob = wk.qw_norm * sh.pw15[segm] * exp(open_kin(c, wk, sh, segm) + sh.qtot * c.s.tau);
        if (sh.flag == 1) prob = 1.0 / prob;
        bool acc = false;
        if (prob >= 1.0) acc = true;
        else if (prob > src.take(3)) acc = true;
        if (acc) {
          if (sh.flag == 1) { sh.exists = 0; sh.qwacc[1] += 1.0; }
          else { sh.exists = 1; sh.qwacc[0] += 1.0; }
        }
      }
    }
    __syncthreads();   // every thread is past the reads of sh.flag / sh.exists above
    // ---------------- advance (mc_qworm.cc:295-355) / recede (:357-400)
    if (sh.exists) {
      int ira_new = 0, atomi_new = 0;
      if (t0) {
        double r = src.take(7);
        sh.adv = r > 0.5;
        sh.flag = 0;
        sh.gneed = 0;
        if (sh.adv) {
          sh.qwtot[4] += 1.0;
          int sg = sh.masha - sh.ira;
          if (sg < 0) sg += P;
          sh.advance = nrnd(src, 2, wk.m) + 1;
          if (sg - sh.advance > 0) sh.gneed = 3 * sh.advance;   // the end point, then the bridge
        }
        sh.gbase = src.gbase();
      }
      prefetch_gauss(src, sh);
      if (sh.adv && sh.gneed > 0) {      // advance: a new end bead and the bridge to it
        if (t0) {
          const int advance = sh.advance;
          src.gskip(sh.gneed);
          int it0 = sh.ira, it2 = sh.ira + advance;
          ira_new = it2 % P;
          atomi_new = sh.atom_i;
          if (ira_new != it2) atomi_new = sh.atom_m;
          // the new end bead: r0 + gauss(1/(advance twave2)) (mc_qworm.cc:324-330)
          size_t i0 = bead(c, wk.first + sh.atom_i, it0 % P);
          const double r0[3] = {c.st.x[i0], c.st.y[i0], c.st.z[i0]};
          double *r2 = sh.sg3 + 3 * advance;
          for (int d = 0; d < 3; d++) r2[d] = fma(sh.sqadv[advance], sh.gz[d], r0[d]);
          store_bead(c, bead(c, wk.first + atomi_new, it2 % P), r2[0], r2[1], r2[2]);
          bridge_ends(c, wk, sh, it0, it2, sh.atom_i, atomi_new, true);
          set_queries(sh, 1, it0, it2 + 1, sh.atom_i, atomi_new);
          sh.flag = 1;
        }
        __syncthreads();
        bridge_block(c, wk, sh, 3, true);
      } else if (t0) {
        if (!sh.adv) {
          sh.qwtot[5] += 1.0;
          int sg = sh.ira - sh.masha;
          if (sg < 0) sg += P;
          int recede = nrnd(src, 2, wk.m) + 1;
          if ((sg - recede) >= 1) {
            int it0 = sh.ira - recede, it1 = sh.ira;
            int a0 = sh.atom_i, a1 = sh.atom_i;
            if (it0 < 0) {
              it0 += P;
              it1 += P;
              a0 = rindex[a1];
            }
            ira_new = it0 % P;
            atomi_new = a0;
            set_queries(sh, 0, it0, it1 + 1, a0, a1);
            sh.flag = 2;
          }
        }
      }
      __syncthreads();
      if (sh.flag) {
        fill_queries(c, wk, sh);
        __syncthreads();
        query_sums(c, frames, wk, sh);
        __syncthreads();
        if (t0) {
          double pot = sh.qtot;
          bool acc = false;
          if (sh.flag == 1) {          // advance
            if (pot < 0.0) acc = true;
            else if (exp(-pot * c.s.tau) > src.take(4)) acc = true;
            if (acc) sh.qwacc[4] += 1.0;
          } else {                     // recede
            if (pot > 0.0) acc = true;
            else if (exp(pot * c.s.tau) > src.take(4)) acc = true;
            if (acc) sh.qwacc[5] += 1.0;
          }
          if (acc) {
            sh.ira = ira_new;
            sh.atom_i = atomi_new;
          }
        }
      }
    }
    __syncthreads();
    // ---------------- swap (mc_qworm.cc:424-551)
    if (bose && sh.exists) {
      int it0 = 0, it1 = 0, pit1 = 0, atomw = 0, a0 = 0, a1 = 0;
      double prob = 0.0;
      if (t0) {
        sh.qwtot[6] += 1.0;
        it0 = sh.ira;
        it1 = it0 + wk.m;
        pit1 = it1 % P;
        atomw = sh.atom_i;
        sh.pw_atom = atomw; sh.pw_pt0 = it0; sh.pw_pt1 = pit1; sh.pw_segm = wk.m; sh.pw_t1 = it1;
        sh.pcount = 0;
      }
      __syncthreads();
      get_ptable(c, wk, sh, rindex, dall);
      if (t0) {
        const int count = min(sh.pcount, PIMC_MAXNEIGHBORS);
        sh.flag = 0;
        if (count > 0) {
          double pn = 0.0;
          for (int ic = 1; ic <= count; ic++) pn += sh.ptab[ic];
          double prand = pn * src.take(5);
          double sum = 0.0;
          int ic = 1;
          while ((ic <= count) && (sum < prand)) {
            sum += sh.ptab[ic];
            ic++;
          }
          ic--;
          a1 = sh.pta[ic];
          pnorm_old = pn;
          a0 = a1;
          if (pit1 != it1) a0 = rindex[a1];
          sh.flag = 1;
        }
        sh.gneed = sh.flag && wk.m >= 2 ? 3 * (wk.m - 1) : 0;
        sh.gbase = src.gbase();
      }
      prefetch_gauss(src, sh);
      if (sh.flag) {
        if (t0) {
          src.gskip(sh.gneed);
          // newcoords: the end points, then the bridge between them
          bridge_ends(c, wk, sh, it0, it1, atomw, a1, false);
          // the new and the old energy of every inner slice, in that order
          set_queries(sh, 2, it0, it1, a0, a1);
        }
        __syncthreads();
        bridge_block(c, wk, sh, 0, false);
        fill_queries(c, wk, sh);
        __syncthreads();
        query_sums(c, frames, wk, sh);
        __syncthreads();
        if (t0) {
          prob = exp(-sh.qtot * c.s.tau);
          sh.pw_atom = a0; sh.pw_pt0 = it0; sh.pw_pt1 = pit1; sh.pw_segm = wk.m; sh.pw_t1 = it1;
          sh.pcount = 0;
        }
        __syncthreads();
        get_ptable(c, wk, sh, rindex, dall);
        if (t0) {
          const int count = min(sh.pcount, PIMC_MAXNEIGHBORS);
          double pn = 0.0;
          for (int ic = 1; ic <= count; ic++) pn += sh.ptab[ic];
          prob *= (pnorm_old / pn);
          bool acc = false;
          if (prob >= 1.0) acc = true;
          else if (prob > src.take(6)) acc = true;
          sh.flag = acc ? 1 : 0;
          if (acc) {
            sh.qwacc[6] += 1.0;
            int g = wk.first + a0;
            for (int it = it0 + 1; it < it1; it++) {
              int pit = it % P;
              if (pit != it) g = wk.first + a1;
              const double *b = sh.sg3 + 3 * (it - it0);
              store_bead(c, bead(c, g, pit), b[0], b[1], b[2]);
            }
            int ratomw = rindex[atomw], ratom0 = rindex[a0];
            c.st.pindex[ratomw] = a0;
            rindex[a0] = ratomw;
            c.st.pindex[ratom0] = atomw;
            rindex[atomw] = ratom0;
            if (sh.ira > sh.masha) {
              if (a0 == sh.atom_m) sh.atom_m = sh.atom_i;
              else if (sh.atom_i == sh.atom_m) sh.atom_m = a0;
            }
            sh.stack[0] = it0; sh.stack[1] = atomw; sh.stack[2] = a0;
          }
        }
        __syncthreads();
        if (sh.flag) {
          // the heads of the two paths up to it0 change places
          const int h0 = sh.stack[0], hw = sh.stack[1], ha = sh.stack[2];
          for (int it = threadIdx.x; it <= h0; it += kThreads) {
            size_t ia = bead(c, wk.first + ha, it), iw = bead(c, wk.first + hw, it);
            double xa = c.st.x[ia], ya = c.st.y[ia], za = c.st.z[ia];
            store_bead(c, ia, c.st.x[iw], c.st.y[iw], c.st.z[iw]);
            store_bead(c, iw, xa, ya, za);
          }
        }
      }
    }
    __syncthreads();
  }
  if (t0) {
    wkp->exists = sh.exists; wkp->ira = sh.ira; wkp->masha = sh.masha;
    wkp->atom_i = sh.atom_i; wkp->atom_m = sh.atom_m;
  }
  if (threadIdx.x < 7) {
    wkp->qwtot[threadIdx.x] = sh.qwtot[threadIdx.x];
    wkp->qwacc[threadIdx.x] = sh.qwacc[threadIdx.x];
  }
}

// MCMolecularMoveExchange (mc_piqmc.cc:104-192) for the boson type: each
// exchange cycle of the permutation is displaced rigidly by one uniform
// step; its atoms are tested in cycle order with their whole-path
// potential change (new beads against the old partner beads) and the cycle
// is kept when every atom passed.  One CTA: thread 0 walks the cycles and
// decides, all threads sum the (slice, partner) terms of the current atom.
// REPLAY takes rnd1()/rnd2() from the caller's streams; otherwise Philox
// keyed by (seed, pass, phase, first atom of the cycle).
constexpr int kMolThreads = 512;

template <bool REPLAY>
__global__ void __launch_bounds__(kMolThreads) k_mol_exchange(Ctx c, Frame *frames, int type, const DevWorm *gate,
                                                              ReplaySrc src, uint64_t seed, const unsigned *pass,
                                                              unsigned phase, int *cyc, char *flag,
                                                              unsigned long long *cnt)
{
  if (gate && gate->exists) return;          // the worm branch moves closed paths only (mc_main.cc:361)
  __shared__ double dd[3];
  __shared__ double wpart[2][kMolThreads / 32];
  __shared__ int ncyc, accepted, stop, perm_bad;
  const int numb = c.s.numb[type], g = c.s.first[type], P = c.s.P;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int a = tid; a < numb; a += kMolThreads) flag[a] = 0;
  __syncthreads();
  for (int atom = 0; atom < numb; atom++) {
    if (tid == 0) {
      ncyc = 0;
      perm_bad = 0;
      if (flag[atom] == 0) {
        cyc[ncyc++] = atom;
        int pa = c.st.pindex[atom];
        // a cycle of a permutation of [0, numb) closes within numb steps;
        // the host validates PIndex, and the walk is bounded all the same
        while (pa != atom) {
          if (ncyc >= numb || pa < 0 || pa >= numb) {
            atomicOr(c.st.err, (unsigned)DERR_PERM);
            perm_bad = 1;
            break;
          }
          cyc[ncyc++] = pa;
          flag[pa] = 1;
          pa = c.st.pindex[pa];
        }
        if (REPLAY) {
          for (int k = 0; k < 3; k++) dd[k] = c.s.mcstep[type] * (src.disp_u(k) - 0.5);
        } else {
          mol_disp(c.s, type, seed, *pass, phase, atom, dd);
        }
      }
      accepted = 1;
      stop = 0;
    }
    __syncthreads();
    if (perm_bad) return;                    // uniform over the CTA: nothing moved
    const int n = ncyc;
    for (int ia = 0; ia < n; ia++) {
      const int ga = g + cyc[ia];
      const double d0 = dd[0], d1 = dd[1], d2 = dd[2];
      double en = 0.0, eo = 0.0;
      // PotEnergy(gatom, pos) (mc_piqmc.cc:1201-1383): partners in order,
      // slices strided over the threads
      const long items = (long)c.s.na * P;
      for (long k = tid; k < items; k += kMolThreads) {
        int a1 = (int)(k / P), it = (int)(k % P);
        if (a1 == ga) continue;
        size_t i = sidx(c.s, it, ga);
        double x = c.st.x[i], y = c.st.y[i], z = c.st.z[i];
        eo += pair_term64(c, frames, ga, a1, it, x, y, z);
        en += pair_term64(c, frames, ga, a1, it, x + d0, y + d1, z + d2);
      }
      for (int o = 16; o > 0; o >>= 1) {
        en += __shfl_xor_sync(0xffffffffu, en, o);
        eo += __shfl_xor_sync(0xffffffffu, eo, o);
      }
      if (lane == 0) { wpart[0][warp] = en; wpart[1][warp] = eo; }
      __syncthreads();
      if (tid == 0) {
        double sn = 0.0, so = 0.0;
        for (int w = 0; w < kMolThreads / 32; w++) { sn += wpart[0][w]; so += wpart[1][w]; }
        double deltav = 0.0;
        deltav += (sn - so);
        bool acc = false;
        if (deltav < 0.0) acc = true;
        else {
          double u;
          if (REPLAY) u = src.accept_u(0);
          else {
            PhiloxSrc ps{seed, ((uint64_t)*pass << 32) | ((uint64_t)phase << 12) | (uint64_t)atom};
            u = ps.accept_u(ia);
          }
          if (exp(-deltav * c.s.tau) > u) acc = true;
        }
        accepted = acc ? 1 : 0;
        if (!acc) stop = 1;
      }
      __syncthreads();
      if (stop) break;
    }
    if (n > 0) {
      if (tid == 0) {
        cnt[(type * 3 + 0) * 2] += 1;
        if (accepted) cnt[(type * 3 + 0) * 2 + 1] += 1;
      }
      if (accepted) {
        const double d0 = dd[0], d1 = dd[1], d2 = dd[2];
        for (long k = tid; k < (long)n * P; k += kMolThreads) {
          int ia = (int)(k / P), it = (int)(k % P);
          size_t i = sidx(c.s, it, g + cyc[ia]);
          store_bead(c, i, c.st.x[i] + d0, c.st.y[i] + d1, c.st.z[i] + d2);
        }
      }
    }
    __syncthreads();
  }
}

// The bisection of one start slice for every atom of a type in turn, as
// PIMCPass calls it (mc_main.cc:510-522) and, with gate set, as the worm
// branch calls it while the worm is closed, at a slice drawn like nrnd2
// (mc_main.cc:361-369); exch 1 joins the rows through the permutation.
template <bool MIX>
__global__ void __launch_bounds__(PIMC_BIS_THREADS) k_bisect_slice(Ctx c, Frame *frames, int type, int time0, int exch,
                                                                const DevWorm *gate, uint64_t seed,
                                                                const unsigned *pass, unsigned phase,
                                                                unsigned long long *cnt)
{
  __shared__ BisectShared sh;
  __shared__ int t0s;
  if (gate && gate->exists) return;
  if (threadIdx.x == 0) {
    t0s = time0;
    if (gate) {
      PhiloxSrc ps{seed, ((uint64_t)(*pass) << 32) | ((uint64_t)phase << 12) | 0xFFFu};
      t0s = min(c.s.P - 1, (int)floor(c.s.P * ps.accept_u(9)));
    }
  }
  __syncthreads();
  for (int atom = 0; atom < c.s.numb[type]; atom++) {
    PhiloxSrc src{seed, ((uint64_t)(*pass) << 32) | ((uint64_t)phase << 12) | (uint64_t)atom};
    int acc = bisect_move<MIX>(c, frames, type, atom, t0s, exch, src, sh, nullptr);
    if (threadIdx.x == 0) {
      cnt[(type * 3 + 1) * 2 + 0] += 1;
      if (acc) cnt[(type * 3 + 1) * 2 + 1] += 1;
    }
    __syncthreads();
  }
}

}  // namespace

int launch_mol_exchange(const Ctx &c, Frame *f, int type, bool replay, ReplaySrc src, uint64_t seed,
                        const unsigned *pass, unsigned phase, void *scratch, unsigned long long *cnt, cudaStream_t s,
                        const DevWorm *gate)
{
  int numb = c.s.numb[type];
  int *cyc = (int *)scratch;
  char *flag = (char *)(cyc + numb);
  if (replay)
    k_mol_exchange<true><<<1, kMolThreads, 0, s>>>(c, f, type, gate, src, seed, pass, phase, cyc, flag, cnt);
  else
    k_mol_exchange<false><<<1, kMolThreads, 0, s>>>(c, f, type, gate, src, seed, pass, phase, cyc, flag, cnt);
  return 1;
}

int launch_bisect_slice(const Ctx &c, Frame *f, int type, int time0, int exch, const DevWorm *gate, uint64_t seed,
                        const unsigned *pass, unsigned phase, unsigned long long *cnt, cudaStream_t s)
{
  if (c.s.mixed)
    k_bisect_slice<true><<<1, PIMC_BIS_THREADS, 0, s>>>(c, f, type, time0, exch, gate, seed, pass, phase, cnt);
  else
    k_bisect_slice<false><<<1, PIMC_BIS_THREADS, 0, s>>>(c, f, type, time0, exch, gate, seed, pass, phase, cnt);
  return 1;
}

void launch_worm_prod(const Ctx &c, Frame *f, DevWorm *wk, int *rindex, uint64_t seed, const unsigned *pass,
                      unsigned phase, void *scratch, int numb, cudaStream_t s)
{
  WormPhilox src;
  src.seed = seed;
  src.pass = pass;
  src.phase = phase;
  double *dall = (double *)scratch;
  Ctx cw = c;
  cw.st.worm = nullptr;
  k_worm_move<WormPhilox><<<1, kThreads, 0, s>>>(cw, f, wk, rindex, src, dall);
}

size_t worm_scratch_bytes(int numb) { return sizeof(double) * (size_t)(numb + 1) + 64; }

void launch_worm_move(const Ctx &c, Frame *f, DevWorm *wk, int *rindex, const double *const *streams,
                      const long *lengths, long *cursors, void *scratch, int numb, cudaStream_t s)
{
  WormSrc src;
  for (int k = 0; k < 9; k++) { src.v[k] = streams[k]; src.n[k] = lengths[k]; }
  src.pos = cursors;
  src.err = c.st.err;
  double *dall = (double *)scratch;
  Ctx cw = c;
  cw.st.worm = nullptr;      // the kernel masks from its own copy of the worm
  k_worm_move<WormSrc><<<1, kThreads, 0, s>>>(cw, f, wk, rindex, src, dall);
}
