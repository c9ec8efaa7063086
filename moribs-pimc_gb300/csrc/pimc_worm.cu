// pimc_worm.cu -- the worm algorithm of mc_qworm.cc on one CTA
//
// MCWormMove (mc_qworm.cc:93-125) is a chain: for every atom of the worm
// type an open or close try, then an advance or recede try, then (bosons) a
// swap try, each depending on the last.  One CTA runs the whole call: thread
// 0 draws the random numbers in the reference's order and takes every
// decision, the Gaussian bridges (sample_middle, mc_qworm.cc:238-283) are
// built on thread 0 in the reference's recursion order, and the potential
// sums over a segment -- the slices of get_potential (mc_qworm.cc:402-422)
// or the new/old pairs of the swap (mc_qworm.cc:470-486) -- run one warp
// per slice over the partners, with the partner beads that lie in the
// worm's gap left out as PotEnergy leaves them out (WorldLine,
// mc_qworm.cc:553-575; mc_piqmc.cc:1816-1817).
#include "pimc_kernels.cuh"
#include "pimc_launch.h"

namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kMaxQ = 2 * (PIMC_WORM_MAXM + 1);   // the swap's new and old slices

struct WormShared {
  int exists, ira, masha, atom_i, atom_m;   // the worm (TPathWorm)
  int flag;                                  // a decision every thread reads
  int nq;                                    // potential queries of the current sum
  int qa[kMaxQ], qpit[kMaxQ];                // global atom and slice of each
  double qx[kMaxQ], qy[kMaxQ], qz[kMaxQ];    // the bead the atom sits on
  double qsum[kMaxQ];
  int stack[4 * 32];                         // sample_middle's recursion
  long gbase;                                // first gauss() draw of the current bridge
  int gneed;                                 // its number of draws
  double gz[3 * (PIMC_WORM_MAXM + 1)];       // the draws, generated by all threads
};

struct WormSrc {
  const double *v[9];
  long n[9];
  long *pos;
  unsigned *err;
  // one draw of stream k: 0..2 nrnd1..3, 3..7 rnd1..5, 8 gauss's x1
  __device__ void init() {}
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

// the production draws: Philox keyed by (seed, pass, phase, stream k, count)
struct WormPhilox {
  uint64_t seed;
  const unsigned *pass;
  unsigned phase;
  uint64_t move;
  unsigned cnt[9];
  __device__ void init()
  {
    move = ((uint64_t)(*pass) << 32) | ((uint64_t)phase << 12) | 0xFFFu;
    for (int k = 0; k < 9; k++) cnt[k] = 0;
  }
  __device__ double draw(int k, unsigned n) const
  {
    double u0, u1;
    philox_u2(seed, move, 0x500000u | ((uint32_t)k << 16) | (n & 0xFFFFu), n >> 16, &u0, &u1);
    if (k == 8) return sqrt(-log(u0)) * cos(2.0 * PIMC_PI * u1);   // gauss()'s x1 (mc_randg.cc:144)
    return u0;
  }
  __device__ double take(int k) { return draw(k, cnt[k]++); }
  __device__ long gbase() const { return cnt[8]; }
  __device__ double gauss_at(long i) const { return draw(8, (unsigned)i); }
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

// PotEnergy(qa[q], bead q, qpit[q]) for every query, one warp per query,
// partners in a fixed per-lane order and a fixed shuffle tree
__device__ void query_sums(const Ctx &c, const Frame *frames, const DevWorm &wk, WormShared &sh)
{
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int q = warp; q < sh.nq; q += kWarps) {
    int a0 = sh.qa[q], it = sh.qpit[q];
    double acc = 0.0;
    for (int a1 = lane; a1 < c.s.na; a1 += 32) {
      if (a1 == a0) continue;
      if (sh.exists && atom_type(c.s, a1) == wk.type && !world_line(sh, a1 - wk.first, it)) continue;
      acc += pair_term64(c, frames, a0, a1, it, sh.qx[q], sh.qy[q], sh.qz[q]);
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) sh.qsum[q] = acc;
  }
}

__device__ __forceinline__ size_t bead(const Ctx &c, int gatom, int pit) { return sidx(c.s, pit, gatom); }

// the queries of get_potential(it0, it1, atom0, atom1, MCCoords)
__device__ void potential_queries(const Ctx &c, const DevWorm &wk, WormShared &sh, int it0, int it1, int atom0,
                                  int atom1)
{
  const int P = c.s.P;
  int pit0 = it0 % P;
  int atom = atom0, nq = 0;
  for (int it = it0 + 1; it < it1; it++) {
    int pit = it % P;
    if ((pit != it) && (pit0 == it0)) atom = atom1;
    int g = wk.first + atom;
    size_t i = bead(c, g, pit);
    sh.qa[nq] = g;
    sh.qpit[nq] = pit;
    sh.qx[nq] = c.st.x[i];
    sh.qy[nq] = c.st.y[i];
    sh.qz[nq] = c.st.z[i];
    nq++;
  }
  sh.nq = nq;
}

__device__ double potential_total(const WormShared &sh)
{
  double pot = 0.0;
  for (int q = 0; q < sh.nq; q++) pot += sh.qsum[q];
  return pot;
}

// sample_middle(it0, it2, atom0, atom2, coords) on thread 0: the
// reference's recursion (middle bead, then the left half, then the right
// half) with an explicit stack.  seg != nullptr writes the segment copy
// seg[3][it - base] (newcoords of the swap) instead of the path.
__device__ void sample_middle(const Ctx &c, const DevWorm &wk, WormShared &sh, int &gi, int it0, int it2,
                              int atom0, int atom2, double *seg, int base)
{
  const int P = c.s.P;
  int sp = 0;
  sh.stack[sp++] = it0; sh.stack[sp++] = it2; sh.stack[sp++] = atom0; sh.stack[sp++] = atom2;
  while (sp > 0) {
    int a2 = sh.stack[--sp], a0 = sh.stack[--sp], t2 = sh.stack[--sp], t0 = sh.stack[--sp];
    if ((t2 - t0) < 2) continue;
    int t1 = (int)rint(0.5 * (double)(t0 + t2));
    int p0 = t0 % P, p1 = t1 % P, p2 = t2 % P;
    int a1 = a0;
    if ((p1 != t1) && (p0 == t0)) a1 = a2;
    double s0 = (double)(t1 - t0), s2 = (double)(t2 - t1);
    double gkin = (s0 + s2) / (wk.twave2 * s0 * s2);
    double r0[3], r2[3], r1[3];
    if (seg) {
      for (int d = 0; d < 3; d++) { r0[d] = seg[3 * (t0 - base) + d]; r2[d] = seg[3 * (t2 - base) + d]; }
    } else {
      size_t i0 = bead(c, wk.first + a0, p0), i2 = bead(c, wk.first + a2, p2);
      r0[0] = c.st.x[i0]; r0[1] = c.st.y[i0]; r0[2] = c.st.z[i0];
      r2[0] = c.st.x[i2]; r2[1] = c.st.y[i2]; r2[2] = c.st.z[i2];
    }
    for (int d = 0; d < 3; d++) {
      r1[d] = (s2 * r0[d] + s0 * r2[d]) / (s0 + s2);
      r1[d] += sh.gz[gi++] / sqrt(gkin);                 // gauss(gkin), mc_randg.cc:149
    }
    if (seg) {
      for (int d = 0; d < 3; d++) seg[3 * (t1 - base) + d] = r1[d];
    } else {
      store_bead(c, bead(c, wk.first + a1, p1), r1[0], r1[1], r1[2]);
    }
    // right half below the left one: the left half is taken first
    sh.stack[sp++] = t1; sh.stack[sp++] = t2; sh.stack[sp++] = a1; sh.stack[sp++] = a2;
    sh.stack[sp++] = t0; sh.stack[sp++] = t1; sh.stack[sp++] = a0; sh.stack[sp++] = a1;
  }
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

// get_ptable (mc_qworm.cc:577-642) on thread 0 into the scratch lists
// dr2[1..count], atm[1..count], ptab[1..count]
__device__ int get_ptable(const Ctx &c, const DevWorm &wk, const WormShared &sh, const int *rindex, int atomw,
                          int pt0, int pt1, int segm, int t1, double *dr2l, int *atml, double *ptab)
{
  size_t iw = bead(c, wk.first + atomw, pt0);
  double rw[3] = {c.st.x[iw], c.st.y[iw], c.st.z[iw]};
  int count = 0;
  for (int a1 = 0; a1 < wk.numb; a1++)
    if (world_line(sh, a1, pt1)) {
      int a0 = a1;
      if (t1 != pt1) a0 = rindex[a1];
      if (a0 != sh.atom_i) {
        size_t i1 = bead(c, wk.first + a1, pt1);
        double r1[3] = {c.st.x[i1], c.st.y[i1], c.st.z[i1]};
        double dr2 = 0.0;
        for (int d = 0; d < 3; d++) {
          double dx = rw[d] - r1[d];
          if (c.s.minimage) dx -= (c.s.box[d] * rint(dx / c.s.box[d]));
          dr2 += (dx * dx);
        }
        if (dr2 < wk.cut2) {
          count++;
          dr2l[count] = dr2;
          atml[count] = a1;
        }
      }
    }
  for (int j = 2; j <= count; j++) {   // mmsort (mc_utils.cc:206-230)
    double dt = dr2l[j];
    int it = atml[j];
    int i = j - 1;
    while ((i > 0) && (dr2l[i] > dt)) {
      dr2l[i + 1] = dr2l[i];
      atml[i + 1] = atml[i];
      i--;
    }
    dr2l[i + 1] = dt;
    atml[i + 1] = it;
  }
  if (count > 100) count = 100;        // MAXNEIGHBORS (mc_qworm.cc:12)
  double norm = 1.0 / ((double)segm * wk.twave2);
  for (int ic = 1; ic <= count; ic++) ptab[ic] = exp(-norm * dr2l[ic]);
  return count;
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
                                                       Src src, double *seg, double *dr2l, int *atml,
                                                       double *ptab)
{
  __shared__ WormShared sh;
  __shared__ double pnorm_old;
  const DevWorm wk = *wkp;
  const int P = c.s.P;
  const bool t0 = threadIdx.x == 0;
  src.init();
  if (t0) {
    sh.exists = wkp->exists; sh.ira = wkp->ira; sh.masha = wkp->masha;
    sh.atom_i = wkp->atom_i; sh.atom_m = wkp->atom_m;
  }
  __syncthreads();
  const bool bose = c.s.stat[wk.type] == 1;      // PIMC_BOSE (pimc_types.h)
  for (int atom = 0; atom < wk.numb; atom++) {
    // ---------------- open (mc_qworm.cc:155-180) / close (:182-236)
    int segm = 0;
    if (t0) {
      sh.gneed = 0;
      if (sh.exists) {
        wkp->qwtot[1] += 1.0;
        segm = sh.masha - sh.ira;
        if (segm < 0) segm += P;
        sh.flag = segm > wk.m ? 0 : 1;
        if (sh.flag && segm >= 2) sh.gneed = 3 * (segm - 1);
        sh.gbase = src.gbase();
      }
    }
    prefetch_gauss(src, sh);
    if (t0) {
      if (sh.exists) {
        if (sh.flag) {
          int gi = 0;
          src.gskip(sh.gneed);
          sample_middle(c, wk, sh, gi, sh.ira, sh.ira + segm, sh.atom_i, sh.atom_m, nullptr, 0);
          potential_queries(c, wk, sh, sh.ira, sh.ira + segm, sh.atom_i, sh.atom_m);
        }
      } else {
        wkp->qwtot[0] += 1.0;
        sh.atom_i = nrnd(src, 0, wk.numb);
        sh.ira = nrnd(src, 1, P);
        segm = nrnd(src, 2, wk.m) + 1;
        sh.masha = (sh.ira + segm) % P;
        sh.atom_m = sh.atom_i;
        if (sh.masha != (sh.ira + segm)) sh.atom_m = c.st.pindex[sh.atom_i];
        sh.flag = 2;
        potential_queries(c, wk, sh, sh.ira, sh.ira + segm, sh.atom_i, sh.atom_m);
      }
    }
    __syncthreads();
    if (sh.flag) {
      query_sums(c, frames, wk, sh);
      __syncthreads();
      if (t0) {
        double prob = wk.qw_norm * pow((double)segm, 1.5) *
                      exp(open_kin(c, wk, sh, segm) + potential_total(sh) * c.s.tau);
        if (sh.flag == 1) prob = 1.0 / prob;
        bool acc = false;
        if (prob >= 1.0) acc = true;
        else if (prob > src.take(3)) acc = true;
        if (acc) {
          if (sh.flag == 1) { sh.exists = 0; wkp->qwacc[1] += 1.0; }
          else { sh.exists = 1; wkp->qwacc[0] += 1.0; }
        }
      }
    }
    __syncthreads();   // every thread is past the reads of sh.flag / sh.exists above
    // ---------------- advance (mc_qworm.cc:295-355) / recede (:357-400)
    if (sh.exists) {
      int ira_new = 0, atomi_new = 0, adv = 0, advance = 0;
      if (t0) {
        double r = src.take(7);
        adv = r > 0.5;
        sh.flag = 0;
        sh.gneed = 0;
        if (adv) {
          wkp->qwtot[4] += 1.0;
          int sg = sh.masha - sh.ira;
          if (sg < 0) sg += P;
          advance = nrnd(src, 2, wk.m) + 1;
          if (sg - advance > 0) sh.gneed = 3 * advance;   // the end point, then the bridge
        }
        sh.gbase = src.gbase();
      }
      prefetch_gauss(src, sh);
      if (t0) {
        if (adv) {
          if (sh.gneed > 0) {
            int gi = 0;
            src.gskip(sh.gneed);
            int it0 = sh.ira, it2 = sh.ira + advance;
            ira_new = it2 % P;
            atomi_new = sh.atom_i;
            if (ira_new != it2) atomi_new = sh.atom_m;
            double gvar = 1.0 / ((double)advance * wk.twave2);
            size_t i0 = bead(c, wk.first + sh.atom_i, it0 % P);
            double r0[3] = {c.st.x[i0], c.st.y[i0], c.st.z[i0]}, r2[3];
            for (int d = 0; d < 3; d++) r2[d] = r0[d] + sh.gz[gi++] / sqrt(gvar);
            store_bead(c, bead(c, wk.first + atomi_new, it2 % P), r2[0], r2[1], r2[2]);
            sample_middle(c, wk, sh, gi, it0, it2, sh.atom_i, atomi_new, nullptr, 0);
            potential_queries(c, wk, sh, it0, it2 + 1, sh.atom_i, atomi_new);
            sh.flag = 1;
          }
        } else {
          wkp->qwtot[5] += 1.0;
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
            potential_queries(c, wk, sh, it0, it1 + 1, a0, a1);
            sh.flag = 2;
          }
        }
      }
      __syncthreads();
      if (sh.flag) {
        query_sums(c, frames, wk, sh);
        __syncthreads();
        if (t0) {
          double pot = potential_total(sh);
          bool acc = false;
          if (sh.flag == 1) {          // advance
            if (pot < 0.0) acc = true;
            else if (exp(-pot * c.s.tau) > src.take(4)) acc = true;
            if (acc) wkp->qwacc[4] += 1.0;
          } else {                     // recede
            if (pot > 0.0) acc = true;
            else if (exp(pot * c.s.tau) > src.take(4)) acc = true;
            if (acc) wkp->qwacc[5] += 1.0;
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
      if (t0) {
        wkp->qwtot[6] += 1.0;
        const int sg = wk.m;
        it0 = sh.ira;
        it1 = it0 + sg;
        pit1 = it1 % P;
        atomw = sh.atom_i;
        sh.flag = 0;
        int count = get_ptable(c, wk, sh, rindex, atomw, it0, pit1, sg, it1, dr2l, atml, ptab);
        if (count > 0) {
          double pn = 0.0;
          for (int ic = 1; ic <= count; ic++) pn += ptab[ic];
          double prand = pn * src.take(5);
          double sum = 0.0;
          int ic = 1;
          while ((ic <= count) && (sum < prand)) {
            sum += ptab[ic];
            ic++;
          }
          ic--;
          a1 = atml[ic];
          pnorm_old = pn;
          a0 = a1;
          if (pit1 != it1) a0 = rindex[a1];
          sh.flag = 1;
          sh.stack[0] = it0; sh.stack[1] = it1; sh.stack[2] = atomw; sh.stack[3] = a0; sh.stack[4] = a1;
        }
        sh.gneed = sh.flag && wk.m >= 2 ? 3 * (wk.m - 1) : 0;
        sh.gbase = src.gbase();
      }
      prefetch_gauss(src, sh);
      if (t0 && sh.flag) {
        const int sg = wk.m;
        it0 = sh.stack[0]; it1 = sh.stack[1]; atomw = sh.stack[2]; a0 = sh.stack[3]; a1 = sh.stack[4];
        pit1 = it1 % P;
        {
          int gi = 0;
          src.gskip(sh.gneed);
          // newcoords: the end points, then the bridge between them
          size_t iw = bead(c, wk.first + atomw, it0), i1 = bead(c, wk.first + a1, pit1);
          seg[0] = c.st.x[iw]; seg[1] = c.st.y[iw]; seg[2] = c.st.z[iw];
          seg[3 * sg + 0] = c.st.x[i1]; seg[3 * sg + 1] = c.st.y[i1]; seg[3 * sg + 2] = c.st.z[i1];
          sample_middle(c, wk, sh, gi, it0, it1, a0, a1, seg, it0);
          // the new and the old energy of every inner slice, in that order
          int g = wk.first + a0, nq = 0;
          for (int it = it0 + 1; it < it1; it++) {
            int pit = it % P;
            if (pit != it) g = wk.first + a1;
            size_t i = bead(c, g, pit);
            sh.qa[nq] = g; sh.qpit[nq] = pit;
            sh.qx[nq] = seg[3 * (it - it0)]; sh.qy[nq] = seg[3 * (it - it0) + 1]; sh.qz[nq] = seg[3 * (it - it0) + 2];
            nq++;
            sh.qa[nq] = g; sh.qpit[nq] = pit;
            sh.qx[nq] = c.st.x[i]; sh.qy[nq] = c.st.y[i]; sh.qz[nq] = c.st.z[i];
            nq++;
          }
          sh.nq = nq;
          sh.stack[0] = it0; sh.stack[1] = it1; sh.stack[2] = atomw; sh.stack[3] = a0; sh.stack[4] = a1;
        }
      }
      __syncthreads();
      if (sh.flag) {
        query_sums(c, frames, wk, sh);
        __syncthreads();
        if (t0) {
          it0 = sh.stack[0]; it1 = sh.stack[1]; atomw = sh.stack[2]; a0 = sh.stack[3]; a1 = sh.stack[4];
          pit1 = it1 % P;
          double pot = 0.0;
          for (int q = 0; q < sh.nq; q += 2) {
            pot += sh.qsum[q];
            pot -= sh.qsum[q + 1];
          }
          double prob = exp(-pot * c.s.tau);
          int count = get_ptable(c, wk, sh, rindex, a0, it0, pit1, wk.m, it1, dr2l, atml, ptab);
          double pn = 0.0;
          for (int ic = 1; ic <= count; ic++) pn += ptab[ic];
          prob *= (pnorm_old / pn);
          bool acc = false;
          if (prob >= 1.0) acc = true;
          else if (prob > src.take(6)) acc = true;
          sh.flag = acc ? 1 : 0;
          if (acc) {
            wkp->qwacc[6] += 1.0;
            int g = wk.first + a0;
            for (int it = it0 + 1; it < it1; it++) {
              int pit = it % P;
              if (pit != it) g = wk.first + a1;
              store_bead(c, bead(c, g, pit), seg[3 * (it - it0)], seg[3 * (it - it0) + 1], seg[3 * (it - it0) + 2]);
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
          }
        }
        __syncthreads();
        if (sh.flag) {
          // the heads of the two paths up to it0 change places
          it0 = sh.stack[0]; atomw = sh.stack[2]; a0 = sh.stack[3];
          for (int it = threadIdx.x; it <= it0; it += kThreads) {
            size_t ia = bead(c, wk.first + a0, it), iw = bead(c, wk.first + atomw, it);
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
  __shared__ int ncyc, accepted, stop;
  const int numb = c.s.numb[type], g = c.s.first[type], P = c.s.P;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int a = tid; a < numb; a += kMolThreads) flag[a] = 0;
  __syncthreads();
  for (int atom = 0; atom < numb; atom++) {
    if (tid == 0) {
      ncyc = 0;
      if (flag[atom] == 0) {
        cyc[ncyc++] = atom;
        int pa = c.st.pindex[atom];
        while (pa != atom) {
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
  double *seg = (double *)scratch;
  double *dr2l = seg + 3 * (PIMC_WORM_MAXM + 1);
  double *ptab = dr2l + (numb + 1);
  int *atml = (int *)(ptab + (numb + 1));
  Ctx cw = c;
  cw.st.worm = nullptr;
  k_worm_move<WormPhilox><<<1, kThreads, 0, s>>>(cw, f, wk, rindex, src, seg, dr2l, atml, ptab);
}

size_t worm_scratch_bytes(int numb) { return sizeof(double) * (3 * (PIMC_WORM_MAXM + 1) + 2 * (size_t)(numb + 1)) + sizeof(int) * (size_t)(numb + 1) + 64; }

void launch_worm_move(const Ctx &c, Frame *f, DevWorm *wk, int *rindex, const double *const *streams,
                      const long *lengths, long *cursors, void *scratch, int numb, cudaStream_t s)
{
  WormSrc src;
  for (int k = 0; k < 9; k++) { src.v[k] = streams[k]; src.n[k] = lengths[k]; }
  src.pos = cursors;
  src.err = c.st.err;
  double *seg = (double *)scratch;
  double *dr2l = seg + 3 * (PIMC_WORM_MAXM + 1);
  double *ptab = dr2l + (numb + 1);
  int *atml = (int *)(ptab + (numb + 1));
  Ctx cw = c;
  cw.st.worm = nullptr;      // the kernel masks from its own copy of the worm
  k_worm_move<WormSrc><<<1, kThreads, 0, s>>>(cw, f, wk, rindex, src, seg, dr2l, atml, ptab);
}
