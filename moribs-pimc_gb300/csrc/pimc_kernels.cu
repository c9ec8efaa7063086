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
    c.st.xf[i] = (float)c.st.x[i];
    c.st.yf[i] = (float)c.st.y[i];
    c.st.zf[i] = (float)c.st.z[i];
  }
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    make_frame(c.st.ang[i], c.st.ang[n + i], c.st.ang[2 * n + i], frames[i]);
    for (int d = 0; d < 3; d++) c.st.cosvf[d * n + i] = (float)c.st.cosv[d * n + i];
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
__global__ void __launch_bounds__(PIMC_BLOCK) k_bisect_replay(Ctx c, Frame *frames, int type, int time0, int exch,
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
__global__ void __launch_bounds__(PIMC_BLOCK) k_bisect_phase(Ctx c, Frame *frames, int type, int s0, int j,
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

// ------------------------------------------------------------ rotations
// one even or odd half of MCRotationsMove / MCRotations3D: CTA b handles
// slice q = parity + 2b and all rotors of the type in order
template <bool REPLAY, bool MIX>
__global__ void __launch_bounds__(PIMC_BLOCK) k_rot(Ctx c, Frame *frames, int parity, const double *urot, long nurot,
                                                     unsigned phase, uint64_t seed, const unsigned *pass,
                                                     double *rd_out, int *acc_out, unsigned long long *cnt)
{
  __shared__ RotShared sh;
  int q = parity + 2 * blockIdx.x;
  if (q >= c.s.Q) return;
  int nr = c.s.nrotors;
  bool linear = c.s.molecule[c.s.imtype] == 1;
  int per = linear ? 3 : 4;
  long n_even = (c.s.Q + 1) / 2;
  for (int r = 0; r < nr; r++) {
    double u[4] = {0.5, 0.5, 0.5, 0.5};
    if (REPLAY) {
      // serial consumption order: even slices then odd, rotors inside a slice
      long idx = ((parity ? n_even : 0) + blockIdx.x) * (long)nr + r;
      for (int k = 0; k < per; k++) {
        long p = idx * per + k;
        u[k] = (p < nurot) ? urot[p] : 0.5;
        if (p >= nurot && threadIdx.x == 0) atomicOr(c.st.err, (unsigned)DERR_STREAM);
      }
    } else {
      uint64_t mv = ((uint64_t)(*pass) << 32) | ((uint64_t)phase << 12) | (uint64_t)blockIdx.x;
      double a, b;
      philox_u2(seed, mv, 0x400000u | (uint32_t)r, 0u, &a, &b);
      u[0] = a; u[1] = b;
      philox_u2(seed, mv, 0x400000u | (uint32_t)r, 1u, &a, &b);
      u[2] = a; u[3] = b;
      if (linear) u[2] = u[3];
    }
    int g0 = c.s.rot_first + r;
    double rd;
    int acc = rot_step<MIX>(c, frames, g0, q, u, linear, sh, &rd);
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

// ------------------------------------------------------------ centroid move
// MCMolecularMove (mc_piqmc.cc:54-102) split in three launches per atom:
// propose (3 displacements), partner sums over all slices, accept/commit.
template <bool REPLAY>
__global__ void k_mol_propose(Ctx c, int type, ReplaySrc src, uint64_t seed, const unsigned *pass, unsigned phase,
                              int atom, MolScratch *ms)
{
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  for (int d = 0; d < 3; d++) {
    double u;
    if (REPLAY) u = src.disp_u(d);
    else {
      PhiloxSrc ps{seed, ((uint64_t)(*pass) << 32) | ((uint64_t)phase << 12) | (uint64_t)atom};
      u = ps.disp_u(d);
    }
    ms->disp[d] = c.s.mcstep[type] * (u - 0.5);
  }
}

// CTA = one partner atom1; threads over slices; new = old + disp; the two
// whole-path sums are reduced warp by warp in a fixed order
template <bool MIX>
__global__ void __launch_bounds__(PIMC_BLOCK) k_mol_pairs(Ctx c, Frame *frames, int gatom, MolScratch *ms)
{
  __shared__ double part[2][PIMC_BLOCK / 32];
  int a1 = blockIdx.x;
  int tid = threadIdx.x;
  double an = 0.0, ao = 0.0;
  if (a1 != gatom) {
    double d0 = ms->disp[0], d1 = ms->disp[1], d2 = ms->disp[2];
    for (int it = tid; it < c.s.P; it += blockDim.x) {
      size_t i = sidx(c.s, it, gatom);
      if (MIX) {
        float x = c.st.xf[i], y = c.st.yf[i], z = c.st.zf[i];
        ao += (double)pair_term32(c, frames, gatom, a1, it, x, y, z);
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
    ms->pair[tid][a1] = s;
  }
}

template <bool REPLAY>
__global__ void __launch_bounds__(PIMC_BLOCK) k_mol_finish(Ctx c, int type, int gatom, ReplaySrc src, uint64_t seed,
                                                            const unsigned *pass, unsigned phase, int atom,
                                                            MolScratch *ms, double *dv_out, int *acc_out,
                                                            unsigned long long *cnt)
{
  __shared__ int acc;
  if (threadIdx.x == 0) {
    double en = 0.0, eo = 0.0;
    for (int a1 = 0; a1 < c.s.na; a1++)
      if (a1 != gatom) { en += ms->pair[0][a1]; eo += ms->pair[1][a1]; }
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
    if (dv_out) { dv_out[atom] = deltav; acc_out[atom] = a; }
    cnt[(type * 3 + 0) * 2 + 0] += 1;
    if (a) cnt[(type * 3 + 0) * 2 + 1] += 1;
  }
  __syncthreads();
  if (acc) {
    double d0 = ms->disp[0], d1 = ms->disp[1], d2 = ms->disp[2];
    for (int it = threadIdx.x; it < c.s.P; it += blockDim.x) {
      size_t i = sidx(c.s, it, gatom);
      store_bead(c, i, c.st.x[i] + d0, c.st.y[i] + d1, c.st.z[i] + d2);
    }
    // the whole path moved: every cached rotor potential is stale
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
  int type = c.st.mctype[a];
  int g = c.s.first[type];
  double acc = 0.0;
  for (int it = threadIdx.x; it < P; it += blockDim.x) {
    int a1 = a;
    if (c.s.stat[type] == 1 && it + 1 == P) a1 = g + c.st.pindex[a - g];
    size_t i0 = sidx(c.s, it, a), i1 = sidx(c.s, (it + 1) % P, a1);
    double d[3] = {c.st.x[i0] - c.st.x[i1], c.st.y[i0] - c.st.y[i1], c.st.z[i0] - c.st.z[i1]};
    for (int k = 0; k < 3; k++) {
      if (c.s.minimage) d[k] -= c.s.box[k] * rint(d[k] / c.s.box[k]);
      acc += d[k] * d[k];
    }
  }
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
  int ty0 = c.st.mctype[a0], ty1 = c.st.mctype[a1];
  int m0 = c.s.molecule[ty0], m1 = c.s.molecule[ty1];
  bool counted = (m0 == 1 || m1 == 1) || (m0 != m1) || (m0 == 2 && m1 == 2 && c.s.numb[c.s.imtype] > 1) ||
                 (ty0 == ty1 && m0 == 0);
  double acc = 0.0;
  if (counted)
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

// GetRotE3D (mc_estim.cc:989-1096) per (rotor, it0) link terms and
// GetRotEnergy (mc_estim.cc:939-987) for the linear rotor:
// out[4*k + {srot, sesq, se_termsq, valid}]
__global__ void k_est_rot(Ctx c, Frame *frames, double *out)
{
  int Q = c.s.Q, nr = c.s.nrotors;
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nr * Q) return;
  int r = k / Q, it0 = k % Q;
  bool linear = c.s.molecule[c.s.imtype] == 1;
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
      rho = rotden_rho(c.t, f1, f2, &bad, &erot, &esq);
      if (c.s.rot_den_type == 1 && c.s.rn_ratio == 1) {
        rsrot(f1, f2, c.s.abc, c.s.rot_tau, c.s.rot_odevn, &rho, &erot);
        srot = rho;
      } else
        srot = erot;
      sesq = esq;
      sts = erot * erot;
    }
  }
  out[4 * k + 0] = srot;
  out[4 * k + 1] = sesq;
  out[4 * k + 2] = sts;
  out[4 * k + 3] = 1.0;
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

// ------------------------------------------------------------ bookkeeping
__global__ void k_pass_begin(unsigned *pass) { *pass += 1; }

// ------------------------------------------------------------ launchers
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
  if (c.s.mixed) k_bisect_replay<true><<<1, PIMC_BLOCK, 0, s>>>(c, f, type, time0, exch, src, ds, lvl, cnt);
  else k_bisect_replay<false><<<1, PIMC_BLOCK, 0, s>>>(c, f, type, time0, exch, src, ds, lvl, cnt);
}

void launch_bisect_phase(const Ctx &c, Frame *f, int type, int s0, int j, unsigned phase, uint64_t seed,
                         const unsigned *pass, unsigned long long *cnt, cudaStream_t s)
{
  int M = 1 << c.s.levels[type];
  if (c.s.mixed) k_bisect_phase<true><<<c.s.P / M, PIMC_BLOCK, 0, s>>>(c, f, type, s0, j, phase, seed, pass, cnt);
  else k_bisect_phase<false><<<c.s.P / M, PIMC_BLOCK, 0, s>>>(c, f, type, s0, j, phase, seed, pass, cnt);
}

void launch_rot_replay(const Ctx &c, Frame *f, int parity, const double *urot, long nurot, double *rd, int *acc,
                       unsigned long long *cnt, cudaStream_t s)
{
  int nb = (c.s.Q - parity + 1) / 2;
  if (nb <= 0) return;
  if (c.s.mixed) k_rot<true, true><<<nb, PIMC_BLOCK, 0, s>>>(c, f, parity, urot, nurot, 0, 0, nullptr, rd, acc, cnt);
  else k_rot<true, false><<<nb, PIMC_BLOCK, 0, s>>>(c, f, parity, urot, nurot, 0, 0, nullptr, rd, acc, cnt);
}

void launch_rot_phase(const Ctx &c, Frame *f, int parity, unsigned phase, uint64_t seed, const unsigned *pass,
                      unsigned long long *cnt, cudaStream_t s)
{
  int nb = (c.s.Q - parity + 1) / 2;
  if (nb <= 0) return;
  if (c.s.mixed)
    k_rot<false, true><<<nb, PIMC_BLOCK, 0, s>>>(c, f, parity, nullptr, 0, phase, seed, pass, nullptr, nullptr, cnt);
  else
    k_rot<false, false><<<nb, PIMC_BLOCK, 0, s>>>(c, f, parity, nullptr, 0, phase, seed, pass, nullptr, nullptr, cnt);
}

void launch_mol(const Ctx &c, Frame *f, int type, int atom, bool replay, ReplaySrc src, uint64_t seed,
                const unsigned *pass, unsigned phase, MolScratch *ms, double *dv, int *acc, unsigned long long *cnt,
                cudaStream_t s)
{
  int g = c.s.first[type] + atom;
  if (replay) k_mol_propose<true><<<1, 32, 0, s>>>(c, type, src, seed, pass, phase, atom, ms);
  else k_mol_propose<false><<<1, 32, 0, s>>>(c, type, src, seed, pass, phase, atom, ms);
  if (c.s.mixed) k_mol_pairs<true><<<c.s.na, PIMC_BLOCK, 0, s>>>(c, f, g, ms);
  else k_mol_pairs<false><<<c.s.na, PIMC_BLOCK, 0, s>>>(c, f, g, ms);
  if (replay) k_mol_finish<true><<<1, PIMC_BLOCK, 0, s>>>(c, type, g, src, seed, pass, phase, atom, ms, dv, acc, cnt);
  else k_mol_finish<false><<<1, PIMC_BLOCK, 0, s>>>(c, type, g, src, seed, pass, phase, atom, ms, dv, acc, cnt);
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

size_t mol_scratch_bytes() { return sizeof(MolScratch); }
