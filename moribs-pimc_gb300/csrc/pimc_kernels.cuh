// pimc_kernels.cuh -- move and energy routines executed by one CTA of
// PIMC_BLOCK threads, shared by the replay (parity) kernels and the
// production phase kernels.  Partner sums are deterministic: thread k holds
// the partners p = k, k+PIMC_BLOCK, ... and the per-thread partials are added
// in thread order, which for natoms <= PIMC_BLOCK is the reference's own
// sequential order over atom1 (mc_piqmc.cc:1808-1962).
#pragma once
#include "pimc_internal.cuh"

#define SLOT_CHUNK 16

__device__ __forceinline__ size_t sidx(const DevSys &s, int t, int a) { return (size_t)t * s.nap + a; }

__device__ __forceinline__ int rot_index(const DevSys &s, int gatom, int q) { return (gatom - s.rot_first) * s.Q + q; }

// one term of PotEnergy(atom0, pos, it) (mc_piqmc.cc:1824-1958): atom0 at
// (px,py,pz), partner atom1 at its current bead, rotor frames from the cache
__device__ __forceinline__ double pair_term(const Ctx &c, const Frame *__restrict__ frames, int a0, int a1, int it,
                                            double px, double py, double pz)
{
  const DevSys &s = c.s;
  int ty0 = c.st.mctype[a0], ty1 = c.st.mctype[a1];
  int m0 = s.molecule[ty0], m1 = s.molecule[ty1];
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

// block-wide deterministic sums of PotEnergy(a0[k], pos_k, its[k]) for
// k < nslots; results land in out[k] (shared or global)
__device__ inline void slot_energies(const Ctx &c, const Frame *frames, int nslots, const int *a0, const int *its,
                              const double *px, const double *py, const double *pz, double *out,
                              double (*part)[PIMC_BLOCK])
{
  int tid = threadIdx.x;
  for (int base = 0; base < nslots; base += SLOT_CHUNK) {
    int ns = min(SLOT_CHUNK, nslots - base);
    for (int k = 0; k < ns; k++) {
      int sl = base + k;
      double acc = 0.0;
      for (int p = tid; p < c.s.na; p += PIMC_BLOCK)
        if (p != a0[sl]) acc += pair_term(c, frames, a0[sl], p, its[sl], px[sl], py[sl], pz[sl]);
      part[k][tid] = acc;
    }
    __syncthreads();
    if (tid < ns) {
      double sum = 0.0;
      for (int k = 0; k < PIMC_BLOCK; k++) sum += part[tid][k];
      out[base + tid] = sum;
    }
    __syncthreads();
  }
}

// ------------------------------------------------------ random sources

// replay of the reference's sequential generator streams (parity mode);
// cursors live in global memory and are touched by thread 0 only
struct ReplaySrc {
  const double *g; long ng; long *gpos;      // gauss() x1 values
  const double *u; long nu; long *upos;      // rnd2()/rnd3()/runif() uniforms
  const double *d; long nd; long *dpos;      // rnd1() displacements
  unsigned int *err;
  __device__ double take(const double *v, long n, long *pos)
  {
    long p = *pos;
    if (p >= n) { atomicOr(err, (unsigned)DERR_STREAM); return 0.5; }
    *pos = p + 1;
    return v[p];
  }
  __device__ double gauss_x1(int, int, int) { return take(g, ng, gpos); }
  __device__ double accept_u(int) { return take(u, nu, upos); }
  __device__ double disp_u(int) { return take(d, nd, dpos); }
};

// counter-based source for production moves: one Philox block per draw
struct PhiloxSrc {
  uint64_t seed, move;
  __device__ double gauss_x1(int level, int k, int dim)
  {
    double r1, r2;
    philox_u2(seed, move, 0x100000u | ((uint32_t)level << 12) | (uint32_t)k, (uint32_t)dim, &r1, &r2);
    return sqrt(-log(r1)) * cos(2.0 * PIMC_PI * r2);        // Box-Muller as gauss() (mc_randg.cc:144)
  }
  __device__ double accept_u(int level)
  {
    double u0, u1;
    philox_u2(seed, move, 0x200000u | (uint32_t)level, 0u, &u0, &u1);
    return u0;
  }
  __device__ double disp_u(int dim)
  {
    double u0, u1;
    philox_u2(seed, move, 0x300000u, (uint32_t)dim, &u0, &u1);
    return u0;
  }
};

// ------------------------------------------------------ bisection move
// MCBisectionMove / MCBisectionMoveExchange (mc_piqmc.cc:194-419) for the
// local atom `atom` of `type` over the window [time0, time0 + 2^levels].
// exch switches the owner of slices past P to pindex[atom] (the permutation
// the path closes through); the midpoint energy is that of the slice's owner.
// Returns 1 when accepted; records per-level action differences.
struct BisectShared {
  double nb[3][PIMC_MAX_SEG + 1];
  double en[PIMC_MAX_SEG + 1], eo[PIMC_MAX_SEG + 1];
  double sx[PIMC_MAX_SEG], sy[PIMC_MAX_SEG], sz[PIMC_MAX_SEG], se[PIMC_MAX_SEG];
  int sa[PIMC_MAX_SEG], st[PIMC_MAX_SEG];
  int owner[PIMC_MAX_SEG + 1], slice[PIMC_MAX_SEG + 1];
  double pot0, pot1;
  int acc, passed;
  double part[SLOT_CHUNK][PIMC_BLOCK];
};

template <class Src>
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
  for (int k = tid; k <= M; k += PIMC_BLOCK) {
    int t = time0 + k;
    int own = (exch && t >= P) ? gx : g0;
    int pt = t % P;
    sh.owner[k] = own;
    sh.slice[k] = pt;
    size_t i = sidx(s, pt, own);
    sh.nb[0][k] = c.st.x[i];
    sh.nb[1][k] = c.st.y[i];
    sh.nb[2][k] = c.st.z[i];
  }
  if (tid == 0) { sh.pot0 = 0.0; sh.pot1 = 0.0; sh.acc = 0; sh.passed = 0; }
  __syncthreads();
  double bnorm = 1.0 / (s.lambda[type] * s.tau);
  for (int level = 0; level < L; level++) {
    int seg = 1 << (L - level), half = seg >> 1, nmid = M / seg;
    double bkin_norm = bnorm / (double)seg;
    if (tid == 0) {
      double sq = sqrt(bkin_norm);
      for (int j = 0; j < nmid; j++) {
        int k0 = j * seg, k1 = k0 + half, k2 = k0 + seg;
        for (int d = 0; d < 3; d++) {
          sh.nb[d][k1] = 0.5 * (sh.nb[d][k0] + sh.nb[d][k2]);
          sh.nb[d][k1] += src.gauss_x1(level, j, d) / sq;       // gauss(bkin_norm) (mc_randg.cc:149)
        }
      }
    }
    __syncthreads();
    // slots: (midpoint j, new) and (midpoint j, old)
    for (int j = tid; j < nmid; j += PIMC_BLOCK) {
      int k1 = j * seg + half;
      int own = sh.owner[k1], pt = sh.slice[k1];
      size_t i = sidx(s, pt, own);
      sh.sa[2 * j] = own; sh.st[2 * j] = pt;
      sh.sx[2 * j] = sh.nb[0][k1]; sh.sy[2 * j] = sh.nb[1][k1]; sh.sz[2 * j] = sh.nb[2][k1];
      sh.sa[2 * j + 1] = own; sh.st[2 * j + 1] = pt;
      sh.sx[2 * j + 1] = c.st.x[i]; sh.sy[2 * j + 1] = c.st.y[i]; sh.sz[2 * j + 1] = c.st.z[i];
    }
    __syncthreads();
    slot_energies(c, frames, 2 * nmid, sh.sa, sh.st, sh.sx, sh.sy, sh.sz, sh.se, sh.part);
    for (int j = tid; j < nmid; j += PIMC_BLOCK) {
      int k1 = j * seg + half;
      sh.en[k1] = sh.se[2 * j];
      sh.eo[k1] = sh.se[2 * j + 1];
    }
    __syncthreads();
    if (tid == 0) {
      sh.pot1 = sh.pot0;
      double pot0 = 0.0;
      for (int j = 0; j < nmid; j++) {
        int k0 = j * seg, k1 = k0 + half;
        pot0 += (sh.en[k1] - sh.eo[k1]);
        if (k0 != 0) pot0 += (sh.en[k0] - sh.eo[k0]);
      }
      sh.pot0 = pot0;
      double deltav = (pot0 - 2.0 * sh.pot1);
      deltav *= s.tau * (double)(seg / 2);
      if (ds_out) ds_out[level] = deltav;
      int a = 0;
      if (deltav < 0.0) a = 1;
      else if (exp(-deltav) > src.accept_u(level)) a = 1;
      sh.acc = a;
      if (a) sh.passed = level + 1;
    }
    __syncthreads();
    if (!sh.acc) break;
  }
  int accepted = sh.acc;
  if (accepted) {
    for (int k = 1 + tid; k < M; k += PIMC_BLOCK) {
      size_t i = sidx(s, sh.slice[k], sh.owner[k]);
      c.st.x[i] = sh.nb[0][k];
      c.st.y[i] = sh.nb[1][k];
      c.st.z[i] = sh.nb[2][k];
    }
  }
  __syncthreads();
  return accepted;
}

// scratch of one centroid move: the displacement and per-partner whole-path
// sums for the displaced and the current path
#define PIMC_MAX_ATOMS 1024
struct MolScratch {
  double disp[3];
  double pair[2][PIMC_MAX_ATOMS];
};

// ------------------------------------------------------ rotational moves
struct RotShared {
  Frame fo[3], fn;          // old frames at q-1, q, q+1 and the proposal at q
  double rho[4], pot[2];
  double vals[2 * 16];      // per (it, old/new) PotRot sums, R <= 16
  double ang_new[3], cos_new[3];
  int bad, acc;
  double rd;
  double part[SLOT_CHUNK][PIMC_BLOCK];
};

// PotRotE3D term (mc_piqmc.cc:2078-2146) for rotor g0 with body frame f at
// slice it against partner a1
__device__ __forceinline__ double rot3d_term(const Ctx &c, const Frame *frames, const Frame &f, int g0, int a1, int it)
{
  const DevSys &s = c.s;
  size_t i0 = sidx(s, it, g0), i1 = sidx(s, it, a1);
  if (c.st.mctype[a1] != s.imtype)
    return vcord(c.t, f, c.st.x[i0], c.st.y[i0], c.st.z[i0], c.st.x[i1], c.st.y[i1], c.st.z[i1]);
  return caleng(f, frames[rot_index(s, a1, it / s.R)], c.st.x[i0], c.st.y[i0], c.st.z[i0], c.st.x[i1], c.st.y[i1],
                c.st.z[i1]);
}

// PotRotEnergy term (mc_piqmc.cc:1987-2040) for the linear rotor g0 with unit
// vector n at slice it against partner a1
__device__ __forceinline__ double rotlin_term(const Ctx &c, const double n[3], int g0, int a1, int it)
{
  const DevSys &s = c.s;
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

// sum over it in [q*R, q*R+R) of the rotor's partner sums for the old
// (slot 0) and new (slot 1) orientation, in the reference's order
__device__ inline void rot_pots(const Ctx &c, const Frame *frames, int g0, int q, bool linear, const double *nold,
                         const double *nnew, RotShared &sh)
{
  const DevSys &s = c.s;
  int tid = threadIdx.x, R = s.R;
  int nslots = 2 * R;
  for (int base = 0; base < nslots; base += SLOT_CHUNK) {
    int ns = min(SLOT_CHUNK, nslots - base);
    for (int k = 0; k < ns; k++) {
      int sl = base + k, it = q * R + (sl >> 1), isnew = sl & 1;
      double acc = 0.0;
      for (int p = tid; p < s.na; p += PIMC_BLOCK)
        if (p != g0) {
          if (linear) acc += rotlin_term(c, isnew ? nnew : nold, g0, p, it);
          else acc += rot3d_term(c, frames, isnew ? sh.fn : sh.fo[1], g0, p, it);
        }
      sh.part[k][tid] = acc;
    }
    __syncthreads();
    if (tid < ns) {
      double sum = 0.0;
      for (int k = 0; k < PIMC_BLOCK; k++) sum += sh.part[tid][k];
      sh.vals[base + tid] = sum;
    }
    __syncthreads();
  }
  if (tid == 0) {
    double po = 0.0, pn = 0.0;
    for (int k = 0; k < R; k++) { po += sh.vals[2 * k]; pn += sh.vals[2 * k + 1]; }
    sh.pot[0] = po;
    sh.pot[1] = pn;
  }
  __syncthreads();
}

// MCRot3Dstep (mc_piqmc.cc:938-1199) for rotor g0 at rotational slice q with
// uniforms u[4]; frames of the rotor slices are read from / written to the
// frame cache.  Returns 1 if accepted.
__device__ inline int rot3d_step(const Ctx &c, Frame *frames, int g0, int q, const double u[4], RotShared &sh, double *rd_out)
{
  const DevSys &s = c.s;
  int tid = threadIdx.x, Q = s.Q;
  size_t n = (size_t)s.nrotors * Q;
  int q0 = q - 1, q2 = q + 1;
  if (q0 < 0) q0 += Q;
  if (q2 >= Q) q2 -= Q;
  int r1 = rot_index(s, g0, q);
  if (tid == 0) {
    double cost = c.st.ang[n + r1], phi = c.st.ang[r1], chi = c.st.ang[2 * n + r1];
    const double pi2 = 2.0 * PIMC_PI;
    cost += (s.rtstep * (u[0] - 0.5));
    phi += 2.0 * PIMC_PI * (s.rtstep * (u[1] - 0.5));
    chi += 2.0 * PIMC_PI * (s.rtstep * (u[2] - 0.5));
    if (phi < 0.0) phi = pi2 + phi;
    if (chi < 0.0) chi = pi2 + chi;
    phi = fmod(phi, pi2);
    chi = fmod(chi, pi2);
    if (cost > 1.0) cost = 2.0 - cost;
    if (cost < -1.0) cost = -2.0 - cost;
    sh.ang_new[0] = phi; sh.ang_new[1] = cost; sh.ang_new[2] = chi;
    make_frame(phi, cost, chi, sh.fn);
    sh.fo[0] = frames[rot_index(s, g0, q0)];
    sh.fo[1] = frames[r1];
    sh.fo[2] = frames[rot_index(s, g0, q2)];
    sh.bad = 0;
  }
  __syncthreads();
  if (tid < 4) {
    const Frame &a = (tid == 0) ? sh.fo[0] : (tid == 1 ? sh.fo[1] : (tid == 2 ? sh.fo[0] : sh.fn));
    const Frame &b = (tid == 0) ? sh.fo[1] : (tid == 1 ? sh.fo[2] : (tid == 2 ? sh.fn : sh.fo[2]));
    double rho = 0.0, erot = 0.0;
    if (s.rot_den_type == 0) {
      int bad = 0;
      rho = rotden_rho(c.t, a, b, &bad, nullptr, nullptr);
      if (bad) atomicOr(&sh.bad, 1);
    } else {
      rsrot(a, b, s.abc, s.rot_tau, s.rot_odevn, &rho, &erot);
    }
    sh.rho[tid] = rho;
  }
  rot_pots(c, frames, g0, q, false, nullptr, nullptr, sh);
  int acc = 0;
  if (tid == 0) {
    double rd;
    if (s.rot_den_type == 0) {
      double dens_old = sh.rho[0] * sh.rho[1], dens_new = sh.rho[2] * sh.rho[3];
      if (fabs(dens_old) < PIMC_RZERO) dens_old = 0.0;
      if (dens_old < 0.0) dens_old = fabs(dens_old);
      if (fabs(dens_new) < PIMC_RZERO) dens_new = 0.0;
      if (dens_new < 0.0) dens_new = fabs(dens_new);
      rd = (dens_old > PIMC_RZERO) ? dens_new / dens_old : 1.0;
      rd *= exp(-s.tau * (sh.pot[1] - sh.pot[0]));
      acc = (rd > 1.0) || (rd > u[3]);
    } else {
      double rhoold = sh.rho[0] + sh.rho[1], rhonew = sh.rho[2] + sh.rho[3];
      rd = (rhonew - rhoold) / (4.0 * (s.rot_tau / PIMC_WNO2K));
      rd -= s.tau * (sh.pot[1] - sh.pot[0]);
      acc = (rd > 0.0) || (rd > log(u[3]));
    }
    if (sh.bad) { atomicOr(c.st.err, (unsigned)DERR_GRID_RANGE); acc = 0; }
    sh.rd = rd;
    sh.acc = acc;
    if (rd_out) *rd_out = rd;
    if (acc) {
      double phi = sh.ang_new[0], cost = sh.ang_new[1], chi = sh.ang_new[2];
      c.st.ang[r1] = phi;
      c.st.ang[n + r1] = cost;
      c.st.ang[2 * n + r1] = chi;
      double sint = sqrt(1.0 - cost * cost);
      c.st.cosv[r1] = sint * cos(phi);
      c.st.cosv[n + r1] = sint * sin(phi);
      c.st.cosv[2 * n + r1] = cost;
      frames[r1] = sh.fn;
    }
  }
  __syncthreads();
  acc = sh.acc;
  __syncthreads();
  return acc;
}

// MCRotLinStep (mc_piqmc.cc:781-936) for the linear rotor g0 at slice q
__device__ inline int rotlin_step(const Ctx &c, Frame *frames, int g0, int q, const double u[3], RotShared &sh, double *rd_out)
{
  const DevSys &s = c.s;
  int tid = threadIdx.x, Q = s.Q;
  size_t n = (size_t)s.nrotors * Q;
  int q0 = q - 1, q2 = q + 1;
  if (q0 < 0) q0 += Q;
  if (q2 >= Q) q2 -= Q;
  int r0 = rot_index(s, g0, q0), r1 = rot_index(s, g0, q), r2 = rot_index(s, g0, q2);
  __shared__ double nold[3], nnew[3];
  if (tid == 0) {
    double cost = c.st.ang[n + r1], phi = c.st.ang[r1];
    cost += (s.rtstep * (u[0] - 0.5));
    phi += (s.rtstep * (u[1] - 0.5));
    if (cost > 1.0) cost = 2.0 - cost;
    if (cost < -1.0) cost = -2.0 - cost;
    double sint = sqrt(1.0 - cost * cost);
    sh.ang_new[0] = phi; sh.ang_new[1] = cost;
    nnew[0] = sint * cos(phi);
    nnew[1] = sint * sin(phi);
    nnew[2] = cost;
    for (int d = 0; d < 3; d++) nold[d] = c.st.cosv[d * n + r1];
    double p0 = 0.0, p1 = 0.0, q0v = 0.0, q1v = 0.0;
    for (int d = 0; d < 3; d++) {
      p0 += (c.st.cosv[d * n + r0] * c.st.cosv[d * n + r1]);
      p1 += (c.st.cosv[d * n + r1] * c.st.cosv[d * n + r2]);
    }
    for (int d = 0; d < 3; d++) {
      q0v += (c.st.cosv[d * n + r0] * nnew[d]);
      q1v += (nnew[d] * c.st.cosv[d * n + r2]);
    }
    sh.rho[0] = p0; sh.rho[1] = p1; sh.rho[2] = q0v; sh.rho[3] = q1v;   // dot products for now
  }
  __syncthreads();
  if (tid < 4) {
    double g = sh.rho[tid];
    double v, erot;
    if (s.rot_den_type == 0) v = srotdens(c.t, g, 0);
    else rsline(s.abc[0], g, s.rot_tau, &v, &erot);
    sh.vals[tid] = v;
  }
  __syncthreads();
  if (tid == 0) {
    for (int k = 0; k < 4; k++) sh.rho[k] = sh.vals[k];
  }
  __syncthreads();
  rot_pots(c, frames, g0, q, true, nold, nnew, sh);
  if (tid == 0) {
    double rd;
    int acc = 0, neg = 0;
    if (s.rot_den_type == 0) {
      double dens_old = sh.rho[0] * sh.rho[1], dens_new = sh.rho[2] * sh.rho[3];
      if (fabs(dens_old) < PIMC_RZERO) dens_old = 0.0;
      if (dens_old < 0.0) neg = 1;
      if (fabs(dens_new) < PIMC_RZERO) dens_new = 0.0;
      if (dens_new < 0.0) neg = 1;
      rd = (dens_old > PIMC_RZERO) ? dens_new / dens_old : 1.0;
      rd *= exp(-s.tau * (sh.pot[1] - sh.pot[0]));
      acc = (rd > 1.0) || (rd > u[2]);
    } else {
      double dens_old = sh.rho[0] + sh.rho[1], dens_new = sh.rho[2] + sh.rho[3];
      if (fabs(dens_old) < PIMC_RZERO) dens_old = 0.0;
      if (fabs(dens_new) < PIMC_RZERO) dens_new = 0.0;
      rd = dens_new - dens_old - s.tau * (sh.pot[1] - sh.pot[0]);
      acc = (rd > 0.0) || (rd > log(u[2]));
    }
    if (neg) { atomicOr(c.st.err, (unsigned)DERR_NEG_DENSITY); acc = 0; }
    sh.acc = acc;
    if (rd_out) *rd_out = rd;
    if (acc) {
      c.st.ang[n + r1] = sh.ang_new[1];
      c.st.ang[r1] = sh.ang_new[0];
      for (int d = 0; d < 3; d++) c.st.cosv[d * n + r1] = nnew[d];
    }
  }
  __syncthreads();
  int acc = sh.acc;
  __syncthreads();
  return acc;
}
