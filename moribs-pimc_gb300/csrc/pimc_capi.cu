// pimc_capi.cu -- the extern "C" entry points of include/pimc_gb300.h: handle
// life cycle, table preparation, path transfers, replay moves, energy
// queries, estimators and the graph-captured production pass.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/pimc_gb300.h"
#include "pimc_kernels.cuh"
#include "pimc_launch.h"

#define CK(x)                                                  \
  do {                                                         \
    cudaError_t e_ = (x);                                      \
    if (e_ != cudaSuccess) {                                   \
      h->last_cuda = e_;                                       \
      return PIMC_ERR_CUDA;                                    \
    }                                                          \
  } while (0)

struct pimc_handle {
  int device = 0;
  cudaStream_t stream = nullptr;
  pimc_system sys;
  Ctx ctx;
  Frame *frames = nullptr;
  unsigned long long *cnt = nullptr;   // [type][kind][total, accepted]
  unsigned *pass = nullptr;
  MolScratch *ms = nullptr;
  long *cursors = nullptr;             // replay cursors: gauss, u, d
  std::vector<void *> owned;           // table buffers
  std::vector<double> angles_host;     // full MCAngles copy (non-rotor rows kept as given)
  std::vector<int> pindex_host;
  std::vector<double> cosine_host;
  bool tables = false, state = false;
  cudaGraphExec_t pass_exec = nullptr;
  cudaGraphExec_t worm_exec = nullptr;  // one captured worm-branch pass (pimc_worm_run)
  cudaGraphExec_t da_exec = nullptr;    // one captured pimc_da_sweeps call and its key
  int da_nsweeps = -1, da_use = -1;
  uint64_t da_seed = 0;
  float da_escale = 0.0f;
  unsigned long long da_mlp = 0;
  const void *da_buf = nullptr;
  long long da_nodes = 0;
  uint64_t worm_seed = 0;
  long long worm_nodes = 0;
  uint64_t pass_seed = 0;
  long long nodes_per_pass = 0;
  long long launches = 0;
  cudaError_t last_cuda = cudaSuccess;
  // growable scratch for queries
  void *qbuf = nullptr;
  size_t qbytes = 0;
  // production schedule: fused bisection blocks and persistent rotation sweeps
  int fused = 1;
  unsigned long long *prog = nullptr;  // per-CTA progress words of the persistent rotation launches
  unsigned *abort_word = nullptr;
  int nprog = 0;
  // the handle as a one-replica batch, for the half-sweep kernel that makes
  // small multi-rotor moves one warp each (uploaded before every pass launch)
  BatchRep self_host{};
  BatchRep *self_rep = nullptr;
  int *self_idx = nullptr;             // the half-sweep kernel's replica order {0} and unit offsets {0, Q/2}
  // pair-density histograms (allocated on first use)
  DensHist dens{nullptr, nullptr, nullptr, nullptr};
  int dens_on = 0;
  // worm algorithm (allocated by pimc_worm_init)
  DevWorm *worm = nullptr;
  int *rindex = nullptr;
  long *wcur = nullptr;
  void *wscr = nullptr;                // production worm scratch (bridge segment, neighbour table, cycles)
  int worm_on = 0;
};

extern "C" const char *pimc_status_string(pimc_status s)
{
  switch (s) {
    case PIMC_OK: return "ok";
    case PIMC_ERR_BAD_ARG: return "bad argument";
    case PIMC_ERR_BAD_TABLE: return "bad or missing table";
    case PIMC_ERR_GRID_RANGE: return "rotational density grid index out of range";
    case PIMC_ERR_NEG_DENSITY: return "negative rotational density";
    case PIMC_ERR_TIMEOUT: return "device wait timed out";
    case PIMC_ERR_CUDA: return "CUDA error";
    case PIMC_ERR_NO_DEVICE: return "no CUDA device";
    case PIMC_ERR_SIZE: return "size beyond a compiled limit";
    case PIMC_ERR_STATE: return "call out of order";
  }
  return "unknown";
}

// ------------------------------------------------------------ helpers

template <class T>
static pimc_status dalloc(pimc_handle *h, T **p, size_t n)
{
  void *v = nullptr;
  CK(cudaMalloc(&v, n * sizeof(T) > 0 ? n * sizeof(T) : 1));
  *p = (T *)v;
  return PIMC_OK;
}

static pimc_status upload(pimc_handle *h, const double *src, size_t n, const double **dst)
{
  double *d = nullptr;
  pimc_status st = dalloc(h, &d, n);
  if (st) return st;
  h->owned.push_back(d);
  CK(cudaMemcpyAsync(d, src, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  *dst = d;
  return PIMC_OK;
}

static pimc_status upload_f32(pimc_handle *h, const double *src, size_t n, const float **dst)
{
  std::vector<float> f(n);
  for (size_t i = 0; i < n; i++) f[i] = (float)src[i];
  float *d = nullptr;
  pimc_status st = dalloc(h, &d, n);
  if (st) return st;
  h->owned.push_back(d);
  CK(cudaMemcpy(d, f.data(), n * sizeof(float), cudaMemcpyHostToDevice));
  *dst = d;
  return PIMC_OK;
}

static pimc_status upload_f4(pimc_handle *h, const std::vector<float4> &v, const float4 **dst)
{
  float4 *d = nullptr;
  pimc_status st = dalloc(h, &d, v.size());
  if (st) return st;
  h->owned.push_back(d);
  CK(cudaMemcpy(d, v.data(), v.size() * sizeof(float4), cudaMemcpyHostToDevice));
  *dst = d;
  return PIMC_OK;
}

static pimc_status scratch(pimc_handle *h, size_t bytes, void **p)
{
  if (bytes > h->qbytes) {
    if (h->qbuf) CK(cudaFree(h->qbuf));
    h->qbuf = nullptr;
    CK(cudaMalloc(&h->qbuf, bytes));
    h->qbytes = bytes;
  }
  *p = h->qbuf;
  return PIMC_OK;
}

static pimc_status check_err(pimc_handle *h)
{
  CK(cudaStreamSynchronize(h->stream));
  unsigned e = 0;
  CK(cudaMemcpy(&e, h->ctx.st.err, sizeof(unsigned), cudaMemcpyDeviceToHost));
  if (e) {
    unsigned z = 0;
    CK(cudaMemcpy(h->ctx.st.err, &z, sizeof(unsigned), cudaMemcpyHostToDevice));
    if (e & DERR_GRID_RANGE) return PIMC_ERR_GRID_RANGE;
    if (e & DERR_NEG_DENSITY) return PIMC_ERR_NEG_DENSITY;
    if (e & DERR_TIMEOUT) {
      // the aborted sweep has ended; the next launches run normally, from
      // freshly evaluated rotor caches
      CK(cudaMemset(h->abort_word, 0, sizeof(unsigned)));
      launch_invalidate_caches(h->ctx, h->stream);
      h->launches++;
      CK(cudaStreamSynchronize(h->stream));
      return PIMC_ERR_TIMEOUT;
    }
    if (e & DERR_STREAM) return PIMC_ERR_BAD_ARG;
    if (e & DERR_PERM) return PIMC_ERR_BAD_ARG;
  }
  return PIMC_OK;
}

// PIndex as the reference keeps it (mc_setup.cc:337, mc_qworm.cc:538-541):
// a bijection of [0, na) whose first numb entries, for every boson type,
// map [0, numb) onto itself (the cycles the exchange moves and estimators
// walk, mc_piqmc.cc:129-138, mc_estim.cc:2008-2013).  Anything else would
// make those walks run off their cycle.
static bool perm_ok(const DevSys &d, const int *p)
{
  std::vector<char> seen(d.na, 0);
  for (int a = 0; a < d.na; a++) {
    int v = p[a];
    if (v < 0 || v >= d.na || seen[v]) return false;
    seen[v] = 1;
  }
  for (int t = 0; t < d.ntypes; t++) {
    if (d.stat[t] != PIMC_BOSE) continue;
    for (int a = 0; a < d.numb[t]; a++)
      if (p[a] >= d.numb[t]) return false;
  }
  return true;
}

// cubic spline second derivatives with end slopes from the first and last
// intervals: init_spline + spline (mc_utils.cc:112-154, 188-201)
static void spline_y2(const double *x, const double *y, int n, double *y2)
{
  double yp1 = (y[1] - y[0]) / (x[1] - x[0]);
  double ypn = (y[n - 1] - y[n - 2]) / (x[n - 1] - x[n - 2]);
  std::vector<double> u(n);
  y2[0] = -.5;
  u[0] = (3. / (x[1] - x[0])) * ((y[1] - y[0]) / (x[1] - x[0]) - yp1);
  for (int i = 1; i < n - 1; i++) {
    double sig = (x[i] - x[i - 1]) / (x[i + 1] - x[i - 1]);
    double p = sig * y2[i - 1] + 2.;
    y2[i] = (sig - 1.) / p;
    u[i] = (y[i + 1] - y[i]) / (x[i + 1] - x[i]) - (y[i] - y[i - 1]) / (x[i] - x[i - 1]);
    u[i] = (6. * u[i] / (x[i + 1] - x[i - 1]) - sig * u[i - 1]) / p;
  }
  double qn = .5;
  double un = (3. / (x[n - 1] - x[n - 2])) * (ypn - (y[n - 1] - y[n - 2]) / (x[n - 1] - x[n - 2]));
  y2[n - 1] = (un - qn * u[n - 2]) / (qn * y2[n - 2] + 1.);
  for (int k = n - 2; k >= 0; k--) y2[k] = y2[k] * y2[k + 1] + u[k];
}

// a grid on which the spline index can be computed: monotonic, and no node
// more than half a step away from x0 + i*h
static bool near_uniform(const double *x, int n, double *x0, double *ih)
{
  if (n < 3) return false;
  double h = (x[n - 1] - x[0]) / (double)(n - 1);
  if (!(h > 0.0)) return false;
  for (int i = 1; i < n; i++) {
    if (!(x[i] > x[i - 1])) return false;
    if (fabs(x[i] - (x[0] + i * h)) > 0.5 * h) return false;
  }
  *x0 = x[0];
  *ih = 1.0 / h;
  return true;
}

// ------------------------------------------------------------ life cycle

// validate a system and derive its device description (mc_setup.cc:135-163,
// 321-453: counts, offsets, tau, RotRatio)
static pimc_status build_devsys(const pimc_system &s, DevSys &d)
{
  if (s.ntypes < 1 || s.ntypes > PIMC_MAX_TYPES || s.nslices < 2 || s.temperature <= 0.0) return PIMC_ERR_BAD_ARG;
  int na = 0, imtype = -1, nmol = 0;
  for (int t = 0; t < s.ntypes; t++) {
    const pimc_type &ty = s.type[t];
    if (ty.numb < 0 || ty.levels < 1 || ty.levels > 6 || ty.lambda <= 0.0) return PIMC_ERR_BAD_ARG;
    // an atom type may be empty beside a molecule type (a replica family whose
    // solvent count is drawn from 0 up); it then has no moves and no partners
    if (ty.numb == 0 && (ty.molecule != PIMC_ATOM || s.ntypes < 2)) return PIMC_ERR_BAD_ARG;
    if ((1 << ty.levels) >= s.nslices) return PIMC_ERR_BAD_ARG;       // mc_setup.cc:397-398
    if (ty.molecule < 0 || ty.molecule > 2) return PIMC_ERR_BAD_ARG;
    if (ty.molecule != PIMC_ATOM) { imtype = t; nmol++; }
    else if (nmol > 0) return PIMC_ERR_BAD_ARG;                       // atoms first (mc_input.cc:194)
    na += ty.numb;
  }
  if (nmol > 1 || na > PIMC_MAX_ATOMS) return PIMC_ERR_SIZE;
  if (imtype >= 0 && s.type[imtype].molecule == PIMC_LINEAR && s.type[imtype].numb != 1) return PIMC_ERR_BAD_ARG;
  if (imtype >= 0 && s.type[imtype].numb > PIMC_MAX_ROTORS) return PIMC_ERR_SIZE;
  int Q = s.rotation ? s.nrotslices : 0;
  if (s.rotation && (imtype < 0 || Q < 1 || s.nslices % Q)) return PIMC_ERR_BAD_ARG;   // mc_setup.cc:382-389
  if (s.rotation && s.nslices / Q > 16) return PIMC_ERR_SIZE;
  memset(&d, 0, sizeof(d));
  d.na = na;
  d.nap = (na + 31) / 32 * 32;
  d.P = s.nslices;
  // without rotation the reference keeps one orientation per translational
  // slice (RotRatio = 1, mc_setup.cc:379); store P orientations then
  d.Q = Q > 0 ? Q : s.nslices;
  d.R = Q > 0 ? s.nslices / Q : 1;
  d.ntypes = s.ntypes;
  d.imtype = imtype;
  int g = 0;
  for (int t = 0; t < s.ntypes; t++) {
    d.numb[t] = s.type[t].numb;
    d.molecule[t] = s.type[t].molecule;
    d.stat[t] = s.type[t].stat;
    d.levels[t] = s.type[t].levels;
    d.first[t] = g;
    d.lambda[t] = s.type[t].lambda;
    d.mcstep[t] = s.type[t].mcstep;
    g += s.type[t].numb;
  }
  d.nrotors = imtype >= 0 ? s.type[imtype].numb : 0;
  d.rot_first = imtype >= 0 ? d.first[imtype] : 0;
  d.beta = 1.0 / s.temperature;                       // mc_setup.cc:373-377
  d.tau = d.beta / (double)s.nslices;
  for (int t = 0; t < s.ntypes; t++) {
    double bnorm = 1.0 / (d.lambda[t] * d.tau);
    for (int l = 0; l < d.levels[t]; l++) {
      d.bis_sq[t][l] = sqrt(bnorm / (double)(1 << (d.levels[t] - l)));
      d.bis_isq[t][l] = 1.0 / d.bis_sq[t][l];
    }
  }
  d.rot_tau = Q > 0 ? d.beta / (double)Q : 0.0;
  d.temperature = s.temperature;
  d.rtstep = s.rtstep;
  d.ispher = s.ispher;
  d.rot_den_type = s.rot_den_type;
  d.rot_odevn = s.rot_odevn;
  d.rn_ratio = s.rn_ratio > 0 ? s.rn_ratio : 1;
  d.rot_eoff = s.rot_eoff;
  for (int k = 0; k < 3; k++) { d.abc[k] = s.rot_abc[k]; d.box[k] = s.box[k]; }
  {
    double b[3];
    for (int k = 0; k < 3; k++) b[k] = d.abc[k] > 0.0 ? 1.0 / d.abc[k] : 0.0;
    d.rs_coef[0] = (float)(b[0] - b[1] - b[2]);
    d.rs_coef[1] = (float)(b[1] - b[2] - b[0]);
    d.rs_coef[2] = (float)(b[2] - b[0] - b[1]);
    d.rs_scale = d.rot_tau > 0.0 ? (float)(1.0 / (4.0 * (d.rot_tau / PIMC_WNO2K))) : 0.0f;
  }
  d.minimage = s.minimage;
  d.wait_ns = 2000000000ull;
  return PIMC_OK;
}

extern "C" pimc_status pimc_create(const pimc_system *sys, int device, pimc_handle **out)
{
  if (!sys || !out) return PIMC_ERR_BAD_ARG;
  *out = nullptr;
  const pimc_system &s = *sys;
  DevSys dsys;
  pimc_status e0 = build_devsys(s, dsys);
  if (e0) return e0;
  const int na = dsys.na;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return PIMC_ERR_NO_DEVICE;
  if (device < 0 || device >= ndev) return PIMC_ERR_BAD_ARG;

  pimc_handle *h = new (std::nothrow) pimc_handle();
  if (!h) return PIMC_ERR_SIZE;
  h->device = device;
  h->sys = s;
  CK(cudaSetDevice(device));
  CK(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
  DevSys &d = h->ctx.s;
  d = dsys;
  int g;
  DevState &st = h->ctx.st;
  size_t nb = (size_t)d.P * d.nap;
  size_t nr = (size_t)(d.nrotors > 0 ? d.nrotors : 1) * d.Q;
  pimc_status e;
  if ((e = dalloc(h, &st.x, nb)) || (e = dalloc(h, &st.y, nb)) || (e = dalloc(h, &st.z, nb)) ||
      (e = dalloc(h, &st.b4, nb)) ||
      (e = dalloc(h, &st.cosvf, 3 * nr)) || (e = dalloc(h, &st.rp_cache, nr)) || (e = dalloc(h, &st.rl_cache, nr)) ||
      (e = dalloc(h, &st.rp_ok, nr)) || (e = dalloc(h, &st.rl_ok, nr)) ||
      (e = dalloc(h, &st.ang, 3 * nr)) || (e = dalloc(h, &st.cosv, 3 * nr)) || (e = dalloc(h, &st.pindex, na)) ||
      (e = dalloc(h, &st.mctype, na)) || (e = dalloc(h, &st.err, 1)) || (e = dalloc(h, &h->frames, nr)) ||
      (e = dalloc(h, &h->cnt, 12)) || (e = dalloc(h, &h->pass, 1)) || (e = dalloc(h, &h->cursors, 8)) ||
      (e = dalloc(h, &h->prog, (size_t)(d.Q > 0 ? d.Q : 1))) || (e = dalloc(h, &h->abort_word, 1)) ||
      (e = dalloc(h, &h->self_rep, 1)) || (e = dalloc(h, &h->self_idx, 3))) {
    pimc_destroy(h);
    return e;
  }
  {
    const int idx[3] = {0, 0, d.Q / 2};
    CK(cudaMemcpy(h->self_idx, idx, sizeof(idx), cudaMemcpyHostToDevice));
  }
  void *msv = nullptr;
  if (cudaMalloc(&msv, mol_scratch_bytes()) != cudaSuccess) { pimc_destroy(h); return PIMC_ERR_CUDA; }
  h->ms = (MolScratch *)msv;
  CK(cudaMemset(st.x, 0, nb * sizeof(double)));
  CK(cudaMemset(st.y, 0, nb * sizeof(double)));
  CK(cudaMemset(st.z, 0, nb * sizeof(double)));
  CK(cudaMemset(st.b4, 0, nb * sizeof(float4)));
  CK(cudaMemset(st.rp_ok, 0, nr * sizeof(int)));
  CK(cudaMemset(st.rl_ok, 0, nr * sizeof(int)));
  CK(cudaMemset(st.err, 0, sizeof(unsigned)));
  CK(cudaMemset(h->cnt, 0, 12 * sizeof(unsigned long long)));
  CK(cudaMemset(h->pass, 0, sizeof(unsigned)));
  h->nprog = d.Q > 0 ? d.Q : 1;
  CK(cudaMemset(h->prog, 0, (size_t)h->nprog * sizeof(unsigned long long)));
  CK(cudaMemset(h->abort_word, 0, sizeof(unsigned)));
  std::vector<int> mct(na), pidx(na);
  g = 0;
  for (int t = 0; t < s.ntypes; t++)
    for (int a = 0; a < s.type[t].numb; a++) mct[g++] = t;        // mc_setup.cc:327-333
  for (int a = 0; a < na; a++) pidx[a] = a;                       // mc_setup.cc:335-339
  CK(cudaMemcpy(st.mctype, mct.data(), na * sizeof(int), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(st.pindex, pidx.data(), na * sizeof(int), cudaMemcpyHostToDevice));
  h->pindex_host = pidx;
  h->angles_host.assign(3 * (size_t)na * d.P, 0.0);
  h->cosine_host.assign(3 * (size_t)na * d.P, 0.0);
  *out = h;
  return PIMC_OK;
}

extern "C" pimc_status pimc_destroy(pimc_handle *h)
{
  if (!h) return PIMC_ERR_BAD_ARG;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  if (h->pass_exec) cudaGraphExecDestroy(h->pass_exec);
  if (h->worm_exec) cudaGraphExecDestroy(h->worm_exec);
  if (h->da_exec) cudaGraphExecDestroy(h->da_exec);
  DevState &st = h->ctx.st;
  void *bufs[] = {st.x, st.y, st.z, st.b4, st.cosvf, st.rp_cache, st.rl_cache, st.rp_ok, st.rl_ok,
                  st.ang, st.cosv, st.pindex, st.mctype, st.err, h->frames, h->cnt, h->pass, h->cursors, h->ms,
                  h->qbuf, h->prog, h->abort_word, h->dens.g1, h->dens.g2, h->dens.g3, h->dens.rel, h->worm, h->rindex,
                  h->wcur, h->wscr, h->self_rep, h->self_idx};
  for (void *b : bufs)
    if (b) cudaFree(b);
  for (void *b : h->owned) cudaFree(b);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return PIMC_OK;
}

// ------------------------------------------------------------ tables

// The tables of the system d into t, buffers owned by h.  parts bit 0: the
// potentials (1D, 2D, 3D, spherical), bit 1: the rotational density
// matrices (linear-rotor .rot spline, top (theta, phi, chi) grid).
#define TAB_POT 1
#define TAB_ROT 2
static pimc_status load_tables_into(pimc_handle *h, const pimc_tables *tb, DevTables &t, const DevSys &d, int parts)
{
  pimc_status e;
  bool need1d = false, need2d = false, need3d = false, needrot = false, need3drho = false;
  for (int k = 0; k < d.ntypes; k++) {
    if (d.molecule[k] == PIMC_ATOM) need1d = true;
    if (d.molecule[k] == PIMC_LINEAR) { need2d = true; if (h->sys.rotation && d.rot_den_type == 0) needrot = true; }
    if (d.molecule[k] == PIMC_NONLINEAR) {
      if (d.ntypes > 1 && !d.ispher) need3d = true;
      if (d.ntypes > 1 && h->sys.rotation) need3d = true;          // PotRotE3D uses vcord regardless of ISPHER
      if (h->sys.rotation && (d.rot_den_type == 0 || d.nrotors > 0)) need3drho = true;
    }
  }
  if (need1d && d.numb[0] < 2) need1d = false;                     // a single atom has no atom partner
  if (!(parts & TAB_POT)) need1d = need2d = need3d = false;
  if (!(parts & TAB_ROT)) needrot = need3drho = false;
  if (need1d) {
    int n = tb->n1d;
    if (n < 2 || !tb->grid1d || !tb->pot1d) return PIMC_ERR_BAD_TABLE;
    std::vector<double> y2(n);
    spline_y2(tb->grid1d, tb->pot1d, n, y2.data());
    t.n1d = n;
    if ((e = upload(h, tb->grid1d, n, &t.g1d)) || (e = upload(h, tb->pot1d, n, &t.p1d)) ||
        (e = upload(h, y2.data(), n, &t.y21d)) || (e = upload_f32(h, tb->grid1d, n, &t.g1d32)) ||
        (e = upload_f32(h, tb->pot1d, n, &t.p1d32)) || (e = upload_f32(h, y2.data(), n, &t.y21d32)))
      return e;
    t.uni1d = near_uniform(tb->grid1d, n, &t.x01d, &t.ih1d) ? 1 : 0;
    if (t.uni1d) {
      // FP32 path: the spline words of interval k in one 16-byte word
      std::vector<float4> w(n - 1);
      for (int k = 0; k < n - 1; k++)
        w[k] = make_float4((float)tb->pot1d[k], (float)y2[k], (float)tb->pot1d[k + 1], (float)y2[k + 1]);
      if ((e = upload_f4(h, w, &t.sp1d4))) return e;
      double hstep = 1.0 / t.ih1d;
      t.f_h1d = (float)hstep;
      t.f_h2_6 = (float)(hstep * hstep / 6.0);
    }
    // short- and long-range extrapolation constants (mc_poten.cc:418-437)
    double fr = tb->pot1d[0] / tb->pot1d[1];
    double dr = tb->grid1d[1] - tb->grid1d[0];
    t.alpha1d = log(fr) / dr;
    t.unode1d = tb->pot1d[0] * exp(t.alpha1d * tb->grid1d[0]);
    double r0 = pow(tb->grid1d[n - 2], 6.0), r1 = pow(tb->grid1d[n - 1], 6.0);
    fr = tb->pot1d[n - 1] - tb->pot1d[n - 2];
    t.c61d = fr / (1.0 / r0 - 1.0 / r1);
  }
  if (need2d) {
    if (tb->nr2d < 2 || tb->nc2d < 2 || !tb->pot2d || !tb->rgrid2d || !tb->cgrid2d || tb->dr2d <= 0 || tb->dc2d <= 0)
      return PIMC_ERR_BAD_TABLE;
    t.nr2d = tb->nr2d; t.nc2d = tb->nc2d; t.dr2d = tb->dr2d; t.dc2d = tb->dc2d;
    if ((e = upload(h, tb->rgrid2d, tb->nr2d, &t.rg2d)) || (e = upload(h, tb->cgrid2d, tb->nc2d, &t.cg2d)) ||
        (e = upload(h, tb->pot2d, (size_t)tb->nr2d * tb->nc2d, &t.pot2d)) ||
        (e = upload_f32(h, tb->rgrid2d, tb->nr2d, &t.rg2d32)) || (e = upload_f32(h, tb->cgrid2d, tb->nc2d, &t.cg2d32)) ||
        (e = upload_f32(h, tb->pot2d, (size_t)tb->nr2d * tb->nc2d, &t.pot2d32)))
      return e;
    // FP32 path: the four corners of each cell in one 16-byte word
    int nr = tb->nr2d, nc = tb->nc2d;
    std::vector<float4> w((size_t)(nr - 1) * (nc - 1));
    for (int ir = 0; ir < nr - 1; ir++)
      for (int ic = 0; ic < nc - 1; ic++) {
        const double *q = tb->pot2d + (size_t)ir * nc + ic;
        w[(size_t)ir * (nc - 1) + ic] = make_float4((float)q[0], (float)q[nc], (float)q[nc + 1], (float)q[1]);
      }
    if ((e = upload_f4(h, w, &t.pot2d4))) return e;
    t.f_rmin2d = (float)tb->rgrid2d[0];
    t.f_cmin2d = (float)tb->cgrid2d[0];
  }
  if (need3d) {
    if (tb->rgrd < 2 || tb->thgrd < 2 || tb->chgrd < 2 || !tb->vtable || tb->rvmax <= tb->rvmin) return PIMC_ERR_BAD_TABLE;
    t.rgrd = tb->rgrd; t.thgrd = tb->thgrd; t.chgrd = tb->chgrd;
    int fold = tb->chi_fold_deg;
    if (fold == 0) fold = (t.chgrd == 181) ? 180 : (t.chgrd == 361 ? 360 : 90);    // vcord.f:78-85
    if (fold != 90 && fold != 180 && fold != 360) return PIMC_ERR_BAD_TABLE;
    t.chfold = fold;
    t.rvmin = tb->rvmin; t.rvmax = tb->rvmax;
    t.rvstep = (t.rvmax - t.rvmin) / (double)(t.rgrd - 1);      // mc_poten.cc:288
    t.dth3 = 180.0 / (double)(t.thgrd - 1);
    t.dch3 = (double)fold / (double)(t.chgrd - 1);
    size_t n = (size_t)t.rgrd * t.thgrd * t.chgrd;
    if ((e = upload(h, tb->vtable, n, &t.vtab)) || (e = upload_f32(h, tb->vtable, n, &t.vtab32))) return e;
    // FP32 path: each point's value and vcalc's one-sided differences
    // (vcalc.f:40-60) in one 16-byte word
    {
      size_t nth = t.thgrd, nch = t.chgrd;
      std::vector<float4> w(n);
      for (int ir = 0; ir < t.rgrd; ir++)
        for (int it = 0; it < t.thgrd; it++)
          for (int ic = 0; ic < t.chgrd; ic++) {
            size_t i0 = ((size_t)ir * nth + it) * nch + ic;
            double v0 = tb->vtable[i0];
            double dr = ir < t.rgrd - 1 ? tb->vtable[i0 + nth * nch] - v0 : 0.0;
            double dt = it < t.thgrd - 1 ? tb->vtable[i0 + nch] - v0 : 0.0;
            double dc = ic < t.chgrd - 1 ? tb->vtable[i0 + 1] - v0 : 0.0;
            w[i0] = make_float4((float)v0, (float)dr, (float)dt, (float)dc);
          }
      if ((e = upload_f4(h, w, &t.vtab4))) return e;
      t.f_irstep = (float)(1.0 / t.rvstep);
    }
  }
  if ((parts & TAB_POT) && d.ispher && d.ntypes > 1) {
    if (tb->nsph < 2 || !tb->sph_table || tb->sph_rstep <= 0) return PIMC_ERR_BAD_TABLE;
    t.nsph = tb->nsph; t.sph_r0 = tb->sph_r0; t.sph_rmax = tb->sph_rmax; t.sph_rstep = tb->sph_rstep;
    if ((e = upload(h, tb->sph_table, tb->nsph, &t.sph))) return e;
  }
  if (needrot) {
    int n = tb->nrot;
    if (n < 2 || !tb->rotgrid || !tb->rotdens || !tb->rotderv || !tb->rotesqr) return PIMC_ERR_BAD_TABLE;
    std::vector<double> a(n), b(n), c(n);
    t.unirot = near_uniform(tb->rotgrid, n, &t.x0rot, &t.ihrot) ? 1 : 0;
    spline_y2(tb->rotgrid, tb->rotdens, n, a.data());              // init_rotdens mc_poten.cc:543-545
    spline_y2(tb->rotgrid, tb->rotderv, n, b.data());
    spline_y2(tb->rotgrid, tb->rotesqr, n, c.data());
    t.nrot = n;
    if ((e = upload(h, tb->rotgrid, n, &t.rg)) || (e = upload(h, tb->rotdens, n, &t.rd)) ||
        (e = upload(h, tb->rotderv, n, &t.rdv)) || (e = upload(h, tb->rotesqr, n, &t.rde)) ||
        (e = upload(h, a.data(), n, &t.rd_y2)) || (e = upload(h, b.data(), n, &t.rdv_y2)) ||
        (e = upload(h, c.data(), n, &t.rde_y2)))
      return e;
    // FP32 path: the density spline words per interval, counted from the top
    // node cos(gamma) = 1 of a uniform grid
    t.rd4 = nullptr;
    if (t.unirot && fabs(tb->rotgrid[n - 1] - 1.0) < 1e-9) {
      std::vector<float4> w(n - 1);
      for (int k = 0; k < n - 1; k++)
        w[k] = make_float4((float)tb->rotdens[k], (float)a[k], (float)tb->rotdens[k + 1], (float)a[k + 1]);
      if ((e = upload_f4(h, w, &t.rd4))) return e;
      double hstep = 1.0 / t.ihrot;
      t.f_ihrot = (float)t.ihrot;
      t.f_hrot2_6 = (float)(hstep * hstep / 6.0);
    }
  }
  if (need3drho) {
    if (tb->nth < 2 || tb->nph < 2 || tb->nch < 2 || !tb->rhoprp || !tb->erotpr || !tb->erotsq) {
      if (d.rot_den_type == 0) return PIMC_ERR_BAD_TABLE;
    } else {
      t.nth = tb->nth; t.nph = tb->nph; t.nch = tb->nch;
      t.dthd = 180.0 / (double)(t.nth - 1);
      t.dphd = 360.0 / (double)(t.nph - 1);
      t.dchd = 360.0 / (double)(t.nch - 1);
      size_t n = (size_t)t.nth * t.nph * t.nch;
      if ((e = upload(h, tb->rhoprp, n, &t.rho)) || (e = upload(h, tb->erotpr, n, &t.erot)) ||
          (e = upload(h, tb->erotsq, n, &t.esq)) || (e = upload_f32(h, tb->rhoprp, n, &t.rho32)))
        return e;
      // FP32 path: value and rotpro's one-sided differences along chi, phi,
      // theta (rotpro_sub.f:30-60) in one 16-byte word
      size_t nph = t.nph, nch = t.nch;
      std::vector<float4> w(n);
      for (int it = 0; it < t.nth; it++)
        for (int ip = 0; ip < t.nph; ip++)
          for (int ic = 0; ic < t.nch; ic++) {
            size_t i0 = ((size_t)it * nph + ip) * nch + ic;
            double r0 = tb->rhoprp[i0];
            double dc = ic < t.nch - 1 ? tb->rhoprp[i0 + 1] - r0 : 0.0;
            double dp = ip < t.nph - 1 ? tb->rhoprp[i0 + nch] - r0 : 0.0;
            double dt = it < t.nth - 1 ? tb->rhoprp[i0 + nph * nch] - r0 : 0.0;
            w[i0] = make_float4((float)r0, (float)dc, (float)dp, (float)dt);
          }
      if ((e = upload_f4(h, w, &t.rho4))) return e;
    }
  }
  // float constants of the FP32 leaves
  const double deg = 180.0 / 3.14159265358979323846;
  t.f_x01d = (float)t.x01d; t.f_ih1d = (float)t.ih1d; t.f_c61d = (float)t.c61d;
  t.f_unode1d = (float)t.unode1d; t.f_alpha1d = (float)t.alpha1d;
  t.f_dr2d = (float)t.dr2d; t.f_dc2d = (float)t.dc2d;
  t.f_thscale = t.dth3 > 0 ? (float)(deg / t.dth3) : 0.f;
  t.f_chscale = t.dch3 > 0 ? (float)(deg / t.dch3) : 0.f;
  t.f_rvmin = (float)t.rvmin; t.f_rvmax = (float)t.rvmax; t.f_rvstep = (float)t.rvstep;
  t.f_dscale[0] = t.dthd > 0 ? (float)(deg / t.dthd) : 0.f;
  t.f_dscale[1] = t.dphd > 0 ? (float)(deg / t.dphd) : 0.f;
  t.f_dscale[2] = t.dchd > 0 ? (float)(deg / t.dchd) : 0.f;
  t.d_thscale = t.dth3 > 0 ? deg / t.dth3 : 0.0;
  t.d_chscale = t.dch3 > 0 ? deg / t.dch3 : 0.0;
  t.d_irstep = t.rvstep > 0 ? 1.0 / t.rvstep : 0.0;
  t.d_idr2d = t.dr2d > 0 ? 1.0 / t.dr2d : 0.0;
  t.d_idc2d = t.dc2d > 0 ? 1.0 / t.dc2d : 0.0;
  t.d_dscale[0] = t.dthd > 0 ? deg / t.dthd : 0.0;
  t.d_dscale[1] = t.dphd > 0 ? deg / t.dphd : 0.0;
  t.d_dscale[2] = t.dchd > 0 ? deg / t.dchd : 0.0;
  return PIMC_OK;
}

extern "C" pimc_status pimc_load_tables(pimc_handle *h, const pimc_tables *tb)
{
  if (!h || !tb) return PIMC_ERR_BAD_ARG;
  CK(cudaSetDevice(h->device));
  pimc_status e = load_tables_into(h, tb, h->ctx.t, h->ctx.s, TAB_POT | TAB_ROT);
  if (e) return e;
  if (h->state) {
    launch_derive_state(h->ctx, h->frames, h->stream);     // the float copies follow the tables' path choice
    h->launches++;
    CK(cudaGetLastError());
  }
  CK(cudaStreamSynchronize(h->stream));
  h->tables = true;
  if (h->pass_exec) { cudaGraphExecDestroy(h->pass_exec); h->pass_exec = nullptr; }
  if (h->worm_exec) { cudaGraphExecDestroy(h->worm_exec); h->worm_exec = nullptr; }
  if (h->da_exec) { cudaGraphExecDestroy(h->da_exec); h->da_exec = nullptr; }
  return PIMC_OK;
}

// ------------------------------------------------------------ path

extern "C" pimc_status pimc_set_state(pimc_handle *h, const double *coords, const double *angles, const int *pindex)
{
  if (!h) return PIMC_ERR_BAD_ARG;
  CK(cudaSetDevice(h->device));
  const DevSys &d = h->ctx.s;
  if (pindex && !perm_ok(d, pindex)) return PIMC_ERR_BAD_ARG;
  size_t nbr = (size_t)d.na * d.P;      // reference layout length per row
  if (coords) {
    // [3][na*P] -> slice-major x/y/z[t*nap + a]
    std::vector<double> buf((size_t)d.P * d.nap, 0.0);
    double *dst[3] = {h->ctx.st.x, h->ctx.st.y, h->ctx.st.z};
    for (int k = 0; k < 3; k++) {
      for (int a = 0; a < d.na; a++)
        for (int t = 0; t < d.P; t++) buf[(size_t)t * d.nap + a] = coords[k * nbr + (size_t)a * d.P + t];
      CK(cudaMemcpy(dst[k], buf.data(), buf.size() * sizeof(double), cudaMemcpyHostToDevice));
    }
  }
  if (angles) {
    memcpy(h->angles_host.data(), angles, 3 * nbr * sizeof(double));
    for (size_t i = 0; i < nbr; i++) {                      // mc_main.cc:193-199
      double phi = angles[i], cost = angles[nbr + i];
      double sint = sqrt(1.0 - cost * cost);
      h->cosine_host[i] = sint * cos(phi);
      h->cosine_host[nbr + i] = sint * sin(phi);
      h->cosine_host[2 * nbr + i] = cost;
    }
    if (d.nrotors > 0) {
      size_t n = (size_t)d.nrotors * d.Q;
      std::vector<double> ang(3 * n), cs(3 * n);
      for (int k = 0; k < 3; k++)
        for (int r = 0; r < d.nrotors; r++)
          for (int q = 0; q < d.Q; q++) {
            size_t src = k * nbr + (size_t)(d.rot_first + r) * d.P + q;
            ang[k * n + r * d.Q + q] = angles[src];
            cs[k * n + r * d.Q + q] = h->cosine_host[src];
          }
      CK(cudaMemcpy(h->ctx.st.ang, ang.data(), 3 * n * sizeof(double), cudaMemcpyHostToDevice));
      CK(cudaMemcpy(h->ctx.st.cosv, cs.data(), 3 * n * sizeof(double), cudaMemcpyHostToDevice));
    }
  }
  if (coords || angles) {
    launch_derive_state(h->ctx, h->frames, h->stream);     // float copies, frames, caches stale
    h->launches++;
    CK(cudaGetLastError());
    CK(cudaMemsetAsync(h->abort_word, 0, sizeof(unsigned), h->stream));   // a new path clears an aborted sweep
  }
  if (pindex) {
    CK(cudaMemcpy(h->ctx.st.pindex, pindex, d.na * sizeof(int), cudaMemcpyHostToDevice));
    h->pindex_host.assign(pindex, pindex + d.na);
    if (h->rindex) {
      std::vector<int> r(d.na);
      for (int a = 0; a < d.na; a++) r[pindex[a]] = a;
      CK(cudaMemcpy(h->rindex, r.data(), d.na * sizeof(int), cudaMemcpyHostToDevice));
    }
  }
  CK(cudaStreamSynchronize(h->stream));
  if (coords && angles) h->state = true;
  return PIMC_OK;
}

extern "C" pimc_status pimc_get_state(pimc_handle *h, double *coords, double *angles, double *cosine, int *pindex)
{
  if (!h) return PIMC_ERR_BAD_ARG;
  CK(cudaSetDevice(h->device));
  CK(cudaStreamSynchronize(h->stream));
  const DevSys &d = h->ctx.s;
  size_t nbr = (size_t)d.na * d.P;
  if (coords) {
    std::vector<double> buf((size_t)d.P * d.nap);
    double *src[3] = {h->ctx.st.x, h->ctx.st.y, h->ctx.st.z};
    for (int k = 0; k < 3; k++) {
      CK(cudaMemcpy(buf.data(), src[k], buf.size() * sizeof(double), cudaMemcpyDeviceToHost));
      for (int a = 0; a < d.na; a++)
        for (int t = 0; t < d.P; t++) coords[k * nbr + (size_t)a * d.P + t] = buf[(size_t)t * d.nap + a];
    }
  }
  if (angles || cosine) {
    if (d.nrotors > 0) {
      size_t n = (size_t)d.nrotors * d.Q;
      std::vector<double> ang(3 * n), cs(3 * n);
      CK(cudaMemcpy(ang.data(), h->ctx.st.ang, 3 * n * sizeof(double), cudaMemcpyDeviceToHost));
      CK(cudaMemcpy(cs.data(), h->ctx.st.cosv, 3 * n * sizeof(double), cudaMemcpyDeviceToHost));
      for (int k = 0; k < 3; k++)
        for (int r = 0; r < d.nrotors; r++)
          for (int q = 0; q < d.Q; q++) {
            size_t dst = k * nbr + (size_t)(d.rot_first + r) * d.P + q;
            h->angles_host[dst] = ang[k * n + r * d.Q + q];
            h->cosine_host[dst] = cs[k * n + r * d.Q + q];
          }
    }
    if (angles) memcpy(angles, h->angles_host.data(), 3 * nbr * sizeof(double));
    if (cosine) memcpy(cosine, h->cosine_host.data(), 3 * nbr * sizeof(double));
  }
  if (pindex) CK(cudaMemcpy(pindex, h->ctx.st.pindex, d.na * sizeof(int), cudaMemcpyDeviceToHost));
  return PIMC_OK;
}

static pimc_status ready(pimc_handle *h)
{
  if (!h) return PIMC_ERR_BAD_ARG;
  if (!h->tables || !h->state) return PIMC_ERR_STATE;
  CK(cudaSetDevice(h->device));
  return PIMC_OK;
}

// ------------------------------------------------------------ replay moves

static pimc_status put_stream(pimc_handle *h, const double *v, long n, double **dv, char *&cursor)
{
  *dv = (double *)cursor;
  if (n > 0) CK(cudaMemcpyAsync(*dv, v, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  cursor += ((size_t)(n > 0 ? n : 1) * sizeof(double) + 255) / 256 * 256;
  return PIMC_OK;
}

extern "C" pimc_status pimc_molecular_move_exchange(pimc_handle *h, int type, const double *u1, long n1,
                                                    const double *u2, long n2, long *consumed)
{
  pimc_status e = ready(h);
  if (e) return e;
  const DevSys &d = h->ctx.s;
  if (type < 0 || type >= d.ntypes || n1 < 0 || n2 < 0 || (n1 && !u1) || (n2 && !u2)) return PIMC_ERR_BAD_ARG;
  if (d.stat[type] != PIMC_BOSE) return PIMC_ERR_BAD_ARG;     // cycles of the boson type (mc_piqmc.cc:110-111)
  int numb = d.numb[type];
  for (int a = 0; a < numb; a++)
    if (h->pindex_host[a] < 0 || h->pindex_host[a] >= numb) return PIMC_ERR_BAD_ARG;
  size_t bytes = ((size_t)n1 + n2 + 16) * sizeof(double) + 2 * (size_t)numb * sizeof(int) + 8192;
  void *buf;
  if ((e = scratch(h, bytes, &buf))) return e;
  char *cur = (char *)buf;
  double *d1, *d2;
  if ((e = put_stream(h, u1, n1, &d1, cur)) || (e = put_stream(h, u2, n2, &d2, cur))) return e;
  CK(cudaMemsetAsync(h->cursors, 0, 8 * sizeof(long), h->stream));
  ReplaySrc src{nullptr, 0, h->cursors + 0, d2, n2, h->cursors + 1, d1, n1, h->cursors + 2, h->ctx.st.err};
  h->launches += launch_mol_exchange(h->ctx, h->frames, type, true, src, 0, h->pass, 0, cur, h->cnt, h->stream);
  launch_invalidate_caches(h->ctx, h->stream);
  h->launches++;
  CK(cudaGetLastError());
  long cz[8];
  CK(cudaMemcpyAsync(cz, h->cursors, 8 * sizeof(long), cudaMemcpyDeviceToHost, h->stream));
  e = check_err(h);
  if (consumed) { consumed[0] = cz[2]; consumed[1] = cz[1]; }
  return e;
}

extern "C" pimc_status pimc_bisection_move(pimc_handle *h, int type, int time, int exchange, const double *gauss,
                                           long ng, const double *u3, long n3, long *consumed, double *ds_out,
                                           int *lvl_out)
{
  pimc_status e = ready(h);
  if (e) return e;
  const DevSys &d = h->ctx.s;
  if (type < 0 || type >= d.ntypes || time < 0 || time >= d.P || ng < 0 || n3 < 0 || (ng && !gauss) || (n3 && !u3))
    return PIMC_ERR_BAD_ARG;
  int numb = d.numb[type], L = d.levels[type];
  if (exchange) {
    // the permutation is sampled for the boson type only (mc_main.cc:366-367)
    if (d.stat[type] != PIMC_BOSE) return PIMC_ERR_BAD_ARG;
    for (int a = 0; a < numb; a++)
      if (h->pindex_host[a] < 0 || h->pindex_host[a] >= numb) return PIMC_ERR_BAD_ARG;
  }
  size_t bytes = ((size_t)ng + n3 + 2 * (size_t)numb * L + numb + 16) * sizeof(double) + 4096;
  void *buf;
  if ((e = scratch(h, bytes, &buf))) return e;
  char *cur = (char *)buf;
  double *dg, *du, *dds;
  if ((e = put_stream(h, gauss, ng, &dg, cur)) || (e = put_stream(h, u3, n3, &du, cur))) return e;
  dds = (double *)cur;
  cur += ((size_t)numb * L * sizeof(double) + 255) / 256 * 256;
  int *dlv = (int *)cur;
  CK(cudaMemsetAsync(h->cursors, 0, 8 * sizeof(long), h->stream));
  CK(cudaMemsetAsync(dds, 0, (size_t)numb * L * sizeof(double), h->stream));
  ReplaySrc src{dg, ng, h->cursors + 0, du, n3, h->cursors + 1, nullptr, 0, h->cursors + 2, h->ctx.st.err};
  launch_bisect_replay(h->ctx, h->frames, type, time, exchange ? 1 : 0, src, dds, dlv, h->cnt, h->stream);
  h->launches++;
  CK(cudaGetLastError());
  long cz[8];
  CK(cudaMemcpyAsync(cz, h->cursors, 8 * sizeof(long), cudaMemcpyDeviceToHost, h->stream));
  if (ds_out) CK(cudaMemcpyAsync(ds_out, dds, (size_t)numb * L * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  if (lvl_out) CK(cudaMemcpyAsync(lvl_out, dlv, numb * sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  e = check_err(h);
  if (consumed) { consumed[0] = cz[0]; consumed[1] = cz[1]; }
  return e;
}

extern "C" pimc_status pimc_molecular_move(pimc_handle *h, int type, const double *u1, long n1, const double *u2,
                                           long n2, long *consumed, double *dv_out, int *acc_out)
{
  pimc_status e = ready(h);
  if (e) return e;
  const DevSys &d = h->ctx.s;
  if (type < 0 || type >= d.ntypes || n1 < 0 || n2 < 0 || (n1 && !u1) || (n2 && !u2)) return PIMC_ERR_BAD_ARG;
  int numb = d.numb[type];
  size_t bytes = ((size_t)n1 + n2 + 2 * (size_t)numb + 16) * sizeof(double) + 4096;
  void *buf;
  if ((e = scratch(h, bytes, &buf))) return e;
  char *cur = (char *)buf;
  double *d1, *d2;
  if ((e = put_stream(h, u1, n1, &d1, cur)) || (e = put_stream(h, u2, n2, &d2, cur))) return e;
  double *ddv = (double *)cur;
  cur += ((size_t)numb * sizeof(double) + 255) / 256 * 256;
  int *dacc = (int *)cur;
  CK(cudaMemsetAsync(h->cursors, 0, 8 * sizeof(long), h->stream));
  ReplaySrc src{nullptr, 0, h->cursors + 0, d2, n2, h->cursors + 1, d1, n1, h->cursors + 2, h->ctx.st.err};
  for (int a = 0; a < numb; a++) {
    launch_mol(h->ctx, h->frames, type, a, true, src, 0, h->pass, 0, h->ms, ddv, dacc, h->cnt, h->stream);
    h->launches += 3;
  }
  CK(cudaGetLastError());
  long cz[8];
  CK(cudaMemcpyAsync(cz, h->cursors, 8 * sizeof(long), cudaMemcpyDeviceToHost, h->stream));
  if (dv_out) CK(cudaMemcpyAsync(dv_out, ddv, numb * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  if (acc_out) CK(cudaMemcpyAsync(acc_out, dacc, numb * sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  e = check_err(h);
  if (consumed) { consumed[0] = cz[2]; consumed[1] = cz[1]; }
  return e;
}

extern "C" pimc_status pimc_rotations_move(pimc_handle *h, const double *urot, long nrot, double *rd_out, int *acc_out)
{
  pimc_status e = ready(h);
  if (e) return e;
  const DevSys &d = h->ctx.s;
  if (d.imtype < 0 || !h->sys.rotation || nrot < 0 || (nrot && !urot)) return PIMC_ERR_BAD_ARG;
  size_t nk = (size_t)d.Q * d.nrotors;
  size_t bytes = ((size_t)nrot + 2 * nk + 16) * sizeof(double) + 4096;
  void *buf;
  if ((e = scratch(h, bytes, &buf))) return e;
  char *cur = (char *)buf;
  double *du;
  if ((e = put_stream(h, urot, nrot, &du, cur))) return e;
  double *drd = (double *)cur;
  cur += (nk * sizeof(double) + 255) / 256 * 256;
  int *dacc = (int *)cur;
  launch_rot_replay(h->ctx, h->frames, 0, du, nrot, drd, dacc, h->cnt, h->stream);
  launch_rot_replay(h->ctx, h->frames, 1, du, nrot, drd, dacc, h->cnt, h->stream);
  launch_refresh_frames(h->ctx, h->frames, h->stream);
  h->launches += 3;
  CK(cudaGetLastError());
  if (rd_out) CK(cudaMemcpyAsync(rd_out, drd, nk * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  if (acc_out) CK(cudaMemcpyAsync(acc_out, dacc, nk * sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  return check_err(h);
}

// ------------------------------------------------------------ energies

extern "C" pimc_status pimc_pot_energy(pimc_handle *h, int n, const int *atom0, const int *it, const double *xyz,
                                       double *out)
{
  pimc_status e = ready(h);
  if (e) return e;
  const DevSys &d = h->ctx.s;
  if (n < 0 || (n && (!atom0 || !it || !xyz || !out))) return PIMC_ERR_BAD_ARG;
  for (int k = 0; k < n; k++)
    if (atom0[k] < 0 || atom0[k] >= d.na || it[k] < 0 || it[k] >= d.P) return PIMC_ERR_BAD_ARG;
  size_t bytes = (size_t)n * (2 * sizeof(int) + 4 * sizeof(double)) + 4096;
  void *buf;
  if ((e = scratch(h, bytes, &buf))) return e;
  char *cur = (char *)buf;
  int *da = (int *)cur; cur += ((size_t)n * sizeof(int) + 255) / 256 * 256;
  int *dt = (int *)cur; cur += ((size_t)n * sizeof(int) + 255) / 256 * 256;
  double *dx = (double *)cur; cur += ((size_t)3 * n * sizeof(double) + 255) / 256 * 256;
  double *dout = (double *)cur;
  CK(cudaMemcpyAsync(da, atom0, n * sizeof(int), cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(dt, it, n * sizeof(int), cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(dx, xyz, 3 * n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  launch_q_slice(h->ctx, h->frames, n, da, dt, dx, dout, h->stream);
  h->launches++;
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(out, dout, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  return check_err(h);
}

extern "C" pimc_status pimc_pot_rot_energy(pimc_handle *h, int n, const int *rotor, const int *it, const double *v3,
                                           double *out)
{
  pimc_status e = ready(h);
  if (e) return e;
  const DevSys &d = h->ctx.s;
  if (d.imtype < 0 || n < 0 || (n && (!rotor || !it || !v3 || !out))) return PIMC_ERR_BAD_ARG;
  for (int k = 0; k < n; k++)
    if (rotor[k] < d.rot_first || rotor[k] >= d.rot_first + d.nrotors || it[k] < 0 || it[k] >= d.P)
      return PIMC_ERR_BAD_ARG;
  size_t bytes = (size_t)n * (2 * sizeof(int) + 4 * sizeof(double)) + 4096;
  void *buf;
  if ((e = scratch(h, bytes, &buf))) return e;
  char *cur = (char *)buf;
  int *da = (int *)cur; cur += ((size_t)n * sizeof(int) + 255) / 256 * 256;
  int *dt = (int *)cur; cur += ((size_t)n * sizeof(int) + 255) / 256 * 256;
  double *dv = (double *)cur; cur += ((size_t)3 * n * sizeof(double) + 255) / 256 * 256;
  double *dout = (double *)cur;
  CK(cudaMemcpyAsync(da, rotor, n * sizeof(int), cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(dt, it, n * sizeof(int), cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(dv, v3, 3 * n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  launch_q_rot(h->ctx, h->frames, n, da, dt, dv, d.molecule[d.imtype] == PIMC_LINEAR, dout, h->stream);
  h->launches++;
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(out, dout, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  return check_err(h);
}

// ------------------------------------------------------------ estimators

extern "C" pimc_status pimc_estimators(pimc_handle *h, double *out)
{
  pimc_status e = ready(h);
  if (e) return e;
  if (!out) return PIMC_ERR_BAD_ARG;
  const DevSys &d = h->ctx.s;
  int npairs = d.na * (d.na - 1) / 2;
  size_t nk = (size_t)d.nrotors * d.Q;
  size_t nd = (size_t)d.na + npairs + 4 * nk + d.Q + 64;
  void *buf;
  if ((e = scratch(h, nd * sizeof(double) + 4096, &buf))) return e;
  double *kin = (double *)buf, *pot = kin + d.na, *rot = pot + npairs, *rcf = rot + 4 * nk;
  launch_est(h->ctx, h->frames, kin, pot, rot, rcf, h->stream);
  h->launches += nk ? 4 : 2;
  if (h->dens_on) h->launches += launch_est_dens(h->ctx, h->frames, h->dens, h->stream);
  CK(cudaGetLastError());
  std::vector<double> hv(nd);
  CK(cudaMemcpyAsync(hv.data(), buf, nd * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  if ((e = check_err(h))) return e;
  // GetKinEnergy: P*T*(0.5*3*N - sum_atoms r2 / (4 beta lambda)) (mc_estim.cc:923-934)
  double r2avr = 0.0;
  for (int a = 0; a < d.na; a++) r2avr += hv[a];
  out[0] = (double)d.P * d.temperature * (0.5 * (double)(3 * d.na) - r2avr);
  double spot = 0.0;
  for (int p = 0; p < npairs; p++) spot += hv[d.na + p];
  out[1] = spot / (double)d.P;
  double erot = 0.0, esq = 0.0, ets = 0.0;
  if (nk && h->sys.rotation) {
    const double *r = hv.data() + d.na + npairs;
    if (d.molecule[d.imtype] == PIMC_LINEAR) {          // GetRotEnergy mc_estim.cc:953-984
      for (int q = 0; q < d.Q; q++) { erot += r[4 * q]; esq += r[4 * q + 1]; ets += r[4 * q + 2]; }
      if (d.rot_den_type == 1) {
        erot = erot / (double)d.Q;
        erot = erot / d.rot_tau + 1.0 / d.rot_tau;
      }
    } else {                                              // GetRotE3D mc_estim.cc:1000-1092
      int skip = d.rot_den_type == 0 ? 1 : d.rn_ratio;
      double nq = (double)(d.Q / skip);
      for (int rr = 0; rr < d.nrotors; rr++) {
        double s = 0.0, q2 = 0.0, t2 = 0.0;
        for (int q = 0; q < d.Q; q++) {
          const double *v = r + 4 * ((size_t)rr * d.Q + q);
          s += v[0]; q2 += v[1]; t2 += v[2];
        }
        double er = s / nq;
        esq += q2 / (nq * nq);
        ets += t2 / (nq * nq);
        // the rattle-and-shake energy of this rotor alone; the reference
        // applies the conversion to the running sum of all rotors
        // (mc_estim.cc:1084-1090), which is the same for one rotor
        if (d.rot_den_type == 1 && d.rn_ratio == 1) {
          er = er / (4.0 * (d.rot_tau / PIMC_WNO2K) * (d.rot_tau / PIMC_WNO2K));
          er += 0.25 * (d.abc[0] + d.abc[1] + d.abc[2]) + 1.5 / (d.rot_tau / PIMC_WNO2K);
          er = er / PIMC_WNO2K;
        }
        erot += er;
      }
    }
  }
  out[2] = erot;
  out[3] = esq;
  out[4] = ets;
  return PIMC_OK;
}

// ------------------------------------------------ densities, cycles, areas

static const size_t kDens1 = (size_t)PIMC_MAX_TYPES * PIMC_BINSR;
static const size_t kDens2 = kDens1 * PIMC_BINST;
static const size_t kDens3 = kDens2 * PIMC_BINSC;
static const size_t kRel = PIMC_BINST + 2 * PIMC_BINSC;

static pimc_status dens_alloc(pimc_handle *h)
{
  if (h->dens.g1) return PIMC_OK;
  CK(cudaMalloc(&h->dens.g1, kDens1 * sizeof(unsigned long long)));
  CK(cudaMalloc(&h->dens.g2, kDens2 * sizeof(unsigned long long)));
  CK(cudaMemsetAsync(h->dens.g1, 0, kDens1 * sizeof(unsigned long long), h->stream));
  CK(cudaMemsetAsync(h->dens.g2, 0, kDens2 * sizeof(unsigned long long), h->stream));
  if (h->ctx.s.nrotors > 0 && h->ctx.s.molecule[h->ctx.s.imtype] == PIMC_NONLINEAR) {
    CK(cudaMalloc(&h->dens.g3, kDens3 * sizeof(unsigned long long)));
    CK(cudaMemsetAsync(h->dens.g3, 0, kDens3 * sizeof(unsigned long long), h->stream));
    CK(cudaMalloc(&h->dens.rel, kRel * sizeof(unsigned long long)));
    CK(cudaMemsetAsync(h->dens.rel, 0, kRel * sizeof(unsigned long long), h->stream));
  }
  return PIMC_OK;
}

extern "C" pimc_status pimc_densities_accumulate(pimc_handle *h)
{
  pimc_status e = ready(h);
  if (e) return e;
  if ((e = dens_alloc(h))) return e;
  h->launches += launch_est_dens(h->ctx, h->frames, h->dens, h->stream);
  CK(cudaGetLastError());
  return PIMC_OK;
}

extern "C" pimc_status pimc_densities_read(pimc_handle *h, double *gr1d, double *gr2d, double *gr3d)
{
  if (!h) return PIMC_ERR_BAD_ARG;
  CK(cudaSetDevice(h->device));
  double *dst[3] = {gr1d, gr2d, gr3d};
  unsigned long long *src[3] = {h->dens.g1, h->dens.g2, h->dens.g3};
  size_t n[3] = {kDens1, kDens2, kDens3};
  std::vector<unsigned long long> tmp;
  for (int k = 0; k < 3; k++) {
    if (!dst[k]) continue;
    if (!src[k]) {
      std::fill(dst[k], dst[k] + n[k], 0.0);
      continue;
    }
    tmp.resize(n[k]);
    CK(cudaMemcpyAsync(tmp.data(), src[k], n[k] * sizeof(unsigned long long), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    for (size_t i = 0; i < n[k]; i++) dst[k][i] = (double)tmp[i];
  }
  return check_err(h);
}

extern "C" pimc_status pimc_densities_reset(pimc_handle *h)
{
  if (!h) return PIMC_ERR_BAD_ARG;
  CK(cudaSetDevice(h->device));
  unsigned long long *src[3] = {h->dens.g1, h->dens.g2, h->dens.g3};
  size_t n[3] = {kDens1, kDens2, kDens3};
  for (int k = 0; k < 3; k++)
    if (src[k]) CK(cudaMemsetAsync(src[k], 0, n[k] * sizeof(unsigned long long), h->stream));
  if (h->dens.rel) CK(cudaMemsetAsync(h->dens.rel, 0, kRel * sizeof(unsigned long long), h->stream));
  return PIMC_OK;
}

extern "C" pimc_status pimc_rel_euler_read(pimc_handle *h, double *the, double *phi, double *chi)
{
  if (!h || !the || !phi || !chi) return PIMC_ERR_BAD_ARG;
  CK(cudaSetDevice(h->device));
  std::vector<unsigned long long> tmp(kRel, 0ull);
  if (h->dens.rel) {
    CK(cudaMemcpyAsync(tmp.data(), h->dens.rel, kRel * sizeof(unsigned long long), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
  }
  for (int i = 0; i < PIMC_BINST; i++) the[i] = (double)tmp[i];
  for (int i = 0; i < PIMC_BINSC; i++) phi[i] = (double)tmp[PIMC_BINST + i];
  for (int i = 0; i < PIMC_BINSC; i++) chi[i] = (double)tmp[PIMC_BINST + PIMC_BINSC + i];
  return check_err(h);
}

// BSTYPE: the last Bose type (mc_setup.cc:409-415), or -1
static int boson_type(const pimc_handle *h)
{
  int bt = -1;
  for (int t = 0; t < h->sys.ntypes; t++)
    if (h->sys.type[t].stat == PIMC_BOSE) bt = t;
  return bt;
}

extern "C" pimc_status pimc_exchange_lengths(pimc_handle *h, double *ploops)
{
  pimc_status e = ready(h);
  if (e) return e;
  if (!ploops) return PIMC_ERR_BAD_ARG;
  int bt = boson_type(h);
  if (bt < 0) return PIMC_ERR_STATE;
  int n = h->sys.type[bt].numb;
  std::vector<int> pidx(h->ctx.s.na);
  CK(cudaMemcpyAsync(pidx.data(), h->ctx.st.pindex, pidx.size() * sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  std::vector<char> seen(n, 0);
  for (int atom = 0; atom < n; atom++) {
    if (seen[atom]) continue;
    int len = 0, p = pidx[atom];
    while (p != atom) {
      if (p < 0 || p >= n || len > n) return PIMC_ERR_STATE;   // not a permutation
      seen[p] = 1;
      p = pidx[p];
      len++;
    }
    ploops[len] += 1.0;
  }
  return PIMC_OK;
}

static pimc_status area_sums(pimc_handle *h, int mode, int bt, const double *mass, double *sums)
{
  int nb = est_area_ctas(h->ctx, bt);
  void *buf;
  pimc_status e;
  if ((e = scratch(h, (size_t)nb * 12 * sizeof(double), &buf))) return e;
  launch_est_area(h->ctx, mode, bt, mass, (double *)buf, h->stream);
  h->launches += 1;
  CK(cudaGetLastError());
  std::vector<double> part((size_t)nb * 12);
  CK(cudaMemcpyAsync(part.data(), buf, part.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  if ((e = check_err(h))) return e;
  for (int k = 0; k < 12; k++) {
    double v = 0.0;
    for (int b = 0; b < nb; b++) v += part[(size_t)b * 12 + k];
    sums[k] = v;
  }
  return PIMC_OK;
}

extern "C" pimc_status pimc_area_estimators(pimc_handle *h, double *out)
{
  pimc_status e = ready(h);
  if (e) return e;
  if (!out) return PIMC_ERR_BAD_ARG;
  int bt = boson_type(h);
  const DevSys &d = h->ctx.s;
  if (bt < 0 || d.nrotors <= 0 || d.molecule[d.imtype] != PIMC_LINEAR) return PIMC_ERR_STATE;
  double v[12];
  if ((e = area_sums(h, 0, bt, nullptr, v))) return e;
  out[0] = v[0];
  out[1] = v[1];
  out[2] = v[0] * v[0];
  out[3] = v[1] * v[1];
  out[4] = v[2] / (double)d.P;
  out[5] = v[3] / (double)d.P;
  return PIMC_OK;
}

extern "C" pimc_status pimc_area_estim3d(pimc_handle *h, int iframe, const double *mass, double *out)
{
  pimc_status e = ready(h);
  if (e) return e;
  if (!out || !mass || (iframe != 0 && iframe != 1)) return PIMC_ERR_BAD_ARG;
  int bt = boson_type(h);
  const DevSys &d = h->ctx.s;
  if (bt < 0 || (iframe == 1 && d.nrotors <= 0)) return PIMC_ERR_STATE;
  double m[2] = {mass[0], d.ntypes > 1 ? mass[1] : mass[0]};
  double v[12];
  if ((e = area_sums(h, iframe == 0 ? 1 : 2, bt, m, v))) return e;
  for (int i = 0; i < 3; i++) out[i] = v[i];
  int ind = 3;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j <= i; j++) out[ind++] = v[i] * v[j];
  for (int k = 0; k < 9; k++) out[9 + k] = v[3 + k] / (double)d.P;
  return PIMC_OK;
}

// ------------------------------------------------------------ worm algorithm

extern "C" pimc_status pimc_worm_init(pimc_handle *h, int type, double c, int m, double density)
{
  if (!h) return PIMC_ERR_BAD_ARG;
  const DevSys &d = h->ctx.s;
  if (type < 0 || type >= d.ntypes || d.molecule[type] != PIMC_ATOM || m < 1 || m >= d.P) return PIMC_ERR_BAD_ARG;
  if (m > PIMC_WORM_MAXM) return PIMC_ERR_SIZE;
  CK(cudaSetDevice(h->device));
  pimc_status e;
  if (!h->worm) {
    if ((e = dalloc(h, &h->worm, 1)) || (e = dalloc(h, &h->rindex, d.na)) || (e = dalloc(h, &h->wcur, 16))) return e;
    CK(cudaMalloc(&h->wscr, worm_scratch_bytes(d.na) + 2 * (size_t)d.na * sizeof(int) + 512));
  }
  // MCWormInit (mc_qworm.cc:49-82): Worm.c scaled by the density per bead
  // and segment, the open-move normalisation and the neighbour cut-off
  DevWorm w{};
  int numb = d.numb[type];
  double cw = c * (density / (double)(numb * d.P * m));
  w.type = type;
  w.m = m;
  w.numb = numb;
  w.first = d.first[type];
  w.qw_norm = cw * numb * d.P * m;
  w.twave2 = 4.0 * d.lambda[type] * d.tau;                   // mc_setup.cc:394
  w.cut2 = 100.0 * 100.0 * ((double)m * 4.0 * d.lambda[type] * d.tau);
  CK(cudaMemcpy(h->worm, &w, sizeof(DevWorm), cudaMemcpyHostToDevice));
  std::vector<int> r(d.na);
  for (int a = 0; a < d.na; a++) r[h->pindex_host[a]] = a;
  CK(cudaMemcpy(h->rindex, r.data(), d.na * sizeof(int), cudaMemcpyHostToDevice));
  h->worm_on = 1;
  h->ctx.st.worm = h->worm;           // every partner sum now masks the worm's gap
  if (h->pass_exec || h->worm_exec) { // a captured pass holds the old context
    CK(cudaStreamSynchronize(h->stream));
    if (h->pass_exec) cudaGraphExecDestroy(h->pass_exec);
    if (h->worm_exec) cudaGraphExecDestroy(h->worm_exec);
    h->pass_exec = nullptr;
    h->worm_exec = nullptr;
  }
  return PIMC_OK;
}

extern "C" pimc_status pimc_worm_move(pimc_handle *h, const double *const *streams, const long *lengths,
                                      long *consumed)
{
  pimc_status e = ready(h);
  if (e) return e;
  if (!h->worm_on) return PIMC_ERR_STATE;
  if (!streams || !lengths) return PIMC_ERR_BAD_ARG;
  if (h->ctx.s.mixed) return PIMC_ERR_STATE;          // the worm moves run on the FP64 path
  size_t bytes = 4096;
  for (int k = 0; k < 9; k++) {
    if (lengths[k] < 0 || (lengths[k] && !streams[k])) return PIMC_ERR_BAD_ARG;
    bytes += ((size_t)(lengths[k] > 0 ? lengths[k] : 1) * sizeof(double) + 255) / 256 * 256;
  }
  int numb = h->ctx.s.numb[0];
  for (int t = 0; t < h->ctx.s.ntypes; t++) numb = std::max(numb, h->ctx.s.numb[t]);
  bytes += worm_scratch_bytes(numb) + 256;
  void *buf;
  if ((e = scratch(h, bytes, &buf))) return e;
  char *cur = (char *)buf;
  double *dv[9];
  for (int k = 0; k < 9; k++)
    if ((e = put_stream(h, streams[k], lengths[k], &dv[k], cur))) return e;
  CK(cudaMemsetAsync(h->wcur, 0, 16 * sizeof(long), h->stream));
  launch_worm_move(h->ctx, h->frames, h->worm, h->rindex, dv, lengths, h->wcur, cur, numb, h->stream);
  launch_invalidate_caches(h->ctx, h->stream);       // beads of the worm type moved
  h->launches += 2;
  CK(cudaGetLastError());
  long cz[16];
  CK(cudaMemcpyAsync(cz, h->wcur, 16 * sizeof(long), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaMemcpyAsync(h->pindex_host.data(), h->ctx.st.pindex, h->ctx.s.na * sizeof(int), cudaMemcpyDeviceToHost,
                     h->stream));
  e = check_err(h);
  if (consumed)
    for (int k = 0; k < 9; k++) consumed[k] = cz[k];
  return e;
}

// The worm branch of the pass loop (mc_main.cc:348-381) with counter-based
// draws: for every time slice, the worm type's MCWormMove and, while the worm
// is closed, its bisection at a drawn slice (exchange for bosons) and at
// slice 0 its exchange-cycle centroid move; the other types' PIMCPass
// (mc_main.cc:510-522).  Uniform keys: phase 4t for the worm tries, 4t+1
// the worm type's bisection, 4t+2 its centroid move, 4t+3 the other types'
// translational moves; the rotational draws (their own key domain) phases
// 2t and 2t+1 for the two half-sweeps at slice t.
static pimc_status upload_self_rep(pimc_handle *h);
static int self_flat_warps(int units);

extern "C" pimc_status pimc_worm_run(pimc_handle *h, int npasses, uint64_t seed)
{
  pimc_status e = ready(h);
  if (e) return e;
  if (!h->worm_on) return PIMC_ERR_STATE;
  if (npasses < 0) return PIMC_ERR_BAD_ARG;
  const DevSys &d = h->ctx.s;
  DevWorm w;
  CK(cudaMemcpyAsync(&w, h->worm, sizeof(DevWorm), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  const int wt = w.type, P = d.P;
  const int bose = d.stat[wt] == PIMC_BOSE;
  char *mscr = (char *)h->wscr + ((worm_scratch_bytes(d.na) + 255) / 256) * 256;
  ReplaySrc none{};
  const bool flat_worm = h->sys.rotation && d.nrotors > 0 && d.Q >= 4 && d.Q % 2 == 0;
  if (flat_worm) {
    if ((e = upload_self_rep(h))) return e;
    if (!batch_flat_setup(8)) return PIMC_ERR_CUDA;
  }
  // one pass, recorded into a CUDA graph on the first call for this seed
  auto record = [&]() -> long long {
    long long n = 0;
    launch_pass_begin(h->pass, h->stream);
    n++;
    for (int t = 0; t < P; t++) {
      for (int type = 0; type < d.ntypes; type++) {
        if (d.numb[type] <= 0) continue;
        if (type == wt) {
          launch_worm_prod(h->ctx, h->frames, h->worm, h->rindex, seed, h->pass, 4u * t, h->wscr, d.na, h->stream);
          launch_invalidate_caches(h->ctx, h->stream);
          n += 2;
          n += launch_bisect_slice(h->ctx, h->frames, type, 0, bose, h->worm, seed, h->pass, 4u * t + 1, h->cnt,
                                   h->stream);
          if (t == 0)
            n += launch_mol_exchange(h->ctx, h->frames, type, false, none, seed, h->pass, 4u * t + 2, mscr, h->cnt,
                                     h->stream, h->worm);
          continue;
        }
        if (t == 0)
          for (int a = 0; a < d.numb[type]; a++)
            n += launch_mol(h->ctx, h->frames, type, a, false, none, seed, h->pass, 4u * t + 3, h->ms, nullptr,
                            nullptr, h->cnt, h->stream);
        n += launch_bisect_slice(h->ctx, h->frames, type, t, 0, nullptr, seed, h->pass, 4u * t + 3, h->cnt,
                                 h->stream);
        if (type == d.imtype && h->sys.rotation) {
          // the two half-sweeps draw from their own phases (slices 2p and 2p+1
          // share the pair index p of the rotational draws' key); with an even
          // Q a warp per slice pair (the half-sweep kernel over this handle),
          // else a CTA per slice
          if (flat_worm)
            for (int parity = 0; parity < 2; parity++) {
              launch_batch_rot_flat(h->self_rep, h->self_idx, h->self_idx + 1, 1, d.Q / 2, 0, 0, parity, 1, seed,
                                    d.mixed, self_flat_warps(d.Q / 2), 2, h->stream, 2LL * t);
              n++;
            }
          else {
            n += launch_rot_phase(h->ctx, h->frames, 0, 2u * t, seed, h->pass, h->cnt, h->stream);
            n += launch_rot_phase(h->ctx, h->frames, 1, 2u * t + 1, seed, h->pass, h->cnt, h->stream);
          }
        }
      }
    }
    launch_refresh_frames(h->ctx, h->frames, h->stream);
    return n + 1;
  };
  if (npasses > 0 && (!h->worm_exec || h->worm_seed != seed)) {
    if (h->worm_exec) { CK(cudaGraphExecDestroy(h->worm_exec)); h->worm_exec = nullptr; }
    cudaGraph_t graph;
    CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    long long n = record();
    cudaError_t le = cudaGetLastError();
    cudaError_t ce = cudaStreamEndCapture(h->stream, &graph);
    if (le != cudaSuccess || ce != cudaSuccess) {
      if (ce == cudaSuccess) cudaGraphDestroy(graph);
      h->last_cuda = le != cudaSuccess ? le : ce;
      return PIMC_ERR_CUDA;
    }
    cudaError_t ie = cudaGraphInstantiate(&h->worm_exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ie != cudaSuccess) { h->last_cuda = ie; return PIMC_ERR_CUDA; }
    h->worm_seed = seed;
    h->worm_nodes = n;
  }
  for (int p = 0; p < npasses; p++) {
    CK(cudaGraphLaunch(h->worm_exec, h->stream));
    h->launches += h->worm_nodes;
  }
  CK(cudaMemcpyAsync(h->pindex_host.data(), h->ctx.st.pindex, d.na * sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  return check_err(h);
}

// ------------------------------------------------------- delayed acceptance

static pimc_status da_check(pimc_handle *h)
{
  const DevSys &d = h->ctx.s;
  if (d.nrotors != 2 || d.na != 2 || d.molecule[d.imtype] != PIMC_NONLINEAR || d.rot_den_type != 0 || d.Q % 2)
    return PIMC_ERR_STATE;     // the water dimer: two tops, no atoms, tabulated densities, even Q
  return PIMC_OK;
}

extern "C" pimc_status pimc_da_samples(pimc_handle *h, float *feat, float *energy)
{
  pimc_status e = ready(h);
  if (e) return e;
  if ((e = da_check(h))) return e;
  if (!feat || !energy) return PIMC_ERR_BAD_ARG;
  const int P = h->ctx.s.P;
  void *buf;
  if ((e = scratch(h, (size_t)P * 7 * sizeof(float) + 512, &buf))) return e;
  float *df = (float *)buf, *de = df + (size_t)P * 6;
  if (h->ctx.s.mixed) {              // the FP32 moves leave the double frames to be derived
    launch_refresh_frames(h->ctx, h->frames, h->stream);
    h->launches++;
  }
  h->launches += launch_da_samples(h->ctx, h->frames, df, de, h->stream);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(feat, df, (size_t)P * 6 * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaMemcpyAsync(energy, de, (size_t)P * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
  return check_err(h);
}

extern "C" pimc_status pimc_da_sweeps(pimc_handle *h, pimc_mlp *m, int nsweeps, uint64_t seed, float escale,
                                      int use_surrogate, double *stats)
{
  pimc_status e = ready(h);
  if (e) return e;
  if ((e = da_check(h))) return e;
  if (nsweeps < 0 || (use_surrogate && !m) || nsweeps > (1 << 18)) return PIMC_ERR_BAD_ARG;
  if (use_surrogate && mlp_poisoned(m)) return PIMC_ERR_TIMEOUT;    // reload its weights first
  const DevSys &d = h->ctx.s;
  const int nm = d.Q / 2, rows = nm * 2 * d.R;
  size_t bytes = (size_t)rows * 7 * sizeof(float) + (size_t)nm * sizeof(DaMove) + 4096;
  void *buf;
  if ((e = scratch(h, bytes, &buf))) return e;
  char *cur = (char *)buf;
  unsigned long long *st = (unsigned long long *)cur;
  cur += 256;
  float *feat = (float *)cur;
  cur += ((size_t)rows * 6 * sizeof(float) + 255) / 256 * 256;
  float *y = (float *)cur;
  cur += ((size_t)rows * sizeof(float) + 255) / 256 * 256;
  DaMove *mv = (DaMove *)cur;
  // the call's launches, recorded into a CUDA graph and replayed while the
  // same sweep count, seed, surrogate, scale and scratch come back
  auto record = [&]() -> long long {
    long long n = 1;
    launch_pass_begin(h->pass, h->stream);
    for (int sw = 0; sw < nsweeps; sw++)
      for (int par = 0; par < 2; par++)
        for (int r = 0; r < 2; r++) {
          unsigned phase = 4u * (unsigned)sw + 2u * par + r;
          n += launch_da_propose(h->ctx, h->frames, r, par, phase, seed, h->pass, feat, mv, h->stream);
          if (use_surrogate) n += mlp_forward_device(m, feat, rows, y, h->stream);
          n += launch_da_decide(h->ctx, h->frames, r, par, phase, seed, h->pass, y, use_surrogate, escale, mv, st,
                                h->cnt, h->stream);
        }
    launch_invalidate_caches(h->ctx, h->stream);
    launch_refresh_frames(h->ctx, h->frames, h->stream);
    return n + 2;
  };
  const unsigned long long mk = use_surrogate ? mlp_uid(m) : 0ull;
  if (!h->da_exec || h->da_nsweeps != nsweeps || h->da_seed != seed || h->da_use != use_surrogate ||
      h->da_escale != escale || h->da_mlp != mk || h->da_buf != buf) {
    if (h->da_exec) { CK(cudaGraphExecDestroy(h->da_exec)); h->da_exec = nullptr; }
    cudaGraph_t graph;
    CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    long long n = record();
    cudaError_t le = cudaGetLastError();
    cudaError_t ce = cudaStreamEndCapture(h->stream, &graph);
    if (le != cudaSuccess || ce != cudaSuccess) {
      if (ce == cudaSuccess) cudaGraphDestroy(graph);
      h->last_cuda = le != cudaSuccess ? le : ce;
      return PIMC_ERR_CUDA;
    }
    cudaError_t ie = cudaGraphInstantiate(&h->da_exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ie != cudaSuccess) { h->last_cuda = ie; return PIMC_ERR_CUDA; }
    h->da_nsweeps = nsweeps; h->da_seed = seed; h->da_use = use_surrogate; h->da_escale = escale;
    h->da_mlp = mk; h->da_buf = buf; h->da_nodes = n;
  }
  CK(cudaMemsetAsync(st, 0, 4 * sizeof(unsigned long long), h->stream));
  CK(cudaGraphLaunch(h->da_exec, h->stream));
  h->launches += h->da_nodes;
  unsigned long long hs[4];
  CK(cudaMemcpyAsync(hs, st, sizeof(hs), cudaMemcpyDeviceToHost, h->stream));
  e = check_err(h);
  if (!e && use_surrogate && mlp_take_error(m)) e = PIMC_ERR_TIMEOUT;
  if (stats)
    for (int k = 0; k < 4; k++) stats[k] = (double)hs[k];
  return e;
}

extern "C" pimc_status pimc_worm_state(pimc_handle *h, int *state)
{
  if (!h || !state) return PIMC_ERR_BAD_ARG;
  if (!h->worm_on) return PIMC_ERR_STATE;
  CK(cudaSetDevice(h->device));
  DevWorm w;
  CK(cudaMemcpyAsync(&w, h->worm, sizeof(DevWorm), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  state[0] = w.exists; state[1] = w.ira; state[2] = w.masha; state[3] = w.atom_i; state[4] = w.atom_m;
  return PIMC_OK;
}

extern "C" pimc_status pimc_worm_set_state(pimc_handle *h, const int *state)
{
  if (!h || !state) return PIMC_ERR_BAD_ARG;
  if (!h->worm_on) return PIMC_ERR_STATE;
  CK(cudaSetDevice(h->device));
  DevWorm w;
  CK(cudaMemcpyAsync(&w, h->worm, sizeof(DevWorm), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  int P = h->ctx.s.P;
  if (state[1] < 0 || state[1] >= P || state[2] < 0 || state[2] >= P || state[3] < 0 || state[3] >= w.numb ||
      state[4] < 0 || state[4] >= w.numb)
    return PIMC_ERR_BAD_ARG;
  w.exists = state[0] ? 1 : 0; w.ira = state[1]; w.masha = state[2]; w.atom_i = state[3]; w.atom_m = state[4];
  CK(cudaMemcpy(h->worm, &w, sizeof(DevWorm), cudaMemcpyHostToDevice));
  return PIMC_OK;
}

extern "C" pimc_status pimc_worm_counters(pimc_handle *h, double *total, double *accep)
{
  if (!h || !total || !accep) return PIMC_ERR_BAD_ARG;
  if (!h->worm_on) return PIMC_ERR_STATE;
  CK(cudaSetDevice(h->device));
  DevWorm w;
  CK(cudaMemcpyAsync(&w, h->worm, sizeof(DevWorm), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  for (int k = 0; k < 7; k++) { total[k] = w.qwtot[k]; accep[k] = w.qwacc[k]; }
  return PIMC_OK;
}

extern "C" pimc_status pimc_rcf(pimc_handle *h, double *rcf)
{
  pimc_status e = ready(h);
  if (e) return e;
  if (!rcf || h->ctx.s.nrotors == 0) return PIMC_ERR_BAD_ARG;
  const DevSys &d = h->ctx.s;
  int npairs = d.na * (d.na - 1) / 2;
  size_t nk = (size_t)d.nrotors * d.Q;
  size_t nd = (size_t)d.na + npairs + 4 * nk + d.Q + 64;
  void *buf;
  if ((e = scratch(h, nd * sizeof(double) + 4096, &buf))) return e;
  double *kin = (double *)buf, *pot = kin + d.na, *rot = pot + npairs, *rc = rot + 4 * nk;
  launch_est(h->ctx, h->frames, kin, pot, rot, rc, h->stream);
  h->launches += 4;
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(rcf, rc, d.Q * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  return check_err(h);
}

// ------------------------------------------------------------ production

// one pass of the independent-set schedule, recorded on h->stream
// The production pass (PIMCPass, mc_main.cc:510-522, as independent sets):
// the centroid move of every atom, then for each (type, s0 < 2^levels) one
// bisection block -- numb phases of windows [s0 + kM, s0 + (k+1)M] -- each
// followed by its share of the P rotational sweeps.  Uniform keys: phase
// index b of bisection phase (type, s0, j) in that order, B + 2 it + parity
// for sweep it, B + 2P + type for the centroid moves.
struct PassPlan {
  std::vector<int> type, s0;
  std::vector<unsigned> phase0;
  unsigned B = 0;
};

static PassPlan pass_plan(const DevSys &d)
{
  PassPlan pl;
  unsigned b = 0;
  for (int t = 0; t < d.ntypes; t++) {
    int M = 1 << d.levels[t];
    for (int s0 = 0; s0 < M; s0++) {
      pl.type.push_back(t);
      pl.s0.push_back(s0);
      pl.phase0.push_back(b);
      b += (unsigned)d.numb[t];
    }
  }
  pl.B = b;
  return pl;
}

static long long launch_bisection_block(pimc_handle *h, const PassPlan &pl, size_t i, uint64_t seed)
{
  const DevSys &d = h->ctx.s;
  int t = pl.type[i];
  if (h->fused) {
    launch_bisect_block(h->ctx, h->frames, t, pl.s0[i], pl.phase0[i], seed, h->pass, h->cnt, h->stream);
    return 1;
  }
  for (int j = 0; j < d.numb[t]; j++)
    launch_bisect_phase(h->ctx, h->frames, t, pl.s0[i], j, pl.phase0[i] + (unsigned)j, seed, h->pass, h->cnt,
                        h->stream);
  return d.numb[t];
}

// the handle's current context for the half-sweep kernel (the recorded
// graphs hold the device copy's address)
static pimc_status upload_self_rep(pimc_handle *h)
{
  h->self_host.c = h->ctx;
  h->self_host.frames = h->frames;
  h->self_host.pass = h->pass;
  h->self_host.cnt = h->cnt;
  h->self_host.seed_mix = 0;
  h->self_host.rotation = h->sys.rotation;
  CK(cudaMemcpyAsync(h->self_rep, &h->self_host, sizeof(BatchRep), cudaMemcpyHostToDevice, h->stream));
  return PIMC_OK;
}

// warps per CTA of the half-sweep kernel over this handle's Q/2 slice pairs:
// spread over the SMs
static int self_flat_warps(int units)
{
  int warps = units / 152;
  if (warps < 1) warps = 1;
  if (warps > 8) warps = 8;
  return warps;
}

// several rotors whose slice moves have few rotor-partner terms (at most a
// warp's worth, R (N - 1) <= 32, e.g. the water dimer): each half-sweep is
// one launch of the batch's half-sweep kernel over this handle, a warp per
// slice pair (its rotors one after the other), instead of a persistent CTA
// looping over slice pairs; the same moves, draws and arithmetic
static bool flat_sweeps(const pimc_handle *h)
{
  const DevSys &d = h->ctx.s;
  return h->fused && d.nrotors > 1 && d.Q >= 4 && d.Q % 2 == 0 && (d.na - 1) * d.R <= 32;
}

// rotational sweeps it0 .. it1-1; group numbers the persistent launches of a pass
static pimc_status launch_sweeps(pimc_handle *h, const PassPlan &pl, int it0, int it1, unsigned group, uint64_t seed,
                                 long long *n)
{
  const DevSys &d = h->ctx.s;
  if (!h->sys.rotation || d.nrotors <= 0 || it1 <= it0) return PIMC_OK;
  if (flat_sweeps(h)) {
    const int units = d.Q / 2, nbk = (int)pl.type.size();
    const int warps = self_flat_warps(units);
    for (int it = it0; it < it1; it++)
      for (int parity = 0; parity < 2; parity++) {
        launch_batch_rot_flat(h->self_rep, h->self_idx, h->self_idx + 1, 1, units, (int)group, it - it0, parity, nbk,
                              seed, d.mixed, warps, 2, h->stream);
        (*n)++;
      }
    return PIMC_OK;
  }
  int nctas = 0;
  if (h->fused && d.Q >= 2 && d.Q % 2 == 0) {
    if (d.nrotors == 1 && rot_slices_max_ctas(d.mixed) >= d.Q) {
      // one CTA per slice, next move prepared while the neighbours move
      CK(launch_rot_slices(h->ctx, h->frames, 2 * (it1 - it0), pl.B + 2u * (unsigned)it0, group, seed, h->pass,
                           h->prog, h->abort_word, h->cnt, h->stream));
      (*n)++;
      return PIMC_OK;
    }
    nctas = rot_sweeps_max_ctas(d.mixed);
    if (nctas > d.Q / 2) nctas = d.Q / 2;
  }
  if (nctas > 0) {
    CK(launch_rot_sweeps(h->ctx, h->frames, nctas, 2 * (it1 - it0), pl.B + 2u * (unsigned)it0, group, seed, h->pass,
                         h->prog, h->abort_word, h->cnt, h->stream));
    (*n)++;
    return PIMC_OK;
  }
  for (int it = it0; it < it1; it++) {
    *n += launch_rot_phase(h->ctx, h->frames, 0, pl.B + 2u * it, seed, h->pass, h->cnt, h->stream);
    *n += launch_rot_phase(h->ctx, h->frames, 1, pl.B + 2u * it + 1, seed, h->pass, h->cnt, h->stream);
  }
  return PIMC_OK;
}

static long long launch_centroid(pimc_handle *h, const PassPlan &pl, uint64_t seed)
{
  const DevSys &d = h->ctx.s;
  long long n = 0;
  unsigned mol_phase = pl.B + 2u * (unsigned)d.P;
  for (int t = 0; t < d.ntypes; t++)
    for (int a = 0; a < d.numb[t]; a++) {
      ReplaySrc none{};
      none.err = h->ctx.st.err;
      n += launch_mol(h->ctx, h->frames, t, a, false, none, seed, h->pass, mol_phase + (unsigned)t, h->ms, nullptr,
                      nullptr, h->cnt, h->stream);
    }
  return n;
}

static pimc_status record_pass(pimc_handle *h, uint64_t seed, long long *nout)
{
  const DevSys &d = h->ctx.s;
  PassPlan pl = pass_plan(d);
  long long n = 0;
  pimc_status e;
  launch_pass_begin(h->pass, h->stream);
  n++;
  n += launch_centroid(h, pl, seed);          // centroid moves at time 0 (mc_main.cc:512-513)
  size_t nbk = pl.type.size();
  for (size_t i = 0; i < nbk; i++) {
    n += launch_bisection_block(h, pl, i, seed);
    int it0 = (int)((long long)i * d.P / (long long)nbk), it1 = (int)((long long)(i + 1) * d.P / (long long)nbk);
    if ((e = launch_sweeps(h, pl, it0, it1, (unsigned)i, seed, &n))) return e;
  }
  *nout = n;
  return PIMC_OK;
}

extern "C" pimc_status pimc_run_passes(pimc_handle *h, int npasses, uint64_t seed)
{
  pimc_status e = ready(h);
  if (e) return e;
  const DevSys &d = h->ctx.s;
  if (npasses < 0) return PIMC_ERR_BAD_ARG;
  for (int t = 0; t < d.ntypes; t++)
    if (d.P % (1 << d.levels[t])) return PIMC_ERR_BAD_ARG;
  if (flat_sweeps(h) && (e = upload_self_rep(h))) return e;
  if (!h->pass_exec || h->pass_seed != seed) {
    if (h->pass_exec) { CK(cudaGraphExecDestroy(h->pass_exec)); h->pass_exec = nullptr; }
    if (flat_sweeps(h) && !batch_flat_setup(8)) return PIMC_ERR_CUDA;
    cudaGraph_t graph;
    CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    long long n = 0;
    pimc_status re = record_pass(h, seed, &n);
    cudaError_t le = cudaGetLastError();
    cudaError_t ce = cudaStreamEndCapture(h->stream, &graph);
    if (re != PIMC_OK || le != cudaSuccess || ce != cudaSuccess) {
      if (ce == cudaSuccess) cudaGraphDestroy(graph);
      if (re != PIMC_OK) return re;
      h->last_cuda = le != cudaSuccess ? le : ce;
      return PIMC_ERR_CUDA;
    }
    cudaError_t ie = cudaGraphInstantiate(&h->pass_exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ie != cudaSuccess) { h->last_cuda = ie; return PIMC_ERR_CUDA; }
    h->pass_seed = seed;
    h->nodes_per_pass = n;
  }
  for (int p = 0; p < npasses; p++) {
    CK(cudaGraphLaunch(h->pass_exec, h->stream));
    h->launches += h->nodes_per_pass;
  }
  if (npasses > 0 && h->sys.rotation && d.nrotors > 0) {
    launch_refresh_frames(h->ctx, h->frames, h->stream);
    h->launches++;
    CK(cudaGetLastError());
  }
  return PIMC_OK;
}

extern "C" pimc_status pimc_profile_pass(pimc_handle *h, uint64_t seed, double *ms, long long *launches)
{
  pimc_status e = ready(h);
  if (e) return e;
  if (!ms || !launches) return PIMC_ERR_BAD_ARG;
  const DevSys &d = h->ctx.s;
  for (int t = 0; t < d.ntypes; t++)
    if (d.P % (1 << d.levels[t])) return PIMC_ERR_BAD_ARG;
  cudaEvent_t ev[6];
  for (int k = 0; k < 6; k++) CK(cudaEventCreate(&ev[k]));
  long long n[3] = {0, 0, 0};
  PassPlan pl = pass_plan(d);
  size_t nbk = pl.type.size();
  launch_pass_begin(h->pass, h->stream);
  CK(cudaEventRecord(ev[0], h->stream));
  n[0] = launch_centroid(h, pl, seed);
  CK(cudaEventRecord(ev[1], h->stream));
  CK(cudaEventRecord(ev[2], h->stream));
  for (size_t i = 0; i < nbk; i++) n[1] += launch_bisection_block(h, pl, i, seed);
  CK(cudaEventRecord(ev[3], h->stream));
  CK(cudaEventRecord(ev[4], h->stream));
  pimc_status e2;
  for (size_t i = 0; i < nbk; i++) {
    int it0 = (int)((long long)i * d.P / (long long)nbk), it1 = (int)((long long)(i + 1) * d.P / (long long)nbk);
    if ((e2 = launch_sweeps(h, pl, it0, it1, (unsigned)i, seed, &n[2]))) return e2;
  }
  CK(cudaEventRecord(ev[5], h->stream));
  if (h->sys.rotation && d.nrotors > 0) {
    launch_refresh_frames(h->ctx, h->frames, h->stream);
    n[2]++;
  }
  CK(cudaGetLastError());
  CK(cudaEventSynchronize(ev[5]));
  for (int k = 0; k < 3; k++) {
    float f = 0.f;
    CK(cudaEventElapsedTime(&f, ev[2 * k], ev[2 * k + 1]));
    ms[k] = f;
    launches[k] = n[k];
  }
  for (int k = 0; k < 6; k++) cudaEventDestroy(ev[k]);
  h->launches += 1 + n[0] + n[1] + n[2];
  return check_err(h);
}

extern "C" pimc_status pimc_set_option(pimc_handle *h, int option, long long value)
{
  if (!h) return PIMC_ERR_BAD_ARG;
  if (option == PIMC_OPT_FUSED) {
    if (value != 0 && value != 1) return PIMC_ERR_BAD_ARG;
    if (h->fused != (int)value && h->pass_exec) {
      CK(cudaSetDevice(h->device));
      CK(cudaStreamSynchronize(h->stream));
      cudaGraphExecDestroy(h->pass_exec);
      h->pass_exec = nullptr;
    }
    h->fused = (int)value;
    return PIMC_OK;
  }
  if (option == PIMC_OPT_DENSITIES) {
    if (value != 0 && value != 1) return PIMC_ERR_BAD_ARG;
    CK(cudaSetDevice(h->device));
    if (value) {
      pimc_status e = dens_alloc(h);
      if (e) return e;
    }
    h->dens_on = (int)value;
    return PIMC_OK;
  }
  if (option == PIMC_OPT_WAIT_NS) {
    if (value < 0 || value > 60000000000ll) return PIMC_ERR_BAD_ARG;
    CK(cudaSetDevice(h->device));
    CK(cudaStreamSynchronize(h->stream));
    h->ctx.s.wait_ns = (unsigned long long)value;
    // the captured graphs hold the system by value
    if (h->pass_exec) { cudaGraphExecDestroy(h->pass_exec); h->pass_exec = nullptr; }
    if (h->worm_exec) { cudaGraphExecDestroy(h->worm_exec); h->worm_exec = nullptr; }
    if (h->da_exec) { cudaGraphExecDestroy(h->da_exec); h->da_exec = nullptr; }
    return PIMC_OK;
  }
  return PIMC_ERR_BAD_ARG;
}

extern "C" pimc_status pimc_synchronize(pimc_handle *h)
{
  if (!h) return PIMC_ERR_BAD_ARG;
  CK(cudaSetDevice(h->device));
  return check_err(h);
}

extern "C" pimc_status pimc_counters(pimc_handle *h, double *total, double *accep)
{
  if (!h || !total || !accep) return PIMC_ERR_BAD_ARG;
  CK(cudaSetDevice(h->device));
  unsigned long long c[12];
  CK(cudaMemcpyAsync(c, h->cnt, sizeof(c), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  for (int i = 0; i < 6; i++) { total[i] = (double)c[2 * i]; accep[i] = (double)c[2 * i + 1]; }
  return PIMC_OK;
}

extern "C" pimc_status pimc_reset_counters(pimc_handle *h)
{
  if (!h) return PIMC_ERR_BAD_ARG;
  CK(cudaSetDevice(h->device));
  CK(cudaMemsetAsync(h->cnt, 0, 12 * sizeof(unsigned long long), h->stream));
  return PIMC_OK;
}

extern "C" pimc_status pimc_set_precision(pimc_handle *h, int mixed)
{
  if (!h || mixed < 0 || mixed > 1) return PIMC_ERR_BAD_ARG;
  CK(cudaSetDevice(h->device));
  h->ctx.s.mixed = mixed;
  // float copies as the moves of this precision write them; caches stale
  launch_derive_state(h->ctx, h->frames, h->stream);
  h->launches++;
  CK(cudaGetLastError());
  if (h->pass_exec) { CK(cudaGraphExecDestroy(h->pass_exec)); h->pass_exec = nullptr; }
  if (h->worm_exec) { CK(cudaGraphExecDestroy(h->worm_exec)); h->worm_exec = nullptr; }
  if (h->da_exec) { CK(cudaGraphExecDestroy(h->da_exec)); h->da_exec = nullptr; }
  return PIMC_OK;
}

extern "C" pimc_status pimc_type_info(const pimc_handle *h, int type, int *numb, int *levels)
{
  if (!h || !numb || !levels || type < 0 || type >= h->ctx.s.ntypes) return PIMC_ERR_BAD_ARG;
  *numb = h->ctx.s.numb[type];
  *levels = h->ctx.s.levels[type];
  return PIMC_OK;
}

extern "C" double pimc_bead_moves_per_pass(const pimc_handle *h)
{
  if (!h) return 0.0;
  const DevSys &d = h->ctx.s;
  double bm = 0.0;
  for (int t = 0; t < d.ntypes; t++) {
    bm += (double)d.numb[t] * d.P * ((1 << d.levels[t]) - 1) + (double)d.numb[t] * d.P;
    if (t == d.imtype && h->sys.rotation) bm += (double)d.numb[t] * d.P * d.Q;
  }
  return bm;
}

extern "C" long long pimc_launch_count(const pimc_handle *h) { return h ? h->launches : 0; }

extern "C" void *pimc_stream(const pimc_handle *h) { return h ? (void *)h->stream : nullptr; }

// ------------------------------------------------------------ allocation-free queries
//
// pimc_pot_energy_noalloc: the PotEnergy query of pimc_pot_energy for callers
// that must not have device memory allocated on their behalf once their set-up
// is done -- for example an application that reserves the device memory up
// front for its own pool allocator, or runs under a fixed device-memory budget,
// where a cudaMalloc at query time can fail (and would also synchronise the
// device).  pimc_pot_energy stages its queries in the handle's scratch buffer,
// which grows with cudaMalloc; this variant stages them in the fixed array
// below instead and calls no cudaMalloc, cudaFree or other allocating routine.
//
// The array holds at most PIMC_NOALLOC_MAX_QUERIES queries; every GPU that
// loads the library holds it (160 KiB) until the process exits.  All calls,
// from every handle on a device, share it and it keeps the last call's
// contents; nothing in it needs to start at zero because each call writes
// every entry it later reads.  Calls that overlap on the GPU (two streams,
// two host threads, two handles on one device) race on the array: callers
// must order them.  Host code cannot use the array's name as an address, so
// the first call on each device, with that device current, looks the address
// up with cudaGetSymbolAddress; make that first call before any stream capture.
#define PIMC_NOALLOC_MAX_QUERIES 4096
#define PIMC_NOALLOC_BYTES (PIMC_NOALLOC_MAX_QUERIES * (4 * sizeof(double) + 2 * sizeof(int)))

static __device__ __align__(256) unsigned char g_noalloc_scratch[PIMC_NOALLOC_BYTES];

#include <mutex>
static std::mutex g_noalloc_mu;
static void *g_noalloc_ptr[256];     // per device: the array's device address

static pimc_status noalloc_scratch(pimc_handle *h, unsigned char **p)
{
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (h->device < 0 || h->device >= 256) return PIMC_ERR_BAD_ARG;
  if (!g_noalloc_ptr[h->device]) {
    void *ptr = nullptr;
    CK(cudaSetDevice(h->device));
    CK(cudaGetSymbolAddress(&ptr, g_noalloc_scratch));
    g_noalloc_ptr[h->device] = ptr;
  }
  *p = (unsigned char *)g_noalloc_ptr[h->device];
  return PIMC_OK;
}

extern "C" pimc_status pimc_pot_energy_noalloc(pimc_handle *h, int n, const int *atom0, const int *it,
                                               const double *xyz, double *out)
{
  pimc_status e = ready(h);
  if (e) return e;
  const DevSys &d = h->ctx.s;
  if (n < 0 || (n && (!atom0 || !it || !xyz || !out))) return PIMC_ERR_BAD_ARG;
  if (n > PIMC_NOALLOC_MAX_QUERIES) return PIMC_ERR_SIZE;
  for (int k = 0; k < n; k++)
    if (atom0[k] < 0 || atom0[k] >= d.na || it[k] < 0 || it[k] >= d.P) return PIMC_ERR_BAD_ARG;
  if (n == 0) return PIMC_OK;
  unsigned char *base = nullptr;
  if ((e = noalloc_scratch(h, &base))) return e;
  double *dx = (double *)base;                                    // 3 * MAX doubles
  double *dout = dx + 3 * PIMC_NOALLOC_MAX_QUERIES;               // MAX doubles
  int *da = (int *)(dout + PIMC_NOALLOC_MAX_QUERIES);             // MAX ints
  int *dt = da + PIMC_NOALLOC_MAX_QUERIES;                        // MAX ints
  CK(cudaMemcpyAsync(da, atom0, n * sizeof(int), cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(dt, it, n * sizeof(int), cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(dx, xyz, 3 * (size_t)n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  launch_q_slice(h->ctx, h->frames, n, da, dt, dx, dout, h->stream);
  h->launches++;
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(out, dout, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  return check_err(h);
}

// ------------------------------------------------------------ replica batches
// A batch owns one base handle (device, stream, the shared potential tables
// and every buffer, freed with it) and pools of per-replica state carved
// into one BatchRep per replica.
struct pimc_batch {
  pimc_handle *base = nullptr;
  int n = 0;
  std::vector<pimc_system> sys;
  std::vector<BatchRep> reps;
  std::vector<int> state_set;
  BatchRep *d_reps = nullptr;
  int *d_order = nullptr;
  unsigned *d_work = nullptr;
  double *d_est = nullptr;
  unsigned long long *d_cnt = nullptr;
  unsigned *d_pass = nullptr;
  int warps = 8, minb = 2;
  int mixed = 0;
  // rotational half-sweeps: 0 inside the persistent pass, 1 one launch per
  // half-sweep over all replicas (per block: replicas ordered by sweeps,
  // prefix sums of their slice pairs, nbk x (n + 1) each on the device)
  int rot_mode = 0, exec_rot_mode = -1, exec_flat_minb = 0;
  long long exec_nodes = 2;
  int *d_flat_sorted = nullptr, *d_flat_pre = nullptr;
  std::vector<int> flat_nact_max;                  // per block: sweeps of its busiest replica
  std::vector<std::vector<int>> flat_act, flat_units;   // per block and sweep: active replicas, warps
  bool tables = false;
  cudaGraphExec_t exec = nullptr;
  uint64_t exec_seed = 0;
  int exec_warps = 0, exec_minb = 0, exec_mixed = -1;
  double bm_pass = 0.0;
  // the captured delayed-acceptance call and what it was captured for
  cudaGraphExec_t da_exec = nullptr;
  int da_count = 0, da_use = -1, da_shape = 0, da_mixed = -1;
  uint64_t da_seed = 0;
  float da_escale = 0.0f;
  unsigned long long da_mlp = 0;
  void *da_buf = nullptr;
  long long da_nodes = 0;
};

#define BK(x)                                                  \
  do {                                                         \
    cudaError_t e_ = (x);                                      \
    if (e_ != cudaSuccess) {                                   \
      b->base->last_cuda = e_;                                 \
      return PIMC_ERR_CUDA;                                    \
    }                                                          \
  } while (0)

extern "C" uint64_t pimc_batch_replica_seed(uint64_t seed, int r)
{
  return seed ^ (0x9E3779B97F4A7C15ull * (uint64_t)(r + 1));
}

template <class T>
static pimc_status pool(pimc_handle *h, T **p, size_t n)
{
  pimc_status e = dalloc(h, p, n > 0 ? n : 1);
  if (e) return e;
  h->owned.push_back(*p);
  CK(cudaMemset(*p, 0, (n > 0 ? n : 1) * sizeof(T)));
  return PIMC_OK;
}

static double system_bead_moves(const DevSys &d, bool rotation)
{
  double bm = 0.0;
  for (int t = 0; t < d.ntypes; t++) bm += (double)d.numb[t] * d.P * ((1 << d.levels[t]) - 1) + (double)d.numb[t] * d.P;
  if (rotation) bm += (double)d.P * d.Q * d.nrotors;
  return bm;
}

extern "C" pimc_status pimc_batch_create(int n, const pimc_system *systems, int device, pimc_batch **out)
{
  if (n < 1 || !systems || !out) return PIMC_ERR_BAD_ARG;
  *out = nullptr;
  const pimc_system &s0 = systems[0];
  std::vector<DevSys> ds(n);
  pimc_system smax = s0;
  for (int r = 0; r < n; r++) {
    const pimc_system &s = systems[r];
    pimc_status e = build_devsys(s, ds[r]);
    if (e) return e;
    if (s.ntypes != s0.ntypes || s.rotation != s0.rotation || s.rot_den_type != s0.rot_den_type ||
        s.ispher != s0.ispher || s.minimage != s0.minimage)
      return PIMC_ERR_BAD_ARG;
    for (int t = 0; t < s.ntypes; t++) {
      const pimc_type &a = s.type[t], &c = s0.type[t];
      if (a.molecule != c.molecule || a.stat != c.stat || a.levels != c.levels || a.lambda != c.lambda ||
          a.mcstep != c.mcstep)
        return PIMC_ERR_BAD_ARG;
      if (a.levels > 4) return PIMC_ERR_SIZE;                     // PIMC_BATCH_MAX_SEG
      if (s.nslices % (1 << a.levels)) return PIMC_ERR_BAD_ARG;   // bisection blocks tile the ring
      if (a.numb > smax.type[t].numb) smax.type[t].numb = a.numb;
    }
    if (ds[r].R > 16) return PIMC_ERR_SIZE;
  }
  pimc_handle *base = nullptr;
  pimc_status e = pimc_create(&smax, device, &base);
  if (e) return e;
  pimc_batch *b = new (std::nothrow) pimc_batch();
  if (!b) { pimc_destroy(base); return PIMC_ERR_SIZE; }
  b->base = base;
  b->n = n;
  b->sys.assign(systems, systems + n);
  b->reps.resize(n);
  b->state_set.assign(n, 0);
  pimc_handle *h = base;
  // pool sizes
  size_t nb = 0, nq = 0, na = 0;
  std::vector<size_t> ob(n), oq(n), oa(n);
  for (int r = 0; r < n; r++) {
    const DevSys &d = ds[r];
    ob[r] = nb; oq[r] = nq; oa[r] = na;
    nb += (size_t)d.P * d.nap;
    nq += (size_t)(d.nrotors > 0 ? d.nrotors : 1) * d.Q;
    na += (size_t)d.na;
  }
  double *x, *y, *z, *ang, *cosv, *rpc, *rlc;
  float4 *b4;
  float *cosvf;
  int *rpo, *rlo, *pidx, *mct;
  Frame *frames;
  if ((e = pool(h, &x, nb)) || (e = pool(h, &y, nb)) || (e = pool(h, &z, nb)) || (e = pool(h, &b4, nb)) ||
      (e = pool(h, &ang, 3 * nq)) || (e = pool(h, &cosv, 3 * nq)) || (e = pool(h, &cosvf, 3 * nq)) ||
      (e = pool(h, &rpc, nq)) || (e = pool(h, &rlc, nq)) || (e = pool(h, &rpo, nq)) || (e = pool(h, &rlo, nq)) ||
      (e = pool(h, &pidx, na)) || (e = pool(h, &mct, na)) || (e = pool(h, &frames, nq)) ||
      (e = pool(h, &b->d_pass, (size_t)n)) || (e = pool(h, &b->d_cnt, (size_t)n * 12)) ||
      (e = pool(h, &b->d_reps, (size_t)n)) || (e = pool(h, &b->d_order, (size_t)n)) ||
      (e = pool(h, &b->d_work, 1)) || (e = pool(h, &b->d_est, (size_t)n * 6))) {
    pimc_batch_destroy(b);
    return e;
  }
  std::vector<int> hp(na), hm(na);
  std::vector<std::pair<double, int>> work(n);
  for (int r = 0; r < n; r++) {
    const DevSys &d = ds[r];
    BatchRep &rp = b->reps[r];
    memset(&rp, 0, sizeof(rp));
    rp.c.s = d;
    DevState &st = rp.c.st;
    st.x = x + ob[r]; st.y = y + ob[r]; st.z = z + ob[r]; st.b4 = b4 + ob[r];
    st.ang = ang + 3 * oq[r]; st.cosv = cosv + 3 * oq[r]; st.cosvf = cosvf + 3 * oq[r];
    st.rp_cache = rpc + oq[r]; st.rl_cache = rlc + oq[r]; st.rp_ok = rpo + oq[r]; st.rl_ok = rlo + oq[r];
    st.pindex = pidx + oa[r]; st.mctype = mct + oa[r];
    st.err = base->ctx.st.err;
    rp.frames = frames + oq[r];
    rp.pass = b->d_pass + r;
    rp.cnt = b->d_cnt + 12 * (size_t)r;
    rp.seed_mix = 0x9E3779B97F4A7C15ull * (uint64_t)(r + 1);
    rp.rotation = systems[r].rotation;
    int g = 0;
    for (int t = 0; t < d.ntypes; t++)
      for (int a = 0; a < d.numb[t]; a++) { hm[oa[r] + g] = t; hp[oa[r] + g] = g; g++; }
    double bm = system_bead_moves(d, systems[r].rotation);
    b->bm_pass += bm;
    work[r] = {bm * (double)d.na, r};
  }
  CK(cudaMemcpy(pidx, hp.data(), na * sizeof(int), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(mct, hm.data(), na * sizeof(int), cudaMemcpyHostToDevice));
  // the largest replicas first: the work queue ends with the short ones
  std::sort(work.begin(), work.end(), [](const std::pair<double, int> &a, const std::pair<double, int> &c) {
    return a.first > c.first || (a.first == c.first && a.second < c.second);
  });
  std::vector<int> order(n);
  for (int k = 0; k < n; k++) order[k] = work[k].second;
  CK(cudaMemcpy(b->d_order, order.data(), n * sizeof(int), cudaMemcpyHostToDevice));
  *out = b;
  return PIMC_OK;
}

extern "C" pimc_status pimc_batch_destroy(pimc_batch *b)
{
  if (!b) return PIMC_ERR_BAD_ARG;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->da_exec) cudaGraphExecDestroy(b->da_exec);
  if (b->base) pimc_destroy(b->base);
  delete b;
  return PIMC_OK;
}

static pimc_status batch_upload_reps(pimc_batch *b)
{
  pimc_handle *h = b->base;
  CK(cudaMemcpy(b->d_reps, b->reps.data(), b->reps.size() * sizeof(BatchRep), cudaMemcpyHostToDevice));
  return PIMC_OK;
}

extern "C" pimc_status pimc_batch_load_tables(pimc_batch *b, const pimc_tables *tables)
{
  if (!b || !tables) return PIMC_ERR_BAD_ARG;
  pimc_handle *h = b->base;
  CK(cudaSetDevice(h->device));
  pimc_status e = load_tables_into(h, &tables[0], h->ctx.t, h->ctx.s, TAB_POT);
  if (e) return e;
  for (int r = 0; r < b->n; r++) {
    DevTables t = h->ctx.t;
    if ((e = load_tables_into(h, &tables[r], t, b->reps[r].c.s, TAB_ROT))) return e;
    b->reps[r].c.t = t;
  }
  if ((e = batch_upload_reps(b))) return e;
  CK(cudaStreamSynchronize(h->stream));
  b->tables = true;
  if (b->exec) { cudaGraphExecDestroy(b->exec); b->exec = nullptr; }
  return PIMC_OK;
}

extern "C" pimc_status pimc_batch_set_state(pimc_batch *b, int r, const double *coords, const double *angles,
                                            const int *pindex)
{
  if (!b || r < 0 || r >= b->n || !coords || !angles) return PIMC_ERR_BAD_ARG;
  pimc_handle *h = b->base;
  CK(cudaSetDevice(h->device));
  const Ctx &c = b->reps[r].c;
  const DevSys &d = c.s;
  if (pindex && !perm_ok(d, pindex)) return PIMC_ERR_BAD_ARG;
  size_t nbr = (size_t)d.na * d.P;
  std::vector<double> buf((size_t)d.P * d.nap, 0.0);
  double *dst[3] = {c.st.x, c.st.y, c.st.z};
  for (int k = 0; k < 3; k++) {
    for (int a = 0; a < d.na; a++)
      for (int t = 0; t < d.P; t++) buf[(size_t)t * d.nap + a] = coords[k * nbr + (size_t)a * d.P + t];
    CK(cudaMemcpy(dst[k], buf.data(), buf.size() * sizeof(double), cudaMemcpyHostToDevice));
  }
  if (d.nrotors > 0) {
    size_t n = (size_t)d.nrotors * d.Q;
    std::vector<double> av(3 * n), cs(3 * n);
    for (int rr = 0; rr < d.nrotors; rr++)
      for (int q = 0; q < d.Q; q++) {
        size_t src = (size_t)(d.rot_first + rr) * d.P + q;
        double phi = angles[src], cost = angles[nbr + src];
        double sint = sqrt(1.0 - cost * cost);                       // mc_main.cc:193-199
        for (int k = 0; k < 3; k++) av[k * n + rr * d.Q + q] = angles[k * nbr + src];
        cs[0 * n + rr * d.Q + q] = sint * cos(phi);
        cs[1 * n + rr * d.Q + q] = sint * sin(phi);
        cs[2 * n + rr * d.Q + q] = cost;
      }
    CK(cudaMemcpy(c.st.ang, av.data(), 3 * n * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c.st.cosv, cs.data(), 3 * n * sizeof(double), cudaMemcpyHostToDevice));
  }
  if (pindex) {
    CK(cudaMemcpy(c.st.pindex, pindex, d.na * sizeof(int), cudaMemcpyHostToDevice));
  }
  launch_derive_state(c, b->reps[r].frames, h->stream);       // float copies, frames, caches stale
  h->launches++;
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(h->stream));
  b->state_set[r] = 1;
  return PIMC_OK;
}

extern "C" pimc_status pimc_batch_get_state(pimc_batch *b, int r, double *coords, double *angles, double *cosine,
                                            int *pindex)
{
  if (!b || r < 0 || r >= b->n) return PIMC_ERR_BAD_ARG;
  pimc_handle *h = b->base;
  CK(cudaSetDevice(h->device));
  CK(cudaStreamSynchronize(h->stream));
  const Ctx &c = b->reps[r].c;
  const DevSys &d = c.s;
  size_t nbr = (size_t)d.na * d.P;
  if (coords) {
    std::vector<double> buf((size_t)d.P * d.nap);
    double *src[3] = {c.st.x, c.st.y, c.st.z};
    for (int k = 0; k < 3; k++) {
      CK(cudaMemcpy(buf.data(), src[k], buf.size() * sizeof(double), cudaMemcpyDeviceToHost));
      for (int a = 0; a < d.na; a++)
        for (int t = 0; t < d.P; t++) coords[k * nbr + (size_t)a * d.P + t] = buf[(size_t)t * d.nap + a];
    }
  }
  if (angles || cosine) {
    // rows of the rotors; the other rows are returned as zeros
    if (angles) memset(angles, 0, 3 * nbr * sizeof(double));
    if (cosine) memset(cosine, 0, 3 * nbr * sizeof(double));
    if (d.nrotors > 0) {
      size_t n = (size_t)d.nrotors * d.Q;
      std::vector<double> av(3 * n), cs(3 * n);
      CK(cudaMemcpy(av.data(), c.st.ang, 3 * n * sizeof(double), cudaMemcpyDeviceToHost));
      CK(cudaMemcpy(cs.data(), c.st.cosv, 3 * n * sizeof(double), cudaMemcpyDeviceToHost));
      for (int k = 0; k < 3; k++)
        for (int rr = 0; rr < d.nrotors; rr++)
          for (int q = 0; q < d.Q; q++) {
            size_t dst = k * nbr + (size_t)(d.rot_first + rr) * d.P + q;
            if (angles) angles[dst] = av[k * n + rr * d.Q + q];
            if (cosine) cosine[dst] = cs[k * n + rr * d.Q + q];
          }
    }
  }
  if (pindex) CK(cudaMemcpy(pindex, c.st.pindex, d.na * sizeof(int), cudaMemcpyDeviceToHost));
  return PIMC_OK;
}

extern "C" pimc_status pimc_batch_set_precision(pimc_batch *b, int mixed)
{
  if (!b || (mixed != 0 && mixed != 1)) return PIMC_ERR_BAD_ARG;
  pimc_handle *h = b->base;
  CK(cudaSetDevice(h->device));
  CK(cudaStreamSynchronize(h->stream));
  b->mixed = mixed;
  for (auto &rp : b->reps) rp.c.s.mixed = mixed;
  pimc_status e = batch_upload_reps(b);
  if (e) return e;
  if (b->tables) {
    // float copies as the moves of this precision write them; caches stale
    launch_batch_refresh(b->d_reps, b->n, 1, h->stream);
    h->launches++;
    CK(cudaGetLastError());
  }
  if (b->exec) { cudaGraphExecDestroy(b->exec); b->exec = nullptr; }
  return PIMC_OK;
}

extern "C" pimc_status pimc_batch_set_shape(pimc_batch *b, int warps, int min_blocks)
{
  if (!b || (warps != 2 && warps != 4 && warps != 8) || min_blocks < 2 || min_blocks > 4) return PIMC_ERR_BAD_ARG;
  b->warps = warps;
  b->minb = min_blocks;      // the persistent pass is bounded for at most 3
  return PIMC_OK;
}

extern "C" pimc_status pimc_batch_set_rotation_mode(pimc_batch *b, int mode)
{
  if (!b || mode < 0 || mode > 1) return PIMC_ERR_BAD_ARG;
  if (mode == 1)
    for (int r = 0; r < b->n; r++) {
      const DevSys &d = b->reps[r].c.s;
      if (d.nrotors > 0 && b->sys[r].rotation && d.Q % 2) return PIMC_ERR_BAD_ARG;   // the odd-Q serial step
    }
  b->rot_mode = mode;
  return PIMC_OK;
}

// the flat mode's tables: per block, the replicas by decreasing sweep count
// in that block and the prefix sums of their slice pairs (Q/2)
static pimc_status batch_flat_tables(pimc_batch *b, int nbk)
{
  pimc_handle *h = b->base;
  if (b->d_flat_sorted) return PIMC_OK;
  std::vector<int> sorted((size_t)nbk * b->n), pre((size_t)nbk * (b->n + 1));
  b->flat_nact_max.assign(nbk, 0);
  for (int blk = 0; blk < nbk; blk++) {
    std::vector<std::pair<int, int>> k(b->n);
    for (int r = 0; r < b->n; r++) {
      const DevSys &d = b->reps[r].c.s;
      int sw = 0;
      if (d.nrotors > 0 && b->sys[r].rotation)
        sw = (int)((long long)(blk + 1) * d.P / nbk) - (int)((long long)blk * d.P / nbk);
      k[r] = {-sw, r};
    }
    std::stable_sort(k.begin(), k.end());
    int acc = 0;
    pre[(size_t)blk * (b->n + 1)] = 0;
    for (int i = 0; i < b->n; i++) {
      sorted[(size_t)blk * b->n + i] = k[i].second;
      acc += b->reps[k[i].second].c.s.Q / 2;
      pre[(size_t)blk * (b->n + 1) + i + 1] = acc;
    }
    b->flat_nact_max[blk] = b->n ? -k[0].first : 0;
  }
  pimc_status e;
  if ((e = pool(h, &b->d_flat_sorted, sorted.size())) || (e = pool(h, &b->d_flat_pre, pre.size()))) return e;
  CK(cudaMemcpy(b->d_flat_sorted, sorted.data(), sorted.size() * sizeof(int), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(b->d_flat_pre, pre.data(), pre.size() * sizeof(int), cudaMemcpyHostToDevice));
  // replicas still active at sweep j of block blk: a prefix of that block's order
  b->flat_act.assign((size_t)nbk, std::vector<int>());
  for (int blk = 0; blk < nbk; blk++) {
    std::vector<int> &act = b->flat_act[blk];
    act.assign(b->flat_nact_max[blk], 0);
    for (int i = 0; i < b->n; i++) {
      const DevSys &d = b->reps[sorted[(size_t)blk * b->n + i]].c.s;
      int sw = (d.nrotors > 0 && b->sys[sorted[(size_t)blk * b->n + i]].rotation)
                   ? (int)((long long)(blk + 1) * d.P / nbk) - (int)((long long)blk * d.P / nbk) : 0;
      for (int j = 0; j < sw; j++) act[j] = i + 1;
    }
    b->flat_units.push_back(std::vector<int>(act.size()));
    for (size_t j = 0; j < act.size(); j++) b->flat_units.back()[j] = pre[(size_t)blk * (b->n + 1) + act[j]];
  }
  return PIMC_OK;
}

static pimc_status batch_ready(pimc_batch *b)
{
  if (!b) return PIMC_ERR_BAD_ARG;
  if (!b->tables) return PIMC_ERR_STATE;
  for (int r = 0; r < b->n; r++)
    if (!b->state_set[r]) return PIMC_ERR_STATE;
  return PIMC_OK;
}

extern "C" pimc_status pimc_batch_run_passes(pimc_batch *b, int npasses, uint64_t seed)
{
  pimc_status e = batch_ready(b);
  if (e) return e;
  if (npasses < 0) return PIMC_ERR_BAD_ARG;
  pimc_handle *h = b->base;
  CK(cudaSetDevice(h->device));
  if (!b->exec || b->exec_seed != seed || b->exec_warps != b->warps || b->exec_minb != b->minb ||
      b->exec_mixed != b->mixed || b->exec_rot_mode != b->rot_mode || b->exec_flat_minb != b->minb) {
    if (b->exec) { BK(cudaGraphExecDestroy(b->exec)); b->exec = nullptr; }
    int nctas = batch_max_ctas(b->mixed, b->warps, b->minb);
    if (nctas <= 0) return PIMC_ERR_CUDA;
    if (nctas > b->n) nctas = b->n;
    const DevSys &d0 = b->reps[0].c.s;
    int nbk = 0;
    for (int t = 0; t < d0.ntypes; t++) nbk += 1 << d0.levels[t];
    if (b->rot_mode == 1) {
      if ((e = batch_flat_tables(b, nbk))) return e;
      if (!batch_flat_setup(b->warps)) return PIMC_ERR_CUDA;
    }
    cudaGraph_t graph;
    CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    if (b->rot_mode == 0) {
      launch_batch_pass(b->d_reps, b->d_order, b->n, seed, b->d_work, b->mixed, b->warps, b->minb, nctas, h->stream);
    } else {
      // per block: the block's bisections of every replica in one persistent
      // launch, then its sweeps, one launch per half-sweep over all replicas
      for (int blk = 0; blk < nbk; blk++) {
        launch_batch_pass(b->d_reps, b->d_order, b->n, seed, b->d_work, b->mixed, b->warps, b->minb, nctas,
                          h->stream, 0, blk, blk + 1);
        for (int j = 0; j < b->flat_nact_max[blk]; j++)
          for (int parity = 0; parity < 2; parity++)
            launch_batch_rot_flat(b->d_reps, b->d_flat_sorted + (size_t)blk * b->n,
                                  b->d_flat_pre + (size_t)blk * (b->n + 1), b->flat_act[blk][j],
                                  b->flat_units[blk][j], blk, j, parity, nbk, seed, b->mixed, b->warps,
                                  b->minb, h->stream);
      }
    }
    cudaError_t le = cudaGetLastError();
    cudaError_t ce = cudaStreamEndCapture(h->stream, &graph);
    if (le != cudaSuccess || ce != cudaSuccess) {
      if (ce == cudaSuccess) cudaGraphDestroy(graph);
      h->last_cuda = le != cudaSuccess ? le : ce;
      return PIMC_ERR_CUDA;
    }
    cudaError_t ie = cudaGraphInstantiate(&b->exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ie != cudaSuccess) { h->last_cuda = ie; return PIMC_ERR_CUDA; }
    b->exec_seed = seed;
    b->exec_warps = b->warps;
    b->exec_minb = b->minb;
    b->exec_mixed = b->mixed;
    b->exec_rot_mode = b->rot_mode;
    b->exec_flat_minb = b->minb;
    long long nodes = 2;
    if (b->rot_mode == 1) {
      nodes = 2LL * nbk;
      for (int blk = 0; blk < nbk; blk++)
        for (int j = 0; j < b->flat_nact_max[blk]; j++) nodes += 2 * (b->flat_units[blk][j] > 0);
    }
    b->exec_nodes = nodes;
  }
  for (int p = 0; p < npasses; p++) {
    CK(cudaGraphLaunch(b->exec, h->stream));
    h->launches += b->exec_nodes;
  }
  if (npasses > 0) {
    launch_batch_refresh(b->d_reps, b->n, 0, h->stream);     // double frames and MCCosine of tops
    h->launches++;
    CK(cudaGetLastError());
  }
  return PIMC_OK;
}

// ---- delayed acceptance over a batch of water dimers

// every replica a water dimer of one shape (two tops, no atoms, tabulated
// densities, the same P, Q and R, even Q): the moves of a sub-phase of all
// replicas are then one flat index range
static pimc_status batch_da_check(pimc_batch *b)
{
  const DevSys &d0 = b->reps[0].c.s;
  for (int r = 0; r < b->n; r++) {
    const DevSys &d = b->reps[r].c.s;
    if (d.nrotors != 2 || d.na != 2 || d.molecule[d.imtype] != PIMC_NONLINEAR || d.rot_den_type != 0 || d.Q % 2 ||
        d.Q != d0.Q || d.R != d0.R || d.P != d0.P || !b->sys[r].rotation)
      return PIMC_ERR_STATE;
  }
  return PIMC_OK;
}

// nsweeps delayed-acceptance sweeps of every replica (pimc_da_sweeps of each,
// with the replica's seed); with translation = 1, `npasses` passes instead:
// each the translational moves of the production pass (rotation off), then
// P sweeps.  One CUDA graph per call shape.
static pimc_status batch_da_run(pimc_batch *b, pimc_mlp *m, int count, int passes, uint64_t seed, float escale,
                                int use_surrogate, double *stats)
{
  pimc_status e = batch_ready(b);
  if (e) return e;
  if ((e = batch_da_check(b))) return e;
  if (count < 0 || (use_surrogate && !m)) return PIMC_ERR_BAD_ARG;
  if (use_surrogate && mlp_poisoned(m)) return PIMC_ERR_TIMEOUT;
  pimc_handle *h = b->base;
  CK(cudaSetDevice(h->device));
  const DevSys &d = b->reps[0].c.s;
  const int nm = d.Q / 2, nsw = passes ? d.P : count;
  if ((long long)nsw * (passes ? count : 1) > (1 << 20)) return PIMC_ERR_SIZE;
  const size_t moves = (size_t)nm * b->n, rows = moves * 2 * d.R;
  size_t bytes = rows * 7 * sizeof(float) + moves * sizeof(DaMove) + 4096;
  void *buf;
  if ((e = scratch(h, bytes, &buf))) return e;
  char *cur = (char *)buf;
  unsigned long long *st = (unsigned long long *)cur;
  cur += 256;
  float *feat = (float *)cur;
  cur += (rows * 6 * sizeof(float) + 255) / 256 * 256;
  float *y = (float *)cur;
  cur += (rows * sizeof(float) + 255) / 256 * 256;
  DaMove *mv = (DaMove *)cur;
  int nctas = 0;
  if (passes) {
    nctas = batch_max_ctas(b->mixed, b->warps, b->minb);
    if (nctas <= 0) return PIMC_ERR_CUDA;
    if (nctas > b->n) nctas = b->n;
  }
  auto sweeps = [&]() -> long long {
    long long n = 0;
    for (int sw = 0; sw < nsw; sw++)
      for (int par = 0; par < 2; par++)
        for (int r = 0; r < 2; r++) {
          unsigned phase = 4u * (unsigned)sw + 2u * par + r;
          n += launch_da_propose_b(b->d_reps, nm, b->n, r, par, phase, seed, feat, mv, b->mixed, h->stream);
          if (use_surrogate) n += mlp_forward_device(m, feat, (int)rows, y, h->stream);
          n += launch_da_decide_b(b->d_reps, nm, b->n, r, par, phase, seed, y, use_surrogate, escale, mv, st,
                                  b->mixed, h->stream);
        }
    return n;
  };
  auto record = [&]() -> long long {
    long long n = 0;
    if (passes) {
      // the translational moves advance the pass counters that key the sweeps' draws
      launch_batch_pass(b->d_reps, b->d_order, b->n, seed, b->d_work, b->mixed, b->warps, b->minb, nctas, h->stream,
                        0);
      n += 2;
    } else {
      n += launch_da_pass_b(b->d_reps, b->n, h->stream);
    }
    n += sweeps();
    launch_batch_rot_changed(b->d_reps, b->n, h->stream);
    return n + 1;
  };
  const unsigned long long mk = use_surrogate ? mlp_uid(m) : 0ull;
  const int key_count = passes ? -1 : count;
  if (!b->da_exec || b->da_count != key_count || b->da_seed != seed || b->da_use != use_surrogate ||
      b->da_escale != escale || b->da_mlp != mk || b->da_buf != buf || b->da_shape != b->warps * 8 + b->minb ||
      b->da_mixed != b->mixed) {
    if (b->da_exec) { BK(cudaGraphExecDestroy(b->da_exec)); b->da_exec = nullptr; }
    cudaGraph_t graph;
    CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    long long n = record();
    cudaError_t le = cudaGetLastError();
    cudaError_t ce = cudaStreamEndCapture(h->stream, &graph);
    if (le != cudaSuccess || ce != cudaSuccess) {
      if (ce == cudaSuccess) cudaGraphDestroy(graph);
      h->last_cuda = le != cudaSuccess ? le : ce;
      return PIMC_ERR_CUDA;
    }
    cudaError_t ie = cudaGraphInstantiate(&b->da_exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ie != cudaSuccess) { h->last_cuda = ie; return PIMC_ERR_CUDA; }
    b->da_count = key_count; b->da_seed = seed; b->da_use = use_surrogate; b->da_escale = escale;
    b->da_mlp = mk; b->da_buf = buf; b->da_nodes = n; b->da_shape = b->warps * 8 + b->minb; b->da_mixed = b->mixed;
  }
  CK(cudaMemsetAsync(st, 0, 4 * sizeof(unsigned long long), h->stream));
  const int nlaunch = passes ? count : 1;
  for (int p = 0; p < nlaunch; p++) {
    CK(cudaGraphLaunch(b->da_exec, h->stream));
    h->launches += b->da_nodes;
  }
  if (b->mixed) {                    // the FP32 moves leave the double frames to be derived from the angles
    launch_batch_refresh(b->d_reps, b->n, 0, h->stream);
    h->launches++;
  }
  unsigned long long hs[4];
  CK(cudaMemcpyAsync(hs, st, sizeof(hs), cudaMemcpyDeviceToHost, h->stream));
  e = check_err(h);
  if (!e && use_surrogate && mlp_take_error(m)) e = PIMC_ERR_TIMEOUT;
  if (stats)
    for (int k = 0; k < 4; k++) stats[k] = (double)hs[k];
  return e;
}

extern "C" pimc_status pimc_batch_da_sweeps(pimc_batch *b, pimc_mlp *m, int nsweeps, uint64_t seed, float escale,
                                            int use_surrogate, double *stats)
{
  if (nsweeps > (1 << 18)) return PIMC_ERR_BAD_ARG;
  return batch_da_run(b, m, nsweeps, 0, seed, escale, use_surrogate, stats);
}

extern "C" pimc_status pimc_batch_da_passes(pimc_batch *b, pimc_mlp *m, int npasses, uint64_t seed, float escale,
                                            int use_surrogate, double *stats)
{
  return batch_da_run(b, m, npasses, 1, seed, escale, use_surrogate, stats);
}

// the shapes tried: warps per CTA x CTAs per SM the registers are bounded for
static const int g_batch_shapes[6][2] = {{2, 2}, {4, 2}, {8, 2}, {4, 3}, {8, 3}, {2, 3}};

extern "C" pimc_status pimc_batch_autotune(pimc_batch *b, uint64_t seed, int *shape_out, double *ms_out)
{
  pimc_status e = batch_ready(b);
  if (e) return e;
  pimc_handle *h = b->base;
  CK(cudaSetDevice(h->device));
  double best = 1e300;
  int bw = b->warps, bm = b->minb;
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  for (int k = 0; k < 6; k++) {
    b->warps = g_batch_shapes[k][0];
    b->minb = g_batch_shapes[k][1];
    if (ms_out) ms_out[k] = 0.0;
    if (batch_max_ctas(b->mixed, b->warps, b->minb) <= 0) continue;
    if ((e = pimc_batch_run_passes(b, 1, seed))) return e;      // graph build and warm-up
    CK(cudaEventRecord(e0, h->stream));
    if ((e = pimc_batch_run_passes(b, 1, seed))) return e;
    CK(cudaEventRecord(e1, h->stream));
    CK(cudaEventSynchronize(e1));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    if (ms_out) ms_out[k] = ms;
    if (ms < best) { best = ms; bw = b->warps; bm = b->minb; }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  b->warps = bw;
  b->minb = bm;
  if (shape_out) { shape_out[0] = bw; shape_out[1] = bm; }
  return check_err(h);
}

extern "C" pimc_status pimc_batch_estimators(pimc_batch *b, double *out)
{
  pimc_status e = batch_ready(b);
  if (e) return e;
  if (!out) return PIMC_ERR_BAD_ARG;
  pimc_handle *h = b->base;
  CK(cudaSetDevice(h->device));
  launch_batch_est(b->d_reps, b->n, b->d_est, h->stream);
  h->launches++;
  CK(cudaGetLastError());
  std::vector<double> v((size_t)b->n * 6);
  CK(cudaMemcpyAsync(v.data(), b->d_est, v.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  if ((e = check_err(h))) return e;
  for (int r = 0; r < b->n; r++) {
    const DevSys &d = b->reps[r].c.s;
    const double *w = v.data() + 6 * (size_t)r;
    double *o = out + 4 * (size_t)r;
    o[0] = (double)d.P * d.temperature * (0.5 * (double)(3 * d.na) - w[0]);    // mc_estim.cc:923-934
    o[1] = w[1] / (double)d.P;
    double erot = 0.0, cz = 0.0;
    if (d.nrotors > 0 && b->sys[r].rotation) {
      if (d.molecule[d.imtype] == PIMC_LINEAR) {                                 // mc_estim.cc:953-984
        erot = w[2];
        if (d.rot_den_type == 1) erot = (erot / (double)d.Q) / d.rot_tau + 1.0 / d.rot_tau;
      } else {                                                                   // mc_estim.cc:1000-1092
        int skip = d.rot_den_type == 0 ? 1 : d.rn_ratio;
        erot = w[2] / (double)(d.Q / skip);
        if (d.rot_den_type == 1 && d.rn_ratio == 1) {          // per rotor, summed (see pimc_estimators)
          erot = erot / (4.0 * (d.rot_tau / PIMC_WNO2K) * (d.rot_tau / PIMC_WNO2K));
          erot += (double)d.nrotors * (0.25 * (d.abc[0] + d.abc[1] + d.abc[2]) + 1.5 / (d.rot_tau / PIMC_WNO2K));
          erot = erot / PIMC_WNO2K;
        }
      }
      cz = w[5] / ((double)d.nrotors * d.Q);
    }
    o[2] = erot;
    o[3] = cz;
  }
  return PIMC_OK;
}

extern "C" pimc_status pimc_batch_counters(pimc_batch *b, double *total, double *accep)
{
  if (!b || !total || !accep) return PIMC_ERR_BAD_ARG;
  pimc_handle *h = b->base;
  CK(cudaSetDevice(h->device));
  CK(cudaStreamSynchronize(h->stream));
  std::vector<unsigned long long> v((size_t)b->n * 12);
  CK(cudaMemcpy(v.data(), b->d_cnt, v.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
  for (int k = 0; k < 6; k++) { total[k] = 0.0; accep[k] = 0.0; }
  for (int r = 0; r < b->n; r++)
    for (int k = 0; k < 6; k++) {
      total[k] += (double)v[12 * (size_t)r + 2 * k];
      accep[k] += (double)v[12 * (size_t)r + 2 * k + 1];
    }
  return PIMC_OK;
}

extern "C" pimc_status pimc_batch_synchronize(pimc_batch *b)
{
  if (!b) return PIMC_ERR_BAD_ARG;
  pimc_handle *h = b->base;
  CK(cudaSetDevice(h->device));
  return check_err(h);
}

extern "C" double pimc_batch_bead_moves_per_pass(const pimc_batch *b) { return b ? b->bm_pass : 0.0; }

extern "C" void *pimc_batch_stream(const pimc_batch *b) { return b ? (void *)b->base->stream : nullptr; }

// ------------------------------------------------------------ checkpoints
// A complete restart file (the reference's ConfigIO, mc_input.cc:560-600,
// writes only the first row of MCCoords and MCCosine): the system's sizes for
// validation, the whole path (MCCoords, MCAngles, PIndex), the pass counter
// the production uniforms are keyed by, and the move counters.  A run that
// loads it and continues with the same seed repeats the uninterrupted run.
static const char g_ckpt_magic[8] = {'P', 'I', 'M', 'C', 'G', 'B', '3', '1'};

struct CkptHead {
  char magic[8];
  int version, na, P, Q, nrotors, ntypes, numb[PIMC_MAX_TYPES], mixed;
  double temperature;
  unsigned pass;
  unsigned long long cnt[12];
};

extern "C" pimc_status pimc_save_checkpoint(pimc_handle *h, const char *path)
{
  pimc_status e = ready(h);
  if (e) return e;
  if (!path) return PIMC_ERR_BAD_ARG;
  const DevSys &d = h->ctx.s;
  size_t nbr = (size_t)d.na * d.P;
  std::vector<double> coords(3 * nbr), angles(3 * nbr), cosine(3 * nbr);
  std::vector<int> pidx(d.na);
  if ((e = pimc_get_state(h, coords.data(), angles.data(), cosine.data(), pidx.data()))) return e;
  CkptHead hd;
  memset(&hd, 0, sizeof(hd));
  memcpy(hd.magic, g_ckpt_magic, 8);
  hd.version = 1;
  hd.na = d.na; hd.P = d.P; hd.Q = d.Q; hd.nrotors = d.nrotors; hd.ntypes = d.ntypes;
  for (int t = 0; t < d.ntypes; t++) hd.numb[t] = d.numb[t];
  hd.mixed = d.mixed;
  hd.temperature = d.temperature;
  CK(cudaMemcpy(&hd.pass, h->pass, sizeof(unsigned), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(hd.cnt, h->cnt, sizeof(hd.cnt), cudaMemcpyDeviceToHost));
  FILE *f = fopen(path, "wb");
  if (!f) return PIMC_ERR_BAD_ARG;
  bool ok = fwrite(&hd, sizeof(hd), 1, f) == 1 && fwrite(coords.data(), sizeof(double), 3 * nbr, f) == 3 * nbr &&
            fwrite(angles.data(), sizeof(double), 3 * nbr, f) == 3 * nbr &&
            fwrite(cosine.data(), sizeof(double), 3 * nbr, f) == 3 * nbr &&
            fwrite(pidx.data(), sizeof(int), d.na, f) == (size_t)d.na;
  ok = (fclose(f) == 0) && ok;
  return ok ? PIMC_OK : PIMC_ERR_BAD_ARG;
}

extern "C" pimc_status pimc_load_checkpoint(pimc_handle *h, const char *path)
{
  if (!h || !path) return PIMC_ERR_BAD_ARG;
  CK(cudaSetDevice(h->device));
  const DevSys &d = h->ctx.s;
  FILE *f = fopen(path, "rb");
  if (!f) return PIMC_ERR_BAD_ARG;
  CkptHead hd;
  size_t nbr = (size_t)d.na * d.P;
  std::vector<double> coords(3 * nbr), angles(3 * nbr), cosine(3 * nbr);
  std::vector<int> pidx(d.na);
  bool ok = fread(&hd, sizeof(hd), 1, f) == 1;
  ok = ok && memcmp(hd.magic, g_ckpt_magic, 8) == 0 && hd.version == 1 && hd.na == d.na && hd.P == d.P &&
       hd.Q == d.Q && hd.nrotors == d.nrotors && hd.ntypes == d.ntypes && hd.temperature == d.temperature;
  for (int t = 0; ok && t < d.ntypes; t++) ok = hd.numb[t] == d.numb[t];
  ok = ok && fread(coords.data(), sizeof(double), 3 * nbr, f) == 3 * nbr &&
       fread(angles.data(), sizeof(double), 3 * nbr, f) == 3 * nbr &&
       fread(cosine.data(), sizeof(double), 3 * nbr, f) == 3 * nbr &&
       fread(pidx.data(), sizeof(int), d.na, f) == (size_t)d.na;
  fclose(f);
  if (!ok) return PIMC_ERR_BAD_ARG;
  pimc_status e = pimc_set_state(h, coords.data(), angles.data(), pidx.data());
  if (e) return e;
  if (d.nrotors > 0) {
    // MCCosine exactly as saved (set_state derives it from the angles on the host)
    size_t n = (size_t)d.nrotors * d.Q;
    std::vector<double> cs(3 * n);
    for (int k = 0; k < 3; k++)
      for (int r = 0; r < d.nrotors; r++)
        for (int q = 0; q < d.Q; q++) {
          size_t src = k * nbr + (size_t)(d.rot_first + r) * d.P + q;
          cs[k * n + r * d.Q + q] = cosine[src];
          h->cosine_host[src] = cosine[src];
        }
    CK(cudaMemcpy(h->ctx.st.cosv, cs.data(), 3 * n * sizeof(double), cudaMemcpyHostToDevice));
    launch_derive_state(h->ctx, h->frames, h->stream);
    h->launches++;
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(h->stream));
  }
  CK(cudaMemcpy(h->pass, &hd.pass, sizeof(unsigned), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(h->cnt, hd.cnt, sizeof(hd.cnt), cudaMemcpyHostToDevice));
  return PIMC_OK;
}

// IOxyz (mc_input.cc:690-760): the number of beads, a comment line, then per
// bead "<label> x cx y cy z cz" (coordinate and MCCosine component per
// dimension), atoms in type order, slices inside an atom
extern "C" pimc_status pimc_write_xyz(pimc_handle *h, const char *path, const char *const *type_names)
{
  pimc_status e = ready(h);
  if (e) return e;
  if (!path) return PIMC_ERR_BAD_ARG;
  const DevSys &d = h->ctx.s;
  size_t nbr = (size_t)d.na * d.P;
  std::vector<double> coords(3 * nbr), angles(3 * nbr), cosine(3 * nbr);
  if ((e = pimc_get_state(h, coords.data(), angles.data(), cosine.data(), nullptr))) return e;
  FILE *f = fopen(path, "w");
  if (!f) return PIMC_ERR_BAD_ARG;
  // IOxyz's layout (mc_input.cc:726-750): the count, the comment line, then
  // per bead the label (type name and atom number, width 5) and x, cx, y,
  // cy, z, cz in io_setout's format (scientific, 6 digits, width 14), each
  // field followed by three blanks (mc_confg.h:28-29, mc_input.h:48, 60)
  fprintf(f, "%zu\n#   xyz format:  [atom type]  x y z (Angstrom) \n", nbr);
  for (int t = 0; t < d.ntypes; t++)
    for (int a = 0; a < d.numb[t]; a++) {
      char label[64];
      snprintf(label, sizeof(label), "%s%d", type_names && type_names[t] ? type_names[t] : (t ? "M" : "A"), a + 1);
      size_t off = (size_t)(d.first[t] + a) * d.P;
      for (int it = 0; it < d.P; it++) {
        fprintf(f, "%5s   ", label);
        for (int k = 0; k < 3; k++)
          fprintf(f, "%14.6e   %14.6e   ", coords[k * nbr + off + it], cosine[k * nbr + off + it]);
        fprintf(f, "\n");
      }
    }
  return fclose(f) == 0 ? PIMC_OK : PIMC_ERR_BAD_ARG;
}

// IOxyz read: coordinates and unit vectors; the angles of the rotor rows
// follow from the unit vector (phi = atan2(cy, cx), cos theta = cz, chi = 0)
extern "C" pimc_status pimc_read_xyz(pimc_handle *h, const char *path)
{
  if (!h || !path) return PIMC_ERR_BAD_ARG;
  const DevSys &d = h->ctx.s;
  size_t nbr = (size_t)d.na * d.P;
  FILE *f = fopen(path, "r");
  if (!f) return PIMC_ERR_BAD_ARG;
  std::vector<double> coords(3 * nbr), angles(3 * nbr, 0.0);
  size_t count = 0;
  char line[512];
  bool ok = fscanf(f, "%zu", &count) == 1 && count == nbr && fgets(line, sizeof(line), f) && fgets(line, sizeof(line), f);
  for (size_t i = 0; ok && i < nbr; i++) {
    char label[64];
    double v[6];
    ok = fscanf(f, "%63s %lf %lf %lf %lf %lf %lf", label, &v[0], &v[1], &v[2], &v[3], &v[4], &v[5]) == 7;
    if (!ok) break;
    for (int k = 0; k < 3; k++) coords[k * nbr + i] = v[2 * k];
    angles[0 * nbr + i] = atan2(v[3], v[1]);
    angles[1 * nbr + i] = v[5];
  }
  fclose(f);
  if (!ok) return PIMC_ERR_BAD_ARG;
  return pimc_set_state(h, coords.data(), angles.data(), nullptr);
}
