// pimc_tables.cu -- propagator-table generators on the GPU
//
//   pimc_linden  : the exact linear-rotor propagator of linear_prop/linden.f
//                  (exarho linden.f:88-122, lgnd linden.f:182-198) for many
//                  (temperature, slices) pairs at once, one thread per
//                  (table, cos gamma) point;
//   pimc_asymrho : the exact asymmetric-top propagator of nmv_prop/asymrho.f
//                  on its 1-degree (theta, phi, chi) grid.
//
// asymrho's per-point sum over (j, state, m, k) (asymrho.f:560-612) is
// regrouped: the states of each (j, K-parity) block are folded on the host
// into weight matrices W^j[m][k] = pre_j sum_n e^{-tau E_n} c_nm c_nk (and the
// E- and E^2-weighted ones), the device contracts them with Wigner d^j_mk(theta)
// over j (an upward three-term recurrence in j), and the (phi, chi) grid is a
// cosine series in m phi + k chi evaluated in two separable passes from
// integer-degree cosine tables.  The eigenproblems are solved on the host by
// cyclic Jacobi rotations.
#include <cmath>
#include <cstring>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/pimc_gb300.h"

#define CKT(x)                                \
  do {                                        \
    cudaError_t e_ = (x);                     \
    if (e_ != cudaSuccess) return PIMC_ERR_CUDA; \
  } while (0)

namespace {

const double kPi = 3.14159265358979323846;

// ------------------------------------------------------------- linden
// one thread per (table t, point ic): rows (cost, rho, erot, erotsq) of
// linden.f:48-68.  ex[t*ldx + l] = exp(-tau_t B l(l+1)) is computed on the
// host; the products and sums run in the reference's order with
// contraction-free double arithmetic.
__global__ void k_linden(int ntab, int npt, int iodevn, double bconst, const int *lmax, const int *nslice,
                         const double *ex, int ldx, double *out)
{
  int ic = blockIdx.x * blockDim.x + threadIdx.x;
  int t = blockIdx.y;
  if (t >= ntab || ic >= npt) return;
  const double pi = kPi, boltz = 0.69503476;
  double cstep = 2.0 / (double)(npt - 1);
  double x = __dsub_rn(__dmul_rn((double)ic, cstep), 1.0);
  int L = lmax[t];
  const double *e = ex + (size_t)t * ldx;
  double pm1 = 0.0, p = 1.0;   // P_{l-1}, P_l
  double r = 0.0, er = 0.0, es = 0.0;
  for (int l = 0; l <= L; l++) {
    if (l == 1) { pm1 = 1.0; p = x; }
    else if (l >= 2) {
      int q = l - 1;           // P_l from P_{q}, P_{q-1}
      double a = __dmul_rn(__dmul_rn(__dadd_rn(2.0 * q, 1.0), x), p);
      double b = __dmul_rn((double)q, pm1);
      double pn = __ddiv_rn(__dsub_rn(a, b), (double)(q + 1));
      pm1 = p;
      p = pn;
    }
    if ((l % 2) == iodevn || iodevn == -1) {
      double tmp = __dmul_rn((double)(2 * l + 1), p);
      tmp = __dmul_rn(tmp, e[l]);
      r = __dadd_rn(r, tmp);
      double te = __dmul_rn(__dmul_rn(__dmul_rn(tmp, (double)l), (double)(l + 1)), bconst);
      er = __dadd_rn(er, te);
      double ts = __dmul_rn(__dmul_rn(__dmul_rn(te, (double)l), (double)(l + 1)), bconst);
      es = __dadd_rn(es, ts);
    }
  }
  double nb = __dmul_rn((double)nslice[t], boltz);
  er = __ddiv_rn(er, nb);
  es = __ddiv_rn(es, __dmul_rn(nb, nb));
  double fpi = 4.0 * pi;
  double *o = out + (size_t)t * 4 * npt;
  o[ic] = x;
  o[npt + ic] = __ddiv_rn(r, fpi);
  o[2 * npt + ic] = __ddiv_rn(er, fpi);
  o[3 * npt + ic] = __ddiv_rn(es, fpi);
}

// ------------------------------------------------------------- asymrho
// K-parity block of j: first k and size (asymrho.f:120-129); par 0 even k
__host__ __device__ inline void block_of(int j, int par, int *kst, int *nd)
{
  if (j % 2 == 0) { *kst = par ? -j + 1 : -j; *nd = par ? j : j + 1; }
  else { *kst = par ? -j : -j + 1; *nd = par ? j + 1 : j; }
}

// d^j0_mk(theta) at j0 = max(|m|,|k|): the one surviving term of the
// factorial sum, sqrt(C(2 j0, j0 + a)) cos(theta/2)^p (-sin(theta/2))^q,
// with the binomial's square root built up factor by factor between the
// powers so that nothing overflows
__device__ double wigner_start(int m, int k, double c, double s)
{
  int j = max(abs(m), abs(k));
  int a, p, q;
  double sgn = 1.0;
  if (abs(m) >= abs(k)) {
    a = abs(k);
    if (m == j) { p = j + k; q = j - k; }
    else { p = j - k; q = j + k; sgn = ((j + k) & 1) ? -1.0 : 1.0; }
  } else {
    a = abs(m);
    if (k == j) { p = j + m; q = j - m; sgn = ((j - m) & 1) ? -1.0 : 1.0; }
    else { p = j - m; q = j + m; }
  }
  double v = 1.0;
  int nf = j - a;
  double ms = -s;
  int pq = 0, pp = 0;
  for (int i = 1; i <= nf; i++) {
    v *= sqrt((double)(j + a + i) / (double)i);
    // interleave the powers so the running product stays bounded
    while (pq < q && fabs(v) > 1.0) { v *= ms; pq++; }
    while (pp < p && fabs(v) > 1.0) { v *= c; pp++; }
  }
  for (; pq < q; pq++) v *= ms;
  for (; pp < p; pp++) v *= c;
  return sgn * v;
}

// A_w[ith][m][k] = sum_j W_w^j[m][k] d^j_mk(theta), one thread per (m, k)
// of one theta; W holds pre_j * sum over the block's states with e^{-tau E},
// E e^{-tau E}, E^2 e^{-tau E} weights (w = 0, 1, 2).  Pairs of unlike
// parity (m - k odd) do not occur in any block and get zeros.
__global__ void k_asym_coef(int jmax, int ith0, const int *woff, const double *W, double *A)
{
  const int M = 2 * jmax + 1;
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  int it = blockIdx.y;
  if (idx >= M * M) return;
  int m = idx / M - jmax, k = idx % M - jmax;
  double a0 = 0.0, a1 = 0.0, a2 = 0.0;
  if (((m - k) & 1) == 0) {
    int par = k & 1;
    double th = (double)(ith0 + it) * kPi / 180.0;
    double c = cos(0.5 * th), s = sin(0.5 * th), x = cos(th);
    int j0 = max(abs(m), abs(k));
    double dm1 = 0.0, d = wigner_start(m, k, c, s);
    for (int j = j0; j <= jmax; j++) {
      if (j > j0) {
        int q = j - 1;
        double dn;
        if (q == 0) dn = x;   // d^1_00 = cos(theta)
        else {
          double aa = (2.0 * q + 1.0) * ((double)q * (q + 1) * x - (double)m * k);
          double bb = (double)(q + 1) * sqrt((double)(q * q - m * m) * (double)(q * q - k * k));
          double cc = (double)q * sqrt((double)((q + 1) * (q + 1) - m * m) * (double)((q + 1) * (q + 1) - k * k));
          dn = (aa * d - bb * dm1) / cc;
        }
        dm1 = d;
        d = dn;
      }
      int kst, nd;
      block_of(j, par, &kst, &nd);
      int im = (m - kst) >> 1, ik = (k - kst) >> 1;
      size_t o = (size_t)woff[2 * j + par] + (size_t)im * nd + ik;
      size_t blk = (size_t)nd * nd;
      a0 += W[o] * d;
      a1 += W[o + blk] * d;
      a2 += W[o + 2 * blk] * d;
    }
  }
  size_t base = (size_t)it * 3 * M * M;
  A[base + idx] = a0;
  A[base + (size_t)M * M + idx] = a1;
  A[base + 2 * (size_t)M * M + idx] = a2;
}

// B/C[ith][w][m][chi] = sum_k A_w[m][k] (cos, sin)(k chi) over k of m's parity
__global__ void k_asym_chi(int jmax, const double *A, const double *cosd, const double *sind, double *B, double *C)
{
  const int M = 2 * jmax + 1;
  __shared__ double row[2 * PIMC_ASYMRHO_MAXJ + 1];
  __shared__ double cs[360], sn[360];
  int wm = blockIdx.x, it = blockIdx.y;
  int w = wm / M, mi = wm % M;
  const double *Ar = A + (size_t)it * 3 * M * M + (size_t)w * M * M + (size_t)mi * M;
  for (int i = threadIdx.x; i < M; i += blockDim.x) row[i] = Ar[i];
  for (int i = threadIdx.x; i < 360; i += blockDim.x) { cs[i] = cosd[i]; sn[i] = sind[i]; }
  __syncthreads();
  int chi = threadIdx.x;
  if (chi > 360) return;
  int m = mi - jmax;
  int k0 = ((m + jmax) & 1) ? -jmax + 1 : -jmax;   // k of m's parity
  double b = 0.0, c = 0.0;
  for (int k = k0; k <= jmax; k += 2) {
    int g = (k * chi) % 360;
    if (g < 0) g += 360;
    double a = row[k + jmax];
    b += a * cs[g];
    c += a * sn[g];
  }
  size_t o = (((size_t)it * 3 + w) * M + mi) * 361 + chi;
  B[o] = b;
  C[o] = c;
}

// the (phi, chi) grid: V_w,par = sum_m cos(m phi) B - sin(m phi) C over m of
// one parity, then the reference's per-point division by rho and the
// combination of the parities (asymrho.f:614-633, 698-719)
__global__ void k_asym_grid(int jmax, int iodevn, const double *B, const double *C, const double *cosd,
                            const double *sind, double *rho, double *erot, double *esq)
{
  const int M = 2 * jmax + 1;
  __shared__ double cm[2 * PIMC_ASYMRHO_MAXJ + 1], sm[2 * PIMC_ASYMRHO_MAXJ + 1];
  int phi = blockIdx.x, it = blockIdx.y;
  for (int i = threadIdx.x; i < M; i += blockDim.x) {
    int g = ((i - jmax) * phi) % 360;
    if (g < 0) g += 360;
    cm[i] = cosd[g];
    sm[i] = sind[g];
  }
  __syncthreads();
  int chi = threadIdx.x;
  if (chi > 360) return;
  double v[2][3] = {{0, 0, 0}, {0, 0, 0}};
  for (int w = 0; w < 3; w++) {
    const double *Bw = B + ((size_t)it * 3 + w) * M * 361, *Cw = C + ((size_t)it * 3 + w) * M * 361;
    for (int mi = 0; mi < M; mi++) {
      int par = (mi - jmax) & 1;
      v[par][w] += cm[mi] * Bw[(size_t)mi * 361 + chi] - sm[mi] * Cw[(size_t)mi * 361 + chi];
    }
  }
  double r[2], e[2], s[2];
  for (int par = 0; par < 2; par++) {
    r[par] = v[par][0];
    if (fabs(r[par]) > 1.0e-16) { e[par] = v[par][1] / r[par]; s[par] = v[par][2] / r[par]; }
    else { e[par] = 0.0; s[par] = 0.0; }
  }
  size_t o = ((size_t)it * 361 + phi) * 361 + chi;
  if (iodevn == 0) { rho[o] = r[0]; erot[o] = e[0]; esq[o] = s[0]; }
  else if (iodevn == 1) { rho[o] = r[1]; erot[o] = e[1]; esq[o] = s[1]; }
  else {
    double rc = r[1] + r[0];
    rho[o] = r[0] + r[1];
    double eo = (e[1] * r[1] + e[0] * r[0]) / (r[0] + r[1]);
    double so = (s[1] * r[1] + s[0] * r[0]) / (r[0] + r[1]);
    if (fabs(rc) < 1.e-16) { eo = 0.0; so = 0.0; }
    erot[o] = eo;
    esq[o] = so;
  }
}

// ------------------------------------------------------------- host side

// symmetric eigenproblem by cyclic Jacobi rotations: a (n x n row-major) is
// destroyed, eigenvalues ascending in w, eigenvector i in column i of v
void jacobi_eigen(int n, std::vector<double> &a, std::vector<double> &v, std::vector<double> &w)
{
  v.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; i++) v[(size_t)i * n + i] = 1.0;
  for (int sweep = 0; sweep < 100; sweep++) {
    double off = 0.0, dia = 0.0;
    for (int p = 0; p < n; p++) {
      dia += a[(size_t)p * n + p] * a[(size_t)p * n + p];
      for (int q = p + 1; q < n; q++) off += a[(size_t)p * n + q] * a[(size_t)p * n + q];
    }
    if (off == 0.0 || off <= 1e-36 * dia) break;
    for (int p = 0; p < n - 1; p++)
      for (int q = p + 1; q < n; q++) {
        double apq = a[(size_t)p * n + q];
        if (apq == 0.0) continue;
        double th = (a[(size_t)q * n + q] - a[(size_t)p * n + p]) / (2.0 * apq);
        double t = fabs(th) > 1e150 ? 0.5 / th : (th >= 0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
        double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; k++) {
          double akp = a[(size_t)k * n + p], akq = a[(size_t)k * n + q];
          a[(size_t)k * n + p] = c * akp - s * akq;
          a[(size_t)k * n + q] = s * akp + c * akq;
        }
        for (int k = 0; k < n; k++) {
          double apk = a[(size_t)p * n + k], aqk = a[(size_t)q * n + k];
          a[(size_t)p * n + k] = c * apk - s * aqk;
          a[(size_t)q * n + k] = s * apk + c * aqk;
        }
        for (int k = 0; k < n; k++) {
          double vkp = v[(size_t)k * n + p], vkq = v[(size_t)k * n + q];
          v[(size_t)k * n + p] = c * vkp - s * vkq;
          v[(size_t)k * n + q] = s * vkp + c * vkq;
        }
      }
  }
  std::vector<int> ord(n);
  for (int i = 0; i < n; i++) ord[i] = i;
  for (int i = 1; i < n; i++)   // insertion sort by eigenvalue
    for (int j = i; j > 0 && a[(size_t)ord[j] * n + ord[j]] < a[(size_t)ord[j - 1] * n + ord[j - 1]]; j--)
      std::swap(ord[j], ord[j - 1]);
  w.resize(n);
  std::vector<double> vs((size_t)n * n);
  for (int i = 0; i < n; i++) {
    w[i] = a[(size_t)ord[i] * n + ord[i]];
    for (int k = 0; k < n; k++) vs[(size_t)k * n + i] = v[(size_t)k * n + ord[i]];
  }
  v.swap(vs);
}

// <j k|H|j k'> of asymrho.f:792-813 (cplus/cminus :752-790)
double cplus(int j, int k) { return (k >= j || k < -j) ? 0.0 : sqrt((double)j * (j + 1.0) - (double)k * (k + 1.0)); }
double cminus(int j, int k) { return (k <= -j || k > j) ? 0.0 : sqrt((double)j * (j + 1.0) - (double)k * (k - 1.0)); }
double rotmat(int j, int k, int kp, double A, double B, double C)
{
  if (abs(k - kp) != 0 && abs(k - kp) != 2) return 0.0;
  if (k == kp) return 0.5 * (A + C) * (double)(j * (j + 1)) + (B - 0.5 * (A + C)) * (double)(k * k);
  if (k == kp + 2) return 0.25 * (A - C) * cplus(j, kp) * cplus(j, kp + 1);
  return 0.25 * (A - C) * cminus(j, kp) * cminus(j, kp - 1);
}

struct DevBuf {
  std::vector<void *> p;
  ~DevBuf()
  {
    for (void *q : p) cudaFree(q);
  }
  template <class T>
  cudaError_t alloc(T **out, size_t n)
  {
    void *q = nullptr;
    cudaError_t e = cudaMalloc(&q, n * sizeof(T) > 0 ? n * sizeof(T) : 1);
    if (e == cudaSuccess) p.push_back(q);
    *out = (T *)q;
    return e;
  }
};

}  // namespace

extern "C" pimc_status pimc_linden(int device, int n, const double *temperature, const int *nslice, double bconst,
                                   int npt, int iodevn, double *out)
{
  if (n <= 0 || npt < 2 || !temperature || !nslice || !out || iodevn < -1 || iodevn > 1) return PIMC_ERR_BAD_ARG;
  const double taunit = 1.4387752224, eps = 1.e-16;
  const int maxl = 500, ldx = maxl + 1;
  std::vector<int> lmax(n);
  std::vector<double> ex((size_t)n * ldx, 0.0);
  for (int t = 0; t < n; t++) {
    if (!(temperature[t] > 0.0) || nslice[t] < 1) return PIMC_ERR_BAD_ARG;
    double tau = taunit / (temperature[t] * nslice[t]);
    int L = maxl;                                   // linden.f:26-36
    for (int l = 0; l <= maxl; l++)
      if (exp(-tau * bconst * l * (l + 1)) < eps) { L = l; break; }
    lmax[t] = L;
    for (int l = 0; l <= L; l++) ex[(size_t)t * ldx + l] = exp(-tau * bconst * (double)(l * (l + 1)));
  }
  CKT(cudaSetDevice(device));
  cudaStream_t s;
  CKT(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  DevBuf db;
  int *dl = nullptr, *dn = nullptr;
  double *dex = nullptr, *dout = nullptr;
  pimc_status st = PIMC_OK;
  if (db.alloc(&dl, n) || db.alloc(&dn, n) || db.alloc(&dex, ex.size()) || db.alloc(&dout, (size_t)n * 4 * npt))
    st = PIMC_ERR_CUDA;
  if (!st && (cudaMemcpyAsync(dl, lmax.data(), n * sizeof(int), cudaMemcpyHostToDevice, s) ||
              cudaMemcpyAsync(dn, nslice, n * sizeof(int), cudaMemcpyHostToDevice, s) ||
              cudaMemcpyAsync(dex, ex.data(), ex.size() * sizeof(double), cudaMemcpyHostToDevice, s)))
    st = PIMC_ERR_CUDA;
  if (!st) {
    dim3 grid((npt + 127) / 128, n);
    k_linden<<<grid, 128, 0, s>>>(n, npt, iodevn, bconst, dl, dn, dex, ldx, dout);
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpyAsync(out, dout, (size_t)n * 4 * npt * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      st = PIMC_ERR_CUDA;
  }
  cudaStreamSynchronize(s);
  cudaStreamDestroy(s);
  return st;
}

extern "C" pimc_status pimc_asymrho(int device, double temperature, int nslice, int iodevn, int ith0, int ith1,
                                    const double *abc, int maxj, double *rho, double *erot, double *esq, double *info)
{
  const double boltz = 0.6950356, eps = 1.e-16;
  if (iodevn > 1 || iodevn < -1 || !abc || !rho || !erot || !esq || nslice < 1 || !(temperature > 0.0))
    return PIMC_ERR_BAD_ARG;
  if (ith0 < 0 || ith1 > 180 || ith1 < ith0 || maxj < 0) return PIMC_ERR_BAD_ARG;
  if (maxj > PIMC_ASYMRHO_MAXJ) return PIMC_ERR_SIZE;
  const double A = abc[0], Bc = abc[1], Cc = abc[2];
  double beta = 1.0 / (boltz * temperature), tau = beta / (double)nslice;
  const int M = 2 * maxj + 1;
  // eigen-decomposition of every (j, K-parity) block (asymrho.f:114-279) and
  // the weight matrices W^j (pre_j = (2j+1)/(8 pi^2), states with
  // e^{-tau E} pre_j < eps left out as asymrho.f:563 leaves them out)
  std::vector<int> woff(2 * (maxj + 1), 0);
  std::vector<double> W;
  std::vector<std::vector<double>> eng(2);
  double emax = -1e300;
  for (int j = 0; j <= maxj; j++) {
    double pre = (double)(2 * j + 1) / (8.0 * kPi * kPi);
    for (int par = 0; par < 2; par++) {
      int kst, nd;
      block_of(j, par, &kst, &nd);
      woff[2 * j + par] = (int)W.size();
      if (nd == 0) continue;
      std::vector<double> h((size_t)nd * nd), v, w;
      for (int r = 0; r < nd; r++)
        for (int c = 0; c < nd; c++) h[(size_t)r * nd + c] = rotmat(j, kst + 2 * r, kst + 2 * c, A, Bc, Cc);
      jacobi_eigen(nd, h, v, w);
      size_t o = W.size();
      W.resize(o + 3 * (size_t)nd * nd, 0.0);
      for (int n = 0; n < nd; n++) {
        double E = w[n];
        eng[par].push_back(E);
        emax = E > emax ? E : emax;
        double expo = exp(-tau * E);
        if (expo * pre < eps) continue;
        double f0 = pre * expo, f1 = f0 * E, f2 = f1 * E;
        for (int a = 0; a < nd; a++)
          for (int b = 0; b < nd; b++) {
            double cc = v[(size_t)a * nd + n] * v[(size_t)b * nd + n];
            W[o + (size_t)a * nd + b] += f0 * cc;
            W[o + (size_t)nd * nd + (size_t)a * nd + b] += f1 * cc;
            W[o + 2 * (size_t)nd * nd + (size_t)a * nd + b] += f2 * cc;
          }
      }
    }
  }
  // asymrho.f:295-297: the highest state must not matter
  if (exp(-beta * emax) > 1.e-8 || exp(-tau * emax) > 1.e-8) return PIMC_ERR_BAD_ARG;
  if (info) {   // "AT BETA" and "AT TAU" (asymrho.f:299-423)
    for (int pass = 0; pass < 2; pass++) {
      double bt = pass ? tau : beta;
      double zp[2] = {0, 0}, ea[2] = {0, 0}, es[2] = {0, 0};
      int ist[2] = {0, 0};
      for (int j = 0; j <= maxj; j++)
        for (int par = 0; par < 2; par++) {
          int kst, nd;
          block_of(j, par, &kst, &nd);
          double s0 = 0, s1 = 0, s2 = 0;
          for (int i = 0; i < nd; i++) {
            double E = eng[par][ist[par] + i];
            s0 = s0 + exp(-bt * E);
            s1 = s1 + E * exp(-bt * E);
            s2 = s2 + E * E * exp(-bt * E);
          }
          zp[par] = zp[par] + (2 * j + 1) * s0;
          ea[par] = ea[par] + (2 * j + 1) * s1;
          es[par] = es[par] + (2 * j + 1) * s2;
          ist[par] += nd;
        }
      double zc = zp[0] + zp[1], e0 = ea[0] / zp[0], e1 = ea[1] / zp[1], ec = (ea[0] + ea[1]) / zc;
      if (pass == 0) {
        double kt2 = boltz * boltz * temperature * temperature;
        info[0] = zp[0]; info[1] = e0; info[2] = (es[0] / zp[0] - e0 * e0) / kt2;
        info[3] = zp[1]; info[4] = e1; info[5] = (es[1] / zp[1] - e1 * e1) / kt2;
        info[6] = zc; info[7] = ec; info[8] = ((es[0] + es[1]) / zc - ec * ec) / kt2;
      } else {
        info[9] = zp[0]; info[10] = e0; info[11] = zp[1]; info[12] = e1; info[13] = zc; info[14] = ec;
      }
    }
  }
  std::vector<double> cosd(360), sind(360);
  for (int i = 0; i < 360; i++) {
    cosd[i] = cos((double)i * kPi / 180.0);
    sind[i] = sin((double)i * kPi / 180.0);
  }
  CKT(cudaSetDevice(device));
  cudaStream_t s;
  CKT(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  const int nth = ith1 - ith0 + 1, chunk = nth < 16 ? nth : 16;
  DevBuf db;
  int *dwoff = nullptr;
  double *dW = nullptr, *dA = nullptr, *dB = nullptr, *dC = nullptr, *dcos = nullptr, *dsin = nullptr;
  double *dr = nullptr, *de = nullptr, *ds = nullptr;
  const size_t slab = 361 * 361;
  pimc_status st = PIMC_OK;
  if (db.alloc(&dwoff, woff.size()) || db.alloc(&dW, W.size()) || db.alloc(&dA, (size_t)chunk * 3 * M * M) ||
      db.alloc(&dB, (size_t)chunk * 3 * M * 361) || db.alloc(&dC, (size_t)chunk * 3 * M * 361) ||
      db.alloc(&dcos, 360) || db.alloc(&dsin, 360) || db.alloc(&dr, chunk * slab) || db.alloc(&de, chunk * slab) ||
      db.alloc(&ds, chunk * slab))
    st = PIMC_ERR_CUDA;
  if (!st && (cudaMemcpyAsync(dwoff, woff.data(), woff.size() * sizeof(int), cudaMemcpyHostToDevice, s) ||
              cudaMemcpyAsync(dW, W.data(), W.size() * sizeof(double), cudaMemcpyHostToDevice, s) ||
              cudaMemcpyAsync(dcos, cosd.data(), 360 * sizeof(double), cudaMemcpyHostToDevice, s) ||
              cudaMemcpyAsync(dsin, sind.data(), 360 * sizeof(double), cudaMemcpyHostToDevice, s)))
    st = PIMC_ERR_CUDA;
  for (int t0 = 0; !st && t0 < nth; t0 += chunk) {
    int nc = nth - t0 < chunk ? nth - t0 : chunk;
    k_asym_coef<<<dim3((M * M + 127) / 128, nc), 128, 0, s>>>(maxj, ith0 + t0, dwoff, dW, dA);
    k_asym_chi<<<dim3(3 * M, nc), 384, 0, s>>>(maxj, dA, dcos, dsin, dB, dC);
    k_asym_grid<<<dim3(361, nc), 384, 0, s>>>(maxj, iodevn, dB, dC, dcos, dsin, dr, de, ds);
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpyAsync(rho + (size_t)t0 * slab, dr, nc * slab * sizeof(double), cudaMemcpyDeviceToHost, s) ||
        cudaMemcpyAsync(erot + (size_t)t0 * slab, de, nc * slab * sizeof(double), cudaMemcpyDeviceToHost, s) ||
        cudaMemcpyAsync(esq + (size_t)t0 * slab, ds, nc * slab * sizeof(double), cudaMemcpyDeviceToHost, s) ||
        cudaStreamSynchronize(s) != cudaSuccess)
      st = PIMC_ERR_CUDA;
  }
  cudaStreamSynchronize(s);
  cudaStreamDestroy(s);
  if (st) return st;
  // the symmetric copies of asymrho.f:636-709, in the reference's order
  double *tab[3] = {rho, erot, esq};
  for (int it = 0; it < nth; it++) {
    size_t b = (size_t)it * slab;
    auto copy = [&](int iphi, int ichi, int iphi0, int ichi0) {
      for (int q = 0; q < 3; q++) tab[q][b + (size_t)iphi * 361 + ichi] = tab[q][b + (size_t)iphi0 * 361 + ichi0];
    };
    for (int iphi = 90; iphi <= 180; iphi++)
      for (int ichi = 180 - iphi; ichi <= iphi; ichi++) copy(iphi, ichi, 180 - ichi, 180 - iphi);
    for (int iphi = 180; iphi <= 270; iphi++)
      for (int ichi = iphi - 180; ichi <= 360 - iphi; ichi++) copy(iphi, ichi, 180 + ichi, iphi - 180);
    for (int iphi = 180; iphi <= 360; iphi++)
      for (int ichi = 360 - iphi; ichi <= iphi; ichi++) copy(iphi, ichi, 360 - ichi, 360 - iphi);
    for (int iphi = 0; iphi <= 360; iphi++)
      for (int ichi = iphi; ichi <= 360; ichi++) copy(iphi, ichi, ichi, iphi);
  }
  return PIMC_OK;
}
