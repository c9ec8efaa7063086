// pimc_stats.cu -- standard error of a correlated Monte Carlo average (host
// only).  The reference leaves the error analysis of its block averages to
// the user (SaveEnergy writes one .eng row per block, mc_main.cc:764-795);
// the time-to-matched-error measurement needs it in the library, applied to
// the energy series a run produces.
//
// Blocking analysis (Flyvbjerg and Petersen, J. Chem. Phys. 91, 461 (1989))
// with the automatic choice of the blocking level of Jonsson, Phys. Rev. E
// 98, 043304 (2018): the series is halved by averaging neighbouring pairs,
// level after level; at level i (n_i values, variance s_i with 1/n_i,
// lag-one autocovariance g_i) the statistic M_j = sum_{i >= j} n_i (g_i /
// s_i)^2 is chi-squared with d - j degrees of freedom when the blocks of
// level j are uncorrelated, and the first level with M_j below the 99 %
// quantile is taken; the error is then sqrt(s_j / n_j).
#include <math.h>
#include <string.h>

#include <vector>

#include "../../include/pimc_gb300.h"

namespace {

// 99 % quantiles of the chi-squared distribution, 1 .. 40 degrees of freedom
const double kChi2q99[40] = {
    6.634897,  9.210340,  11.344867, 13.276704, 15.086272, 16.811894, 18.475307, 20.090235, 21.665994, 23.209251,
    24.724970, 26.216967, 27.688250, 29.141238, 30.577914, 31.999927, 33.408664, 34.805306, 36.190869, 37.566235,
    38.932173, 40.289360, 41.638398, 42.979820, 44.314105, 45.641683, 46.962942, 48.278236, 49.587884, 50.892181,
    52.191395, 53.485772, 54.775540, 56.060909, 57.342073, 58.619215, 59.892500, 61.162087, 62.428121, 63.690740};

}  // namespace

extern "C" pimc_status pimc_blocking_se(const double *x, long n, double *out)
{
  if (!x || !out || n < 16) return PIMC_ERR_BAD_ARG;
  for (long i = 0; i < n; i++)
    if (!isfinite(x[i])) return PIMC_ERR_BAD_ARG;
  int d = 0;
  while (d < 40 && (2L << d) <= n) d++;          // 2^d <= n < 2^(d+1)
  const long n2 = 1L << d;
  // the last 2^d values: the start of a run is the part most likely to carry
  // equilibration
  std::vector<double> b(x + (n - n2), x + n);
  double mu = 0.0;
  for (double v : b) mu += v;
  mu /= (double)n2;
  std::vector<double> s(d), g(d);
  long m = n2;
  for (int i = 0; i < d; i++) {
    double ss = 0.0, gg = 0.0;
    for (long k = 0; k < m; k++) ss += (b[k] - mu) * (b[k] - mu);
    for (long k = 0; k + 1 < m; k++) gg += (b[k] - mu) * (b[k + 1] - mu);
    s[i] = ss / (double)m;
    g[i] = gg / (double)m;
    for (long k = 0; k < m / 2; k++) b[k] = 0.5 * (b[2 * k] + b[2 * k + 1]);
    m /= 2;
  }
  // M_j from the top level down
  std::vector<double> M(d);
  double acc = 0.0;
  for (int i = d - 1; i >= 0; i--) {
    double ni = (double)(n2 >> i);
    double r = s[i] > 0.0 ? g[i] / s[i] : 0.0;
    acc += ni * r * r;
    M[i] = acc;
  }
  int level = d - 1, found = 0;
  for (int j = 0; j < d; j++)
    if (M[j] < kChi2q99[d - j - 1]) { level = j; found = 1; break; }
  const double nj = (double)(n2 >> level);
  const double se = sqrt(s[level] / nj);
  const double se0 = sqrt(s[0] / (double)n2);
  out[0] = mu;
  out[1] = sqrt(s[0] * (double)n2 / (double)(n2 - 1));
  out[2] = se0;
  out[3] = se;
  out[4] = se0 > 0.0 ? (se * se) / (se0 * se0) : 1.0;
  out[5] = (double)(1L << level);
  out[6] = (double)found;
  out[7] = (double)n2;
  return PIMC_OK;
}

// ---- the FP64 roofline denominator: a dependent-FMA throughput kernel.
// Eight independent chains per thread keep the FP64 pipe's latency hidden;
// every thread's result is stored so that nothing is eliminated.
namespace {
__global__ void __launch_bounds__(1024) k_fp64_fma(double *out, int iters, double a, double b, int lanes)
{
  if ((int)(threadIdx.x & 31) >= lanes) return;
  double x[8];
  for (int k = 0; k < 8; k++) x[k] = 1.0 + 1e-3 * (double)(threadIdx.x + k);
  for (int i = 0; i < iters; i++)
#pragma unroll
    for (int k = 0; k < 8; k++) x[k] = fma(x[k], a, b);
  double s = 0.0;
  for (int k = 0; k < 8; k++) s += x[k];
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}
}  // namespace

extern "C" pimc_status pimc_fp64_peak(int device, double *gflops)
{
  if (!gflops) return PIMC_ERR_BAD_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return PIMC_ERR_NO_DEVICE;
  int nsm = 0;
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return PIMC_ERR_CUDA;
  const int blocks = nsm * 8, threads = 256, iters = 8192;
  double *out = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  pimc_status st = PIMC_OK;
  float ms = 0.0f;
  if (cudaMalloc(&out, (size_t)blocks * threads * sizeof(double)) != cudaSuccess) return PIMC_ERR_CUDA;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) { st = PIMC_ERR_CUDA; goto done; }
  k_fp64_fma<<<blocks, threads>>>(out, iters / 8, 0.9999999, 1e-7, 32);       // warm-up
  cudaEventRecord(e0);
  k_fp64_fma<<<blocks, threads>>>(out, iters, 0.9999999, 1e-7, 32);
  cudaEventRecord(e1);
  if (cudaEventSynchronize(e1) != cudaSuccess || cudaGetLastError() != cudaSuccess ||
      cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess || ms <= 0.0f) {
    st = PIMC_ERR_CUDA;
    goto done;
  }
  *gflops = 2.0 * 8.0 * (double)iters * (double)blocks * (double)threads / ((double)ms * 1e-3) / 1e9;
done:
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(out);
  return st;
}

extern "C" pimc_status pimc_fp64_probe(int device, int warps, int lanes, int iters, double *ms_out)
{
  if (!ms_out || warps < 1 || warps > 32 || lanes < 1 || lanes > 32 || iters < 1 || iters > (1 << 24))
    return PIMC_ERR_BAD_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return PIMC_ERR_NO_DEVICE;
  int nsm = 0;
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return PIMC_ERR_CUDA;
  const int threads = 32 * warps;
  double *out = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  pimc_status st = PIMC_OK;
  float ms = 0.0f;
  if (cudaMalloc(&out, (size_t)nsm * threads * sizeof(double)) != cudaSuccess) return PIMC_ERR_CUDA;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) { st = PIMC_ERR_CUDA; goto done; }
  k_fp64_fma<<<nsm, threads>>>(out, iters / 8 + 1, 0.9999999, 1e-7, lanes);      // warm-up
  cudaEventRecord(e0);
  k_fp64_fma<<<nsm, threads>>>(out, iters, 0.9999999, 1e-7, lanes);
  cudaEventRecord(e1);
  if (cudaEventSynchronize(e1) != cudaSuccess || cudaGetLastError() != cudaSuccess ||
      cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess || ms <= 0.0f) {
    st = PIMC_ERR_CUDA;
    goto done;
  }
  *ms_out = (double)ms;
done:
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(out);
  return st;
}
