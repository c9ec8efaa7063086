// pimc_mlp.cu -- the rotor-rotor surrogate: an MLP 6 -> 256 -> 256 -> 256 -> 1
// (BF16 weights of the two 256x256 layers, FP32 accumulation) on the
// 5th-generation tensor cores.
//
// One CTA of 128 threads takes 128 configurations.  The hidden layers are
// one tcgen05.mma chain each (M = 128 rows, N = 256, K = 256 in sixteen K=16
// steps) issued by one thread from shared-memory operands in the canonical
// no-swizzle K-major layout, accumulating in 256 TMEM columns; the epilogue
// reads the accumulator back with tcgen05.ld (warp w owns TMEM lanes
// 32w..32w+31, i.e. its 32 rows), adds the bias, applies SiLU and writes the
// BF16 activations as the next layer's A operand.  The weights arrive by
// one bulk copy (cp.async.bulk) per layer, already in the B-operand layout.
// The 6 -> 256 and 256 -> 1 layers are FP32 on the CUDA cores.
#include <cstdint>
#include <cstring>
#include <vector>

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "../../include/pimc_gb300.h"

namespace {

constexpr int kRows = 128;            // configurations per CTA (MMA M)
constexpr int kH = 256;               // hidden width (MMA N and K)
constexpr int kIn = 6;                // input features
constexpr int kA = kRows * kH * 2;    // A operand bytes (BF16)
constexpr int kB = kH * kH * 2;       // B operand bytes
constexpr int kSmem = kA + kB + 1024; // + barriers and the TMEM address
constexpr long kSpin = 1L << 26;      // bounded waits

// byte offset of element (r, k) of a rows x 256 K-major BF16 operand in the
// canonical no-swizzle layout: 8x8 core matrices of 16-byte rows, core
// matrices adjacent along K (LBO = 128 B), 8-row groups 32 core matrices apart
// (SBO = 4096 B)
__host__ __device__ constexpr uint32_t canon(int r, int k)
{
  return (uint32_t)((r >> 3) * 4096 + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// shared-memory matrix descriptor (tcgen05): start address >> 4 in bits 0-13,
// leading byte offset >> 4 in 16-29, stride byte offset >> 4 in 32-45, the
// fixed 0b001 in 46-48, no swizzle (bits 61-63 = 0)
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr)
{
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
  d |= (uint64_t)(128 >> 4) << 16;
  d |= (uint64_t)(4096 >> 4) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// instruction descriptor, kind::f16: F32 accumulator (bits 4-5 = 1), BF16 A
// and B (bits 7-9, 10-12 = 1), both K-major, N >> 3 in bits 17-22, M >> 4 in
// bits 24-28
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N)
{
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count)
{
  asm volatile("mbarrier.init.shared.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ uint64_t gtimer()
{
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// bounded wait on phase `parity` (2 s of %globaltimer at most); returns false
// when it gave up
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity)
{
  const uint64_t t0 = gtimer();
  for (long i = 0; i < kSpin; i++) {
    if ((i & 255) == 255 && gtimer() - t0 > 2000000000ull) return false;
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.b32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// bytes (a multiple of 16 KB) from global to shared memory by bulk copies of
// 16 KB that complete on bar; one arrival with the whole transaction count
__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
  asm volatile(
      "{\n\t.reg .b64 st;\n\t"
      "mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(smem_u32(bar)),
      "r"(bytes)
      : "memory");
  const uint32_t chunk = 16384;
  for (uint32_t o = 0; o < bytes; o += chunk)
    asm volatile("cp.async.bulk.shared::cta.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32((char *)dst + o)),
                 "l"((const char *)src + o), "r"(chunk), "r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void umma(uint32_t tmem, uint64_t ad, uint64_t bd, uint32_t idesc, uint32_t acc)
{
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
      "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
      : "memory");
}

__device__ __forceinline__ void umma_commit(uint64_t *bar)
{
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float v[16])
{
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, "
      "[%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ float silu(float z) { return z / (1.0f + __expf(-z)); }

// D[128 x 256] (TMEM) = A[128 x 256] . B[256 x 256]^T from shared memory,
// sixteen K=16 steps issued by thread 0, completion on bar (phase `ph`)
__device__ __forceinline__ bool gemm_128x256(uint32_t tmem, const char *sA, const char *sB, uint64_t *bar,
                                             unsigned ph)
{
  if (threadIdx.x == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t id = idesc_bf16(kRows, kH);
    const uint32_t a0 = smem_u32(sA), b0 = smem_u32(sB);
    for (int k = 0; k < kH / 16; k++)      // one step = two core matrices along K
      umma(tmem, smem_desc(a0 + k * 256), smem_desc(b0 + k * 256), id, k > 0 ? 1u : 0u);
    umma_commit(bar);
  }
  bool ok = mbar_wait(bar, ph);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  return ok;
}

struct MlpParams {
  const float *w1, *b1;          // [6][256], [256]
  const char *w2c, *w3c;         // B operands: W^T in the canonical layout (BF16)
  const float *b2, *b3, *w4;     // [256] each
  float b4;
};

// y[n] = MLP(x[n][0..5]); one CTA per 128 rows; err[0] |= 1 when a wait gave up
__global__ void __launch_bounds__(kRows) k_mlp_forward(MlpParams p, const float *x, int n, float *y, unsigned *err)
{
  extern __shared__ __align__(1024) char smem[];
  char *sA = smem, *sB = smem + kA;
  uint64_t *bar_w = (uint64_t *)(smem + kA + kB);
  uint64_t *bar_m = bar_w + 1;
  uint32_t *tslot = (uint32_t *)(bar_w + 2);
  const int tid = threadIdx.x, warp = tid >> 5;
  const int row = blockIdx.x * kRows + tid;
  if (tid == 0) {
    mbar_init(bar_w, 1);
    mbar_init(bar_m, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)), "r"(kH)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tslot;
  const uint32_t tlane = tmem + ((uint32_t)(warp * 32) << 16);
  if (tid == 0) bulk_load(sB, p.w2c, kB, bar_w);
  // layer 1 on the CUDA cores, written as the A operand
  float xin[kIn];
  for (int i = 0; i < kIn; i++) xin[i] = row < n ? x[(size_t)row * kIn + i] : 0.0f;
  for (int j = 0; j < kH; j += 2) {
    float z0 = p.b1[j], z1 = p.b1[j + 1];
    for (int i = 0; i < kIn; i++) {
      z0 = fmaf(xin[i], p.w1[i * kH + j], z0);
      z1 = fmaf(xin[i], p.w1[i * kH + j + 1], z1);
    }
    *(__nv_bfloat162 *)(sA + canon(tid, j)) = __floats2bfloat162_rn(silu(z0), silu(z1));
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  __syncthreads();
  bool ok = mbar_wait(bar_w, 0);
  unsigned ph = 0;
  float out = p.b4;
  for (int layer = 0; layer < 2 && ok; layer++) {
    ok = gemm_128x256(tmem, sA, sB, bar_m, ph);
    ph ^= 1u;
    __syncthreads();                                   // every thread saw the MMAs complete
    if (layer == 0 && tid == 0) bulk_load(sB, p.w3c, kB, bar_w);
    const float *bias = layer == 0 ? p.b2 : p.b3;
    for (int c = 0; c < kH; c += 16) {
      float v[16];
      tmem_ld16(tlane + c, v);
      if (layer == 0) {
#pragma unroll
        for (int i = 0; i < 16; i += 2)
          *(__nv_bfloat162 *)(sA + canon(tid, c + i)) =
              __floats2bfloat162_rn(silu(v[i] + bias[c + i]), silu(v[i + 1] + bias[c + i + 1]));
      } else {
#pragma unroll
        for (int i = 0; i < 16; i++) out = fmaf(silu(v[i] + bias[c + i]), p.w4[c + i], out);
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (layer == 0) ok = ok && mbar_wait(bar_w, 1);
  }
  if (!ok && tid == 0) atomicOr(err, 1u);
  if (row < n) y[row] = out;
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kH) : "memory");
}

}  // namespace

// ------------------------------------------------------------------ host

struct pimc_mlp {
  int device = 0;
  cudaStream_t stream = nullptr;
  float *w1 = nullptr, *b1 = nullptr, *b2 = nullptr, *b3 = nullptr, *w4 = nullptr;
  char *w2c = nullptr, *w3c = nullptr;
  float b4 = 0.0f;
  unsigned *err = nullptr;
  float *xbuf = nullptr, *ybuf = nullptr;
  size_t cap = 0;
};

#define MCK(x)                                  \
  do {                                          \
    if ((x) != cudaSuccess) return PIMC_ERR_CUDA; \
  } while (0)

static void to_canon(const float *w, std::vector<uint16_t> &out)
{
  // B operand of y = h . W: element (n, k) = W[k][n], K-major canonical
  out.assign((size_t)kH * kH, 0);
  for (int nn = 0; nn < kH; nn++)
    for (int k = 0; k < kH; k++) {
      __nv_bfloat16 b = __float2bfloat16_rn(w[(size_t)k * kH + nn]);
      uint16_t bits;
      memcpy(&bits, &b, 2);
      out[canon(nn, k) / 2] = bits;
    }
}

extern "C" pimc_status pimc_mlp_create(int device, pimc_mlp **out)
{
  if (!out) return PIMC_ERR_BAD_ARG;
  int nd = 0;
  if (cudaGetDeviceCount(&nd) != cudaSuccess || nd <= device) return PIMC_ERR_NO_DEVICE;
  pimc_mlp *m = new (std::nothrow) pimc_mlp();
  if (!m) return PIMC_ERR_BAD_ARG;
  m->device = device;
  MCK(cudaSetDevice(device));
  MCK(cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking));
  MCK(cudaMalloc(&m->w1, kIn * kH * sizeof(float)));
  MCK(cudaMalloc(&m->b1, kH * sizeof(float)));
  MCK(cudaMalloc(&m->b2, kH * sizeof(float)));
  MCK(cudaMalloc(&m->b3, kH * sizeof(float)));
  MCK(cudaMalloc(&m->w4, kH * sizeof(float)));
  MCK(cudaMalloc(&m->w2c, kB));
  MCK(cudaMalloc(&m->w3c, kB));
  MCK(cudaMalloc(&m->err, sizeof(unsigned)));
  MCK(cudaMemset(m->err, 0, sizeof(unsigned)));
  MCK(cudaFuncSetAttribute(k_mlp_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmem));
  *out = m;
  return PIMC_OK;
}

extern "C" pimc_status pimc_mlp_destroy(pimc_mlp *m)
{
  if (!m) return PIMC_ERR_BAD_ARG;
  cudaSetDevice(m->device);
  if (m->stream) cudaStreamSynchronize(m->stream);
  void *b[] = {m->w1, m->b1, m->b2, m->b3, m->w4, m->w2c, m->w3c, m->err, m->xbuf, m->ybuf};
  for (void *p : b)
    if (p) cudaFree(p);
  if (m->stream) cudaStreamDestroy(m->stream);
  delete m;
  return PIMC_OK;
}

extern "C" pimc_status pimc_mlp_set_weights(pimc_mlp *m, const float *w1, const float *b1, const float *w2,
                                            const float *b2, const float *w3, const float *b3, const float *w4,
                                            float b4)
{
  if (!m || !w1 || !b1 || !w2 || !b2 || !w3 || !b3 || !w4) return PIMC_ERR_BAD_ARG;
  MCK(cudaSetDevice(m->device));
  std::vector<uint16_t> c2, c3;
  to_canon(w2, c2);
  to_canon(w3, c3);
  MCK(cudaMemcpy(m->w1, w1, kIn * kH * sizeof(float), cudaMemcpyHostToDevice));
  MCK(cudaMemcpy(m->b1, b1, kH * sizeof(float), cudaMemcpyHostToDevice));
  MCK(cudaMemcpy(m->b2, b2, kH * sizeof(float), cudaMemcpyHostToDevice));
  MCK(cudaMemcpy(m->b3, b3, kH * sizeof(float), cudaMemcpyHostToDevice));
  MCK(cudaMemcpy(m->w4, w4, kH * sizeof(float), cudaMemcpyHostToDevice));
  MCK(cudaMemcpy(m->w2c, c2.data(), kB, cudaMemcpyHostToDevice));
  MCK(cudaMemcpy(m->w3c, c3.data(), kB, cudaMemcpyHostToDevice));
  m->b4 = b4;
  return PIMC_OK;
}

extern "C" pimc_status pimc_mlp_forward(pimc_mlp *m, int n, const float *x, float *y)
{
  if (!m || n < 0 || (n && (!x || !y))) return PIMC_ERR_BAD_ARG;
  if (n == 0) return PIMC_OK;
  MCK(cudaSetDevice(m->device));
  if ((size_t)n > m->cap) {
    if (m->xbuf) cudaFree(m->xbuf);
    if (m->ybuf) cudaFree(m->ybuf);
    m->xbuf = m->ybuf = nullptr;
    MCK(cudaMalloc(&m->xbuf, (size_t)n * kIn * sizeof(float)));
    MCK(cudaMalloc(&m->ybuf, (size_t)n * sizeof(float)));
    m->cap = (size_t)n;
  }
  MCK(cudaMemcpyAsync(m->xbuf, x, (size_t)n * kIn * sizeof(float), cudaMemcpyHostToDevice, m->stream));
  MlpParams p{m->w1, m->b1, m->w2c, m->w3c, m->b2, m->b3, m->w4, m->b4};
  k_mlp_forward<<<(n + kRows - 1) / kRows, kRows, kSmem, m->stream>>>(p, m->xbuf, n, m->ybuf, m->err);
  MCK(cudaGetLastError());
  MCK(cudaMemcpyAsync(y, m->ybuf, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost, m->stream));
  MCK(cudaStreamSynchronize(m->stream));
  unsigned e = 0;
  MCK(cudaMemcpy(&e, m->err, sizeof(unsigned), cudaMemcpyDeviceToHost));
  if (e) {
    cudaMemset(m->err, 0, sizeof(unsigned));
    return PIMC_ERR_TIMEOUT;
  }
  return PIMC_OK;
}
