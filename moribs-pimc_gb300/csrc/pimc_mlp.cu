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
#include <atomic>
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
constexpr int kW1B = (kIn + 1) * kH * 4;   // W1 and b1 (contiguous parameters), FP32
constexpr int kVecB = 3 * kH * 4;           // b2, then b3 and w4 (contiguous), FP32
// + barriers, the TMEM address, the half sums, then W1, b1, b2, b3, w4
constexpr int kSmem = kA + kB + 2048 + kW1B + kVecB;
// + the column-sum buffer of the training kernel, then W1, b1, b2, b3, w4
constexpr int kSmemT = kA + kB + 8192 + (kIn + 1) * kH * 4 + 3 * kH * 4;
// the parameter vector: w1[6][256], b1, w2[256][256], b2, w3[256][256], b3, w4, b4
constexpr int kOW1 = 0, kOB1 = kOW1 + kIn * kH, kOW2 = kOB1 + kH, kOB2 = kOW2 + kH * kH, kOW3 = kOB2 + kH,
              kOB3 = kOW3 + kH * kH, kOW4 = kOB3 + kH, kOB4 = kOW4 + kH, kNP = kOB4 + 1;
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
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t sbo = 4096)
{
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
  d |= (uint64_t)(128 >> 4) << 16;
  d |= (uint64_t)(sbo >> 4) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// element (r, k) of a K = 128 operand (the batch as the reduction index of a
// weight gradient): 8-row groups 16 core matrices apart (SBO = 2048 B)
__host__ __device__ constexpr uint32_t canon128(int r, int k)
{
  return (uint32_t)((r >> 3) * 2048 + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
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
// one arrival on bar announcing `bytes` of copies to come
__device__ __forceinline__ void bulk_expect(uint64_t *bar, uint32_t bytes)
{
  asm volatile(
      "{\n\t.reg .b64 st;\n\t"
      "mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(smem_u32(bar)),
      "r"(bytes)
      : "memory");
}

// one cp.async.bulk of `bytes` (a multiple of 16) completing on bar, whose
// bytes an earlier bulk_expect announced
__device__ __forceinline__ void bulk_copy(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
  asm volatile("cp.async.bulk.shared::cta.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

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

// SiLU and its derivative with the fast exponential and division (the
// surrogate is BF16 throughout; 2-ulp FP32 activations are far below that)
__device__ __forceinline__ float silu(float z) { return __fdividef(z, 1.0f + __expf(-z)); }

// eight BF16 values (round to nearest even) as one 16-byte shared store
__device__ __forceinline__ void store8(char *dst, float a, float b, float c, float d, float e, float f, float g,
                                       float h)
{
  __nv_bfloat162 q0 = __floats2bfloat162_rn(a, b), q1 = __floats2bfloat162_rn(c, d);
  __nv_bfloat162 q2 = __floats2bfloat162_rn(e, f), q3 = __floats2bfloat162_rn(g, h);
  uint4 u;
  u.x = *(uint32_t *)&q0;
  u.y = *(uint32_t *)&q1;
  u.z = *(uint32_t *)&q2;
  u.w = *(uint32_t *)&q3;
  *(uint4 *)dst = u;
}

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
  const float *b4;
};

// y[n] = MLP(x[n][0..5]); one CTA of 256 threads per 128 rows: thread t
// serves row t % 128 (TMEM lane quarter of its warp) and column half t / 128
// of the CUDA-core layers and epilogues; err[0] |= 1 when a wait gave up
constexpr int kFwdThreads = 256;

__global__ void __launch_bounds__(kFwdThreads) k_mlp_forward(MlpParams p, const float *x, int n, float *y,
                                                             unsigned *err)
{
  extern __shared__ __align__(1024) char smem[];
  char *sA = smem, *sB = smem + kA;
  uint64_t *bar_w = (uint64_t *)(smem + kA + kB);
  uint64_t *bar_m = bar_w + 1;
  uint32_t *tslot = (uint32_t *)(bar_w + 2);
  uint64_t *bar_x = bar_w + 3;                            // the copies of W1 and the vectors
  float *outp = (float *)(smem + kA + kB + 64);          // [256] half sums of the last layer
  float *sw1 = (float *)(smem + kA + kB + 2048), *sb1 = sw1 + kIn * kH;
  float *sb2 = sb1 + kH, *sb3 = sb2 + kH, *sw4 = sb3 + kH;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int r = tid & (kRows - 1), half = tid >> 7, c0 = half * (kH / 2);
  const int row = blockIdx.x * kRows + r;
  // the row's inputs and the weight copies are in flight while TMEM is
  // allocated; W1 and the bias and output vectors (10 KB) on their own
  // barrier, so that the first layer does not wait for W2
  float xin[kIn];
  for (int i = 0; i < kIn; i++) xin[i] = row < n ? x[(size_t)row * kIn + i] : 0.0f;
  if (tid == 0) {
    mbar_init(bar_w, 1);
    mbar_init(bar_m, 1);
    mbar_init(bar_x, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    bulk_expect(bar_x, kW1B + kVecB);
    bulk_copy(sw1, p.w1, kW1B, bar_x);                    // W1, b1
    bulk_copy(sb2, p.b2, kH * 4, bar_x);
    bulk_copy(sb3, p.b3, 2 * kH * 4, bar_x);              // b3, w4
    bulk_load(sB, p.w2c, kB, bar_w);
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
  const uint32_t tlane = tmem + ((uint32_t)((warp & 3) * 32) << 16);
  // layer 1 on the CUDA cores, written as the A operand: eight columns of a
  // row are one 16-byte run of the canonical layout, stored at once
  bool ok = __syncthreads_and(mbar_wait(bar_x, 0));
  for (int j = c0; j < c0 + kH / 2 && ok; j += 8) {
    float z[8];
    const float4 b0 = *(const float4 *)(sb1 + j), b1 = *(const float4 *)(sb1 + j + 4);
    z[0] = b0.x; z[1] = b0.y; z[2] = b0.z; z[3] = b0.w;
    z[4] = b1.x; z[5] = b1.y; z[6] = b1.z; z[7] = b1.w;
#pragma unroll
    for (int i = 0; i < kIn; i++) {
      const float4 w0 = *(const float4 *)(sw1 + i * kH + j), w1 = *(const float4 *)(sw1 + i * kH + j + 4);
      z[0] = fmaf(xin[i], w0.x, z[0]); z[1] = fmaf(xin[i], w0.y, z[1]);
      z[2] = fmaf(xin[i], w0.z, z[2]); z[3] = fmaf(xin[i], w0.w, z[3]);
      z[4] = fmaf(xin[i], w1.x, z[4]); z[5] = fmaf(xin[i], w1.y, z[5]);
      z[6] = fmaf(xin[i], w1.z, z[6]); z[7] = fmaf(xin[i], w1.w, z[7]);
    }
    store8(sA + canon(r, j), silu(z[0]), silu(z[1]), silu(z[2]), silu(z[3]), silu(z[4]), silu(z[5]), silu(z[6]),
           silu(z[7]));
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  ok = __syncthreads_and(mbar_wait(bar_w, 0)) && ok;
  unsigned ph = 0;
  float out = 0.0f;
  bool w3_sent = false;
  int nmma = 0;
  for (int layer = 0; layer < 2 && ok; layer++) {
    ok = __syncthreads_and(gemm_128x256(tmem, sA, sB, bar_m, ph));   // every thread saw the MMAs complete
    ph ^= 1u;
    nmma++;
    if (!ok) break;
    if (layer == 0 && tid == 0) bulk_load(sB, p.w3c, kB, bar_w);
    if (layer == 0) w3_sent = true;
    const float *bias = layer == 0 ? sb2 : sb3;
    for (int c = c0; c < c0 + kH / 2; c += 16) {
      float v[16], bb[16];
      tmem_ld16(tlane + c, v);
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const float4 t = *((const float4 *)(bias + c) + q);
        bb[4 * q] = t.x; bb[4 * q + 1] = t.y; bb[4 * q + 2] = t.z; bb[4 * q + 3] = t.w;
      }
      if (layer == 0) {
#pragma unroll
        for (int i = 0; i < 16; i += 8)
          store8(sA + canon(r, c + i), silu(v[i] + bb[i]), silu(v[i + 1] + bb[i + 1]), silu(v[i + 2] + bb[i + 2]),
                 silu(v[i + 3] + bb[i + 3]), silu(v[i + 4] + bb[i + 4]), silu(v[i + 5] + bb[i + 5]),
                 silu(v[i + 6] + bb[i + 6]), silu(v[i + 7] + bb[i + 7]));
      } else {
        float ww[16];
#pragma unroll
        for (int q = 0; q < 4; q++) {
          const float4 t = *((const float4 *)(sw4 + c) + q);
          ww[4 * q] = t.x; ww[4 * q + 1] = t.y; ww[4 * q + 2] = t.z; ww[4 * q + 3] = t.w;
        }
#pragma unroll
        for (int i = 0; i < 16; i++) out = fmaf(silu(v[i] + bb[i]), ww[i], out);
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    if (layer == 0) ok = __syncthreads_and(mbar_wait(bar_w, 1));
  }
  if (!ok) {
    // a wait gave up (ok is uniform over the CTA): let the copies and the
    // MMAs that may still be in flight land, each with a bounded wait,
    // before this CTA's shared memory and TMEM are released
    // (only the last phase issued on each barrier: phases complete in order)
    if (tid == 0) atomicOr(err, 1u);
    mbar_wait(bar_x, 0);
    mbar_wait(bar_w, w3_sent ? 1u : 0u);
    if (nmma > 0) mbar_wait(bar_m, (unsigned)(nmma - 1) & 1u);
    __syncthreads();
  }
  outp[tid] = out;
  __syncthreads();
  if (half == 0 && row < n) y[row] = (outp[r] + outp[r + kRows]) + *p.b4;
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kH) : "memory");
}

// ------------------------------------------------------------- training
// D(tmem) = A[128 x K] . B[256 x K]^T, both K-major canonical with SBO =
// 16 K bytes; issued by thread 0, completion on bar (phase ph)
__device__ __forceinline__ bool gemm_k(uint32_t tmem, const char *sA, const char *sB, int K, uint64_t *bar, unsigned ph)
{
  if (threadIdx.x == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t id = idesc_bf16(kRows, kH), sbo = (uint32_t)K * 16;
    const uint32_t a0 = smem_u32(sA), b0 = smem_u32(sB);
    for (int k = 0; k < K / 16; k++) umma(tmem, smem_desc(a0 + k * 256, sbo), smem_desc(b0 + k * 256, sbo), id, k > 0);
    umma_commit(bar);
  }
  bool ok = mbar_wait(bar, ph);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  return ok;
}

// two M tiles of a weight gradient, D0 = A0 . B^T at tmem, D1 = A1 . B^T at tmem + 256
__device__ __forceinline__ bool gemm_dw(uint32_t tmem, const char *sA, const char *sB, uint64_t *bar, unsigned ph)
{
  if (threadIdx.x == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t id = idesc_bf16(kRows, kH);
    const uint32_t a0 = smem_u32(sA), b0 = smem_u32(sB);
    for (int t = 0; t < 2; t++)
      for (int k = 0; k < kRows / 16; k++)
        umma(tmem + 256 * t, smem_desc(a0 + t * 32768 + k * 256, 2048), smem_desc(b0 + k * 256, 2048), id, k > 0);
    umma_commit(bar);
  }
  bool ok = mbar_wait(bar, ph);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  return ok;
}

__device__ __forceinline__ float dsilu(float z)
{
  float s = __fdividef(1.0f, 1.0f + __expf(-z));
  return s * (1.0f + z * (1.0f - s));
}

struct MlpTrainParams {
  MlpParams w;
  const char *w2n, *w3n;       // W in the canonical layout of the B operand of dh = dz . W^T
  const float *x, *e;          // inputs [n][6], targets [n]
  int n;
  float gscale;                // d loss / d y = gscale * (y - e)
  // per-CTA scratch and partial gradients
  char *h1t, *h2t, *dzt;       // [cta][64 KB] each: h1^T, h2^T, dz^T (K = 128 canonical)
  float *z2;                   // [cta][256][128]: pre-activations of layer 2, column-major
  float *part;                 // [cta][kNP] partial gradients in the parameter order
  float *loss;                 // [cta]
};

// the weight gradient tile pair in TMEM (rows of warp w: features 32w.. and
// 128+32w..) to the CTA's partial gW[in][out]
__device__ __forceinline__ void store_dw(uint32_t tlane, float *gw)
{
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int t = 0; t < 2; t++) {
    const int fin = t * 128 + warp * 32 + lane;
    for (int c = 0; c < kH; c += 16) {
      float v[16];
      tmem_ld16(tlane + 256 * t + c, v);
#pragma unroll
      for (int i = 0; i < 16; i++) gw[(size_t)fin * kH + c + i] = v[i];
    }
  }
}

// per-column sum over the CTA's 128 rows: warp shuffles, then the four warps
// in order through red[4][256]; column j's total lands in out[j]
__device__ __forceinline__ void col_sum16(float v[16], int c, float *red)
{
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
  for (int i = 0; i < 16; i++) {
    float a = v[i];
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    if (lane == 0) red[warp * kH + c + i] = a;
  }
}

// One CTA = 128 samples: the forward pass saving what the backward pass
// needs, then the backward pass with the four 256-wide products on the
// tensor cores (dW3 = h2^T dz3, dh2 = dz3 W3^T, dW2 = h1^T dz2,
// dh1 = dz2 W2^T) and the rest on the CUDA cores; partial gradients per CTA.
__global__ void __launch_bounds__(kRows) k_mlp_train(MlpTrainParams p, unsigned *err)
{
  extern __shared__ __align__(1024) char smem[];
  char *sA = smem, *sB = smem + kA;
  uint64_t *bar_w = (uint64_t *)(smem + kA + kB);
  uint64_t *bar_m = bar_w + 1;
  uint32_t *tslot = (uint32_t *)(bar_w + 2);
  float *red = (float *)(smem + kA + kB + 64);          // [4][256]
  uint64_t *bar_x = bar_w + 3;                          // the copies of W1 and the vectors
  float *sw1 = (float *)(smem + kA + kB + 8192), *sb1 = sw1 + kIn * kH;
  float *sb2 = sb1 + kH, *sb3 = sb2 + kH, *sw4 = sb3 + kH;
  const int tid = threadIdx.x, warp = tid >> 5, cta = blockIdx.x;
  const int row = cta * kRows + tid;
  const bool live = row < p.n;
  char *h1t = p.h1t + (size_t)cta * 65536, *h2t = p.h2t + (size_t)cta * 65536, *dzt = p.dzt + (size_t)cta * 65536;
  float *z2g = p.z2 + (size_t)cta * kRows * kH;
  if (tid == 0) {
    mbar_init(bar_w, 1);
    mbar_init(bar_m, 1);
    mbar_init(bar_x, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    bulk_expect(bar_x, (kIn + 1) * kH * 4 + 3 * kH * 4);
    bulk_copy(sw1, p.w.w1, (kIn + 1) * kH * 4, bar_x);    // W1, b1
    bulk_copy(sb2, p.w.b2, kH * 4, bar_x);
    bulk_copy(sb3, p.w.b3, 2 * kH * 4, bar_x);            // b3, w4
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)), "r"(512)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tslot, tlane = tmem + ((uint32_t)(warp * 32) << 16);
  unsigned pw = 0, pm = 0, w_last = 0, m_last = 0;
  int nload = 0, nmma = 0;
  // ok stays uniform over the CTA; after a wait gives up nothing more is
  // issued, so the last copy / MMA issued is the only one still in flight
  bool ok = __syncthreads_and(mbar_wait(bar_x, 0));
  auto load_b = [&](const char *src, uint32_t bytes, char *dst) {
    if (!ok) return;
    if (tid == 0) bulk_load(dst, src, bytes, bar_w);
    ok = __syncthreads_and(mbar_wait(bar_w, pw));
    w_last = pw;
    nload++;
    pw ^= 1u;
  };
  auto mma_done = [&](bool issued_ok) {
    ok = __syncthreads_and(issued_ok);
    m_last = pm;
    nmma++;
    pm ^= 1u;
  };
  auto sync_async = [&]() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    asm volatile("fence.proxy.async;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  };
  // ---- forward: layer 1 (h1 as A operand and h1^T for dW2)
  float xin[kIn];
  for (int i = 0; i < kIn; i++) xin[i] = live ? p.x[(size_t)row * kIn + i] : 0.0f;
  const float ey = live ? p.e[row] : 0.0f;
  for (int j = 0; j < kH; j += 2) {
    float z0 = sb1[j], z1 = sb1[j + 1];
    for (int i = 0; i < kIn; i++) {
      z0 = fmaf(xin[i], sw1[i * kH + j], z0);
      z1 = fmaf(xin[i], sw1[i * kH + j + 1], z1);
    }
    __nv_bfloat162 h = __floats2bfloat162_rn(silu(z0), silu(z1));
    *(__nv_bfloat162 *)(sA + canon(tid, j)) = h;
    *(__nv_bfloat16 *)(h1t + canon128(j, tid)) = h.x;
    *(__nv_bfloat16 *)(h1t + canon128(j + 1, tid)) = h.y;
  }
  sync_async();
  load_b(p.w.w2c, kB, sB);
  // ---- layer 2: z2 saved, h2 as A operand and h2^T
  if (ok) mma_done(gemm_k(tmem, sA, sB, kH, bar_m, pm));
  __syncthreads();
  for (int c = 0; c < kH; c += 16) {
    float v[16];
    tmem_ld16(tlane + c, v);
#pragma unroll
    for (int i = 0; i < 16; i += 2) {
      float za = v[i] + sb2[c + i], zb = v[i + 1] + sb2[c + i + 1];
      z2g[(size_t)(c + i) * kRows + tid] = za;             // column-major: a warp's rows are contiguous
      z2g[(size_t)(c + i + 1) * kRows + tid] = zb;
      __nv_bfloat162 h = __floats2bfloat162_rn(silu(za), silu(zb));
      *(__nv_bfloat162 *)(sA + canon(tid, c + i)) = h;
      *(__nv_bfloat16 *)(h2t + canon128(c + i, tid)) = h.x;
      *(__nv_bfloat16 *)(h2t + canon128(c + i + 1, tid)) = h.y;
    }
  }
  sync_async();
  load_b(p.w.w3c, kB, sB);
  // ---- layer 3 and the output
  if (ok) mma_done(gemm_k(tmem, sA, sB, kH, bar_m, pm));
  __syncthreads();
  float y = *p.w.b4;
  for (int c = 0; c < kH; c += 16) {
    float v[16];
    tmem_ld16(tlane + c, v);
#pragma unroll
    for (int i = 0; i < 16; i++) y = fmaf(silu(v[i] + sb3[c + i]), sw4[c + i], y);
  }
  const float dy = live ? p.gscale * (y - ey) : 0.0f;
  // loss, db4
  {
    float l = live ? (y - ey) * (y - ey) : 0.0f, d = dy;
    for (int o = 16; o > 0; o >>= 1) {
      l += __shfl_xor_sync(0xffffffffu, l, o);
      d += __shfl_xor_sync(0xffffffffu, d, o);
    }
    if ((tid & 31) == 0) { red[warp] = l; red[4 + warp] = d; }
    __syncthreads();
    if (tid == 0) {
      p.loss[cta] = red[0] + red[1] + red[2] + red[3];
      p.part[(size_t)cta * kNP + kOB4] = red[4] + red[5] + red[6] + red[7];
    }
    __syncthreads();
  }
  // dW4, db3 and dz3 (A operand for dh2, dz3^T for dW3)
  for (int c = 0; c < kH; c += 16) {
    float v[16], h3[16], dz[16];
    tmem_ld16(tlane + c, v);
#pragma unroll
    for (int i = 0; i < 16; i++) {
      float z = v[i] + sb3[c + i];
      h3[i] = silu(z) * dy;
      dz[i] = dy * sw4[c + i] * dsilu(z);
    }
    col_sum16(h3, c, red);
    __syncthreads();
    if (tid < 16) p.part[(size_t)cta * kNP + kOW4 + c + tid] = red[c + tid] + red[kH + c + tid] + red[2 * kH + c + tid] + red[3 * kH + c + tid];
    __syncthreads();
    col_sum16(dz, c, red);
    __syncthreads();
    if (tid < 16) p.part[(size_t)cta * kNP + kOB3 + c + tid] = red[c + tid] + red[kH + c + tid] + red[2 * kH + c + tid] + red[3 * kH + c + tid];
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 16; i += 2) {
      __nv_bfloat162 h = __floats2bfloat162_rn(dz[i], dz[i + 1]);
      *(__nv_bfloat162 *)(sA + canon(tid, c + i)) = h;
      *(__nv_bfloat16 *)(dzt + canon128(c + i, tid)) = h.x;
      *(__nv_bfloat16 *)(dzt + canon128(c + i + 1, tid)) = h.y;
    }
  }
  sync_async();
  // ---- dW3 = h2^T dz3 (two M tiles) with h2^T and dz3^T staged in sB
  load_b(h2t, 65536, sB);
  load_b(dzt, 65536, sB + 65536);
  if (ok) mma_done(gemm_dw(tmem, sB, sB + 65536, bar_m, pm));
  __syncthreads();
  store_dw(tlane, p.part + (size_t)cta * kNP + kOW3);
  sync_async();
  // ---- dh2 = dz3 W3^T; dz2 = dh2 silu'(z2) as A operand and dz2^T
  load_b(p.w3n, kB, sB);
  if (ok) mma_done(gemm_k(tmem, sA, sB, kH, bar_m, pm));
  __syncthreads();
  for (int c = 0; c < kH; c += 16) {
    float v[16], dz[16];
    tmem_ld16(tlane + c, v);
#pragma unroll
    for (int i = 0; i < 16; i++) dz[i] = v[i] * dsilu(z2g[(size_t)(c + i) * kRows + tid]);
    col_sum16(dz, c, red);
    __syncthreads();
    if (tid < 16) p.part[(size_t)cta * kNP + kOB2 + c + tid] = red[c + tid] + red[kH + c + tid] + red[2 * kH + c + tid] + red[3 * kH + c + tid];
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 16; i += 2) {
      __nv_bfloat162 h = __floats2bfloat162_rn(dz[i], dz[i + 1]);
      *(__nv_bfloat162 *)(sA + canon(tid, c + i)) = h;
      *(__nv_bfloat16 *)(dzt + canon128(c + i, tid)) = h.x;
      *(__nv_bfloat16 *)(dzt + canon128(c + i + 1, tid)) = h.y;
    }
  }
  sync_async();
  // ---- dW2 = h1^T dz2
  load_b(h1t, 65536, sB);
  load_b(dzt, 65536, sB + 65536);
  if (ok) mma_done(gemm_dw(tmem, sB, sB + 65536, bar_m, pm));
  __syncthreads();
  store_dw(tlane, p.part + (size_t)cta * kNP + kOW2);
  sync_async();
  // ---- dh1 = dz2 W2^T; dz1 = dh1 silu'(z1); dW1 = x^T dz1, db1
  load_b(p.w2n, kB, sB);
  if (ok) mma_done(gemm_k(tmem, sA, sB, kH, bar_m, pm));
  __syncthreads();
  for (int c = 0; c < kH; c += 16) {
    float v[16], dz[16];
    tmem_ld16(tlane + c, v);
#pragma unroll
    for (int i = 0; i < 16; i++) {
      float z = sb1[c + i];
      for (int q = 0; q < kIn; q++) z = fmaf(xin[q], sw1[q * kH + c + i], z);
      dz[i] = v[i] * dsilu(z);
    }
    col_sum16(dz, c, red);
    __syncthreads();
    if (tid < 16) p.part[(size_t)cta * kNP + kOB1 + c + tid] = red[c + tid] + red[kH + c + tid] + red[2 * kH + c + tid] + red[3 * kH + c + tid];
    __syncthreads();
    for (int q = 0; q < kIn; q++) {
      float t[16];
#pragma unroll
      for (int i = 0; i < 16; i++) t[i] = xin[q] * dz[i];
      col_sum16(t, c, red);
      __syncthreads();
      if (tid < 16)
        p.part[(size_t)cta * kNP + kOW1 + q * kH + c + tid] =
            red[c + tid] + red[kH + c + tid] + red[2 * kH + c + tid] + red[3 * kH + c + tid];
      __syncthreads();
    }
  }
  if (!ok) {
    // a wait gave up: the last bulk copy and the last MMA issued may still
    // be in flight; wait for them (bounded) before the CTA's shared memory
    // and TMEM are released
    if (tid == 0) atomicOr(err, 1u);
    if (nload > 0) mbar_wait(bar_w, w_last);
    if (nmma > 0) mbar_wait(bar_m, m_last);
    __syncthreads();
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512) : "memory");
}

// sum of the per-CTA partials in CTA order: g[i] = sum_c part[c][i]
__global__ void k_mlp_reduce(const float *part, int ncta, size_t len, float *g)
{
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += (size_t)gridDim.x * blockDim.x) {
    float s = 0.0f;
    for (int c = 0; c < ncta; c++) s += part[(size_t)c * len + i];
    g[i] = s;
  }
}

// Adam on the FP32 master weights (bias-corrected step size lr_t)
__global__ void k_mlp_adam(float *w, const float *g, float *m1, float *m2, size_t len, float lr_t, float b1,
                           float b2, float eps)
{
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += (size_t)gridDim.x * blockDim.x) {
    float gi = g[i];
    float a = m1[i] = b1 * m1[i] + (1.0f - b1) * gi;
    float b = m2[i] = b2 * m2[i] + (1.0f - b2) * gi * gi;
    w[i] -= lr_t * a / (sqrtf(b) + eps);
  }
}

// BF16 canonical copies of a 256 x 256 weight W[in][out]: t = the B operand
// of h . W (element (out, in)), nrm = the B operand of dz . W^T (element (in, out))
__global__ void k_mlp_canon(const float *w, char *t, char *nrm)
{
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < kH * kH; idx += gridDim.x * blockDim.x) {
    int in = idx / kH, out = idx % kH;
    __nv_bfloat16 b = __float2bfloat16_rn(w[idx]);
    *(__nv_bfloat16 *)(t + canon(out, in)) = b;
    *(__nv_bfloat16 *)(nrm + canon(in, out)) = b;
  }
}

}  // namespace

// ------------------------------------------------------------------ host

struct pimc_mlp {
  int device = 0;
  cudaStream_t stream = nullptr;
  float *prm = nullptr, *grad = nullptr, *m1 = nullptr, *m2 = nullptr;   // [kNP] each
  char *w2c = nullptr, *w3c = nullptr, *w2n = nullptr, *w3n = nullptr;    // BF16 canonical copies
  unsigned *err = nullptr;
  float *xbuf = nullptr, *ybuf = nullptr, *ebuf = nullptr;
  size_t cap = 0;
  // training scratch for up to tcap CTAs
  char *h1t = nullptr, *h2t = nullptr, *dzt = nullptr;
  float *z2 = nullptr, *part = nullptr, *loss = nullptr;
  int tcap = 0;
  long long step = 0;
  unsigned long long uid = 0;   // never reused within the process (keys captured graphs)
  // a training step whose kernel gave up a wait has applied an incomplete
  // gradient: the weights are unusable until pimc_mlp_set_weights loads new ones
  bool poisoned = false;
};

static std::atomic<unsigned long long> g_mlp_uid{0};

unsigned long long mlp_uid(const pimc_mlp *m) { return m ? m->uid : 0ull; }

#define MCK(x)                                  \
  do {                                          \
    if ((x) != cudaSuccess) return PIMC_ERR_CUDA; \
  } while (0)

static MlpParams params_of(const pimc_mlp *m)
{
  return MlpParams{m->prm + kOW1, m->prm + kOB1, m->w2c, m->w3c, m->prm + kOB2, m->prm + kOB3, m->prm + kOW4,
                   m->prm + kOB4};
}

static pimc_status refresh_canon(pimc_mlp *m)
{
  k_mlp_canon<<<256, 256, 0, m->stream>>>(m->prm + kOW2, m->w2c, m->w2n);
  k_mlp_canon<<<256, 256, 0, m->stream>>>(m->prm + kOW3, m->w3c, m->w3n);
  MCK(cudaGetLastError());
  return PIMC_OK;
}

extern "C" pimc_status pimc_mlp_create(int device, pimc_mlp **out)
{
  if (!out) return PIMC_ERR_BAD_ARG;
  int nd = 0;
  if (cudaGetDeviceCount(&nd) != cudaSuccess || nd <= device) return PIMC_ERR_NO_DEVICE;
  pimc_mlp *m = new (std::nothrow) pimc_mlp();
  if (!m) return PIMC_ERR_BAD_ARG;
  m->uid = ++g_mlp_uid;
  m->device = device;
  MCK(cudaSetDevice(device));
  MCK(cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking));
  MCK(cudaMalloc(&m->prm, kNP * sizeof(float)));
  MCK(cudaMalloc(&m->grad, kNP * sizeof(float)));
  MCK(cudaMalloc(&m->m1, kNP * sizeof(float)));
  MCK(cudaMalloc(&m->m2, kNP * sizeof(float)));
  MCK(cudaMemset(m->prm, 0, kNP * sizeof(float)));
  MCK(cudaMemset(m->m1, 0, kNP * sizeof(float)));
  MCK(cudaMemset(m->m2, 0, kNP * sizeof(float)));
  MCK(cudaMalloc(&m->w2c, kB));
  MCK(cudaMalloc(&m->w3c, kB));
  MCK(cudaMalloc(&m->w2n, kB));
  MCK(cudaMalloc(&m->w3n, kB));
  MCK(cudaMalloc(&m->err, sizeof(unsigned)));
  MCK(cudaMemset(m->err, 0, sizeof(unsigned)));
  MCK(cudaFuncSetAttribute(k_mlp_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmem));
  MCK(cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemT));
  *out = m;
  return PIMC_OK;
}

extern "C" pimc_status pimc_mlp_destroy(pimc_mlp *m)
{
  if (!m) return PIMC_ERR_BAD_ARG;
  cudaSetDevice(m->device);
  if (m->stream) cudaStreamSynchronize(m->stream);
  void *b[] = {m->prm, m->grad, m->m1, m->m2, m->w2c, m->w3c, m->w2n, m->w3n, m->err, m->xbuf, m->ybuf, m->ebuf,
               m->h1t, m->h2t, m->dzt, m->z2, m->part, m->loss};
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
  m->poisoned = false;
  std::vector<float> h(kNP);
  memcpy(&h[kOW1], w1, kIn * kH * sizeof(float));
  memcpy(&h[kOB1], b1, kH * sizeof(float));
  memcpy(&h[kOW2], w2, kH * kH * sizeof(float));
  memcpy(&h[kOB2], b2, kH * sizeof(float));
  memcpy(&h[kOW3], w3, kH * kH * sizeof(float));
  memcpy(&h[kOB3], b3, kH * sizeof(float));
  memcpy(&h[kOW4], w4, kH * sizeof(float));
  h[kOB4] = b4;
  MCK(cudaMemcpyAsync(m->prm, h.data(), kNP * sizeof(float), cudaMemcpyHostToDevice, m->stream));
  MCK(cudaMemsetAsync(m->m1, 0, kNP * sizeof(float), m->stream));
  MCK(cudaMemsetAsync(m->m2, 0, kNP * sizeof(float), m->stream));
  m->step = 0;
  pimc_status e = refresh_canon(m);
  if (e) return e;
  MCK(cudaStreamSynchronize(m->stream));
  return PIMC_OK;
}

extern "C" pimc_status pimc_mlp_get_params(pimc_mlp *m, float *prm)
{
  if (!m || !prm) return PIMC_ERR_BAD_ARG;
  MCK(cudaSetDevice(m->device));
  MCK(cudaMemcpyAsync(prm, m->prm, kNP * sizeof(float), cudaMemcpyDeviceToHost, m->stream));
  MCK(cudaStreamSynchronize(m->stream));
  return PIMC_OK;
}

extern "C" int pimc_mlp_param_count(void) { return kNP; }

static pimc_status ensure_io(pimc_mlp *m, size_t n)
{
  if (n <= m->cap) return PIMC_OK;
  if (m->xbuf) cudaFree(m->xbuf);
  if (m->ybuf) cudaFree(m->ybuf);
  if (m->ebuf) cudaFree(m->ebuf);
  m->xbuf = m->ybuf = m->ebuf = nullptr;
  MCK(cudaMalloc(&m->xbuf, n * kIn * sizeof(float)));
  MCK(cudaMalloc(&m->ybuf, n * sizeof(float)));
  MCK(cudaMalloc(&m->ebuf, n * sizeof(float)));
  m->cap = n;
  return PIMC_OK;
}

static pimc_status ensure_train(pimc_mlp *m, int ncta)
{
  if (ncta <= m->tcap) return PIMC_OK;
  void *b[] = {m->h1t, m->h2t, m->dzt, m->z2, m->part, m->loss};
  for (void *p : b)
    if (p) cudaFree(p);
  MCK(cudaMalloc(&m->h1t, (size_t)ncta * 65536));
  MCK(cudaMalloc(&m->h2t, (size_t)ncta * 65536));
  MCK(cudaMalloc(&m->dzt, (size_t)ncta * 65536));
  MCK(cudaMalloc(&m->z2, (size_t)ncta * kRows * kH * sizeof(float)));
  MCK(cudaMalloc(&m->part, (size_t)ncta * kNP * sizeof(float)));
  MCK(cudaMalloc(&m->loss, (size_t)ncta * sizeof(float)));
  m->tcap = ncta;
  return PIMC_OK;
}

// gradients of mean((y - e)^2) over the n device-resident samples into m->grad;
// the per-CTA losses summed on the host into *loss (optional)
static pimc_status device_grads(pimc_mlp *m, const float *xd, const float *ed, int n, double *loss)
{
  int ncta = (n + kRows - 1) / kRows;
  pimc_status e = ensure_train(m, ncta);
  if (e) return e;
  MlpTrainParams p;
  p.w = params_of(m);
  p.w2n = m->w2n;
  p.w3n = m->w3n;
  p.x = xd;
  p.e = ed;
  p.n = n;
  p.gscale = 2.0f / (float)n;
  p.h1t = m->h1t; p.h2t = m->h2t; p.dzt = m->dzt; p.z2 = m->z2;
  p.part = m->part;
  p.loss = m->loss;
  k_mlp_train<<<ncta, kRows, kSmemT, m->stream>>>(p, m->err);
  k_mlp_reduce<<<(kNP + 255) / 256, 256, 0, m->stream>>>(m->part, ncta, (size_t)kNP, m->grad);
  MCK(cudaGetLastError());
  if (loss) {
    std::vector<float> l(ncta);
    MCK(cudaMemcpyAsync(l.data(), m->loss, ncta * sizeof(float), cudaMemcpyDeviceToHost, m->stream));
    MCK(cudaStreamSynchronize(m->stream));
    double s = 0.0;
    for (float v : l) s += v;
    *loss = s / n;
  }
  return PIMC_OK;
}

static pimc_status check_mlp_err(pimc_mlp *m)
{
  MCK(cudaStreamSynchronize(m->stream));
  unsigned e = 0;
  MCK(cudaMemcpy(&e, m->err, sizeof(unsigned), cudaMemcpyDeviceToHost));
  if (e) {
    cudaMemset(m->err, 0, sizeof(unsigned));
    return PIMC_ERR_TIMEOUT;
  }
  return PIMC_OK;
}

extern "C" pimc_status pimc_mlp_gradients(pimc_mlp *m, int n, const float *x, const float *e, float *grad,
                                          double *loss)
{
  if (!m || n <= 0 || !x || !e || !grad) return PIMC_ERR_BAD_ARG;
  if (m->poisoned) return PIMC_ERR_TIMEOUT;
  MCK(cudaSetDevice(m->device));
  pimc_status st = ensure_io(m, (size_t)n);
  if (st) return st;
  MCK(cudaMemcpyAsync(m->xbuf, x, (size_t)n * kIn * sizeof(float), cudaMemcpyHostToDevice, m->stream));
  MCK(cudaMemcpyAsync(m->ebuf, e, (size_t)n * sizeof(float), cudaMemcpyHostToDevice, m->stream));
  if ((st = device_grads(m, m->xbuf, m->ebuf, n, loss))) return st;
  MCK(cudaMemcpyAsync(grad, m->grad, kNP * sizeof(float), cudaMemcpyDeviceToHost, m->stream));
  return check_mlp_err(m);
}

// epochs over n samples in minibatches of `batch` (a multiple of 128) in a
// seeded order, Adam with step size lr; loss_out[epoch] = mean loss of the
// epoch's minibatches (optional)
extern "C" pimc_status pimc_mlp_train(pimc_mlp *m, int n, const float *x, const float *e, int epochs, int batch,
                                      float lr, uint64_t seed, double *loss_out)
{
  if (!m || n <= 0 || !x || !e || epochs < 0 || batch < kRows || batch % kRows) return PIMC_ERR_BAD_ARG;
  if (m->poisoned) return PIMC_ERR_TIMEOUT;
  MCK(cudaSetDevice(m->device));
  pimc_status st = ensure_io(m, (size_t)n);
  if (st) return st;
  std::vector<int> order(n);
  for (int i = 0; i < n; i++) order[i] = i;
  uint64_t s = seed * 0x9E3779B97F4A7C15ull + 1;
  for (int i = n - 1; i > 0; i--) {      // a seeded shuffle (xorshift64*)
    s ^= s >> 12; s ^= s << 25; s ^= s >> 27;
    int j = (int)((s * 0x2545F4914F6CDD1Dull) % (uint64_t)(i + 1));
    std::swap(order[i], order[j]);
  }
  std::vector<float> xs((size_t)n * kIn), es(n);
  for (int i = 0; i < n; i++) {
    memcpy(&xs[(size_t)i * kIn], x + (size_t)order[i] * kIn, kIn * sizeof(float));
    es[i] = e[order[i]];
  }
  MCK(cudaMemcpyAsync(m->xbuf, xs.data(), xs.size() * sizeof(float), cudaMemcpyHostToDevice, m->stream));
  MCK(cudaMemcpyAsync(m->ebuf, es.data(), es.size() * sizeof(float), cudaMemcpyHostToDevice, m->stream));
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  for (int ep = 0; ep < epochs; ep++) {
    double lsum = 0.0;
    int nb = 0;
    for (int o = 0; o + batch <= n; o += batch) {
      double l = 0.0;
      if ((st = device_grads(m, m->xbuf + (size_t)o * kIn, m->ebuf + o, batch, loss_out ? &l : nullptr))) return st;
      m->step++;
      double c1 = 1.0 - pow((double)b1, (double)m->step), c2 = 1.0 - pow((double)b2, (double)m->step);
      float lr_t = (float)(lr * sqrt(c2) / c1);
      k_mlp_adam<<<(kNP + 255) / 256, 256, 0, m->stream>>>(m->prm, m->grad, m->m1, m->m2, (size_t)kNP, lr_t, b1, b2,
                                                            eps);
      if ((st = refresh_canon(m))) return st;
      lsum += l;
      nb++;
    }
    if (loss_out) loss_out[ep] = nb ? lsum / nb : 0.0;
  }
  st = check_mlp_err(m);
  if (st) m->poisoned = true;
  return st;
}

int mlp_forward_device(pimc_mlp *m, const float *x, int n, float *y, cudaStream_t s)
{
  if (n <= 0) return 0;
  MlpParams p = params_of(m);
  k_mlp_forward<<<(n + kRows - 1) / kRows, kFwdThreads, kSmem, s>>>(p, x, n, y, m->err);
  return 1;
}

// the forward kernel again on the rows the last pimc_mlp_forward uploaded,
// on the surrogate's stream, results left on the device (kernel timing)
extern "C" pimc_status pimc_mlp_forward_resident(pimc_mlp *m, int n)
{
  if (!m || n <= 0 || (size_t)n > m->cap) return PIMC_ERR_BAD_ARG;
  if (m->poisoned) return PIMC_ERR_TIMEOUT;
  MCK(cudaSetDevice(m->device));
  mlp_forward_device(m, m->xbuf, n, m->ybuf, m->stream);
  MCK(cudaGetLastError());
  return PIMC_OK;
}

extern "C" void *pimc_mlp_stream(const pimc_mlp *m) { return m ? (void *)m->stream : nullptr; }

// whether a surrogate launch gave up a wait since the last call (clears it)
bool mlp_take_error(pimc_mlp *m)
{
  if (m->poisoned) return true;
  unsigned e = 0;
  if (cudaMemcpy(&e, m->err, sizeof(unsigned), cudaMemcpyDeviceToHost) != cudaSuccess) return true;
  if (e) cudaMemset(m->err, 0, sizeof(unsigned));
  return e != 0;
}

extern "C" pimc_status pimc_mlp_forward(pimc_mlp *m, int n, const float *x, float *y)
{
  if (!m || n < 0 || (n && (!x || !y))) return PIMC_ERR_BAD_ARG;
  if (m->poisoned) return PIMC_ERR_TIMEOUT;
  if (n == 0) return PIMC_OK;
  MCK(cudaSetDevice(m->device));
  pimc_status st = ensure_io(m, (size_t)n);
  if (st) return st;
  MCK(cudaMemcpyAsync(m->xbuf, x, (size_t)n * kIn * sizeof(float), cudaMemcpyHostToDevice, m->stream));
  MlpParams p = params_of(m);
  k_mlp_forward<<<(n + kRows - 1) / kRows, kFwdThreads, kSmem, m->stream>>>(p, m->xbuf, n, m->ybuf, m->err);
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

bool mlp_poisoned(const pimc_mlp *m) { return m->poisoned; }
