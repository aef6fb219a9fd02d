// cvo_learn.cu -- learned proposal of initial poses for global registration.
//
// The reference picks the initial rotation of a global registration from a fixed
// grid: the cos-angle of every grid rotation is evaluated and the best one is
// refined (get_nearest_init_pose, src/cvo/CvoGPU.cpp:367-398, grids at :279-363).
// Here a small point-set network proposes K poses per pair instead; they are refined
// by the batched align and judged by the final cos-angle, with the grid kept as the
// fallback.  The network has no counterpart in the reference.
//
// Network (per pair; P points sampled from each cloud):
//   point input  x = [R (p - m) / 10, f_0 .. f_4, 0 x 8]      16 columns (8 used)
//   encoder      e = maxpool_p relu(relu(x W1 + b1) W2 + b2)   8 -> 64 -> 128
//   head         o = relu([e_src, e_tgt] W3 + b3) W4 + b4       256 -> 256 -> K * 9
//   hypothesis k o[9k .. 9k+5] = first two columns of R_k (Gram-Schmidt),
//                o[9k+6 .. 9k+8] = (t_k - (c_tgt - R_k c_src)) / 10
// Every matrix product runs on the tensor cores (mma.sync m16n8k16, BF16 operands
// rounded from FP32 when a tile is staged, FP32 accumulation); activations, weights,
// gradients and the Adam moments are FP32.  Training minimises the relaxed
// winner-takes-all loss over the K hypotheses (0.95 on the best, 0.05 spread over
// the others) with Adam; the whole step runs on the device.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>
#include <cuda_bf16.h>
#include "cvo_internal.h"
#include "cvo_device.cuh"

namespace cvo_gb {

constexpr int kNetIn = 16;       // padded input width (8 used)
constexpr int kNetInUsed = 8;
constexpr int kNetH1 = 64;
constexpr int kNetH2 = 128;
constexpr int kNetHead = 256;    // [e_src, e_tgt]
constexpr int kNetH3 = 256;
constexpr int kNetK = 8;         // hypotheses per pair
constexpr int kNetOut = 9 * kNetK;
constexpr float kNetInvScale = 0.1f;

// parameter block layout (floats), row-major weights [in][out]
constexpr size_t kOffW1 = 0;
constexpr size_t kOffB1 = kOffW1 + (size_t)kNetIn * kNetH1;
constexpr size_t kOffW2 = kOffB1 + kNetH1;
constexpr size_t kOffB2 = kOffW2 + (size_t)kNetH1 * kNetH2;
constexpr size_t kOffW3 = kOffB2 + kNetH2;
constexpr size_t kOffB3 = kOffW3 + (size_t)kNetHead * kNetH3;
constexpr size_t kOffW4 = kOffB3 + kNetH3;
constexpr size_t kOffB4 = kOffW4 + (size_t)kNetH3 * kNetOut;
constexpr size_t kNetParams = kOffB4 + kNetOut;

// One cloud of a network batch: points p_i = xyz[i * xyz_stride + 0..2] moved by the
// row-major 3x4 transform T, features feat[i * feat_stride + 0 .. nfeat-1].
struct NetSlot {
  const float *xyz;
  const float *feat;
  int xyz_stride, feat_stride, nfeat, n;
  float T[12];
};

namespace {

// --------------------------------------------------------------- sampling
// Point p of slot s is index ((h * n) >> 32) with h = mix(mix(seed + 0x9E3779B9 (s + 1)) ^ p),
// mix = the "lowbias32" integer hash (C. Wellons' hash-prospector constants).
__host__ __device__ inline uint32_t mix32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352dU;
  x ^= x >> 15;
  x *= 0x846ca68bU;
  x ^= x >> 16;
  return x;
}

__device__ inline int sample_index(uint32_t seed, int slot, int p, int n) {
  const uint32_t h = mix32(mix32(seed + 0x9E3779B9U * (uint32_t)(slot + 1)) ^ (uint32_t)p);
  return (int)(((uint64_t)h * (uint64_t)n) >> 32);
}

// ------------------------------------------------------------------ GEMM
// C[m][n] = sum_k A(m, k) B(k, n) (+ bias[n]) (ReLU), with A(m, k) = A[m sam + k sak],
// B(k, n) = B[k sbk + n sbn] and C row-major (leading dimension ldc).  A block of 4
// warps computes a 64 x 64 tile (2 x 2 warps of 32 x 32) over the k range
// [z kc, (z + 1) kc); with several k ranges (PARTIAL) each block stores its tile in
// plane z of a [splits][M][N] workspace and k_split_sum adds the planes in z order,
// so the result does not depend on the order in which the blocks finish.
constexpr int kGT = 64;

__device__ __forceinline__ uint32_t bf16x2(float lo, float hi) {
  return (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(lo)) |
         ((uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(hi)) << 16);
}

__device__ __forceinline__ void ldsm4(const void *p, uint32_t &r0, uint32_t &r1, uint32_t &r2, uint32_t &r3) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0, %1, %2, %3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(smem_addr(p))
               : "memory");
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
      "{%0, %1, %2, %3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

template <bool RELU, bool PARTIAL>
__global__ void __launch_bounds__(128) k_gemm_bf16(int M, int N, int K, int kc, const float *__restrict__ A,
                                                   long long sam, long long sak, const float *__restrict__ B,
                                                   long long sbk, long long sbn, const float *__restrict__ bias,
                                                   float *__restrict__ C, long long ldc) {
  // Operand tiles as planes of 8 BF16 (16 bytes): plane 0 holds k 0-7 of a row (A)
  // or column (B), plane 1 k 8-15, so each 8 x 8 block is one ldmatrix matrix.
  __shared__ __align__(16) uint4 As[2][kGT];
  __shared__ __align__(16) uint4 Bs[2][kGT];
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const int m0 = blockIdx.y * kGT, n0 = blockIdx.x * kGT;
  const int kb = blockIdx.z * kc, ke = min(K, kb + kc);
  const int wm = (w >> 1) * 32, wn = (w & 1) * 32;
  float acc[2][4][4];
#pragma unroll
  for (int a = 0; a < 2; a++)
#pragma unroll
    for (int b = 0; b < 4; b++)
#pragma unroll
      for (int c = 0; c < 4; c++) acc[a][b][c] = 0.f;
  const int sr = tid & 63, spl = tid >> 6;
  for (int k0 = kb; k0 < ke; k0 += 16) {
    {
      uint32_t wa[4], wb[4];
      const int m = m0 + sr, n = n0 + sr;
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const int k = k0 + 8 * spl + 2 * q;
        float a0 = 0.f, a1 = 0.f, b0 = 0.f, b1 = 0.f;
        if (m < M) {
          if (k < ke) a0 = A[m * sam + k * sak];
          if (k + 1 < ke) a1 = A[m * sam + (k + 1) * sak];
        }
        if (n < N) {
          if (k < ke) b0 = B[k * sbk + n * sbn];
          if (k + 1 < ke) b1 = B[(k + 1) * sbk + n * sbn];
        }
        wa[q] = bf16x2(a0, a1);
        wb[q] = bf16x2(b0, b1);
      }
      As[spl][sr] = make_uint4(wa[0], wa[1], wa[2], wa[3]);
      Bs[spl][sr] = make_uint4(wb[0], wb[1], wb[2], wb[3]);
    }
    __syncthreads();
    const int mi = lane >> 3, r8 = lane & 7;
    uint32_t af[2][4], bfr[2][4];
#pragma unroll
    for (int m = 0; m < 2; m++)
      ldsm4(&As[mi >> 1][wm + 16 * m + 8 * (mi & 1) + r8], af[m][0], af[m][1], af[m][2], af[m][3]);
#pragma unroll
    for (int j = 0; j < 2; j++)
      ldsm4(&Bs[mi & 1][wn + 16 * j + 8 * (mi >> 1) + r8], bfr[j][0], bfr[j][1], bfr[j][2], bfr[j][3]);
#pragma unroll
    for (int m = 0; m < 2; m++)
#pragma unroll
      for (int n = 0; n < 4; n++)
        mma_bf16(acc[m][n], af[m], bfr[n >> 1][2 * (n & 1)], bfr[n >> 1][2 * (n & 1) + 1]);
    __syncthreads();
  }
  const int gid = lane >> 2, t4 = lane & 3;
#pragma unroll
  for (int m = 0; m < 2; m++)
#pragma unroll
    for (int n = 0; n < 4; n++)
#pragma unroll
      for (int e = 0; e < 4; e++) {
        const int row = m0 + wm + 16 * m + gid + 8 * (e >> 1);
        const int col = n0 + wn + 8 * n + 2 * t4 + (e & 1);
        if (row >= M || col >= N) continue;
        float v = acc[m][n][e];
        if (PARTIAL) {
          C[((size_t)blockIdx.z * M + row) * N + col] = v;
        } else {
          if (bias) v += bias[col];
          if (RELU) v = fmaxf(v, 0.f);
          C[row * ldc + col] = v;
        }
      }
}

// ------------------------------------------------------- tcgen05 GEMM
// The same product on the fifth-generation tensor cores: one CTA of 4 warps owns a
// 128 x 64 tile of C, accumulated in tensor memory (TMEM, 64 FP32 columns x 128
// lanes).  The k range is consumed in stages of 64: every thread converts one row of A
// (threads 0-127) and half of a column of B (two threads per column) from FP32 to BF16
// -- with 16-byte loads where k is the contiguous dimension -- and stores them in the
// no-swizzle K-major layout of the tensor core's shared-memory descriptors: per 16-wide
// k slice, 8 x 8 core matrices of 128 bytes, the slice's two k halves 128 bytes apart
// (leading offset) and consecutive groups of 8 rows 256 bytes apart (stride offset).
// One elected thread issues the stage's four tcgen05.mma (kind::f16, BF16 x BF16 ->
// FP32, M = 128, N = 64, K = 16 each) and commits them to the stage's mbarrier; the
// staging of the next stage overlaps the running MMAs (two stages).  The epilogue
// reads the accumulator with tcgen05.ld (warp w owns TMEM lanes 32w .. 32w + 31, i.e.
// tile rows) and adds bias / ReLU or stores a split-K plane exactly as k_gemm_bf16
// does.  Every mbarrier wait is bounded: after kTcSpin clock cycles the kernel records
// kTcTimeout in *err, issues no further MMA, drains what it issued (again bounded) and
// frees its TMEM before returning.
constexpr int kTcM = 128, kTcN = 64, kTcK = 16, kTcSlices = 4, kTcKS = kTcK * kTcSlices;
constexpr uint32_t kTcCols = 64;            // TMEM columns: the FP32 accumulator of a 128 x 64 tile
constexpr int kTcStages = 2;
constexpr long long kTcSpin = 1LL << 31;    // SM clock cycles (about 1 s) before an mbarrier wait gives up
constexpr int kTcTimeout = 1;
constexpr int kTcSliceA = kTcM * kTcK * 2;  // bytes of one 16-wide k slice of A (4 KB)
constexpr int kTcSliceB = kTcN * kTcK * 2;  // and of B (2 KB)
// Dynamic shared memory per CTA: at most 4 CTAs fit on an SM (228 KB), so their TMEM
// columns (4 x 64) never exceed the SM's 512 and tcgen05.alloc never waits.
constexpr int kTcSmemBytes = 52 * 1024;

struct __align__(1024) TcSmem {
  uint4 a[kTcStages][kTcSlices * kTcSliceA / 16];   // 128 rows x 64 k BF16 (16 KB) per stage
  uint4 b[kTcStages][kTcSlices * kTcSliceB / 16];   // 64 columns x 64 k BF16 (8 KB) per stage
  unsigned long long bar[kTcStages];
  uint32_t tmem;
  int failed;
};
static_assert(sizeof(TcSmem) <= kTcSmemBytes, "tcgen05 GEMM shared memory");
static_assert(kTcSmemBytes * 5 > 228 * 1024, "at most 4 tcgen05 GEMM CTAs per SM");

// Byte offset of row r (M or N index), k half g inside one 16-wide slice (no-swizzle
// K-major core matrices).
__device__ __forceinline__ int tc_off(int r, int g) { return (r >> 3) * 256 + g * 128 + (r & 7) * 16; }

// Shared-memory matrix descriptor: start address, leading (k) and stride (row-group)
// byte offsets, each >> 4; bit 46 = descriptor version 1; layout type 0 = no swizzle.
__device__ __forceinline__ uint64_t tc_desc(const void *p) {
  uint64_t d = (uint64_t)((smem_addr(p) >> 4) & 0x3FFFu);
  d |= (uint64_t)(128u >> 4) << 16;
  d |= (uint64_t)(256u >> 4) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both K-major,
// N >> 3 at bit 17, M >> 4 at bit 24.
constexpr uint32_t kTcIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kTcN >> 3) << 17) |
                              ((uint32_t)(kTcM >> 4) << 24);

__device__ __forceinline__ void tc_bar_init(unsigned long long *bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_addr(bar)) : "memory");
}

// Waits for phase `parity` of the barrier (non-blocking polls); false once kTcSpin SM
// clock cycles (about a second) have passed.
__device__ __forceinline__ bool tc_bar_wait(unsigned long long *bar, uint32_t parity) {
  const uint32_t a = smem_addr(bar);
  const long long t0 = clock64();
  while (true) {
    uint32_t done = 0;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
    if (clock64() - t0 > kTcSpin) return false;
  }
}

// Four consecutive k values of an operand row starting at k (zero beyond ke): one
// 16-byte load when all four are in range, element loads at the ragged end.
__device__ __forceinline__ float4 tc_load4(const float *src, int k, int ke) {
  if (k + 3 < ke) return __ldg(reinterpret_cast<const float4 *>(src));
  float4 x = make_float4(0.f, 0.f, 0.f, 0.f);
  if (k < ke) x.x = src[0];
  if (k + 1 < ke) x.y = src[1];
  if (k + 2 < ke) x.z = src[2];
  return x;
}

template <bool RELU, bool PARTIAL>
__global__ void __launch_bounds__(128) k_gemm_tc(int M, int N, int K, int kc, const float *__restrict__ A,
                                                 long long sam, long long sak, const float *__restrict__ B,
                                                 long long sbk, long long sbn, const float *__restrict__ bias,
                                                 float *__restrict__ C, long long ldc, int *err) {
  extern __shared__ __align__(1024) unsigned char tc_smem_raw[];
  // k contiguous in memory, rows 16-byte aligned: operands are read with 16-byte loads
  const bool vec_a = sak == 1 && (sam & 3) == 0 && ((reinterpret_cast<uintptr_t>(A) & 15) == 0);
  const bool vec_b = sbk == 1 && (sbn & 3) == 0 && ((reinterpret_cast<uintptr_t>(B) & 15) == 0);
  TcSmem &sm = *reinterpret_cast<TcSmem *>(tc_smem_raw);
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const int m0 = blockIdx.y * kTcM, n0 = blockIdx.x * kTcN;
  const int kb = blockIdx.z * kc, ke = min(K, kb + kc);
  if (w == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_addr(&sm.tmem)),
                 "r"(kTcCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  if (tid == 0) {
    for (int st = 0; st < kTcStages; st++) tc_bar_init(&sm.bar[st]);
    sm.failed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = sm.tmem;
  const int steps = ke > kb ? (ke - kb + kTcKS - 1) / kTcKS : 0;
  int issued = 0;
  for (int it = 0; it < steps; it++) {
    const int st = it & 1, k0 = kb + it * kTcKS;
    const int nsl = min(kTcSlices, (ke - k0 + kTcK - 1) / kTcK);   // 16-wide slices holding data
    // the MMAs that read this stage two steps ago must be done before it is overwritten
    if (it >= kTcStages && !tc_bar_wait(&sm.bar[st], (uint32_t)(((it - kTcStages) >> 1) & 1))) sm.failed = 1;
    __syncthreads();
    if (sm.failed) break;
    unsigned char *ab = reinterpret_cast<unsigned char *>(sm.a[st]);
    unsigned char *bb = reinterpret_cast<unsigned char *>(sm.b[st]);
    const int m = m0 + tid;
    const int nn = tid & 63, g = tid >> 6, n = n0 + nn;
    for (int sl = 0; sl < nsl; sl++) {
      const int ks = k0 + kTcK * sl;
      // A: thread t converts row m0 + t, ks .. ks + 15
      uint32_t wv[8];
      if (vec_a) {
#pragma unroll
        for (int q = 0; q < 4; q++) {
          const float4 x = m < M ? tc_load4(A + m * sam + ks + 4 * q, ks + 4 * q, ke) : make_float4(0.f, 0.f, 0.f, 0.f);
          wv[2 * q] = bf16x2(x.x, x.y);
          wv[2 * q + 1] = bf16x2(x.z, x.w);
        }
      } else {
#pragma unroll
        for (int q = 0; q < 8; q++) {
          const int k = ks + 2 * q;
          float x0 = 0.f, x1 = 0.f;
          if (m < M) {
            if (k < ke) x0 = A[m * sam + k * sak];
            if (k + 1 < ke) x1 = A[m * sam + (k + 1) * sak];
          }
          wv[q] = bf16x2(x0, x1);
        }
      }
      *reinterpret_cast<uint4 *>(ab + sl * kTcSliceA + tc_off(tid, 0)) = make_uint4(wv[0], wv[1], wv[2], wv[3]);
      *reinterpret_cast<uint4 *>(ab + sl * kTcSliceA + tc_off(tid, 1)) = make_uint4(wv[4], wv[5], wv[6], wv[7]);
      // B: column n0 + (t & 63), k half t >> 6 of the slice
      uint32_t wb[4];
      const int kh = ks + 8 * g;
      if (vec_b) {
#pragma unroll
        for (int q = 0; q < 2; q++) {
          const float4 y = n < N ? tc_load4(B + n * sbn + kh + 4 * q, kh + 4 * q, ke) : make_float4(0.f, 0.f, 0.f, 0.f);
          wb[2 * q] = bf16x2(y.x, y.y);
          wb[2 * q + 1] = bf16x2(y.z, y.w);
        }
      } else {
#pragma unroll
        for (int q = 0; q < 4; q++) {
          const int k = kh + 2 * q;
          float y0 = 0.f, y1 = 0.f;
          if (n < N) {
            if (k < ke) y0 = B[k * sbk + n * sbn];
            if (k + 1 < ke) y1 = B[(k + 1) * sbk + n * sbn];
          }
          wb[q] = bf16x2(y0, y1);
        }
      }
      *reinterpret_cast<uint4 *>(bb + sl * kTcSliceB + tc_off(nn, g)) = make_uint4(wb[0], wb[1], wb[2], wb[3]);
    }
    // generic-proxy stores -> visible to the tensor core's (async proxy) reads
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      for (int sl = 0; sl < nsl; sl++) {
        const uint64_t da = tc_desc(ab + sl * kTcSliceA), db = tc_desc(bb + sl * kTcSliceB);
        const uint32_t acc = (it > 0 || sl > 0) ? 1u : 0u;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "setp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
            "l"(da), "l"(db), "r"(kTcIdesc), "r"(acc)
            : "memory");
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                       smem_addr(&sm.bar[st]))
                   : "memory");
    }
    issued = it + 1;
  }
  // every issued MMA has completed once the last stage's commit arrived (one thread
  // issues them all, in order)
  bool ok = !sm.failed;
  if (ok && issued > 0 && !tc_bar_wait(&sm.bar[(issued - 1) & 1], (uint32_t)(((issued - 1) >> 1) & 1))) ok = false;
  if (!ok && issued > 0) tc_bar_wait(&sm.bar[(issued - 1) & 1], (uint32_t)(((issued - 1) >> 1) & 1));   // drain
  ok = __syncthreads_and(ok) != 0;
  if (!ok && tid == 0) atomicOr(err, kTcTimeout);
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  if (ok) {
    const int row = m0 + 32 * w + lane;
#pragma unroll
    for (int c0 = 0; c0 < kTcN; c0 += 16) {
      uint32_t r[16];
      const uint32_t ta = tmem + ((uint32_t)(32 * w) << 16) + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
          "%15}, [%16];\n"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
          : "r"(ta)
          : "memory");
      asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
      if (row < M) {
#pragma unroll
        for (int e = 0; e < 16; e++) {
          const int col = n0 + c0 + e;
          if (col >= N) continue;
          float v = issued > 0 ? __uint_as_float(r[e]) : 0.f;
          if (PARTIAL) {
            C[((size_t)blockIdx.z * M + row) * N + col] = v;
          } else {
            if (bias) v += bias[col];
            if (RELU) v = fmaxf(v, 0.f);
            C[row * ldc + col] = v;
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (w == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kTcCols) : "memory");
  }
}

// ------------------------------------------------------------ batch input
// Mean of each slot's points (before its transform), FP64 in a fixed tree order.
__global__ void __launch_bounds__(256) k_slot_mean(const NetSlot *slots, float *mean, float *cent) {
  const NetSlot s = slots[blockIdx.x];
  __shared__ double red[3][256];
  double a[3] = {0.0, 0.0, 0.0};
  for (int i = threadIdx.x; i < s.n; i += 256)
    for (int d = 0; d < 3; d++) a[d] += (double)s.xyz[(size_t)i * s.xyz_stride + d];
  for (int d = 0; d < 3; d++) red[d][threadIdx.x] = a[d];
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
      for (int d = 0; d < 3; d++) red[d][threadIdx.x] += red[d][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    float m[3];
    for (int d = 0; d < 3; d++) m[d] = s.n > 0 ? (float)(red[d][0] / s.n) : 0.f;
    for (int d = 0; d < 3; d++) {
      mean[3 * blockIdx.x + d] = m[d];
      // centroid of the moved points, T m
      cent[3 * blockIdx.x + d] = s.T[4 * d] * m[0] + s.T[4 * d + 1] * m[1] + s.T[4 * d + 2] * m[2] + s.T[4 * d + 3];
    }
  }
}

// X row (slot, p) = [R (x_j - mean) / 10, features of j (5), zeros], j sampled.
__global__ void k_net_inputs(int n_slots, int P, uint32_t seed, const NetSlot *slots, const float *mean, float *X) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= (long long)n_slots * P) return;
  const int slot = (int)(i / P), p = (int)(i % P);
  const NetSlot &s = slots[slot];
  float *x = X + (size_t)i * kNetIn;
  float v[kNetIn];
#pragma unroll
  for (int k = 0; k < kNetIn; k++) v[k] = 0.f;
  if (s.n > 0) {
    const int j = sample_index(seed, slot, p, s.n);
    const float *q = s.xyz + (size_t)j * s.xyz_stride;
    const float d0 = q[0] - mean[3 * slot], d1 = q[1] - mean[3 * slot + 1], d2 = q[2] - mean[3 * slot + 2];
#pragma unroll
    for (int r = 0; r < 3; r++) v[r] = (s.T[4 * r] * d0 + s.T[4 * r + 1] * d1 + s.T[4 * r + 2] * d2) * kNetInvScale;
    const int nf = min(s.nfeat, kNetInUsed - 3);
    for (int k = 0; k < nf; k++) v[3 + k] = s.feat[(size_t)j * s.feat_stride + k];
  }
#pragma unroll
  for (int k = 0; k < kNetIn; k += 4) *reinterpret_cast<float4 *>(x + k) = make_float4(v[k], v[k + 1], v[k + 2], v[k + 3]);
}

// max over the P points of each slot; the first index of the maximum is kept
__global__ void k_maxpool(int n_slots, int P, const float *H, float *G, int *arg) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_slots * kNetH2) return;
  const int c = i / kNetH2, f = i % kNetH2;
  float best = -INFINITY;
  int bi = 0;
  for (int p = 0; p < P; p++) {
    const float v = H[((size_t)c * P + p) * kNetH2 + f];
    if (v > best) {
      best = v;
      bi = p;
    }
  }
  G[i] = best;
  arg[i] = bi;
}

// dH2 (zeroed) at the pooled rows, through the ReLU of H2 (H2 = G there)
__global__ void k_maxpool_bwd(int n_slots, int P, const float *G, const float *dG, const int *arg, float *dH) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_slots * kNetH2) return;
  const int c = i / kNetH2, f = i % kNetH2;
  if (G[i] > 0.f) dH[((size_t)c * P + arg[i]) * kNetH2 + f] = dG[i];
}

// --------------------------------------------------------------- outputs
__device__ inline void hypothesis_pose(const float *o, const float *cs, const float *ct, float *Tc) {
  const float a1[3] = {o[0], o[1], o[2]}, a2[3] = {o[3], o[4], o[5]};
  const float n1 = sqrtf(a1[0] * a1[0] + a1[1] * a1[1] + a1[2] * a1[2]);
  float b1[3], b2[3], b3[3];
  if (!(n1 > 1e-20f)) {
    b1[0] = 1.f; b1[1] = 0.f; b1[2] = 0.f;
  } else {
    for (int d = 0; d < 3; d++) b1[d] = a1[d] / n1;
  }
  const float dp = b1[0] * a2[0] + b1[1] * a2[1] + b1[2] * a2[2];
  for (int d = 0; d < 3; d++) b2[d] = a2[d] - dp * b1[d];
  float n2 = sqrtf(b2[0] * b2[0] + b2[1] * b2[1] + b2[2] * b2[2]);
  if (!(n2 > 1e-20f)) {
    // any unit vector orthogonal to b1
    const float e[3] = {fabsf(b1[0]) < 0.9f ? 1.f : 0.f, fabsf(b1[0]) < 0.9f ? 0.f : 1.f, 0.f};
    const float de = b1[0] * e[0] + b1[1] * e[1];
    for (int d = 0; d < 3; d++) b2[d] = e[d] - de * b1[d];
    n2 = sqrtf(b2[0] * b2[0] + b2[1] * b2[1] + b2[2] * b2[2]);
  }
  for (int d = 0; d < 3; d++) b2[d] /= n2;
  b3[0] = b1[1] * b2[2] - b1[2] * b2[1];
  b3[1] = b1[2] * b2[0] - b1[0] * b2[2];
  b3[2] = b1[0] * b2[1] - b1[1] * b2[0];
  // column-major 4x4: R columns b1 b2 b3, t = c_tgt - R c_src + 10 o[6..8]
  for (int r = 0; r < 3; r++) {
    Tc[0 * 4 + r] = b1[r];
    Tc[1 * 4 + r] = b2[r];
    Tc[2 * 4 + r] = b3[r];
    const float Rc = b1[r] * cs[0] + b2[r] * cs[1] + b3[r] * cs[2];
    Tc[12 + r] = ct[r] - Rc + o[6 + r] / kNetInvScale;
  }
  Tc[3] = Tc[7] = Tc[11] = 0.f;
  Tc[15] = 1.f;
}

__global__ void k_hypotheses(int Bn, const float *O, const float *cent, float *Tout) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= Bn * kNetK) return;
  const int b = i / kNetK, k = i % kNetK;
  hypothesis_pose(O + (size_t)b * kNetOut + 9 * k, cent + 6 * b, cent + 6 * b + 3, Tout + 16 * (size_t)i);
}

// Relaxed winner-takes-all loss per pair against the label pose T (row-major 3x4 of
// the target slot): y = [R(:,0), R(:,1), (t - (c_tgt - R c_src)) / 10] for every
// hypothesis; L_k = |o_k - y|^2, loss = 0.95 L_best + 0.05 / (K - 1) sum_{k != best} L_k,
// dO = (weight_k / Bn) 2 (o_k - y).
__global__ void k_wta_loss(int Bn, const float *O, const NetSlot *slots, const float *cent, float *dO, float *loss,
                           int *best_out) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= Bn) return;
  const float *T = slots[2 * b + 1].T;
  const float *cs = cent + 6 * b, *ct = cent + 6 * b + 3;
  float y[9];
  for (int r = 0; r < 3; r++) {
    y[r] = T[4 * r];
    y[3 + r] = T[4 * r + 1];
    const float Rc = T[4 * r] * cs[0] + T[4 * r + 1] * cs[1] + T[4 * r + 2] * cs[2];
    y[6 + r] = (T[4 * r + 3] - (ct[r] - Rc)) * kNetInvScale;
  }
  float L[kNetK];
  int best = 0;
  for (int k = 0; k < kNetK; k++) {
    float s = 0.f;
    for (int j = 0; j < 9; j++) {
      const float d = O[(size_t)b * kNetOut + 9 * k + j] - y[j];
      s += d * d;
    }
    L[k] = s;
    if (s < L[best]) best = k;
  }
  float tot = 0.f;
  for (int k = 0; k < kNetK; k++) {
    const float wk = k == best ? 0.95f : 0.05f / (kNetK - 1);
    tot += wk * L[k];
    for (int j = 0; j < 9; j++)
      dO[(size_t)b * kNetOut + 9 * k + j] = wk / Bn * 2.f * (O[(size_t)b * kNetOut + 9 * k + j] - y[j]);
  }
  loss[b] = tot;
  if (best_out) best_out[b] = best;
}

__global__ void k_relu_bwd(long long n, const float *H, float *dH) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n && !(H[i] > 0.f)) dH[i] = 0.f;
}

// part[y][c] = sum of D[r][c] over the rows r of block row y (2048 rows, 8 row groups
// of a block of 32 columns added in a fixed order)
__global__ void __launch_bounds__(256) k_colsum(int M, int N, const float *D, float *part) {
  const int c = blockIdx.x * 32 + (threadIdx.x & 31), g = threadIdx.x >> 5;
  const int r0 = blockIdx.y * 2048, r1 = min(M, r0 + 2048);
  __shared__ float red[8][33];
  float s = 0.f;
  if (c < N)
    for (int r = r0 + g; r < r1; r += 8) s += D[(size_t)r * N + c];
  red[g][threadIdx.x & 31] = s;
  __syncthreads();
  if (g == 0 && c < N) {
    float t = 0.f;
    for (int q = 0; q < 8; q++) t += red[q][threadIdx.x];
    part[(size_t)blockIdx.y * N + c] = t;
  }
}

// C[i / N][i % N] = sum over z of part[z][i], i < M N: warp g of a block of 32 outputs
// adds the planes z = g, g + 8, ... and the 8 warp sums are added in warp order.
__global__ void __launch_bounds__(256) k_split_sum(int M, int N, int splits, const float *part, float *C,
                                                   long long ldc) {
  const long long mn = (long long)M * N, i = blockIdx.x * 32LL + (threadIdx.x & 31);
  const int g = threadIdx.x >> 5;
  __shared__ float red[8][33];
  float s = 0.f;
  if (i < mn)
    for (int z = g; z < splits; z += 8) s += part[z * mn + i];
  red[g][threadIdx.x & 31] = s;
  __syncthreads();
  if (g == 0 && i < mn) {
    float t = 0.f;
    for (int q = 0; q < 8; q++) t += red[q][threadIdx.x];
    C[(i / N) * ldc + i % N] = t;
  }
}

__global__ void k_adam(int n, float *w, const float *g, float *m, float *v, float lr, float b1, float b2, float eps,
                       float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

}  // namespace

// ------------------------------------------------------------------ host
struct NetDev {
  int P = 0;
  int cap_pairs = 0;
  long long steps = 0;
  float *w = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;   // parameters, gradients, Adam moments
  NetSlot *slots = nullptr;
  float *mean = nullptr, *cent = nullptr;
  float *X = nullptr, *H1 = nullptr, *H2 = nullptr, *G = nullptr, *H3 = nullptr, *O = nullptr;
  float *dO = nullptr, *dH3 = nullptr, *dG = nullptr, *dH2 = nullptr, *dH1 = nullptr, *loss = nullptr;
  float *Tout = nullptr;
  float *part = nullptr;                 // split-K and column-sum partials of the backward pass
  size_t part_cap = 0;
  int *arg = nullptr, *best = nullptr;
  int gemm_kind = 0;                     // 0: tcgen05 (TMEM accumulators), 1: mma.sync (the second opinion)
  int *err = nullptr;                    // device word: bounded waits that gave up (kTcTimeout)
};

size_t net_num_params() { return kNetParams; }

static void net_free_acts(NetDev *n) {
  float *fs[] = {n->mean, n->cent, n->X, n->H1, n->H2, n->G, n->H3, n->O, n->dO, n->dH3, n->dG, n->dH2, n->dH1,
                 n->loss, n->Tout};
  for (float *p : fs) cudaFree(p);
  cudaFree(n->slots);
  cudaFree(n->arg);
  cudaFree(n->best);
  cudaFree(n->part);
  n->part = nullptr;
  n->part_cap = 0;
  n->mean = n->cent = n->X = n->H1 = n->H2 = n->G = n->H3 = n->O = nullptr;
  n->dO = n->dH3 = n->dG = n->dH2 = n->dH1 = n->loss = n->Tout = nullptr;
  n->slots = nullptr;
  n->arg = n->best = nullptr;
  n->cap_pairs = 0;
}

static int net_ensure(Handle *h, NetDev *n, int Bn) {
  if (Bn <= n->cap_pairs) return 0;
  net_free_acts(n);
  const size_t slots = 2 * (size_t)Bn, rows = slots * n->P;
  bool ok = true;
  auto al = [&](float **p, size_t count) {
    ok = ok && cudaMalloc((void **)p, sizeof(float) * (count ? count : 1)) == cudaSuccess;
  };
  al(&n->mean, 3 * slots);
  al(&n->cent, 3 * slots);
  al(&n->X, rows * kNetIn);
  al(&n->H1, rows * kNetH1);
  al(&n->H2, rows * kNetH2);
  al(&n->G, slots * kNetH2);
  al(&n->H3, (size_t)Bn * kNetH3);
  al(&n->O, (size_t)Bn * kNetOut);
  al(&n->dO, (size_t)Bn * kNetOut);
  al(&n->dH3, (size_t)Bn * kNetH3);
  al(&n->dG, slots * kNetH2);
  al(&n->dH2, rows * kNetH2);
  al(&n->dH1, rows * kNetH1);
  al(&n->loss, Bn);
  al(&n->Tout, (size_t)Bn * kNetK * 16);
  ok = ok && cudaMalloc((void **)&n->slots, sizeof(NetSlot) * slots) == cudaSuccess;
  ok = ok && cudaMalloc((void **)&n->arg, sizeof(int) * slots * kNetH2) == cudaSuccess;
  ok = ok && cudaMalloc((void **)&n->best, sizeof(int) * Bn) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    net_free_acts(n);
    h->last_error = "out of device memory for the proposal network's activations";
    return CVO_ERR_OUT_OF_MEMORY;
  }
  n->cap_pairs = Bn;
  return 0;
}

// Number of k ranges gemm() uses for a requested split count (ranges of whole
// 16-wide k steps).
static int gemm_splits(long long K, int splits) {
  const long long kc = ((K + splits - 1) / splits + 15) / 16 * 16;
  return (int)((K + kc - 1) / kc);
}

// C = A B (+bias, ReLU) on the tensor cores; with splits > 1 the k range is split over
// blockIdx.z, the partial tiles go to part (gemm_splits(K, splits) M N floats) and are
// added in a fixed order.
static void gemm(Handle *h, const NetDev *net, bool relu, int M, int N, int K, const float *A, long long sam,
                 long long sak, const float *B, long long sbk, long long sbn, const float *bias, float *C,
                 long long ldc, int splits = 1, float *part = nullptr) {
  const int kc = ((K + splits - 1) / splits + 15) / 16 * 16;
  splits = (K + kc - 1) / kc;
  if (net->gemm_kind == 0) {
    // opt in above the 48 KB default of dynamic shared memory, once per device
    static unsigned long long set_mask = 0;
    int dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess && !(set_mask & (1ull << (dev & 63)))) {
      cudaFuncSetAttribute(k_gemm_tc<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmemBytes);
      cudaFuncSetAttribute(k_gemm_tc<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmemBytes);
      cudaFuncSetAttribute(k_gemm_tc<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmemBytes);
      set_mask |= 1ull << (dev & 63);
    }
    const dim3 tgrid((N + kTcN - 1) / kTcN, (M + kTcM - 1) / kTcM, splits);
    if (splits > 1) {
      k_gemm_tc<false, true><<<tgrid, 128, kTcSmemBytes, h->stream>>>(M, N, K, kc, A, sam, sak, B, sbk, sbn,
                                                                      nullptr, part, N, net->err);
      k_split_sum<<<(unsigned)(((long long)M * N + 31) / 32), 256, 0, h->stream>>>(M, N, splits, part, C, ldc);
      h->launches++;
    } else if (relu) {
      k_gemm_tc<true, false><<<tgrid, 128, kTcSmemBytes, h->stream>>>(M, N, K, kc, A, sam, sak, B, sbk, sbn, bias,
                                                                      C, ldc, net->err);
    } else {
      k_gemm_tc<false, false><<<tgrid, 128, kTcSmemBytes, h->stream>>>(M, N, K, kc, A, sam, sak, B, sbk, sbn, bias,
                                                                       C, ldc, net->err);
    }
    h->launches++;
    return;
  }
  const dim3 grid((N + kGT - 1) / kGT, (M + kGT - 1) / kGT, splits);
  if (splits > 1) {
    k_gemm_bf16<false, true><<<grid, 128, 0, h->stream>>>(M, N, K, kc, A, sam, sak, B, sbk, sbn, nullptr, part, N);
    k_split_sum<<<(unsigned)(((long long)M * N + 31) / 32), 256, 0, h->stream>>>(M, N, splits, part, C, ldc);
    h->launches++;
  } else if (relu) {
    k_gemm_bf16<true, false><<<grid, 128, 0, h->stream>>>(M, N, K, kc, A, sam, sak, B, sbk, sbn, bias, C, ldc);
  } else {
    k_gemm_bf16<false, false><<<grid, 128, 0, h->stream>>>(M, N, K, kc, A, sam, sak, B, sbk, sbn, bias, C, ldc);
  }
  h->launches++;
}

// Row blocks of colsum(): its workspace holds colsum_blocks(M) N floats.
static int colsum_blocks(long long M) { return (int)std::max<long long>(1, (M + 2047) / 2048); }

// out[c] = sum_r D[r][c], in a fixed order.
static void colsum(Handle *h, int M, int N, const float *D, float *out, float *part) {
  const int ry = colsum_blocks(M);
  k_colsum<<<dim3((N + 31) / 32, ry), 256, 0, h->stream>>>(M, N, D, part);
  k_split_sum<<<(N + 31) / 32, 256, 0, h->stream>>>(1, N, ry, part, out, N);
  h->launches += 2;
}

int net_create(Handle *h, int P, unsigned seed, NetDev **out) {
  if (P < 1 || P > 65536 || !out) return CVO_ERR_INVALID_ARG;
  NetDev *n = new NetDev();
  n->P = P;
  const size_t np = kNetParams;
  if (cudaMalloc((void **)&n->w, sizeof(float) * np) != cudaSuccess ||
      cudaMalloc((void **)&n->g, sizeof(float) * np) != cudaSuccess ||
      cudaMalloc((void **)&n->m, sizeof(float) * np) != cudaSuccess ||
      cudaMalloc((void **)&n->v, sizeof(float) * np) != cudaSuccess ||
      cudaMalloc((void **)&n->err, sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    net_destroy(n);
    return CVO_ERR_OUT_OF_MEMORY;
  }
  // uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) for weights and biases; the padded
  // input rows of W1 stay zero
  std::vector<float> w(np, 0.f);
  std::mt19937 rng(seed);
  auto fill = [&](size_t off, size_t count, int fan_in) {
    const float a = 1.f / std::sqrt((float)fan_in);
    std::uniform_real_distribution<float> u(-a, a);
    for (size_t i = 0; i < count; i++) w[off + i] = u(rng);
  };
  fill(kOffW1, (size_t)kNetInUsed * kNetH1, kNetInUsed);
  fill(kOffB1, kNetH1, kNetInUsed);
  fill(kOffW2, (size_t)kNetH1 * kNetH2, kNetH1);
  fill(kOffB2, kNetH2, kNetH1);
  fill(kOffW3, (size_t)kNetHead * kNetH3, kNetHead);
  fill(kOffB3, kNetH3, kNetHead);
  fill(kOffW4, (size_t)kNetH3 * kNetOut, kNetH3);
  fill(kOffB4, kNetOut, kNetH3);
  int rc = CVO_OK;
  if (cudaMemcpy(n->w, w.data(), sizeof(float) * np, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemset(n->g, 0, sizeof(float) * np) != cudaSuccess || cudaMemset(n->m, 0, sizeof(float) * np) != cudaSuccess ||
      cudaMemset(n->v, 0, sizeof(float) * np) != cudaSuccess || cudaMemset(n->err, 0, sizeof(int)) != cudaSuccess)
    rc = set_cuda_error(h, cudaGetLastError(), "proposal network upload");
  if (rc) {
    net_destroy(n);
    return rc;
  }
  *out = n;
  return CVO_OK;
}

void net_destroy(NetDev *n) {
  if (!n) return;
  net_free_acts(n);
  cudaFree(n->w);
  cudaFree(n->g);
  cudaFree(n->m);
  cudaFree(n->v);
  cudaFree(n->err);
  delete n;
}

// Reads (and clears) the network's device error word after the stream is synchronised:
// a tensor-core GEMM whose bounded wait gave up reports CVO_ERR_TIMEOUT.
static int net_check(Handle *h, NetDev *n) {
  int e = 0;
  CVO_CUDA_TRY(h, cudaMemcpyAsync(&e, n->err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  CVO_CUDA_TRY(h, cudaStreamSynchronize(h->stream));
  if (!e) return CVO_OK;
  CVO_CUDA_TRY(h, cudaMemsetAsync(n->err, 0, sizeof(int), h->stream));
  h->last_error = "proposal network: a tensor-core GEMM gave up waiting for its MMAs";
  return CVO_ERR_TIMEOUT;
}

int net_set_gemm(NetDev *n, int kind) {
  if (kind != 0 && kind != 1) return CVO_ERR_INVALID_ARG;
  n->gemm_kind = kind;
  return CVO_OK;
}

int net_points(const NetDev *n) { return n->P; }

// Forward pass over the 2 Bn slots (pair b: source slot 2b, target slot 2b + 1):
// outputs in n->O, centroids of the moved clouds in n->cent.
static int net_forward(Handle *h, NetDev *n, int Bn, const std::vector<NetSlot> &slots, uint32_t seed) {
  NvtxRange nvtx_range("proposal_forward");
  int rc = net_ensure(h, n, Bn);
  if (rc) return rc;
  const int S = 2 * Bn, P = n->P;
  const long long rows = (long long)S * P;
  CVO_CUDA_TRY(h, cudaMemcpyAsync(n->slots, slots.data(), sizeof(NetSlot) * S, cudaMemcpyHostToDevice, h->stream));
  k_slot_mean<<<S, 256, 0, h->stream>>>(n->slots, n->mean, n->cent);
  k_net_inputs<<<(unsigned)((rows + 255) / 256), 256, 0, h->stream>>>(S, P, seed, n->slots, n->mean, n->X);
  h->launches += 2;
  gemm(h, n, true, (int)rows, kNetH1, kNetIn, n->X, kNetIn, 1, n->w + kOffW1, kNetH1, 1, n->w + kOffB1, n->H1, kNetH1);
  gemm(h, n, true, (int)rows, kNetH2, kNetH1, n->H1, kNetH1, 1, n->w + kOffW2, kNetH2, 1, n->w + kOffB2, n->H2, kNetH2);
  k_maxpool<<<(S * kNetH2 + 255) / 256, 256, 0, h->stream>>>(S, P, n->H2, n->G, n->arg);
  h->launches++;
  // [e_src, e_tgt] of pair b is row b of G viewed as Bn x 256
  gemm(h, n, true, Bn, kNetH3, kNetHead, n->G, kNetHead, 1, n->w + kOffW3, kNetH3, 1, n->w + kOffB3, n->H3, kNetH3);
  gemm(h, n, false, Bn, kNetOut, kNetH3, n->H3, kNetH3, 1, n->w + kOffW4, kNetOut, 1, n->w + kOffB4, n->O, kNetOut);
  CVO_CUDA_TRY(h, cudaGetLastError());
  return CVO_OK;
}

static NetSlot pool_slot(const float *base, int n_pts, int scene, const float *T12) {
  static const float I[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
  NetSlot s;
  s.xyz = base + (size_t)scene * n_pts * 8;
  s.feat = s.xyz + 3;
  s.xyz_stride = 8;
  s.feat_stride = 8;
  s.nfeat = 5;
  s.n = n_pts;
  std::memcpy(s.T, T12 ? T12 : I, sizeof(s.T));
  return s;
}

static int check_pool_args(int n_scenes, int n_pts, const float *src, const float *tgt, int Bn, const int *scene) {
  if (n_scenes <= 0 || n_pts <= 0 || !src || !tgt || Bn <= 0 || !scene) return CVO_ERR_INVALID_ARG;
  for (int b = 0; b < Bn; b++)
    if (scene[b] < 0 || scene[b] >= n_scenes) return CVO_ERR_INVALID_ARG;
  return 0;
}

static int hypotheses_out(Handle *h, NetDev *n, int Bn, float *raw_out, float *T_out) {
  k_hypotheses<<<(Bn * kNetK + 127) / 128, 128, 0, h->stream>>>(Bn, n->O, n->cent, n->Tout);
  h->launches++;
  if (raw_out)
    CVO_CUDA_TRY(h, cudaMemcpyAsync(raw_out, n->O, sizeof(float) * Bn * kNetOut, cudaMemcpyDeviceToHost, h->stream));
  if (T_out)
    CVO_CUDA_TRY(h, cudaMemcpyAsync(T_out, n->Tout, sizeof(float) * Bn * kNetK * 16, cudaMemcpyDeviceToHost,
                                    h->stream));
  return net_check(h, n);
}

// Forward over pool scenes (device arrays n_scenes x n_pts x 8: xyz + 5 features),
// the target of pair b moved by T_tgt[b] (row-major 3x4, may be null = identity).
int net_forward_pool(Handle *h, NetDev *n, int n_scenes, int n_pts, const float *src, const float *tgt, int Bn,
                     const int *scene, const float *T_tgt, uint32_t seed, float *raw_out, float *T_out) {
  int rc = check_pool_args(n_scenes, n_pts, src, tgt, Bn, scene);
  if (rc) return rc;
  std::vector<NetSlot> slots(2 * (size_t)Bn);
  for (int b = 0; b < Bn; b++) {
    slots[2 * b] = pool_slot(src, n_pts, scene[b], nullptr);
    slots[2 * b + 1] = pool_slot(tgt, n_pts, scene[b], T_tgt ? T_tgt + 12 * (size_t)b : nullptr);
  }
  if ((rc = net_forward(h, n, Bn, slots, seed))) return rc;
  return hypotheses_out(h, n, Bn, raw_out, T_out);
}

// Hypotheses for device clouds (original order: float4 positions, FP-strided features).
int net_hypotheses(Handle *h, NetDev *n, int Bn, DevCloud *const *src, DevCloud *const *tgt, uint32_t seed,
                   float *T_out) {
  static const float I[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
  if (Bn <= 0 || !src || !tgt || !T_out) return CVO_ERR_INVALID_ARG;
  std::vector<NetSlot> slots(2 * (size_t)Bn);
  for (int b = 0; b < Bn; b++)
    for (int side = 0; side < 2; side++) {
      const DevCloud *d = side ? tgt[b] : src[b];
      if (!d) return CVO_ERR_INVALID_ARG;
      NetSlot &s = slots[2 * b + side];
      s.xyz = reinterpret_cast<const float *>(d->pos);
      s.xyz_stride = 4;
      s.feat = d->feat;
      s.feat_stride = d->FP;
      s.nfeat = d->F;
      s.n = d->n;
      std::memcpy(s.T, I, sizeof(s.T));
    }
  int rc = net_forward(h, n, Bn, slots, seed);
  if (rc) return rc;
  return hypotheses_out(h, n, Bn, nullptr, T_out);
}

// Loss and gradients (kept in the gradient block) for Bn labelled pool pairs; with
// lr > 0 also one Adam step.  T_label: row-major 3x4 per pair (target = T source).
int net_train_pool(Handle *h, NetDev *n, int n_scenes, int n_pts, const float *src, const float *tgt, int Bn,
                   const int *scene, const float *T_label, float lr, uint32_t seed, float *loss_out) {
  NvtxRange nvtx_range("proposal_train");
  int rc = check_pool_args(n_scenes, n_pts, src, tgt, Bn, scene);
  if (rc) return rc;
  if (!T_label || !(lr >= 0.f)) return CVO_ERR_INVALID_ARG;
  std::vector<NetSlot> slots(2 * (size_t)Bn);
  for (int b = 0; b < Bn; b++) {
    slots[2 * b] = pool_slot(src, n_pts, scene[b], nullptr);
    slots[2 * b + 1] = pool_slot(tgt, n_pts, scene[b], T_label + 12 * (size_t)b);
  }
  if ((rc = net_forward(h, n, Bn, slots, seed))) return rc;
  const int S = 2 * Bn, P = n->P;
  const long long rows = (long long)S * P;
  const float *w = n->w;
  float *g = n->g;
  // split the row range of the encoder's weight gradients so that about 4 blocks per
  // SM run, each over at least 64 rows
  const int sms = h->num_sms > 0 ? h->num_sms : 152;
  auto split_for = [&](int tiles) {
    return (int)std::max<long long>(1, std::min<long long>((4LL * sms + tiles - 1) / tiles, rows / 64));
  };
  const int sp2 = split_for(2), sp1 = split_for(1);
  const size_t need = std::max<size_t>(
      {(size_t)gemm_splits(Bn, 2) * std::max(kNetH3 * kNetOut, kNetHead * kNetH3), (size_t)gemm_splits(rows, sp2) * kNetH1 * kNetH2,
       (size_t)gemm_splits(rows, sp1) * kNetIn * kNetH1, (size_t)colsum_blocks(rows) * kNetH2,
       (size_t)colsum_blocks(Bn) * std::max(kNetOut, kNetH3)});
  if (need > n->part_cap) {
    cudaFree(n->part);
    n->part = nullptr;
    n->part_cap = 0;
    if (cudaMalloc((void **)&n->part, sizeof(float) * need) != cudaSuccess) {
      cudaGetLastError();
      h->last_error = "out of device memory for the proposal network's gradient partials";
      return CVO_ERR_OUT_OF_MEMORY;
    }
    n->part_cap = need;
  }
  float *part = n->part;
  k_wta_loss<<<(Bn + 127) / 128, 128, 0, h->stream>>>(Bn, n->O, n->slots, n->cent, n->dO, n->loss, n->best);
  h->launches++;
  // head: O = H3 W4 + b4, H3 = relu(G' W3 + b3) with G' = G as Bn x 256
  gemm(h, n, false, kNetH3, kNetOut, Bn, n->H3, 1, kNetH3, n->dO, kNetOut, 1, nullptr, g + kOffW4, kNetOut, 2, part);
  colsum(h, Bn, kNetOut, n->dO, g + kOffB4, part);
  gemm(h, n, false, Bn, kNetH3, kNetOut, n->dO, kNetOut, 1, w + kOffW4, 1, kNetOut, nullptr, n->dH3, kNetH3);
  k_relu_bwd<<<(unsigned)(((long long)Bn * kNetH3 + 255) / 256), 256, 0, h->stream>>>((long long)Bn * kNetH3, n->H3,
                                                                                      n->dH3);
  gemm(h, n, false, kNetHead, kNetH3, Bn, n->G, 1, kNetHead, n->dH3, kNetH3, 1, nullptr, g + kOffW3, kNetH3, 2, part);
  colsum(h, Bn, kNetH3, n->dH3, g + kOffB3, part);
  gemm(h, n, false, Bn, kNetHead, kNetH3, n->dH3, kNetH3, 1, w + kOffW3, 1, kNetH3, nullptr, n->dG, kNetHead);
  // encoder: the max-pool routes dG to the pooled rows, then two ReLU layers
  CVO_CUDA_TRY(h, cudaMemsetAsync(n->dH2, 0, sizeof(float) * rows * kNetH2, h->stream));
  k_maxpool_bwd<<<(S * kNetH2 + 255) / 256, 256, 0, h->stream>>>(S, P, n->G, n->dG, n->arg, n->dH2);
  gemm(h, n, false, kNetH1, kNetH2, (int)rows, n->H1, 1, kNetH1, n->dH2, kNetH2, 1, nullptr, g + kOffW2, kNetH2, sp2,
       part);
  colsum(h, (int)rows, kNetH2, n->dH2, g + kOffB2, part);
  gemm(h, n, false, (int)rows, kNetH1, kNetH2, n->dH2, kNetH2, 1, w + kOffW2, 1, kNetH2, nullptr, n->dH1, kNetH1);
  k_relu_bwd<<<(unsigned)((rows * kNetH1 + 255) / 256), 256, 0, h->stream>>>(rows * kNetH1, n->H1, n->dH1);
  gemm(h, n, false, kNetIn, kNetH1, (int)rows, n->X, 1, kNetIn, n->dH1, kNetH1, 1, nullptr, g + kOffW1, kNetH1, sp1,
       part);
  colsum(h, (int)rows, kNetH1, n->dH1, g + kOffB1, part);
  h->launches += 3;
  if (lr > 0.f) {
    n->steps++;
    const float c1 = 1.f - (float)std::pow(0.9, (double)n->steps), c2 = 1.f - (float)std::pow(0.999, (double)n->steps);
    k_adam<<<(unsigned)((kNetParams + 255) / 256), 256, 0, h->stream>>>((int)kNetParams, n->w, n->g, n->m, n->v, lr,
                                                                        0.9f, 0.999f, 1e-8f, c1, c2);
    h->launches++;
  }
  CVO_CUDA_TRY(h, cudaGetLastError());
  std::vector<float> lh(Bn);
  CVO_CUDA_TRY(h, cudaMemcpyAsync(lh.data(), n->loss, sizeof(float) * Bn, cudaMemcpyDeviceToHost, h->stream));
  if (int rc_err = net_check(h, n)) return rc_err;
  if (loss_out) {
    double s = 0.0;
    for (float x : lh) s += x;
    *loss_out = (float)(s / Bn);
  }
  return CVO_OK;
}

int net_get(Handle *h, NetDev *n, int which, float *out) {
  const float *p = which == 0 ? n->w : which == 1 ? n->g : which == 2 ? n->m : which == 3 ? n->v : nullptr;
  if (!p || !out) return CVO_ERR_INVALID_ARG;
  CVO_CUDA_TRY(h, cudaStreamSynchronize(h->stream));
  CVO_CUDA_TRY(h, cudaMemcpy(out, p, sizeof(float) * kNetParams, cudaMemcpyDeviceToHost));
  return CVO_OK;
}

// New weights; the Adam state restarts.
int net_set(Handle *h, NetDev *n, const float *in) {
  if (!in) return CVO_ERR_INVALID_ARG;
  CVO_CUDA_TRY(h, cudaStreamSynchronize(h->stream));
  CVO_CUDA_TRY(h, cudaMemcpy(n->w, in, sizeof(float) * kNetParams, cudaMemcpyHostToDevice));
  CVO_CUDA_TRY(h, cudaMemset(n->m, 0, sizeof(float) * kNetParams));
  CVO_CUDA_TRY(h, cudaMemset(n->v, 0, sizeof(float) * kNetParams));
  n->steps = 0;
  return CVO_OK;
}

}  // namespace cvo_gb
