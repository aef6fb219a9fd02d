// cvo_noalloc.cu -- an inner product that allocates no memory.
//
// Some callers cannot allocate device memory at the time they need a result:
// code running inside a real-time loop with a fixed memory budget, code that
// hands every buffer out of its own pre-reserved pool, or a plugin whose host
// process forbids cudaMalloc after start-up.  cvo_inner_product_noalloc serves
// them: the caller passes device-resident clouds and a device output word, and
// the only scratch the computation needs (one partial sum per thread block and a
// completion counter) lives in a fixed-size array compiled into this library.
//
// The pass is the index-ordered variant of the association: every source row
// scans the targets in ascending index and keeps the first nearest_neighbors_max
// pairs whose kernel value exceeds sp_thres -- the set the reference's
// fill_in_A_mat_gpu keeps (src/cvo/CvoGPU.cu:994-1075) -- so it needs no spatial
// grid (building one would allocate).  It costs O(N * M) pair tests, so a call
// is also limited to kNoAllocMaxPairTests (N * M <= 2^33, e.g. 92k x 92k
// points), which keeps one launch well under a few seconds on a GB300.
//
// Limits and sharing: at most kNoAllocMaxRows source points per call.  All
// calls in the process share the one scratch array and leave their partial sums
// in it; a call clears the completion counter before it starts, but two calls
// whose kernels overlap on the GPU (different streams, or host threads without
// ordering) race on the array and produce wrong results.  The first call on a
// device looks up the array's device address (cudaGetSymbolAddress) with that
// device current; make that first call before any stream capture.
#include <atomic>
#include <cmath>
#include <cstring>
#include "cvo_internal.h"
#include "cvo_device.cuh"

namespace cvo_gb {
namespace {

constexpr int kNoAllocThreads = 128;
constexpr int kNoAllocMaxBlocks = 8192;
constexpr int kNoAllocMaxRows = kNoAllocThreads * kNoAllocMaxBlocks;   // 1,048,576 source points
constexpr int kNoAllocMaxDevices = 64;
constexpr long long kNoAllocMaxPairTests = 1LL << 33;                   // N * M per call

// [0, 256): completion counter (unsigned int); [256, ...): one double per block
constexpr size_t kScratchBytes = 256 + sizeof(double) * kNoAllocMaxBlocks;   // 65,792 bytes
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// device address of g_noalloc_scratch, per device (looked up on first use)
std::atomic<void *> g_scratch_addr[kNoAllocMaxDevices];
std::atomic_flag g_setup_lock = ATOMIC_FLAG_INIT;

struct NoAllocArgs {
  const float *sx, *sf, *sl, *sg;   // source xyz (stride sxs), features, labels, geometric types
  const float *tx, *tf, *tl, *tg;   // target
  int sxs, txs;
  int n, m, F, C, cap;
  float Ri[9], Ti[3];               // target transform R^T, -R^T T
  float ell;
};

// One thread per source row; all threads of a block walk the targets in the
// same order, so every target load is a broadcast.  Arithmetic follows the
// grid path exactly (same canonical operation order), so the kept set and the
// kernel values are the same as cvo_inner_product's.
__global__ void __launch_bounds__(kNoAllocThreads) k_ip_index_order(NoAllocArgs A, KParams K, unsigned char *scratch,
                                                                     float *out) {
  __shared__ double sh[kNoAllocThreads / 32];
  __shared__ bool last;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double rowsum = 0.0;
  if (i < A.n) {
    const float x0 = A.sx[(size_t)i * A.sxs], x1 = A.sx[(size_t)i * A.sxs + 1], x2 = A.sx[(size_t)i * A.sxs + 2];
    const float nrm = range_norm(x0, x1, x2);
    const float l = range_ell(A.ell, nrm);
    const float d2t = K.use_geo ? geo_d2_thres(l, K.log_geo) : INFINITY;
    const float inv2l2 = __frcp_rn(fm(fm(2.f, l), l));
    float asum = 0.f;
    int kept = 0;
    for (int j = 0; j < A.m && kept < A.cap; j++) {
      const float *yp = A.tx + (size_t)j * A.txs;
      const float y0 = xform_row(&A.Ri[0], A.Ti[0], yp[0], yp[1], yp[2]);
      const float y1 = xform_row(&A.Ri[3], A.Ti[1], yp[0], yp[1], yp[2]);
      const float y2 = xform_row(&A.Ri[6], A.Ti[2], yp[0], yp[1], yp[2]);
      float geo = 1.f;
      if (K.use_gtype) {
        const float *ga = A.sg + 2 * (size_t)i, *gb = A.tg + 2 * (size_t)j;
        float n2a = fa(fm(ga[0], ga[0]), fm(ga[1], ga[1]));
        float n2b = fa(fm(gb[0], gb[0]), fm(gb[1], gb[1]));
        float dab = fa(fm(ga[0], gb[0]), fm(ga[1], gb[1]));
        geo = __fdiv_rn(fm(dab, dab), fm(n2a, n2b));
        if ((double)geo < 0.01) continue;
      }
      float d2 = 0.f;
      if (K.use_geo) {
        d2 = sqdist3(y0, y1, y2, x0, x1, x2);
        if (!(d2 < d2t)) continue;
      }
      float d2c = 0.f;
      if (K.use_int) {
        for (int q = 0; q < A.F; q++) {
          float t = fs(A.sf[(size_t)i * A.F + q], A.tf[(size_t)j * A.F + q]);
          d2c = fa(d2c, fm(t, t));
        }
        if (!(d2c < K.d2_c_thres)) continue;
      }
      float d2s = 0.f;
      if (K.use_sem) {
        for (int q = 0; q < A.C; q++) {
          float t = fs(A.sl[(size_t)i * A.C + q], A.tl[(size_t)j * A.C + q]);
          d2s = fa(d2s, fm(t, t));
        }
        if (!(d2s < K.d2_s_thres)) continue;
      }
      float kf = K.use_geo ? fm(K.sigma2, __expf(fm(-d2, inv2l2))) : 1.f;
      float ckf = K.use_int ? fm(K.c_sigma2, __expf(fm(-d2c, __frcp_rn(fm(2.f, K.c2))))) : 1.f;
      float skf = K.use_sem ? fm(K.s_sigma_sq, __expf(fm(-d2s, __frcp_rn(fm(fm(2.f, K.s_ell), K.s_ell))))) : 1.f;
      float a = fm(fm(fm(ckf, kf), skf), geo);
      if (fabsf(fs(a, K.sp_thres)) <= 2e-5f * K.sp_thres) {
        float kk = 1.f, ck = 1.f, sk = 1.f;
        if (K.use_geo) kk = __double2float_rn(dm((double)K.sigma2, exp(__ddiv_rn(-(double)d2, dm(dm(2.0, (double)l), (double)l)))));
        if (K.use_int) ck = __double2float_rn(dm((double)K.c_sigma2, exp(__ddiv_rn(-(double)d2c, dm(2.0, (double)K.c2)))));
        if (K.use_sem)
          sk = __double2float_rn(dm((double)K.s_sigma_sq, exp(__ddiv_rn(-(double)d2s, dm(dm(2.0, (double)K.s_ell), (double)K.s_ell)))));
        a = fm(fm(fm(ck, kk), sk), geo);
      }
      if (a > K.sp_thres) {
        asum += a;
        kept++;
      }
    }
    rowsum = asum;
  }
  // block sum -> this block's slot of the scratch array; the last block to
  // finish sums the slots in block order (deterministic) into *out
  double v = warp_sum(rowsum);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  unsigned int *counter = reinterpret_cast<unsigned int *>(scratch);
  double *partial = reinterpret_cast<double *>(scratch + 256);
  if (threadIdx.x == 0) {
    double b = 0.0;
    for (int w = 0; w < kNoAllocThreads / 32; w++) b += sh[w];
    partial[blockIdx.x] = b;
    __threadfence();
    unsigned prev = atomicAdd(counter, 1u);
    last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (!last || threadIdx.x != 0) return;
  __threadfence();
  volatile double *pv = partial;
  double tot = 0.0;
  for (unsigned b = 0; b < gridDim.x; b++) tot += pv[b];
  *out = (float)tot;
}

// Looks up (once per device) the device address of the scratch array.
int scratch_for_current_device(unsigned char **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return CVO_ERR_CUDA;
  if (dev < 0 || dev >= kNoAllocMaxDevices) return CVO_ERR_UNSUPPORTED;
  void *p = g_scratch_addr[dev].load(std::memory_order_acquire);
  if (!p) {
    while (g_setup_lock.test_and_set(std::memory_order_acquire)) {
    }
    p = g_scratch_addr[dev].load(std::memory_order_relaxed);
    if (!p) {
      e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess || !p) {
        g_setup_lock.clear(std::memory_order_release);
        cudaGetLastError();
        return CVO_ERR_CUDA;
      }
      g_scratch_addr[dev].store(p, std::memory_order_release);
    }
    g_setup_lock.clear(std::memory_order_release);
  }
  *out = static_cast<unsigned char *>(p);
  return CVO_OK;
}

}  // namespace
}  // namespace cvo_gb

using namespace cvo_gb;

// See include/cvo_gb300.h.
extern "C" int cvo_inner_product_noalloc(const cvo_params *p, const cvo_cloud *src_dev, const cvo_cloud *tgt_dev,
                                         const float T[16], float ell, float *out_dev, void *cuda_stream) {
  if (!p || !src_dev || !tgt_dev || !T || !out_dev) return CVO_ERR_INVALID_ARG;
  if (src_dev->n < 0 || tgt_dev->n < 0 || src_dev->F != tgt_dev->F || src_dev->C != tgt_dev->C)
    return CVO_ERR_INVALID_ARG;
  if (src_dev->n > kNoAllocMaxRows) return CVO_ERR_CAPACITY;   // more rows than the scratch array serves
  if ((long long)src_dev->n * (long long)tgt_dev->n > kNoAllocMaxPairTests) return CVO_ERR_CAPACITY;
  if ((src_dev->n > 0 && !src_dev->xyz) || (tgt_dev->n > 0 && !tgt_dev->xyz)) return CVO_ERR_INVALID_ARG;
  if ((src_dev->xyz_stride != 3 && src_dev->xyz_stride != 4) || (tgt_dev->xyz_stride != 3 && tgt_dev->xyz_stride != 4))
    return CVO_ERR_INVALID_ARG;
  if (p->is_using_intensity && src_dev->F > 0 && (!src_dev->features || !tgt_dev->features)) return CVO_ERR_INVALID_ARG;
  if (p->is_using_semantics && src_dev->C > 0 && (!src_dev->labels || !tgt_dev->labels)) return CVO_ERR_INVALID_ARG;
  if (p->is_using_geometric_type && (!src_dev->geom_type || !tgt_dev->geom_type)) return CVO_ERR_INVALID_ARG;
  cudaStream_t st = (cudaStream_t)cuda_stream;
  unsigned char *scratch = nullptr;
  int rc = scratch_for_current_device(&scratch);
  if (rc) return rc;
  if (src_dev->n == 0 || tgt_dev->n == 0) {
    if (cudaMemsetAsync(out_dev, 0, sizeof(float), st) != cudaSuccess) return CVO_ERR_CUDA;
    return CVO_OK;
  }
  KParams K = make_kparams(*p);
  NoAllocArgs A;
  memset(&A, 0, sizeof(A));
  A.sx = src_dev->xyz; A.sf = src_dev->features; A.sl = src_dev->labels; A.sg = src_dev->geom_type;
  A.tx = tgt_dev->xyz; A.tf = tgt_dev->features; A.tl = tgt_dev->labels; A.tg = tgt_dev->geom_type;
  A.sxs = src_dev->xyz_stride; A.txs = tgt_dev->xyz_stride;
  A.n = src_dev->n; A.m = tgt_dev->n; A.F = src_dev->F; A.C = src_dev->C;
  A.cap = p->nearest_neighbors_max > 0 ? p->nearest_neighbors_max : 0;
  A.ell = ell;
  {
    // target moved by inverse(T): R^T, -R^T t in the canonical order
    float R[9], t[3];
    for (int r = 0; r < 3; r++) { for (int c = 0; c < 3; c++) R[3 * r + c] = T[c * 4 + r]; t[r] = T[12 + r]; }
    for (int r = 0; r < 3; r++) for (int c = 0; c < 3; c++) A.Ri[3 * r + c] = R[3 * c + r];
    for (int r = 0; r < 3; r++) {
      float a = A.Ri[3 * r] * t[0], b = A.Ri[3 * r + 1] * t[1], c = A.Ri[3 * r + 2] * t[2];
      A.Ti[r] = -((a + b) + c);
    }
  }
  // the completion counter must start at zero
  if (cudaMemsetAsync(scratch, 0, sizeof(unsigned int), st) != cudaSuccess) return CVO_ERR_CUDA;
  const int blocks = (A.n + kNoAllocThreads - 1) / kNoAllocThreads;
  k_ip_index_order<<<blocks, kNoAllocThreads, 0, st>>>(A, K, scratch, out_dev);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? CVO_OK : CVO_ERR_CUDA;
}
