// cvo_device.cuh -- device helpers shared by the CVO kernels.
//
// Floating-point contract: every operation that decides whether a pair enters
// the sparse kernel matrix (target transform, squared distances, range-scaled
// lengthscale, thresholds) uses explicitly rounded intrinsics in a fixed order
// (no fused multiply-add), so the decisions match a CPU evaluation of the same
// expressions bit for bit.  Kernel values on the fast path use __expf; pairs
// whose value lies within a narrow band around the sparsification threshold
// are re-evaluated in double with exp(), the arithmetic of the reference
// (src/cvo/CvoGPU.cu:1023,1041,1050).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "cvo_internal.h"

namespace cvo_gb {

#define FULLMASK 0xFFFFFFFFu

__device__ __forceinline__ float fm(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fa(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fs(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double dm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double da(double a, double b) { return __dadd_rn(a, b); }

// ||p|| = sqrtf((x*x + y*y) + z*z)  (src/cvo/CvoGPU.cu:977)
__host__ __device__ __forceinline__ float range_norm(float x, float y, float z) {
#ifdef __CUDA_ARCH__
  return __fsqrt_rn(fa(fa(fm(x, x), fm(y, y)), fm(z, z)));
#else
  float a = x * x, b = y * y, c = z * z;
  return sqrtf((a + b) + c);
#endif
}

// compute_range_ell (src/cvo/CvoGPU.cu:90-94): ((d / 500.0 + 1.0) * ell) in double
__device__ __forceinline__ float range_ell(float ell, float dist) {
  return __double2float_rn(dm(da(__ddiv_rn((double)dist, 500.0), 1.0), (double)ell));
}

// d2_thres = -2.0 * l * l * log(sp_thres / sigma^2)   (src/cvo/CvoGPU.cu:981-982)
__device__ __forceinline__ float geo_d2_thres(float l, float log_geo) {
  return __double2float_rn(dm(dm(dm(-2.0, (double)l), (double)l), (double)log_geo));
}

// squared_dist of two points (include/UnifiedCvo/cvo/gpu_utils.cuh:61-66)
__device__ __forceinline__ float sqdist3(float ax, float ay, float az, float bx, float by, float bz) {
  float dx = fs(ax, bx), dy = fs(ay, by), dz = fs(az, bz);
  return fa(fa(fm(dx, dx), fm(dy, dy)), fm(dz, dz));
}

// y' = Ri * y + Ti in the canonical order ((r0*y0 + r1*y1) + r2*y2) + t
__device__ __forceinline__ float xform_row(const float *r, float t, float x, float y, float z) {
  return fa(fa(fa(fm(r[0], x), fm(r[1], y)), fm(r[2], z)), t);
}

__host__ __device__ __forceinline__ unsigned long long cell_key(int cx, int cy, int cz) {
  return ((unsigned long long)(unsigned)cx << 42) | ((unsigned long long)(unsigned)cy << 21) |
         (unsigned long long)(unsigned)cz;
}

__host__ __device__ __forceinline__ unsigned long long cell_hash(unsigned long long k) {
  k ^= k >> 33;
  k *= 0xff51afd7ed558ccdull;
  k ^= k >> 33;
  k *= 0xc4ceb9fe1a85ec53ull;
  k ^= k >> 33;
  return k;
}

// Returns (start, count) of a grid cell, (0, 0) if empty or outside the grid.
__device__ __forceinline__ int2 grid_lookup(const GridDesc &g, int cx, int cy, int cz) {
  if (cx < 0 || cy < 0 || cz < 0 || cx >= g.dimx || cy >= g.dimy || cz >= g.dimz) return make_int2(0, 0);
  unsigned long long key = cell_key(cx, cy, cz);
  unsigned int mask = (1u << g.tbits) - 1u;
  unsigned int slot = (unsigned int)cell_hash(key) & mask;
  for (unsigned int probe = 0; probe <= mask; probe++) {
    unsigned long long k = __ldg(&g.keys[slot]);
    if (k == key) return make_int2(__ldg(&g.cstart[slot]), __ldg(&g.ccount[slot]));
    if (k == kEmptyKey) return make_int2(0, 0);
    slot = (slot + 1u) & mask;
  }
  return make_int2(0, 0);
}

__device__ __forceinline__ float warp_min(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(FULLMASK, v, o));
  return v;
}
__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(FULLMASK, v, o));
  return v;
}
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULLMASK, v, o);
  return v;
}
__device__ __forceinline__ float warp_sumf(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULLMASK, v, o);
  return v;
}
__device__ __forceinline__ int warp_sumi(int v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULLMASK, v, o);
  return v;
}
__device__ __forceinline__ int warp_maxi(int v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(FULLMASK, v, o));
  return v;
}

// Shared-memory address of a generic pointer (for ldmatrix).
__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

constexpr float kBand = 2e-5f;      // relative band around sp_thres re-evaluated in double

// Exact kernel value as the reference computes it (double exp, float products);
// used only for pairs whose fast FP32 value is within kBand of the threshold,
// so it is kept out of line to keep the hot loop's register count low.
static __device__ __noinline__ float exact_value(const KParams &K, float l, float d2, float d2c, float d2s, float geo) {
  float kk = 1.f, ck = 1.f, sk = 1.f;
  if (K.val_scale != 1.f && K.use_geo && !K.use_int && !K.use_sem)   // one double expression, rounded once
    return __double2float_rn(dm(dm((double)K.sigma2, exp(__ddiv_rn(-(double)d2, dm(dm(2.0, (double)l), (double)l)))),
                                (double)K.val_scale));
  if (K.use_geo) kk = __double2float_rn(dm((double)K.sigma2, exp(__ddiv_rn(-(double)d2, dm(dm(2.0, (double)l), (double)l)))));
  if (K.use_int) ck = __double2float_rn(dm((double)K.c_sigma2, exp(__ddiv_rn(-(double)d2c, K.two_c2))));
  if (K.use_sem)
    sk = __double2float_rn(dm((double)K.s_sigma_sq, exp(__ddiv_rn(-(double)d2s, dm(dm(2.0, (double)K.s_ell), (double)K.s_ell)))));
  return fm(fm(fm(ck, kk), sk), geo);
}

// Pair index of a flat work item, by binary search in an offsets array.
__device__ __forceinline__ int find_segment(const int *off, int nseg, int item) {
  int lo = 0, hi = nseg - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (__ldg(&off[mid]) <= item) lo = mid; else hi = mid - 1;
  }
  return lo;
}

}  // namespace cvo_gb
