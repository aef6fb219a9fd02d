// cvo_kernels.cuh -- per-iteration kernels of the batched CVO engine.
//
// One iteration of the reference's align loop (src/cvo/CvoGPU.cu:1303-1433) is a
// fixed sequence of launches over every active pair of a batch:
//   k_transform  target transform y' = R^T (y - T)            (CvoGPU_impl.cu:32-83)
//   k_assoc_cta  association: grid candidates -> tensor-core prefilter -> exact kernel
//                value -> threshold -> ELL row (first cap) + spill list (the rest)
//                (cvo_assoc_cta.cuh; per-warp path assoc_warp below)
//                                                               (CvoGPU.cu:951-1099)
//   k_select / k_rescan  rows with more than cap kept pairs: their cap smallest indices
//   k_rowsum     per-row gradient partials from the final ELL    (CvoGPU.cu:2001-2062)
//   k_reduce     per-pair FP64 sums of the row partials; gradient normalisation
//                                                               (CvoGPU.cu:2065-2120)
//   k_step       Taylor step-size terms over the ELL rows; the last block of each pair
//                runs the scalar tail of the iteration: cubic roots, step clamp,
//                Exp_SEK3 pose update, SE(3) distance, lengthscale schedule, cap update
//                                                               (CvoGPU.cu:333-544, 547-665, 1339-1433)
#pragma once
#include <cuda_fp16.h>
#include "cvo_device.cuh"

namespace cvo_gb {

enum { MODE_ALIGN = 0, MODE_IP = 1, MODE_EXPORT = 2 };
constexpr int kAssocThreads = 128;
constexpr int kReduceRows = 1024;
constexpr int kReduceThreads = 256;
constexpr int kStepThreads = 256;
constexpr int kPartStride = 12;

// ------------------------------------------------------------ pair value
// Kernel value of one (source, target) pair with the semantics of
// fill_in_A_mat_gpu (src/cvo/CvoGPU.cu:996-1075).  `pre` is the lane's
// participation; returns whether the pair is kept and its value in a.
// All lanes of the warp must call it together.
template <int FCH, int LCH, bool GT>
__device__ __forceinline__ bool eval_pair(const KParams &K, int F, int C, bool pre, float l, float d2t, float inv2l2,
                                          const float4 &x, const float4 (&xf)[FCH > 0 ? FCH : 1],
                                          const float4 (&xl)[LCH > 0 ? LCH : 1], float2 xg, const float4 &y,
                                          const float4 *yfp, const float4 *ylp, const float4 *ygp, float &a) {
  bool pass = pre;
  float d2 = 0.f;
  if (K.use_geo) {
    d2 = sqdist3(y.x, y.y, y.z, x.x, x.y, x.z);
    pass = pass && (d2 < d2t);
  }
  if (!__any_sync(FULLMASK, pass)) return false;
  float geo = 1.f;
  if (GT) {
    float4 yg = *ygp;
    float n2a = fa(fm(xg.x, xg.x), fm(xg.y, xg.y));
    float n2b = fa(fm(yg.x, yg.x), fm(yg.y, yg.y));
    float dab = fa(fm(xg.x, yg.x), fm(xg.y, yg.y));
    geo = __fdiv_rn(fm(dab, dab), fm(n2a, n2b));
    pass = pass && !((double)geo < 0.01);
  }
  float d2c = 0.f;
  if (FCH > 0 && K.use_int) {
#pragma unroll
    for (int q = 0; q < FCH; q++) {
      float4 yf = yfp[q];
      float av[4] = {xf[q].x, xf[q].y, xf[q].z, xf[q].w};
      float bv[4] = {yf.x, yf.y, yf.z, yf.w};
#pragma unroll
      for (int r = 0; r < 4; r++)
        if (4 * q + r < F) { float t = fs(av[r], bv[r]); d2c = fa(d2c, fm(t, t)); }
    }
    pass = pass && (d2c < K.d2_c_thres);
  } else if (K.use_int) {
    pass = pass && (d2c < K.d2_c_thres);
  }
  float d2s = 0.f;
  if (LCH > 0 && K.use_sem) {
#pragma unroll
    for (int q = 0; q < LCH; q++) {
      float4 yl = ylp[q];
      float av[4] = {xl[q].x, xl[q].y, xl[q].z, xl[q].w};
      float bv[4] = {yl.x, yl.y, yl.z, yl.w};
#pragma unroll
      for (int r = 0; r < 4; r++)
        if (4 * q + r < C) { float t = fs(av[r], bv[r]); d2s = fa(d2s, fm(t, t)); }
    }
    pass = pass && (d2s < K.d2_s_thres);
  } else if (K.use_sem) {
    pass = pass && (d2s < K.d2_s_thres);
  }
  if (!__any_sync(FULLMASK, pass)) return false;
  // fast FP32 value
  float kf = K.use_geo ? fm(K.sigma2, __expf(fm(-d2, inv2l2))) : 1.f;
  float ckf = K.use_int ? fm(K.c_sigma2, __expf(fm(-d2c, K.inv2c2))) : 1.f;
  float skf = K.use_sem ? fm(K.s_sigma_sq, __expf(fm(-d2s, __frcp_rn(fm(fm(2.f, K.s_ell), K.s_ell))))) : 1.f;
  float af = fm(fm(fm(fm(ckf, kf), skf), geo), K.val_scale);
  if (pass && fabsf(fs(af, K.sp_thres)) <= kBand * K.sp_thres) af = exact_value(K, l, d2, d2c, d2s, geo);
  a = af;
  return pass && (af > K.sp_thres);
}

// Per-source-point kernel constants.
struct RowConst {
  float l, d2t, inv2l2, rq;
};

__device__ __forceinline__ RowConst row_const(const KParams &K, float ell, float norm, float Tn) {
  RowConst rc;
  rc.l = range_ell(ell, norm);
  rc.d2t = K.use_geo ? geo_d2_thres(rc.l, K.log_geo) : INFINITY;
  rc.inv2l2 = __frcp_rn(fm(fm(2.f, rc.l), rc.l));
  rc.rq = K.use_geo ? sqrtf(rc.d2t) * 1.00001f + 1e-5f * (norm + Tn + sqrtf(rc.d2t)) + 1e-6f : 0.f;
  return rc;
}

// Cell range of the box [lo, hi] in grid g; returns false if empty.
__device__ __forceinline__ bool cell_range(const GridDesc &g, float lox, float loy, float loz, float hix, float hiy,
                                           float hiz, int &x0, int &y0, int &z0, int &nx, int &ny, int &nz) {
  if (g.dimx == 1 && g.dimy == 1 && g.dimz == 1 && g.inv_h == 0.f) {
    x0 = y0 = z0 = 0; nx = ny = nz = 1;
    return true;
  }
  float a0 = floorf((lox - g.ox) * g.inv_h), a1 = floorf((hix - g.ox) * g.inv_h);
  float b0 = floorf((loy - g.oy) * g.inv_h), b1 = floorf((hiy - g.oy) * g.inv_h);
  float c0 = floorf((loz - g.oz) * g.inv_h), c1 = floorf((hiz - g.oz) * g.inv_h);
  if (!(a1 >= 0.f && b1 >= 0.f && c1 >= 0.f)) return false;
  if (!(a0 < (float)g.dimx && b0 < (float)g.dimy && c0 < (float)g.dimz)) return false;
  x0 = (int)fmaxf(a0, 0.f); int x1 = (int)fminf(a1, (float)(g.dimx - 1));
  y0 = (int)fmaxf(b0, 0.f); int y1 = (int)fminf(b1, (float)(g.dimy - 1));
  z0 = (int)fmaxf(c0, 0.f); int z1 = (int)fminf(c1, (float)(g.dimz - 1));
  nx = x1 - x0 + 1; ny = y1 - y0 + 1; nz = z1 - z0 + 1;
  return nx > 0 && ny > 0 && nz > 0;
}

// ------------------------------------------------------------- transform
// Writes the transformed targets twice: in grid order (read by the association
// scan) and in original order (gathered by index from the ELL rows).
__global__ void k_transform(BatchDev B) {
  int gt = blockIdx.x * blockDim.x + threadIdx.x;
  if (gt == 0) {
    if (*B.active > 0) *B.active_iters += 1;
    *B.sel_count = 0;
    *B.scan_count = 0;
    *B.assoc_next = 0;
  }
  if (gt >= B.total_targets) return;
  int p = find_segment(B.tgt_off, B.npairs, gt);
  PairDev *P = &B.pairs[p];
  if (P->done) return;
  int t = gt - B.tgt_off[p];
  const GridDesc &G = P->levels[P->level];
  float4 y = __ldg(&G.pos[t]);
  float o0 = xform_row(&P->Ri[0], P->Ti[0], y.x, y.y, y.z);
  float o1 = xform_row(&P->Ri[3], P->Ti[1], y.x, y.y, y.z);
  float o2 = xform_row(&P->Ri[6], P->Ti[2], y.x, y.y, y.z);
  float4 o = make_float4(o0, o1, o2, y.w);
  P->ycur[t] = o;
  P->yorig[__float_as_int(y.w)] = o;
}

// -------------------------------------------------------- row selection
// The reference keeps the first `cap` kept pairs of a row in ascending target
// index (its scan stops at `cap`, src/cvo/CvoGPU.cu:994-996).  Here candidates
// arrive in grid order, so k_assoc writes the first `cap` kept pairs of a row to
// its ELL slots and the first `ov` to the row's list (row-major); a row that kept
// more than `cap` is listed, and k_select (count <= ov) or k_rescan (count > ov)
// rewrites its ELL row with the `cap` smallest kept indices, i.e. the
// reference's set.
struct EllRow {
  int *j;
  float *v;
  size_t stride;
  __device__ __forceinline__ int &J(int c) const { return j[(size_t)c * stride]; }
  __device__ __forceinline__ float &V(int c) const { return v[(size_t)c * stride]; }
};

// ------------------------------------------------------- candidate staging
// A chunk of up to CH candidate targets in shared memory.  The grid stores the
// members of one cell contiguously (positions, features, labels, geometric
// types); the warp fills a chunk from consecutive cells with 16-byte loads.
template <int FCH, int LCH, bool GT>
struct __align__(16) StageBuf {
  static constexpr int CH = (LCH > 5) ? 16 : 32;
  float4 pos[CH];
  float4 feat[CH * (FCH > 0 ? FCH : 1)];
  float4 lab[CH * (LCH > 0 ? LCH : 1)];
  float4 geo[GT ? CH : 1];
};

// Copies the nk grid-order candidates t0 .. t0+nk-1 into slots at .. at+nk-1 of a
// staging buffer; the warp copies each array (positions, features, labels,
// geometric types) as one contiguous run of 16-byte vectors.
template <int FCH, int LCH, bool GT>
__device__ __forceinline__ void stage_piece(StageBuf<FCH, LCH, GT> &buf, const float4 *ycur, const GridDesc &G,
                                            int at, int t0, int nk, int lane) {
#pragma unroll 1
  for (int i = lane; i < nk; i += 32) buf.pos[at + i] = __ldg(ycur + t0 + i);
  if (FCH > 0) {
    const float4 *src = reinterpret_cast<const float4 *>(G.feat) + (size_t)t0 * FCH;
#pragma unroll 1
    for (int i = lane; i < nk * FCH; i += 32) buf.feat[at * FCH + i] = __ldg(src + i);
  }
  if (LCH > 0) {
    const float4 *src = reinterpret_cast<const float4 *>(G.lab) + (size_t)t0 * LCH;
#pragma unroll 1
    for (int i = lane; i < nk * LCH; i += 32) buf.lab[at * LCH + i] = __ldg(src + i);
  }
  if (GT) {
#pragma unroll 1
    for (int i = lane; i < nk; i += 32) buf.geo[at + i] = __ldg(G.geo + t0 + i);
  }
}

// ------------------------------------------------- tensor-core prefilter
// A kept pair satisfies  u = g_s |x - y|^2 + c |xc - yc|^2 < tau  with
// g_s = 1/(2 l_s^2), c = 1/(2 c_ell^2), tau = ln(sigma^2 c_sigma^2 s_sigma^2 / sp_thres)
// (+ slack): the kernel value is at most the product of the three scales times
// exp(-u), and the geometric-type factor is at most 1.  Around a per-warp centre
// p (x~ = x - p, y~ = y - p) u is the inner product of two 16-vectors,
//   A_s = [-2 g x~ | -2 c xc | g | c | g|x~|^2 + c|xc|^2 | -kappa |A_s| | 0]
//   B_t = [ y~     |  yc     | |y~|^2 | |yc|^2 | 1       |  |B_t|        | 0]
// so a 32-source x 32-candidate tile of u is a 32x32x16 GEMM.  Each vector is
// split into f16 hi + lo parts and the tile is Ahi*Bhi + Ahi*Blo + Alo*Bhi
// (mma.sync m16n8k16, FP32 accumulation): the error is below 2^-16 |A||B|, and
// the -kappa |A||B| column (kappa = 2^-12) lowers u by more than that, so the
// test "u < tau" never rejects a pair the exact evaluation keeps.  Only pairs
// that pass go through the exact per-pair arithmetic (eval_pair), in the same
// candidate order as an unfiltered scan, so the kernel matrix is unchanged.
constexpr float kMmaKappa = 1.f / 4096.f;
constexpr float kMmaMaxAbs = 6.0e4f;    // larger components would leave the f16 range: no filtering

struct __align__(16) MmaTile {
  uint4 a[4][32];   // source rows:  [hi k0-7, hi k8-15, lo k0-7, lo k8-15][row]
  uint4 b[4][32];   // candidates:   same layout
};

__device__ __forceinline__ float f4_at(const float4 &v, int i) {
  return i == 0 ? v.x : (i == 1 ? v.y : (i == 2 ? v.z : v.w));
}

// Splits v into f16 hi + lo and stores entry `idx` of the 4 planes (plane p at
// dst + p * stride); returns false
// if a component is outside the f16-safe range (or not finite).
__device__ __forceinline__ bool mma_store_vec(const float (&v)[16], uint4 *dst, int stride, int idx) {
  uint32_t hw[8], lw[8];
  bool ok = true;
#pragma unroll
  for (int i = 0; i < 8; i++) {
    float v0 = v[2 * i], v1 = v[2 * i + 1];
    ok = ok && (fabsf(v0) <= kMmaMaxAbs) && (fabsf(v1) <= kMmaMaxAbs);
    __half h0 = __float2half_rn(v0), h1 = __float2half_rn(v1);
    __half l0 = __float2half_rn(v0 - __half2float(h0)), l1 = __float2half_rn(v1 - __half2float(h1));
    hw[i] = (uint32_t)__half_as_ushort(h0) | ((uint32_t)__half_as_ushort(h1) << 16);
    lw[i] = (uint32_t)__half_as_ushort(l0) | ((uint32_t)__half_as_ushort(l1) << 16);
  }
  dst[idx] = make_uint4(hw[0], hw[1], hw[2], hw[3]);
  dst[stride + idx] = make_uint4(hw[4], hw[5], hw[6], hw[7]);
  dst[2 * stride + idx] = make_uint4(lw[0], lw[1], lw[2], lw[3]);
  dst[3 * stride + idx] = make_uint4(lw[4], lw[5], lw[6], lw[7]);
  return ok;
}

__device__ __forceinline__ void ldsm_x4(const void *p, uint32_t &r0, uint32_t &r1, uint32_t &r2, uint32_t &r3) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0, %1, %2, %3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(smem_addr(p))
               : "memory");
}

__device__ __forceinline__ void mma_16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
      "{%0, %1, %2, %3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Row partials as k_reduce reads them: omega / c, v / d (align mode only), sum of a.
__device__ __forceinline__ void write_row_sums(float *rs, int mode, const KParams &K, float w0, float w1, float w2,
                                               float v0, float v1, float v2, float as) {
  if (mode == MODE_ALIGN) {
    rs[0] = __fdiv_rn(w0, K.c); rs[1] = __fdiv_rn(w1, K.c); rs[2] = __fdiv_rn(w2, K.c);
    rs[3] = __fdiv_rn(v0, K.d); rs[4] = __fdiv_rn(v1, K.d); rs[5] = __fdiv_rn(v2, K.d);
  } else {
    rs[0] = rs[1] = rs[2] = rs[3] = rs[4] = rs[5] = 0.f;
  }
  rs[6] = as;
}

// The warp's 32 source rows, for lanes that evaluate another lane's row.
template <int FCH, int LCH>
struct __align__(16) SrcRows {
  float4 x[32];                                // position, ||x||
  float4 rc[32];                               // l, d2 threshold, 1 / (2 l^2), geometric type g0
  float4 f[32 * (FCH > 0 ? FCH : 1)];
  float4 l[32 * (LCH > 0 ? LCH : 1)];
  float g1[32];                                // geometric type g1
};

// Position of the (n+1)-th set bit of m (n >= 0, m has more than n set bits):
// a binary search on population counts of the low halves, fixed latency.
__device__ __forceinline__ int nth_set_bit(uint32_t m, int n) {
  int pos = 0;
#pragma unroll
  for (int w = 16; w > 0; w >>= 1) {
    const uint32_t low = (m >> pos) & ((1u << w) - 1u);
    const int c = __popc(low);
    if (n >= c) {
      n -= c;
      pos += w;
    }
  }
  return pos;
}

// Kept count of a finished row; a row with more than cap kept pairs is listed for
// k_select (its ELL row and its spill list hold them all) or k_rescan.
__device__ __forceinline__ void finish_row(const BatchDev &B, PairDev *P, int p, int s, int cnt, int cap, int ov) {
  P->nnz_row[s] = cnt < cap ? cnt : cap;
  if (cnt > cap && cap > 0) {
    if (cnt - cap <= ov) B.sel_list[atomicAdd(B.sel_count, 1)] = make_int4(p, s, cnt, 0);
    else B.scan_list[atomicAdd(B.scan_count, 1)] = make_int4(p, s, cnt, 0);
  }
}

// Stores kept pair number `slot` of source row sidx: the first cap go to the row's
// ELL slots, the next ov to its spill list (row-major), the rest are only counted.
__device__ __forceinline__ void put_kept(PairDev *P, int ld, int cap, int ov, size_t sidx, int slot, int j, float a) {
  if (slot < cap) {
    P->A_j[sidx * ld + slot] = j;
    P->A_v[sidx * ld + slot] = a;
  } else if (slot - cap < ov) {
    P->ovf[sidx * ov + (slot - cap)] = make_int2(j, __float_as_int(a));
  }
}

// Dynamic shared memory of one k_assoc block: per warp two staging buffers, the
// prefilter tile and the grid descriptor (16-byte aligned pieces).
template <int FCH, int LCH, bool GT>
struct AssocSmem {
  static constexpr int kWarps = kAssocThreads / 32;
  static constexpr size_t align16(size_t v) { return (v + 15) & ~(size_t)15; }
  static constexpr size_t kStage = 0;
  static constexpr size_t kMma = align16(kStage + sizeof(StageBuf<FCH, LCH, GT>) * 2 * kWarps);
  static constexpr size_t kRows = align16(kMma + sizeof(MmaTile) * kWarps);
  static constexpr size_t kGrid = align16(kRows + sizeof(SrcRows<FCH, LCH>) * kWarps);
  static constexpr size_t kBytes = align16(kGrid + sizeof(GridDesc) * kWarps);
};

// Plane p of a row/candidate block: entry i at base[p * stride + i] (16 B = 8 halves).
// A fragments (rows 16m..16m+15) of plane pair `hl` (0 = hi, 2 = lo).
__device__ __forceinline__ void mma_load_a(const uint4 *a, int stride, int hl, int m, int lane, uint32_t (&r)[4]) {
  const int mi = lane >> 3, r8 = lane & 7;
  ldsm_x4(&a[(hl + (mi >> 1)) * stride + 16 * m + 8 * (mi & 1) + r8], r[0], r[1], r[2], r[3]);
}

// B fragments of candidate groups 2j and 2j+1 (candidates 16j..16j+15).
__device__ __forceinline__ void mma_load_b(const uint4 *b, int stride, int hl, int j, int lane, uint32_t (&r)[4]) {
  const int mi = lane >> 3, r8 = lane & 7;
  ldsm_x4(&b[(hl + (mi & 1)) * stride + 16 * j + 8 * (mi >> 1) + r8], r[0], r[1], r[2], r[3]);
}

// u-tile of 32 rows (planes at a, stride as) against 32 candidates (planes at b,
// stride bs); returns, for the lane's own row, the bit mask of candidates with
// u < tau.  All lanes call it.
__device__ __forceinline__ uint32_t mma_filter(const uint4 *a, int as, const uint4 *b, int bs, int lane, float tau) {
  uint32_t word = 0;   // byte (2m + h), bit (2n + jj): row 16m + 8h + lane/4, column 8n + 2(lane%4) + jj
#pragma unroll
  for (int j = 0; j < 2; j++) {
    uint32_t bh[4], bl[4];
    mma_load_b(b, bs, 0, j, lane, bh);
    mma_load_b(b, bs, 2, j, lane, bl);
#pragma unroll
    for (int m = 0; m < 2; m++) {
      uint32_t ah[4], al[4];
      mma_load_a(a, as, 0, m, lane, ah);
      mma_load_a(a, as, 2, m, lane, al);
#pragma unroll
      for (int q = 0; q < 2; q++) {
        const int n = 2 * j + q;
        float d[4] = {0.f, 0.f, 0.f, 0.f};
        mma_16816(d, ah, bh[2 * q], bh[2 * q + 1]);
        mma_16816(d, ah, bl[2 * q], bl[2 * q + 1]);
        mma_16816(d, al, bh[2 * q], bh[2 * q + 1]);
        word |= (d[0] < tau ? 1u : 0u) << (8 * (2 * m) + 2 * n);
        word |= (d[1] < tau ? 1u : 0u) << (8 * (2 * m) + 2 * n + 1);
        word |= (d[2] < tau ? 1u : 0u) << (8 * (2 * m + 1) + 2 * n);
        word |= (d[3] < tau ? 1u : 0u) << (8 * (2 * m + 1) + 2 * n + 1);
      }
    }
  }
  // gather the lane's row: held by lanes 4 (row % 8) + t, t = 0..3
  const int sh = 8 * (2 * (lane >> 4) + ((lane >> 3) & 1));
  const int src0 = 4 * (lane & 7);
  uint32_t mask = 0;
#pragma unroll
  for (int t = 0; t < 4; t++) {
    const uint32_t w = __shfl_sync(FULLMASK, word, src0 + t);
    const uint32_t bb = (w >> sh) & 0xFFu;
    const uint32_t sp = (bb & 0x3u) | ((bb & 0xCu) << 6) | ((bb & 0x30u) << 12) | ((bb & 0xC0u) << 18);
    mask |= sp << (2 * t);
  }
  return mask;
}

// Filter vector of a source row (A) or a candidate (B), relative to the centre p.
template <int FCH>
__device__ __forceinline__ void mma_row_vec(float (&av)[16], bool valid, const float4 &x, const float4 (&xf)[FCH > 0 ? FCH : 1],
                                            int F, float g, float cw, float px, float py, float pz) {
  const float tx = x.x - px, ty = x.y - py, tz = x.z - pz;
  g = valid ? g : 0.f;
  av[0] = -2.f * g * tx; av[1] = -2.f * g * ty; av[2] = -2.f * g * tz;
  float xc2 = 0.f;
#pragma unroll
  for (int f = 0; f < 8; f++) {
    float xv = 0.f;
    if (FCH > 0 && (f >> 2) < FCH && f < F) xv = f4_at(xf[(f >> 2) < FCH ? (f >> 2) : 0], f & 3);
    av[3 + f] = valid ? -2.f * cw * xv : 0.f;
    xc2 += xv * xv;
  }
  av[11] = g;
  av[12] = valid ? cw : 0.f;
  av[13] = valid ? g * (tx * tx + ty * ty + tz * tz) + cw * xc2 : 0.f;
  float na = 0.f;
#pragma unroll
  for (int k = 0; k < 14; k++) na += av[k] * av[k];
  av[14] = -kMmaKappa * sqrtf(na);
  av[15] = 0.f;
}

template <int FCH>
__device__ __forceinline__ void mma_cand_vec(float (&bv)[16], bool has, const float4 &y, const float4 *yf, int F,
                                             float px, float py, float pz) {
#pragma unroll
  for (int q = 0; q < 16; q++) bv[q] = 0.f;
  if (!has) return;
  bv[0] = y.x - px; bv[1] = y.y - py; bv[2] = y.z - pz;
  float yc2 = 0.f;
#pragma unroll
  for (int f = 0; f < 8; f++) {
    float yv = 0.f;
    if (FCH > 0 && (f >> 2) < FCH && f < F) yv = f4_at(yf[(f >> 2) < FCH ? (f >> 2) : 0], f & 3);
    bv[3 + f] = yv;
    yc2 += yv * yv;
  }
  bv[11] = bv[0] * bv[0] + bv[1] * bv[1] + bv[2] * bv[2];
  bv[12] = yc2;
  bv[13] = 1.f;
  float nb = 0.f;
#pragma unroll
  for (int q = 0; q < 14; q++) nb += bv[q] * bv[q];
  bv[14] = sqrtf(nb);
}

// Exact evaluation of the surviving pairs of one candidate group, 32 at a time:
// pair number i of the warp (rows in order, each row's candidates ascending) goes
// to lane i % 32, so a row's kept pairs still enter it in ascending candidate
// order.  `cand` is the lane's own row mask, `cnt` its kept count (updated);
// put(r, slot, j, a) stores kept pair number `slot` of row r.
template <int FCH, int LCH, bool GT, class Put>
__device__ __forceinline__ void eval_survivors(const KParams &K, int F, int C, int lane, uint32_t cand, int &cnt,
                                               const SrcRows<FCH, LCH> &sr, const float4 *cpos, const float4 *cfeat,
                                               const float4 *clab, const float4 *cgeo, Put put) {
  const int cc = __popc(cand);
  int incl = cc;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(FULLMASK, incl, o);
    if (lane >= o) incl += t;
  }
  const int excl = incl - cc;
  const int total = __shfl_sync(FULLMASK, incl, 31);
  for (int b0 = 0; b0 < total; b0 += 32) {
    const int idx = b0 + lane;
    const bool has = idx < total;
    int r = 0;   // row of pair idx: the last row whose first pair is at or before idx
#pragma unroll
    for (int st = 16; st > 0; st >>= 1) {
      const int e = __shfl_sync(FULLMASK, excl, r + st);
      if (e <= idx) r += st;
    }
    const int er = __shfl_sync(FULLMASK, excl, r);
    const uint32_t mr = __shfl_sync(FULLMASK, cand, r);
    const int cr = __shfl_sync(FULLMASK, cnt, r);
    const int k = has ? nth_set_bit(mr, idx - er) : 0;
    const float4 xr = sr.x[r];
    const float4 rr = sr.rc[r];
    float4 xfr[FCH > 0 ? FCH : 1];
    float4 xlr[LCH > 0 ? LCH : 1];
#pragma unroll
    for (int q = 0; q < (FCH > 0 ? FCH : 1); q++) xfr[q] = sr.f[r * (FCH > 0 ? FCH : 1) + q];
#pragma unroll
    for (int q = 0; q < (LCH > 0 ? LCH : 1); q++) xlr[q] = sr.l[r * (LCH > 0 ? LCH : 1) + q];
    const float2 xgr = make_float2(rr.w, sr.g1[r]);
    const float4 y = cpos[k];
    float a;
    const bool acc = eval_pair<FCH, LCH, GT>(K, F, C, has, rr.x, rr.y, rr.z, xr, xfr, xlr, xgr, y,
                                             &cfeat[k * (FCH > 0 ? FCH : 1)], &clab[k * (LCH > 0 ? LCH : 1)],
                                             &cgeo[GT ? k : 0], a);
    const uint32_t bal = __ballot_sync(FULLMASK, acc);
    if (acc) {
      const int lo = max(er - b0, 0);
      const uint32_t before = bal & ((1u << lane) - 1u) & ~((1u << lo) - 1u);
      put(r, cr + __popc(before), __float_as_int(y.w), a);
    }
    // row owners count their kept pairs of this group
    const int lo = min(max(excl - b0, 0), 32), hi = min(max(incl - b0, 0), 32);
    const uint32_t seg = (uint32_t)(((1ull << hi) - 1ull) & ~((1ull << lo) - 1ull));
    cnt += __popc(bal & seg);
  }
}

// ------------------------------------------------------------ association
// One warp per tile of 32 spatially adjacent source points (Morton order).  The
// warp scans the grid cells overlapping the union of its lanes' query boxes;
// each candidate target is staged once per warp in shared memory and tested by
// every lane against its own source point.  Chunks are double-buffered: the copy
// of chunk k+1 is in flight while the lanes test chunk k.
template <int FCH, int LCH, bool GT>
__device__ __forceinline__ void assoc_warp(const BatchDev &B, const KParams &K, int gw, unsigned char *assoc_smem) {
  using Buf = StageBuf<FCH, LCH, GT>;
  using L = AssocSmem<FCH, LCH, GT>;
  constexpr int CH = Buf::CH;
  Buf(*stage_all)[2] = reinterpret_cast<Buf(*)[2]>(assoc_smem + L::kStage);
  MmaTile *mma_all = reinterpret_cast<MmaTile *>(assoc_smem + L::kMma);
  SrcRows<FCH, LCH> *rows_all = reinterpret_cast<SrcRows<FCH, LCH> *>(assoc_smem + L::kRows);
  GridDesc *grid_all = reinterpret_cast<GridDesc *>(assoc_smem + L::kGrid);
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  Buf *stage = stage_all[wib];
  MmaTile &mt = mma_all[wib];
  SrcRows<FCH, LCH> &sr = rows_all[wib];
  if (gw >= B.total_warps) return;
  const int p = find_segment(B.tile_off, B.npairs, gw);
  PairDev *P = &B.pairs[p];
  if (P->done) return;
  if (lane == 0) grid_all[wib] = P->levels[P->level];
  __syncwarp();
  const GridDesc &G = grid_all[wib];
  const int n = P->n;
  const int s = (gw - B.tile_off[p]) * 32 + lane;
  const bool valid = s < n;
  const float ell = P->ell;
  const int cap = P->cap;
  const int F = P->F, C = P->C;
  float4 x = valid ? __ldg(&P->xs[s]) : make_float4(0.f, 0.f, 0.f, 0.f);
  float4 xf[FCH > 0 ? FCH : 1];
  float4 xl[LCH > 0 ? LCH : 1];
  float2 xg = make_float2(0.f, 0.f);
#pragma unroll
  for (int q = 0; q < (FCH > 0 ? FCH : 1); q++)
    xf[q] = (FCH > 0 && valid) ? __ldg(reinterpret_cast<const float4 *>(P->xf) + (size_t)s * FCH + q)
                               : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
  for (int q = 0; q < (LCH > 0 ? LCH : 1); q++)
    xl[q] = (LCH > 0 && valid) ? __ldg(reinterpret_cast<const float4 *>(P->xl) + (size_t)s * LCH + q)
                               : make_float4(0.f, 0.f, 0.f, 0.f);
  if (GT && valid) xg = __ldg(&P->xg[s]);
  const float Tn = fabsf(P->T[0]) + fabsf(P->T[1]) + fabsf(P->T[2]);
  RowConst rc = row_const(K, ell, x.w, Tn);
  // query box in the target's initial frame: q = R x + T
  const float *R = P->R;
  float qx = fmaf(R[0], x.x, fmaf(R[1], x.y, fmaf(R[2], x.z, P->T[0])));
  float qy = fmaf(R[3], x.x, fmaf(R[4], x.y, fmaf(R[5], x.z, P->T[1])));
  float qz = fmaf(R[6], x.x, fmaf(R[7], x.y, fmaf(R[8], x.z, P->T[2])));
  float lox = valid ? qx - rc.rq : INFINITY, hix = valid ? qx + rc.rq : -INFINITY;
  float loy = valid ? qy - rc.rq : INFINITY, hiy = valid ? qy + rc.rq : -INFINITY;
  float loz = valid ? qz - rc.rq : INFINITY, hiz = valid ? qz + rc.rq : -INFINITY;
  // own box of this lane (used when the warp's union box is too sparse)
  int ox0 = 0, oy0 = 0, oz0 = 0, onx = 0, ony = 0, onz = 0;
  long long own_cells = 0;
  if (valid && cell_range(G, lox, loy, loz, hix, hiy, hiz, ox0, oy0, oz0, onx, ony, onz))
    own_cells = (long long)onx * ony * onz;
  long long own_sum = own_cells;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) own_sum += __shfl_xor_sync(FULLMASK, own_sum, o);
  lox = warp_min(lox); loy = warp_min(loy); loz = warp_min(loz);
  hix = warp_max(hix); hiy = warp_max(hiy); hiz = warp_max(hiz);
  int ux0, uy0, uz0, unx, uny, unz;
  const bool union_ok = cell_range(G, lox, loy, loz, hix, hiy, hiz, ux0, uy0, uz0, unx, uny, unz);
  const long long union_cells = union_ok ? (long long)unx * uny * unz : 0;
  // One pass over the union box of the tile, or, when that box is much larger
  // than the lanes' own boxes together, one pass per lane over its own box.
  const bool per_lane = union_cells > 64 && union_cells > 2 * own_sum;
  const int npass = per_lane ? 32 : (union_ok ? 1 : 0);
  // Tensor-core prefilter for the tile (one pass over the union box, F <= 8).
  bool use_mma = K.use_mma && npass == 1 && !per_lane && F <= 8;
  float pcx = 0.f, pcy = 0.f, pcz = 0.f;   // centre of the tile's valid source points
  const float cw = K.use_int ? K.inv2c2 : 0.f;
  if (use_mma) {
    const int nv = warp_sumi(valid ? 1 : 0);
    const float inv = 1.f / (float)max(nv, 1);
    pcx = warp_sumf(valid ? x.x : 0.f) * inv;
    pcy = warp_sumf(valid ? x.y : 0.f) * inv;
    pcz = warp_sumf(valid ? x.z : 0.f) * inv;
    float av[16];
    mma_row_vec<FCH>(av, valid, x, xf, F, rc.inv2l2, cw, pcx, pcy, pcz);
    const bool ok = mma_store_vec(av, &mt.a[0][0], 32, lane);
    use_mma = __all_sync(FULLMASK, ok);
    // this row's data for the lanes that evaluate its surviving pairs
    sr.x[lane] = x;
    sr.rc[lane] = make_float4(rc.l, rc.d2t, rc.inv2l2, xg.x);
    sr.g1[lane] = xg.y;
#pragma unroll
    for (int q = 0; q < (FCH > 0 ? FCH : 1); q++) sr.f[lane * (FCH > 0 ? FCH : 1) + q] = xf[q];
#pragma unroll
    for (int q = 0; q < (LCH > 0 ? LCH : 1); q++) sr.l[lane * (LCH > 0 ? LCH : 1) + q] = xl[q];
    __syncwarp();
  }
  int cnt = 0;
  const float4 *__restrict__ ycur = P->ycur;
  const int ov = P->ov;
  const int tile0 = (gw - B.tile_off[p]) * 32;   // source index of lane 0's row
  // kept pair number `slot` of row r enters its ELL slot (first cap) or its spill list
  const int ld = P->ld;
  auto put = [&](int r, int slot, int j, float a) { put_kept(P, ld, cap, ov, (size_t)(tile0 + r), slot, j, a); };
  for (int pass = 0; pass < npass; pass++) {
    int x0, y0, z0, nx, ny, nz;
    bool me = valid;
    if (per_lane) {
      x0 = __shfl_sync(FULLMASK, ox0, pass); y0 = __shfl_sync(FULLMASK, oy0, pass);
      z0 = __shfl_sync(FULLMASK, oz0, pass); nx = __shfl_sync(FULLMASK, onx, pass);
      ny = __shfl_sync(FULLMASK, ony, pass); nz = __shfl_sync(FULLMASK, onz, pass);
      if (__shfl_sync(FULLMASK, own_cells, pass) == 0) continue;
      me = valid && lane == pass;
    } else {
      x0 = ux0; y0 = uy0; z0 = uz0; nx = unx; ny = uny; nz = unz;
    }
    // bounding box of this pass's query points and their largest search radius
    float bl0 = qx, bl1 = qy, bl2 = qz, bh0 = qx, bh1 = qy, bh2 = qz, brq = valid ? rc.rq : 0.f;
    if (per_lane) {
      bl0 = bh0 = __shfl_sync(FULLMASK, qx, pass); bl1 = bh1 = __shfl_sync(FULLMASK, qy, pass);
      bl2 = bh2 = __shfl_sync(FULLMASK, qz, pass); brq = __shfl_sync(FULLMASK, brq, pass);
    } else {
      bl0 = warp_min(valid ? qx : INFINITY); bl1 = warp_min(valid ? qy : INFINITY); bl2 = warp_min(valid ? qz : INFINITY);
      bh0 = warp_max(valid ? qx : -INFINITY); bh1 = warp_max(valid ? qy : -INFINITY); bh2 = warp_max(valid ? qz : -INFINITY);
      brq = warp_max(brq);
    }
    const float slack = 1e-3f * G.h;
    const float prune_r2 = (brq + slack) * (brq + slack);
    const int ncells = nx * ny * nz;
    for (int cb = 0; cb < ncells; cb += 32) {
      int ci = cb + lane;
      int2 se = make_int2(0, 0);
      if (ci < ncells) {
        int cx = x0 + ci % nx, cy = y0 + (ci / nx) % ny, cz = z0 + ci / (nx * ny);
        // skip cells farther than the largest radius from every query point of the pass
        bool near = true;
        if (G.inv_h != 0.f) {
          const float c0 = fmaf((float)cx, G.h, G.ox), c1 = fmaf((float)cy, G.h, G.oy), c2 = fmaf((float)cz, G.h, G.oz);
          const float dx = fmaxf(fmaxf(c0 - bh0, bl0 - (c0 + G.h)), 0.f);
          const float dy = fmaxf(fmaxf(c1 - bh1, bl1 - (c1 + G.h)), 0.f);
          const float dz = fmaxf(fmaxf(c2 - bh2, bl2 - (c2 + G.h)), 0.f);
          near = dx * dx + dy * dy + dz * dz <= prune_r2;
        }
        if (near) se = grid_lookup(G, cx, cy, cz);
      }
      unsigned mk = __ballot_sync(FULLMASK, se.y > 0);
      if (!mk) continue;
      // Chunks of up to CH candidates filled from consecutive non-empty cells of this
      // batch; the warp walks a cursor (cell, offset) in lockstep.
      int c_start = 0, c_cnt = 0, c_off = 0;
      auto fill = [&](int bi) -> int {
        int filled = 0;
        while (filled < CH) {
          if (c_off >= c_cnt) {
            if (!mk) break;
            const int bb = __ffs(mk) - 1;
            mk &= mk - 1;
            c_start = __shfl_sync(FULLMASK, se.x, bb);
            c_cnt = __shfl_sync(FULLMASK, se.y, bb);
            c_off = 0;
          }
          const int take = min(CH - filled, c_cnt - c_off);
          stage_piece<FCH, LCH, GT>(stage[bi], ycur, G, filled, c_start + c_off, take, lane);
          filled += take;
          c_off += take;
        }
        __syncwarp();   // the chunk is visible to every lane
        return filled;
      };
      int cur = 0;
      int nk = fill(cur);
      while (nk > 0) {
        const Buf &sb = stage[cur];
        if (use_mma) {
          // candidate vectors of this chunk (lane k builds candidate k; empty slots are zero)
          float bv[16];
          mma_cand_vec<FCH>(bv, lane < nk, sb.pos[lane], &sb.feat[lane * (FCH > 0 ? FCH : 1)], F, pcx, pcy, pcz);
          const bool ok = __all_sync(FULLMASK, mma_store_vec(bv, &mt.b[0][0], 32, lane));
          __syncwarp();
          uint32_t cand = ok ? mma_filter(&mt.a[0][0], 32, &mt.b[0][0], 32, lane, K.mma_tau) : 0xFFFFFFFFu;
          cand &= (nk >= 32) ? 0xFFFFFFFFu : ((1u << nk) - 1u);
          if (!me) cand = 0u;
          eval_survivors<FCH, LCH, GT>(K, F, C, lane, cand, cnt, sr, sb.pos, sb.feat, sb.lab, sb.geo, put);
        } else {
          for (int k = 0; k < nk; k++) {
            const float4 y = sb.pos[k];
            float a;
            bool acc = eval_pair<FCH, LCH, GT>(K, F, C, me, rc.l, rc.d2t, rc.inv2l2, x, xf, xl, xg, y,
                                               &sb.feat[k * (FCH > 0 ? FCH : 1)], &sb.lab[k * (LCH > 0 ? LCH : 1)],
                                               &sb.geo[GT ? k : 0], a);
            if (acc) { put(lane, cnt, __float_as_int(y.w), a); cnt++; }
          }
        }
        __syncwarp();   // every lane is done with the chunk before the next one is staged
        cur ^= 1;
        nk = fill(cur);
      }
    }
  }
  if (valid) finish_row(B, P, p, s, cnt, cap, ov);
}

template <int FCH, int LCH, bool GT>
__global__ void __launch_bounds__(kAssocThreads) k_assoc(BatchDev B, KParams K) {
  extern __shared__ __align__(128) unsigned char assoc_smem[];
  assoc_warp<FCH, LCH, GT>(B, K, (blockIdx.x * blockDim.x + threadIdx.x) >> 5, assoc_smem);
}

// ------------------------------------------------------------ selection
constexpr int kSelMax = 4096;      // kept pairs beyond cap one spill list can hold
constexpr int kSelStage = 1024;    // rows up to this many entries are selected from shared memory
constexpr int kSelThreads = 128;

// Row partials of one source row from its final ELL entries, in slot order
// (thread per row): omega = sum a (x cross y), v = sum a (y - x), sum a.
// (CvoGPU.cu:2001-2062 computes the same sums from the sparse kernel matrix.)
__global__ void __launch_bounds__(256) k_rowsum(BatchDev B, KParams K) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= B.total_rows) return;
  const int p = find_segment(B.row_off, B.npairs, g);
  const PairDev *P = &B.pairs[p];
  if (P->done) return;
  const int s = g - B.row_off[p];
  const int z = P->nnz_row[s];
  const float4 x = __ldg(&P->xs[s]);
  float w0 = 0.f, w1 = 0.f, w2 = 0.f, v0 = 0.f, v1 = 0.f, v2 = 0.f, as = 0.f;
  const int *__restrict__ Aj = P->A_j + (size_t)s * P->ld;
  const float *__restrict__ Av = P->A_v + (size_t)s * P->ld;
  const float4 *__restrict__ yorig = P->yorig;
  auto add = [&](float a, const float4 &y) {
    w0 = fmaf(a, fs(fm(x.y, y.z), fm(x.z, y.y)), w0);
    w1 = fmaf(a, fs(fm(x.z, y.x), fm(x.x, y.z)), w1);
    w2 = fmaf(a, fs(fm(x.x, y.y), fm(x.y, y.x)), w2);
    v0 = fmaf(a, y.x - x.x, v0);
    v1 = fmaf(a, y.y - x.y, v1);
    v2 = fmaf(a, y.z - x.z, v2);
    as += a;
  };
  int c = 0;
  // four entries per 16-byte load (rows are 16-byte aligned); the sums keep slot order
  for (; c + 4 <= z; c += 4) {
    const int4 j4 = *reinterpret_cast<const int4 *>(Aj + c);
    const float4 a4 = *reinterpret_cast<const float4 *>(Av + c);
    const float4 y0 = __ldg(&yorig[j4.x]), y1 = __ldg(&yorig[j4.y]), y2 = __ldg(&yorig[j4.z]), y3 = __ldg(&yorig[j4.w]);
    add(a4.x, y0);
    add(a4.y, y1);
    add(a4.z, y2);
    add(a4.w, y3);
  }
  for (; c < z; c++) add(Av[c], __ldg(&yorig[Aj[c]]));
  write_row_sums(P->row_sums + (size_t)s * 8, P->mode, K, w0, w1, w2, v0, v1, v2, as);
}

// One warp per listed row with cap < count <= cap + ov: its ELL slots hold the
// first cap kept pairs and its spill list (row-major) the rest, in the order they
// were kept.  The indices of a row of up to kSelStage entries are first staged in
// shared memory (16-byte loads: many loads in flight per lane), so the radix passes
// read no global memory; the values stay in global memory and are read once, by
// the compaction, for the kept entries only.  A radix select over d = j - jmin
// (jmin, jmax: the row's smallest and largest kept index; 9-bit digits from the
// highest bit of jmax - jmin, warp-private histograms) finds the cap-th smallest
// index r.  Offsetting by jmin spreads the indices over the bins, each lane counts
// its own run of the list (so one instruction's increments come from different
// grid cells and rarely collide), and a row whose indices span fewer than 512 values
// needs one pass.  The entries with index <= r (exactly cap: indices are distinct)
// are compacted in list order into the ELL slots, in place: an entry is read before
// any write can reach its slot, and a __syncwarp between a chunk's reads and its
// writes orders the lanes' accesses.  Longer rows read their indices from global
// memory on every pass.  Eight blocks of four warps per SM: 6.2 KB of shared memory
// per warp and at most 64 registers a thread keep 32 warps resident, which hide the
// latency of the dependent passes of each warp's rows.
constexpr int kSelBins = 512;
constexpr int kSelDigit = 9;
constexpr int kSelBlocksPerSm = 8;
// bin b lives at b + b / 16: lane l's scan reads its 16 bins at stride 17 words, on
// distinct banks
constexpr int kSelHist = kSelBins + kSelBins / 16;
__device__ __forceinline__ int sel_bin(int b) { return b + (b >> 4); }
__global__ void __launch_bounds__(kSelThreads, kSelBlocksPerSm) k_select(BatchDev B, KParams K) {
  __shared__ int jbuf_all[kSelThreads / 32][kSelStage];
  __shared__ int hist_all[kSelThreads / 32][kSelHist];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int *jb = jbuf_all[w];
  int *hist = hist_all[w];
  const int count = *B.sel_count;
  const int nwarps = gridDim.x * (kSelThreads / 32);
  const int e0 = blockIdx.x * (kSelThreads / 32) + w;
  int4 next = e0 < count ? B.sel_list[e0] : make_int4(0, 0, 0, 0);
  for (int e = e0; e < count; e += nwarps) {
    const int4 it = next;            // this row's list entry; the next one is loaded meanwhile
    if (e + nwarps < count) next = B.sel_list[e + nwarps];
    const PairDev *P = &B.pairs[it.x];
    const int s = it.y, cap = P->cap, ov = P->ov;
    const int E = it.z;
    const int2 *lst = P->ovf + (size_t)s * ov;
    int *Aj = P->A_j + (size_t)s * P->ld;
    float *Av = P->A_v + (size_t)s * P->ld;
    const bool staged = E <= kSelStage;
    auto gidx = [&](int t) -> int { return t < cap ? Aj[t] : lst[t - cap].x; };
    int jmin = 0x7FFFFFFF, jmax = -1;
    if (staged) {
      // ELL part: 4 indices per 16-byte load (rows are 16-byte aligned, the pitch covers
      // the rounded-up chunk); spill part: 2 entries per 16-byte load (rows start 16-byte
      // aligned).  Each lane issues up to 4 loads before it stores any: the loads go
      // through generic pointers, which the compiler must not move past a shared-memory
      // store, so loads and stores interleaved one by one would wait for memory in turn.
      const int nq = (cap + 3) >> 2;
      for (int q0 = lane; q0 < nq; q0 += 128) {
        int4 j4[4];
#pragma unroll
        for (int u = 0; u < 4; u++)
          if (q0 + 32 * u < nq) j4[u] = reinterpret_cast<const int4 *>(Aj)[q0 + 32 * u];
#pragma unroll
        for (int u = 0; u < 4; u++) {
          const int q = q0 + 32 * u;
          if (q < nq) {
            const int jv[4] = {j4[u].x, j4[u].y, j4[u].z, j4[u].w};
#pragma unroll
            for (int i = 0; i < 4; i++)
              if (4 * q + i < cap) {
                jb[4 * q + i] = jv[i];
                jmin = min(jmin, jv[i]);
                jmax = max(jmax, jv[i]);
              }
          }
        }
      }
      const int ns = E - cap, np = (ns + 1) >> 1;
      for (int q0 = lane; q0 < np; q0 += 128) {
        int4 v4[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
          const int q = q0 + 32 * u;
          if (2 * q + 1 < ns) v4[u] = reinterpret_cast<const int4 *>(lst)[q];
          else if (2 * q < ns) v4[u] = make_int4(lst[2 * q].x, 0, -1, 0);
        }
#pragma unroll
        for (int u = 0; u < 4; u++) {
          const int q = q0 + 32 * u;
          if (2 * q < ns) {
            jb[cap + 2 * q] = v4[u].x;
            jmin = min(jmin, v4[u].x);
            jmax = max(jmax, v4[u].x);
            if (2 * q + 1 < ns) {
              jb[cap + 2 * q + 1] = v4[u].z;
              jmin = min(jmin, v4[u].z);
              jmax = max(jmax, v4[u].z);
            }
          }
        }
      }
    } else {
      for (int t = lane; t < E; t += 32) {
        const int j = gidx(t);
        jmin = min(jmin, j);
        jmax = max(jmax, j);
      }
    }
    jmin = __reduce_min_sync(FULLMASK, jmin);
    jmax = __reduce_max_sync(FULLMASK, jmax);
    __syncwarp();
    auto entry = [&](int t) -> int { return staged ? jb[t] : gidx(t); };
    const int span = jmax - jmin;
    const int bits = span > 0 ? 32 - __clz(span) : 1;
    // lane l counts the contiguous run of entries l * per .. : neighbouring entries of
    // the list come from one grid cell and share their high index bits, so the 32
    // increments of one instruction then go to different bins instead of colliding (an
    // odd run length keeps the 32 lanes' shared-memory reads on distinct banks)
    const int per = ((E + 31) >> 5) | 1;
    const int t_lo = lane * per, t_hi = min(t_lo + per, E);
    int prefix = 0, target = cap;
    for (int hs = bits; hs > 0; hs -= kSelDigit) {
      const int sh = max(hs - kSelDigit, 0), wd = hs - sh;
      for (int b = lane; b < kSelHist; b += 32) hist[b] = 0;
      __syncwarp();
      const int want = prefix >> hs, mask = (1 << wd) - 1;
#pragma unroll 4
      for (int t = t_lo; t < t_hi; t++) {
        const int d = entry(t) - jmin;
        if ((d >> hs) == want) atomicAdd(&hist[sel_bin((d >> sh) & mask)], 1);
      }
      __syncwarp();
      // lane l owns bins 16 l .. 16 l + 15: their total, an exclusive scan over the lanes,
      // the lane L whose bins reach target, then the bin inside L's 16 (lanes 0..15 read
      // one bin each and scan them)
      constexpr int kPer = kSelBins / 32;
      int loc = 0;
#pragma unroll
      for (int i = 0; i < kPer; i++) loc += hist[sel_bin(lane * kPer + i)];
      int incl = loc;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(FULLMASK, incl, o);
        if (lane >= o) incl += t;
      }
      int L = __ffs(__ballot_sync(FULLMASK, incl >= target)) - 1;
      if (L < 0) L = 31;             // unreachable: the counted entries always reach target
      const int before = __shfl_sync(FULLMASK, incl - loc, L);
      const int hb = lane < kPer ? hist[sel_bin(L * kPer + lane)] : 0;
      int hin = hb;
#pragma unroll
      for (int o = 1; o < kPer; o <<= 1) {
        const int t = __shfl_up_sync(FULLMASK, hin, o);
        if (lane >= o) hin += t;
      }
      int i_bin = __ffs(__ballot_sync(FULLMASK, lane < kPer && before + hin >= target)) - 1;
      if (i_bin < 0) i_bin = kPer - 1;  // unreachable, as above
      const int run = before + __shfl_sync(FULLMASK, hin - hb, i_bin);
      prefix |= (L * kPer + i_bin) << sh;
      target -= run;
      __syncwarp();
    }
    const int r = jmin + prefix;   // the cap-th smallest kept index
    // compaction, 128 entries per round: every lane reads its 4 entries (index, and the
    // value of a kept one: 4 independent loads in flight), a __syncwarp orders these reads
    // before the round's writes (which go to slots below the round's end), then the 4
    // chunks are placed in list order
    int base = 0;
    for (int t0 = 0; t0 < E; t0 += 128) {
      int j[4];
      float a[4];
      bool k[4];
#pragma unroll
      for (int u = 0; u < 4; u++) {
        const int t = t0 + 32 * u + lane;
        j[u] = t < E ? entry(t) : 0;
        k[u] = t < E && j[u] <= r;
        a[u] = 0.f;
      }
#pragma unroll
      for (int u = 0; u < 4; u++) {
        const int t = t0 + 32 * u + lane;
        if (k[u]) a[u] = t < cap ? Av[t] : __int_as_float(lst[t - cap].y);
      }
      __syncwarp();
#pragma unroll
      for (int u = 0; u < 4; u++) {
        const unsigned bal = __ballot_sync(FULLMASK, k[u]);
        const int c = base + __popc(bal & ((1u << lane) - 1u));
        if (k[u] && c < cap) {
          Aj[c] = j[u];
          Av[c] = a[u];
        }
        base += __popc(bal);
      }
    }
    __syncwarp();
  }
}

// One warp per listed row with count > cap + ov: the reference's own order, i.e. a
// scan of the targets by ascending original index (32 per step, one per lane) that
// stops once cap pairs are kept.  Same per-pair arithmetic as k_assoc.
template <int FCH, int LCH, bool GT>
__global__ void __launch_bounds__(kSelThreads) k_rescan(BatchDev B, KParams K) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int count = *B.scan_count;
  const int nwarps = gridDim.x * (kSelThreads / 32);
  for (int e = blockIdx.x * (kSelThreads / 32) + w; e < count; e += nwarps) {
    const int4 it = B.scan_list[e];
    const PairDev *P = &B.pairs[it.x];
    const int s = it.y, m = P->m, cap = P->cap, F = P->F, C = P->C;
    const float4 x = P->xs[s];
    float4 xf[FCH > 0 ? FCH : 1];
    float4 xl[LCH > 0 ? LCH : 1];
#pragma unroll
    for (int q = 0; q < (FCH > 0 ? FCH : 1); q++)
      xf[q] = FCH > 0 ? __ldg(reinterpret_cast<const float4 *>(P->xf) + (size_t)s * FCH + q) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int q = 0; q < (LCH > 0 ? LCH : 1); q++)
      xl[q] = LCH > 0 ? __ldg(reinterpret_cast<const float4 *>(P->xl) + (size_t)s * LCH + q) : make_float4(0.f, 0.f, 0.f, 0.f);
    const float2 xg = GT ? __ldg(&P->xg[s]) : make_float2(0.f, 0.f);
    const float Tn = fabsf(P->T[0]) + fabsf(P->T[1]) + fabsf(P->T[2]);
    const RowConst rc = row_const(K, P->ell, x.w, Tn);
    int taken = 0;
    for (int j0 = 0; j0 < m && taken < cap; j0 += 32) {
      const int j = j0 + lane;
      const bool pre = j < m;
      const int jj = pre ? j : 0;
      const float4 y = __ldg(&P->yorig[jj]);
      float4 yg = make_float4(0.f, 0.f, 0.f, 0.f);
      if (GT) { const float2 g2 = __ldg(&P->tg[jj]); yg.x = g2.x; yg.y = g2.y; }
      const float4 *yfp = reinterpret_cast<const float4 *>(P->tf) + (size_t)jj * (FCH > 0 ? FCH : 1);
      const float4 *ylp = reinterpret_cast<const float4 *>(P->tl) + (size_t)jj * (LCH > 0 ? LCH : 1);
      float a = 0.f;
      const bool k = eval_pair<FCH, LCH, GT>(K, F, C, pre, rc.l, rc.d2t, rc.inv2l2, x, xf, xl, xg, y, yfp, ylp, &yg, a);
      const unsigned bal = __ballot_sync(FULLMASK, k);
      if (k) {
        const int c = taken + __popc(bal & ((1u << lane) - 1u));
        if (c < cap) {
          P->A_j[(size_t)s * P->ld + c] = j;
          P->A_v[(size_t)s * P->ld + c] = a;
        }
      }
      taken += __popc(bal);
    }
  }
}

}  // namespace cvo_gb
