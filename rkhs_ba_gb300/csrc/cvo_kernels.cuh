// cvo_kernels.cuh -- per-iteration kernels of the batched CVO engine.
//
// One iteration of the reference's align loop (src/cvo/CvoGPU.cu:1303-1433) is
// four launches over every active pair of a batch:
//   k_transform  target transform y' = R^T (y - T)            (CvoGPU_impl.cu:32-83)
//   k_assoc      fused association: grid candidates -> kernel value -> threshold
//                -> first-`cap`-by-index selection -> ELL row -> gradient partials
//                                                               (CvoGPU.cu:951-1099, 2001-2062)
//   k_reduce     per-pair FP64 sums of the row partials; gradient normalisation
//                                                               (CvoGPU.cu:2065-2120)
//   k_step       Taylor step-size terms over the ELL rows; the last block of each pair
//                runs the scalar tail of the iteration: cubic roots, step clamp,
//                Exp_SEK3 pose update, SE(3) distance, lengthscale schedule, cap update
//                                                               (CvoGPU.cu:333-544, 547-665, 1339-1433)
#pragma once
#include "cvo_device.cuh"

namespace cvo_gb {

enum { MODE_ALIGN = 0, MODE_IP = 1, MODE_EXPORT = 2 };
constexpr int kAssocThreads = 128;
constexpr int kReduceRows = 1024;
constexpr int kReduceThreads = 256;
constexpr int kStepThreads = 256;
constexpr int kPartStride = 12;
constexpr float kBand = 2e-5f;      // relative band around sp_thres re-evaluated in double
constexpr int kWaitLimit = 1 << 22; // mbarrier polls before a staged copy is declared lost

// ------------------------------------------------------------ pair value
// Exact kernel value as the reference computes it (double exp, float products);
// used only for pairs whose fast FP32 value is within kBand of the threshold,
// so it is kept out of line to keep the hot loop's register count low.
__device__ __noinline__ float exact_value(const KParams &K, float l, float d2, float d2c, float d2s, float geo) {
  float kk = 1.f, ck = 1.f, sk = 1.f;
  if (K.use_geo) kk = __double2float_rn(dm((double)K.sigma2, exp(__ddiv_rn(-(double)d2, dm(dm(2.0, (double)l), (double)l)))));
  if (K.use_int) ck = __double2float_rn(dm((double)K.c_sigma2, exp(__ddiv_rn(-(double)d2c, dm(2.0, (double)K.c2)))));
  if (K.use_sem)
    sk = __double2float_rn(dm((double)K.s_sigma_sq, exp(__ddiv_rn(-(double)d2s, dm(dm(2.0, (double)K.s_ell), (double)K.s_ell)))));
  return fm(fm(fm(ck, kk), sk), geo);
}

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
  float ckf = K.use_int ? fm(K.c_sigma2, __expf(fm(-d2c, __frcp_rn(fm(2.f, K.c2))))) : 1.f;
  float skf = K.use_sem ? fm(K.s_sigma_sq, __expf(fm(-d2s, __frcp_rn(fm(fm(2.f, K.s_ell), K.s_ell))))) : 1.f;
  float af = fm(fm(fm(ckf, kf), skf), geo);
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
  if (gt == 0 && *B.active > 0) *B.active_iters += 1;
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
// arrive in grid order, so once a row holds `cap` pairs its ELL row becomes a
// max-heap keyed by the original target index: a later pair with a smaller
// index replaces the root.  At the end the row holds exactly the `cap` smallest
// kept indices, i.e. the reference's set.
struct EllRow {
  int *j;
  float *v;
  size_t stride;
  __device__ __forceinline__ int &J(int c) const { return j[(size_t)c * stride]; }
  __device__ __forceinline__ float &V(int c) const { return v[(size_t)c * stride]; }
  __device__ void sift_down(int i, int cap, int jn, float vn) const {
    while (true) {
      int l = 2 * i + 1;
      if (l >= cap) break;
      int c = l;
      int jc = J(l);
      if (l + 1 < cap) {
        int jr = J(l + 1);
        if (jr > jc) { c = l + 1; jc = jr; }
      }
      if (jc <= jn) break;
      J(i) = jc;
      V(i) = V(c);
      i = c;
    }
    J(i) = jn;
    V(i) = vn;
  }
  __device__ void heapify(int cap) const {
    for (int i = cap / 2 - 1; i >= 0; i--) sift_down(i, cap, J(i), V(i));
  }
};

// ------------------------------------------------------- candidate staging
// A chunk of up to CH candidate targets in shared memory.  The grid stores the
// members of one cell contiguously (positions, features, labels, geometric
// types), so one chunk is 1-4 contiguous 16-byte-aligned ranges that a single
// lane copies with bulk copies (the TMA unit) completed on an mbarrier.
template <int FCH, int LCH, bool GT>
struct __align__(16) StageBuf {
  static constexpr int CH = (LCH > 5) ? 16 : 32;
  float4 pos[CH];
  float4 feat[CH * (FCH > 0 ? FCH : 1)];
  float4 lab[CH * (LCH > 0 ? LCH : 1)];
  float4 geo[GT ? CH : 1];
};

template <int FCH, int LCH, bool GT>
__device__ __forceinline__ void stage_issue(StageBuf<FCH, LCH, GT> &buf, uint64_t *mbar, const float4 *ycur,
                                            const GridDesc &G, int t0, int nk) {
  constexpr uint32_t rec = 16u * (1 + FCH + LCH + (GT ? 1 : 0));
  fence_proxy_async_smem();   // the lanes' reads of this buffer precede the copy into it
  mbar_arrive_expect_tx(mbar, rec * (uint32_t)nk);
  bulk_g2s(buf.pos, ycur + t0, 16u * nk, mbar);
  if (FCH > 0)
    bulk_g2s(buf.feat, reinterpret_cast<const float4 *>(G.feat) + (size_t)t0 * FCH, 16u * FCH * nk, mbar);
  if (LCH > 0)
    bulk_g2s(buf.lab, reinterpret_cast<const float4 *>(G.lab) + (size_t)t0 * LCH, 16u * LCH * nk, mbar);
  if (GT) bulk_g2s(buf.geo, G.geo + t0, 16u * nk, mbar);
}

// ------------------------------------------------------------ association
// One warp per tile of 32 spatially adjacent source points (Morton order).  The
// warp scans the grid cells overlapping the union of its lanes' query boxes;
// each candidate target is staged once per warp in shared memory and tested by
// every lane against its own source point.  Chunks are double-buffered: the copy
// of chunk k+1 is in flight while the lanes test chunk k.
template <int FCH, int LCH, bool GT>
__global__ void __launch_bounds__(kAssocThreads) k_assoc(BatchDev B, KParams K) {
  using Buf = StageBuf<FCH, LCH, GT>;
  constexpr int CH = Buf::CH;
  __shared__ Buf stage_all[kAssocThreads / 32][2];
  __shared__ __align__(8) uint64_t mbar_all[kAssocThreads / 32][2];
  __shared__ GridDesc grid_all[kAssocThreads / 32];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  Buf *stage = stage_all[wib];
  uint64_t *mbar = mbar_all[wib];
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (gw >= B.total_warps) return;
  const int p = find_segment(B.tile_off, B.npairs, gw);
  PairDev *P = &B.pairs[p];
  if (P->done) return;
  if (lane == 0) {
    grid_all[wib] = P->levels[P->level];
    mbar_init(&mbar[0], 1);
    mbar_init(&mbar[1], 1);
    fence_proxy_async_smem();
  }
  __syncwarp();
  const GridDesc &G = grid_all[wib];
  uint32_t parity[2] = {0u, 0u};
  const int n = P->n;
  const int s = (gw - B.tile_off[p]) * 32 + lane;
  const bool valid = s < n;
  const float ell = P->ell;
  const int cap = P->cap;
  const int mode = P->mode;
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
  int cnt = 0;
  int root_j = 0x7FFFFFFF;   // largest kept index once the row is a heap
  float w0 = 0.f, w1 = 0.f, w2 = 0.f, v0 = 0.f, v1 = 0.f, v2 = 0.f, as = 0.f;
  const float4 *__restrict__ ycur = P->ycur;
  const EllRow row{P->A_j + (valid ? s : 0), P->A_v + (valid ? s : 0), (size_t)n};
  bool lost = false;
  for (int pass = 0; pass < npass && !lost; pass++) {
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
    const int ncells = nx * ny * nz;
    for (int cb = 0; cb < ncells && !lost; cb += 32) {
      int ci = cb + lane;
      int2 se = make_int2(0, 0);
      if (ci < ncells) {
        int cx = x0 + ci % nx, cy = y0 + (ci / nx) % ny, cz = z0 + ci / (nx * ny);
        se = grid_lookup(G, cx, cy, cz);
      }
      unsigned mk = __ballot_sync(FULLMASK, se.y > 0);
      if (!mk) continue;
      // chunk walk over the non-empty cells' segments
      int b = __ffs(mk) - 1;
      mk &= mk - 1;
      int seg_start = __shfl_sync(FULLMASK, se.x, b);
      int seg_cnt = __shfl_sync(FULLMASK, se.y, b);
      int off = 0;
      int cur = 0;
      if (lane == 0) stage_issue<FCH, LCH, GT>(stage[cur], &mbar[cur], ycur, G, seg_start, min(CH, seg_cnt));
      while (true) {
        const int nk = min(CH, seg_cnt - off);
        // next chunk: rest of this segment, else the next non-empty cell
        int n_start = seg_start, n_cnt = seg_cnt, n_off = off + CH;
        bool has_next = true;
        if (n_off >= seg_cnt) {
          if (mk) {
            int b2 = __ffs(mk) - 1;
            mk &= mk - 1;
            n_start = __shfl_sync(FULLMASK, se.x, b2);
            n_cnt = __shfl_sync(FULLMASK, se.y, b2);
            n_off = 0;
          } else {
            has_next = false;
          }
        }
        if (has_next && lane == 0)
          stage_issue<FCH, LCH, GT>(stage[cur ^ 1], &mbar[cur ^ 1], ycur, G, n_start + n_off,
                                    min(CH, n_cnt - n_off));
        const bool ok = __all_sync(FULLMASK, mbar_wait(&mbar[cur], parity[cur], kWaitLimit));
        parity[cur] ^= 1u;
        if (!ok) {
          // a staged copy did not complete: record it, drain the other buffer, stop
          if (lane == 0) atomicExch(B.err, CVO_ERR_TIMEOUT);
          if (has_next) mbar_wait(&mbar[cur ^ 1], parity[cur ^ 1], kWaitLimit);
          lost = true;
          break;
        }
        const Buf &sb = stage[cur];
        for (int k = 0; k < nk; k++) {
          const float4 y = sb.pos[k];
          float a;
          bool acc = eval_pair<FCH, LCH, GT>(K, F, C, me, rc.l, rc.d2t, rc.inv2l2, x, xf, xl, xg, y,
                                             &sb.feat[k * (FCH > 0 ? FCH : 1)], &sb.lab[k * (LCH > 0 ? LCH : 1)],
                                             &sb.geo[GT ? k : 0], a);
          if (acc) {
            const int j = __float_as_int(y.w);
            if (cnt < cap) {
              row.J(cnt) = j;
              row.V(cnt) = a;
              w0 = fmaf(a, fs(fm(x.y, y.z), fm(x.z, y.y)), w0);
              w1 = fmaf(a, fs(fm(x.z, y.x), fm(x.x, y.z)), w1);
              w2 = fmaf(a, fs(fm(x.x, y.y), fm(x.y, y.x)), w2);
              v0 = fmaf(a, y.x - x.x, v0);
              v1 = fmaf(a, y.y - x.y, v1);
              v2 = fmaf(a, y.z - x.z, v2);
              as += a;
            } else if (cap > 0) {
              if (cnt == cap) {
                row.heapify(cap);
                root_j = row.J(0);
              }
              if (j < root_j) {
                row.sift_down(0, cap, j, a);
                root_j = row.J(0);
              }
            }
            cnt++;
          }
        }
        __syncwarp();
        if (!has_next) break;
        seg_start = n_start;
        seg_cnt = n_cnt;
        off = n_off;
        cur ^= 1;
      }
    }
  }
  if (valid && !lost) {
    if (cnt > cap && cap > 0) {
      // the row overflowed: its sums come from the selected entries
      const float4 *__restrict__ yorig = P->yorig;
      w0 = w1 = w2 = v0 = v1 = v2 = as = 0.f;
      for (int c = 0; c < cap; c++) {
        float a = row.V(c);
        float4 y = __ldg(&yorig[row.J(c)]);
        w0 = fmaf(a, fs(fm(x.y, y.z), fm(x.z, y.y)), w0);
        w1 = fmaf(a, fs(fm(x.z, y.x), fm(x.x, y.z)), w1);
        w2 = fmaf(a, fs(fm(x.x, y.y), fm(x.y, y.x)), w2);
        v0 = fmaf(a, y.x - x.x, v0);
        v1 = fmaf(a, y.y - x.y, v1);
        v2 = fmaf(a, y.z - x.z, v2);
        as += a;
      }
    }
    int kept = cnt < cap ? cnt : cap;
    P->nnz_row[s] = kept;
    float *rs = P->row_sums + (size_t)s * 8;
    if (mode == MODE_ALIGN) {
      rs[0] = __fdiv_rn(w0, K.c); rs[1] = __fdiv_rn(w1, K.c); rs[2] = __fdiv_rn(w2, K.c);
      rs[3] = __fdiv_rn(v0, K.d); rs[4] = __fdiv_rn(v1, K.d); rs[5] = __fdiv_rn(v2, K.d);
    } else {
      rs[0] = rs[1] = rs[2] = rs[3] = rs[4] = rs[5] = 0.f;
    }
    rs[6] = as;
  }
}

}  // namespace cvo_gb
