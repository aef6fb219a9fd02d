// cvo_kernels.cuh -- per-iteration kernels of the batched CVO engine.
//
// One iteration of the reference's align loop (src/cvo/CvoGPU.cu:1303-1433) is
// five launches over every active pair of a batch:
//   k_transform  target transform y' = R^T (y - T)            (CvoGPU_impl.cu:32-83)
//   k_assoc      fused association: grid candidates -> kernel value -> threshold
//                -> ELL write -> gradient partials             (CvoGPU.cu:951-1099, 2001-2062)
//   k_overflow   rows holding more than `cap` kept pairs: exact first-`cap`-by-index
//                selection (radix select on the target index)  (CvoGPU.cu:994-996)
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
constexpr int kAssocThreads = 256;
constexpr int kOvfThreads = 128;
constexpr int kReduceRows = 1024;
constexpr int kReduceThreads = 256;
constexpr int kStepThreads = 256;
constexpr int kPartStride = 12;
constexpr float kBand = 2e-5f;      // relative band around sp_thres re-evaluated in double

// ------------------------------------------------------------ pair value
// Kernel value of one (source, target) pair with the semantics of
// fill_in_A_mat_gpu (src/cvo/CvoGPU.cu:996-1075).  `pre` is the lane's
// participation; returns whether the pair is kept and its value in a.
// All lanes of the warp must call it together.
template <int FCH, int LCH, bool GT>
__device__ __forceinline__ bool eval_pair(const KParams &K, int F, int C, bool pre, float l, float d2t, float inv2l2,
                                          const float4 &x, const float4 (&xf)[FCH > 0 ? FCH : 1],
                                          const float4 (&xl)[LCH > 0 ? LCH : 1], float2 xg, const float4 &y,
                                          const float4 *__restrict__ yfp, const float4 *__restrict__ ylp,
                                          const float2 *__restrict__ ygp, float &a) {
  bool pass = pre;
  float d2 = 0.f;
  if (K.use_geo) {
    d2 = sqdist3(y.x, y.y, y.z, x.x, x.y, x.z);
    pass = pass && (d2 < d2t);
  }
  if (!__any_sync(FULLMASK, pass)) return false;
  float geo = 1.f;
  if (GT) {
    float2 yg = __ldg(ygp);
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
      float4 yf = __ldg(yfp + q);
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
      float4 yl = __ldg(ylp + q);
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
  if (pass && fabsf(fs(af, K.sp_thres)) <= kBand * K.sp_thres) {
    // exact evaluation as in the reference (double exp, float products)
    float kk = 1.f, ck = 1.f, sk = 1.f;
    if (K.use_geo) kk = __double2float_rn(dm((double)K.sigma2, exp(__ddiv_rn(-(double)d2, dm(dm(2.0, (double)l), (double)l)))));
    if (K.use_int) ck = __double2float_rn(dm((double)K.c_sigma2, exp(__ddiv_rn(-(double)d2c, dm(2.0, (double)K.c2)))));
    if (K.use_sem)
      sk = __double2float_rn(dm((double)K.s_sigma_sq, exp(__ddiv_rn(-(double)d2s, dm(dm(2.0, (double)K.s_ell), (double)K.s_ell)))));
    af = fm(fm(fm(ck, kk), sk), geo);
  }
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
__global__ void k_transform(BatchDev B) {
  int gt = blockIdx.x * blockDim.x + threadIdx.x;
  if (gt == 0) *B.ovf_n = 0;
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
  P->ycur[t] = make_float4(o0, o1, o2, y.w);
}

// ------------------------------------------------------------ association
template <int FCH, int LCH, bool GT>
__global__ void __launch_bounds__(kAssocThreads) k_assoc(BatchDev B, KParams K) {
  const int lane = threadIdx.x & 31;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (gw >= B.total_warps) return;
  const int p = find_segment(B.tile_off, B.npairs, gw);
  PairDev *P = &B.pairs[p];
  if (P->done) return;
  const int n = P->n;
  const int s = (gw - B.tile_off[p]) * 32 + lane;
  const bool valid = s < n;
  const float ell = P->ell;
  const int cap = P->cap;
  const int mode = P->mode;
  const GridDesc G = P->levels[P->level];
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
  lox = warp_min(lox); loy = warp_min(loy); loz = warp_min(loz);
  hix = warp_max(hix); hiy = warp_max(hiy); hiz = warp_max(hiz);
  int x0, y0, z0, nx, ny, nz;
  int cnt = 0;
  float w0 = 0.f, w1 = 0.f, w2 = 0.f, v0 = 0.f, v1 = 0.f, v2 = 0.f, as = 0.f;
  if (cell_range(G, lox, loy, loz, hix, hiy, hiz, x0, y0, z0, nx, ny, nz)) {
    const int ncells = nx * ny * nz;
    const float4 *__restrict__ ycur = P->ycur;
    int *__restrict__ Aj = P->A_j;
    float *__restrict__ Av = P->A_v;
    for (int cb = 0; cb < ncells; cb += 32) {
      int ci = cb + lane;
      int2 se = make_int2(0, 0);
      if (ci < ncells) {
        int cx = x0 + ci % nx, cy = y0 + (ci / nx) % ny, cz = z0 + ci / (nx * ny);
        se = grid_lookup(G, cx, cy, cz);
      }
      unsigned mk = __ballot_sync(FULLMASK, se.y > 0);
      while (mk) {
        int b = __ffs(mk) - 1;
        mk &= mk - 1;
        int start = __shfl_sync(FULLMASK, se.x, b);
        int end = start + __shfl_sync(FULLMASK, se.y, b);
        for (int t = start; t < end; t++) {
          float4 y = __ldg(&ycur[t]);
          float a;
          bool acc = eval_pair<FCH, LCH, GT>(K, F, C, valid, rc.l, rc.d2t, rc.inv2l2,
                                             x, xf, xl, xg, y,
                                             reinterpret_cast<const float4 *>(G.feat) + (size_t)t * FCH,
                                             reinterpret_cast<const float4 *>(G.lab) + (size_t)t * LCH, G.geo + t, a);
          if (acc) {
            if (cnt < cap) {
              if (mode != MODE_IP) {
                Aj[(size_t)cnt * n + s] = t;
                Av[(size_t)cnt * n + s] = a;
              }
              if (mode == MODE_ALIGN) {
                w0 = fmaf(a, fs(fm(x.y, y.z), fm(x.z, y.y)), w0);
                w1 = fmaf(a, fs(fm(x.z, y.x), fm(x.x, y.z)), w1);
                w2 = fmaf(a, fs(fm(x.x, y.y), fm(x.y, y.x)), w2);
                v0 = fmaf(a, y.x - x.x, v0);
                v1 = fmaf(a, y.y - x.y, v1);
                v2 = fmaf(a, y.z - x.z, v2);
              }
              as += a;
            }
            cnt++;
          }
        }
      }
    }
  }
  if (valid) {
    int kept = cnt < cap ? cnt : cap;
    P->nnz_row[s] = kept;
    float *rs = P->row_sums + (size_t)s * 8;
    rs[0] = __fdiv_rn(w0, K.c); rs[1] = __fdiv_rn(w1, K.c); rs[2] = __fdiv_rn(w2, K.c);
    rs[3] = __fdiv_rn(v0, K.d); rs[4] = __fdiv_rn(v1, K.d); rs[5] = __fdiv_rn(v2, K.d);
    rs[6] = as;
    if (cnt > cap && cap > 0) {
      int idx = atomicAdd(B.ovf_n, 1);
      if (idx < B.ovf_cap) { B.ovf[idx].pair = p; B.ovf[idx].row = s; }
      else atomicExch(B.err, CVO_ERR_CAPACITY);
    }
  }
}

// --------------------------------------------------------------- overflow
// One warp per overflowing row.  The kept set of the reference is the first
// `cap` kept pairs in ascending target index; it equals {kept j : j <= J*} with
// J* the cap-th smallest kept index, found by a two-digit radix select.
template <int FCH, int LCH, bool GT>
__global__ void __launch_bounds__(kOvfThreads) k_overflow(BatchDev B, KParams K) {
  __shared__ int hist_all[kOvfThreads / 32][1 << kHist1Bits];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  int *hist = hist_all[wib];
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  const int novf = min(*B.ovf_n, B.ovf_cap);
  for (int idx = gw; idx < novf; idx += nw) {
    const int p = B.ovf[idx].pair, s = B.ovf[idx].row;
    PairDev *P = &B.pairs[p];
    const int n = P->n, m = P->m, cap = P->cap, mode = P->mode;
    const GridDesc G = P->levels[P->level];
    float4 x = __ldg(&P->xs[s]);
    float4 xf[FCH > 0 ? FCH : 1];
    float4 xl[LCH > 0 ? LCH : 1];
    float2 xg = make_float2(0.f, 0.f);
#pragma unroll
    for (int q = 0; q < (FCH > 0 ? FCH : 1); q++)
      xf[q] = FCH > 0 ? __ldg(reinterpret_cast<const float4 *>(P->xf) + (size_t)s * FCH + q) : make_float4(0, 0, 0, 0);
#pragma unroll
    for (int q = 0; q < (LCH > 0 ? LCH : 1); q++)
      xl[q] = LCH > 0 ? __ldg(reinterpret_cast<const float4 *>(P->xl) + (size_t)s * LCH + q) : make_float4(0, 0, 0, 0);
    if (GT) xg = __ldg(&P->xg[s]);
    const float Tn = fabsf(P->T[0]) + fabsf(P->T[1]) + fabsf(P->T[2]);
    RowConst rc = row_const(K, P->ell, x.w, Tn);
    const float *R = P->R;
    float qx = fmaf(R[0], x.x, fmaf(R[1], x.y, fmaf(R[2], x.z, P->T[0])));
    float qy = fmaf(R[3], x.x, fmaf(R[4], x.y, fmaf(R[5], x.z, P->T[1])));
    float qz = fmaf(R[6], x.x, fmaf(R[7], x.y, fmaf(R[8], x.z, P->T[2])));
    int x0, y0, z0, nx, ny, nz;
    if (!cell_range(G, qx - rc.rq, qy - rc.rq, qz - rc.rq, qx + rc.rq, qy + rc.rq, qz + rc.rq, x0, y0, z0, nx, ny, nz))
      continue;
    const int ncells = nx * ny * nz;
    int bits = 1;
    while ((1 << bits) < m) bits++;
    const int sh = bits > kHist1Bits ? bits - kHist1Bits : 0;
    const float4 *__restrict__ ycur = P->ycur;
    const int Fv = P->F, Cv = P->C;
    // pass 0: bin histogram of kept target indices; pass 1: low digits inside
    // the selected bin; pass 2: accumulate pairs with index <= J*.
    int bin = 0, need = cap, jstar = 0x7FFFFFFF;
    for (int pass = 0; pass < 3; pass++) {
      if (pass < 2) {
        for (int k = lane; k < (1 << kHist1Bits); k += 32) hist[k] = 0;
        __syncwarp();
      }
      int slot_base = 0;
      float w0 = 0.f, w1 = 0.f, w2 = 0.f, v0 = 0.f, v1 = 0.f, v2 = 0.f, as = 0.f;
      for (int cb = 0; cb < ncells; cb += 32) {
        int ci = cb + lane;
        int2 se = make_int2(0, 0);
        if (ci < ncells) {
          int cx = x0 + ci % nx, cy = y0 + (ci / nx) % ny, cz = z0 + ci / (nx * ny);
          se = grid_lookup(G, cx, cy, cz);
        }
        unsigned mk = __ballot_sync(FULLMASK, se.y > 0);
        while (mk) {
          int b = __ffs(mk) - 1;
          mk &= mk - 1;
          int start = __shfl_sync(FULLMASK, se.x, b);
          int end = start + __shfl_sync(FULLMASK, se.y, b);
          for (int tb = start; tb < end; tb += 32) {
            int t = tb + lane;
            bool act = t < end;
            int tt = act ? t : start;
            float4 y = __ldg(&ycur[tt]);
            float a;
            bool acc = eval_pair<FCH, LCH, GT>(K, Fv, Cv, act, rc.l, rc.d2t, rc.inv2l2, x, xf, xl, xg, y,
                                               reinterpret_cast<const float4 *>(G.feat) + (size_t)tt * FCH,
                                               reinterpret_cast<const float4 *>(G.lab) + (size_t)tt * LCH, G.geo + tt, a);
            int j = __float_as_int(y.w);
            if (pass == 0) {
              if (acc) atomicAdd(&hist[j >> sh], 1);
            } else if (pass == 1) {
              if (acc && (j >> sh) == bin) atomicAdd(&hist[j & ((1 << sh) - 1)], 1);
            } else {
              bool keep = acc && j <= jstar;
              unsigned km = __ballot_sync(FULLMASK, keep);
              if (keep) {
                int slot = slot_base + __popc(km & ((1u << lane) - 1u));
                if (mode != MODE_IP && slot < cap) {
                  P->A_j[(size_t)slot * n + s] = tt;
                  P->A_v[(size_t)slot * n + s] = a;
                }
                if (mode == MODE_ALIGN) {
                  w0 = fmaf(a, fs(fm(x.y, y.z), fm(x.z, y.y)), w0);
                  w1 = fmaf(a, fs(fm(x.z, y.x), fm(x.x, y.z)), w1);
                  w2 = fmaf(a, fs(fm(x.x, y.y), fm(x.y, y.x)), w2);
                  v0 = fmaf(a, y.x - x.x, v0);
                  v1 = fmaf(a, y.y - x.y, v1);
                  v2 = fmaf(a, y.z - x.z, v2);
                }
                as += a;
              }
              slot_base += __popc(km);
            }
          }
        }
      }
      __syncwarp();
      if (pass < 2) {
        // find the bin where the running count reaches `need`
        const int nb = pass == 0 ? (1 << kHist1Bits) : (1 << sh);
        const int per = (nb + 31) / 32;
        int loc = 0;
        for (int k = 0; k < per; k++) { int bi = lane * per + k; if (bi < nb) loc += hist[bi]; }
        int incl = loc;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) { int tv = __shfl_up_sync(FULLMASK, incl, o); if (lane >= o) incl += tv; }
        int excl = incl - loc;
        bool mine = excl < need && incl >= need;
        unsigned who = __ballot_sync(FULLMASK, mine);
        int src = who ? __ffs(who) - 1 : 31;
        int found = 0, before = 0;
        if (lane == src) {
          int run = excl;
          found = lane * per + per - 1;
          for (int k = 0; k < per; k++) {
            int bi = lane * per + k;
            int c = bi < nb ? hist[bi] : 0;
            if (run + c >= need) { found = bi; break; }
            run += c;
          }
          before = run;
        }
        found = __shfl_sync(FULLMASK, found, src);
        before = __shfl_sync(FULLMASK, before, src);
        if (pass == 0) { bin = found; need = need - before; }
        else jstar = (bin << sh) | found;
        __syncwarp();
      } else {
        w0 = warp_sumf(w0); w1 = warp_sumf(w1); w2 = warp_sumf(w2);
        v0 = warp_sumf(v0); v1 = warp_sumf(v1); v2 = warp_sumf(v2);
        as = warp_sumf(as);
        if (lane == 0) {
          P->nnz_row[s] = cap;
          float *rs = P->row_sums + (size_t)s * 8;
          rs[0] = __fdiv_rn(w0, K.c); rs[1] = __fdiv_rn(w1, K.c); rs[2] = __fdiv_rn(w2, K.c);
          rs[3] = __fdiv_rn(v0, K.d); rs[4] = __fdiv_rn(v1, K.d); rs[5] = __fdiv_rn(v2, K.d);
          rs[6] = as;
        }
      }
    }
  }
}

}  // namespace cvo_gb
