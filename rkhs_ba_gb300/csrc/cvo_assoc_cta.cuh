// cvo_assoc_cta.cuh -- block-cooperative association for dense tiles.
//
// Same result as assoc_warp (the kernel matrix of fill_in_A_mat_gpu,
// src/cvo/CvoGPU.cu:951-1099, with the first-`cap`-by-index rows): a block of four
// warps owns 128 consecutive source rows (4 Morton tiles of one pair).  The block
// lists the non-empty grid cells near the union of its rows' query balls once, then
// streams their members through shared memory 128 candidates at a time: every
// thread loads one candidate (coalesced) and builds its prefilter vector, and each
// warp runs the tensor-core prefilter of its 32 rows against all 128 candidates and
// the exact per-pair evaluation of the survivors.  A row's first `cap` kept pairs
// go to its ELL slots and any further ones to its spill list (put_kept).  Candidate
// order (cell list order, members ascending) is fixed, so rows receive their kept
// pairs in a deterministic order.  Blocks whose union box is sparse, or whose prefilter
// vectors leave the f16 range, run the per-warp path instead.
#pragma once
#include "cvo_kernels.cuh"

namespace cvo_gb {

constexpr int kCtaWarps = 4;
constexpr int kCtaRows = 32 * kCtaWarps;     // source rows per block
constexpr int kCtaCand = 128;                // candidates per streaming step
constexpr int kCtaCells = 1024;              // listed cells per streaming pass
constexpr int kCtaFlushCands = 4096;         // stream once this many candidates are listed

template <int FCH, int LCH, bool GT>
struct __align__(16) CtaDense {
  static constexpr int FP = FCH > 0 ? FCH : 1, LP = LCH > 0 ? LCH : 1;
  float4 pos[kCtaCand];
  float4 feat[kCtaCand * FP];
  float4 lab[kCtaCand * LP];
  float4 geo[GT ? kCtaCand : 1];
  uint4 bpl[4][kCtaCand];                    // candidate planes: hi k0-7, hi k8-15, lo k0-7, lo k8-15
  uint4 apl[kCtaWarps][4][32];               // row planes per warp
  SrcRows<FCH, LCH> rows[kCtaWarps];
  int2 cell[kCtaCells];                      // listed cells: first sorted position, member count
  int cpre[kCtaCells + 1];                   // prefix of member counts
  float fred[kCtaWarps][12];                 // block reductions
  long long lred[kCtaWarps][2];
  int ired[kCtaWarps][2];
  int okg[kCtaCand / 32];
  int gcnt[kCtaWarps][32];                   // split items: kept pairs per row and candidate group
  GridDesc G;
};

template <int FCH, int LCH, bool GT>
struct CtaSmem {
  static constexpr size_t kDense = sizeof(CtaDense<FCH, LCH, GT>);
  static constexpr size_t kWarp = AssocSmem<FCH, LCH, GT>::kBytes;
  static constexpr size_t kBytes = kDense > kWarp ? kDense : kWarp;
};

// Exclusive prefix over the block of a per-thread count; returns the block total.
__device__ __forceinline__ int block_excl_scan(int v, int &excl, int (*scratch)[2]) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(FULLMASK, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) scratch[w][0] = incl;
  __syncthreads();
  int base = 0, total = 0;
#pragma unroll
  for (int k = 0; k < kCtaWarps; k++) {
    const int c = scratch[k][0];
    if (k < w) base += c;
    total += c;
  }
  __syncthreads();
  excl = base + incl - v;
  return total;
}

// One work item: the four tiles gw0 .. gw0 + 3 (one pair), each warp owning one tile.
// split >= 0 (a heavy item, split by k_order_items): only tile gw0 + split, with the
// four warps sharing its candidate stream -- warp w evaluates candidate group w of
// every 128-candidate step for the tile's 32 rows.  The kept pairs of a row are then
// placed in the order (step, group, candidate) exactly as one warp would place them:
// each warp counts its group's kept pairs per row, and after a block barrier writes
// them behind the counts of the lower groups (a second, identical evaluation of its
// survivors).  So the kernel matrix and the order of every row's entries do not
// depend on which items are split.
template <int FCH, int LCH, bool GT>
__device__ __forceinline__ void assoc_block(const BatchDev &B, const KParams &K, int gw0, int split,
                                            unsigned char *cta_smem) {
  using D = CtaDense<FCH, LCH, GT>;
  constexpr int FP = D::FP, LP = D::LP;
  D &sm = *reinterpret_cast<D *>(cta_smem);
  const int tid = threadIdx.x, lane = tid & 31, wib = tid >> 5;
  const int gw = gw0 + (split >= 0 ? split : wib);
  // the per-warp fallback runs once per tile: in a split item only warp 0 takes it
  const bool fallback_warp = split < 0 || wib == 0;
  const int p = find_segment(B.tile_off, B.npairs, gw0);
  PairDev *P = &B.pairs[p];
  if (P->done) return;
  if (!K.use_mma || P->F > 8) {
    if (fallback_warp) assoc_warp<FCH, LCH, GT>(B, K, gw, cta_smem);
    return;
  }
  const int n = P->n;
  const int s = (gw - B.tile_off[p]) * 32 + lane;
  const bool valid = s < n;
  const int cap = P->cap, F = P->F, C = P->C;
  const float4 x = valid ? __ldg(&P->xs[s]) : make_float4(0.f, 0.f, 0.f, 0.f);
  float4 xf[FP];
  float4 xl[LP];
#pragma unroll
  for (int q = 0; q < FP; q++)
    xf[q] = (FCH > 0 && valid) ? __ldg(reinterpret_cast<const float4 *>(P->xf) + (size_t)s * FCH + q)
                               : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
  for (int q = 0; q < LP; q++)
    xl[q] = (LCH > 0 && valid) ? __ldg(reinterpret_cast<const float4 *>(P->xl) + (size_t)s * LCH + q)
                               : make_float4(0.f, 0.f, 0.f, 0.f);
  const float2 xg = (GT && valid) ? __ldg(&P->xg[s]) : make_float2(0.f, 0.f);
  const float Tn = fabsf(P->T[0]) + fabsf(P->T[1]) + fabsf(P->T[2]);
  const RowConst rc = row_const(K, P->ell, x.w, Tn);
  const float *R = P->R;
  const float qx = fmaf(R[0], x.x, fmaf(R[1], x.y, fmaf(R[2], x.z, P->T[0])));
  const float qy = fmaf(R[3], x.x, fmaf(R[4], x.y, fmaf(R[5], x.z, P->T[1])));
  const float qz = fmaf(R[6], x.x, fmaf(R[7], x.y, fmaf(R[8], x.z, P->T[2])));
  if (tid == 0) sm.G = P->levels[P->level];
  __syncthreads();
  const GridDesc &G = sm.G;
  // per-warp reductions: query-point box, radius, source sum, counts, cells
  {
    const float lo0 = valid ? qx - rc.rq : INFINITY, lo1 = valid ? qy - rc.rq : INFINITY, lo2 = valid ? qz - rc.rq : INFINITY;
    const float hi0 = valid ? qx + rc.rq : -INFINITY, hi1 = valid ? qy + rc.rq : -INFINITY, hi2 = valid ? qz + rc.rq : -INFINITY;
    int ox0, oy0, oz0, onx, ony, onz;
    long long own = 0;
    if (valid && cell_range(G, lo0, lo1, lo2, hi0, hi1, hi2, ox0, oy0, oz0, onx, ony, onz)) own = (long long)onx * ony * onz;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) own += __shfl_xor_sync(FULLMASK, own, o);
    const float w0 = warp_min(lo0), w1 = warp_min(lo1), w2 = warp_min(lo2);
    const float w3 = warp_max(hi0), w4 = warp_max(hi1), w5 = warp_max(hi2);
    const float q0 = warp_min(valid ? qx : INFINITY), q1 = warp_min(valid ? qy : INFINITY), q2 = warp_min(valid ? qz : INFINITY);
    const float q3 = warp_max(valid ? qx : -INFINITY), q4 = warp_max(valid ? qy : -INFINITY), q5 = warp_max(valid ? qz : -INFINITY);
    const float rq = warp_max(valid ? rc.rq : 0.f);
    const float sx = warp_sumf(valid ? x.x : 0.f), sy = warp_sumf(valid ? x.y : 0.f), sz = warp_sumf(valid ? x.z : 0.f);
    const int nv = warp_sumi(valid ? 1 : 0);
    long long wc = 0;
    int ux0, uy0, uz0, unx, uny, unz;
    if (nv > 0 && cell_range(G, w0, w1, w2, w3, w4, w5, ux0, uy0, uz0, unx, uny, unz)) wc = (long long)unx * uny * unz;
    if (lane == 0) {
      float *f = sm.fred[wib];
      f[0] = w0; f[1] = w1; f[2] = w2; f[3] = w3; f[4] = w4; f[5] = w5;
      f[6] = q0; f[7] = q1; f[8] = q2; f[9] = q3; f[10] = q4; f[11] = q5;
      sm.lred[wib][0] = own;
      sm.lred[wib][1] = wc;
      sm.ired[wib][0] = nv;
      sm.ired[wib][1] = __float_as_int(rq);
      sm.rows[wib].rc[0].w = sx; sm.rows[wib].rc[1].w = sy; sm.rows[wib].rc[2].w = sz;   // scratch, rewritten below
    }
  }
  __syncthreads();
  float blo[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
  float qlo[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
  float brq = 0.f, bsx = 0.f, bsy = 0.f, bsz = 0.f;
  long long own_sum = 0, warp_cells = 0;
  int nvb = 0;
#pragma unroll
  for (int w = 0; w < kCtaWarps; w++) {
    const float *f = sm.fred[w];
    for (int k = 0; k < 3; k++) {
      blo[k] = fminf(blo[k], f[k]); blo[3 + k] = fmaxf(blo[3 + k], f[3 + k]);
      qlo[k] = fminf(qlo[k], f[6 + k]); qlo[3 + k] = fmaxf(qlo[3 + k], f[9 + k]);
    }
    own_sum += sm.lred[w][0];
    warp_cells += sm.lred[w][1];
    nvb += sm.ired[w][0];
    brq = fmaxf(brq, __int_as_float(sm.ired[w][1]));
    bsx += sm.rows[w].rc[0].w; bsy += sm.rows[w].rc[1].w; bsz += sm.rows[w].rc[2].w;
  }
  int x0, y0, z0, nx, ny, nz;
  const bool union_ok = nvb > 0 && cell_range(G, blo[0], blo[1], blo[2], blo[3], blo[4], blo[5], x0, y0, z0, nx, ny, nz);
  const long long ucells = union_ok ? (long long)nx * ny * nz : 0;
  // dense: the union box is not much larger than the rows' own boxes together (the
  // per-warp path's sparse test) nor than the four warps' boxes together
  const bool dense = union_ok && !(ucells > 64 && ucells > 2 * own_sum) && ucells <= 2 * warp_cells;
  __syncthreads();
  if (!dense) {
    if (fallback_warp) assoc_warp<FCH, LCH, GT>(B, K, gw, cta_smem);
    return;
  }
  // ---- dense: prefilter vectors of the rows around the block's centre
  const float inv = 1.f / (float)nvb;
  const float pcx = bsx * inv, pcy = bsy * inv, pcz = bsz * inv;
  const float cw = K.use_int ? K.inv2c2 : 0.f;
  bool okA;
  {
    float av[16];
    mma_row_vec<FCH>(av, valid, x, xf, F, rc.inv2l2, cw, pcx, pcy, pcz);
    okA = mma_store_vec(av, &sm.apl[wib][0][0], 32, lane);
  }
  SrcRows<FCH, LCH> &sr = sm.rows[wib];
  sr.x[lane] = x;
  sr.rc[lane] = make_float4(rc.l, rc.d2t, rc.inv2l2, xg.x);
  sr.g1[lane] = xg.y;
#pragma unroll
  for (int q = 0; q < FP; q++) sr.f[lane * FP + q] = xf[q];
#pragma unroll
  for (int q = 0; q < LP; q++) sr.l[lane * LP + q] = xl[q];
  if (!__syncthreads_and(okA)) {
    if (fallback_warp) assoc_warp<FCH, LCH, GT>(B, K, gw, cta_smem);
    return;
  }
  int cnt = 0;
  const int ov = P->ov;
  const int tile0 = (gw - B.tile_off[p]) * 32;
  const int ld = P->ld;
  auto put = [&](int r, int slot, int j, float a) { put_kept(P, ld, cap, ov, (size_t)(tile0 + r), slot, j, a); };
  // cells farther than the largest radius from every query point are skipped
  const float slack = 1e-3f * G.h;
  const float prune_r2 = (brq + slack) * (brq + slack);
  const float4 *__restrict__ ycur = P->ycur;
  if (tid == 0) sm.cpre[0] = 0;
  long long ci0 = 0;
  int listed = 0, lcands = 0;
  while (true) {
    // list the near non-empty cells (thread per cell, ordered compaction)
    while (ci0 < ucells && listed + kCtaRows <= kCtaCells && lcands < kCtaFlushCands) {
      const long long ci = ci0 + tid;
      int2 se = make_int2(0, 0);
      if (ci < ucells) {
        const int cx = x0 + (int)(ci % nx), cy = y0 + (int)((ci / nx) % ny), cz = z0 + (int)(ci / ((long long)nx * ny));
        const float c0 = fmaf((float)cx, G.h, G.ox), c1 = fmaf((float)cy, G.h, G.oy), c2 = fmaf((float)cz, G.h, G.oz);
        const float dx = fmaxf(fmaxf(c0 - qlo[3], qlo[0] - (c0 + G.h)), 0.f);
        const float dy = fmaxf(fmaxf(c1 - qlo[4], qlo[1] - (c1 + G.h)), 0.f);
        const float dz = fmaxf(fmaxf(c2 - qlo[5], qlo[2] - (c2 + G.h)), 0.f);
        if (dx * dx + dy * dy + dz * dz <= prune_r2) se = grid_lookup(G, cx, cy, cz);
      }
      const int f = se.y > 0 ? 1 : 0;
      int ex, exc;
      const int tot = block_excl_scan(f, ex, sm.ired);
      const int totc = block_excl_scan(f ? se.y : 0, exc, sm.ired);
      if (f) {
        sm.cell[listed + ex] = se;
        sm.cpre[listed + ex + 1] = lcands + exc + se.y;
      }
      listed += tot;
      lcands += totc;
      ci0 += kCtaRows;
    }
    __syncthreads();
    // stream the listed members, kCtaCand per step
    for (int st0 = 0; st0 < lcands; st0 += kCtaCand) {
      const int gi = st0 + tid;
      const bool has = gi < lcands;
      int gp = 0;
      if (has) {
        int lo = 0, hi = listed - 1;
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (sm.cpre[mid] <= gi) lo = mid; else hi = mid - 1;
        }
        gp = sm.cell[lo].x + (gi - sm.cpre[lo]);
      }
      const float4 y = has ? __ldg(&ycur[gp]) : make_float4(0.f, 0.f, 0.f, 0.f);
      float4 yf[FP];
#pragma unroll
      for (int q = 0; q < FP; q++)
        yf[q] = (FCH > 0 && has) ? __ldg(reinterpret_cast<const float4 *>(G.feat) + (size_t)gp * FCH + q)
                                 : make_float4(0.f, 0.f, 0.f, 0.f);
      sm.pos[tid] = y;
#pragma unroll
      for (int q = 0; q < FP; q++) sm.feat[tid * FP + q] = yf[q];
      if (LCH > 0) {
#pragma unroll
        for (int q = 0; q < LP; q++)
          sm.lab[tid * LP + q] = has ? __ldg(reinterpret_cast<const float4 *>(G.lab) + (size_t)gp * LCH + q)
                                     : make_float4(0.f, 0.f, 0.f, 0.f);
      }
      if (GT) sm.geo[tid] = has ? __ldg(&G.geo[gp]) : make_float4(0.f, 0.f, 0.f, 0.f);
      {
        float bv[16];
        mma_cand_vec<FCH>(bv, has, y, yf, F, pcx, pcy, pcz);
        const bool okb = __all_sync(FULLMASK, mma_store_vec(bv, &sm.bpl[0][0], kCtaCand, tid));
        if (lane == 0) sm.okg[wib] = okb ? 1 : 0;
      }
      __syncthreads();
      const int nk = min(kCtaCand, lcands - st0);
      if (split < 0) {
#pragma unroll 1
        for (int g = 0; g < kCtaCand / 32; g++) {
          const int gk = nk - 32 * g;
          if (gk <= 0) break;
          uint32_t cand = sm.okg[g] ? mma_filter(&sm.apl[wib][0][0], 32, &sm.bpl[0][32 * g], kCtaCand, lane, K.mma_tau)
                                    : 0xFFFFFFFFu;
          cand &= gk >= 32 ? 0xFFFFFFFFu : ((1u << gk) - 1u);
          if (!valid) cand = 0u;
          eval_survivors<FCH, LCH, GT>(K, F, C, lane, cand, cnt, sr, sm.pos + 32 * g, sm.feat + 32 * g * FP,
                                       sm.lab + 32 * g * LP, sm.geo + (GT ? 32 * g : 0), put);
        }
      } else {
        const int g = wib, gk = nk - 32 * g;
        uint32_t cand = 0u;
        if (gk > 0) {
          cand = sm.okg[g] ? mma_filter(&sm.apl[wib][0][0], 32, &sm.bpl[0][32 * g], kCtaCand, lane, K.mma_tau)
                           : 0xFFFFFFFFu;
          cand &= gk >= 32 ? 0xFFFFFFFFu : ((1u << gk) - 1u);
          if (!valid) cand = 0u;
        }
        // pass 1: kept pairs per row in this group (nothing stored)
        int kept = 0;
        auto count_only = [](int, int, int, float) {};
        eval_survivors<FCH, LCH, GT>(K, F, C, lane, cand, kept, sr, sm.pos + 32 * g, sm.feat + 32 * g * FP,
                                     sm.lab + 32 * g * LP, sm.geo + (GT ? 32 * g : 0), count_only);
        sm.gcnt[g][lane] = kept;
        __syncthreads();
        int base = cnt, total = cnt;
#pragma unroll
        for (int q = 0; q < kCtaWarps; q++) {
          const int c = sm.gcnt[q][lane];
          if (q < g) base += c;
          total += c;
        }
        // pass 2: the same survivors, stored behind the lower groups' pairs
        eval_survivors<FCH, LCH, GT>(K, F, C, lane, cand, base, sr, sm.pos + 32 * g, sm.feat + 32 * g * FP,
                                     sm.lab + 32 * g * LP, sm.geo + (GT ? 32 * g : 0), put);
        cnt = total;
      }
      __syncthreads();
    }
    listed = 0;
    lcands = 0;
    if (ci0 >= ucells) break;
  }
  if (valid && fallback_warp) finish_row(B, P, p, s, cnt, cap, P->ov);
}

// Persistent blocks take work items from a counter, so blocks that finish early pick
// up the remaining ones.  An entry of the item order is (item << 3) | mode: mode 4 runs
// the item's four tiles (one per warp), modes 0-3 one tile of a split item.  Thread 0
// adds the SM clock cycles an entry took (>> 8) to its item's cost.
constexpr int kItemWhole = 4;

template <int FCH, int LCH, bool GT>
__global__ void __launch_bounds__(kCtaRows, 4) k_assoc_cta(BatchDev B, KParams K) {
  extern __shared__ __align__(128) unsigned char cta_smem[];
  __shared__ int item;
  const int entries = *B.n_order;
  int last = -1;
  long long t0 = 0;
  while (true) {
    __syncthreads();   // every thread has finished the previous item; shared memory is free
    if (threadIdx.x == 0) {
      if (last >= 0) atomicAdd(&B.item_cost[last], (int)min((clock64() - t0) >> 8, 0x3FFFFFFFLL));
      item = atomicAdd(B.assoc_next, 1);
    }
    __syncthreads();
    const int it = item;
    if (it >= entries) break;
    const int code = B.item_order[it];
    const int wi = code >> 3, mode = code & 7;
    if (threadIdx.x == 0) {
      last = wi;
      t0 = clock64();
    }
    assoc_block<FCH, LCH, GT>(B, K, wi * kCtaWarps, mode == kItemWhole ? -1 : mode, cta_smem);
  }
}

__device__ __forceinline__ int cost_bucket(long long c) { return c > 0 ? min(63 - __clzll(c), 32) + 1 : 0; }

// Orders the work items for the next pass (one block) from the cost each took in this
// one, and resets the costs.  An item that cost more than one block's fair share of
// the pass (total / blocks) cannot finish with the rest of the pass; it is split into
// its four tiles, each run by a whole block (estimated 3/8 of the item's cost each:
// a quarter of the work plus the counting pass).  Entries are placed in descending
// buckets of log2 cost; the order inside a bucket is arbitrary and, like the split,
// changes no result.
__global__ void __launch_bounds__(1024) k_order_items(int n, int blocks, int *cost, int *order, int *n_order) {
  __shared__ int hist[34], off[34];
  __shared__ long long wsum[32];
  long long t = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) t += cost[i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(FULLMASK, t, o);
  if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = t;
  for (int b = threadIdx.x; b < 34; b += blockDim.x) hist[b] = 0;
  __syncthreads();
  long long total = 0;
  for (int w = 0; w < (int)(blockDim.x >> 5); w++) total += wsum[w];
  const long long share = blocks > 0 ? total / blocks : 0;
  auto is_split = [&](long long c) { return share > 0 && c > share; };
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const long long c = cost[i];
    if (is_split(c)) atomicAdd(&hist[cost_bucket(c * 3 / 8)], kCtaWarps);
    else atomicAdd(&hist[cost_bucket(c)], 1);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int run = 0;
    for (int b = 33; b >= 0; b--) {
      off[b] = run;
      run += hist[b];
    }
    *n_order = run;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const long long c = cost[i];
    if (is_split(c)) {
      const int at = atomicAdd(&off[cost_bucket(c * 3 / 8)], kCtaWarps);
      for (int q = 0; q < kCtaWarps; q++) order[at + q] = (i << 3) | q;
    } else {
      order[atomicAdd(&off[cost_bucket(c)], 1)] = (i << 3) | kItemWhole;
    }
    cost[i] = 0;
  }
}

}  // namespace cvo_gb
