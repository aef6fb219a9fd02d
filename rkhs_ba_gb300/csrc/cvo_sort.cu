// cvo_sort.cu -- stable LSD radix sort of (uint32 key, int value) pairs and an
// exclusive prefix scan.  Used to build the spatial-hash grids and the source
// tile order (the reference builds a kd-tree with per-node thrust::sort,
// thirdparty/cugicp/cukdtree/cukdtree.cuh:236-284; this replaces it).
#include "cvo_internal.h"

namespace cvo_gb {

namespace {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 8;
constexpr int kSortTile = kSortThreads * kSortItems;   // 2048 keys per block
constexpr int kRadixBits = 8;
constexpr int kRadix = 1 << kRadixBits;
constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

// Digit histogram of one tile; hist is digit-major: hist[d * nblocks + b].
__global__ void k_digit_hist(const unsigned int *keys, int n, int shift, int *hist, int nblocks) {
  __shared__ int h[kRadix];
  for (int d = threadIdx.x; d < kRadix; d += blockDim.x) h[d] = 0;
  __syncthreads();
  const int base = blockIdx.x * kSortTile;
  for (int r = 0; r < kSortItems; r++) {
    int i = base + r * kSortThreads + threadIdx.x;
    if (i < n) atomicAdd(&h[(keys[i] >> shift) & (kRadix - 1)], 1);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < kRadix; d += blockDim.x) hist[d * nblocks + blockIdx.x] = h[d];
}

// Stable scatter: items are ranked in (round, warp, lane) order, which is the
// original order within the tile.
__global__ void k_digit_scatter(const unsigned int *keys_in, const int *vals_in, unsigned int *keys_out,
                                int *vals_out, int n, int shift, const int *offsets, int nblocks) {
  __shared__ int warp_cnt[kSortThreads / 32][kRadix];
  __shared__ int running[kRadix];
  __shared__ int round_tot[kRadix];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int d = threadIdx.x; d < kRadix; d += blockDim.x) running[d] = offsets[d * nblocks + blockIdx.x];
  for (int t = threadIdx.x; t < (kSortThreads / 32) * kRadix; t += blockDim.x) (&warp_cnt[0][0])[t] = 0;
  __syncthreads();
  const int base = blockIdx.x * kSortTile;
  const unsigned lt_mask = (1u << lane) - 1u;
  for (int r = 0; r < kSortItems; r++) {
    int i = base + r * kSortThreads + threadIdx.x;
    bool valid = i < n;
    unsigned int key = valid ? keys_in[i] : 0u;
    int val = valid ? vals_in[i] : 0;
    int d = valid ? (int)((key >> shift) & (kRadix - 1)) : kRadix;   // kRadix = invalid sentinel
    unsigned peers = __match_any_sync(0xFFFFFFFFu, d);
    int rank = __popc(peers & lt_mask);
    int leader = __ffs(peers) - 1;
    if (valid && lane == leader) warp_cnt[warp][d] = __popc(peers);
    __syncthreads();
    for (int dd = threadIdx.x; dd < kRadix; dd += blockDim.x) {
      int run = 0;
      for (int w = 0; w < kSortThreads / 32; w++) {
        int c = warp_cnt[w][dd];
        warp_cnt[w][dd] = run;
        run += c;
      }
      round_tot[dd] = run;
    }
    __syncthreads();
    if (valid) {
      int pos = running[d] + warp_cnt[warp][d] + rank;
      keys_out[pos] = key;
      vals_out[pos] = val;
    }
    __syncthreads();
    for (int dd = threadIdx.x; dd < kRadix; dd += blockDim.x) {
      running[dd] += round_tot[dd];
      for (int w = 0; w < kSortThreads / 32; w++) warp_cnt[w][dd] = 0;
    }
    __syncthreads();
  }
}

// Block-local exclusive scan of kScanTile ints; writes the tile total.
__global__ void k_scan_tiles(const int *in, int *out, int n, int *tile_sums) {
  __shared__ int warp_tot[kScanThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
  int v[kScanItems];
  int tsum = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    int i = base + k;
    v[k] = (i < n) ? in[i] : 0;
    tsum += v[k];
  }
  int incl = tsum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) warp_tot[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    int wt = (lane < kScanThreads / 32) ? warp_tot[lane] : 0;
    int wi = wt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int t = __shfl_up_sync(0xFFFFFFFFu, wi, o);
      if (lane >= o) wi += t;
    }
    if (lane < kScanThreads / 32) warp_tot[lane] = wi - wt;
    if (lane == kScanThreads / 32 - 1 && tile_sums) tile_sums[blockIdx.x] = wi;
  }
  __syncthreads();
  int run = warp_tot[warp] + incl - tsum;
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    int i = base + k;
    if (i < n) out[i] = run;
    run += v[k];
  }
}

__global__ void k_scan_add(int *out, int n, const int *tile_off) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] += tile_off[i / kScanTile];
}

}  // namespace

size_t scan_scratch_ints(int n) {
  size_t total = 0;
  while (n > kScanTile) {
    int t = (n + kScanTile - 1) / kScanTile;
    total += 2 * (size_t)t;
    n = t;
  }
  return total + 16;
}

void exclusive_scan_int(Handle *h, const int *in, int *out, int n, int *scratch, int scratch_n) {
  if (n <= 0) return;
  int tiles = (n + kScanTile - 1) / kScanTile;
  if (tiles == 1) {
    k_scan_tiles<<<1, kScanThreads, 0, h->stream>>>(in, out, n, nullptr);
    h->launches++;
    return;
  }
  int *sums = scratch;
  int *sums_scan = scratch + tiles;
  k_scan_tiles<<<tiles, kScanThreads, 0, h->stream>>>(in, out, n, sums);
  exclusive_scan_int(h, sums, sums_scan, tiles, scratch + 2 * tiles, scratch_n - 2 * tiles);
  k_scan_add<<<(n + 255) / 256, 256, 0, h->stream>>>(out, n, sums_scan);
  h->launches += 2;
}

// Sorts (keys, vals) by the low key_bits bits of keys, stable.  Result ends in
// keys/vals (tmp buffers are scratch of the same size).
int radix_sort_pairs(Handle *h, unsigned int *keys, int *vals, unsigned int *keys_tmp, int *vals_tmp, int n,
                     int key_bits) {
  if (n <= 1) return 0;
  int nblocks = (n + kSortTile - 1) / kSortTile;
  int hist_n = nblocks * kRadix;
  int *hist = nullptr;
  size_t scr = scan_scratch_ints(hist_n);
  CVO_CUDA_TRY(h, cudaMallocAsync((void **)&hist, sizeof(int) * ((size_t)hist_n * 2 + scr), h->stream));
  int *offs = hist + hist_n;
  int *scratch = offs + hist_n;
  unsigned int *kin = keys, *kout = keys_tmp;
  int *vin = vals, *vout = vals_tmp;
  int passes = (key_bits + kRadixBits - 1) / kRadixBits;
  for (int pass = 0; pass < passes; pass++) {
    int shift = pass * kRadixBits;
    k_digit_hist<<<nblocks, kSortThreads, 0, h->stream>>>(kin, n, shift, hist, nblocks);
    exclusive_scan_int(h, hist, offs, hist_n, scratch, (int)scr);
    k_digit_scatter<<<nblocks, kSortThreads, 0, h->stream>>>(kin, vin, kout, vout, n, shift, offs, nblocks);
    h->launches += 2;
    unsigned int *tk = kin; kin = kout; kout = tk;
    int *tv = vin; vin = vout; vout = tv;
  }
  if (kin != keys) {
    CVO_CUDA_TRY(h, cudaMemcpyAsync(keys, kin, sizeof(unsigned int) * n, cudaMemcpyDeviceToDevice, h->stream));
    CVO_CUDA_TRY(h, cudaMemcpyAsync(vals, vin, sizeof(int) * n, cudaMemcpyDeviceToDevice, h->stream));
  }
  CVO_CUDA_TRY(h, cudaFreeAsync(hist, h->stream));
  return 0;
}

}  // namespace cvo_gb
