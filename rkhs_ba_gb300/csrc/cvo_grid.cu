// cvo_grid.cu -- device clouds: packed SoA upload, source tile (Morton) order,
// and spatial-hash grid levels over target clouds.
//
// Replaces CvoPointCloud_to_gpu (src/cvo/CvoGPU_impl.cu:220-289) and the kd-tree
// association structure (thirdparty/cugicp/cukdtree/cukdtree.cuh:236-509): a
// radius query becomes a scan of the hash cells that overlap the query box.
#include <cmath>
#include <cstring>
#include <algorithm>
#include "cvo_internal.h"
#include "cvo_device.cuh"

namespace cvo_gb {

float level_cell_size(int e) { return exp2f(0.5f * (float)e); }

// Smallest quantised cell size h = 2^(e/2) with h >= r.
int level_for_radius(float r) {
  if (!(r > 0.f)) return -60;
  if (!std::isfinite(r)) return 1000;
  int e = (int)std::ceil(2.0 * std::log2((double)r));
  while (level_cell_size(e) < r) e++;
  while (e > -60 && level_cell_size(e - 1) >= r) e--;
  return e;
}

namespace {

__global__ void k_pack_positions(const float *xyz, int stride, int n, float4 *pos) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float x = xyz[(size_t)i * stride], y = xyz[(size_t)i * stride + 1], z = xyz[(size_t)i * stride + 2];
  pos[i] = make_float4(x, y, z, range_norm(x, y, z));
}

__global__ void k_pad_rows(const float *in, int n, int F, int FP, float *out) {
  size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (size_t)n * FP) return;
  int i = (int)(t / FP), k = (int)(t % FP);
  out[t] = (k < F) ? in[(size_t)i * F + k] : 0.f;
}

__device__ __forceinline__ unsigned int spread10(unsigned int v) {
  v &= 0x3FFu;
  v = (v | (v << 16)) & 0x030000FFu;
  v = (v | (v << 8)) & 0x0300F00Fu;
  v = (v | (v << 4)) & 0x030C30C3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}

__global__ void k_morton(const float4 *pos, int n, float ox, float oy, float oz, float inv, unsigned int *keys,
                         int *vals) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float4 p = pos[i];
  auto q = [&](float v, float o) {
    float c = (v - o) * inv;
    c = fminf(fmaxf(c, 0.f), 1023.f);
    return (unsigned int)c;
  };
  keys[i] = spread10(q(p.x, ox)) | (spread10(q(p.y, oy)) << 1) | (spread10(q(p.z, oz)) << 2);
  vals[i] = i;
}

// Bounding-box diagonal of each block of 128 consecutive tile-order points (one
// thread per block of points).
__global__ void k_tile_extent(const float4 *spos, int n, float *ext) {
  const int tile = blockIdx.x * blockDim.x + threadIdx.x;
  const int tiles = (n + 127) / 128;
  if (tile >= tiles) return;
  float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int s = tile * 128; s < min(n, tile * 128 + 128); s++) {
    const float4 p = spos[s];
    lo[0] = fminf(lo[0], p.x); lo[1] = fminf(lo[1], p.y); lo[2] = fminf(lo[2], p.z);
    hi[0] = fmaxf(hi[0], p.x); hi[1] = fmaxf(hi[1], p.y); hi[2] = fmaxf(hi[2], p.z);
  }
  const float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
  ext[tile] = sqrtf(dx * dx + dy * dy + dz * dz);
}

__global__ void k_gather_source(const int *perm, int n, const float4 *pos, const float *feat, int FP, const float *lab,
                                int CP, const float2 *geo, float4 *spos, float *sfeat, float *slab, float2 *sgeo) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  int i = perm[s];
  spos[s] = pos[i];
  for (int k = 0; k < FP; k++) sfeat[(size_t)s * FP + k] = feat[(size_t)i * FP + k];
  for (int k = 0; k < CP; k++) slab[(size_t)s * CP + k] = lab[(size_t)i * CP + k];
  if (geo) sgeo[s] = geo[i];
}

__global__ void k_hash_insert(const float4 *pos, int n, float ox, float oy, float oz, float inv_h, int dimx, int dimy,
                              int dimz, unsigned long long *keys, int *ccount, int tbits, unsigned int *slot_of,
                              int *vals, int *err) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  float4 p = pos[j];
  int cx = min(max((int)floorf((p.x - ox) * inv_h), 0), dimx - 1);
  int cy = min(max((int)floorf((p.y - oy) * inv_h), 0), dimy - 1);
  int cz = min(max((int)floorf((p.z - oz) * inv_h), 0), dimz - 1);
  unsigned long long key = cell_key(cx, cy, cz);
  unsigned int mask = (1u << tbits) - 1u;
  unsigned int slot = (unsigned int)cell_hash(key) & mask;
  for (unsigned int probe = 0; probe <= mask; probe++) {
    unsigned long long prev = atomicCAS(&keys[slot], kEmptyKey, key);
    if (prev == kEmptyKey || prev == key) {
      atomicAdd(&ccount[slot], 1);
      slot_of[j] = slot;
      vals[j] = j;
      return;
    }
    slot = (slot + 1u) & mask;
  }
  atomicExch(err, 1);   // table full: cannot happen with load factor <= 1/2
  slot_of[j] = 0;
  vals[j] = j;
}

__global__ void k_gather_target(const int *perm, int n, const float4 *pos, const float *feat, int FP, const float *lab,
                                int CP, const float2 *geo, float4 *tpos, float *tfeat, float *tlab, float4 *tgeo) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  int j = perm[t];
  float4 p = pos[j];
  tpos[t] = make_float4(p.x, p.y, p.z, __int_as_float(j));
  for (int k = 0; k < FP; k++) tfeat[(size_t)t * FP + k] = feat[(size_t)j * FP + k];
  for (int k = 0; k < CP; k++) tlab[(size_t)t * CP + k] = lab[(size_t)j * CP + k];
  if (geo) { float2 g = geo[j]; tgeo[t] = make_float4(g.x, g.y, 0.f, 0.f); }
}

template <typename T>
int dalloc(Handle *h, T **p, size_t count) {
  if (count == 0) count = 1;
  cudaError_t e = cudaMalloc((void **)p, sizeof(T) * count);
  if (e != cudaSuccess) {
    set_cuda_error(h, e, "cudaMalloc");
    return e == cudaErrorMemoryAllocation ? CVO_ERR_OUT_OF_MEMORY : CVO_ERR_CUDA;
  }
  return 0;
}

}  // namespace

// Device part of a cloud's construction from staged device arrays (xyz with stride
// 3 or 4, features n x F, labels n x C, geometric types n float2 or null) and its
// bounding box: packed original-order records, Morton tile order, tile extents.
static int cloud_build(Handle *h, DevCloud *d, const float *xyz_d, int stride, const float *feat_in,
                       const float *lab_in, const float2 *geo_in, const float mn[3], const float mx[3]) {
  const int n = d->n;
  int rc = 0;
  int *perm_vals = nullptr, *perm_tmp = nullptr;
  unsigned int *keys = nullptr, *keys_tmp = nullptr;
  if ((rc = dalloc(h, &d->pos, n)) || (rc = dalloc(h, &d->feat, (size_t)n * d->FP)) ||
      (rc = dalloc(h, &d->lab, (size_t)n * d->CP)) || (rc = dalloc(h, &d->sperm, n)) ||
      (rc = dalloc(h, &d->spos, n)) || (rc = dalloc(h, &d->sfeat, (size_t)n * d->FP)) ||
      (rc = dalloc(h, &d->slab, (size_t)n * d->CP)))
    return rc;
  if (d->has_geo) {
    if ((rc = dalloc(h, &d->geo, n)) || (rc = dalloc(h, &d->sgeo, n))) return rc;
  }
  k_pack_positions<<<(n + 255) / 256, 256, 0, h->stream>>>(xyz_d, stride, n, d->pos);
  h->launches++;
  if (d->FP > 0) {
    size_t tot = (size_t)n * d->FP;
    k_pad_rows<<<(unsigned)((tot + 255) / 256), 256, 0, h->stream>>>(feat_in, n, d->F, d->FP, d->feat);
    h->launches++;
  }
  if (d->CP > 0) {
    size_t tot = (size_t)n * d->CP;
    k_pad_rows<<<(unsigned)((tot + 255) / 256), 256, 0, h->stream>>>(lab_in, n, d->C, d->CP, d->lab);
    h->launches++;
  }
  if (d->has_geo)
    CVO_CUDA_TRY(h, cudaMemcpyAsync(d->geo, geo_in, sizeof(float2) * n, cudaMemcpyDeviceToDevice, h->stream));

  // source tile order: Morton order of a 1024^3 lattice over the bounding box
  if ((rc = dalloc(h, &keys, n)) || (rc = dalloc(h, &keys_tmp, n)) || (rc = dalloc(h, &perm_vals, n)) ||
      (rc = dalloc(h, &perm_tmp, n)))
    return rc;
  float ext = std::max(std::max(mx[0] - mn[0], mx[1] - mn[1]), mx[2] - mn[2]);
  float inv = ext > 0 ? 1023.999f / ext : 0.f;
  k_morton<<<(n + 255) / 256, 256, 0, h->stream>>>(d->pos, n, mn[0], mn[1], mn[2], inv, keys, perm_vals);
  h->launches++;
  if ((rc = radix_sort_pairs(h, keys, perm_vals, keys_tmp, perm_tmp, n, 30))) return rc;
  CVO_CUDA_TRY(h, cudaMemcpyAsync(d->sperm, perm_vals, sizeof(int) * n, cudaMemcpyDeviceToDevice, h->stream));
  k_gather_source<<<(n + 255) / 256, 256, 0, h->stream>>>(d->sperm, n, d->pos, d->feat, d->FP, d->lab, d->CP, d->geo,
                                                         d->spos, d->sfeat, d->slab, d->sgeo);
  h->launches++;
  // mean bounding-box diagonal of the 128-point source blocks (sizes the grid cells)
  const int tiles = (n + 127) / 128;
  float *ext_d = reinterpret_cast<float *>(keys);
  k_tile_extent<<<(tiles + 127) / 128, 128, 0, h->stream>>>(d->spos, n, ext_d);
  h->launches++;
  std::vector<float> ext_h(tiles);
  CVO_CUDA_TRY(h, cudaMemcpyAsync(ext_h.data(), ext_d, sizeof(float) * tiles, cudaMemcpyDeviceToHost, h->stream));
  CVO_CUDA_TRY(h, cudaStreamSynchronize(h->stream));
  double es = 0.0;
  for (float e : ext_h) es += e;
  d->tile_ext = tiles > 0 ? (float)(es / tiles) : 0.f;
  cudaFree(keys); cudaFree(keys_tmp); cudaFree(perm_vals); cudaFree(perm_tmp);
  return 0;
}

static DevCloud *new_cloud(int n, int F, int C, bool has_geo) {
  DevCloud *d = new DevCloud();
  d->n = n; d->F = F; d->C = C;
  d->FP = (F + 3) / 4 * 4;
  d->CP = 4 * label_chunks(C);
  d->has_geo = has_geo;
  return d;
}

static void set_extent(DevCloud *d, const float mn[3], const float mx[3], double maxn2) {
  for (int k = 0; k < 3; k++) { d->bbmin[k] = mn[k]; d->bbmax[k] = mx[k]; }
  d->max_norm = (float)std::sqrt(maxn2) * (1.f + 1e-6f);
}

int cloud_upload(Handle *h, const cvo_cloud *c, DevCloud **out) {
  NvtxRange nvtx_range("cloud_upload");
  if (!c || !out) return CVO_ERR_INVALID_ARG;
  if (c->n < 0 || c->F < 0 || c->C < 0) return CVO_ERR_INVALID_ARG;
  if (c->n > 0 && (!c->xyz || (c->xyz_stride != 3 && c->xyz_stride != 4))) return CVO_ERR_INVALID_ARG;
  if (c->F > 0 && c->n > 0 && !c->features) return CVO_ERR_INVALID_ARG;
  if (c->C > 0 && c->n > 0 && !c->labels) return CVO_ERR_INVALID_ARG;
  if (c->n > (1 << kMaxTargetBits)) return CVO_ERR_CAPACITY;
  int n = c->n;
  // bounding box and largest range on the host (input is host memory)
  float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
  double maxn2 = 0;
  for (int i = 0; i < n; i++) {
    const float *p = c->xyz + (size_t)i * c->xyz_stride;
    for (int k = 0; k < 3; k++) {
      if (!std::isfinite(p[k])) return CVO_ERR_INVALID_ARG;
      mn[k] = std::min(mn[k], p[k]);
      mx[k] = std::max(mx[k], p[k]);
    }
    double n2 = (double)p[0] * p[0] + (double)p[1] * p[1] + (double)p[2] * p[2];
    maxn2 = std::max(maxn2, n2);
  }
  if (n == 0) { for (int k = 0; k < 3; k++) mn[k] = mx[k] = 0.f; }
  DevCloud *d = new_cloud(n, c->F, c->C, c->geom_type != nullptr);
  set_extent(d, mn, mx, maxn2);
  *out = d;
  if (n == 0) return 0;

  float *xyz_d = nullptr, *feat_in = nullptr, *lab_in = nullptr;
  float2 *geo_in = nullptr;
  int rc = 0;
  auto release = [&]() { cudaFree(xyz_d); cudaFree(feat_in); cudaFree(lab_in); cudaFree(geo_in); };
  if ((rc = dalloc(h, &xyz_d, (size_t)n * c->xyz_stride))) { release(); return rc; }
  CVO_CUDA_TRY(h, cudaMemcpyAsync(xyz_d, c->xyz, sizeof(float) * (size_t)n * c->xyz_stride, cudaMemcpyHostToDevice,
                                  h->stream));
  if (d->FP > 0) {
    if ((rc = dalloc(h, &feat_in, (size_t)n * c->F))) { release(); return rc; }
    CVO_CUDA_TRY(h, cudaMemcpyAsync(feat_in, c->features, sizeof(float) * (size_t)n * c->F, cudaMemcpyHostToDevice,
                                    h->stream));
  }
  if (d->CP > 0) {
    if ((rc = dalloc(h, &lab_in, (size_t)n * c->C))) { release(); return rc; }
    CVO_CUDA_TRY(h, cudaMemcpyAsync(lab_in, c->labels, sizeof(float) * (size_t)n * c->C, cudaMemcpyHostToDevice,
                                    h->stream));
  }
  if (d->has_geo) {
    if ((rc = dalloc(h, &geo_in, n))) { release(); return rc; }
    CVO_CUDA_TRY(h, cudaMemcpyAsync(geo_in, c->geom_type, sizeof(float2) * n, cudaMemcpyHostToDevice, h->stream));
  }
  rc = cloud_build(h, d, xyz_d, c->xyz_stride, feat_in, lab_in, geo_in, mn, mx);
  release();
  return rc;
}

// Bounding box (min, max per axis) and largest squared norm of n device points
// (xyz stride 3), one block.
__global__ void k_extent(const float *xyz, int n, float *box, double *maxn2) {
  __shared__ float sl[3][256], sh[3][256];
  __shared__ double sn[256];
  float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  double m2 = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const float *p = xyz + 3 * (size_t)i;
    for (int k = 0; k < 3; k++) { lo[k] = fminf(lo[k], p[k]); hi[k] = fmaxf(hi[k], p[k]); }
    m2 = fmax(m2, (double)p[0] * p[0] + (double)p[1] * p[1] + (double)p[2] * p[2]);
  }
  for (int k = 0; k < 3; k++) { sl[k][threadIdx.x] = lo[k]; sh[k][threadIdx.x] = hi[k]; }
  sn[threadIdx.x] = m2;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int t = 1; t < blockDim.x; t++) {
      for (int k = 0; k < 3; k++) { lo[k] = fminf(lo[k], sl[k][t]); hi[k] = fmaxf(hi[k], sh[k][t]); }
      m2 = fmax(m2, sn[t]);
    }
    for (int k = 0; k < 3; k++) { box[k] = lo[k]; box[3 + k] = hi[k]; }
    *maxn2 = m2;
  }
}

int cloud_from_device(Handle *h, int n, int F, int C, const float *xyz_d, const float *feat_d, const float *lab_d,
                      const float2 *geo_d, DevCloud **out) {
  if (n < 0 || F < 0 || C < 0 || !out) return CVO_ERR_INVALID_ARG;
  if (n > (1 << kMaxTargetBits)) return CVO_ERR_CAPACITY;
  float mn[3] = {0.f, 0.f, 0.f}, mx[3] = {0.f, 0.f, 0.f};
  double maxn2 = 0.0;
  if (n > 0) {
    float *box = nullptr;
    double *m2 = nullptr;
    int rc = 0;
    if ((rc = dalloc(h, &box, 6)) || (rc = dalloc(h, &m2, 1))) { cudaFree(box); return rc; }
    k_extent<<<1, 256, 0, h->stream>>>(xyz_d, n, box, m2);
    h->launches++;
    float bh[6];
    cudaError_t e = cudaMemcpyAsync(bh, box, sizeof(bh), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&maxn2, m2, sizeof(double), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    cudaFree(box);
    cudaFree(m2);
    if (e != cudaSuccess) return set_cuda_error(h, e, "cloud extent");
    for (int k = 0; k < 3; k++) { mn[k] = bh[k]; mx[k] = bh[3 + k]; }
  }
  DevCloud *d = new_cloud(n, F, C, geo_d != nullptr);
  set_extent(d, mn, mx, maxn2);
  *out = d;
  if (n == 0) return 0;
  return cloud_build(h, d, xyz_d, 3, feat_d, lab_d, geo_d, mn, mx);
}

void cloud_free(DevCloud *d) {
  if (!d) return;
  cudaFree(d->pos); cudaFree(d->feat); cudaFree(d->lab); cudaFree(d->geo);
  cudaFree(d->sperm); cudaFree(d->spos); cudaFree(d->sfeat); cudaFree(d->slab); cudaFree(d->sgeo);
  for (void *p : d->level_allocs) cudaFree(p);
  for (auto &kv : d->levels_dev) cudaFree(kv.second);
  delete d;
}

// Builds (or returns the cached) grid level with cell size 2^(e/2) over the
// target cloud.  e >= 1000 selects a single cell holding every point (used
// when the geometric kernel is disabled and every target is a candidate).
int cloud_level(Handle *h, DevCloud *d, int e, GridDesc *host_desc) {
  auto it = d->levels_host.find(e);
  if (it != d->levels_host.end()) { *host_desc = it->second; return 0; }
  int n = d->n;
  GridDesc g;
  memset(&g, 0, sizeof(g));
  float ext[3];
  for (int k = 0; k < 3; k++) ext[k] = d->bbmax[k] - d->bbmin[k];
  float hsz = (e >= 1000) ? INFINITY : level_cell_size(e);
  // keep at most 2^20 cells per axis
  float emax = std::max(std::max(ext[0], ext[1]), ext[2]);
  if (std::isfinite(hsz) && emax / hsz > 1048000.f) hsz = emax / 1048000.f;
  g.h = hsz;
  g.inv_h = std::isfinite(hsz) ? 1.f / hsz : 0.f;
  g.ox = d->bbmin[0]; g.oy = d->bbmin[1]; g.oz = d->bbmin[2];
  g.dimx = std::isfinite(hsz) ? (int)std::floor(ext[0] * g.inv_h) + 1 : 1;
  g.dimy = std::isfinite(hsz) ? (int)std::floor(ext[1] * g.inv_h) + 1 : 1;
  g.dimz = std::isfinite(hsz) ? (int)std::floor(ext[2] * g.inv_h) + 1 : 1;
  int tbits = 10;
  while ((1 << tbits) < 2 * std::max(n, 1)) tbits++;
  g.tbits = tbits;
  size_t T = (size_t)1 << tbits;
  unsigned long long *keys = nullptr;
  int *cstart = nullptr, *ccount = nullptr, *perm = nullptr, *vals_tmp = nullptr, *err = nullptr;
  unsigned int *slot_of = nullptr, *slot_tmp = nullptr;
  float4 *tpos = nullptr;
  float *tfeat = nullptr, *tlab = nullptr;
  float4 *tgeo = nullptr;   // 16-byte records so that bulk copies stay aligned
  int rc = 0;
  if ((rc = dalloc(h, &keys, T)) || (rc = dalloc(h, &cstart, T)) || (rc = dalloc(h, &ccount, T)) ||
      (rc = dalloc(h, &perm, n)) || (rc = dalloc(h, &tpos, n)) || (rc = dalloc(h, &tfeat, (size_t)n * d->FP)) ||
      (rc = dalloc(h, &tlab, (size_t)n * d->CP)) || (rc = dalloc(h, &slot_of, n)) || (rc = dalloc(h, &slot_tmp, n)) ||
      (rc = dalloc(h, &vals_tmp, n)) || (rc = dalloc(h, &err, 1)))
    return rc;
  if (d->has_geo && (rc = dalloc(h, &tgeo, n))) return rc;
  size_t scr = scan_scratch_ints((int)T);
  int *scan_scr = nullptr;
  if ((rc = dalloc(h, &scan_scr, scr))) return rc;
  CVO_CUDA_TRY(h, cudaMemsetAsync(keys, 0xFF, sizeof(unsigned long long) * T, h->stream));
  CVO_CUDA_TRY(h, cudaMemsetAsync(ccount, 0, sizeof(int) * T, h->stream));
  CVO_CUDA_TRY(h, cudaMemsetAsync(err, 0, sizeof(int), h->stream));
  if (n > 0) {
    k_hash_insert<<<(n + 255) / 256, 256, 0, h->stream>>>(d->pos, n, g.ox, g.oy, g.oz, g.inv_h, g.dimx, g.dimy, g.dimz,
                                                          keys, ccount, tbits, slot_of, perm, err);
    h->launches++;
    if ((rc = radix_sort_pairs(h, slot_of, perm, slot_tmp, vals_tmp, n, tbits))) return rc;
  }
  exclusive_scan_int(h, ccount, cstart, (int)T, scan_scr, (int)scr);
  if (n > 0) {
    k_gather_target<<<(n + 255) / 256, 256, 0, h->stream>>>(perm, n, d->pos, d->feat, d->FP, d->lab, d->CP, d->geo,
                                                           tpos, tfeat, tlab, tgeo);
    h->launches++;
  }
  int herr = 0;
  CVO_CUDA_TRY(h, cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  CVO_CUDA_TRY(h, cudaStreamSynchronize(h->stream));
  cudaFree(slot_of); cudaFree(slot_tmp); cudaFree(vals_tmp); cudaFree(err); cudaFree(scan_scr);
  if (herr) return CVO_ERR_CAPACITY;
  g.keys = keys; g.cstart = cstart; g.ccount = ccount; g.perm = perm;
  g.pos = tpos; g.feat = tfeat; g.lab = tlab; g.geo = tgeo;
  for (void *p : {(void *)keys, (void *)cstart, (void *)ccount, (void *)perm, (void *)tpos, (void *)tfeat,
                  (void *)tlab, (void *)tgeo})
    if (p) d->level_allocs.push_back(p);
  d->levels_host[e] = g;
  *host_desc = g;
  return 0;
}

}  // namespace cvo_gb
