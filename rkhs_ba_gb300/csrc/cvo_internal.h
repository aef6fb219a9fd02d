// cvo_internal.h -- internal types shared by the CUDA translation units.
//
// Data layout in HBM (replaces the reference's 176-240 B AoS CvoPoint records,
// include/UnifiedCvo/utils/PointSegmentedDistribution.hpp:51-144):
//   positions : float4 {x, y, z, w}   (w = ||p|| for sources, original index bits for targets)
//   features  : n * FP floats, FP = F rounded up to 4 (float4 loads)
//   labels    : n * CP floats, CP = C rounded up to 4
//   geom_type : float2
// A source cloud is additionally kept in "tile order" (Morton order, 32 points per
// warp tile); a target cloud keeps one spatial-hash grid per cell size ("level").
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <vector>
#include <map>
#include <new>
#include <nvtx3/nvToolsExt.h>
#include "../../include/cvo_gb300.h"

namespace cvo_gb {

constexpr int kWarp = 32;
constexpr int kMaxIndicatorWindow = 128;
constexpr int kMaxTargetBits = 22;          // targets per cloud <= 4M
constexpr unsigned long long kEmptyKey = 0xFFFFFFFFFFFFFFFFull;

// ------------------------------------------------------------------ grid
// One spatial-hash grid over a target cloud at cell size h.  Cells are keyed by
// integer coordinates relative to the cloud's bounding-box minimum; the table
// uses linear probing.  Points are stored sorted by (table slot, original index),
// so the members of one cell are contiguous and in ascending original index.
struct GridDesc {
  float h, inv_h;
  float ox, oy, oz;
  int dimx, dimy, dimz;         // number of cells per axis over the bounding box
  int tbits;                    // table size = 1 << tbits
  const unsigned long long *keys;
  const int *cstart;
  const int *ccount;
  const int *perm;              // sorted position -> original index
  const float4 *pos;            // sorted copy: x, y, z, original index (int bits)
  const float *feat;            // sorted copy, n * FP
  const float *lab;             // sorted copy, n * CP
  const float4 *geo;            // sorted copy {g0, g1, 0, 0} (may be null)
};

struct DevCloud {
  int n = 0, F = 0, C = 0, FP = 0, CP = 0;
  bool has_geo = false;
  float bbmin[3] = {0, 0, 0}, bbmax[3] = {0, 0, 0};
  float max_norm = 0.f;
  float tile_ext = 0.f;          // mean bounding-box diagonal of 128 consecutive tile-order points
  // original order
  float4 *pos = nullptr;
  float *feat = nullptr;
  float *lab = nullptr;
  float2 *geo = nullptr;
  // source tile order
  int *sperm = nullptr;
  float4 *spos = nullptr;
  float *sfeat = nullptr;
  float *slab = nullptr;
  float2 *sgeo = nullptr;
  // target grids keyed by quantised cell-size exponent
  std::map<int, GridDesc *> levels_dev;   // device copies of descriptors
  std::map<int, GridDesc> levels_host;
  std::vector<void *> level_allocs;
};

// ----------------------------------------------------------- kernel params
// Per-call kernel constants (identical for all pairs of a batch).
struct KParams {
  float sigma2, c2, c_sigma2, s_ell, s_sigma2, s_sigma_sq, sp_thres;
  float log_geo;         // logf(sp_thres / sigma2), evaluated on the host
  float d2_c_thres, d2_s_thres;
  float c, d;            // so(3) / R^3 inner-product scales
  float eps, eps_2, min_step, max_step;
  float ell_decay_rate, ell_min, indicator_stable_threshold;
  int ell_decay_start, indicator_window_size, max_iter, nn_max, use_range_ell_step;
  int use_geo, use_int, use_sem, use_gtype;
  float inv2c2;          // 1 / (2 c_ell^2), rounded once (IEEE division)
  // Tensor-core prefilter: a kept pair needs d2/(2l^2) + d2c/(2c_ell^2) < mma_tau
  // (mma_tau = ln(sigma^2 c_sigma^2 s_sigma^2 / sp_thres) + slack), see k_assoc.
  float mma_tau;
  int use_mma;
  // Value scale (1 on the two-view path; c_sigma for the adaptive path's geometric-only
  // values s^2 exp(-d2/2l^2) c_sigma) and the colour denominator 2 c_ell^2 of the exact
  // (double) value as each path rounds it.
  float val_scale;
  double two_c2;
};

// Per-pair device state.  One struct per pair, in device memory.
struct PairDev {
  // problem
  int n, m;                       // source rows, target points
  const float4 *xs;               // source, tile order (x,y,z,||x||)
  const float *xf, *xl;
  const float2 *xg;
  const int *sperm;
  const GridDesc *levels;         // device array of grid levels of the target
  int nlevels;
  float level_r[24];              // largest search radius each level serves
  float4 *ycur;                   // transformed targets, current level order
  float4 *yorig;                  // transformed targets, original order
  int *A_j; float *A_v;           // ELL, row-major: entry c of row s at [s * ld + c] (original target index)
  int ld;                         // ELL row pitch (capmax rounded up to a multiple of 4)
  int2 *ovf;                      // spill lists: kept pair cap + t of row s at [s * ov + t] = {j, bits of a}
  int ov;                         // row-list entries per row
  const float *tf, *tl;           // target features / labels, original order (float4 chunks)
  const float2 *tg;               // target geometric types, original order
  int *nnz_row;                   // n
  float *row_sums;                // n * 8: omega(3)/c, v(3)/d, asum, count
  double *part;                   // reduce partials
  unsigned int *counter;          // last-block counters [2]
  int F, C;                       // feature / label dimensions (source and target agree)
  int capmax;
  int mode;                       // 0 align, 1 inner product, 2 export
  // iteration state
  float R[9], T[3];               // internal pose
  float Ri[9], Ti[3];             // target transform R^T, -R^T T
  float ell;
  int cap;
  int level, level_used;
  int iter, done, ret;
  float xi[6];
  double grad[6];
  double asum;
  long long nnz_sum;
  int max_row;
  double bcde[4];
  double step, dist;
  float rq_max;                   // largest search radius of this iteration
  // indicator queues (ring buffers)
  float qs[kMaxIndicatorWindow], qe[kMaxIndicatorWindow];
  int qs_head, qs_len, qe_head, qe_len;
  float ssum, esum;
};


// Batch of pairs processed together by every kernel launch.
struct BatchDev {
  int npairs;
  int total_warps;                // association tiles over all pairs
  int total_rows;                 // sum of n
  int total_targets;              // sum of m
  PairDev *pairs;                 // device array
  const int *tile_off;            // npairs + 1 (prefix of tile counts)
  const int *row_off;             // npairs + 1 (prefix of n)
  const int *tgt_off;             // npairs + 1 (prefix of m)
  int *err;                       // error word (0 ok)
  const int *rblk_off;            // reduce blocks per pair (prefix)
  const int *sblk_off;            // step blocks per pair (prefix)
  int total_rblocks, total_sblocks;
  int *active;                    // number of pairs not done
  int *active_iters;              // iterations that started with an active pair
  double *assoc_bytes;            // algorithmic bytes of the association passes
  int record_bytes;               // packed bytes of one target record
  // rows with more than `cap` kept pairs, {pair, row, kept count, 0}; reset by k_transform
  int4 *sel_list;                 // cap < count <= ov: select from the row list
  int *sel_count;
  int4 *scan_list;                // count > ov: index-ordered rescan of the row
  int *scan_count;
  int *assoc_next;                // next association work item (persistent blocks); reset by k_transform
  // work items (four tiles of one pair) in the order the persistent blocks take them:
  // heaviest first by the cost each took in the previous pass (SM clock / 256); an
  // entry is (item << 3) | mode, mode 4 = whole item, 0-3 = one tile of a split item
  int n_items;
  int *item_order;                // up to 4 n_items entries
  int *item_cost;
  int *n_order;                   // entries of item_order
};

// ------------------------------------------------------------- host side
struct Workspace;

struct Profile {
  bool on = false;
  double assoc_ms = 0.0;
  double kernel_ms[5] = {0, 0, 0, 0, 0};   // transform, assoc, reduce, step, all four
  double assoc_split_ms[3] = {0, 0, 0};    // association kernel, selection, row sums
  long long assoc_launches = 0;
  double assoc_bytes = 0.0;
  long long iterations = 0;
};

// Association tuning: grid cell size h = max(r / cell_div_r, (ext + 2 r) / cell_div_ext)
// for search radius r and source tiles of diagonal ext, and the resident association
// blocks per SM of the persistent launch (0: as many as the occupancy allows).  Results
// do not depend on either (the kept pairs are defined by index order), only the work per
// row and how the work items spread over the SMs do.
struct TuneConfig {
  float cell_div_r = 4.f;
  float cell_div_ext = 8.f;
  int blocks_per_sm = 0;
};

struct Handle {
  cvo_params params;
  cudaStream_t stream = nullptr;
  cudaStream_t own_stream = nullptr;
  Profile prof;
  int device = 0;
  int num_sms = 0;
  long long launches = 0;
  std::string last_error;
  Workspace *ws = nullptr;
  std::map<long long, TuneConfig> tuned;    // (F, C, log2 rows) -> fastest cell size
  std::map<long long, int> tuned_bps;       // (F, C, log2 work items of a batch) -> blocks per SM
  const TuneConfig *tune_force = nullptr;   // set while the autotuner times a configuration
};

long long tune_key(int F, int C, long long rows);
// Association work items (128 source rows each) of a pair of `rows` source points.
long long tune_items(long long rows);
// Times one association pass of (src, tgt) at pose T and lengthscale ell for every
// candidate configuration and records the fastest for the batches that match its key.
int autotune_association(Handle *h, DevCloud *src, DevCloud *tgt, const float T[16], float ell, int reps,
                         std::vector<TuneConfig> *configs, std::vector<float> *ms, int *best);

// Label rows are padded to 5 float4 chunks (C <= 20) or 9 chunks (C <= 36).
inline int label_chunks(int C) { return C <= 0 ? 0 : (C <= 20 ? 5 : (C <= 36 ? 9 : (C + 3) / 4)); }

// RGB-D frame -> device cloud, device cloud -> host arrays (cvo_frontend.cu)
int cloud_from_rgbd(Handle *h, const uint8_t *image, int rows, int cols, int channels, const float *depth,
                    const float intrinsic[4], float scaling_factor, const int *uv, int n_sel, const float *geom_type,
                    int num_classes, const float *semantics, DevCloud **out);
int cloud_download(Handle *h, const DevCloud *d, float *xyz, float *features, float *labels, float *geom_type);

// grid / cloud management (cvo_grid.cu)
int cloud_upload(Handle *h, const cvo_cloud *c, DevCloud **out);
// A cloud from device arrays (xyz n x 3, features n x F, labels n x C, geometric
// types n float2 or null); the arrays stay owned by the caller.
int cloud_from_device(Handle *h, int n, int F, int C, const float *xyz_d, const float *feat_d, const float *lab_d,
                      const float2 *geo_d, DevCloud **out);
void cloud_free(DevCloud *c);
int cloud_level(Handle *h, DevCloud *c, int level_exp, GridDesc *host_desc);
float level_cell_size(int level_exp);
int level_for_radius(float r);

// radix sort / scan (cvo_sort.cu)
int radix_sort_pairs(Handle *h, unsigned int *keys, int *vals, unsigned int *keys_tmp, int *vals_tmp,
                     int n, int key_bits);
void exclusive_scan_int(Handle *h, const int *in, int *out, int n, int *scratch, int scratch_n);
size_t scan_scratch_ints(int n);

// engine (cvo_engine.cu)
KParams make_kparams(const cvo_params &p);
struct BatchResult {
  std::vector<float> T_out;     // 16 per pair, column-major [R^T, -R^T T]
  std::vector<int> ret, iters;
  std::vector<double> asum;
  std::vector<long long> nnz;
};
int run_align_batch(Handle *h, const std::vector<DevCloud *> &srcs, const std::vector<DevCloud *> &tgts,
                    const std::vector<float> &T_init, BatchResult *res, double *secs,
                    bool export_assoc, std::vector<std::vector<int>> *a_rows,
                    std::vector<std::vector<int>> *a_cols, std::vector<std::vector<float>> *a_vals);
int run_inner_product_batch(Handle *h, DevCloud *src, DevCloud *tgt, const std::vector<float> &T, float ell,
                            int cap, std::vector<double> *asum, std::vector<long long> *nnz,
                            bool export_assoc, std::vector<int> *a_rowptr_host, std::vector<int> *a_cols,
                            std::vector<float> *a_vals);

// Inner products of independent (source, target, pose) triples in one batch.
int run_inner_product_pairs(Handle *h, const std::vector<DevCloud *> &srcs, const std::vector<DevCloud *> &tgts,
                            const std::vector<float> &T, float ell, int cap, std::vector<double> *asum);

// One association pass per edge between world-frame clouds (multi-frame solver).
// src_world: per edge, the source frame's points already in world coordinates in
// tile order ({x, y, z, ||x||}); tgt_pose: per edge 12 floats, the target frame's
// pose (row-major 3x4, frame -> world) applied to the target points.  The result
// arrays stay valid until the next batch is built on the handle.
struct EdgeAssoc {
  const int *A_j;        // ELL, row-major over tile-ordered rows (pitch ld), original target indices
  const float *A_v;
  int ld;
  const int *nnz_row;
  int n, m;
  long long nnz;
  int max_row;
};
// Replayable launch sequence of an edge-association batch: the upload of the pair
// records, the association kernels, and the read-back of the records and of the error
// word, captured once as a CUDA graph and relaunched while the batch's launch
// parameters are byte-identical.  The pair records travel through pinned staging
// buffers, whose addresses the graph's copy nodes hold.  One object serves the
// successive batches of one caller (the outer iterations of a window solve).
struct AssocGraph {
  cudaGraphExec_t exec = nullptr;
  std::vector<unsigned char> key;
  long long launches = 0;       // kernel launches of one replay
  PairDev *pin_in = nullptr, *pin_out = nullptr;
  int *pin_err = nullptr;
  int pin_pairs = 0;
  int captures = 0, replays = 0;
  AssocGraph() = default;
  AssocGraph(const AssocGraph &) = delete;
  AssocGraph &operator=(const AssocGraph &) = delete;
  ~AssocGraph();
};
int run_association_edges(Handle *h, const std::vector<DevCloud *> &srcs, const std::vector<DevCloud *> &tgts,
                          const std::vector<const float4 *> &src_world, const std::vector<float> &src_world_norm,
                          const std::vector<float> &tgt_pose, const std::vector<float> &ells,
                          const std::vector<int> &caps, int capmax, std::vector<EdgeAssoc> *out,
                          const KParams *kparams = nullptr, AssocGraph *graph = nullptr);

// Non-isotropic association (cvo_aniso.cu): CSR of the kernel matrix with a 3x3
// geometric kernel (column-major), first `cap` pairs per row in index order.
void kernel_inverse3(const float K[9], float Ki[9]);
int run_association_aniso(Handle *h, DevCloud *src, DevCloud *tgt, const float T[16], const float kernel[9],
                          int cap, std::vector<int> *rowptr, std::vector<int> *col, std::vector<float> *val);

// Adaptive-lengthscale CVO (cvo_adaptive.cu).  trace (optional): per iteration
// {ell, dl, step, nnz A, nnz Axx, nnz Ayy}.
int run_association_adaptive(Handle *h, DevCloud *src, DevCloud *tgt, const float T[16], float ell,
                             std::vector<int> *rowptr, std::vector<int> *col, std::vector<float> *val);
int run_align_adaptive(Handle *h, DevCloud *src, DevCloud *tgt, const float T_init[16], float T_out[16],
                       double *secs, int *iters_out, double *trace, int trace_len);

// IRLS (cvo_irls.cu)
int run_align_multi(Handle *h, int n_frames, DevCloud *const *clouds, double *poses, const uint8_t *hold_const,
                    int n_edges, const int *edges, double *secs, int *iters);

// Learned pose proposal (cvo_learn.cu)
struct NetDev;
size_t net_num_params();
int net_create(Handle *h, int P, unsigned seed, NetDev **out);
void net_destroy(NetDev *n);
int net_points(const NetDev *n);
int net_forward_pool(Handle *h, NetDev *n, int n_scenes, int n_pts, const float *src, const float *tgt, int Bn,
                     const int *scene, const float *T_tgt, uint32_t seed, float *raw_out, float *T_out);
int net_hypotheses(Handle *h, NetDev *n, int Bn, DevCloud *const *src, DevCloud *const *tgt, uint32_t seed,
                   float *T_out);
int net_train_pool(Handle *h, NetDev *n, int n_scenes, int n_pts, const float *src, const float *tgt, int Bn,
                   const int *scene, const float *T_label, float lr, uint32_t seed, float *loss_out);
int net_get(Handle *h, NetDev *n, int which, float *out);
int net_set(Handle *h, NetDev *n, const float *in);
int net_set_gemm(NetDev *n, int kind);

// error helpers
int set_cuda_error(Handle *h, cudaError_t e, const char *where);
#define CVO_CUDA_TRY(h, call)                                      \
  do {                                                             \
    cudaError_t e__ = (call);                                      \
    if (e__ != cudaSuccess) return set_cuda_error((h), e__, #call); \
  } while (0)

// NVTX range over a host phase (no-op unless a profiler is attached): ncu can select
// launches by phase with --nvtx --nvtx-include "<name>/".
struct NvtxRange {
  explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange &) = delete;
  NvtxRange &operator=(const NvtxRange &) = delete;
};

// Status of the exception being handled: the C entry points catch everything, so no
// C++ exception crosses the C ABI (host allocation failure -> out of memory).
inline int status_from_exception() {
  try {
    throw;
  } catch (const std::bad_alloc &) {
    return CVO_ERR_OUT_OF_MEMORY;
  } catch (...) {
    return CVO_ERR_INVALID_ARG;
  }
}

}  // namespace cvo_gb
