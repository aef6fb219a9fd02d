/*
 * cvo_gb300.h -- C ABI of the GB300-native CVO / RKHS-BA registration core.
 *
 * Drop-in boundary for the `cvo::CvoGPU` registration path of UMich-CURLY/RKHS_BA.
 * Every entry point takes plain pointers and sizes, returns an int status
 * (CVO_OK == 0) and never calls exit().  Each declaration cites the reference
 * member it replaces (paths relative to the reference project root).
 *
 * Conventions kept from the reference:
 *  - 4x4 matrices are COLUMN-MAJOR float[16] (Eigen default storage).
 *  - cvo_align(): the target cloud is moved by inverse(T_init); the returned
 *    T_out satisfies x_src ~= T_out * y_tgt   (src/cvo/CvoGPU.cu:98-116,1265-1467).
 *  - cvo_function_angle()/cvo_inner_product(): the target is moved by inverse(T)
 *    (src/cvo/CvoGPU.cpp:215-221, src/cvo/CvoGPU.cu:1685-1702).
 *  - multi-frame poses are double[12], ROW-major 3x4 [R|t], frame -> world
 *    (include/UnifiedCvo/cvo/CvoFrame.hpp:26).
 *  - association rows are source indices, columns are target indices.
 *
 * Threading: one handle owns one CUDA stream and private device workspaces.
 * Calls on one handle are blocking and must not be made concurrently.
 */
#ifndef CVO_GB300_H
#define CVO_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ status */
enum {
  CVO_OK = 0,
  CVO_ZERO_GRADIENT = -1,      /* align stopped on a zero gradient (CvoGPU.cu:1356-1360) */
  CVO_ERR_INVALID_ARG = -2,
  CVO_ERR_EMPTY_CLOUD = -3,    /* reference returns 0 / -1 / cos 0 on empty input (CvoGPU.cu:1492-1495,1526-1529,1573-1577) */
  CVO_ERR_BAD_YAML = -4,
  CVO_ERR_CUDA = -5,
  CVO_ERR_OUT_OF_MEMORY = -6,
  CVO_ERR_TIMEOUT = -7,        /* a bounded device wait gave up (the proposal GEMM's MMA completions); the association kernels wait on nothing */
  CVO_ERR_UNSUPPORTED = -8,
  CVO_ERR_IO = -9,
  CVO_ERR_CAPACITY = -10
};

/* -------------------------------------------------------------- parameters
 * Field-for-field mirror of cvo::CvoParams (include/UnifiedCvo/cvo/CvoParams.hpp:12-79).
 * cvo_params_default() reproduces the constructor defaults (:80-136); the
 * reference leaves max_step uninitialised, here it defaults to 0.8 (the value of
 * cvo_params/cvo_geometric_params_gpu.yaml).
 */
typedef struct cvo_params {
  float ell_init_first_frame;
  float ell_init;
  float ell_min;
  int   min_ell_iter_limit;
  float ell_max;
  double dl;
  double dl_step;
  float sigma;
  float sp_thres;
  float c;
  float d;
  float c_ell;
  float c_sigma;
  float s_ell;
  float s_sigma;
  int   MAX_ITER;
  float eps;
  float eps_2;
  float min_step;
  float max_step;
  float step;
  int   nearest_neighbors_max;
  float ell_decay_rate;
  float ell_decay_rate_first_frame;
  int   ell_decay_start;
  int   ell_decay_start_first_frame;
  int   indicator_window_size;
  float indicator_stable_threshold;
  int   is_pcl_visualization_on;
  int   is_using_least_square;
  int   is_ell_adaptive;
  int   is_full_ip_matrix;
  int   is_using_geometry;
  int   is_using_intensity;
  int   is_using_semantics;
  int   is_using_range_ell;
  int   is_using_kdtree;
  int   is_exporting_association;
  int   is_using_geometric_type;
  int   is_global_angle_registration;
  int   multiframe_using_cpu;
  int   multiframe_max_iters;
  float multiframe_ell_init;
  float multiframe_ell_min;
  float multiframe_ell_max;
  int   multiframe_iter_per_ell;
  float multiframe_ell_decay_rate;
  int   multiframe_iterations_per_ell;
  int   multiframe_iterations_per_solve;
  int   multiframe_expected_points;
  float multiframe_downsample_voxel_size;
  int   multiframe_num_neighbors;
  int   multiframe_least_squares_num_threads;
  int   multiframe_min_nonzeros;
  int   multiframe_is_optimizing_ell;
  int   multiframe_is_sorting_inner_product;
  int   multiframe_is_free_memory_each_iter;
} cvo_params;

/* ------------------------------------------------------------------ clouds
 * Host-side cloud descriptor; the caller owns the memory (as with the
 * reference's CvoPointCloud, "ownership: user", src/cvo/CvoState.cuh:23-24).
 * Replaces the AoS CvoPoint record (include/UnifiedCvo/utils/PointSegmentedDistribution.hpp:51-144).
 *   xyz       : n * xyz_stride floats (stride 3 or 4; extra component ignored)
 *   features  : n * F floats, row-major, values in [0,1] (NULL when F == 0)
 *   labels    : n * C floats, row-major label distributions (NULL when C == 0)
 *   geom_type : n * 2 floats (NULL unless is_using_geometric_type)
 */
typedef struct cvo_cloud {
  int n;
  int F;
  int C;
  int xyz_stride;
  const float *xyz;
  const float *features;
  const float *labels;
  const float *geom_type;
} cvo_cloud;

typedef struct cvo_handle cvo_handle;         /* replaces cvo::CvoGPU */
typedef struct cvo_gpu_cloud cvo_gpu_cloud;   /* replaces CvoPointCloudGPU (thrust::device_vector<CvoPoint>) */
typedef struct cvo_assoc cvo_assoc;           /* replaces cvo::Association (include/UnifiedCvo/cvo/Association.hpp:5-12) */

/* ------------------------------------------------------------ parameters */
/* CvoParams::CvoParams() defaults (CvoParams.hpp:80-136). */
void cvo_params_default(cvo_params *p);
/* read_CvoParams_yaml (CvoParams.hpp:203-323): sets only the keys present in the file. */
int cvo_params_read_yaml(const char *yaml_path, cvo_params *inout);

/* ---------------------------------------------------------------- handle */
/* CvoGPU::CvoGPU(const std::string&) (src/cvo/CvoGPU.cu:65-74). */
int cvo_create(const char *yaml_path, cvo_handle **out);
/* Same as cvo_create with an explicit parameter block (no file). */
int cvo_create_with_params(const cvo_params *p, cvo_handle **out);
/* CvoGPU::~CvoGPU (src/cvo/CvoGPU.cu:83-86). */
int cvo_destroy(cvo_handle *h);
/* CvoGPU::get_params (include/UnifiedCvo/cvo/CvoGPU.hpp:66). */
int cvo_get_params(const cvo_handle *h, cvo_params *out);
/* CvoGPU::write_params (src/cvo/CvoGPU.cu:76-80); here both the host and device copies change. */
int cvo_write_params(cvo_handle *h, const cvo_params *p);

/* ----------------------------------------------------------- device clouds */
/* CvoPointCloud_to_gpu (src/cvo/CvoGPU_impl.cu:220-289): upload once, reuse across calls. */
int cvo_cloud_upload(cvo_handle *h, const cvo_cloud *c, cvo_gpu_cloud **out);
int cvo_cloud_free(cvo_handle *h, cvo_gpu_cloud *c);
int cvo_cloud_size(const cvo_gpu_cloud *c);
/* Feature and class counts of a device cloud and whether it has geometric types. */
int cvo_cloud_dims(const cvo_gpu_cloud *c, int *F, int *C, int *has_geom_type);
/* Copies a device cloud back in its original point order: xyz n x 3, features n x F,
 * labels n x C, geom_type n x 2 (row-major floats); any pointer may be NULL.  The
 * reference's counterpart is reading a CvoPointCloud's accessors (CvoPointCloud.hpp:32-221). */
int cvo_cloud_download(cvo_handle *h, const cvo_gpu_cloud *c, float *xyz, float *features, float *labels,
                       float *geom_type);
/* CvoPointCloud(const ImageRGBD<float>&, const Calibration&, PointSelectionMethod)
 * (src/utils/CvoPointCloud.cpp:458-560) with RawImage's intensity and gradient
 * (src/utils/RawImage.cpp:9-45, 117-143), built on the device.  image: rows x cols x
 * channels bytes (BGR for 3 channels, as cv::Mat); depth: rows x cols floats in raw
 * units; intrinsic: fx, fy, cx, cy; scaling_factor: raw depth units per metre
 * (Calibration::scaling_factor); uv: n_sel (u, v) selected pixels; geom_type: n_sel x 2
 * or NULL (the selector's edge/surface weights); semantics: rows x cols x num_classes
 * or NULL.  Features are B, G, R (or grey) / 255 and two gradient terms / 500 + 0.5;
 * pixels without depth, non-finite points and points farther than 55 are dropped,
 * the rest keep the selection order.  The image is used as given: the reference's
 * default denoising (OpenCV fastNlMeans) and its pixel selectors (FAST, DSO, edges)
 * are left to the caller.  *n_points receives the number of points kept. */
int cvo_cloud_from_rgbd(cvo_handle *h, const uint8_t *image, int rows, int cols, int channels, const float *depth,
                        const float intrinsic[4], float scaling_factor, const int *uv, int n_sel,
                        const float *geom_type, int num_classes, const float *semantics, cvo_gpu_cloud **out,
                        int *n_points);

/* ------------------------------------------------------------- two-view */
/* int CvoGPU::align(src, tgt, T_init, T_out&, Association*, double* secs, int* iters)
 * (src/cvo/CvoGPU.cu:1516-1563).  assoc may be NULL; it is filled only when
 * params.is_exporting_association is set, as in the reference (:1468-1472).
 * Returns CVO_OK or CVO_ZERO_GRADIENT (the reference's ret -1). */
int cvo_align(cvo_handle *h, const cvo_cloud *src, const cvo_cloud *tgt,
              const float T_init[16], float T_out[16], cvo_assoc *assoc,
              double *secs, int *iters);
/* Device-resident variant of cvo_align (clouds already uploaded). */
int cvo_align_dev(cvo_handle *h, cvo_gpu_cloud *src, cvo_gpu_cloud *tgt,
                  const float T_init[16], float T_out[16], cvo_assoc *assoc,
                  double *secs, int *iters);
/* CvoResultInfo CvoGPU::align(src, tgt, T_s2t, is_returning_association)
 * (src/cvo/CvoGPU.cu:1566-1611): takes the source->target transform and
 * inverts it before iterating.  ret_code receives the reference's return_code. */
int cvo_align_s2t(cvo_handle *h, const cvo_cloud *src, const cvo_cloud *tgt,
                  const float T_s2t[16], int want_assoc, float T_out[16],
                  cvo_assoc *assoc, double *secs, int *iters, int *ret_code);

/* Batched two-view align: n_pairs independent registrations in one persistent
 * batch (one launch per kernel per iteration for all pairs).  srcs/tgts hold
 * n_pairs device clouds (repeats allowed), T_init/T_out are n_pairs*16 floats.
 * rets/iters are n_pairs ints (may be NULL).  No reference counterpart: it
 * batches the loop of CvoGPU::align (src/cvo/CvoGPU.cu:1239-1477). */
int cvo_align_batch_dev(cvo_handle *h, int n_pairs, cvo_gpu_cloud *const *srcs,
                        cvo_gpu_cloud *const *tgts, const float *T_init,
                        float *T_out, int *rets, int *iters, double *secs);

/* ------------------------------------------------- inner product / angle */
/* CvoGPU::inner_product_gpu (src/cvo/CvoGPU.cu:1734-1748): <f(X), f(T^-1 Y)> with
 * the GPU semantics (range-scaled ell, first nearest_neighbors_max hits per row). */
int cvo_inner_product(cvo_handle *h, const cvo_cloud *src, const cvo_cloud *tgt,
                      const float T[16], float ell, float *out);
int cvo_inner_product_dev(cvo_handle *h, cvo_gpu_cloud *src, cvo_gpu_cloud *tgt,
                          const float T[16], float ell, float *out);
/* CvoGPU::inner_product_cpu (src/cvo/CvoGPU.cpp:204-231): host implementation
 * with the reference CPU semantics (radius search, no neighbour cap, no range ell). */
int cvo_inner_product_cpu(cvo_handle *h, const cvo_cloud *src, const cvo_cloud *tgt,
                          const float T[16], float ell, float *out);
/* CvoGPU::function_angle (src/cvo/CvoGPU.cu:1768-1806). */
int cvo_function_angle(cvo_handle *h, const cvo_cloud *src, const cvo_cloud *tgt,
                       const float T[16], float ell, int is_approximate, int is_gpu,
                       float *out);
/* Batched inner products of one source/target pair under n_poses transforms
 * (n_poses*16 floats), all in one launch; out receives n_poses floats.  This is
 * the batched form of the loop in CvoGPU::get_nearest_init_pose (src/cvo/CvoGPU.cpp:367-398). */
int cvo_inner_product_batch_dev(cvo_handle *h, cvo_gpu_cloud *src, cvo_gpu_cloud *tgt,
                                int n_poses, const float *T, float ell, float *out);

/* Inner product that allocates nothing.  No counterpart in the reference: it
 * is for callers that cannot allocate device memory when they need the value
 * (fixed-budget real-time loops, hosts that hand out all device memory from
 * their own pool, plugins forbidden to call cudaMalloc after start-up).
 * src_dev / tgt_dev describe DEVICE-resident arrays (same layout as cvo_cloud);
 * the result (same semantics as cvo_inner_product) is written to the device
 * float *out_dev on `cuda_stream` (NULL = default stream); the call does not
 * synchronize.  Its only scratch is a fixed 65,792-byte array inside this
 * library, so at most 1,048,576 source points per call; it scans every target
 * for every source row (O(N * M)), so N * M is limited to 2^33 pair tests per
 * call (about 92k x 92k points; larger calls return CVO_ERR_CAPACITY before
 * touching the device).  All calls share that array: calls
 * whose kernels overlap on the GPU race and must be ordered by the caller.  The
 * first call on a device looks the array up with that device current; make it
 * before any stream capture.  No handle is needed. */
int cvo_inner_product_noalloc(const cvo_params *p, const cvo_cloud *src_dev, const cvo_cloud *tgt_dev,
                              const float T[16], float ell, float *out_dev, void *cuda_stream);

/* --------------------------------------------------------- association */
/* CvoGPU::compute_association_gpu (src/cvo/CvoGPU.cu:1836-1871). */
int cvo_compute_association(cvo_handle *h, const cvo_cloud *src, const cvo_cloud *tgt,
                            const float T[16], float ell, cvo_assoc *out);
/* CvoGPU::compute_association_gpu with a non-isotropic kernel (src/cvo/CvoGPU.cu:1936-1950,
 * inner_product_non_isotropic_impl :1873-1934, fill_in_A_mat_gpu_dense_mat_kernel :719-830):
 * kernel = 3x3 geometric kernel, column-major (Eigen::Matrix3f); it is inverted, rotated
 * per source point (rotate_kernel_and_inverse, :135-160) and used as a Mahalanobis
 * distance; no distance threshold, geometric type off.  Target moved by T^-1. */
int cvo_compute_association_aniso(cvo_handle *h, const cvo_cloud *src, const cvo_cloud *tgt,
                                  const float T[16], const float kernel[9], cvo_assoc *out);
int cvo_compute_association_aniso_dev(cvo_handle *h, const cvo_gpu_cloud *src, const cvo_gpu_cloud *tgt,
                                      const float T[16], const float kernel[9], cvo_assoc *out);
int cvo_assoc_create(cvo_assoc **out);
int cvo_assoc_destroy(cvo_assoc *a);
/* Sizes of the stored association: rows (= source points), cols (= target points),
 * nnz, and the number of source / target inlier entries. */
int cvo_assoc_info(const cvo_assoc *a, int *rows, int *cols, int64_t *nnz,
                   int64_t *n_source_inliers, int64_t *n_target_inliers);
/* Copies the row-major CSR (row_ptr[rows+1], col[nnz], val[nnz], columns sorted
 * ascending within each row) and the inlier lists.  Any pointer may be NULL. */
int cvo_assoc_copy(const cvo_assoc *a, int64_t *row_ptr, int *col, float *val,
                   int *source_inliers, int *target_inliers);

/* --------------------------------------------------- global registration */
/* CvoGPU::get_nearest_init_pose (src/cvo/CvoGPU.cpp:367-398): argmax of the
 * approximate cos-angle over a rotation grid at ell.  grid_kind 0 selects the
 * reference's 60-element icosahedral grid (gen_icosahedron_init_rots, :279-342);
 * grid_kind 1 the 24-element octahedral grid; grid_kind 2 the n^3 roll-pitch-yaw
 * grid of gen_rand_init_pose (:344-363) with n = num_guess.  T_out receives the
 * chosen [rot|0] (source frame -> target frame), secs the elapsed seconds. */
int cvo_get_nearest_init_pose(cvo_handle *h, const cvo_cloud *src, const cvo_cloud *tgt,
                              float ell, int num_guess, int grid_kind,
                              float T_out[16], double *secs);
int cvo_get_nearest_init_pose_dev(cvo_handle *h, cvo_gpu_cloud *src, cvo_gpu_cloud *tgt,
                                  float ell, int num_guess, int grid_kind,
                                  float T_out[16], double *secs);
/* Rotation grids themselves (row-major 3x3 each): returns the count, writes up to
 * max_rots rotations into rots (rots may be NULL to query the count). */
int cvo_rotation_grid(int grid_kind, int num_guess, float *rots, int max_rots);

/* Global registration of one pair from a set of initial poses: every hypothesis
 * (n_hyp column-major 4x4 internal init poses, as taken by cvo_align) is refined
 * by the batched align and judged by the final approximate cos-angle at
 * judge_ell; the best pose is returned in T_out (cvo_align convention) and its
 * index in best.  cos_out (n_hyp floats, may be NULL) receives every judged value. */
int cvo_register_hypotheses_dev(cvo_handle *h, cvo_gpu_cloud *src, cvo_gpu_cloud *tgt,
                                int n_hyp, const float *T_init, float judge_ell,
                                float T_out[16], int *best, float *cos_out, double *secs);

/* ------------------------------------------------------------ autotuner */
/* The association's grid cell size for search radius r and source tiles of diagonal
 * ext is max(r / div_r, (ext + 2 r) / div_ext).  cvo_autotune_dev times one
 * association pass of (src, tgt) at pose T and lengthscale ell (<= 0: ell_init) for
 * each candidate (div_r in {2, 3, 4, 6} x div_ext in {4, 8, 16}; median of reps), then
 * the best of these with 1 to 3 resident blocks per SM, and keeps the fastest for every
 * later batch with the same (F, C, log2 rows) key (the arrays list all 15 candidates).  The
 * kernel matrix does not depend on the choice (kept pairs are defined by index order);
 * only the candidate work per row does.  Arrays (max_configs entries, may be NULL)
 * receive every candidate and its time in ms; best its index.  No reference
 * counterpart: the reference's block size and kd-tree are compile-time choices
 * (CMakeLists.txt:473-558, src/experiments/cuda_performance_tune.cu:3-45). */
int cvo_autotune_dev(cvo_handle *h, cvo_gpu_cloud *src, cvo_gpu_cloud *tgt, const float T[16], float ell, int reps,
                     int max_configs, int *n_configs, float *div_r, float *div_ext, float *ms, int *best);
/* Set / read the configuration of a key (for a cache the caller persists); get returns
 * CVO_ERR_INVALID_ARG and the defaults (4, 8) for a key that was never tuned. */
int cvo_tune_set(cvo_handle *h, int F, int C, int64_t rows, float div_r, float div_ext);
int cvo_tune_get(const cvo_handle *h, int F, int C, int64_t rows, float *div_r, float *div_ext);
/* The same with the launch dimension: after the 12 cell sizes, cvo_autotune_launch_dev
 * times the best one with 1, 2 and 3 resident association blocks per SM (0 = as many as
 * the occupancy allows, the default) and keeps the fastest of all 15; blocks_per_sm
 * receives each candidate's value.  Like the cell size, the choice changes no result.
 * The cell size applies to later batches of pairs of the key's size; the blocks per SM
 * only to batches with as many work items (128 source rows each) as the tuned pair, i.e.
 * single-pair batches of that size (batches of many pairs keep the occupancy default).
 * No reference counterpart (its block sizes are compile-time, CMakeLists.txt:473-558). */
int cvo_autotune_launch_dev(cvo_handle *h, cvo_gpu_cloud *src, cvo_gpu_cloud *tgt, const float T[16], float ell,
                            int reps, int max_configs, int *n_configs, float *div_r, float *div_ext,
                            int *blocks_per_sm, float *ms, int *best);
int cvo_tune_set_launch(cvo_handle *h, int F, int C, int64_t rows, float div_r, float div_ext, int blocks_per_sm);
int cvo_tune_get_launch(const cvo_handle *h, int F, int C, int64_t rows, float *div_r, float *div_ext,
                        int *blocks_per_sm);

/* ---------------------------------------------------- adaptive-ell CVO */
/* AdaptiveCvoGPU::align(source, target, init_guess_transform, transform, seconds)
 * (include/UnifiedCvo/cvo/AdaptiveCvoGPU.hpp:171-175, src/cvo/AdaptiveCvoGPU.cu:
 * 1077-1250): CVO whose lengthscale follows the gradient of the inner product
 * (ell <- ell - dl_step dl, backed off to 0.7 ell_max at ell_max, floor ell_min),
 * with the three kernel matrices A, Axx, Ayy of fill_in_A_mat_gpu (:263-407: no
 * range scaling, first 512 kept pairs per row in index order).  Same pose
 * conventions as cvo_align; CVO_ZERO_GRADIENT for the reference's return -1. */
int cvo_align_adaptive(cvo_handle *h, const cvo_cloud *src, const cvo_cloud *tgt, const float T_init[16],
                       float T_out[16], double *secs, int *iters);
/* Device clouds; trace (may be NULL) receives per iteration {ell, dl, step, nnz(A),
 * nnz(Axx), nnz(Ayy)} for the first trace_len iterations. */
int cvo_align_adaptive_dev(cvo_handle *h, cvo_gpu_cloud *src, cvo_gpu_cloud *tgt, const float T_init[16],
                           float T_out[16], double *secs, int *iters, double *trace, int trace_len);
/* The kernel matrix A of the adaptive path at pose T and lengthscale ell
 * (se_kernel -> fill_in_A_mat_gpu, src/cvo/AdaptiveCvoGPU.cu:263-443). */
int cvo_compute_association_adaptive(cvo_handle *h, const cvo_cloud *src, const cvo_cloud *tgt,
                                     const float T[16], float ell, cvo_assoc *out);

/* ---------------------------------------------------------- pose graph */
/* FP64 SE(3) pose graph for the reference's keyframe graph
 * (src/graph_optimizer/PoseGraph.cpp:321-345 prior, :367-470 between factors,
 * :471-495 GTSAM ISAM2 / fixed-lag update).  Poses are row-major 3x4 doubles
 * [R | t], frame -> world; a between measurement is Xi^-1 Xj.  Errors follow GTSAM's
 * PriorFactor / BetweenFactor<Pose3> (Log of the residual pose, rotation first),
 * whitened by diagonal sigmas; cvo_pose_graph_optimize runs Levenberg-Marquardt to
 * the batch optimum (ISAM2's estimate).  A graph needs at least one prior
 * (CVO_ERR_UNSUPPORTED otherwise: the reference's GTSAM call throws on the
 * indeterminate system). */
typedef struct cvo_pose_graph cvo_pose_graph;
int cvo_pose_graph_create(cvo_pose_graph **out);
int cvo_pose_graph_destroy(cvo_pose_graph *g);
/* initial (or new) value of a pose variable */
int cvo_pose_graph_insert(cvo_pose_graph *g, int64_t key, const double pose[12]);
int cvo_pose_graph_add_prior(cvo_pose_graph *g, int64_t key, const double pose[12], const double sigmas[6]);
int cvo_pose_graph_add_between(cvo_pose_graph *g, int64_t from, int64_t to, const double rel[12],
                               const double sigmas[6]);
int cvo_pose_graph_optimize(cvo_pose_graph *g, int max_iters, double *initial_cost, double *final_cost, int *iters);
int cvo_pose_graph_get(const cvo_pose_graph *g, int64_t key, double pose[12]);
int cvo_pose_graph_size(const cvo_pose_graph *g, int *n_poses, int *n_factors);
int cvo_pose_graph_cost(const cvo_pose_graph *g, double *cost);

/* ---------------------------------------------------- learned proposal */
/* A point-set network that proposes K = 8 poses per pair for global registration,
 * standing in for the rotation grid of get_nearest_init_pose (src/cvo/CvoGPU.cpp:
 * 367-398, grids :279-363), which stays the fallback.  No reference counterpart:
 * the reference has no learned component.  Per-point MLP 8 -> 64 -> 128 (ReLU),
 * max-pool over points_per_cloud sampled points, pair head 256 -> 256 -> K * 9
 * (6D rotation + translation residual), BF16 tensor-core products with FP32
 * accumulation; training (relaxed winner-takes-all loss, Adam) runs on the device.
 * Poses are column-major 4x4 in cvo_align's T_init convention (target = R source + t). */
typedef struct cvo_proposal cvo_proposal;
int cvo_proposal_create(cvo_handle *h, int points_per_cloud, uint32_t seed, cvo_proposal **out);
int cvo_proposal_destroy(cvo_proposal *p);
/* parameter count, points per cloud and hypotheses per pair (p may be NULL) */
int cvo_proposal_dims(const cvo_proposal *p, int *num_params, int *points_per_cloud, int *num_hyp);
/* which: 0 weights, 1 gradients of the last training call, 2 / 3 Adam moments */
int cvo_proposal_get(cvo_handle *h, cvo_proposal *p, int which, float *out);
/* new weights (num_params floats); the Adam state restarts */
int cvo_proposal_set(cvo_handle *h, cvo_proposal *p, const float *weights);
/* Which kernel computes the network's matrix products: 0 (default) the tcgen05
 * tensor-core GEMM with TMEM accumulators, 1 the warp-level mma.sync GEMM (kept as a
 * second opinion for tests).  No reference counterpart. */
int cvo_proposal_set_gemm(cvo_proposal *p, int kind);
/* One training step on n_pairs labelled pairs drawn from a device-resident pool:
 * src_pts / tgt_pts are device arrays of n_scenes x n_pts x 8 floats (x, y, z and
 * 5 features); pair b takes scene[b] and moves its target by T_label[b] (12 floats,
 * row-major 3x4, target = R source + t), which is also its label.  Computes the
 * loss (mean over pairs) and the gradients; with lr > 0 applies one Adam step. */
int cvo_proposal_train_pool_dev(cvo_handle *h, cvo_proposal *p, int n_scenes, int n_pts, const float *src_pts,
                                const float *tgt_pts, int n_pairs, const int *scene, const float *T_label,
                                float lr, uint32_t seed, float *loss);
/* Forward pass on pool pairs (T_tgt may be NULL = identity): raw_out n_pairs x 72
 * network outputs, T_out n_pairs x 8 x 16 hypotheses (either may be NULL). */
int cvo_proposal_forward_pool_dev(cvo_handle *h, cvo_proposal *p, int n_scenes, int n_pts, const float *src_pts,
                                  const float *tgt_pts, int n_pairs, const int *scene, const float *T_tgt,
                                  uint32_t seed, float *raw_out, float *T_out);
/* Hypotheses for device clouds: T_out n_pairs x 8 x 16. */
int cvo_proposal_hypotheses_dev(cvo_handle *h, cvo_proposal *p, int n_pairs, cvo_gpu_cloud *const *srcs,
                                cvo_gpu_cloud *const *tgts, uint32_t seed, float *T_out);
/* Learned global registration of n_pairs pairs: hypotheses ranked by the cos-angle
 * at rank_ell, the best n_refine (1..8) of each pair refined by one batched align
 * and judged by the final cos-angle at judge_ell; pairs judged below fallback_cos
 * are registered again from the 24-rotation grid and keep the better result.
 * refine_ell > 0 starts the hypotheses' refinement at that lengthscale instead of
 * ell_init (the grid fallback keeps ell_init).
 * T_out: n_pairs x 16 (cvo_align's T_out convention); cos_out, used_fallback and
 * iters (align iterations summed over the pair's refinements) may be NULL. */
int cvo_register_learned_batch_dev(cvo_handle *h, cvo_proposal *p, int n_pairs, cvo_gpu_cloud *const *srcs,
                                   cvo_gpu_cloud *const *tgts, int n_refine, float rank_ell, float judge_ell,
                                   float fallback_cos, float refine_ell, uint32_t seed, float *T_out,
                                   float *cos_out, int *used_fallback, int *iters, double *secs);

/* Global registration of n_pairs host pairs in one call (poses in cvo_align's T_out
 * convention, n_pairs x 16; iters n_pairs ints, may be NULL).  use_learned = 0: the
 * plain grid, CvoGPU::get_nearest_init_pose (src/cvo/CvoGPU.cpp:367-398) over the 24
 * cube rotations at ell_init_first_frame, then align from the inverted grid pose as
 * CvoGPU::align's int overload does (src/cvo/CvoGPU.cu:1533-1543), all pairs in one
 * batched align.  use_learned = 1: cvo_register_learned_batch_dev with proposal (best 2
 * of 8 hypotheses refined, ranked and judged at ell_init_first_frame, grid fallback
 * below cos-angle 0).  No reference counterpart as one call. */
int cvo_global_register(cvo_handle *h, int n_pairs, const cvo_cloud *srcs, const cvo_cloud *tgts,
                        int use_learned, cvo_proposal *proposal, float *T_out, int *iters, double *secs);

/* ---------------------------------------------------------- multi-frame */
/* CvoGPU::align(frames, frames_to_hold_const, edges, secs) (src/cvo/CvoGPU.cu:1615-1670)
 * -> CvoBatchIRLS::solve (src/cvo/IRLS.cpp:148-367).  poses: n_frames*12 doubles
 * (row-major 3x4, frame->world), updated in place.  hold_const: n_frames bytes.
 * edges: n_edges*2 frame indices.  iters receives the number of outer iterations. */
int cvo_align_multi(cvo_handle *h, int n_frames, const cvo_cloud *clouds,
                    double *poses, const uint8_t *hold_const, int n_edges,
                    const int *edges, double *secs, int *iters);
int cvo_align_multi_dev(cvo_handle *h, int n_frames, cvo_gpu_cloud *const *clouds,
                        double *poses, const uint8_t *hold_const, int n_edges,
                        const int *edges, double *secs, int *iters);

/* -------------------------------------------------------------- misc */
const char *cvo_status_string(int status);
/* Number of kernel launches this handle has issued since creation (all kernels
 * of this library; used by benchmarks to report launch counts). */
int64_t cvo_kernel_launch_count(const cvo_handle *h);
/* Stream used by the handle's work (a cudaStream_t passed as void*).  The
 * reference runs everything on the default stream; here a caller may hand its
 * own stream so that its CUDA events bracket the library's kernels.  NULL
 * restores the handle's private stream. */
int cvo_set_stream(cvo_handle *h, void *cuda_stream);
void *cvo_get_stream(const cvo_handle *h);
/* Kernel profiling (no reference counterpart; the reference only times the
 * whole align loop with cudaEvents, src/cvo/CvoGPU.cu:1270-1273,1436-1465).
 * When enabled, every association-kernel launch of the align loop is bracketed
 * by CUDA events on the handle's stream and its algorithmic bytes
 * ((N + M) * record_bytes + 4 N + 8 nnz per pair) are accumulated. */
int cvo_profile_enable(cvo_handle *h, int on);
int cvo_profile_read(const cvo_handle *h, double *assoc_ms, int64_t *assoc_launches,
                     double *assoc_bytes, int64_t *iterations);
int cvo_profile_reset(cvo_handle *h);
/* Accumulated event-timed milliseconds of the kernels of the align iterations:
 * [transform, association, reduction, step, all four]. */
int cvo_profile_kernels(const cvo_handle *h, double ms[5]);
/* The association phase of the same iterations split into [association kernel
 * (with its work-item ordering), row selection (first cap by index), row sums]. */
int cvo_profile_assoc_split(const cvo_handle *h, double ms[3]);
/* Last CUDA error text recorded by the handle (empty if none). */
const char *cvo_last_error(const cvo_handle *h);

#ifdef __cplusplus
}
#endif
#endif /* CVO_GB300_H */
