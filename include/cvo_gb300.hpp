/* cvo_gb300.hpp -- header-only C++ mirror of cvo::CvoGPU over the C ABI of cvo_gb300.h.
 *
 * For C++ callers of the reference class (include/UnifiedCvo/cvo/CvoGPU.hpp:43-274):
 * the same method names and argument meaning, without Eigen or PCL in the interface.
 * Poses are column-major float[16] (the layout of Eigen::Matrix4f::data()), multi-frame
 * poses row-major double[12] (frame -> world), clouds the plain PointCloud below (the
 * accessors of the reference's CvoPointCloud, include/UnifiedCvo/utils/CvoPointCloud.hpp).
 *
 * Error behaviour: the reference prints and returns -1 on a zero gradient and exits on a
 * CUDA error; here align returns 0 or -1 exactly as the reference does, and every
 * failure status of the library (bad yaml, empty input where the reference rejects it,
 * CUDA error, out of memory, ...) throws cvo_gb300::Error carrying the status code.
 * Link with -lcvo_gb300.
 */
#pragma once

#include <array>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "cvo_gb300.h"

namespace cvo_gb300 {

using Mat4 = std::array<float, 16>;                 // column-major 4x4

inline Mat4 identity() { return Mat4{1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1}; }

class Error : public std::runtime_error {
 public:
  Error(int status, const std::string &what)
      : std::runtime_error(what + ": " + cvo_status_string(status)), code(status) {}
  int code;
};

inline int check(int status, const char *what, const cvo_handle *h = nullptr) {
  if (status < 0 && status != CVO_ZERO_GRADIENT) {
    std::string w(what);
    const char *detail = h ? cvo_last_error(h) : "";
    if (detail && *detail) w += std::string(" [") + detail + "]";
    throw Error(status, w);
  }
  return status;
}

/* A host point cloud: n points, F features and C class probabilities per point
 * (row-major), optional geometric types (2 per point).  The library copies it. */
struct PointCloud {
  int F = 0, C = 0;
  std::vector<float> xyz, features, labels, geometric_types;

  int num_points() const { return (int)(xyz.size() / 3); }
  int feature_dimensions() const { return F; }
  int num_classes() const { return C; }
  cvo_cloud view() const {
    const int n = num_points();
    return cvo_cloud{n, F, C, 3, n ? xyz.data() : nullptr, (F && n) ? features.data() : nullptr,
                     (C && n) ? labels.data() : nullptr, geometric_types.empty() ? nullptr : geometric_types.data()};
  }
};

/* cvo::Association (include/UnifiedCvo/cvo/Association.hpp:5-12) as row-major CSR:
 * rows are source indices, columns target indices (ascending within a row). */
struct Association {
  int rows = 0, cols = 0;
  std::vector<int64_t> row_ptr;
  std::vector<int> col;
  std::vector<float> val;
  std::vector<int> source_inliers, target_inliers;
};

class CvoGPU {
 public:
  /* CvoGPU::CvoGPU(const std::string &param_file) (src/cvo/CvoGPU.cu:65-74) */
  explicit CvoGPU(const std::string &param_file) { check(cvo_create(param_file.c_str(), &h_), "cvo_create"); }
  explicit CvoGPU(const cvo_params &params) { check(cvo_create_with_params(&params, &h_), "cvo_create_with_params"); }
  ~CvoGPU() {
    if (h_) cvo_destroy(h_);
  }
  CvoGPU(const CvoGPU &) = delete;
  CvoGPU &operator=(const CvoGPU &) = delete;
  CvoGPU(CvoGPU &&o) noexcept : h_(std::exchange(o.h_, nullptr)) {}
  CvoGPU &operator=(CvoGPU &&o) noexcept {
    std::swap(h_, o.h_);
    return *this;
  }
  cvo_handle *handle() const { return h_; }

  cvo_params get_params() const {
    cvo_params p;
    check(cvo_get_params(h_, &p), "cvo_get_params", h_);
    return p;
  }
  void write_params(const cvo_params &p) { check(cvo_write_params(h_, &p), "cvo_write_params", h_); }

  /* int CvoGPU::align(source, target, init_guess_T, T_out, association, registration_seconds, num_iters)
   * (src/cvo/CvoGPU.cu:1516-1563): 0, or -1 on a zero gradient, like the reference. */
  int align(const PointCloud &source, const PointCloud &target, const Mat4 &init_guess_T, Mat4 &T_out,
            Association *association = nullptr, double *registration_seconds = nullptr,
            int *num_iters = nullptr) const {
    const cvo_cloud s = source.view(), t = target.view();
    cvo_assoc *a = nullptr;
    if (association) check(cvo_assoc_create(&a), "cvo_assoc_create");
    const int rc = cvo_align(h_, &s, &t, init_guess_T.data(), T_out.data(), a, registration_seconds, num_iters);
    if (a) {
      if (rc >= 0 || rc == CVO_ZERO_GRADIENT) read_assoc(a, association);
      cvo_assoc_destroy(a);
    }
    check(rc, "cvo_align", h_);
    return rc == CVO_ZERO_GRADIENT ? -1 : 0;
  }

  /* CvoGPU::inner_product_gpu / inner_product_cpu (src/cvo/CvoGPU.cu:1734-1748,
   * src/cvo/CvoGPU.cpp:204-231): <f(X), f(T^-1 Y)>. */
  float inner_product_gpu(const PointCloud &source, const PointCloud &target, const Mat4 &T, float ell) const {
    const cvo_cloud s = source.view(), t = target.view();
    float v = 0.f;
    check(cvo_inner_product(h_, &s, &t, T.data(), ell, &v), "cvo_inner_product", h_);
    return v;
  }
  float inner_product_cpu(const PointCloud &source, const PointCloud &target, const Mat4 &T, float ell) const {
    const cvo_cloud s = source.view(), t = target.view();
    float v = 0.f;
    check(cvo_inner_product_cpu(h_, &s, &t, T.data(), ell, &v), "cvo_inner_product_cpu", h_);
    return v;
  }

  /* CvoGPU::function_angle (src/cvo/CvoGPU.cu:1768-1806) */
  float function_angle(const PointCloud &source, const PointCloud &target, const Mat4 &T, float ell,
                       bool is_approximate = true, bool is_gpu = true) const {
    const cvo_cloud s = source.view(), t = target.view();
    float v = 0.f;
    check(cvo_function_angle(h_, &s, &t, T.data(), ell, is_approximate ? 1 : 0, is_gpu ? 1 : 0, &v),
          "cvo_function_angle", h_);
    return v;
  }

  /* CvoGPU::compute_association_gpu (src/cvo/CvoGPU.cu:1836-1871), isotropic lengthscale */
  Association compute_association_gpu(const PointCloud &source, const PointCloud &target, const Mat4 &T,
                                      float lengthscale) const {
    const cvo_cloud s = source.view(), t = target.view();
    cvo_assoc *a = nullptr;
    check(cvo_assoc_create(&a), "cvo_assoc_create");
    const int rc = cvo_compute_association(h_, &s, &t, T.data(), lengthscale, a);
    Association out;
    if (rc >= 0) read_assoc(a, &out);
    cvo_assoc_destroy(a);
    check(rc, "cvo_compute_association", h_);
    return out;
  }

  /* CvoGPU::get_nearest_init_pose (src/cvo/CvoGPU.cpp:367-398): the grid rotation with
   * the largest approximate cos-angle at init_guess_ell; grid_kind 0 = the reference's
   * 60 icosahedral rotations, 1 = 24 cube rotations, 2 = num_guess^3 roll-pitch-yaw. */
  Mat4 get_nearest_init_pose(const PointCloud &source, const PointCloud &target, float init_guess_ell,
                             int num_guess = 0, double *times = nullptr, int grid_kind = 0) const {
    const cvo_cloud s = source.view(), t = target.view();
    Mat4 T = identity();
    double secs = 0.0;
    check(cvo_get_nearest_init_pose(h_, &s, &t, init_guess_ell, num_guess, grid_kind, T.data(), &secs),
          "cvo_get_nearest_init_pose", h_);
    if (times) *times += secs;
    return T;
  }

  /* Global registration of host pairs in one call (cvo_global_register): the plain grid
   * (nearest of the 24 cube rotations, then one batched align), or the learned proposal
   * when proposal is non-null.  Poses in align's T_out convention. */
  std::vector<Mat4> global_register(const std::vector<PointCloud> &sources, const std::vector<PointCloud> &targets,
                                    cvo_proposal *proposal = nullptr, std::vector<int> *iters = nullptr,
                                    double *seconds = nullptr) const {
    if (sources.size() != targets.size())
      throw Error(CVO_ERR_INVALID_ARG, "global_register: one target per source");
    std::vector<cvo_cloud> s, t;
    for (size_t k = 0; k < sources.size(); k++) {
      s.push_back(sources[k].view());
      t.push_back(targets[k].view());
    }
    std::vector<Mat4> T(sources.size());
    std::vector<int> it(sources.size(), 0);
    check(cvo_global_register(h_, (int)sources.size(), s.data(), t.data(), proposal ? 1 : 0, proposal,
                              T.empty() ? nullptr : T[0].data(), it.data(), seconds),
          "cvo_global_register", h_);
    if (iters) *iters = it;
    return T;
  }

  /* CvoGPU::align(frames, frames_to_hold_const, edges, secs) (src/cvo/CvoGPU.cu:1615-1670):
   * poses n_frames x 12 doubles (row-major [R|t], frame -> world), updated in place. */
  int align(const std::vector<PointCloud> &frames, std::vector<std::array<double, 12>> &poses,
            const std::vector<uint8_t> &hold_const, const std::vector<std::pair<int, int>> &edges,
            double *registration_seconds = nullptr, int *num_iters = nullptr) const {
    if (poses.size() != frames.size() || hold_const.size() != frames.size())
      throw Error(CVO_ERR_INVALID_ARG, "align(frames): one pose and one hold flag per frame");
    std::vector<cvo_cloud> c;
    for (const PointCloud &f : frames) c.push_back(f.view());
    std::vector<int> e;
    for (const auto &ij : edges) {
      e.push_back(ij.first);
      e.push_back(ij.second);
    }
    const int rc = cvo_align_multi(h_, (int)frames.size(), c.data(), poses.empty() ? nullptr : poses[0].data(),
                                   hold_const.data(), (int)edges.size(), e.empty() ? nullptr : e.data(),
                                   registration_seconds, num_iters);
    check(rc, "cvo_align_multi", h_);
    return rc == CVO_ZERO_GRADIENT ? -1 : 0;
  }

 private:
  static void read_assoc(const cvo_assoc *a, Association *out) {
    int64_t nnz = 0, ns = 0, nt = 0;
    check(cvo_assoc_info(a, &out->rows, &out->cols, &nnz, &ns, &nt), "cvo_assoc_info");
    out->row_ptr.assign((size_t)out->rows + 1, 0);
    out->col.assign((size_t)nnz, 0);
    out->val.assign((size_t)nnz, 0.f);
    out->source_inliers.assign((size_t)ns, 0);
    out->target_inliers.assign((size_t)nt, 0);
    check(cvo_assoc_copy(a, out->row_ptr.data(), out->col.data(), out->val.data(), out->source_inliers.data(),
                         out->target_inliers.data()),
          "cvo_assoc_copy");
  }
  cvo_handle *h_ = nullptr;
};

/* cvo::AdaptiveCvoGPU (include/UnifiedCvo/cvo/AdaptiveCvoGPU.hpp:161-180): CVO whose
 * lengthscale follows the gradient of the inner product (src/cvo/AdaptiveCvoGPU.cu:1077-1250). */
class AdaptiveCvoGPU {
 public:
  explicit AdaptiveCvoGPU(const std::string &param_file) { check(cvo_create(param_file.c_str(), &h_), "cvo_create"); }
  explicit AdaptiveCvoGPU(const cvo_params &params) {
    check(cvo_create_with_params(&params, &h_), "cvo_create_with_params");
  }
  ~AdaptiveCvoGPU() {
    if (h_) cvo_destroy(h_);
  }
  AdaptiveCvoGPU(const AdaptiveCvoGPU &) = delete;
  AdaptiveCvoGPU &operator=(const AdaptiveCvoGPU &) = delete;
  cvo_handle *handle() const { return h_; }

  /* AdaptiveCvoGPU::align(source, target, init_guess_transform, transform, registration_seconds)
   * (AdaptiveCvoGPU.hpp:171-175): 0, or -1 on a zero gradient; an empty cloud throws
   * (CVO_ERR_EMPTY_CLOUD). */
  int align(const PointCloud &source, const PointCloud &target, const Mat4 &init_guess_transform, Mat4 &transform,
            double *registration_seconds = nullptr, int *num_iters = nullptr) const {
    const cvo_cloud s = source.view(), t = target.view();
    const int rc = cvo_align_adaptive(h_, &s, &t, init_guess_transform.data(), transform.data(),
                                      registration_seconds, num_iters);
    check(rc, "cvo_align_adaptive", h_);
    return rc == CVO_ZERO_GRADIENT ? -1 : 0;
  }

 private:
  cvo_handle *h_ = nullptr;
};

/* The keyframe pose graph's solver (GTSAM's Prior / Between Pose3 factors of
 * src/graph_optimizer/PoseGraph.cpp:321-495): poses row-major double[12]; sigmas
 * rotation first, as in GTSAM. */
class PoseGraphSolver {
 public:
  PoseGraphSolver() { check(cvo_pose_graph_create(&g_), "cvo_pose_graph_create"); }
  ~PoseGraphSolver() {
    if (g_) cvo_pose_graph_destroy(g_);
  }
  PoseGraphSolver(const PoseGraphSolver &) = delete;
  PoseGraphSolver &operator=(const PoseGraphSolver &) = delete;

  void insert(int64_t key, const std::array<double, 12> &pose) {
    check(cvo_pose_graph_insert(g_, key, pose.data()), "cvo_pose_graph_insert");
  }
  void add_prior(int64_t key, const std::array<double, 12> &pose, const std::array<double, 6> &sigmas) {
    check(cvo_pose_graph_add_prior(g_, key, pose.data(), sigmas.data()), "cvo_pose_graph_add_prior");
  }
  void add_between(int64_t from, int64_t to, const std::array<double, 12> &rel, const std::array<double, 6> &sigmas) {
    check(cvo_pose_graph_add_between(g_, from, to, rel.data(), sigmas.data()), "cvo_pose_graph_add_between");
  }
  /* Levenberg-Marquardt to convergence or max_iters; returns the final cost. */
  double optimize(int max_iters = 100, double *initial_cost = nullptr, int *iters = nullptr) {
    double c0 = 0.0, c1 = 0.0;
    int it = 0;
    check(cvo_pose_graph_optimize(g_, max_iters, &c0, &c1, &it), "cvo_pose_graph_optimize");
    if (initial_cost) *initial_cost = c0;
    if (iters) *iters = it;
    return c1;
  }
  std::array<double, 12> get(int64_t key) const {
    std::array<double, 12> X{};
    check(cvo_pose_graph_get(g_, key, X.data()), "cvo_pose_graph_get");
    return X;
  }

 private:
  cvo_pose_graph *g_ = nullptr;
};

}  // namespace cvo_gb300
