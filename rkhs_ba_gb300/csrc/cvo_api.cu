// cvo_api.cu -- the C ABI (include/cvo_gb300.h): parameters and their yaml
// reader, handles, device clouds, and the CvoGPU entry points.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cctype>
#include <string>
#include <vector>
#include <algorithm>
#include <chrono>
#include <fstream>
#include <sstream>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "cvo_internal.h"

using namespace cvo_gb;

struct cvo_handle { Handle h; };
struct cvo_gpu_cloud { DevCloud *d; cvo_handle *owner; };
struct cvo_assoc {
  int rows = 0, cols = 0;
  std::vector<int64_t> row_ptr;
  std::vector<int> col;
  std::vector<float> val;
  std::vector<int> source_inliers, target_inliers;
};

namespace cvo_gb { void free_workspace(Handle *h); }

// ------------------------------------------------------------ parameters
extern "C" void cvo_params_default(cvo_params *p) {
  if (!p) return;
  memset(p, 0, sizeof(*p));
  // CvoParams::CvoParams() (include/UnifiedCvo/cvo/CvoParams.hpp:80-136)
  p->ell_init_first_frame = 0.5f;
  p->ell_init = 0.5f;
  p->ell_min = 0.05f;
  p->min_ell_iter_limit = 1;
  p->ell_max = 1.2f;
  p->dl = 0.0;
  p->dl_step = 0.3;
  p->sigma = 0.1f;
  p->sp_thres = 0.0006f;
  p->c = 7.0f;
  p->d = 7.0f;
  p->c_ell = 0.15f;
  p->c_sigma = 0.6f;
  p->s_ell = 0.1f;
  p->s_sigma = 0.8f;
  p->MAX_ITER = 10000;
  p->min_step = 2e-5f;
  p->max_step = 0.8f;   // left uninitialised by the reference constructor
  p->step = 0.f;
  p->eps = 0.00005f;
  p->eps_2 = 0.000012f;
  p->ell_decay_rate = 0.9f;
  p->ell_decay_rate_first_frame = 0.99f;
  p->ell_decay_start = 30;
  p->ell_decay_start_first_frame = 300;
  p->indicator_window_size = 15;
  p->indicator_stable_threshold = 0.2f;
  p->is_pcl_visualization_on = 0;
  p->is_using_least_square = 0;
  p->is_ell_adaptive = 0;
  p->is_full_ip_matrix = 0;
  p->is_using_geometry = 1;
  p->is_using_intensity = 0;
  p->is_using_semantics = 0;
  p->is_using_range_ell = 0;
  p->is_using_kdtree = 0;
  p->is_using_geometric_type = 0;
  p->is_global_angle_registration = 0;
  p->is_exporting_association = 0;
  p->multiframe_using_cpu = 1;
  p->multiframe_max_iters = 200;
  p->nearest_neighbors_max = 512;
  p->multiframe_ell_init = 0.15f;
  p->multiframe_ell_min = 0.05f;
  p->multiframe_ell_max = 5.0f;
  p->multiframe_iter_per_ell = 10;
  p->multiframe_ell_decay_rate = 0.7f;
  p->multiframe_iterations_per_ell = 50;
  p->multiframe_iterations_per_solve = 8;
  p->multiframe_downsample_voxel_size = 0.5f;
  p->multiframe_expected_points = 1000;
  p->multiframe_num_neighbors = 128;
  p->multiframe_min_nonzeros = 300;
  p->multiframe_least_squares_num_threads = 24;
  p->multiframe_is_optimizing_ell = 0;
  p->multiframe_is_sorting_inner_product = 0;
  p->multiframe_is_free_memory_each_iter = 0;
}

namespace {

std::string trim(const std::string &s) {
  size_t a = 0, b = s.size();
  while (a < b && isspace((unsigned char)s[a])) a++;
  while (b > a && isspace((unsigned char)s[b - 1])) b--;
  return s.substr(a, b - a);
}

bool parse_double(const std::string &v, double *out) {
  if (v.empty()) return false;
  char *end = nullptr;
  double d = strtod(v.c_str(), &end);
  if (end == v.c_str() || *end != '\0') return false;
  *out = d;
  return true;
}

bool parse_int(const std::string &v, int *out) {
  if (v.empty()) return false;
  char *end = nullptr;
  long x = strtol(v.c_str(), &end, 10);
  if (end == v.c_str() || *end != '\0') return false;
  *out = (int)x;
  return true;
}

}  // namespace

// read_CvoParams_yaml (include/UnifiedCvo/cvo/CvoParams.hpp:203-323): a flat
// "key: value" reader that sets a field only when its key is present; keys the
// reference does not read are ignored.  Values that the reference's yaml-cpp
// `as<T>()` would reject (e.g. "True" for an int field) give CVO_ERR_BAD_YAML.
extern "C" int cvo_params_read_yaml(const char *path, cvo_params *p) try {
  if (!path || !p) return CVO_ERR_INVALID_ARG;
  std::ifstream f(path);
  if (!f.is_open()) return CVO_ERR_IO;
  struct FK { const char *k; float *f; };
  struct IK { const char *k; int *i; };
  struct DK { const char *k; double *d; };
  const FK fkeys[] = {
      {"ell_init_first_frame", &p->ell_init_first_frame}, {"ell_init", &p->ell_init}, {"ell_min", &p->ell_min},
      {"ell_max", &p->ell_max}, {"sigma", &p->sigma}, {"sp_thres", &p->sp_thres}, {"c", &p->c}, {"d", &p->d},
      {"c_ell", &p->c_ell}, {"c_sigma", &p->c_sigma}, {"s_ell", &p->s_ell}, {"s_sigma", &p->s_sigma},
      {"eps", &p->eps}, {"eps_2", &p->eps_2}, {"min_step", &p->min_step}, {"max_step", &p->max_step},
      {"ell_decay_rate", &p->ell_decay_rate}, {"ell_decay_rate_first_frame", &p->ell_decay_rate_first_frame},
      {"indicator_stable_threshold", &p->indicator_stable_threshold},
      {"multiframe_ell_init", &p->multiframe_ell_init}, {"multiframe_ell_min", &p->multiframe_ell_min},
      {"multiframe_ell_max", &p->multiframe_ell_max}, {"multiframe_ell_decay_rate", &p->multiframe_ell_decay_rate},
      {"multiframe_downsample_voxel_size", &p->multiframe_downsample_voxel_size}};
  const IK ikeys[] = {
      {"min_ell_iter_limit", &p->min_ell_iter_limit}, {"MAX_ITER", &p->MAX_ITER},
      {"ell_decay_start", &p->ell_decay_start}, {"ell_decay_start_first_frame", &p->ell_decay_start_first_frame},
      {"indicator_window_size", &p->indicator_window_size}, {"is_pcl_visualization_on", &p->is_pcl_visualization_on},
      {"is_using_least_square", &p->is_using_least_square}, {"is_full_ip_matrix", &p->is_full_ip_matrix},
      {"is_using_geometry", &p->is_using_geometry}, {"is_using_intensity", &p->is_using_intensity},
      {"is_using_semantics", &p->is_using_semantics}, {"is_using_range_ell", &p->is_using_range_ell},
      {"is_using_kdtree", &p->is_using_kdtree}, {"is_using_geometric_type", &p->is_using_geometric_type},
      {"is_global_angle_registration", &p->is_global_angle_registration},
      {"is_exporting_association", &p->is_exporting_association},
      {"nearest_neighbors_max", &p->nearest_neighbors_max}, {"multiframe_using_cpu", &p->multiframe_using_cpu},
      {"multiframe_max_iters", &p->multiframe_max_iters},
      // the reference reads this key into multiframe_iterations_per_ell, not multiframe_iter_per_ell
      {"multiframe_iterations_per_ell", &p->multiframe_iterations_per_ell},
      {"multiframe_iterations_per_solve", &p->multiframe_iterations_per_solve},
      {"multiframe_expected_points", &p->multiframe_expected_points},
      {"multiframe_num_neighbors", &p->multiframe_num_neighbors},
      {"multiframe_min_nonzeros", &p->multiframe_min_nonzeros},
      {"multiframe_least_squares_num_threads", &p->multiframe_least_squares_num_threads},
      {"multiframe_is_optimizing_ell", &p->multiframe_is_optimizing_ell},
      {"multiframe_is_sorting_inner_product", &p->multiframe_is_sorting_inner_product},
      {"multiframe_is_free_memory_each_iter", &p->multiframe_is_free_memory_each_iter}};
  const DK dkeys[] = {{"dl", &p->dl}, {"dl_step", &p->dl_step}};
  std::string line;
  while (std::getline(f, line)) {
    // strip comments
    size_t hash = line.find('#');
    if (hash != std::string::npos) line = line.substr(0, hash);
    std::string t = trim(line);
    if (t.empty() || t[0] == '%' || t == "---" || t == "...") continue;
    size_t colon = t.find(':');
    if (colon == std::string::npos) continue;
    std::string key = trim(t.substr(0, colon));
    std::string val = trim(t.substr(colon + 1));
    if (val.size() >= 2 && (val[0] == '"' || val[0] == '\'') && val.back() == val[0]) val = val.substr(1, val.size() - 2);
    bool done = false;
    for (const FK &k : fkeys)
      if (key == k.k) {
        double d;
        if (!parse_double(val, &d)) return CVO_ERR_BAD_YAML;
        *k.f = (float)d;
        done = true;
        break;
      }
    if (done) continue;
    for (const IK &k : ikeys)
      if (key == k.k) {
        int i;
        if (!parse_int(val, &i)) return CVO_ERR_BAD_YAML;
        *k.i = i;
        done = true;
        break;
      }
    if (done) continue;
    for (const DK &k : dkeys)
      if (key == k.k) {
        double d;
        if (!parse_double(val, &d)) return CVO_ERR_BAD_YAML;
        *k.d = d;
        break;
      }
  }
  return CVO_OK;
} catch (...) {
  return status_from_exception();
}

// --------------------------------------------------------------- handles
// A handle can be created without a CUDA device: the host-only entry points
// (parameters, cvo_inner_product_cpu, cvo_function_angle with is_gpu = 0) then
// work and every GPU entry point returns CVO_ERR_CUDA.
static int init_handle(cvo_handle *H) {
  Handle &h = H->h;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    h.last_error = "no CUDA device";
    h.stream = nullptr;
    return CVO_OK;
  }
  e = cudaGetDevice(&h.device);
  if (e != cudaSuccess) return set_cuda_error(&h, e, "cudaGetDevice");
  e = cudaDeviceGetAttribute(&h.num_sms, cudaDevAttrMultiProcessorCount, h.device);
  if (e != cudaSuccess) return set_cuda_error(&h, e, "cudaDeviceGetAttribute");
  e = cudaStreamCreateWithFlags(&h.own_stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) return set_cuda_error(&h, e, "cudaStreamCreate");
  h.stream = h.own_stream;
  return CVO_OK;
}

extern "C" int cvo_create_with_params(const cvo_params *p, cvo_handle **out) try {
  if (!p || !out) return CVO_ERR_INVALID_ARG;
  *out = nullptr;
  cvo_handle *H = new cvo_handle();
  H->h.params = *p;
  int rc = init_handle(H);
  if (rc) { delete H; return rc; }
  *out = H;
  return CVO_OK;
} catch (...) {
  return status_from_exception();
}

extern "C" int cvo_create(const char *yaml_path, cvo_handle **out) try {
  if (!yaml_path || !out) return CVO_ERR_INVALID_ARG;
  cvo_params p;
  cvo_params_default(&p);
  int rc = cvo_params_read_yaml(yaml_path, &p);
  if (rc) return rc;
  return cvo_create_with_params(&p, out);
} catch (...) {
  return status_from_exception();
}

extern "C" int cvo_destroy(cvo_handle *H) try {
  if (!H) return CVO_ERR_INVALID_ARG;
  if (H->h.stream) cudaStreamSynchronize(H->h.stream);
  free_workspace(&H->h);
  if (H->h.own_stream) cudaStreamDestroy(H->h.own_stream);
  delete H;
  return CVO_OK;
} catch (...) {
  return status_from_exception();
}

extern "C" int cvo_get_params(const cvo_handle *H, cvo_params *out) try {
  if (!H || !out) return CVO_ERR_INVALID_ARG;
  *out = H->h.params;
  return CVO_OK;
} catch (...) {
  return status_from_exception();
}

extern "C" int cvo_write_params(cvo_handle *H, const cvo_params *p) try {
  if (!H || !p) return CVO_ERR_INVALID_ARG;
  H->h.params = *p;
  return CVO_OK;
} catch (...) {
  return status_from_exception();
}

extern "C" const char *cvo_status_string(int s) {
  switch (s) {
    case CVO_OK: return "ok";
    case CVO_ZERO_GRADIENT: return "zero gradient";
    case CVO_ERR_INVALID_ARG: return "invalid argument";
    case CVO_ERR_EMPTY_CLOUD: return "empty point cloud";
    case CVO_ERR_BAD_YAML: return "bad yaml parameter file";
    case CVO_ERR_CUDA: return "CUDA error";
    case CVO_ERR_OUT_OF_MEMORY: return "out of device memory";
    case CVO_ERR_TIMEOUT: return "timeout";
    case CVO_ERR_UNSUPPORTED: return "unsupported configuration";
    case CVO_ERR_IO: return "I/O error";
    case CVO_ERR_CAPACITY: return "capacity exceeded";
    default: return "unknown status";
  }
}

extern "C" int64_t cvo_kernel_launch_count(const cvo_handle *H) { return H ? H->h.launches : 0; }
extern "C" const char *cvo_last_error(const cvo_handle *H) { return H ? H->h.last_error.c_str() : ""; }

extern "C" int cvo_set_stream(cvo_handle *H, void *stream) try {
  if (!H) return CVO_ERR_INVALID_ARG;
  if (!H->h.own_stream) return CVO_ERR_CUDA;
  cudaStreamSynchronize(H->h.stream);
  H->h.stream = stream ? (cudaStream_t)stream : H->h.own_stream;
  return CVO_OK;
} catch (...) {
  return status_from_exception();
}

extern "C" void *cvo_get_stream(const cvo_handle *H) { return H ? (void *)H->h.stream : nullptr; }

extern "C" int cvo_profile_enable(cvo_handle *H, int on) try {
  if (!H) return CVO_ERR_INVALID_ARG;
  H->h.prof.on = on != 0;
  return CVO_OK;
} catch (...) {
  return status_from_exception();
}

extern "C" int cvo_profile_read(const cvo_handle *H, double *assoc_ms, int64_t *assoc_launches, double *assoc_bytes,
                                int64_t *iterations) try {
  if (!H) return CVO_ERR_INVALID_ARG;
  if (assoc_ms) *assoc_ms = H->h.prof.assoc_ms;
  if (assoc_launches) *assoc_launches = H->h.prof.assoc_launches;
  if (assoc_bytes) *assoc_bytes = H->h.prof.assoc_bytes;
  if (iterations) *iterations = H->h.prof.iterations;
  return CVO_OK;
} catch (...) {
  return status_from_exception();
}

extern "C" int cvo_profile_kernels(const cvo_handle *H, double ms[5]) try {
  if (!H || !ms) return CVO_ERR_INVALID_ARG;
  for (int k = 0; k < 5; k++) ms[k] = H->h.prof.kernel_ms[k];
  return CVO_OK;
} catch (...) {
  return status_from_exception();
}

extern "C" int cvo_profile_assoc_split(const cvo_handle *H, double ms[3]) try {
  if (!H || !ms) return CVO_ERR_INVALID_ARG;
  for (int k = 0; k < 3; k++) ms[k] = H->h.prof.assoc_split_ms[k];
  return CVO_OK;
} catch (...) {
  return status_from_exception();
}

extern "C" int cvo_profile_reset(cvo_handle *H) try {
  if (!H) return CVO_ERR_INVALID_ARG;
  bool on = H->h.prof.on;
  H->h.prof = Profile();
  H->h.prof.on = on;
  return CVO_OK;
} catch (...) {
  return status_from_exception();
}

// ----------------------------------------------------------------- clouds
extern "C" int cvo_cloud_upload(cvo_handle *H, const cvo_cloud *c, cvo_gpu_cloud **out) try {
  if (!H || !c || !out) return CVO_ERR_INVALID_ARG;
  if (!H->h.stream) return CVO_ERR_CUDA;   // handle created without a CUDA device
  DevCloud *d = nullptr;
  int rc = cloud_upload(&H->h, c, &d);
  if (rc) { cloud_free(d); return rc; }
  cvo_gpu_cloud *g = new cvo_gpu_cloud();
  g->d = d;
  g->owner = H;
  *out = g;
  return CVO_OK;
} catch (...) {
  return status_from_exception();
}

extern "C" int cvo_cloud_free(cvo_handle *H, cvo_gpu_cloud *c) try {
  if (!c) return CVO_ERR_INVALID_ARG;
  if (H && H->h.stream) cudaStreamSynchronize(H->h.stream);
  cloud_free(c->d);
  delete c;
  return CVO_OK;
} catch (...) {
  return status_from_exception();
}

extern "C" int cvo_cloud_size(const cvo_gpu_cloud *c) { return c && c->d ? c->d->n : 0; }

extern "C" int cvo_cloud_dims(const cvo_gpu_cloud *c, int *F, int *C, int *has_geom_type) try {
  if (!c || !c->d) return CVO_ERR_INVALID_ARG;
  if (F) *F = c->d->F;
  if (C) *C = c->d->C;
  if (has_geom_type) *has_geom_type = c->d->has_geo ? 1 : 0;
  return CVO_OK;
} catch (...) {
  return status_from_exception();
}

extern "C" int cvo_cloud_download(cvo_handle *H, const cvo_gpu_cloud *c, float *xyz, float *features, float *labels,
                                  float *geom_type) try {
  if (!H || !c || !c->d) return CVO_ERR_INVALID_ARG;
  if (!H->h.stream) return CVO_ERR_CUDA;
  return cloud_download(&H->h, c->d, xyz, features, labels, geom_type);
} catch (...) {
  return status_from_exception();
}

extern "C" int cvo_cloud_from_rgbd(cvo_handle *H, const uint8_t *image, int rows, int cols, int channels,
                                   const float *depth, const float intrinsic[4], float scaling_factor, const int *uv,
                                   int n_sel, const float *geom_type, int num_classes, const float *semantics,
                                   cvo_gpu_cloud **out, int *n_points) try {
  if (!H || !out) return CVO_ERR_INVALID_ARG;
  if (!H->h.stream) return CVO_ERR_CUDA;
  DevCloud *d = nullptr;
  int rc = cloud_from_rgbd(&H->h, image, rows, cols, channels, depth, intrinsic, scaling_factor, uv, n_sel, geom_type,
                           num_classes, semantics, &d);
  if (rc) {
    if (d) cloud_free(d);
    return rc;
  }
  *out = new cvo_gpu_cloud{d, H};
  if (n_points) *n_points = d->n;
  return CVO_OK;
} catch (...) {
  return status_from_exception();
}

namespace {

struct TmpClouds {
  cvo_handle *H;
  std::vector<cvo_gpu_cloud *> v;
  ~TmpClouds() { for (auto *c : v) cvo_cloud_free(H, c); }
};

void copy16(const float *a, float *b) { memcpy(b, a, 16 * sizeof(float)); }

// Column-major 4x4 inverse of a rigid transform (R^T, -R^T t), canonical order.
void rigid_inverse(const float *T, float *out) {
  float R[9], t[3];
  for (int r = 0; r < 3; r++) { for (int c = 0; c < 3; c++) R[3 * r + c] = T[c * 4 + r]; t[r] = T[12 + r]; }
  memset(out, 0, 16 * sizeof(float));
  for (int r = 0; r < 3; r++) {
    for (int c = 0; c < 3; c++) out[c * 4 + r] = R[3 * c + r];
    float a = R[r] * t[0], b = R[3 + r] * t[1], c2 = R[6 + r] * t[2];
    out[12 + r] = -((a + b) + c2);
  }
  out[15] = 1.f;
}

void fill_assoc(cvo_assoc *a, int rows, int cols, const std::vector<int> &rowptr, const std::vector<int> &col,
                const std::vector<float> &val) {
  a->rows = rows;
  a->cols = cols;
  a->row_ptr.assign(rowptr.begin(), rowptr.end());
  a->col = col;
  a->val = val;
  a->source_inliers.clear();
  a->target_inliers.clear();
  // gpu_association_to_cpu (src/cvo/CvoGPU_impl.cu:370-431): rows with any
  // pair are source inliers; every pair's column is appended to the target list
  for (int i = 0; i < rows; i++) {
    if (rowptr[i + 1] > rowptr[i]) a->source_inliers.push_back(i);
    for (int k = rowptr[i]; k < rowptr[i + 1]; k++) a->target_inliers.push_back(col[k]);
  }
}

}  // namespace

// ---------------------------------------------------------------- align
extern "C" int cvo_align_batch_dev(cvo_handle *H, int n_pairs, cvo_gpu_cloud *const *srcs, cvo_gpu_cloud *const *tgts,
                                   const float *T_init, float *T_out, int *rets, int *iters, double *secs) try {
  if (!H || n_pairs < 0 || (n_pairs > 0 && (!srcs || !tgts || !T_init || !T_out))) return CVO_ERR_INVALID_ARG;
  std::vector<DevCloud *> s, t;
  std::vector<float> Ti(T_init, T_init + 16 * (size_t)n_pairs);
  for (int p = 0; p < n_pairs; p++) {
    if (!srcs[p] || !tgts[p]) return CVO_ERR_INVALID_ARG;
    s.push_back(srcs[p]->d);
    t.push_back(tgts[p]->d);
  }
  BatchResult r;
  int rc = run_align_batch(&H->h, s, t, Ti, &r, secs, false, nullptr, nullptr, nullptr);
  if (rc) return rc;
  for (int p = 0; p < n_pairs; p++) {
    if (s[p]->n == 0 || t[p]->n == 0) {
      copy16(T_init + 16 * p, T_out + 16 * p);   // the reference leaves the output untouched
      if (rets) rets[p] = 0;
      if (iters) iters[p] = 0;
      continue;
    }
    copy16(&r.T_out[16 * p], T_out + 16 * p);
    if (rets) rets[p] = r.ret[p];
    if (iters) iters[p] = r.iters[p];
  }
  return CVO_OK;
} catch (...) {
  return status_from_exception();
}

static int nearest_init_pose_impl(cvo_handle *H, DevCloud *s, DevCloud *t, float ell, int num_guess, int grid_kind,
                                  float T_out[16], double *secs, std::vector<float> *cos_all);

static int align_dev_impl(cvo_handle *H, DevCloud *s, DevCloud *t, const float T_init[16], float T_out[16],
                          cvo_assoc *assoc, double *secs, int *iters, bool s2t) {
  if (s->n == 0 || t->n == 0) {
    if (secs) *secs = 0;
    if (iters) *iters = 0;
    return s2t ? CVO_ZERO_GRADIENT : CVO_OK;
  }
  float init[16];
  if (s2t) rigid_inverse(T_init, init);
  else copy16(T_init, init);
  double gsecs = 0;
  if (H->h.params.is_global_angle_registration > 0) {
    float g[16];
    int rc = nearest_init_pose_impl(H, s, t, H->h.params.ell_init_first_frame, H->h.params.is_global_angle_registration,
                                    0, g, &gsecs, nullptr);
    if (rc) return rc;
    // the int overload inverts the grid pose; the CvoResultInfo overload does not
    // (src/cvo/CvoGPU.cu:1533-1543 vs 1581-1587)
    if (s2t) copy16(g, init);
    else rigid_inverse(g, init);
  }
  BatchResult r;
  std::vector<float> Ti(init, init + 16);
  bool want = assoc && H->h.params.is_exporting_association;
  if (s2t && assoc) want = true;
  std::vector<std::vector<int>> ar, ac;
  std::vector<std::vector<float>> av;
  int rc = run_align_batch(&H->h, {s}, {t}, Ti, &r, secs, want, &ar, &ac, &av);
  if (rc) return rc;
  copy16(&r.T_out[0], T_out);
  if (iters) *iters = r.iters[0];
  if (secs) *secs += gsecs;
  if (want) fill_assoc(assoc, s->n, t->n, ar[0], ac[0], av[0]);
  return r.ret[0] == -1 ? CVO_ZERO_GRADIENT : CVO_OK;
}

extern "C" int cvo_align_dev(cvo_handle *H, cvo_gpu_cloud *src, cvo_gpu_cloud *tgt, const float T_init[16],
                             float T_out[16], cvo_assoc *assoc, double *secs, int *iters) try {
  if (!H || !src || !tgt || !T_init || !T_out) return CVO_ERR_INVALID_ARG;
  return align_dev_impl(H, src->d, tgt->d, T_init, T_out, assoc, secs, iters, false);
} catch (...) {
  return status_from_exception();
}

extern "C" int cvo_align(cvo_handle *H, const cvo_cloud *src, const cvo_cloud *tgt, const float T_init[16],
                         float T_out[16], cvo_assoc *assoc, double *secs, int *iters) try {
  if (!H || !src || !tgt || !T_init || !T_out) return CVO_ERR_INVALID_ARG;
  if (src->n == 0 || tgt->n == 0) { if (iters) *iters = 0; if (secs) *secs = 0; return CVO_OK; }
  TmpClouds tc{H, {}};
  cvo_gpu_cloud *s = nullptr, *t = nullptr;
  int rc = cvo_cloud_upload(H, src, &s);
  if (rc) return rc;
  tc.v.push_back(s);
  if ((rc = cvo_cloud_upload(H, tgt, &t))) return rc;
  tc.v.push_back(t);
  return align_dev_impl(H, s->d, t->d, T_init, T_out, assoc, secs, iters, false);
} catch (...) {
  return status_from_exception();
}

extern "C" int cvo_align_s2t(cvo_handle *H, const cvo_cloud *src, const cvo_cloud *tgt, const float T_s2t[16],
                             int want_assoc, float T_out[16], cvo_assoc *assoc, double *secs, int *iters,
                             int *ret_code) try {
  if (!H || !src || !tgt || !T_s2t || !T_out) return CVO_ERR_INVALID_ARG;
  if (src->n == 0 || tgt->n == 0) { if (ret_code) *ret_code = -1; return CVO_OK; }
  TmpClouds tc{H, {}};
  cvo_gpu_cloud *s = nullptr, *t = nullptr;
  int rc = cvo_cloud_upload(H, src, &s);
  if (rc) return rc;
  tc.v.push_back(s);
  if ((rc = cvo_cloud_upload(H, tgt, &t))) return rc;
  tc.v.push_back(t);
  rc = align_dev_impl(H, s->d, t->d, T_s2t, T_out, want_assoc ? assoc : nullptr, secs, iters, true);
  if (rc == CVO_ZERO_GRADIENT) { if (ret_code) *ret_code = -1; return CVO_OK; }
  if (rc == CVO_OK && ret_code) *ret_code = 0;
  return rc;
} catch (...) {
  return status_from_exception();
}

// ---------------------------------------------------------- inner products
static int ip_dev(cvo_handle *H, DevCloud *s, DevCloud *t, const float T[16], float ell, float *out) {
  if (s->n == 0 || t->n == 0) { *out = 0.f; return CVO_OK; }
  std::vector<double> asum;
  std::vector<long long> nnz;
  std::vector<float> Tv(T, T + 16);
  int rc = run_inner_product_batch(&H->h, s, t, Tv, ell, H->h.params.nearest_neighbors_max, &asum, &nnz, false,
                                   nullptr, nullptr, nullptr);
  if (rc) return rc;
  *out = (float)asum[0];
  return CVO_OK;
}

extern "C" int cvo_inner_product_dev(cvo_handle *H, cvo_gpu_cloud *src, cvo_gpu_cloud *tgt, const float T[16],
                                     float ell, float *out) try {
  if (!H || !src || !tgt || !T || !out) return CVO_ERR_INVALID_ARG;
  return ip_dev(H, src->d, tgt->d, T, ell, out);
} catch (...) {
  return status_from_exception();
}

extern "C" int cvo_inner_product(cvo_handle *H, const cvo_cloud *src, const cvo_cloud *tgt, const float T[16],
                                 float ell, float *out) try {
  if (!H || !src || !tgt || !T || !out) return CVO_ERR_INVALID_ARG;
  if (src->n == 0 || tgt->n == 0) { *out = 0.f; return CVO_OK; }
  TmpClouds tc{H, {}};
  cvo_gpu_cloud *s = nullptr, *t = nullptr;
  int rc = cvo_cloud_upload(H, src, &s);
  if (rc) return rc;
  tc.v.push_back(s);
  if ((rc = cvo_cloud_upload(H, tgt, &t))) return rc;
  tc.v.push_back(t);
  return ip_dev(H, s->d, t->d, T, ell, out);
} catch (...) {
  return status_from_exception();
}

extern "C" int cvo_inner_product_batch_dev(cvo_handle *H, cvo_gpu_cloud *src, cvo_gpu_cloud *tgt, int n_poses,
                                           const float *T, float ell, float *out) try {
  if (!H || !src || !tgt || n_poses < 0 || (n_poses > 0 && (!T || !out))) return CVO_ERR_INVALID_ARG;
  if (n_poses == 0) return CVO_OK;
  if (src->d->n == 0 || tgt->d->n == 0) { for (int i = 0; i < n_poses; i++) out[i] = 0.f; return CVO_OK; }
  std::vector<double> asum;
  std::vector<long long> nnz;
  std::vector<float> Tv(T, T + 16 * (size_t)n_poses);
  int rc = run_inner_product_batch(&H->h, src->d, tgt->d, Tv, ell, H->h.params.nearest_neighbors_max, &asum, &nnz,
                                   false, nullptr, nullptr, nullptr);
  if (rc) return rc;
  for (int i = 0; i < n_poses; i++) out[i] = (float)asum[i];
  return CVO_OK;
} catch (...) {
  return status_from_exception();
}

// CvoGPU::inner_product_cpu (src/cvo/CvoGPU.cpp:113-231) on the host: radius
// search (squared radius -2 l^2 ln(sp/sigma^2), strict <), no neighbour cap, no
// range-scaled ell; colour/semantic factors without thresholds.
extern "C" int cvo_inner_product_cpu(cvo_handle *H, const cvo_cloud *src, const cvo_cloud *tgt, const float T[16],
                                     float ell, float *out) try {
  if (!H || !src || !tgt || !T || !out) return CVO_ERR_INVALID_ARG;
  if (src->n == 0 || tgt->n == 0) { *out = 0.f; return CVO_OK; }
  if (src->F != tgt->F || src->C != tgt->C) return CVO_ERR_INVALID_ARG;
  const cvo_params &p = H->h.params;
  const int n = src->n, m = tgt->n, F = src->F, C = src->C;
  float Ri[9], Ti[3];
  {
    float R[9], t[3];
    for (int r = 0; r < 3; r++) { for (int c = 0; c < 3; c++) R[3 * r + c] = T[c * 4 + r]; t[r] = T[12 + r]; }
    for (int r = 0; r < 3; r++) for (int c = 0; c < 3; c++) Ri[3 * r + c] = R[3 * c + r];
    for (int r = 0; r < 3; r++) {
      float a = Ri[3 * r] * t[0], b = Ri[3 * r + 1] * t[1], c = Ri[3 * r + 2] * t[2];
      Ti[r] = -((a + b) + c);
    }
  }
  std::vector<float> y(3 * (size_t)m);
  for (int j = 0; j < m; j++) {
    const float *q = tgt->xyz + (size_t)j * tgt->xyz_stride;
    for (int r = 0; r < 3; r++) {
      float a = Ri[3 * r] * q[0], b = Ri[3 * r + 1] * q[1], c = Ri[3 * r + 2] * q[2];
      y[3 * j + r] = ((a + b) + c) + Ti[r];
    }
  }
  const float s2 = p.sigma * p.sigma;
  const float l = ell;
  const float d2_thres = (float)(-2.0 * (double)l * (double)l * (double)logf(p.sp_thres / s2));
  // uniform grid over the transformed targets, cell >= radius
  float h = std::sqrt(std::max(d2_thres, 0.f)) * 1.001f + 1e-6f;
  float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int j = 0; j < m; j++)
    for (int k = 0; k < 3; k++) { mn[k] = std::min(mn[k], y[3 * j + k]); mx[k] = std::max(mx[k], y[3 * j + k]); }
  float ext = std::max(std::max(mx[0] - mn[0], mx[1] - mn[1]), mx[2] - mn[2]);
  if (ext / h > 1.0e6f) h = ext / 1.0e6f;
  auto key_of = [&](float a, float b, float c) -> int64_t {
    int64_t cx = (int64_t)std::floor((a - mn[0]) / h) + (1 << 20);
    int64_t cy = (int64_t)std::floor((b - mn[1]) / h) + (1 << 20);
    int64_t cz = (int64_t)std::floor((c - mn[2]) / h) + (1 << 20);
    return (cx << 42) | (cy << 21) | cz;
  };
  std::vector<std::pair<int64_t, int>> ent(m);
  for (int j = 0; j < m; j++) ent[j] = {key_of(y[3 * j], y[3 * j + 1], y[3 * j + 2]), j};
  std::sort(ent.begin(), ent.end());
  std::vector<double> rows(n, 0.0);
#pragma omp parallel for schedule(dynamic, 64)
  for (int i = 0; i < n; i++) {
    const float *x = src->xyz + (size_t)i * src->xyz_stride;
    int64_t cx = (int64_t)std::floor((x[0] - mn[0]) / h), cy = (int64_t)std::floor((x[1] - mn[1]) / h),
            cz = (int64_t)std::floor((x[2] - mn[2]) / h);
    double r = 0.0;
    for (int dx = -1; dx <= 1; dx++)
      for (int dy = -1; dy <= 1; dy++)
        for (int dz = -1; dz <= 1; dz++) {
          int64_t key = ((cx + dx + (1 << 20)) << 42) | ((cy + dy + (1 << 20)) << 21) | (cz + dz + (1 << 20));
          auto it = std::lower_bound(ent.begin(), ent.end(), std::make_pair(key, -1));
          for (; it != ent.end() && it->first == key; ++it) {
            int j = it->second;
            const float *q = &y[3 * (size_t)j];
            float ddx = x[0] - q[0], ddy = x[1] - q[1], ddz = x[2] - q[2];
            float d2 = ddx * ddx;
            d2 += ddy * ddy;
            d2 += ddz * ddz;
            if (!(d2 < d2_thres)) continue;
            float kk = 1.f, ck = 1.f, sk = 1.f;
            if (p.is_using_semantics) {
              float d2s = 0.f;
              for (int c = 0; c < C; c++) { float tt = src->labels[(size_t)i * C + c] - tgt->labels[(size_t)j * C + c]; d2s += tt * tt; }
              sk = (float)((double)(p.s_sigma * p.s_sigma) * exp(-(double)d2s / (2.0 * (double)p.s_ell * (double)p.s_ell)));
            }
            if (p.is_using_geometry) kk = (float)((double)s2 * exp(-(double)d2 / (2.0 * (double)l * (double)l)));
            if (p.is_using_intensity) {
              float d2c = 0.f;
              for (int c = 0; c < F; c++) { float tt = src->features[(size_t)i * F + c] - tgt->features[(size_t)j * F + c]; d2c += tt * tt; }
              ck = (float)((double)(p.c_sigma * p.c_sigma) * exp(-(double)d2c / (2.0 * (double)p.c_ell * (double)p.c_ell)));
            }
            float a = ck * kk * sk;
            if (a > p.sp_thres) r += a;
          }
        }
    rows[i] = r;
  }
  double tot = 0.0;
  for (int i = 0; i < n; i++) tot += rows[i];
  *out = (float)tot;
  return CVO_OK;
} catch (...) {
  return status_from_exception();
}

extern "C" int cvo_function_angle(cvo_handle *H, const cvo_cloud *src, const cvo_cloud *tgt, const float T[16],
                                  float ell, int is_approximate, int is_gpu, float *out) try {
  if (!H || !src || !tgt || !T || !out) return CVO_ERR_INVALID_ARG;
  if (src->n == 0 || tgt->n == 0) { *out = 0.f; return CVO_OK; }
  float I[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
  float fxfz = 0.f, fx = 0.f, fz = 0.f;
  int rc;
  if (is_gpu) {
    TmpClouds tc{H, {}};
    cvo_gpu_cloud *s = nullptr, *t = nullptr;
    if ((rc = cvo_cloud_upload(H, src, &s))) return rc;
    tc.v.push_back(s);
    if ((rc = cvo_cloud_upload(H, tgt, &t))) return rc;
    tc.v.push_back(t);
    if ((rc = ip_dev(H, s->d, t->d, T, ell, &fxfz))) return rc;
    if (is_approximate) {
      fx = (float)std::sqrt((double)src->n);
      fz = (float)std::sqrt((double)tgt->n);
    } else {
      float a, b;
      if ((rc = ip_dev(H, s->d, s->d, I, ell, &a))) return rc;
      if ((rc = ip_dev(H, t->d, t->d, I, ell, &b))) return rc;
      fx = std::sqrt(a);
      fz = std::sqrt(b);
    }
  } else {
    if ((rc = cvo_inner_product_cpu(H, src, tgt, T, ell, &fxfz))) return rc;
    if (is_approximate) {
      fx = (float)std::sqrt((double)src->n);
      fz = (float)std::sqrt((double)tgt->n);
    } else {
      float a, b;
      if ((rc = cvo_inner_product_cpu(H, src, src, I, ell, &a))) return rc;
      if ((rc = cvo_inner_product_cpu(H, tgt, tgt, I, ell, &b))) return rc;
      fx = std::sqrt(a);
      fz = std::sqrt(b);
    }
  }
  *out = fxfz / (fx * fz);
  return CVO_OK;
} catch (...) {
  return status_from_exception();
}

// -------------------------------------------------------------- association
extern "C" int cvo_assoc_create(cvo_assoc **out) try {
  if (!out) return CVO_ERR_INVALID_ARG;
  *out = new cvo_assoc();
  return CVO_OK;
} catch (...) {
  return status_from_exception();
}
extern "C" int cvo_assoc_destroy(cvo_assoc *a) try {
  delete a;
  return CVO_OK;
} catch (...) {
  return status_from_exception();
}
extern "C" int cvo_assoc_info(const cvo_assoc *a, int *rows, int *cols, int64_t *nnz, int64_t *ns, int64_t *nt) try {
  if (!a) return CVO_ERR_INVALID_ARG;
  if (rows) *rows = a->rows;
  if (cols) *cols = a->cols;
  if (nnz) *nnz = (int64_t)a->col.size();
  if (ns) *ns = (int64_t)a->source_inliers.size();
  if (nt) *nt = (int64_t)a->target_inliers.size();
  return CVO_OK;
} catch (...) {
  return status_from_exception();
}
extern "C" int cvo_assoc_copy(const cvo_assoc *a, int64_t *row_ptr, int *col, float *val, int *si, int *ti) try {
  if (!a) return CVO_ERR_INVALID_ARG;
  if (row_ptr && !a->row_ptr.empty()) memcpy(row_ptr, a->row_ptr.data(), sizeof(int64_t) * a->row_ptr.size());
  if (row_ptr && a->row_ptr.empty()) row_ptr[0] = 0;
  if (col && !a->col.empty()) memcpy(col, a->col.data(), sizeof(int) * a->col.size());
  if (val && !a->val.empty()) memcpy(val, a->val.data(), sizeof(float) * a->val.size());
  if (si && !a->source_inliers.empty()) memcpy(si, a->source_inliers.data(), sizeof(int) * a->source_inliers.size());
  if (ti && !a->target_inliers.empty()) memcpy(ti, a->target_inliers.data(), sizeof(int) * a->target_inliers.size());
  return CVO_OK;
} catch (...) {
  return status_from_exception();
}

extern "C" int cvo_compute_association(cvo_handle *H, const cvo_cloud *src, const cvo_cloud *tgt, const float T[16],
                                       float ell, cvo_assoc *out) try {
  if (!H || !src || !tgt || !T || !out) return CVO_ERR_INVALID_ARG;
  if (src->n == 0 || tgt->n == 0) { out->rows = src->n; out->cols = tgt->n; return CVO_OK; }
  TmpClouds tc{H, {}};
  cvo_gpu_cloud *s = nullptr, *t = nullptr;
  int rc = cvo_cloud_upload(H, src, &s);
  if (rc) return rc;
  tc.v.push_back(s);
  if ((rc = cvo_cloud_upload(H, tgt, &t))) return rc;
  tc.v.push_back(t);
  std::vector<double> asum;
  std::vector<long long> nnz;
  std::vector<int> rowptr, col;
  std::vector<float> val;
  std::vector<float> Tv(T, T + 16);
  rc = run_inner_product_batch(&H->h, s->d, t->d, Tv, ell, H->h.params.nearest_neighbors_max, &asum, &nnz, true,
                               &rowptr, &col, &val);
  if (rc) return rc;
  fill_assoc(out, src->n, tgt->n, rowptr, col, val);
  return CVO_OK;
} catch (...) {
  return status_from_exception();
}

extern "C" int cvo_compute_association_aniso_dev(cvo_handle *H, const cvo_gpu_cloud *src, const cvo_gpu_cloud *tgt,
                                                 const float T[16], const float kernel[9], cvo_assoc *out) try {
  if (!H || !src || !tgt || !T || !kernel || !out) return CVO_ERR_INVALID_ARG;
  if (!H->h.stream) return CVO_ERR_CUDA;
  std::vector<int> rowptr, col;
  std::vector<float> val;
  int rc = run_association_aniso(&H->h, src->d, tgt->d, T, kernel, H->h.params.nearest_neighbors_max, &rowptr, &col,
                                 &val);
  if (rc) return rc;
  fill_assoc(out, src->d->n, tgt->d->n, rowptr, col, val);
  return CVO_OK;
} catch (...) {
  return status_from_exception();
}

extern "C" int cvo_compute_association_aniso(cvo_handle *H, const cvo_cloud *src, const cvo_cloud *tgt,
                                             const float T[16], const float kernel[9], cvo_assoc *out) try {
  if (!H || !src || !tgt || !T || !kernel || !out) return CVO_ERR_INVALID_ARG;
  // compute_association_gpu returns without output for an empty cloud (CvoGPU.cu:1942-1943)
  if (src->n == 0 || tgt->n == 0) { out->rows = src->n; out->cols = tgt->n; return CVO_OK; }
  TmpClouds tc{H, {}};
  cvo_gpu_cloud *s = nullptr, *t = nullptr;
  int rc = cvo_cloud_upload(H, src, &s);
  if (rc) return rc;
  tc.v.push_back(s);
  if ((rc = cvo_cloud_upload(H, tgt, &t))) return rc;
  tc.v.push_back(t);
  return cvo_compute_association_aniso_dev(H, s, t, T, kernel, out);
} catch (...) {
  return status_from_exception();
}

// ------------------------------------------------------------ rotation grids
namespace {

void mat_mul3(const double *a, const double *b, double *c) {
  for (int r = 0; r < 3; r++)
    for (int k = 0; k < 3; k++) c[3 * r + k] = a[3 * r] * b[k] + a[3 * r + 1] * b[3 + k] + a[3 * r + 2] * b[6 + k];
}

void axis_angle(double ax, double ay, double az, double ang, double *R) {
  double n = std::sqrt(ax * ax + ay * ay + az * az);
  ax /= n; ay /= n; az /= n;
  double c = std::cos(ang), s = std::sin(ang), t = 1 - c;
  double M[9] = {t * ax * ax + c, t * ax * ay - s * az, t * ax * az + s * ay,
                 t * ax * ay + s * az, t * ay * ay + c, t * ay * az - s * ax,
                 t * ax * az - s * ay, t * ay * az + s * ax, t * az * az + c};
  memcpy(R, M, sizeof(M));
}

// Closure of a set of generator rotations (the finite group they generate).
std::vector<std::vector<double>> closure(const std::vector<std::vector<double>> &gens) {
  std::vector<std::vector<double>> G = {{1, 0, 0, 0, 1, 0, 0, 0, 1}};
  for (size_t i = 0; i < G.size(); i++)
    for (const auto &g : gens) {
      std::vector<double> m(9);
      mat_mul3(G[i].data(), g.data(), m.data());
      bool seen = false;
      for (const auto &x : G) {
        double d = 0;
        for (int k = 0; k < 9; k++) d = std::max(d, std::fabs(x[k] - m[k]));
        if (d < 1e-9) { seen = true; break; }
      }
      if (!seen) G.push_back(m);
      if (G.size() > 200) return G;
    }
  std::sort(G.begin(), G.end(), [](const std::vector<double> &a, const std::vector<double> &b) {
    for (int k = 0; k < 9; k++) {
      double x = std::round(a[k] * 1e6), y = std::round(b[k] * 1e6);
      if (x != y) return x > y;
    }
    return false;
  });
  return G;
}

std::vector<float> rotation_grid(int kind, int num_guess) {
  std::vector<float> out;
  if (kind == 0) {
    // rotation group of the icosahedron: a 3-fold axis along x, 2-fold axes along
    // y and along (phi^2, 0, 1); the same 60 rotations as gen_icosahedron_init_rots
    // (src/cvo/CvoGPU.cpp:279-342), regenerated from the symmetry.
    const double phi = (1.0 + std::sqrt(5.0)) / 2.0;
    std::vector<double> g1(9), g2(9), g3(9);
    axis_angle(1, 0, 0, 2.0 * M_PI / 3.0, g1.data());
    axis_angle(0, 1, 0, M_PI, g2.data());
    axis_angle(phi * phi, 0, 1, M_PI, g3.data());
    for (auto &m : closure({g1, g2, g3})) for (double v : m) out.push_back((float)v);
  } else if (kind == 1) {
    // rotation group of the cube (24 signed permutation matrices with det +1)
    std::vector<double> g1(9), g2(9);
    axis_angle(0, 0, 1, M_PI / 2.0, g1.data());
    axis_angle(1, 1, 1, 2.0 * M_PI / 3.0, g2.data());
    for (auto &m : closure({g1, g2})) for (double v : m) out.push_back((float)std::round(v));
  } else if (kind == 2) {
    // gen_rand_init_pose (src/cvo/CvoGPU.cpp:344-363): Rx(i/n pi) Ry(j/n pi) Rz(k/n pi), float
    int n = std::max(num_guess, 1);
    for (int i = 0; i < n; i++)
      for (int j = 0; j < n; j++)
        for (int k = 0; k < n; k++) {
          auto rot = [](int axis, float a, float *R) {
            float c = std::cos(a), s = std::sin(a);
            for (int t = 0; t < 9; t++) R[t] = 0.f;
            if (axis == 0) { R[0] = 1; R[4] = c; R[5] = -s; R[7] = s; R[8] = c; }
            if (axis == 1) { R[4] = 1; R[0] = c; R[2] = s; R[6] = -s; R[8] = c; }
            if (axis == 2) { R[8] = 1; R[0] = c; R[1] = -s; R[3] = s; R[4] = c; }
          };
          float A[9], B[9], Cm[9], AB[9], R[9];
          rot(0, (float)(i / (float)n * M_PI), A);
          rot(1, (float)(j / (float)n * M_PI), B);
          rot(2, (float)(k / (float)n * M_PI), Cm);
          for (int r = 0; r < 3; r++)
            for (int c = 0; c < 3; c++) AB[3 * r + c] = A[3 * r] * B[c] + A[3 * r + 1] * B[3 + c] + A[3 * r + 2] * B[6 + c];
          for (int r = 0; r < 3; r++)
            for (int c = 0; c < 3; c++) R[3 * r + c] = AB[3 * r] * Cm[c] + AB[3 * r + 1] * Cm[3 + c] + AB[3 * r + 2] * Cm[6 + c];
          for (int t = 0; t < 9; t++) out.push_back(R[t]);
        }
  }
  return out;
}

}  // namespace

extern "C" int cvo_rotation_grid(int grid_kind, int num_guess, float *rots, int max_rots) try {
  if (grid_kind < 0 || grid_kind > 2) return CVO_ERR_INVALID_ARG;
  std::vector<float> g = rotation_grid(grid_kind, num_guess);
  int cnt = (int)(g.size() / 9);
  if (rots) {
    int k = std::min(cnt, std::max(max_rots, 0));
    memcpy(rots, g.data(), sizeof(float) * 9 * (size_t)k);
  }
  return cnt;
} catch (...) {
  return status_from_exception();
}

// get_nearest_init_pose (src/cvo/CvoGPU.cpp:367-398): every grid rotation's
// cos-angle in one batched launch, then the argmax (strictly greater, from 0).
static int nearest_init_pose_impl(cvo_handle *H, DevCloud *s, DevCloud *t, float ell, int num_guess, int grid_kind,
                                  float T_out[16], double *secs, std::vector<float> *cos_all) {
  auto t0 = std::chrono::steady_clock::now();
  std::vector<float> rots = rotation_grid(grid_kind, num_guess);
  int nr = (int)(rots.size() / 9);
  std::vector<float> T(16 * (size_t)nr, 0.f);
  for (int r = 0; r < nr; r++) {
    float *M = &T[16 * r];
    for (int a = 0; a < 3; a++)
      for (int b = 0; b < 3; b++) M[b * 4 + a] = rots[9 * r + 3 * b + a];   // [rot^T | 0]
    M[15] = 1.f;
  }
  for (int k = 0; k < 16; k++) T_out[k] = (k % 5 == 0) ? 1.f : 0.f;
  if (s->n == 0 || t->n == 0) return CVO_OK;
  std::vector<double> asum;
  std::vector<long long> nnz;
  int rc = run_inner_product_batch(&H->h, s, t, T, ell, H->h.params.nearest_neighbors_max, &asum, &nnz, false,
                                   nullptr, nullptr, nullptr);
  if (rc) return rc;
  float fx = (float)std::sqrt((double)s->n), fz = (float)std::sqrt((double)t->n);
  float best = 0.f;
  int bi = -1;
  if (cos_all) cos_all->assign(nr, 0.f);
  for (int r = 0; r < nr; r++) {
    float c = (float)asum[r] / (fx * fz);
    if (cos_all) (*cos_all)[r] = c;
    if (c > best) { best = c; bi = r; }
  }
  if (bi >= 0)
    for (int a = 0; a < 3; a++)
      for (int b = 0; b < 3; b++) T_out[b * 4 + a] = rots[9 * bi + 3 * a + b];
  auto t1 = std::chrono::steady_clock::now();
  if (secs) *secs += std::chrono::duration<double>(t1 - t0).count();
  return CVO_OK;
}

extern "C" int cvo_get_nearest_init_pose_dev(cvo_handle *H, cvo_gpu_cloud *src, cvo_gpu_cloud *tgt, float ell,
                                             int num_guess, int grid_kind, float T_out[16], double *secs) try {
  if (!H || !src || !tgt || !T_out || grid_kind < 0 || grid_kind > 2) return CVO_ERR_INVALID_ARG;
  if (secs) *secs = 0;
  return nearest_init_pose_impl(H, src->d, tgt->d, ell, num_guess, grid_kind, T_out, secs, nullptr);
} catch (...) {
  return status_from_exception();
}

extern "C" int cvo_get_nearest_init_pose(cvo_handle *H, const cvo_cloud *src, const cvo_cloud *tgt, float ell,
                                         int num_guess, int grid_kind, float T_out[16], double *secs) try {
  if (!H || !src || !tgt || !T_out || grid_kind < 0 || grid_kind > 2) return CVO_ERR_INVALID_ARG;
  if (secs) *secs = 0;
  if (src->n == 0 || tgt->n == 0) { for (int k = 0; k < 16; k++) T_out[k] = (k % 5 == 0) ? 1.f : 0.f; return CVO_OK; }
  TmpClouds tc{H, {}};
  cvo_gpu_cloud *s = nullptr, *t = nullptr;
  int rc = cvo_cloud_upload(H, src, &s);
  if (rc) return rc;
  tc.v.push_back(s);
  if ((rc = cvo_cloud_upload(H, tgt, &t))) return rc;
  tc.v.push_back(t);
  return nearest_init_pose_impl(H, s->d, t->d, ell, num_guess, grid_kind, T_out, secs, nullptr);
} catch (...) {
  return status_from_exception();
}

// Batched refinement of pose hypotheses, judged by the final approximate cos-angle.
extern "C" int cvo_register_hypotheses_dev(cvo_handle *H, cvo_gpu_cloud *src, cvo_gpu_cloud *tgt, int n_hyp,
                                           const float *T_init, float judge_ell, float T_out[16], int *best,
                                           float *cos_out, double *secs) try {
  if (!H || !src || !tgt || n_hyp <= 0 || !T_init || !T_out) return CVO_ERR_INVALID_ARG;
  auto t0 = std::chrono::steady_clock::now();
  std::vector<DevCloud *> s(n_hyp, src->d), t(n_hyp, tgt->d);
  std::vector<float> Ti(T_init, T_init + 16 * (size_t)n_hyp);
  BatchResult r;
  int rc = run_align_batch(&H->h, s, t, Ti, &r, nullptr, false, nullptr, nullptr, nullptr);
  if (rc) return rc;
  // judge: inner product with the internal pose (target moved by its inverse)
  std::vector<float> Tj(16 * (size_t)n_hyp);
  for (int p = 0; p < n_hyp; p++) rigid_inverse(&r.T_out[16 * p], &Tj[16 * p]);
  std::vector<double> asum;
  std::vector<long long> nnz;
  if ((rc = run_inner_product_batch(&H->h, src->d, tgt->d, Tj, judge_ell, H->h.params.nearest_neighbors_max, &asum,
                                    &nnz, false, nullptr, nullptr, nullptr)))
    return rc;
  float fx = (float)std::sqrt((double)src->d->n), fz = (float)std::sqrt((double)tgt->d->n);
  int bi = 0;
  float bc = -INFINITY;
  for (int p = 0; p < n_hyp; p++) {
    float c = (float)asum[p] / (fx * fz);
    if (cos_out) cos_out[p] = c;
    if (c > bc) { bc = c; bi = p; }
  }
  copy16(&r.T_out[16 * bi], T_out);
  if (best) *best = bi;
  auto t1 = std::chrono::steady_clock::now();
  if (secs) *secs = std::chrono::duration<double>(t1 - t0).count();
  return CVO_OK;
} catch (...) {
  return status_from_exception();
}

// ------------------------------------------------------------ autotuner
extern "C" int cvo_autotune_launch_dev(cvo_handle *H, cvo_gpu_cloud *src, cvo_gpu_cloud *tgt, const float T[16],
                                       float ell, int reps, int max_configs, int *n_configs, float *div_r,
                                       float *div_ext, int *blocks_per_sm, float *ms, int *best) try {
  if (!H || !src || !tgt || !T || max_configs < 0) return CVO_ERR_INVALID_ARG;
  if (!(ell > 0.f)) ell = H->h.params.ell_init;
  std::vector<TuneConfig> cfg;
  std::vector<float> t;
  int bi = 0;
  int rc = autotune_association(&H->h, src->d, tgt->d, T, ell, reps, &cfg, &t, &bi);
  if (rc) return rc;
  if (n_configs) *n_configs = (int)cfg.size();
  for (int k = 0; k < (int)cfg.size() && k < max_configs; k++) {
    if (div_r) div_r[k] = cfg[k].cell_div_r;
    if (div_ext) div_ext[k] = cfg[k].cell_div_ext;
    if (blocks_per_sm) blocks_per_sm[k] = cfg[k].blocks_per_sm;
    if (ms) ms[k] = t[k];
  }
  if (best) *best = bi;
  return CVO_OK;
} catch (...) {
  return status_from_exception();
}

extern "C" int cvo_autotune_dev(cvo_handle *H, cvo_gpu_cloud *src, cvo_gpu_cloud *tgt, const float T[16], float ell,
                                int reps, int max_configs, int *n_configs, float *div_r, float *div_ext, float *ms,
                                int *best) try {
  if (!H || !src || !tgt || !T || max_configs < 0) return CVO_ERR_INVALID_ARG;
  if (!(ell > 0.f)) ell = H->h.params.ell_init;
  std::vector<TuneConfig> cfg;
  std::vector<float> t;
  int bi = 0;
  int rc = autotune_association(&H->h, src->d, tgt->d, T, ell, reps, &cfg, &t, &bi);
  if (rc) return rc;
  if (n_configs) *n_configs = (int)cfg.size();
  for (int k = 0; k < (int)cfg.size() && k < max_configs; k++) {
    if (div_r) div_r[k] = cfg[k].cell_div_r;
    if (div_ext) div_ext[k] = cfg[k].cell_div_ext;
    if (ms) ms[k] = t[k];
  }
  if (best) *best = bi;
  return CVO_OK;
} catch (...) {
  return status_from_exception();
}

extern "C" int cvo_tune_set(cvo_handle *H, int F, int C, int64_t rows, float div_r, float div_ext) try {
  if (!H || F < 0 || C < 0 || rows < 0 || !(div_r > 0.f) || !(div_ext > 0.f)) return CVO_ERR_INVALID_ARG;
  TuneConfig c;
  c.cell_div_r = div_r;
  c.cell_div_ext = div_ext;
  H->h.tuned[tune_key(F, C, rows)] = c;
  return CVO_OK;
} catch (...) {
  return status_from_exception();
}

extern "C" int cvo_tune_set_launch(cvo_handle *H, int F, int C, int64_t rows, float div_r, float div_ext,
                                   int blocks_per_sm) try {
  if (!H || F < 0 || C < 0 || rows < 0 || !(div_r > 0.f) || !(div_ext > 0.f) || blocks_per_sm < 0)
    return CVO_ERR_INVALID_ARG;
  TuneConfig c;
  c.cell_div_r = div_r;
  c.cell_div_ext = div_ext;
  H->h.tuned[tune_key(F, C, rows)] = c;
  H->h.tuned_bps[tune_key(F, C, tune_items(rows))] = blocks_per_sm;
  return CVO_OK;
} catch (...) {
  return status_from_exception();
}

extern "C" int cvo_tune_get_launch(const cvo_handle *H, int F, int C, int64_t rows, float *div_r, float *div_ext,
                                   int *blocks_per_sm) try {
  if (!H || !div_r || !div_ext || !blocks_per_sm) return CVO_ERR_INVALID_ARG;
  TuneConfig c;
  auto it = H->h.tuned.find(tune_key(F, C, rows));
  if (it != H->h.tuned.end()) c = it->second;
  *div_r = c.cell_div_r;
  *div_ext = c.cell_div_ext;
  auto ib = H->h.tuned_bps.find(tune_key(F, C, tune_items(rows)));
  *blocks_per_sm = ib != H->h.tuned_bps.end() ? ib->second : 0;
  return it != H->h.tuned.end() ? CVO_OK : CVO_ERR_INVALID_ARG;
} catch (...) {
  return status_from_exception();
}

extern "C" int cvo_tune_get(const cvo_handle *H, int F, int C, int64_t rows, float *div_r, float *div_ext) try {
  if (!H || !div_r || !div_ext) return CVO_ERR_INVALID_ARG;
  TuneConfig c;
  auto it = H->h.tuned.find(tune_key(F, C, rows));
  if (it != H->h.tuned.end()) c = it->second;
  *div_r = c.cell_div_r;
  *div_ext = c.cell_div_ext;
  return it != H->h.tuned.end() ? CVO_OK : CVO_ERR_INVALID_ARG;
} catch (...) {
  return status_from_exception();
}

// ----------------------------------------------------- adaptive-ell CVO
extern "C" int cvo_align_adaptive_dev(cvo_handle *H, cvo_gpu_cloud *src, cvo_gpu_cloud *tgt, const float T_init[16],
                                      float T_out[16], double *secs, int *iters, double *trace, int trace_len) try {
  if (!H || !src || !tgt || !T_init || !T_out || trace_len < 0 || (trace_len > 0 && !trace)) return CVO_ERR_INVALID_ARG;
  if (src->d->n == 0 || tgt->d->n == 0) {
    if (iters) *iters = 0;
    if (secs) *secs = 0;
    return CVO_ERR_EMPTY_CLOUD;
  }
  return run_align_adaptive(&H->h, src->d, tgt->d, T_init, T_out, secs, iters, trace, trace_len);
} catch (...) {
  return status_from_exception();
}

extern "C" int cvo_align_adaptive(cvo_handle *H, const cvo_cloud *src, const cvo_cloud *tgt, const float T_init[16],
                                  float T_out[16], double *secs, int *iters) try {
  if (!H || !src || !tgt || !T_init || !T_out) return CVO_ERR_INVALID_ARG;
  if (src->n == 0 || tgt->n == 0) {
    if (iters) *iters = 0;
    if (secs) *secs = 0;
    return CVO_ERR_EMPTY_CLOUD;
  }
  TmpClouds tc{H, {}};
  cvo_gpu_cloud *s = nullptr, *t = nullptr;
  int rc = cvo_cloud_upload(H, src, &s);
  if (rc) return rc;
  tc.v.push_back(s);
  if ((rc = cvo_cloud_upload(H, tgt, &t))) return rc;
  tc.v.push_back(t);
  return run_align_adaptive(&H->h, s->d, t->d, T_init, T_out, secs, iters, nullptr, 0);
} catch (...) {
  return status_from_exception();
}

extern "C" int cvo_compute_association_adaptive(cvo_handle *H, const cvo_cloud *src, const cvo_cloud *tgt,
                                                const float T[16], float ell, cvo_assoc *out) try {
  if (!H || !src || !tgt || !T || !out) return CVO_ERR_INVALID_ARG;
  if (src->n == 0 || tgt->n == 0) {
    fill_assoc(out, src->n, tgt->n, std::vector<int>((size_t)src->n + 1, 0), {}, {});
    return CVO_OK;
  }
  TmpClouds tc{H, {}};
  cvo_gpu_cloud *s = nullptr, *t = nullptr;
  int rc = cvo_cloud_upload(H, src, &s);
  if (rc) return rc;
  tc.v.push_back(s);
  if ((rc = cvo_cloud_upload(H, tgt, &t))) return rc;
  tc.v.push_back(t);
  std::vector<int> rp, col;
  std::vector<float> val;
  if ((rc = run_association_adaptive(&H->h, s->d, t->d, T, ell, &rp, &col, &val))) return rc;
  fill_assoc(out, src->n, tgt->n, rp, col, val);
  return CVO_OK;
} catch (...) {
  return status_from_exception();
}

// ------------------------------------------------------ learned proposal
struct cvo_proposal { NetDev *n; };

extern "C" int cvo_proposal_create(cvo_handle *H, int points_per_cloud, uint32_t seed, cvo_proposal **out) try {
  if (!H || !out || points_per_cloud < 1 || points_per_cloud > 65536) return CVO_ERR_INVALID_ARG;
  NetDev *n = nullptr;
  int rc = net_create(&H->h, points_per_cloud, seed, &n);
  if (rc) return rc;
  *out = new cvo_proposal{n};
  return CVO_OK;
} catch (...) {
  return status_from_exception();
}

extern "C" int cvo_proposal_destroy(cvo_proposal *p) try {
  if (!p) return CVO_OK;
  net_destroy(p->n);
  delete p;
  return CVO_OK;
} catch (...) {
  return status_from_exception();
}

extern "C" int cvo_proposal_dims(const cvo_proposal *p, int *num_params, int *points_per_cloud, int *num_hyp) try {
  if (num_params) *num_params = (int)net_num_params();
  if (points_per_cloud) *points_per_cloud = p ? net_points(p->n) : 0;
  if (num_hyp) *num_hyp = 8;
  return CVO_OK;
} catch (...) {
  return status_from_exception();
}

extern "C" int cvo_proposal_get(cvo_handle *H, cvo_proposal *p, int which, float *out) try {
  if (!H || !p || !out) return CVO_ERR_INVALID_ARG;
  return net_get(&H->h, p->n, which, out);
} catch (...) {
  return status_from_exception();
}

extern "C" int cvo_proposal_set(cvo_handle *H, cvo_proposal *p, const float *weights) try {
  if (!H || !p || !weights) return CVO_ERR_INVALID_ARG;
  return net_set(&H->h, p->n, weights);
} catch (...) {
  return status_from_exception();
}

extern "C" int cvo_proposal_set_gemm(cvo_proposal *p, int kind) try {
  if (!p) return CVO_ERR_INVALID_ARG;
  return net_set_gemm(p->n, kind);
} catch (...) {
  return status_from_exception();
}

extern "C" int cvo_proposal_train_pool_dev(cvo_handle *H, cvo_proposal *p, int n_scenes, int n_pts,
                                           const float *src_pts, const float *tgt_pts, int n_pairs, const int *scene,
                                           const float *T_label, float lr, uint32_t seed, float *loss) try {
  if (!H || !p) return CVO_ERR_INVALID_ARG;
  return net_train_pool(&H->h, p->n, n_scenes, n_pts, src_pts, tgt_pts, n_pairs, scene, T_label, lr, seed, loss);
} catch (...) {
  return status_from_exception();
}

extern "C" int cvo_proposal_forward_pool_dev(cvo_handle *H, cvo_proposal *p, int n_scenes, int n_pts,
                                             const float *src_pts, const float *tgt_pts, int n_pairs,
                                             const int *scene, const float *T_tgt, uint32_t seed, float *raw_out,
                                             float *T_out) try {
  if (!H || !p) return CVO_ERR_INVALID_ARG;
  return net_forward_pool(&H->h, p->n, n_scenes, n_pts, src_pts, tgt_pts, n_pairs, scene, T_tgt, seed, raw_out,
                          T_out);
} catch (...) {
  return status_from_exception();
}

static int collect_clouds(int n, cvo_gpu_cloud *const *a, std::vector<DevCloud *> *out) {
  out->resize(n);
  for (int i = 0; i < n; i++) {
    if (!a[i]) return CVO_ERR_INVALID_ARG;
    (*out)[i] = a[i]->d;
  }
  return 0;
}

extern "C" int cvo_proposal_hypotheses_dev(cvo_handle *H, cvo_proposal *p, int n_pairs, cvo_gpu_cloud *const *srcs,
                                           cvo_gpu_cloud *const *tgts, uint32_t seed, float *T_out) try {
  if (!H || !p || n_pairs <= 0 || !srcs || !tgts || !T_out) return CVO_ERR_INVALID_ARG;
  std::vector<DevCloud *> s, t;
  int rc;
  if ((rc = collect_clouds(n_pairs, srcs, &s)) || (rc = collect_clouds(n_pairs, tgts, &t))) return rc;
  return net_hypotheses(&H->h, p->n, n_pairs, s.data(), t.data(), seed, T_out);
} catch (...) {
  return status_from_exception();
}

// Global registration of n_pairs pairs from the network's hypotheses: every pair's
// K hypotheses are ranked by the approximate cos-angle at rank_ell (one batch for
// all pairs), the best n_refine of each pair are refined by one batched align, and
// the final cos-angle at judge_ell picks each pair's result.  A pair whose best
// judged cos-angle stays below fallback_cos is registered again from the 24-rotation
// grid (nearest grid rotation + align, judged the same way) and keeps the better of
// the two.
extern "C" int cvo_register_learned_batch_dev(cvo_handle *H, cvo_proposal *p, int n_pairs,
                                              cvo_gpu_cloud *const *srcs, cvo_gpu_cloud *const *tgts, int n_refine,
                                              float rank_ell, float judge_ell, float fallback_cos, float refine_ell,
                                              uint32_t seed, float *T_out, float *cos_out, int *used_fallback,
                                              int *iters, double *secs) try {
  constexpr int kHyp = 8;
  if (!H || !p || n_pairs <= 0 || !srcs || !tgts || !T_out || n_refine < 1 || n_refine > kHyp)
    return CVO_ERR_INVALID_ARG;
  auto t0 = std::chrono::steady_clock::now();
  Handle *h = &H->h;
  std::vector<DevCloud *> s, t;
  int rc;
  if ((rc = collect_clouds(n_pairs, srcs, &s)) || (rc = collect_clouds(n_pairs, tgts, &t))) return rc;
  for (int b = 0; b < n_pairs; b++)
    if (s[b]->n == 0 || t[b]->n == 0) return CVO_ERR_EMPTY_CLOUD;
  std::vector<float> hyp(16 * (size_t)n_pairs * kHyp);
  if ((rc = net_hypotheses(h, p->n, n_pairs, s.data(), t.data(), seed, hyp.data()))) return rc;
  const int cap = h->params.nearest_neighbors_max;
  // rank the hypotheses of every pair (internal poses: the target moved by the inverse)
  std::vector<int> pick;   // n_pairs * n_refine hypothesis indices
  if (n_refine < kHyp) {
    std::vector<DevCloud *> rs, rt;
    for (int b = 0; b < n_pairs; b++)
      for (int k = 0; k < kHyp; k++) {
        rs.push_back(s[b]);
        rt.push_back(t[b]);
      }
    std::vector<double> asum;
    if ((rc = run_inner_product_pairs(h, rs, rt, hyp, rank_ell, cap, &asum))) return rc;
    for (int b = 0; b < n_pairs; b++) {
      std::vector<int> order(kHyp);
      for (int k = 0; k < kHyp; k++) order[k] = k;
      std::stable_sort(order.begin(), order.end(),
                       [&](int x, int y) { return asum[(size_t)b * kHyp + x] > asum[(size_t)b * kHyp + y]; });
      for (int r = 0; r < n_refine; r++) pick.push_back(order[r]);
    }
  } else {
    for (int b = 0; b < n_pairs; b++)
      for (int k = 0; k < kHyp; k++) pick.push_back(k);
  }
  // refine the picked hypotheses in one batch, judge them in one batch
  auto refine_and_judge = [&](const std::vector<int> &pairs_of, const std::vector<float> &inits,
                              std::vector<float> *Tres, std::vector<float> *cosv, std::vector<int> *its) -> int {
    std::vector<DevCloud *> as, at;
    for (int b : pairs_of) {
      as.push_back(s[b]);
      at.push_back(t[b]);
    }
    BatchResult r;
    int e = run_align_batch(h, as, at, inits, &r, nullptr, false, nullptr, nullptr, nullptr);
    if (e) return e;
    std::vector<float> Tj(inits.size());
    for (size_t q = 0; q < pairs_of.size(); q++) rigid_inverse(&r.T_out[16 * q], &Tj[16 * q]);
    std::vector<double> asum;
    if ((e = run_inner_product_pairs(h, as, at, Tj, judge_ell, cap, &asum))) return e;
    cosv->resize(pairs_of.size());
    for (size_t q = 0; q < pairs_of.size(); q++) {
      const int b = pairs_of[q];
      (*cosv)[q] = (float)(asum[q] / (std::sqrt((double)s[b]->n) * std::sqrt((double)t[b]->n)));
    }
    *Tres = r.T_out;
    *its = r.iters;
    return 0;
  };
  std::vector<int> owner;
  std::vector<float> inits;
  for (int b = 0; b < n_pairs; b++)
    for (int r = 0; r < n_refine; r++) {
      owner.push_back(b);
      const float *src = &hyp[16 * ((size_t)b * kHyp + pick[(size_t)b * n_refine + r])];
      inits.insert(inits.end(), src, src + 16);
    }
  std::vector<float> Tr, cv;
  std::vector<int> it;
  {
    // the hypotheses' refinement may start at a finer lengthscale than a grid start
    const float ell0 = h->params.ell_init;
    if (refine_ell > 0.f) h->params.ell_init = refine_ell;
    rc = refine_and_judge(owner, inits, &Tr, &cv, &it);
    h->params.ell_init = ell0;
    if (rc) return rc;
  }
  std::vector<float> best_cos(n_pairs, -INFINITY);
  std::vector<int> total_it(n_pairs, 0);
  for (size_t q = 0; q < owner.size(); q++) {
    const int b = owner[q];
    total_it[b] += it[q];
    if (cv[q] > best_cos[b]) {
      best_cos[b] = cv[q];
      copy16(&Tr[16 * q], T_out + 16 * (size_t)b);
    }
  }
  // grid fallback for the pairs whose judged cos-angle stays low
  std::vector<int> fb;
  std::vector<float> fb_init;
  for (int b = 0; b < n_pairs; b++) {
    if (used_fallback) used_fallback[b] = 0;
    if (!(best_cos[b] < fallback_cos)) continue;
    float g[16], gi[16];
    if ((rc = nearest_init_pose_impl(H, s[b], t[b], h->params.ell_init_first_frame, 0, 1, g, nullptr, nullptr)))
      return rc;
    rigid_inverse(g, gi);
    fb.push_back(b);
    fb_init.insert(fb_init.end(), gi, gi + 16);
  }
  if (!fb.empty()) {
    if ((rc = refine_and_judge(fb, fb_init, &Tr, &cv, &it))) return rc;
    for (size_t q = 0; q < fb.size(); q++) {
      const int b = fb[q];
      total_it[b] += it[q];
      if (used_fallback) used_fallback[b] = 1;
      if (cv[q] > best_cos[b]) {
        best_cos[b] = cv[q];
        copy16(&Tr[16 * q], T_out + 16 * (size_t)b);
      }
    }
  }
  for (int b = 0; b < n_pairs; b++) {
    if (cos_out) cos_out[b] = best_cos[b];
    if (iters) iters[b] = total_it[b];
  }
  if (secs) *secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return CVO_OK;
} catch (...) {
  return status_from_exception();
}

// ---------------------------------------------------- global registration
// Host pairs in, poses out: the plain grid (the reference's get_nearest_init_pose over
// the 24 cube rotations, then align from the inverted grid pose as the int overload of
// CvoGPU::align does, src/cvo/CvoGPU.cu:1533-1543), every pair in one batched align; or
// the learned proposal with the Python binding's defaults (best 2 hypotheses refined,
// ranked and judged at ell_init_first_frame, grid fallback below cos-angle 0).
extern "C" int cvo_global_register(cvo_handle *H, int n_pairs, const cvo_cloud *srcs, const cvo_cloud *tgts,
                                   int use_learned, cvo_proposal *proposal, float *T_out, int *iters,
                                   double *secs) try {
  if (!H || n_pairs < 0 || (n_pairs > 0 && (!srcs || !tgts || !T_out)) || (use_learned && !proposal))
    return CVO_ERR_INVALID_ARG;
  if (secs) *secs = 0;
  if (n_pairs == 0) return CVO_OK;
  if (!H->h.stream) return CVO_ERR_CUDA;
  const auto t0 = std::chrono::steady_clock::now();
  std::vector<cvo_gpu_cloud *> s(n_pairs, nullptr), t(n_pairs, nullptr);
  int rc = 0;
  for (int b = 0; b < n_pairs && !rc; b++) {
    rc = cvo_cloud_upload(H, &srcs[b], &s[b]);
    if (!rc) rc = cvo_cloud_upload(H, &tgts[b], &t[b]);
  }
  const float ell = H->h.params.ell_init_first_frame;
  if (!rc && use_learned) {
    rc = cvo_register_learned_batch_dev(H, proposal, n_pairs, s.data(), t.data(), 2, ell, ell, 0.f, 0.f, 0u, T_out,
                                        nullptr, nullptr, iters, nullptr);
  } else if (!rc) {
    std::vector<float> inits(16 * (size_t)n_pairs);
    for (int b = 0; b < n_pairs && !rc; b++) {
      float g[16];
      rc = cvo_get_nearest_init_pose_dev(H, s[b], t[b], ell, 0, 1, g, nullptr);
      if (!rc) rigid_inverse(g, &inits[16 * (size_t)b]);
    }
    if (!rc) rc = cvo_align_batch_dev(H, n_pairs, s.data(), t.data(), inits.data(), T_out, nullptr, iters, nullptr);
  }
  for (cvo_gpu_cloud *c : s)
    if (c) cvo_cloud_free(H, c);
  for (cvo_gpu_cloud *c : t)
    if (c) cvo_cloud_free(H, c);
  if (secs) *secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return rc;
} catch (...) {
  return status_from_exception();
}

// ------------------------------------------------------------ multi-frame
extern "C" int cvo_align_multi_dev(cvo_handle *H, int n_frames, cvo_gpu_cloud *const *clouds, double *poses,
                                   const uint8_t *hold_const, int n_edges, const int *edges, double *secs,
                                   int *iters) try {
  if (!H || n_frames <= 0 || !clouds || !poses || !hold_const || n_edges < 0 || (n_edges > 0 && !edges))
    return CVO_ERR_INVALID_ARG;
  std::vector<DevCloud *> c(n_frames);
  for (int i = 0; i < n_frames; i++) {
    if (!clouds[i]) return CVO_ERR_INVALID_ARG;
    c[i] = clouds[i]->d;
  }
  for (int e = 0; e < n_edges; e++)
    if (edges[2 * e] < 0 || edges[2 * e] >= n_frames || edges[2 * e + 1] < 0 || edges[2 * e + 1] >= n_frames)
      return CVO_ERR_INVALID_ARG;
  return run_align_multi(&H->h, n_frames, c.data(), poses, hold_const, n_edges, edges, secs, iters);
} catch (...) {
  return status_from_exception();
}

extern "C" int cvo_align_multi(cvo_handle *H, int n_frames, const cvo_cloud *clouds, double *poses,
                               const uint8_t *hold_const, int n_edges, const int *edges, double *secs, int *iters) try {
  if (!H || n_frames <= 0 || !clouds) return CVO_ERR_INVALID_ARG;
  TmpClouds tc{H, {}};
  std::vector<cvo_gpu_cloud *> g(n_frames);
  for (int i = 0; i < n_frames; i++) {
    int rc = cvo_cloud_upload(H, &clouds[i], &g[i]);
    if (rc) return rc;
    tc.v.push_back(g[i]);
  }
  return cvo_align_multi_dev(H, n_frames, g.data(), poses, hold_const, n_edges, edges, secs, iters);
} catch (...) {
  return status_from_exception();
}
