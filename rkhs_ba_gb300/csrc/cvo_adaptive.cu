// cvo_adaptive.cu -- adaptive-lengthscale CVO (AdaptiveCvoGPU, src/cvo/AdaptiveCvoGPU.cu).
//
// Every iteration needs three kernel matrices at the current lengthscale ell
// (fill_in_A_mat_gpu, :263-407): A (source rows against the moved target), Axx
// (source against itself) and Ayy (moved target against itself).  Each row keeps its
// first 512 kept pairs in target index order (KDTREE_K_SIZE,
// thirdparty/cugicp/cukdtree/cukdtree.h:12).  The reference scans every target for
// every row; here the three matrices are three edges of one batched association
// pass of the two-view engine (grid pruning, row lists, first-512-by-index
// selection), run with this path's own kernel constants: ell without range scaling
// (rows carry |x| = 0), no geometric-type factor, no semantic gate, the colour
// threshold -2 c_ell c_ell log(sp / c_s / c_s), and geometric-only values
// s^2 exp(-d2/2l^2) c_sigma.  The gradient (omega, v, not normalised), the lengthscale
// derivative dl and the step-size Taylor terms follow compute_flow_gpu_no_eigen
// (:548-719), compute_flow_gpu_ell_Ayy_no_eigen (:721-760), compute_flow (:793-891)
// and compute_step_size (:893-1075); the loop follows AdaptiveCvoGPU::align
// (:1077-1250): ell <- ell - dl_step dl, backed off to 0.7 ell_max at ell_max.
#include <cmath>
#include <cstring>
#include <chrono>
#include <vector>
#include <algorithm>
#include "cvo_internal.h"
#include "cvo_device.cuh"
#include "cvo_lie.cuh"

namespace cvo_gb {

constexpr int kAdCap = 512;
constexpr int kAdRedThreads = 256;

namespace {

// y' = Ri y + Ti in the canonical order, w = 0 (no range scaling of ell for these rows)
__global__ void k_ad_xform(int m, const float4 *y, const float *RiTi, float4 *out) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= m) return;
  const float4 p = y[j];
  out[j] = make_float4(xform_row(RiTi, RiTi[9], p.x, p.y, p.z), xform_row(RiTi + 3, RiTi[10], p.x, p.y, p.z),
                       xform_row(RiTi + 6, RiTi[11], p.x, p.y, p.z), 0.f);
}

// Sums NV per-thread doubles over the block; thread 0 writes them to out[blockIdx.x * NV].
template <int NV>
__device__ __forceinline__ void block_sum_out(double (&v)[NV], double *out) {
  __shared__ double red[NV][kAdRedThreads / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; k++) {
    double s = v[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xFFFFFFFFu, s, o);
    if (lane == 0) red[k][w] = s;
  }
  __syncthreads();
  if (threadIdx.x == 0)
#pragma unroll
    for (int k = 0; k < NV; k++) {
      double s = 0.0;
      for (int q = 0; q < kAdRedThreads / 32; q++) s += red[k][q];
      out[(size_t)blockIdx.x * NV + k] = s;
    }
}

// ELL of one edge: entry c of (tile-order) row s at [s * ld + c], original column indices.
struct Ell {
  const int *j;       // row-major with pitch ld
  const float *v;
  const int *nnz;
  int ld;
};

// Source rows (tile order xs): omega / c, v / d (FP32 per row, as
// compute_flow_gpu_no_eigen), the lengthscale derivative
// 2/l^3 (-sum_A a |y-x|^2) + 1/l^3 sum_Axx a |x'-x|^2, and the nnz of A and Axx.
// y: moved target, original order; xo: source, original order.  Block partials: 9 doubles.
__global__ void __launch_bounds__(kAdRedThreads) k_ad_flow(int n, const float4 *xs, const float4 *xo, const float4 *y,
                                                           Ell A, Ell X, float c, float d, float ell, double *part) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  double v[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  if (s < n) {
    const float4 p = xs[s];
    float w0 = 0.f, w1 = 0.f, w2 = 0.f, v0 = 0.f, v1 = 0.f, v2 = 0.f, dl = 0.f;
    const int na = A.nnz[s];
    for (int t = 0; t < na; t++) {
      const int j = A.j[(size_t)s * A.ld + t];
      const float a = A.v[(size_t)s * A.ld + t];
      const float4 q = y[j];
      const float cx = fs(fm(p.y, q.z), fm(p.z, q.y)), cy = fs(fm(p.z, q.x), fm(p.x, q.z)), cz = fs(fm(p.x, q.y), fm(p.y, q.x));
      const float dx = fs(q.x, p.x), dy = fs(q.y, p.y), dz = fs(q.z, p.z);
      w0 = fa(w0, fm(cx, a)); w1 = fa(w1, fm(cy, a)); w2 = fa(w2, fm(cz, a));
      v0 = fa(v0, fm(dx, a)); v1 = fa(v1, fm(dy, a)); v2 = fa(v2, fm(dz, a));
      dl = fs(dl, fm(fa(fa(fm(dx, dx), fm(dy, dy)), fm(dz, dz)), a));
    }
    const float ell3 = fm(fm(ell, ell), ell);
    float dxx = 0.f;
    const int nx = X.nnz[s];
    for (int t = 0; t < nx; t++) {
      const float4 q = xo[X.j[(size_t)s * X.ld + t]];
      dxx = fa(dxx, fm(sqdist3(q.x, q.y, q.z, p.x, p.y, p.z), X.v[(size_t)s * X.ld + t]));
    }
    v[0] = (double)__fdiv_rn(w0, c); v[1] = (double)__fdiv_rn(w1, c); v[2] = (double)__fdiv_rn(w2, c);
    v[3] = (double)__fdiv_rn(v0, d); v[4] = (double)__fdiv_rn(v1, d); v[5] = (double)__fdiv_rn(v2, d);
    v[6] = (double)fm(__fdiv_rn(2.f, ell3), dl) + (double)fm(__fdiv_rn(1.f, ell3), dxx);
    v[7] = (double)na;
    v[8] = (double)nx;
  }
  block_sum_out<9>(v, part);
}

// Moved-target rows (tile order ys): 1/l^3 sum_Ayy a |y'-y|^2 and the nnz of Ayy.
// y: moved target, original order.  Block partials: 2 doubles.
__global__ void __launch_bounds__(kAdRedThreads) k_ad_flow_yy(int m, const float4 *ys, const float4 *y, Ell Y,
                                                              float ell, double *part) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  double v[2] = {0, 0};
  if (s < m) {
    const float4 p = ys[s];
    float prod = 0.f;
    const int ny = Y.nnz[s];
    for (int t = 0; t < ny; t++) {
      const float4 q = y[Y.j[(size_t)s * Y.ld + t]];
      prod = fa(prod, fm(Y.v[(size_t)s * Y.ld + t], sqdist3(q.x, q.y, q.z, p.x, p.y, p.z)));
    }
    const float ell3 = fm(fm(ell, ell), ell);
    v[0] = (double)fm(__fdiv_rn(1.f, ell3), prod);
    v[1] = (double)ny;
  }
  block_sum_out<2>(v, part);
}

// Taylor terms B, C, D, E of the step size along (omega, v) (compute_step_size_xi and
// compute_step_size_poly_coeff, :893-1004), per entry in double.  Block partials: 4 doubles.
__global__ void __launch_bounds__(kAdRedThreads) k_ad_step(int n, const float4 *xs, const float4 *y, Ell A,
                                                           const float *xi6, double coef, double *part) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  double v[4] = {0, 0, 0, 0};
  if (s < n) {
    const double w[3] = {xi6[0], xi6[1], xi6[2]}, vv[3] = {xi6[3], xi6[4], xi6[5]};
    const float4 p = xs[s];
    const int na = A.nnz[s];
    for (int t = 0; t < na; t++) {
      const double a = A.v[(size_t)s * A.ld + t];
      const float4 q = y[A.j[(size_t)s * A.ld + t]];
      const double yy[3] = {q.x, q.y, q.z};
      double u[3], u2[3], u3[3], u4[3];
      u[0] = w[1] * yy[2] - w[2] * yy[1] + vv[0];
      u[1] = w[2] * yy[0] - w[0] * yy[2] + vv[1];
      u[2] = w[0] * yy[1] - w[1] * yy[0] + vv[2];
      u2[0] = w[1] * u[2] - w[2] * u[1]; u2[1] = w[2] * u[0] - w[0] * u[2]; u2[2] = w[0] * u[1] - w[1] * u[0];
      u3[0] = w[1] * u2[2] - w[2] * u2[1]; u3[1] = w[2] * u2[0] - w[0] * u2[2]; u3[2] = w[0] * u2[1] - w[1] * u2[0];
      u4[0] = w[1] * u3[2] - w[2] * u3[1]; u4[1] = w[2] * u3[0] - w[0] * u3[2]; u4[2] = w[0] * u3[1] - w[1] * u3[0];
      const double dd[3] = {(double)p.x - yy[0], (double)p.y - yy[1], (double)p.z - yy[2]};
      const double nz2 = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
      const double zdz2 = -(u[0] * u2[0] + u[1] * u2[1] + u[2] * u2[2]);
      const double ec = (u2[0] * u2[0] + u2[1] * u2[1] + u2[2] * u2[2]) + 2.0 * (u[0] * u3[0] + u[1] * u3[1] + u[2] * u3[2]);
      const double ud = u[0] * dd[0] + u[1] * dd[1] + u[2] * dd[2];
      const double u2d = u2[0] * dd[0] + u2[1] * dd[1] + u2[2] * dd[2];
      const double u3d = u3[0] * dd[0] + u3[1] * dd[1] + u3[2] * dd[2];
      const double u4d = u4[0] * dd[0] + u4[1] * dd[1] + u4[2] * dd[2];
      const double beta = -2.0 * coef * ud;
      const double gamma = -coef * (nz2 + 2.0 * u2d);
      const double delta = 2.0 * coef * (zdz2 - u3d);
      const double epsil = -coef * (ec + 2.0 * u4d);
      v[0] += a * beta;
      v[1] += a * (gamma + beta * beta / 2.0);
      v[2] += a * (delta + beta * gamma + beta * beta * beta / 6.0);
      v[3] += a * (epsil + beta * delta + 0.5 * beta * beta * gamma + 0.5 * gamma * gamma + beta * beta * beta * beta / 24.0);
    }
  }
  block_sum_out<4>(v, part);
}

// Pose update of one iteration (Exp_SEK3 in float, then T = R dT + T, R = R dR in
// float): st = {R[9], T[3]} updated in place, dist = ||log(dR, dT)||.
__global__ void k_ad_update(float *st, const float *xi6, float step, double *dist) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  float X[12], xi[6];
  for (int k = 0; k < 6; k++) xi[k] = xi6[k];
  exp_sek3(xi, step, X);
  float R[9], T[3], Rn[9], Tn[3];
  for (int k = 0; k < 9; k++) R[k] = st[k];
  for (int k = 0; k < 3; k++) T[k] = st[9 + k];
  for (int r = 0; r < 3; r++) Tn[r] = fa(fa(fa(fm(R[3 * r], X[3]), fm(R[3 * r + 1], X[7])), fm(R[3 * r + 2], X[11])), T[r]);
  for (int r = 0; r < 3; r++)
    for (int c = 0; c < 3; c++)
      Rn[3 * r + c] = fa(fa(fm(R[3 * r], X[c]), fm(R[3 * r + 1], X[4 + c])), fm(R[3 * r + 2], X[8 + c]));
  for (int k = 0; k < 9; k++) st[k] = Rn[k];
  for (int k = 0; k < 3; k++) st[9 + k] = Tn[k];
  double dR[9], dT[3];
  for (int r = 0; r < 3; r++) {
    for (int c = 0; c < 3; c++) dR[3 * r + c] = X[4 * r + c];
    dT[r] = X[4 * r + 3];
  }
  *dist = dist_se3(dR, dT);
}

}  // namespace

// ------------------------------------------------------------------ host
namespace {

// Kernel constants of fill_in_A_mat_gpu (:279-283, :316-370) on the two-view engine.
KParams adaptive_kparams(const cvo_params &p) {
  KParams k = make_kparams(p);
  k.use_geo = 1;                 // the distance gate is unconditional on this path
  k.use_gtype = 0;               // no geometric-type factor
  k.d2_s_thres = INFINITY;       // no semantic gate
  if (k.use_int)
    k.d2_c_thres = (float)(-2.0 * (double)p.c_ell * (double)p.c_ell * (double)logf(p.sp_thres / p.c_sigma / p.c_sigma));
  k.two_c2 = 2.0 * (double)p.c_ell * (double)p.c_ell;
  if (!k.use_int && !k.use_sem) {
    // geometric only: s^2 exp(-d2 / 2 l^2) c_sigma; the prefilter bound grows by c_sigma
    k.val_scale = p.c_sigma;
    if (k.use_mma) {
      if (p.c_sigma > 0.f) k.mma_tau = (float)((double)k.mma_tau + std::log((double)p.c_sigma));
      else k.use_mma = 0;
    }
  }
  return k;
}

// Target transform of the internal pose (R, T): Ri = R^T, Ti = -R^T T (update_tf, :240-262).
void pose_rinv(const float R[9], const float T[3], float RiTi[12]) {
  for (int r = 0; r < 3; r++)
    for (int c = 0; c < 3; c++) RiTi[3 * r + c] = R[3 * c + r];
  for (int r = 0; r < 3; r++) {
    const float a = RiTi[3 * r] * T[0], b = RiTi[3 * r + 1] * T[1], c = RiTi[3 * r + 2] * T[2];
    RiTi[9 + r] = -((a + b) + c);
  }
}

// Row-major 3x4 pose of a target transform (edge pose convention).
void pose12(const float RiTi[12], float Q[12]) {
  for (int r = 0; r < 3; r++) {
    for (int c = 0; c < 3; c++) Q[4 * r + c] = RiTi[3 * r + c];
    Q[4 * r + 3] = RiTi[9 + r];
  }
}

const float kIdentity12[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
const float kIdentityRiTi[12] = {1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0};

struct AdBuffers {
  float4 *xs = nullptr, *ys = nullptr, *yo = nullptr;     // source tile order (w = 0), moved target tile / original order
  double *part = nullptr, *dist = nullptr;
  float *xi = nullptr, *st = nullptr, *RiTi = nullptr, *Id = nullptr;
  ~AdBuffers() {
    void *ps[] = {xs, ys, yo, part, dist, xi, st, RiTi, Id};
    for (void *p : ps) cudaFree(p);
  }
};

template <class T>
bool dalloc(T **p, size_t count) {
  return cudaMalloc((void **)p, sizeof(T) * (count ? count : 1)) == cudaSuccess;
}

}  // namespace

int run_association_adaptive(Handle *h, DevCloud *src, DevCloud *tgt, const float T[16], float ell,
                             std::vector<int> *rowptr, std::vector<int> *col, std::vector<float> *val) {
  NvtxRange nvtx_range("adaptive_association");
  const int n = src->n, m = tgt->n;
  if (src->F != tgt->F || src->C != tgt->C) return CVO_ERR_INVALID_ARG;
  rowptr->assign((size_t)n + 1, 0);
  col->clear();
  val->clear();
  if (n == 0 || m == 0) return CVO_OK;
  const KParams K = adaptive_kparams(h->params);
  float R[9], Tt[3], RiTi[12], Q[12];
  for (int r = 0; r < 3; r++) {
    for (int c = 0; c < 3; c++) R[3 * r + c] = T[4 * c + r];
    Tt[r] = T[12 + r];
  }
  pose_rinv(R, Tt, RiTi);
  pose12(RiTi, Q);
  AdBuffers b;
  if (!dalloc(&b.xs, n) || !dalloc(&b.Id, 12)) {
    cudaGetLastError();
    return CVO_ERR_OUT_OF_MEMORY;
  }
  CVO_CUDA_TRY(h, cudaMemcpyAsync(b.Id, kIdentityRiTi, sizeof(kIdentityRiTi), cudaMemcpyHostToDevice, h->stream));
  k_ad_xform<<<(n + 255) / 256, 256, 0, h->stream>>>(n, src->spos, b.Id, b.xs);
  h->launches++;
  std::vector<EdgeAssoc> E;
  int rc = run_association_edges(h, {src}, {tgt}, {b.xs}, {0.f}, std::vector<float>(Q, Q + 12), {ell}, {kAdCap},
                                 kAdCap, &E, &K);
  if (rc) return rc;
  const int ld = E[0].ld;
  std::vector<int> nz(n), jj((size_t)n * ld), sperm(n);
  std::vector<float> vv((size_t)n * ld);
  CVO_CUDA_TRY(h, cudaMemcpyAsync(nz.data(), E[0].nnz_row, sizeof(int) * n, cudaMemcpyDeviceToHost, h->stream));
  CVO_CUDA_TRY(h, cudaMemcpyAsync(jj.data(), E[0].A_j, sizeof(int) * jj.size(), cudaMemcpyDeviceToHost, h->stream));
  CVO_CUDA_TRY(h, cudaMemcpyAsync(vv.data(), E[0].A_v, sizeof(float) * vv.size(), cudaMemcpyDeviceToHost, h->stream));
  CVO_CUDA_TRY(h, cudaMemcpyAsync(sperm.data(), src->sperm, sizeof(int) * n, cudaMemcpyDeviceToHost, h->stream));
  CVO_CUDA_TRY(h, cudaStreamSynchronize(h->stream));
  // tile-order rows back to source indices, each row in ascending target index
  std::vector<int> cnt(n, 0);
  for (int s = 0; s < n; s++) cnt[sperm[s]] = nz[s];
  for (int i = 0; i < n; i++) (*rowptr)[i + 1] = (*rowptr)[i] + cnt[i];
  col->resize((size_t)(*rowptr)[n]);
  val->resize((size_t)(*rowptr)[n]);
  std::vector<std::pair<int, float>> row;
  for (int s = 0; s < n; s++) {
    row.clear();
    for (int t = 0; t < nz[s]; t++) row.emplace_back(jj[(size_t)s * ld + t], vv[(size_t)s * ld + t]);
    std::sort(row.begin(), row.end(), [](const std::pair<int, float> &a, const std::pair<int, float> &b2) {
      return a.first < b2.first;
    });
    const int base = (*rowptr)[sperm[s]];
    for (size_t t = 0; t < row.size(); t++) {
      (*col)[base + t] = row[t].first;
      (*val)[base + t] = row[t].second;
    }
  }
  return CVO_OK;
}

int run_align_adaptive(Handle *h, DevCloud *src, DevCloud *tgt, const float T_init[16], float T_out[16],
                       double *secs, int *iters_out, double *trace, int trace_len) {
  NvtxRange nvtx_range("adaptive_align");
  const cvo_params &p = h->params;
  const int n = src->n, m = tgt->n;
  if (src->F != tgt->F || src->C != tgt->C) return CVO_ERR_INVALID_ARG;
  auto t0 = std::chrono::steady_clock::now();
  const KParams K = adaptive_kparams(p);
  const int bn = (n + kAdRedThreads - 1) / kAdRedThreads, bm = (m + kAdRedThreads - 1) / kAdRedThreads;
  AdBuffers b;
  if (!dalloc(&b.xs, n) || !dalloc(&b.ys, m) || !dalloc(&b.yo, m) || !dalloc(&b.part, (size_t)9 * bn + 2 * bm + 8) ||
      !dalloc(&b.dist, 1) || !dalloc(&b.xi, 6) || !dalloc(&b.st, 12) || !dalloc(&b.RiTi, 12) || !dalloc(&b.Id, 12)) {
    cudaGetLastError();
    h->last_error = "out of device memory for the adaptive path";
    return CVO_ERR_OUT_OF_MEMORY;
  }
  CVO_CUDA_TRY(h, cudaMemcpyAsync(b.Id, kIdentityRiTi, sizeof(kIdentityRiTi), cudaMemcpyHostToDevice, h->stream));
  k_ad_xform<<<(n + 255) / 256, 256, 0, h->stream>>>(n, src->spos, b.Id, b.xs);
  h->launches++;
  float R[9], T[3];
  for (int r = 0; r < 3; r++) {
    for (int c = 0; c < 3; c++) R[3 * r + c] = T_init[4 * c + r];
    T[r] = T_init[12 + r];
  }
  float ell = p.ell_init, ell_max = p.ell_max;
  int iter = p.MAX_ITER, ret = 0;
  std::vector<double> part((size_t)9 * bn + 2 * bm);
  for (int k = 0; k < p.MAX_ITER; k++) {
    float RiTi[12], Q[12];
    pose_rinv(R, T, RiTi);
    pose12(RiTi, Q);
    CVO_CUDA_TRY(h, cudaMemcpyAsync(b.RiTi, RiTi, sizeof(RiTi), cudaMemcpyHostToDevice, h->stream));
    k_ad_xform<<<(m + 255) / 256, 256, 0, h->stream>>>(m, tgt->spos, b.RiTi, b.ys);
    k_ad_xform<<<(m + 255) / 256, 256, 0, h->stream>>>(m, tgt->pos, b.RiTi, b.yo);
    h->launches += 2;
    // A, Axx, Ayy as three edges of one association pass
    std::vector<float> poses(Q, Q + 12);
    poses.insert(poses.end(), kIdentity12, kIdentity12 + 12);
    poses.insert(poses.end(), Q, Q + 12);
    std::vector<EdgeAssoc> E;
    int rc = run_association_edges(h, {src, src, tgt}, {tgt, src, tgt}, {b.xs, b.xs, b.ys}, {0.f, 0.f, 0.f}, poses,
                                   {ell, ell, ell}, {kAdCap, kAdCap, kAdCap}, kAdCap, &E, &K);
    if (rc) return rc;
    const Ell A{E[0].A_j, E[0].A_v, E[0].nnz_row, E[0].ld}, X{E[1].A_j, E[1].A_v, E[1].nnz_row, E[1].ld};
    const Ell Y{E[2].A_j, E[2].A_v, E[2].nnz_row, E[2].ld};
    k_ad_flow<<<bn, kAdRedThreads, 0, h->stream>>>(n, b.xs, src->pos, b.yo, A, X, p.c, p.d, ell, b.part);
    k_ad_flow_yy<<<bm, kAdRedThreads, 0, h->stream>>>(m, b.ys, b.yo, Y, ell, b.part + (size_t)9 * bn);
    h->launches += 2;
    CVO_CUDA_TRY(h, cudaMemcpyAsync(part.data(), b.part, sizeof(double) * part.size(), cudaMemcpyDeviceToHost,
                                    h->stream));
    CVO_CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    double g[6] = {0, 0, 0, 0, 0, 0}, dlA = 0.0, dlY = 0.0, nA = 0.0, nX = 0.0, nY = 0.0;
    for (int q = 0; q < bn; q++) {
      const double *s = &part[(size_t)9 * q];
      for (int t = 0; t < 6; t++) g[t] += s[t];
      dlA += s[6];
      nA += s[7];
      nX += s[8];
    }
    for (int q = 0; q < bm; q++) {
      dlY += part[(size_t)9 * bn + 2 * q];
      nY += part[(size_t)9 * bn + 2 * q + 1];
    }
    // the reference's normaliser is unsigned: Axx + Ayy - 2 A wraps around (:886)
    const uint32_t denom = (uint32_t)nX + (uint32_t)nY - 2u * (uint32_t)nA;
    const double dl = (double)((float)dlA + (float)dlY) / (double)denom;
    float xi[6];
    for (int t = 0; t < 6; t++) xi[t] = (float)g[t];
    CVO_CUDA_TRY(h, cudaMemcpyAsync(b.xi, xi, sizeof(xi), cudaMemcpyHostToDevice, h->stream));
    k_ad_step<<<bn, kAdRedThreads, 0, h->stream>>>(n, b.xs, b.yo, A, b.xi, 1.0 / (2.0 * (double)ell * (double)ell),
                                                   b.part);
    h->launches++;
    CVO_CUDA_TRY(h, cudaMemcpyAsync(part.data(), b.part, sizeof(double) * 4 * (size_t)bn, cudaMemcpyDeviceToHost,
                                    h->stream));
    CVO_CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    double bcde[4] = {0, 0, 0, 0};
    for (int q = 0; q < bn; q++)
      for (int t = 0; t < 4; t++) bcde[t] += part[(size_t)4 * q + t];
    // coefficients rounded to float, smallest positive real root, else min_step, at most 0.8 (:1055-1073)
    double re[3], im[3], temp = 1.7976931348623157e308;
    const float c3 = (float)(4.0 * (double)(float)bcde[3]), c2 = (float)(3.0 * (double)(float)bcde[2]);
    const float c1 = (float)(2.0 * (double)(float)bcde[1]), c0 = (float)bcde[0];
    if (cubic_roots(c3, c2, c1, c0, re, im))
      for (int t = 0; t < 3; t++)
        if (re[t] > 0 && re[t] < temp && im[t] == 0.0) temp = re[t];
    double step = temp == 1.7976931348623157e308 ? (double)p.min_step : temp;
    if (step > 0.8) step = 0.8;
    const float stepf = (float)step;
    if (trace && k < trace_len) {
      double *tr = trace + 6 * (size_t)k;
      tr[0] = ell; tr[1] = dl; tr[2] = stepf; tr[3] = nA; tr[4] = nX; tr[5] = nY;
    }
    const double wn = std::sqrt((double)xi[0] * xi[0] + (double)xi[1] * xi[1] + (double)xi[2] * xi[2]);
    const double vn = std::sqrt((double)xi[3] * xi[3] + (double)xi[4] * xi[4] + (double)xi[5] * xi[5]);
    if (wn < p.eps && vn < p.eps) {
      iter = k;
      if (wn < 1e-8 && vn < 1e-8) ret = -1;
      break;
    }
    float st[12];
    memcpy(st, R, sizeof(R));
    memcpy(st + 9, T, sizeof(T));
    CVO_CUDA_TRY(h, cudaMemcpyAsync(b.st, st, sizeof(st), cudaMemcpyHostToDevice, h->stream));
    k_ad_update<<<1, 32, 0, h->stream>>>(b.st, b.xi, stepf, b.dist);
    h->launches++;
    double dist = 0.0;
    CVO_CUDA_TRY(h, cudaMemcpyAsync(st, b.st, sizeof(st), cudaMemcpyDeviceToHost, h->stream));
    CVO_CUDA_TRY(h, cudaMemcpyAsync(&dist, b.dist, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CVO_CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    memcpy(R, st, sizeof(R));
    memcpy(T, st + 9, sizeof(T));
    if (dist < (double)p.eps_2) {
      iter = k;
      break;
    }
    ell = (float)((double)ell - p.dl_step * dl);
    if (ell >= ell_max) {
      ell = (float)((double)ell_max * 0.7);
      ell_max = (float)((double)ell_max * 0.7);
    }
    if (ell < p.ell_min) ell = p.ell_min;
  }
  if (iters_out) *iters_out = iter;
  float RiTi[12];
  pose_rinv(R, T, RiTi);
  memset(T_out, 0, sizeof(float) * 16);
  for (int r = 0; r < 3; r++) {
    for (int c = 0; c < 3; c++) T_out[4 * c + r] = RiTi[3 * r + c];
    T_out[12 + r] = RiTi[9 + r];
  }
  T_out[15] = 1.f;
  if (secs) *secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return ret == -1 ? CVO_ZERO_GRADIENT : CVO_OK;
}

}  // namespace cvo_gb
