// cvo_aniso.cu -- association with a non-isotropic (3x3) geometric kernel.
//
// CvoGPU::compute_association_gpu(source, target, T, non_isotropic_kernel, association)
// (src/cvo/CvoGPU.cu:1936-1950 -> inner_product_non_isotropic_impl, :1873-1934):
// the kernel is inverted once on the host; for every source point a the inverse is
// rotated into a frame built from the point's direction (rotate_kernel_and_inverse,
// :135-160: z = a/|a|, x = (1, 1, -(z0+z1)/z2), y = z cross x, neither x nor y
// normalised, M = U K^-1 U^T with U = [x y z]), and the geometric factor of a pair is
// sigma^2 exp(-(a-b)^T M (a-b) / 2) (mahananobis_distance, :165-183) -- no distance
// threshold and no range-scaled lengthscale.  Colour and semantic factors keep their
// thresholds; the geometric type is off.  Each row keeps its first `cap` pairs in
// ascending target index (fill_in_A_mat_gpu_dense_mat_kernel, :719-830).
//
// Without a distance threshold there is no spatial pruning, so this is an
// index-ordered scan of all targets per source row: a block of 128 rows stages 128
// targets at a time in shared memory (coalesced loads), every thread tests its row
// against them, and the block stops as soon as all of its rows hold `cap` pairs.
#include <cmath>
#include <cstring>
#include <vector>
#include "cvo_internal.h"
#include "cvo_device.cuh"

namespace cvo_gb {
namespace {

constexpr int kAnisoRows = 128;

struct AnisoParams {
  KParams K;
  float Ki[9];        // inverse kernel, column-major
  float Ri[9], Ti[3]; // target transform
  int n, m, cap, F, C;
};

__global__ void k_aniso_transform(const float4 *pos, int m, AnisoParams A, float4 *ytr) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= m) return;
  const float4 y = pos[j];
  ytr[j] = make_float4(xform_row(&A.Ri[0], A.Ti[0], y.x, y.y, y.z), xform_row(&A.Ri[3], A.Ti[1], y.x, y.y, y.z),
                       xform_row(&A.Ri[6], A.Ti[2], y.x, y.y, y.z), 0.f);
}

// M (row-major) = U Ki U^T for source point x, in the oracle's order.
__device__ __forceinline__ void aniso_row_matrix(const float *Ki, float x0, float x1, float x2, float (&M)[9]) {
  const float nrm = __fsqrt_rn(fa(fa(fm(x0, x0), fm(x1, x1)), fm(x2, x2)));
  const float z[3] = {__fdiv_rn(x0, nrm), __fdiv_rn(x1, nrm), __fdiv_rn(x2, nrm)};
  const float t = __fdiv_rn(-1.f, z[2]);
  const float xv[3] = {1.f, 1.f, fm(t, fa(z[0], z[1]))};
  const float yv[3] = {fs(fm(z[1], xv[2]), fm(z[2], xv[1])), fs(fm(z[2], xv[0]), fm(z[0], xv[2])),
                       fs(fm(z[0], xv[1]), fm(z[1], xv[0]))};
  float U[3][3];
#pragma unroll
  for (int i = 0; i < 3; i++) { U[i][0] = xv[i]; U[i][1] = yv[i]; U[i][2] = z[i]; }
  float P[3][3];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++)
      P[i][j] = fa(fa(fm(U[i][0], Ki[3 * j + 0]), fm(U[i][1], Ki[3 * j + 1])), fm(U[i][2], Ki[3 * j + 2]));
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) M[3 * i + j] = fa(fa(fm(P[i][0], U[j][0]), fm(P[i][1], U[j][1])), fm(P[i][2], U[j][2]));
}

// One pair: kept?  Value in a (FP32 fast path, FP64 re-evaluation near sp_thres).
template <int FCH, int LCH>
__device__ __forceinline__ bool aniso_pair(const KParams &K, int F, int C, const float (&M)[9], const float4 &x,
                                           const float4 (&xf)[FCH > 0 ? FCH : 1], const float4 (&xl)[LCH > 0 ? LCH : 1],
                                           const float4 &y, const float4 *yf, const float4 *yl, float &a) {
  float d2 = 0.f;
  if (K.use_geo) {
    const float d0 = fs(x.x, y.x), d1 = fs(x.y, y.y), dd = fs(x.z, y.z);
    float v[3];
#pragma unroll
    for (int j = 0; j < 3; j++) v[j] = fa(fa(fm(d0, M[j]), fm(d1, M[3 + j])), fm(dd, M[6 + j]));
    d2 = fa(fa(fm(v[0], d0), fm(v[1], d1)), fm(v[2], dd));
  }
  float d2c = 0.f;
  if (K.use_int) {
#pragma unroll
    for (int q = 0; q < (FCH > 0 ? FCH : 1); q++) {
      if (FCH == 0) break;
      const float av[4] = {xf[q].x, xf[q].y, xf[q].z, xf[q].w};
      const float4 b4 = yf[q];
      const float bv[4] = {b4.x, b4.y, b4.z, b4.w};
#pragma unroll
      for (int r = 0; r < 4; r++)
        if (4 * q + r < F) { const float t = fs(av[r], bv[r]); d2c = fa(d2c, fm(t, t)); }
    }
    if (!(d2c < K.d2_c_thres)) return false;
  }
  float d2s = 0.f;
  if (K.use_sem) {
#pragma unroll
    for (int q = 0; q < (LCH > 0 ? LCH : 1); q++) {
      if (LCH == 0) break;
      const float av[4] = {xl[q].x, xl[q].y, xl[q].z, xl[q].w};
      const float4 b4 = yl[q];
      const float bv[4] = {b4.x, b4.y, b4.z, b4.w};
#pragma unroll
      for (int r = 0; r < 4; r++)
        if (4 * q + r < C) { const float t = fs(av[r], bv[r]); d2s = fa(d2s, fm(t, t)); }
    }
    if (!(d2s < K.d2_s_thres)) return false;
  }
  const float kf = K.use_geo ? fm(K.sigma2, __expf(fm(-d2, 0.5f))) : 1.f;
  const float ckf = K.use_int ? fm(K.c_sigma2, __expf(fm(-d2c, K.inv2c2))) : 1.f;
  const float skf = K.use_sem ? fm(K.s_sigma_sq, __expf(fm(-d2s, __frcp_rn(fm(fm(2.f, K.s_ell), K.s_ell))))) : 1.f;
  float af = fm(fm(fm(ckf, kf), skf), 1.f);
  // sigma^2 exp(-d2 / 2) is the isotropic value with l = 1
  if (fabsf(fs(af, K.sp_thres)) <= kBand * K.sp_thres) af = exact_value(K, 1.f, d2, d2c, d2s, 1.f);
  a = af;
  return af > K.sp_thres;
}

template <int FCH, int LCH>
__global__ void __launch_bounds__(kAnisoRows) k_assoc_aniso(AnisoParams A, const float4 *xpos, const float *xfeat,
                                                            const float *xlab, const float4 *ytr, const float *yfeat,
                                                            const float *ylab, int *ell_j, float *ell_v, int *nnz) {
  constexpr int FP = FCH > 0 ? FCH : 1, LP = LCH > 0 ? LCH : 1;
  __shared__ float4 cpos[kAnisoRows];
  __shared__ float4 cfeat[kAnisoRows * FP];
  __shared__ float4 clab[kAnisoRows * LP];
  const int tid = threadIdx.x;
  const int i = blockIdx.x * kAnisoRows + tid;
  const bool valid = i < A.n;
  const float4 x = valid ? xpos[i] : make_float4(0.f, 0.f, 0.f, 0.f);
  float4 xf[FP], xl[LP];
#pragma unroll
  for (int q = 0; q < FP; q++)
    xf[q] = (FCH > 0 && valid) ? reinterpret_cast<const float4 *>(xfeat)[(size_t)i * FCH + q] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
  for (int q = 0; q < LP; q++)
    xl[q] = (LCH > 0 && valid) ? reinterpret_cast<const float4 *>(xlab)[(size_t)i * LCH + q] : make_float4(0.f, 0.f, 0.f, 0.f);
  float M[9];
  aniso_row_matrix(A.Ki, x.x, x.y, x.z, M);
  int cnt = 0;
  for (int j0 = 0; j0 < A.m; j0 += kAnisoRows) {
    if (__syncthreads_and(!valid || cnt >= A.cap)) break;   // every row of the block is full
    const int j = j0 + tid;
    const bool has = j < A.m;
    cpos[tid] = has ? ytr[j] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int q = 0; q < FP; q++)
      cfeat[tid * FP + q] = (FCH > 0 && has) ? reinterpret_cast<const float4 *>(yfeat)[(size_t)j * FCH + q]
                                             : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int q = 0; q < LP; q++)
      clab[tid * LP + q] = (LCH > 0 && has) ? reinterpret_cast<const float4 *>(ylab)[(size_t)j * LCH + q]
                                            : make_float4(0.f, 0.f, 0.f, 0.f);
    __syncthreads();
    const int nk = min(kAnisoRows, A.m - j0);
    if (valid) {
      for (int k = 0; k < nk && cnt < A.cap; k++) {
        float a;
        if (aniso_pair<FCH, LCH>(A.K, A.F, A.C, M, x, xf, xl, cpos[k], &cfeat[k * FP], &clab[k * LP], a)) {
          ell_j[(size_t)i * A.cap + cnt] = j0 + k;
          ell_v[(size_t)i * A.cap + cnt] = a;
          cnt++;
        }
      }
    }
  }
  if (valid) nnz[i] = cnt;
}

using AnisoFn = void (*)(AnisoParams, const float4 *, const float *, const float *, const float4 *, const float *,
                         const float *, int *, float *, int *);

AnisoFn pick_aniso(int fch, int lch) {
#define CVO_ANISO(FC, LC) \
  if (fch == FC && lch == LC) return k_assoc_aniso<FC, LC>;
  CVO_ANISO(0, 0) CVO_ANISO(1, 0) CVO_ANISO(2, 0)
  CVO_ANISO(0, 5) CVO_ANISO(1, 5) CVO_ANISO(2, 5)
  CVO_ANISO(0, 9) CVO_ANISO(1, 9) CVO_ANISO(2, 9)
#undef CVO_ANISO
  return nullptr;
}

}  // namespace

// Float 3x3 inverse of a column-major matrix: cofactors of column 0, det = their
// dot product with column 0, every entry times 1/det (the order of Eigen's 3x3 inverse).
void kernel_inverse3(const float K[9], float Ki[9]) {
  auto km = [&](int r, int c) { return K[3 * c + r]; };
  float cof[3][3];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      const int i1 = (i + 1) % 3, i2 = (i + 2) % 3, j1 = (j + 1) % 3, j2 = (j + 2) % 3;
      const float u = km(i1, j1) * km(i2, j2), v = km(i1, j2) * km(i2, j1);
      cof[i][j] = u - v;
    }
  const float d0 = cof[0][0] * km(0, 0), d1 = cof[1][0] * km(1, 0), d2 = cof[2][0] * km(2, 0);
  const float det = (d0 + d1) + d2;
  const float invdet = 1.f / det;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) Ki[3 * j + i] = cof[j][i] * invdet;
}

int run_association_aniso(Handle *h, DevCloud *src, DevCloud *tgt, const float T[16], const float kernel[9],
                          int cap, std::vector<int> *rowptr, std::vector<int> *col, std::vector<float> *val) {
  NvtxRange nvtx_range("aniso_association");
  const int n = src->n, m = tgt->n;
  if (src->F != tgt->F || src->C != tgt->C) return CVO_ERR_INVALID_ARG;
  rowptr->assign((size_t)n + 1, 0);
  col->clear();
  val->clear();
  if (n == 0 || m == 0 || cap <= 0) return CVO_OK;
  AnisoParams A;
  memset(&A, 0, sizeof(A));
  A.K = make_kparams(h->params);
  kernel_inverse3(kernel, A.Ki);
  // target moved by T^-1 (update_tf, src/cvo/CvoGPU.cu:98-130): Ri = R^T, Ti = -R^T t
  for (int r = 0; r < 3; r++)
    for (int c = 0; c < 3; c++) A.Ri[3 * r + c] = T[4 * r + c];   // (R^T)(r, c) = R(c, r) = T[4 r + c]
  for (int r = 0; r < 3; r++) {
    const float a = A.Ri[3 * r] * T[12], b = A.Ri[3 * r + 1] * T[13], c = A.Ri[3 * r + 2] * T[14];
    A.Ti[r] = -((a + b) + c);
  }
  A.n = n; A.m = m; A.cap = cap; A.F = src->F; A.C = src->C;
  const int fch = A.K.use_int ? (src->F + 3) / 4 : 0;
  const int lch = A.K.use_sem ? label_chunks(src->C) : 0;
  AnisoFn fn = pick_aniso(fch, lch);
  if (!fn) return CVO_ERR_UNSUPPORTED;
  float4 *ytr = nullptr;
  int *ej = nullptr, *nz = nullptr;
  float *ev = nullptr;
  auto release = [&]() { cudaFree(ytr); cudaFree(ej); cudaFree(ev); cudaFree(nz); };
  if (cudaMalloc((void **)&ytr, sizeof(float4) * m) != cudaSuccess ||
      cudaMalloc((void **)&ej, sizeof(int) * (size_t)n * cap) != cudaSuccess ||
      cudaMalloc((void **)&ev, sizeof(float) * (size_t)n * cap) != cudaSuccess ||
      cudaMalloc((void **)&nz, sizeof(int) * n) != cudaSuccess) {
    cudaGetLastError();
    release();
    return CVO_ERR_OUT_OF_MEMORY;
  }
  k_aniso_transform<<<(m + 255) / 256, 256, 0, h->stream>>>(tgt->pos, m, A, ytr);
  fn<<<(n + kAnisoRows - 1) / kAnisoRows, kAnisoRows, 0, h->stream>>>(A, src->pos, src->feat, src->lab, ytr, tgt->feat,
                                                                      tgt->lab, ej, ev, nz);
  h->launches += 2;
  std::vector<int> nzh(n);
  std::vector<int> jh((size_t)n * cap);
  std::vector<float> vh((size_t)n * cap);
  cudaError_t e = cudaMemcpyAsync(nzh.data(), nz, sizeof(int) * n, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(jh.data(), ej, sizeof(int) * jh.size(), cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(vh.data(), ev, sizeof(float) * vh.size(), cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  release();
  if (e != cudaSuccess) return set_cuda_error(h, e, "association (non-isotropic kernel)");
  for (int i = 0; i < n; i++) (*rowptr)[i + 1] = (*rowptr)[i] + nzh[i];
  col->resize((size_t)(*rowptr)[n]);
  val->resize((size_t)(*rowptr)[n]);
  for (int i = 0; i < n; i++)
    for (int t = 0; t < nzh[i]; t++) {
      (*col)[(size_t)(*rowptr)[i] + t] = jh[(size_t)i * cap + t];
      (*val)[(size_t)(*rowptr)[i] + t] = vh[(size_t)i * cap + t];
    }
  return CVO_OK;
}

}  // namespace cvo_gb
