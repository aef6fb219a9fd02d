// cvo_irls.cu -- multi-frame RKHS-BA window (CvoBatchIRLS::solve, src/cvo/IRLS.cpp:148-367).
//
// Per outer iteration: every frame is moved to world coordinates with its float
// pose (CvoFrameGPU::transform_pointcloud, src/cvo/CvoFrameGPU.cu:130-149); every
// edge gets its sparse kernel matrix between the two world-frame clouds in one
// batched association launch (BinaryStateGPU::update_inner_product,
// src/cvo/IRLS_State_GPU.cu:144-336); the poses are then refined by a
// Levenberg-Marquardt solve over the residuals r = a |T1 p1 - T2 p2|^2 with the
// reference's analytic Jacobian (IRLS_Cost_CPU.hpp:260-371) composed with the SE(3)
// local parameterisation (local_parameterization_se3.hpp:13-100).  The reference
// hands that solve to Ceres (LM, SPARSE_NORMAL_CHOLESKY, IRLS.cpp:273-290); here the
// normal equations are accumulated on the GPU (one pass over all kernel-matrix entries
// of all edges) and the 6F x 6F system is solved on the host, with the LM iteration
// stated in oracle/cvo_oracle.c (lm_solve).
#include <cmath>
#include <cstring>
#include <algorithm>
#include <chrono>
#include <vector>
#include "cvo_internal.h"
#include "cvo_device.cuh"
#include "cvo_lie.cuh"

namespace cvo_gb {
namespace {

constexpr int kIrlsThreads = 128;
constexpr int kNormTerms = 91;   // 78 upper-triangle Hessian terms (12x12), 12 gradient, 1 cost

// frame points (tile order, local) -> world with the float pose, canonical order
__global__ void k_world(const float4 *local, int n, const float *pose, float4 *world) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  float4 p = local[s];
  // rows of the 3x4 pose: [r00 r01 r02 t0 | r10 r11 r12 t1 | r20 r21 r22 t2]
  float R[9] = {pose[0], pose[1], pose[2], pose[4], pose[5], pose[6], pose[8], pose[9], pose[10]};
  float o0 = xform_row(&R[0], pose[3], p.x, p.y, p.z);
  float o1 = xform_row(&R[3], pose[7], p.x, p.y, p.z);
  float o2 = xform_row(&R[6], pose[11], p.x, p.y, p.z);
  world[s] = make_float4(o0, o1, o2, range_norm(o0, o1, o2));
}

struct IrlsEdge {
  const int *A_j;     // ELL, row-major with pitch ld
  const float *A_v;
  const int *nnz_row;
  int ld;
  const float4 *p1;   // frame-1 local points, tile order (rows of A)
  const float4 *p2;   // frame-2 local points, original order (columns of A)
  int n, lim;         // rows, entries used per row
  int f1, f2;
  int blk0;           // first block of this edge
};

// Accumulates, per block, the cost and (WANT_J) the 12x12 J^T J and J^T r of the
// residuals of one edge.  One thread per row; the row's point is moved with the FP64
// poses once, every entry is then single precision (see the residual below); per-row
// sums in FP32, block sums in FP64.
template <bool WANT_J>
__global__ void __launch_bounds__(kIrlsThreads) k_irls_accum(const IrlsEdge *E, int ne, const double *poses,
                                                              double *partial) {
  __shared__ double sh[kIrlsThreads / 32][kNormTerms];
  int lo = 0, hi = ne - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (E[mid].blk0 <= (int)blockIdx.x) lo = mid; else hi = mid - 1;
  }
  const IrlsEdge ed = E[lo];
  const int s = ((int)blockIdx.x - ed.blk0) * kIrlsThreads + threadIdx.x;
  constexpr int NT = WANT_J ? kNormTerms : 1;
  float acc[NT];
#pragma unroll
  for (int k = 0; k < NT; k++) acc[k] = 0.f;
  double cost = 0.0;
  if (s < ed.n) {
    const double *T1 = poses + 12 * ed.f1, *T2 = poses + 12 * ed.f2;
    const int z = min(ed.nnz_row[s], ed.lim);
    const float4 a1 = ed.p1[s];
    // The residual vector e = T1 p1 - T2 p2 (world frame) is a difference of two points
    // tens of metres out that lie centimetres apart.  Per row, p1 is taken to the target
    // frame in double, p1' = R2^T (T1 p1 - t2), and split into float hi + lo; per entry
    // d = (hi - p2) + lo is then exact to float rounding of d itself (hi - p2 cancels
    // without error for nearby points), e = R2 d, |e| = |d|, R2^T e = d and
    // R1^T e = (R1^T R2) d.  So the per-entry arithmetic is single precision without the
    // cancellation a float e = q1 - q2 would suffer.
    const double p1[3] = {a1.x, a1.y, a1.z};
    double q1[3], pd[3];
    for (int r = 0; r < 3; r++) q1[r] = T1[4 * r] * p1[0] + T1[4 * r + 1] * p1[1] + T1[4 * r + 2] * p1[2] + T1[4 * r + 3];
    for (int r = 0; r < 3; r++)
      pd[r] = T2[r] * (q1[0] - T2[3]) + T2[4 + r] * (q1[1] - T2[7]) + T2[8 + r] * (q1[2] - T2[11]);
    float ph[3], pl[3], R12[9];
    for (int r = 0; r < 3; r++) {
      ph[r] = (float)pd[r];
      pl[r] = (float)(pd[r] - (double)ph[r]);
    }
    for (int r = 0; r < 3; r++)
      for (int c = 0; c < 3; c++)
        R12[3 * r + c] = (float)(T1[r] * T2[c] + T1[4 + r] * T2[4 + c] + T1[8 + r] * T2[8 + c]);
    float cost_f = 0.f;
    for (int c = 0; c < z; c++) {
      const int j = ed.A_j[(size_t)s * ed.ld + c];
      const float a = ed.A_v[(size_t)s * ed.ld + c];
      const float4 b2 = __ldg(&ed.p2[j]);
      const float d[3] = {(ph[0] - b2.x) + pl[0], (ph[1] - b2.y) + pl[1], (ph[2] - b2.z) + pl[2]};
      const float rr = a * (d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
      cost_f = fmaf(0.5f * rr, rr, cost_f);
      if (WANT_J) {
        float u1[3], J[12];
        const float *u2 = d;                                                        // R2^T e
        for (int r = 0; r < 3; r++) u1[r] = R12[3 * r] * d[0] + R12[3 * r + 1] * d[1] + R12[3 * r + 2] * d[2];   // R1^T e
        const float x1 = a1.x, y1 = a1.y, z1 = a1.z, x2 = b2.x, y2 = b2.y, z2 = b2.z;
        J[0] = u1[0]; J[1] = u1[1]; J[2] = u1[2];
        J[3] = y1 * u1[2] - z1 * u1[1]; J[4] = z1 * u1[0] - x1 * u1[2]; J[5] = x1 * u1[1] - y1 * u1[0];
        J[6] = -u2[0]; J[7] = -u2[1]; J[8] = -u2[2];
        J[9] = -(y2 * u2[2] - z2 * u2[1]); J[10] = -(z2 * u2[0] - x2 * u2[2]); J[11] = -(x2 * u2[1] - y2 * u2[0]);
        const float rf = rr;
        int k = 0;
#pragma unroll
        for (int p = 0; p < 12; p++)
#pragma unroll
          for (int q = p; q < 12; q++, k++) acc[k] = fmaf(J[p], J[q], acc[k]);
#pragma unroll
        for (int p = 0; p < 12; p++) acc[78 + p] = fmaf(J[p], rf, acc[78 + p]);
      }
    }
    cost = (double)cost_f;
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (WANT_J) {
#pragma unroll
    for (int k = 0; k < 90; k++) {
      double v = warp_sum((double)acc[k]);
      if (lane == 0) sh[w][k] = v;
    }
    double v = warp_sum(cost);
    if (lane == 0) sh[w][90] = v;
  } else {
    double v = warp_sum(cost);
    if (lane == 0) sh[w][0] = v;
  }
  __syncthreads();
  const int nt = WANT_J ? kNormTerms : 1;
  for (int k = threadIdx.x; k < nt; k += blockDim.x) {
    double t = 0.0;
    for (int ww = 0; ww < kIrlsThreads / 32; ww++) t += sh[ww][k];
    partial[(size_t)blockIdx.x * kNormTerms + k] = t;
  }
}

// per edge: sum of its blocks' partials in block order
__global__ void k_irls_sum(const IrlsEdge *E, int ne, int total_blocks, int nt, const double *partial, double *out) {
  const int e = blockIdx.x;
  if (e >= ne) return;
  const int b0 = E[e].blk0, b1 = (e + 1 < ne) ? E[e + 1].blk0 : total_blocks;
  for (int k = threadIdx.x; k < nt; k += blockDim.x) {
    double t = 0.0;
    for (int b = b0; b < b1; b++) t += partial[(size_t)b * kNormTerms + k];
    out[(size_t)e * kNormTerms + k] = t;
  }
}

// ------------------------------------------------------------- host LM
void se3_exp(const double d[6], double X[12]) {
  // Exp_SE3(v, is_wu = false) (src/cvo/LieGroup.cpp:169-192): u = v.head(3), w = v.tail(3)
  const double *u = d, *w = d + 3;
  double th = std::sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
  double A[9] = {0, -w[2], w[1], w[2], 0, -w[0], -w[1], w[0], 0}, A2[9], R[9], J[9];
  for (int r = 0; r < 3; r++)
    for (int c = 0; c < 3; c++) A2[3 * r + c] = A[3 * r] * A[c] + A[3 * r + 1] * A[3 + c] + A[3 * r + 2] * A[6 + c];
  if (th < (double)1e-6f) {
    for (int t = 0; t < 9; t++) R[t] = J[t] = (t % 4 == 0) ? 1.0 : 0.0;
  } else {
    double s1 = std::sin(th) / th, c1 = (1.0 - std::cos(th)) / (th * th), c2 = (th - std::sin(th)) / (th * th * th);
    for (int t = 0; t < 9; t++) {
      double I = (t % 4 == 0) ? 1.0 : 0.0;
      R[t] = I + s1 * A[t] + c1 * A2[t];
      J[t] = I + c1 * A[t] + c2 * A2[t];
    }
  }
  for (int r = 0; r < 3; r++) {
    for (int c = 0; c < 3; c++) X[4 * r + c] = R[3 * r + c];
    X[4 * r + 3] = J[3 * r] * u[0] + J[3 * r + 1] * u[1] + J[3 * r + 2] * u[2];
  }
}

void compose(const double A[12], const double B[12], double out[12]) {
  double o[12];
  for (int r = 0; r < 3; r++)
    for (int c = 0; c < 4; c++) {
      double s = A[4 * r] * B[c] + A[4 * r + 1] * B[4 + c] + A[4 * r + 2] * B[8 + c];
      if (c == 3) s += A[4 * r + 3];
      o[4 * r + c] = s;
    }
  memcpy(out, o, sizeof(o));
}

double pose_change(const double A[12], const double B[12]) {
  double Ai[12], M[12];
  for (int r = 0; r < 3; r++) {
    for (int c = 0; c < 3; c++) Ai[4 * r + c] = A[4 * c + r];
    Ai[4 * r + 3] = -(A[r] * A[3] + A[4 + r] * A[7] + A[8 + r] * A[11]);
  }
  compose(Ai, B, M);
  double R[9] = {M[0], M[1], M[2], M[4], M[5], M[6], M[8], M[9], M[10]}, t[3] = {M[3], M[7], M[11]};
  return dist_se3(R, t);
}

bool chol_solve(int n, std::vector<double> &A, std::vector<double> &b) {
  for (int j = 0; j < n; j++) {
    double s = A[(size_t)j * n + j];
    for (int k = 0; k < j; k++) s -= A[(size_t)j * n + k] * A[(size_t)j * n + k];
    if (!(s > 0.0)) return false;
    double d = std::sqrt(s);
    A[(size_t)j * n + j] = d;
    for (int i = j + 1; i < n; i++) {
      double t = A[(size_t)i * n + j];
      for (int k = 0; k < j; k++) t -= A[(size_t)i * n + k] * A[(size_t)j * n + k];
      A[(size_t)i * n + j] = t / d;
    }
  }
  for (int i = 0; i < n; i++) {
    double t = b[i];
    for (int k = 0; k < i; k++) t -= A[(size_t)i * n + k] * b[k];
    b[i] = t / A[(size_t)i * n + i];
  }
  for (int i = n - 1; i >= 0; i--) {
    double t = b[i];
    for (int k = i + 1; k < n; k++) t -= A[(size_t)k * n + i] * b[k];
    b[i] = t / A[(size_t)i * n + i];
  }
  return true;
}

// Normal equations of the window's residuals at given poses.  One evaluation is the
// upload of the poses, the accumulation over every kernel-matrix entry of every edge, the
// per-edge sums and their read-back; it runs as a CUDA graph (one per kind: with or
// without H and g) that is captured once and replayed by every evaluation of the LM
// solves until the edges' layout changes.  The poses and sums travel through pinned
// buffers, whose addresses the graph's copy nodes hold.
struct Normal {
  Handle *h;
  int nf;
  std::vector<IrlsEdge> edges;    // edges with residuals
  IrlsEdge *edges_d = nullptr;
  double *poses_d = nullptr;
  double *partial_d = nullptr;
  double *out_d = nullptr;
  double *poses_pin = nullptr;    // 12 nf
  double *out_pin = nullptr;      // kNormTerms per edge
  int out_pin_edges = 0;
  int total_blocks = 0;
  cudaGraphExec_t exec[2] = {nullptr, nullptr};
  std::vector<unsigned char> key[2];

  Normal() = default;
  Normal(const Normal &) = delete;
  Normal &operator=(const Normal &) = delete;
  ~Normal() {
    for (auto &e : exec)
      if (e) cudaGraphExecDestroy(e);
    cudaFree(partial_d);
    cudaFree(out_d);
    cudaFree(edges_d);
    cudaFree(poses_d);
    cudaFreeHost(poses_pin);
    cudaFreeHost(out_pin);
  }

  int record(bool want) {
    const int ne = (int)edges.size();
    const int w = want ? 1 : 0;
    std::vector<unsigned char> k;
    auto add = [&](const void *p, size_t n) {
      const unsigned char *c = static_cast<const unsigned char *>(p);
      k.insert(k.end(), c, c + n);
    };
    const void *ptrs[6] = {edges_d, poses_d, partial_d, out_d, poses_pin, out_pin};
    add(ptrs, sizeof(ptrs));
    add(&ne, sizeof(ne));
    add(&total_blocks, sizeof(total_blocks));
    add(&nf, sizeof(nf));
    add(&h->stream, sizeof(h->stream));
    if (exec[w] && key[w] == k) return 0;
    if (exec[w]) cudaGraphExecDestroy(exec[w]);
    exec[w] = nullptr;
    CVO_CUDA_TRY(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e1 = cudaMemcpyAsync(poses_d, poses_pin, sizeof(double) * 12 * nf, cudaMemcpyHostToDevice, h->stream);
    if (want) k_irls_accum<true><<<total_blocks, kIrlsThreads, 0, h->stream>>>(edges_d, ne, poses_d, partial_d);
    else k_irls_accum<false><<<total_blocks, kIrlsThreads, 0, h->stream>>>(edges_d, ne, poses_d, partial_d);
    k_irls_sum<<<ne, 128, 0, h->stream>>>(edges_d, ne, total_blocks, want ? kNormTerms : 1, partial_d, out_d);
    cudaError_t e2 = cudaMemcpyAsync(out_pin, out_d, sizeof(double) * ne * kNormTerms, cudaMemcpyDeviceToHost,
                                     h->stream);
    cudaGraph_t g = nullptr;
    cudaError_t e3 = cudaStreamEndCapture(h->stream, &g);
    cudaError_t e4 = cudaSuccess;
    if (e1 == cudaSuccess && e2 == cudaSuccess && e3 == cudaSuccess) e4 = cudaGraphInstantiate(&exec[w], g, 0);
    if (g) cudaGraphDestroy(g);
    for (cudaError_t e : {e1, e2, e3, e4})
      if (e != cudaSuccess) {
        exec[w] = nullptr;
        return set_cuda_error(h, e, "normal-equation graph capture");
      }
    key[w] = k;
    return 0;
  }

  // cost (and, if want, H and g over all 6 nf parameters) at `poses`
  int eval(const double *poses, bool want, std::vector<double> *H, std::vector<double> *g, double *cost) {
    const int ne = (int)edges.size();
    *cost = 0.0;
    if (want) {
      H->assign((size_t)36 * nf * nf, 0.0);
      g->assign((size_t)6 * nf, 0.0);
    }
    if (ne == 0) return 0;
    if (int rc = record(want)) return rc;
    memcpy(poses_pin, poses, sizeof(double) * 12 * nf);
    CVO_CUDA_TRY(h, cudaGraphLaunch(exec[want ? 1 : 0], h->stream));
    h->launches += 2;
    CVO_CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    const double *out_h = out_pin;
    const int D = 6 * nf;
    for (int e = 0; e < ne; e++) {
      const double *o = &out_h[(size_t)e * kNormTerms];
      if (!want) { *cost += o[0]; continue; }
      *cost += o[90];
      int off[2] = {6 * edges[e].f1, 6 * edges[e].f2};
      int k = 0;
      for (int p = 0; p < 12; p++)
        for (int q = p; q < 12; q++, k++) {
          int ip = off[p / 6] + p % 6, iq = off[q / 6] + q % 6;
          (*H)[(size_t)ip * D + iq] += o[k];
          if (ip != iq || p != q) (*H)[(size_t)iq * D + ip] += o[k];
        }
      for (int p = 0; p < 12; p++) (*g)[off[p / 6] + p % 6] += o[78 + p];
    }
    return 0;
  }
};

// One Levenberg-Marquardt solve (the iteration stated in oracle/cvo_oracle.c, lm_solve).
int lm_solve(Normal &N, int nf, double *poses, const uint8_t *hold, int max_iter, int *successes) {
  const int D = 6 * nf;
  std::vector<int> idx(D);
  int nfree = 0;
  for (int f = 0; f < nf; f++)
    for (int k = 0; k < 6; k++) idx[6 * f + k] = hold[f] ? -1 : nfree++;
  std::vector<double> H, g, Hf((size_t)std::max(nfree, 1) * std::max(nfree, 1)), gf(std::max(nfree, 1)), A, b,
      cand(12 * (size_t)nf);
  double radius = 1e4, nu = 2.0, cost = 0.0;
  int rc = N.eval(poses, true, &H, &g, &cost);
  if (rc) return rc;
  for (int it = 0; it < max_iter && nfree > 0; it++) {
    for (int i = 0; i < D; i++) {
      if (idx[i] < 0) continue;
      gf[idx[i]] = g[i];
      for (int j = 0; j < D; j++)
        if (idx[j] >= 0) Hf[(size_t)idx[i] * nfree + idx[j]] = H[(size_t)i * D + j];
    }
    double gmax = 0.0;
    for (int i = 0; i < nfree; i++) gmax = std::max(gmax, std::fabs(gf[i]));
    if (gmax <= 1e-5) break;
    A = Hf;
    b.assign(nfree, 0.0);
    for (int i = 0; i < nfree; i++) {
      double dg = Hf[(size_t)i * nfree + i];
      dg = dg < 1e-6 ? 1e-6 : (dg > 1e32 ? 1e32 : dg);
      A[(size_t)i * nfree + i] += dg / radius;
      b[i] = -gf[i];
    }
    if (!chol_solve(nfree, A, b)) { radius /= nu; nu *= 2.0; continue; }
    double dn = 0.0, xn = 0.0;
    for (int i = 0; i < nfree; i++) dn += b[i] * b[i];
    for (int t = 0; t < 12 * nf; t++) xn += poses[t] * poses[t];
    if (std::sqrt(dn) <= 1e-5 * (std::sqrt(xn) + 1e-5)) break;
    double model = 0.0;
    for (int i = 0; i < nfree; i++) {
      double hd = 0.0;
      for (int j = 0; j < nfree; j++) hd += Hf[(size_t)i * nfree + j] * b[j];
      model += gf[i] * b[i] + 0.5 * b[i] * hd;
    }
    model = -model;
    memcpy(cand.data(), poses, sizeof(double) * 12 * nf);
    for (int f = 0; f < nf; f++) {
      if (hold[f]) continue;
      double d6[6], X[12];
      for (int k = 0; k < 6; k++) d6[k] = b[idx[6 * f + k]];
      se3_exp(d6, X);
      compose(poses + 12 * f, X, &cand[12 * f]);
    }
    double cnew = 0.0;
    if ((rc = N.eval(cand.data(), false, nullptr, nullptr, &cnew))) return rc;
    double rho = model > 0.0 ? (cost - cnew) / model : -1.0;
    if (rho > 1e-3) {
      memcpy(poses, cand.data(), sizeof(double) * 12 * nf);
      (*successes)++;
      double rel = std::fabs(cost - cnew);
      double fac = 1.0 - std::pow(2.0 * rho - 1.0, 3.0);
      radius = radius / (fac > 1.0 / 3.0 ? fac : 1.0 / 3.0);
      nu = 2.0;
      bool stop = rel <= 1e-5 * cost;
      cost = cnew;
      if (stop) break;
      if ((rc = N.eval(poses, true, &H, &g, &cost))) return rc;
    } else {
      radius /= nu;
      nu *= 2.0;
    }
  }
  return 0;
}

}  // namespace

int run_align_multi(Handle *h, int nf, DevCloud *const *clouds, double *poses, const uint8_t *hold, int ne,
                    const int *edges, double *secs, int *iters) {
  NvtxRange nvtx_range("align_multi");
  auto t0 = std::chrono::steady_clock::now();
  const cvo_params &p = h->params;
  if (p.multiframe_is_optimizing_ell) return CVO_ERR_UNSUPPORTED;
  for (int f = 0; f < nf; f++)
    if (clouds[f]->F != clouds[0]->F || clouds[f]->C != clouds[0]->C) return CVO_ERR_INVALID_ARG;
  if (ne == 0) {   // no edge has pairs: the first outer iteration stops (counter == 0)
    if (iters) *iters = 0;
    if (secs) *secs = 0.0;
    return CVO_OK;
  }
  // world-frame copies of every frame (tile order) and the frames' float poses
  std::vector<float4 *> world(nf, nullptr);
  float *pose_d = nullptr;
  int rc = 0;
  auto cleanup = [&]() {
    for (auto *w : world) cudaFree(w);
    cudaFree(pose_d);
  };
  for (int f = 0; f < nf; f++) {
    if (cudaMalloc((void **)&world[f], sizeof(float4) * std::max(clouds[f]->n, 1)) != cudaSuccess) {
      cleanup();
      return CVO_ERR_OUT_OF_MEMORY;
    }
  }
  if (cudaMalloc((void **)&pose_d, sizeof(float) * 12 * nf) != cudaSuccess) { cleanup(); return CVO_ERR_OUT_OF_MEMORY; }
  Normal N;
  N.h = h;
  N.nf = nf;
  if (cudaMallocHost((void **)&N.poses_pin, sizeof(double) * 12 * nf) != cudaSuccess ||
      cudaMallocHost((void **)&N.out_pin, sizeof(double) * kNormTerms * ne) != cudaSuccess) {
    cudaGetLastError();
    cleanup();
    return CVO_ERR_OUT_OF_MEMORY;
  }
  // the edge association of every outer iteration replays one captured graph while its
  // launch parameters stay the same
  AssocGraph ag;
  // per-edge state (BinaryStateGPU members)
  std::vector<double> ell(ne, (double)p.multiframe_ell_init);
  std::vector<int> nn(ne, p.multiframe_num_neighbors), prev_max(ne, 0), iters_per_ell(ne, 0);
  std::vector<long long> prev_nnz(ne, 0), nz_last(ne, 0);
  const int init_nn = p.multiframe_num_neighbors;
  const double ell_min = p.multiframe_ell_min, ell_max = (double)p.multiframe_ell_init * 1.2;
  std::vector<double> old(12 * (size_t)nf);
  int iter = 0, steps = 0;
  size_t max_blocks = 0;
  for (;;) {
    memcpy(old.data(), poses, sizeof(double) * 12 * nf);
    std::vector<float> fpose(12 * (size_t)nf);
    for (int t = 0; t < 12 * nf; t++) fpose[t] = (float)poses[t];
    if (cudaMemcpyAsync(pose_d, fpose.data(), sizeof(float) * 12 * nf, cudaMemcpyHostToDevice, h->stream) !=
        cudaSuccess) { cleanup(); return CVO_ERR_CUDA; }
    std::vector<float> wnorm(nf, 0.f);
    for (int f = 0; f < nf; f++) {
      int n = clouds[f]->n;
      if (n > 0) {
        k_world<<<(n + 255) / 256, 256, 0, h->stream>>>(clouds[f]->spos, n, pose_d + 12 * f, world[f]);
        h->launches++;
      }
      double tn = std::sqrt(poses[12 * f + 3] * poses[12 * f + 3] + poses[12 * f + 7] * poses[12 * f + 7] +
                            poses[12 * f + 11] * poses[12 * f + 11]);
      wnorm[f] = (float)(clouds[f]->max_norm + tn) * 1.0001f;
    }
    // association of every edge in one batch
    std::vector<DevCloud *> es(ne), et(ne);
    std::vector<const float4 *> ew(ne);
    std::vector<float> enorm(ne), epose(12 * (size_t)ne), eell(ne);
    for (int e = 0; e < ne; e++) {
      int f1 = edges[2 * e], f2 = edges[2 * e + 1];
      nz_last[e] = prev_nnz[e];
      if (prev_max[e] > 0) nn[e] = std::min(init_nn, (int)((double)prev_max[e] * 1.1));
      es[e] = clouds[f1];
      et[e] = clouds[f2];
      ew[e] = world[f1];
      enorm[e] = wnorm[f1];
      for (int t = 0; t < 12; t++) epose[12 * e + t] = fpose[12 * f2 + t];
      eell[e] = (float)ell[e];
    }
    std::vector<EdgeAssoc> EA;
    if ((rc = run_association_edges(h, es, et, ew, enorm, epose, eell, nn, init_nn, &EA, nullptr, &ag))) {
      cleanup();
      return rc;
    }
    int counter = 0;
    N.edges.clear();
    int blk = 0;
    for (int e = 0; e < ne; e++) {
      prev_nnz[e] = EA[e].nnz;
      prev_max[e] = EA[e].max_row;
      if (EA[e].nnz > p.multiframe_min_nonzeros) counter++;
      // add_residual_to_problem (IRLS_State_GPU.cpp:17-20): edges with too few pairs add nothing
      if (EA[e].nnz != 0 && EA[e].nnz >= p.multiframe_min_nonzeros) {
        IrlsEdge E;
        E.A_j = EA[e].A_j; E.A_v = EA[e].A_v; E.nnz_row = EA[e].nnz_row;
        E.ld = EA[e].ld;
        E.p1 = clouds[edges[2 * e]]->spos;
        E.p2 = clouds[edges[2 * e + 1]]->pos;
        E.n = EA[e].n;
        E.lim = std::min(p.nearest_neighbors_max, nn[e]);
        E.f1 = edges[2 * e]; E.f2 = edges[2 * e + 1];
        E.blk0 = blk;
        blk += (E.n + kIrlsThreads - 1) / kIrlsThreads;
        N.edges.push_back(E);
      }
    }
    if (counter == 0) break;
    N.total_blocks = blk;
    if ((size_t)blk > max_blocks || !N.partial_d) {
      cudaFree(N.partial_d); cudaFree(N.out_d); cudaFree(N.edges_d); cudaFree(N.poses_d);
      N.partial_d = N.out_d = N.poses_d = nullptr;
      N.edges_d = nullptr;
      max_blocks = std::max<size_t>(blk, 1) * 2;
      if (cudaMalloc((void **)&N.partial_d, sizeof(double) * kNormTerms * max_blocks) != cudaSuccess ||
          cudaMalloc((void **)&N.out_d, sizeof(double) * kNormTerms * std::max(ne, 1)) != cudaSuccess ||
          cudaMalloc((void **)&N.edges_d, sizeof(IrlsEdge) * std::max(ne, 1)) != cudaSuccess ||
          cudaMalloc((void **)&N.poses_d, sizeof(double) * 12 * nf) != cudaSuccess) {
        cleanup();
        return CVO_ERR_OUT_OF_MEMORY;
      }
    }
    if (!N.edges.empty() && cudaMemcpyAsync(N.edges_d, N.edges.data(), sizeof(IrlsEdge) * N.edges.size(),
                                            cudaMemcpyHostToDevice, h->stream) != cudaSuccess) {
      cleanup();
      return CVO_ERR_CUDA;
    }
    if ((rc = lm_solve(N, nf, poses, hold, p.multiframe_iterations_per_solve, &steps))) { cleanup(); return rc; }
    double change = 0.0;
    for (int f = 0; f < nf; f++) change += pose_change(&old[12 * f], poses + 12 * f);
    bool all_min = true;
    for (int e = 0; e < ne; e++) {
      // BinaryStateGPU::update_ell (IRLS_State_GPU.cpp:117-146)
      iters_per_ell[e]++;
      if (nz_last[e] > 0 && prev_nnz[e] <= nz_last[e] && iters_per_ell[e] / p.multiframe_iter_per_ell > 0) {
        ell[e] = ell[e] * (double)p.multiframe_ell_decay_rate;
        nz_last[e] = 0;
        iters_per_ell[e] = 0;
      }
      if (ell[e] < ell_min) ell[e] = ell_min;
      else if (ell[e] > ell_max) ell[e] = ell_max;
      all_min = all_min && std::fabs((double)(float)ell[e] - ell_min) < 1e-4;
    }
    iter++;
    if (all_min && change < 1e-5) break;
    if (iter >= p.multiframe_max_iters) break;
  }
  cleanup();
  if (iters) *iters = iter;
  auto t1 = std::chrono::steady_clock::now();
  if (secs) *secs = std::chrono::duration<double>(t1 - t0).count();
  return CVO_OK;
}

}  // namespace cvo_gb
