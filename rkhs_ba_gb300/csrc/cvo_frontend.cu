// cvo_frontend.cu -- RGB-D frame -> device cloud.
//
// CvoPointCloud(const ImageRGBD<float>&, const Calibration&, PointSelectionMethod)
// (src/utils/CvoPointCloud.cpp:458-560) with RawImage's intensity and gradient
// (src/utils/RawImage.cpp:9-45, 117-143), on the device, so an image frame becomes
// a registration-ready cloud without a host-built point array:
//   intensity  grey level of the (BGR) image: ITU-R BT.601 luma in 14-bit fixed point,
//              (1868 B + 9617 G + 4899 R + 2^13) >> 14, as OpenCV's 8-bit BGR2GRAY;
//              the pixel value for one-channel images
//   gradient   0.5 (I[i+1] - I[i-1]), 0.5 (I[i+w] - I[i-w]) on interior pixels, 0 on
//              the border rows and columns, non-finite values set to 0
//   point      z = depth / scaling_factor, x = (u - cx) z / fx, y = (v - cy) z / fy for
//              each selected pixel with depth != 0 and not NaN; kept if finite and
//              |p| <= 55 (is_good_point, :61-71)
//   features   B/255, G/255, R/255 (or grey/255), then gradient[v w + u] / 500 + 0.5 and
//              gradient[v w + u + 1] / 500 + 0.5 -- the reference indexes the
//              interleaved (dx, dy) gradient array by the pixel index, and that is kept
//   labels     the pixel's class distribution; geometric type from the selection
// Points keep the selection order.  The image is used as given: RawImage's default
// denoising (OpenCV fastNlMeans) and the pixel selectors (FAST, DSO, edges) belong
// to the caller.
#include <cmath>
#include <cstring>
#include <vector>
#include "cvo_internal.h"
#include "cvo_device.cuh"

namespace cvo_gb {
namespace {

__global__ void k_intensity(const uint8_t *img, int total, int channels, float *gray) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total) return;
  if (channels == 3) {
    const int b = img[3 * (size_t)i], g = img[3 * (size_t)i + 1], r = img[3 * (size_t)i + 2];
    gray[i] = (float)((b * 1868 + g * 9617 + r * 4899 + (1 << 13)) >> 14);
  } else {
    gray[i] = (float)img[i];
  }
}

// grad must be zero on entry (rows 0 and rows-1 are not written).
__global__ void k_gradient(const float *I, int rows, int cols, float *grad) {
  const int idx = cols + blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= cols * (rows - 1)) return;
  const int c = idx % cols;
  if (c == 0 || c == cols - 1) {
    grad[2 * (size_t)idx] = 0.f;
    grad[2 * (size_t)idx + 1] = 0.f;
    return;
  }
  float dx = fm(0.5f, fs(I[idx + 1], I[idx - 1]));
  float dy = fm(0.5f, fs(I[idx + cols], I[idx - cols]));
  if (!isfinite(dx)) dx = 0.f;
  if (!isfinite(dy)) dy = 0.f;
  grad[2 * (size_t)idx] = dx;
  grad[2 * (size_t)idx + 1] = dy;
}

struct FrontParams {
  int rows, cols, channels, n_sel, F, C;
  float fx, fy, cx, cy, scale;
};

// One selected pixel: point, features, labels, geometric type, kept flag.
__global__ void k_rgbd_points(FrontParams A, const uint8_t *img, const float *depth, const float *grad, const int *uv,
                              const float *geom_in, const float *sem, float *xyz, float *feat, float *lab,
                              float2 *geo, int *flag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= A.n_sel) return;
  const int u = uv[2 * (size_t)i], v = uv[2 * (size_t)i + 1];
  int ok = 0;
  if (u >= 0 && u < A.cols && v >= 0 && v < A.rows) {
    const size_t pix = (size_t)v * A.cols + u;
    const float dep = depth[pix];
    if (dep != 0.f && !isnan(dep)) {
      const float z = __fdiv_rn(dep, A.scale);
      const float x = __fdiv_rn(fm(fs((float)u, A.cx), z), A.fx);
      const float y = __fdiv_rn(fm(fs((float)v, A.cy), z), A.fy);
      const bool finite = isfinite(x) && isfinite(y) && isfinite(z);
      const float nrm = __fsqrt_rn(fa(fa(fm(x, x), fm(y, y)), fm(z, z)));
      if (finite && !(nrm > 55.f)) {
        ok = 1;
        xyz[3 * (size_t)i] = x; xyz[3 * (size_t)i + 1] = y; xyz[3 * (size_t)i + 2] = z;
        float *f = feat + (size_t)i * A.F;
        const int nc = A.channels == 3 ? 3 : 1;
        for (int k = 0; k < nc; k++)
          f[k] = __double2float_rn(__ddiv_rn((double)img[pix * A.channels + k], 255.0));
        const float g0 = grad[pix], g1 = grad[pix + 1];
        f[nc] = __double2float_rn(da(__ddiv_rn((double)g0, 500.0), 0.5));
        f[nc + 1] = __double2float_rn(da(__ddiv_rn((double)g1, 500.0), 0.5));
        for (int k = 0; k < A.C; k++) lab[(size_t)i * A.C + k] = sem[pix * A.C + k];
        if (geo) geo[i] = geom_in ? make_float2(geom_in[2 * (size_t)i], geom_in[2 * (size_t)i + 1]) : make_float2(0.f, 0.f);
      }
    }
  }
  flag[i] = ok;
}

// Kept points to their packed positions (exclusive prefix of the flags).
__global__ void k_compact_points(int n_sel, int F, int C, const int *flag, const int *pos, const float *xyz,
                                 const float *feat, const float *lab, const float2 *geo, float *oxyz, float *ofeat,
                                 float *olab, float2 *ogeo) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_sel || !flag[i]) return;
  const int o = pos[i];
  for (int k = 0; k < 3; k++) oxyz[3 * (size_t)o + k] = xyz[3 * (size_t)i + k];
  for (int k = 0; k < F; k++) ofeat[(size_t)o * F + k] = feat[(size_t)i * F + k];
  for (int k = 0; k < C; k++) olab[(size_t)o * C + k] = lab[(size_t)i * C + k];
  if (geo) ogeo[o] = geo[i];
}

}  // namespace

int cloud_from_rgbd(Handle *h, const uint8_t *image, int rows, int cols, int channels, const float *depth,
                    const float intrinsic[4], float scaling_factor, const int *uv, int n_sel, const float *geom_type,
                    int num_classes, const float *semantics, DevCloud **out) {
  NvtxRange nvtx_range("cloud_from_rgbd");
  if (rows < 3 || cols < 3 || (channels != 1 && channels != 3) || n_sel < 0 || num_classes < 0) return CVO_ERR_INVALID_ARG;
  if (!image || !depth || !intrinsic || (n_sel > 0 && !uv) || (num_classes > 0 && !semantics)) return CVO_ERR_INVALID_ARG;
  const size_t total = (size_t)rows * cols;
  FrontParams A;
  A.rows = rows; A.cols = cols; A.channels = channels; A.n_sel = n_sel;
  A.F = channels + 2; A.C = num_classes;
  A.fx = intrinsic[0]; A.fy = intrinsic[1]; A.cx = intrinsic[2]; A.cy = intrinsic[3];
  A.scale = scaling_factor;
  const bool has_geo = geom_type != nullptr;
  const int ns = n_sel > 0 ? n_sel : 1;
  uint8_t *img_d = nullptr;
  float *dep_d = nullptr, *gray = nullptr, *grad = nullptr, *sem_d = nullptr, *geo_in = nullptr;
  float *xyz = nullptr, *feat = nullptr, *lab = nullptr, *oxyz = nullptr, *ofeat = nullptr, *olab = nullptr;
  float2 *geo = nullptr, *ogeo = nullptr;
  int *uv_d = nullptr, *flag = nullptr, *pos = nullptr, *scratch = nullptr;
  auto release = [&]() {
    cudaFree(img_d); cudaFree(dep_d); cudaFree(gray); cudaFree(grad); cudaFree(sem_d); cudaFree(geo_in);
    cudaFree(xyz); cudaFree(feat); cudaFree(lab); cudaFree(oxyz); cudaFree(ofeat); cudaFree(olab);
    cudaFree(geo); cudaFree(ogeo); cudaFree(uv_d); cudaFree(flag); cudaFree(pos); cudaFree(scratch);
  };
  const size_t scr = scan_scratch_ints(ns);
  bool ok = cudaMalloc((void **)&img_d, total * channels) == cudaSuccess &&
            cudaMalloc((void **)&dep_d, sizeof(float) * total) == cudaSuccess &&
            cudaMalloc((void **)&gray, sizeof(float) * total) == cudaSuccess &&
            cudaMalloc((void **)&grad, sizeof(float) * 2 * total) == cudaSuccess &&
            cudaMalloc((void **)&sem_d, sizeof(float) * (num_classes > 0 ? total * num_classes : 1)) == cudaSuccess &&
            cudaMalloc((void **)&geo_in, sizeof(float) * 2 * ns) == cudaSuccess &&
            cudaMalloc((void **)&xyz, sizeof(float) * 3 * ns) == cudaSuccess &&
            cudaMalloc((void **)&feat, sizeof(float) * A.F * ns) == cudaSuccess &&
            cudaMalloc((void **)&lab, sizeof(float) * (num_classes > 0 ? (size_t)num_classes * ns : 1)) == cudaSuccess &&
            cudaMalloc((void **)&oxyz, sizeof(float) * 3 * ns) == cudaSuccess &&
            cudaMalloc((void **)&ofeat, sizeof(float) * A.F * ns) == cudaSuccess &&
            cudaMalloc((void **)&olab, sizeof(float) * (num_classes > 0 ? (size_t)num_classes * ns : 1)) == cudaSuccess &&
            cudaMalloc((void **)&geo, sizeof(float2) * ns) == cudaSuccess &&
            cudaMalloc((void **)&ogeo, sizeof(float2) * ns) == cudaSuccess &&
            cudaMalloc((void **)&uv_d, sizeof(int) * 2 * ns) == cudaSuccess &&
            cudaMalloc((void **)&flag, sizeof(int) * ns) == cudaSuccess &&
            cudaMalloc((void **)&pos, sizeof(int) * (ns + 1)) == cudaSuccess &&
            cudaMalloc((void **)&scratch, sizeof(int) * (scr > 0 ? scr : 1)) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    release();
    return CVO_ERR_OUT_OF_MEMORY;
  }
  cudaStream_t st = h->stream;
  cudaError_t e = cudaMemcpyAsync(img_d, image, total * channels, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dep_d, depth, sizeof(float) * total, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && num_classes > 0)
    e = cudaMemcpyAsync(sem_d, semantics, sizeof(float) * total * num_classes, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && n_sel > 0) e = cudaMemcpyAsync(uv_d, uv, sizeof(int) * 2 * n_sel, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && has_geo && n_sel > 0)
    e = cudaMemcpyAsync(geo_in, geom_type, sizeof(float) * 2 * n_sel, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(grad, 0, sizeof(float) * 2 * total, st);
  if (e != cudaSuccess) { release(); return set_cuda_error(h, e, "front-end upload"); }
  k_intensity<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(img_d, (int)total, channels, gray);
  const int inner = cols * (rows - 2);
  k_gradient<<<(inner + 255) / 256, 256, 0, st>>>(gray, rows, cols, grad);
  h->launches += 2;
  int kept = 0;
  if (n_sel > 0) {
    k_rgbd_points<<<(n_sel + 255) / 256, 256, 0, st>>>(A, img_d, dep_d, grad, uv_d, has_geo ? geo_in : nullptr, sem_d,
                                                       xyz, feat, lab, has_geo ? geo : nullptr, flag);
    exclusive_scan_int(h, flag, pos, n_sel, scratch, (int)scr);
    k_compact_points<<<(n_sel + 255) / 256, 256, 0, st>>>(n_sel, A.F, A.C, flag, pos, xyz, feat, lab,
                                                          has_geo ? geo : nullptr, oxyz, ofeat, olab, ogeo);
    h->launches += 2;
    int last_pos = 0, last_flag = 0;
    e = cudaMemcpyAsync(&last_pos, pos + (n_sel - 1), sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&last_flag, flag + (n_sel - 1), sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) { release(); return set_cuda_error(h, e, "front-end points"); }
    kept = last_pos + last_flag;
  }
  int rc = cloud_from_device(h, kept, A.F, A.C, oxyz, ofeat, A.C > 0 ? olab : nullptr, has_geo ? ogeo : nullptr, out);
  if (rc == 0) {
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) rc = set_cuda_error(h, e, "front-end cloud");
  }
  release();
  return rc;
}

int cloud_download(Handle *h, const DevCloud *d, float *xyz, float *features, float *labels, float *geom_type) {
  const int n = d->n;
  if (n == 0) return CVO_OK;
  std::vector<float4> p(n);
  std::vector<float> f((size_t)n * (d->FP > 0 ? d->FP : 1)), l((size_t)n * (d->CP > 0 ? d->CP : 1));
  std::vector<float2> g(d->has_geo ? n : 1);
  cudaError_t e = cudaMemcpyAsync(p.data(), d->pos, sizeof(float4) * n, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess && d->FP > 0 && features)
    e = cudaMemcpyAsync(f.data(), d->feat, sizeof(float) * (size_t)n * d->FP, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess && d->CP > 0 && labels)
    e = cudaMemcpyAsync(l.data(), d->lab, sizeof(float) * (size_t)n * d->CP, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess && d->has_geo && geom_type)
    e = cudaMemcpyAsync(g.data(), d->geo, sizeof(float2) * n, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return set_cuda_error(h, e, "cloud download");
  for (int i = 0; i < n; i++) {
    if (xyz) { xyz[3 * (size_t)i] = p[i].x; xyz[3 * (size_t)i + 1] = p[i].y; xyz[3 * (size_t)i + 2] = p[i].z; }
    if (features)
      for (int k = 0; k < d->F; k++) features[(size_t)i * d->F + k] = f[(size_t)i * d->FP + k];
    if (labels)
      for (int k = 0; k < d->C; k++) labels[(size_t)i * d->C + k] = l[(size_t)i * d->CP + k];
    if (geom_type && d->has_geo) { geom_type[2 * (size_t)i] = g[i].x; geom_type[2 * (size_t)i + 1] = g[i].y; }
  }
  return CVO_OK;
}

}  // namespace cvo_gb
