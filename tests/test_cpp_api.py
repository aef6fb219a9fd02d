"""The header-only C++ mirror of cvo::CvoGPU (include/cvo_gb300.hpp): a C++17 client
built with -Wall -Wextra -Werror links the library and runs the host paths the way a
reference user would call them: construction from a parameter file, parameters read
and written back, the CPU inner product and cos-angle, empty-input returns, errors as
exceptions carrying the status, the multi-frame argument checks and the pose-graph
solver, the adaptive-lengthscale class.  On a machine without a GPU the GPU methods must
throw the CUDA status."""
import os
import subprocess
import tempfile

import pytest

from rkhs_ba_gb300 import _lib as L
from rkhs_ba_gb300 import params_path

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

_CLIENT = r"""
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>
#include "cvo_gb300.hpp"

using namespace cvo_gb300;

static int fail(int code, const char *what) { std::fprintf(stderr, "FAIL %d: %s\n", code, what); return code; }

int main(int argc, char **argv) {
  if (argc < 2) return fail(20, "usage: client params.yaml");
  const std::string yaml = argv[1];
  CvoGPU cvo(yaml);
  const bool has_gpu = cvo_get_stream(cvo.handle()) != nullptr;   // a handle made without a CUDA device has none
  cvo_params p = cvo.get_params();
  const float ell0 = p.ell_init;
  p.ell_init = 0.25f;
  cvo.write_params(p);
  if (cvo.get_params().ell_init != 0.25f) return fail(1, "write_params");
  p.ell_init = ell0;
  cvo.write_params(p);

  std::mt19937 rng(7);
  std::uniform_real_distribution<float> u(-2.f, 2.f);
  PointCloud a;
  for (int i = 0; i < 400; i++) { a.xyz.push_back(u(rng)); a.xyz.push_back(u(rng)); a.xyz.push_back(0.3f * u(rng)); }
  const Mat4 I = identity();
  const float ip = cvo.inner_product_cpu(a, a, I, 0.3f);
  if (!(ip > 0.f)) return fail(2, "inner_product_cpu");
  const float cosv = cvo.function_angle(a, a, I, 0.3f, /*is_approximate=*/false, /*is_gpu=*/false);
  if (std::fabs(cosv - 1.f) > 1e-5f) return fail(3, "exact CPU cos-angle of a cloud with itself");

  // empty input: align returns 0 with no iterations, as the reference does
  PointCloud empty;
  Mat4 T_out{};
  int iters = -1;
  if (cvo.align(empty, a, I, T_out, nullptr, nullptr, &iters) != 0 || iters != 0) return fail(4, "empty align");

  // failures are exceptions carrying the library status
  try {
    CvoGPU bad("/nonexistent/params.yaml");
    return fail(5, "missing parameter file accepted");
  } catch (const Error &e) {
    if (e.code != CVO_ERR_IO) return fail(6, "missing file status");
  }
  try {
    std::vector<std::array<double, 12>> poses(1);
    std::vector<uint8_t> hold(2, 0);
    cvo.align(std::vector<PointCloud>{a, a}, poses, hold, {{0, 1}});
    return fail(7, "mismatched pose count accepted");
  } catch (const Error &e) {
    if (e.code != CVO_ERR_INVALID_ARG) return fail(8, "pose count status");
  }
  if (!has_gpu) {
    try {
      cvo.inner_product_gpu(a, a, I, 0.3f);
      return fail(9, "GPU call without a GPU");
    } catch (const Error &e) {
      if (e.code != CVO_ERR_CUDA) return fail(10, "no-GPU status");
    }
    try {
      cvo.global_register({a}, {a});
      return fail(15, "global registration without a GPU");
    } catch (const Error &e) {
      if (e.code != CVO_ERR_CUDA) return fail(16, "no-GPU status of global_register");
    }
  }
  try {
    cvo.global_register({a, a}, {a});
    return fail(17, "mismatched pairs accepted");
  } catch (const Error &e) {
    if (e.code != CVO_ERR_INVALID_ARG) return fail(18, "mismatched pairs status");
  }
  if (!cvo.global_register({}, {}).empty()) return fail(19, "no pairs");
  AdaptiveCvoGPU acvo(yaml);
  try {
    Mat4 T2{};
    acvo.align(empty, a, I, T2);
    return fail(21, "adaptive align of an empty cloud accepted");
  } catch (const Error &e) {
    if (e.code != CVO_ERR_EMPTY_CLOUD) return fail(22, "adaptive empty-cloud status");
  }

  // pose graph: a chain with a prior recovers the odometry
  PoseGraphSolver g;
  const std::array<double, 12> X0{1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0}, Z{1, 0, 0, 0.5, 0, 1, 0, 0, 0, 0, 1, 0};
  const std::array<double, 6> sig{0.1, 0.1, 0.1, 0.1, 0.1, 0.1};
  g.insert(0, X0);
  g.insert(1, X0);
  g.insert(2, X0);
  g.add_prior(0, X0, sig);
  g.add_between(0, 1, Z, sig);
  g.add_between(1, 2, Z, sig);
  double c0 = 0.0;
  const double c1 = g.optimize(100, &c0);
  if (!(c1 < 1e-16 && c0 > c1)) return fail(11, "pose graph cost");
  if (std::fabs(g.get(2)[3] - 1.0) > 1e-9) return fail(12, "pose graph chain");
  try {
    g.get(7);
    return fail(13, "unknown key accepted");
  } catch (const Error &e) {
    if (e.code != CVO_ERR_INVALID_ARG) return fail(14, "unknown key status");
  }
  std::printf("ok %.6g %.6g\n", (double)ip, (double)cosv);
  return 0;
}
"""


def test_cpp_client_of_the_cvogpu_mirror():
    lib_dir = os.path.dirname(L.LIB_PATH)
    inc = os.path.join(ROOT, "include")
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "client.cpp")
        open(src, "w").write(_CLIENT)
        exe = os.path.join(d, "client")
        subprocess.run(["g++", "-std=c++17", "-Wall", "-Wextra", "-Werror", "-I" + inc, src, "-o", exe,
                        "-L" + lib_dir, "-lcvo_gb300", "-Wl,-rpath," + lib_dir], check=True)
        r = subprocess.run([exe, params_path("geometric")], capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, (r.returncode, r.stderr[-2000:])
        assert r.stdout.startswith("ok ")

