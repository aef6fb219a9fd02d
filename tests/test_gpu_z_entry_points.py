"""GPU checks of the entry points added on top of the engine.  The file sorts after
every kernel-parity file (test_gpu_*), so that under ``pytest -x`` a failure here
cannot hide the results of those tests:

* the C++ mirror (include/cvo_gb300.hpp) registers and computes inner products exactly
  as the Python binding does;
* cvo_global_register gives exactly what the calls it composes give;
* non-finite points are rejected on the host before upload.
"""
import os
import subprocess

import numpy as np
import pytest

from rkhs_ba_gb300 import CvoGPU, CvoParams, CvoPointCloud, params_path, scenes
from rkhs_ba_gb300 import _lib as L
from rkhs_ba_gb300.proposal import ProposalNet

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


_GPU_CLIENT = r"""
#include <cstdio>
#include <fstream>
#include "cvo_gb300.hpp"

using namespace cvo_gb300;

static PointCloud read_cloud(std::ifstream &in) {
  int n = 0;
  in.read(reinterpret_cast<char *>(&n), sizeof(int));
  PointCloud c;
  c.xyz.resize(3 * (size_t)n);
  in.read(reinterpret_cast<char *>(c.xyz.data()), sizeof(float) * 3 * (size_t)n);
  return c;
}

int main(int argc, char **argv) {
  if (argc < 3) return 2;
  std::ifstream in(argv[2], std::ios::binary);
  PointCloud src = read_cloud(in), tgt = read_cloud(in);
  CvoGPU cvo(argv[1]);
  Mat4 T{};
  int iters = 0;
  const int ret = cvo.align(src, tgt, identity(), T, nullptr, nullptr, &iters);
  const float ip = cvo.inner_product_gpu(src, tgt, identity(), 0.25f);
  std::printf("%d %d %.9g", ret, iters, (double)ip);
  for (float v : T) std::printf(" %.9g", (double)v);
  std::printf("\n");
  return 0;
}
"""


def test_cpp_client_align_equals_python_api(cuda_device, tmp_path):
    """The C++ mirror and the Python binding reach the same entry points: the same
    registration (pose, iterations, return code) and the same GPU inner product."""
    src, tgt, _ = scenes.room_pair(n=3000, seed=3)
    data = tmp_path / "pair.bin"
    with open(data, "wb") as fh:
        for c in (src, tgt):
            fh.write(np.int32(c.num_points()).tobytes())
            fh.write(np.ascontiguousarray(c.xyz, np.float32).tobytes())
    lib_dir = os.path.dirname(L.LIB_PATH)
    exe = tmp_path / "client"
    cpp = tmp_path / "client.cpp"
    cpp.write_text(_GPU_CLIENT)
    subprocess.run(["g++", "-std=c++17", "-Wall", "-Wextra", "-Werror", "-I" + os.path.join(ROOT, "include"), str(cpp),
                    "-o", str(exe), "-L" + lib_dir, "-lcvo_gb300", "-Wl,-rpath," + lib_dir], check=True)
    yaml = params_path("geometric")
    r = subprocess.run([str(exe), yaml, str(data)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    vals = r.stdout.split()
    ret_c, it_c, ip_c = int(vals[0]), int(vals[1]), np.float32(float(vals[2]))   # %.9g round-trips a float
    T_c = np.array([float(v) for v in vals[3:19]], np.float32).reshape(4, 4, order="F")
    cvo = CvoGPU(params=CvoParams(yaml))
    ret, T, _, _, iters = cvo.align(src, tgt, np.eye(4))
    assert ret_c == ret and it_c == iters
    assert np.array_equal(T_c, np.asarray(T, np.float32))
    assert ip_c == np.float32(cvo.inner_product_gpu(src, tgt, np.eye(4), 0.25))


def test_global_register_equals_the_calls_it_composes(cuda_device):
    """cvo_global_register (host pairs in, poses out) gives exactly what its parts give:
    the plain grid (nearest of the 24 rotations, inverted, one batched align) and the
    learned registration with register_learned_batch's defaults."""
    cvo = CvoGPU(params=CvoParams(params_path("color")))
    net = ProposalNet(cvo, points_per_cloud=512, seed=0)        # equality needs no training
    pairs = [scenes.global_pair(n=6000, seed=4_100_000 + k) for k in range(3)]
    srcs = [s for s, _, _ in pairs]
    tgts = [t for _, t, _ in pairs]
    gs = [cvo.upload(s) for s in srcs]
    gt = [cvo.upload(t) for t in tgts]
    p = cvo.get_params()
    T_g, it_g, _ = cvo.global_register(srcs, tgts)
    inits = [scenes.inv_T(cvo.get_nearest_init_pose(s, t, p.ell_init_first_frame, 0, 1)[0]) for s, t in zip(gs, gt)]
    Tp, _, itp, _ = cvo.align_batch(gs, gt, inits)
    for k in range(len(pairs)):
        assert np.array_equal(T_g[k], Tp[k]) and it_g[k] == itp[k], k
    T_l, it_l, _ = cvo.global_register(srcs, tgts, net)
    Tr, _, _, itr, _ = cvo.register_learned_batch(net, gs, gt)
    for k in range(len(pairs)):
        assert np.array_equal(T_l[k], Tr[k]) and it_l[k] == itr[k], k


def test_non_finite_points_are_rejected_before_upload(cuda_device):
    """Coordinates are checked on the host (cloud_upload): a NaN or infinite point is an
    invalid argument and nothing reaches the device."""
    from rkhs_ba_gb300._lib import CvoError, CVO_ERR_INVALID_ARG
    cvo = CvoGPU(params=CvoParams(params_path("geometric")))
    src, _, _ = scenes.room_pair(n=500, seed=1)
    for bad in (np.nan, np.inf):
        xyz = src.xyz.copy()
        xyz[123, 1] = bad
        with pytest.raises(CvoError) as e:
            cvo.upload(CvoPointCloud(xyz))
        assert e.value.code == CVO_ERR_INVALID_ARG
    assert len(cvo.upload(src)) == 500
