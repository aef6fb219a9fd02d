"""cvo_inner_product_noalloc: the inner product for callers that cannot allocate
device memory when they need the value.

The entry point takes device-resident clouds and a device output word and keeps
its only scratch in a fixed array inside the library.  This test calls it
through the C ABI twice in a row (the second call reuses the scratch left by
the first) and checks both results against cvo_inner_product, the allocating
entry point with the same semantics, and against the CPU oracle, within the
relative tolerance the other parity tests use (1e-5).  The cases cover every
branch of the kernel: geometry only with the index-ordered cap active, colour
features, semantic labels, the geometric-type factor, and xyz records of
stride 4.  The file is named so that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as orc
from rkhs_ba_gb300 import CvoGPU, CvoParams, CvoPointCloud, params_path, scenes
from rkhs_ba_gb300 import _lib as L

pytestmark = pytest.mark.gpu

REL = 1e-5


def _device_cloud(cloud, torch, xyz_stride=3):
    """cvo_cloud descriptor whose arrays live on the GPU (torch tensors keep them alive)."""
    keep = []
    fp = C.POINTER(C.c_float)

    def dev(a):
        if a is None:
            return fp()
        t = torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()
        keep.append(t)
        return C.cast(C.c_void_p(t.data_ptr()), fp)

    xyz = cloud.xyz
    if xyz_stride == 4:                       # {x, y, z, pad} records; the pad is never read
        xyz = np.concatenate([xyz, np.full((len(xyz), 1), 7.0, np.float32)], 1)
    c = L.CvoCloudC()
    c.n, c.F, c.C, c.xyz_stride = cloud.num_points(), cloud.feature_dimensions(), cloud.num_classes(), xyz_stride
    c.xyz, c.features, c.labels, c.geom_type = dev(xyz), dev(cloud.features), dev(cloud.labels), dev(cloud.geom_type)
    return c, keep


def _noalloc(params, cs, ct, T, ell, out, stream):
    Tm = np.ascontiguousarray(np.asarray(T, np.float32).T.reshape(16))
    return L.lib().cvo_inner_product_noalloc(C.byref(params._c), C.byref(cs), C.byref(ct),
                                             Tm.ctypes.data_as(C.POINTER(C.c_float)), float(ell),
                                             C.c_void_p(out.data_ptr()), C.c_void_p(stream))


def _with_geom_type(cloud, seed):
    g = np.random.default_rng(seed).uniform(0.05, 1, size=(cloud.num_points(), 2)).astype(np.float32)
    return CvoPointCloud(cloud.xyz, cloud.features, cloud.labels, g)


def _case(which):
    """(source, target, params, lengthscale, xyz stride) of one parametrised case."""
    if which == "geometric_capped":
        src, tgt, _ = scenes.room_pair(n=3000, seed=31)
        p = CvoParams(params_path("geometric"))
        p.nearest_neighbors_max = 8           # index-ordered truncation active
        return src, tgt, p, 0.35, 3
    if which == "color":
        src, tgt, _ = scenes.stereo_pair(n=3000, seed=32)
        return src, tgt, CvoParams(params_path("color")), 0.5, 3
    if which == "color_stride4":
        src, tgt, _ = scenes.stereo_pair(n=3000, seed=33)
        p = CvoParams(params_path("color"))
        p.nearest_neighbors_max = 24
        return src, tgt, p, 0.5, 4
    if which == "semantic":
        src, tgt, _ = scenes.lidar_pair(n=4000, seed=34)
        return src, tgt, CvoParams(params_path("lidar_semantic")), 0.8, 3
    if which == "semantic_geotype":
        src, tgt, _ = scenes.lidar_pair(n=4000, seed=35)
        p = CvoParams(params_path("lidar_semantic"))
        p.is_using_geometric_type = 1
        p.nearest_neighbors_max = 32
        return _with_geom_type(src, 1), _with_geom_type(tgt, 2), p, 0.6, 3
    raise ValueError(which)


@pytest.mark.parametrize("which", ["geometric_capped", "color", "color_stride4", "semantic", "semantic_geotype"])
def test_noalloc_inner_product_matches_allocating_entry_point(cuda_device, which):
    import torch
    src, tgt, p, ell, stride = _case(which)
    T = scenes.make_T(scenes.rot_axis_angle([0.1, 1.0, 0.2], np.radians(4.0)), [0.05, -0.02, 0.3]).astype(np.float32)
    expected = CvoGPU(params=p).inner_product_gpu(src, tgt, T, ell)
    oracle_ip, _ = orc.inner_product_gpu_semantics(p, src, tgt, T, ell)
    assert expected > 0
    assert expected == pytest.approx(oracle_ip, rel=REL)
    _, _, nnz = orc.association(p, src, tgt, T, ell)
    assert nnz.sum() > 200
    if which == "geometric_capped":
        assert (nnz == p.nearest_neighbors_max).sum() > 200         # the cap truncates rows
    cs, ks = _device_cloud(src, torch, stride)
    ct, kt = _device_cloud(tgt, torch, stride)
    out = torch.full((1,), -1.0, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for _ in range(2):                        # two calls in a row share the scratch array
        out.fill_(-1.0)
        rc = _noalloc(p, cs, ct, T, ell, out, stream)
        assert rc == L.CVO_OK, L.lib().cvo_status_string(rc)
        torch.cuda.synchronize()
        assert out.item() == pytest.approx(expected, rel=REL)
        assert out.item() == pytest.approx(oracle_ip, rel=REL)


def test_noalloc_rejects_oversized_input(cuda_device):
    """More source rows than the scratch array serves, or more pair tests than the
    per-call budget, are refused before anything reaches the device."""
    import torch
    p = CvoParams(params_path("geometric"))
    small = CvoPointCloud(np.zeros((4, 3), np.float32))
    cs, ks = _device_cloud(small, torch)
    out = torch.zeros(1, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    big = L.CvoCloudC()
    big.n, big.F, big.C, big.xyz_stride = (1 << 20) + 1, 0, 0, 3
    big.xyz = cs.xyz                            # never read: the size check comes first
    assert _noalloc(p, big, cs, np.eye(4), 0.3, out, stream) == L.CVO_ERR_CAPACITY
    rows = L.CvoCloudC()
    rows.n, rows.F, rows.C, rows.xyz_stride = 1 << 20, 0, 0, 3      # within the row limit ...
    rows.xyz = cs.xyz
    wide = L.CvoCloudC()
    wide.n, wide.F, wide.C, wide.xyz_stride = (1 << 13) + 1, 0, 0, 3   # ... but N * M above 2^33
    wide.xyz = cs.xyz
    assert _noalloc(p, rows, wide, np.eye(4), 0.3, out, stream) == L.CVO_ERR_CAPACITY
