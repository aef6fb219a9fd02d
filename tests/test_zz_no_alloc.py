"""cvo_inner_product_noalloc: the inner product for callers that cannot allocate
device memory when they need the value.

The entry point takes device-resident clouds and a device output word and keeps
its only scratch in a fixed array inside the library.  This test calls it
through the C ABI twice in a row (the second call reuses the scratch left by
the first) and checks both results against cvo_inner_product, the allocating
entry point with the same semantics, within the relative tolerance the other
parity tests use (1e-5).  The file is named so that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

from rkhs_ba_gb300 import CvoGPU, CvoParams, CvoPointCloud, params_path, scenes
from rkhs_ba_gb300 import _lib as L

pytestmark = pytest.mark.gpu

REL = 1e-5


def _device_cloud(cloud, torch):
    """cvo_cloud descriptor whose arrays live on the GPU (torch tensors keep them alive)."""
    keep = []
    fp = C.POINTER(C.c_float)

    def dev(a):
        if a is None:
            return fp()
        t = torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()
        keep.append(t)
        return C.cast(C.c_void_p(t.data_ptr()), fp)

    c = L.CvoCloudC()
    c.n, c.F, c.C, c.xyz_stride = cloud.num_points(), cloud.feature_dimensions(), cloud.num_classes(), 3
    c.xyz, c.features, c.labels, c.geom_type = dev(cloud.xyz), dev(cloud.features), dev(cloud.labels), dev(cloud.geom_type)
    return c, keep


def _noalloc(params, cs, ct, T, ell, out, stream):
    Tm = np.ascontiguousarray(np.asarray(T, np.float32).T.reshape(16))
    return L.lib().cvo_inner_product_noalloc(C.byref(params._c), C.byref(cs), C.byref(ct),
                                             Tm.ctypes.data_as(C.POINTER(C.c_float)), float(ell),
                                             C.c_void_p(out.data_ptr()), C.c_void_p(stream))


@pytest.mark.parametrize("which", ["geometric", "color"])
def test_noalloc_inner_product_matches_allocating_entry_point(cuda_device, which):
    import torch
    if which == "geometric":
        src, tgt, _ = scenes.room_pair(n=3000, seed=31)
        p = CvoParams(params_path("geometric"))
        p.nearest_neighbors_max = 16          # index-ordered truncation active
        ell = 0.35
    else:
        src, tgt, _ = scenes.stereo_pair(n=3000, seed=32)
        p = CvoParams(params_path("color"))
        ell = 0.5
    T = scenes.make_T(scenes.rot_axis_angle([0.1, 1.0, 0.2], np.radians(4.0)), [0.05, -0.02, 0.3]).astype(np.float32)
    expected = CvoGPU(params=p).inner_product_gpu(src, tgt, T, ell)
    assert expected > 0
    cs, ks = _device_cloud(src, torch)
    ct, kt = _device_cloud(tgt, torch)
    out = torch.full((1,), -1.0, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for _ in range(2):                        # two calls in a row share the scratch array
        out.fill_(-1.0)
        rc = _noalloc(p, cs, ct, T, ell, out, stream)
        assert rc == L.CVO_OK, L.lib().cvo_status_string(rc)
        torch.cuda.synchronize()
        assert out.item() == pytest.approx(expected, rel=REL)


def test_noalloc_rejects_oversized_input(cuda_device):
    import torch
    p = CvoParams(params_path("geometric"))
    small = CvoPointCloud(np.zeros((4, 3), np.float32))
    cs, ks = _device_cloud(small, torch)
    big = L.CvoCloudC()
    big.n, big.F, big.C, big.xyz_stride = (1 << 20) + 1, 0, 0, 3
    big.xyz = cs.xyz                            # never read: the size check comes first
    out = torch.zeros(1, dtype=torch.float32, device="cuda")
    rc = _noalloc(p, big, cs, np.eye(4), 0.3, out, torch.cuda.current_stream().cuda_stream)
    assert rc == L.CVO_ERR_CAPACITY
