"""GPU parity of the association with a non-isotropic geometric kernel
(CvoGPU::compute_association_gpu(source, target, T, kernel, association),
src/cvo/CvoGPU.cu:1936-1950) against the oracle (orc_association_aniso):
identical column sets per row (first `cap` kept pairs by target index), values
within 1e-5 relative."""
import numpy as np
import pytest

from oracle import oracle as orc
from rkhs_ba_gb300 import CvoGPU, CvoParams, params_path, scenes

pytestmark = pytest.mark.gpu

REL = 1e-5
K_DIAG = np.diag([0.5, 0.5, 0.6]).astype(np.float32)          # the kernel the reference's experiments use
K_FULL = np.array([[0.45, 0.06, -0.02], [0.06, 0.55, 0.03], [-0.02, 0.03, 0.7]], np.float32)


def _pose(deg, axis, t):
    return scenes.make_T(scenes.rot_axis_angle(axis, np.radians(deg)), t).astype(np.float32)


def _csr_equals_ell(a, ind, val, nnz):
    assert a.rows == nnz.shape[0]
    rp = a.row_ptr
    assert int(rp[-1]) == int(nnz.sum())
    for i in range(a.rows):
        cols = a.col[rp[i]:rp[i + 1]]
        assert np.array_equal(cols, ind[i, :nnz[i]]), (i, cols[:8], ind[i, :8])
        assert np.allclose(a.val[rp[i]:rp[i + 1]], val[i, :nnz[i]], rtol=REL, atol=0), i


@pytest.mark.parametrize("cap,K", [(512, K_DIAG), (6, K_DIAG), (64, K_FULL)])
def test_nonisotropic_association_room(cuda_device, cap, K):
    src, tgt, _ = scenes.room_pair(n=3000, seed=11)
    p = CvoParams(params_path("geometric"))
    p.nearest_neighbors_max = cap
    cvo = CvoGPU(params=p)
    T = _pose(3.0, [0.2, 1, 0.1], [0.05, -0.1, 0.02])
    a = cvo.compute_association_gpu(src, tgt, T, K)
    ind, val, nnz = orc.association_aniso(p, src, tgt, T, K, cap=cap)
    _csr_equals_ell(a, ind, val, nnz)
    assert nnz.sum() > 0
    if cap == 6:
        assert (nnz == 6).sum() > 100        # the index-ordered truncation ran
    assert np.array_equal(a.source_inliers, np.nonzero(nnz)[0])


def test_nonisotropic_association_colour(cuda_device):
    src, tgt, _ = scenes.stereo_pair(n=3000, seed=5)
    p = CvoParams(params_path("color"))
    p.nearest_neighbors_max = 64
    cvo = CvoGPU(params=p)
    T = _pose(1.0, [0, 1, 0], [0.0, 0.0, 0.3])
    a = cvo.compute_association_gpu(src, tgt, T, K_FULL)
    ind, val, nnz = orc.association_aniso(p, src, tgt, T, K_FULL, cap=64)
    _csr_equals_ell(a, ind, val, nnz)
    assert nnz.sum() > 0


def test_nonisotropic_association_device_clouds(cuda_device):
    src, tgt, _ = scenes.room_pair(n=2000, seed=3)
    p = CvoParams(params_path("geometric"))
    p.nearest_neighbors_max = 32
    cvo = CvoGPU(params=p)
    T = _pose(2.0, [1, 0, 0], [0.02, 0.0, 0.0])
    a_host = cvo.compute_association_gpu(src, tgt, T, K_DIAG)
    a_dev = cvo.compute_association_gpu(cvo.upload(src), cvo.upload(tgt), T, K_DIAG)
    assert np.array_equal(a_host.row_ptr, a_dev.row_ptr)
    assert np.array_equal(a_host.col, a_dev.col)
    assert np.array_equal(a_host.val, a_dev.val)
