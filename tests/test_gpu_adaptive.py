"""GPU parity of the adaptive-lengthscale CVO (AdaptiveCvoGPU, src/cvo/AdaptiveCvoGPU.cu)
against the oracle (orc_fill_adaptive, orc_align_adaptive):

* the kernel matrix at a given pose and lengthscale: identical columns per row (first
  512 kept pairs in index order), values within 1e-5 relative;
* the first iterations: identical nnz of A, Axx and Ayy at the initial pose, and the
  lengthscale, dl and step of the first 8 iterations within 1e-4 relative;
* a full registration: the final pose within 1e-3 rad / 1e-3 m of the oracle's and
  within 1 deg / 5 cm of the generated motion.  (The loop's lengthscale update feeds on
  sums of ~1e4 pair terms, so FP32 row sums against the oracle's double sums move the
  trajectory by more than the two-view path's 1e-4 bound after hundreds of iterations.)
"""
import numpy as np
import pytest

from oracle import oracle as orc
from rkhs_ba_gb300 import AdaptiveCvoGPU, CvoParams, params_path, scenes

pytestmark = pytest.mark.gpu

REL = 1e-5


def _pose(deg, axis, t):
    return scenes.make_T(scenes.rot_axis_angle(axis, np.radians(deg)), t).astype(np.float32)


def _scaled(cloud, f):
    from rkhs_ba_gb300 import CvoPointCloud
    return CvoPointCloud((cloud.xyz * f).astype(np.float32), cloud.features, cloud.labels, cloud.geom_type)


@pytest.mark.parametrize("kind,ell", [("geometric", 2.0), ("geometric", 0.3), ("color", 0.6)])
def test_adaptive_association_matches_oracle(cuda_device, kind, ell):
    if kind == "geometric":
        s, t, _ = scenes.room_pair(n=3000, seed=12)
        p = CvoParams(params_path("geometric"))
        s, t = _scaled(s, 0.2), _scaled(t, 0.2)
    else:
        s, t, _ = scenes.stereo_pair(n=4000, seed=12)
        p = CvoParams(params_path("color"))
    cvo = AdaptiveCvoGPU(params=p)
    T = _pose(2.0, [0.3, 1, 0.2], [0.04, -0.02, 0.03])
    a = cvo.compute_association_gpu(s, t, T, ell)
    ytr = orc.transform_target(T, t)
    ind, val, nnz = orc.fill_adaptive(p, s.xyz, s.features if p.is_using_intensity else None, None, ytr,
                                      t.features if p.is_using_intensity else None, None, ell)
    rp = a.row_ptr
    assert a.rows == len(s.xyz) and int(rp[-1]) == int(nnz.sum()) > 0
    for i in range(a.rows):
        assert np.array_equal(a.col[rp[i]:rp[i + 1]], ind[i, :nnz[i]]), i
        assert np.allclose(a.val[rp[i]:rp[i + 1]], val[i, :nnz[i]], rtol=REL, atol=0), i
    if ell == 2.0:
        assert (nnz == orc.ADAPTIVE_CAP).any()


def test_adaptive_first_iterations_match_oracle(cuda_device):
    s, t, _ = scenes.room_pair(n=2500, seed=7)
    p = CvoParams(params_path("geometric"))
    p.MAX_ITER = 8
    cvo = AdaptiveCvoGPU(params=p)
    gs, gt = cvo.upload(s), cvo.upload(t)
    ret, T, secs, iters, tr = cvo.align(gs, gt, np.eye(4), trace_len=8)
    ret_o, T_o, iters_o, tro = orc.align_adaptive(p, s, t, np.eye(4), trace_len=8)
    assert ret == ret_o and iters == iters_o
    k = min(len(tr), 8)
    assert np.array_equal(tr[0, 3:6].astype(np.int64), tro["nnz3"][0])      # identical pose: identical matrices
    assert np.allclose(tr[:k, 0], tro["ell"][:k], rtol=1e-4, atol=0)
    assert np.allclose(tr[:k, 1], tro["dl"][:k], rtol=1e-4, atol=1e-9)
    assert np.allclose(tr[:k, 2], tro["step"][:k], rtol=1e-4, atol=1e-7)
    assert np.allclose(T, T_o, atol=1e-5)


def test_adaptive_registration_matches_oracle(cuda_device):
    s, t, T_gt = scenes.room_pair(n=2000, seed=3)
    p = CvoParams(params_path("geometric"))
    cvo = AdaptiveCvoGPU(params=p)
    ret, T, secs, iters = cvo.align(s, t, np.eye(4))
    ret_o, T_o, iters_o, _ = orc.align_adaptive(p, s, t, np.eye(4))
    assert ret == ret_o == 0
    r, tt = scenes.pose_error(T, T_gt)
    assert r < 1.0 and tt < 0.05, (r, tt)
    dR = T[:3, :3].T.astype(np.float64) @ T_o[:3, :3].astype(np.float64)
    ang = np.arccos(np.clip((np.trace(dR) - 1) / 2, -1, 1))
    assert ang < 1e-3 and np.linalg.norm(T[:3, 3] - T_o[:3, 3]) < 1e-3, (ang, iters, iters_o)


def test_adaptive_empty_cloud(cuda_device):
    from rkhs_ba_gb300 import CvoPointCloud
    from rkhs_ba_gb300._lib import CvoError
    s, _, _ = scenes.room_pair(n=300, seed=1)
    cvo = AdaptiveCvoGPU(params=CvoParams(params_path("geometric")))
    with pytest.raises(CvoError):
        cvo.align(s, CvoPointCloud(np.zeros((0, 3), np.float32)), np.eye(4))
