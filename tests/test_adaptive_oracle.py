"""CPU checks of the adaptive-lengthscale oracle (AdaptiveCvoGPU, src/cvo/AdaptiveCvoGPU.cu):
its kernel matrix against an independent numpy restatement of fill_in_A_mat_gpu's
index-ordered scan (:263-407), and the behaviour of its align loop (:1077-1250)."""
import numpy as np
import pytest

from oracle import oracle as orc
from rkhs_ba_gb300 import CvoParams, params_path, scenes

CAP = orc.ADAPTIVE_CAP


def _numpy_fill(p, xs, fx, ys, fy, ell):
    """fill_in_A_mat_gpu restated with float32 numpy arithmetic: rows scan targets in
    index order and stop after CAP kept pairs."""
    f32 = np.float32
    s2 = f32(p.sigma) * f32(p.sigma)
    sp = f32(p.sp_thres)
    d2t = f32(-2.0 * float(f32(ell)) * float(f32(ell)) * float(np.log(sp / s2, dtype=np.float32)))
    cs = f32(p.c_sigma)
    d2ct = f32(-2.0 * float(f32(p.c_ell)) * float(f32(p.c_ell)) * float(np.log((sp / cs) / cs, dtype=np.float32)))
    use_int = bool(p.is_using_intensity)
    rows = []
    for i in range(len(xs)):
        d = (ys - xs[i]).astype(np.float32)                     # y - x per component
        d2 = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]
        keep = d2 < d2t
        q = -d2.astype(np.float64) / (2.0 * float(f32(ell)) * float(f32(ell)))
        if not use_int:
            a = (float(s2) * np.exp(q) * float(cs)).astype(np.float32)
        else:
            t = (fx[i][None, :] - fy).astype(np.float32)
            d2c = np.zeros(len(ys), np.float32)
            for k in range(fx.shape[1]):
                d2c = d2c + t[:, k] * t[:, k]
            keep &= d2c < d2ct
            kk = (float(s2) * np.exp(q)).astype(np.float32)
            ck = (float(cs * cs) * np.exp(-d2c.astype(np.float64) / (2.0 * float(f32(p.c_ell)) * float(f32(p.c_ell))))).astype(np.float32)
            a = (ck * kk).astype(np.float32)
        keep &= a > sp
        j = np.nonzero(keep)[0][:CAP]
        rows.append((j, a[j]))
    return rows


@pytest.mark.parametrize("kind", ["geometric", "color"])
def test_adaptive_fill_matches_numpy_restatement(kind):
    rng = np.random.default_rng(5)
    if kind == "geometric":
        s, t, _ = scenes.room_pair(n=700, seed=2)
        p = CvoParams(params_path("geometric"))
        xs, ys, fx, fy = s.xyz, t.xyz, None, None
        ell = 2.0
    else:
        s, t, _ = scenes.stereo_pair(n=700, seed=2)
        p = CvoParams(params_path("color"))
        xs, ys = s.xyz, t.xyz
        fx, fy = s.features, t.features
        ell = 0.6
    # a compact copy of the scene so that some rows reach the cap
    xs = (xs * 0.2).astype(np.float32)
    ys = (ys * 0.2).astype(np.float32)
    ind, val, nnz = orc.fill_adaptive(p, xs, fx, None, ys, fy, None, ell)
    ref = _numpy_fill(p, xs, fx, ys, fy, ell)
    capped = 0
    for i, (j, a) in enumerate(ref):
        assert nnz[i] == len(j), i
        assert np.array_equal(ind[i, :nnz[i]], j), i
        assert np.array_equal(val[i, :nnz[i]], a), i
        capped += len(j) == CAP
    assert sum(len(j) for j, _ in ref) > 0
    if kind == "geometric":
        assert capped > 0          # the index-ordered truncation is exercised


def test_adaptive_align_converges_and_adapts_ell():
    s, t, T_gt = scenes.room_pair(n=1500, seed=4)
    p = CvoParams(params_path("geometric"))
    ret, T, iters, tr = orc.align_adaptive(p, s, t, np.eye(4), trace_len=4000)
    r, tt = scenes.pose_error(T, T_gt)
    assert ret == 0 and iters > 0
    assert r < 1.0 and tt < 0.05, (r, tt)
    ell = tr["ell"][:iters]
    assert ell[0] == np.float32(p.ell_init)
    assert np.all(ell <= np.float32(p.ell_max)) and np.all(ell >= np.float32(p.ell_min))
    assert np.any(ell != ell[0])                     # the lengthscale moves
    nz = tr["nnz3"][:iters]
    assert np.all(nz[:, 1] >= len(s.xyz))            # Axx keeps every diagonal pair
    assert np.all(tr["step"][:iters] <= np.float32(0.8))


def test_adaptive_align_empty_cloud_is_a_no_op():
    s, t, _ = scenes.room_pair(n=300, seed=1)
    from rkhs_ba_gb300 import CvoPointCloud
    empty = CvoPointCloud(np.zeros((0, 3), np.float32))
    p = CvoParams(params_path("geometric"))
    ret, T, iters, _ = orc.align_adaptive(p, s, empty, np.eye(4))
    assert ret == 0 and iters == 0
