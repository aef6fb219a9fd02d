"""The association autotuner (cvo_autotune_launch_dev): every candidate configuration --
12 cell sizes, then 1-3 resident blocks per SM -- gives the same kernel matrix (identical
columns per row, values within 1e-6 relative) and the same inner product (1e-5
relative: row sums may add in another order); the fastest configuration is kept for
later batches of the same key."""
import numpy as np
import pytest

from rkhs_ba_gb300 import CvoGPU, CvoParams, params_path, scenes

pytestmark = pytest.mark.gpu


def test_autotune_configurations_agree(cuda_device):
    s, t, T_gt = scenes.stereo_pair(n=12000, seed=21)
    p = CvoParams(params_path("color"))
    cvo = CvoGPU(params=p)
    gs, gt = cvo.upload(s), cvo.upload(t)
    T = np.linalg.inv(T_gt) @ scenes.make_T(scenes.rot_axis_angle([0, 1, 0], np.radians(1.0)), [0.05, 0, 0.1])
    res = cvo.autotune(gs, gt, T, reps=2)
    cfgs = res["configs"]
    assert len(cfgs) == 15 and 0 <= res["best"] < 15
    assert all(np.isfinite(ms) and ms > 0 for _, _, _, ms in cfgs)
    assert [bp for _, _, bp, _ in cfgs] == [0] * 12 + [1, 2, 3]
    F, Cn = s.features.shape[1], 0
    a, b, bp, tuned = cvo.tune_get_launch(F, Cn, len(s.xyz))
    assert tuned and (a, b, bp) == cfgs[res["best"]][:3]
    ref_assoc, ref_ip = None, None
    for div_r, div_ext, bps, _ in cfgs:
        cvo.tune_set_launch(F, Cn, len(s.xyz), div_r, div_ext, bps)
        assoc = cvo.compute_association_gpu(s, t, T, p.ell_init)
        ip = cvo.inner_product_batch(gs, gt, [T], p.ell_init)[0]
        if ref_assoc is None:
            ref_assoc, ref_ip = assoc, ip
            assert assoc.nnz > 0
            continue
        assert np.array_equal(assoc.row_ptr, ref_assoc.row_ptr) and np.array_equal(assoc.col, ref_assoc.col)
        assert np.allclose(assoc.val, ref_assoc.val, rtol=1e-6, atol=0)
        assert abs(ip - ref_ip) <= 1e-5 * abs(ref_ip)


def test_tune_get_untuned_key(cuda_device):
    cvo = CvoGPU(params=CvoParams(params_path("color")))
    a, b, tuned = cvo.tune_get(5, 0, 1000)
    assert not tuned and (a, b) == (4.0, 8.0)
