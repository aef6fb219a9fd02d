"""GPU parity of the RGB-D front-end (CvoPointCloud(ImageRGBD, Calibration, ...),
src/utils/CvoPointCloud.cpp:458-560, with RawImage's intensity and gradient) against
the oracle's restatement: identical points, features, labels and geometric types."""
import numpy as np
import pytest

from oracle import oracle as orc
from rkhs_ba_gb300 import CvoGPU, CvoParams, params_path

pytestmark = pytest.mark.gpu


def _frame(rows, cols, channels, seed, n_classes=0):
    rng = np.random.default_rng(seed)
    # smooth texture plus noise, so gradients vary
    yy, xx = np.mgrid[0:rows, 0:cols]
    base = 127 + 80 * np.sin(xx / 7.0) * np.cos(yy / 5.0)
    shape = (rows, cols, channels) if channels == 3 else (rows, cols)
    noise = rng.normal(0, 20, size=shape)
    img = np.clip((base[..., None] if channels == 3 else base) + noise, 0, 255).astype(np.uint8)
    depth = rng.uniform(800, 30000, size=(rows, cols)).astype(np.float32)
    depth[rng.random((rows, cols)) < 0.05] = 0.0
    depth[rng.random((rows, cols)) < 0.02] = np.nan
    depth[rng.random((rows, cols)) < 0.02] = 80000.0        # beyond 55 m
    sel = rng.random((rows, cols)) < 0.3
    sel[0, :] = True                                         # border rows / columns
    sel[:, -1] = True
    v, u = np.nonzero(sel)
    uv = np.stack([u, v], 1).astype(np.int32)
    geo = rng.random((uv.shape[0], 2)).astype(np.float32)
    sem = None
    if n_classes:
        logits = rng.normal(size=(rows, cols, n_classes))
        sem = (np.exp(logits) / np.exp(logits).sum(-1, keepdims=True)).astype(np.float32)
    return img, depth, uv, geo, sem


@pytest.mark.parametrize("channels,n_classes", [(3, 0), (1, 0), (3, 19)])
def test_rgbd_front_end_matches_oracle(cuda_device, channels, n_classes):
    img, depth, uv, geo, sem = _frame(240, 320, channels, seed=channels + n_classes, n_classes=n_classes)
    intr = np.array([718.0, 718.0, 160.5, 119.5], np.float32)
    cvo = CvoGPU(params=CvoParams(params_path("color")))
    g = cvo.cloud_from_rgbd(img, depth, intr, 1000.0, uv, geom_type=geo, semantics=sem)
    got = g.download()
    xyz, feat, lab, og = orc.cloud_from_rgbd(img, depth, intr, 1000.0, uv, geom_type=geo, semantics=sem)
    assert len(g) == xyz.shape[0] > 1000
    assert np.array_equal(got.xyz, xyz)
    assert np.array_equal(got.features, feat)
    assert np.array_equal(got.geom_type, og)
    if n_classes:
        assert np.array_equal(got.labels, lab)


def test_rgbd_cloud_registers_against_itself(cuda_device):
    img, depth, uv, _, _ = _frame(200, 280, 3, seed=4)
    intr = np.array([500.0, 500.0, 140.0, 100.0], np.float32)
    cvo = CvoGPU(params=CvoParams(params_path("color")))
    g = cvo.cloud_from_rgbd(img, depth, intr, 1000.0, uv)
    cos = cvo.function_angle(g.download(), g.download(), np.eye(4, dtype=np.float32), 0.5)
    assert cos > 0.99
