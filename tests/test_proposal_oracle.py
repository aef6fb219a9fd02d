"""CPU checks of the proposal network's oracle: its analytic gradients against finite
differences of its own loss (float64, no rounding), its bfloat16 rounding against
torch's, the sampling hash, the hypothesis poses and the training-pool helpers."""
import numpy as np
import pytest

from oracle import proposal as op


def _random_case(rng, B=3, P=12):
    w = np.zeros(op.NUM_PARAMS)
    p = op.unpack(w)
    for name, a in p.items():
        fan = {"W1": op.IN_USED, "b1": op.IN_USED, "W2": op.H1, "b2": op.H1, "W3": op.HEAD, "b3": op.HEAD,
               "W4": op.H3, "b4": op.H3}[name]
        a[...] = rng.uniform(-1, 1, a.shape) / np.sqrt(fan)
    p["W1"][op.IN_USED:] = 0.0
    w = op.pack(p)
    X = np.zeros((2 * B, P, op.IN))
    X[..., :op.IN_USED] = rng.normal(size=(2 * B, P, op.IN_USED))
    cent = rng.normal(size=(2 * B, 3))
    T = []
    for _ in range(B):
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        a, b, c, d = q
        R = np.array([[a * a + b * b - c * c - d * d, 2 * (b * c - a * d), 2 * (b * d + a * c)],
                      [2 * (b * c + a * d), a * a - b * b + c * c - d * d, 2 * (c * d - a * b)],
                      [2 * (b * d - a * c), 2 * (c * d + a * b), a * a - b * b - c * c + d * d]])
        T.append(np.concatenate([R, rng.normal(size=(3, 1))], 1))
    return w, X, cent, np.stack(T)


def test_oracle_gradients_match_finite_differences():
    rng = np.random.default_rng(4)
    w, X, cent, T = _random_case(rng)
    act = op.forward(w, X, len(T), bf16_ops=False)
    loss, dO, _ = op.wta_loss(act["O"], op.wta_targets(T, cent))
    g = op.backward(w, act, dO, bf16_ops=False)
    assert np.isclose(loss, op.loss_only(w, X, cent, T))
    # every parameter block, a few coordinates each (skip the zero padding rows of W1)
    offs = np.cumsum([0] + [int(np.prod(s)) for _, s in op._SHAPES])
    idx = []
    for k, (name, shape) in enumerate(op._SHAPES):
        n = offs[k + 1] - offs[k]
        lim = op.IN_USED * op.H1 if name == "W1" else n
        idx += list(offs[k] + rng.choice(lim, size=min(6, lim), replace=False))
    eps = 1e-6
    for i in idx:
        wp, wm = w.copy(), w.copy()
        wp[i] += eps
        wm[i] -= eps
        fd = (op.loss_only(wp, X, cent, T) - op.loss_only(wm, X, cent, T)) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(fd), (i, fd, g[i])


def test_oracle_padding_rows_get_no_gradient():
    rng = np.random.default_rng(5)
    w, X, cent, T = _random_case(rng)
    act = op.forward(w, X, len(T), bf16_ops=True)
    _, dO, _ = op.wta_loss(act["O"], op.wta_targets(T, cent))
    g = op.unpack(op.backward(w, act, dO, bf16_ops=True))
    assert np.all(g["W1"][op.IN_USED:] == 0.0)


def test_bf16_rounding_matches_torch():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(6)
    x = np.concatenate([rng.normal(size=5000).astype(np.float32) * 10.0 ** rng.integers(-6, 6, 5000),
                        np.array([0.0, -0.0, 1.0, 1.00390625, 1.01171875, 3.0e38, -1.5e-38], np.float32)])
    ours = op.bf16(x)
    ref = torch.from_numpy(x).to(torch.bfloat16).to(torch.float32).numpy()
    assert np.array_equal(ours.view(np.uint32), ref.view(np.uint32))


def test_sample_indices_are_in_range_and_seeded():
    a = op.sample_indices(7, 3, 4096, 1000)
    assert a.min() >= 0 and a.max() < 1000
    assert np.array_equal(a, op.sample_indices(7, 3, 4096, 1000))
    assert not np.array_equal(a, op.sample_indices(8, 3, 4096, 1000))
    assert not np.array_equal(a, op.sample_indices(7, 4, 4096, 1000))
    # roughly uniform
    h = np.bincount(op.sample_indices(1, 0, 200000, 10), minlength=10)
    assert h.min() > 0.95 * 20000 and h.max() < 1.05 * 20000


def test_hypotheses_are_rigid_and_follow_the_centroids():
    rng = np.random.default_rng(8)
    O = rng.normal(size=(2, op.OUT))
    cent = rng.normal(size=(4, 3))
    H = op.hypotheses(O, cent)
    for b in range(2):
        for k in range(op.K):
            R = H[b, k, :3, :3]
            assert np.allclose(R.T @ R, np.eye(3), atol=1e-12) and np.isclose(np.linalg.det(R), 1.0)
            o = O[b].reshape(op.K, 9)[k]
            assert np.allclose(R[:, 0], o[0:3] / np.linalg.norm(o[0:3]))
            assert np.allclose(H[b, k, :3, 3], cent[2 * b + 1] - R @ cent[2 * b] + o[6:9] / op.INV_SCALE)


def test_wta_targets_recover_the_label():
    rng = np.random.default_rng(9)
    _, _, cent, T = _random_case(rng, B=4)
    y = op.wta_targets(T, cent)
    # a network output equal to y gives back the label pose through hypotheses()
    O = np.tile(y, (1, op.K))
    H = op.hypotheses(O, cent)
    for b in range(4):
        assert np.allclose(H[b, 0, :3, :], T[b], atol=1e-9)
    loss, dO, _ = op.wta_loss(O, y)
    assert loss == 0.0 and np.all(dO == 0.0)


def test_pool_views_match_global_pairs():
    from rkhs_ba_gb300 import scenes
    src, tgt = scenes.global_views(400, seed=21)
    s, t, Tgt = scenes.global_pair(n=400, seed=21)
    assert np.array_equal(src[:, :3], s.xyz) and np.array_equal(src[:, 3:], s.features)
    G = scenes.inv_T(Tgt)
    assert np.allclose(tgt[:, :3] @ G[:3, :3].T + G[:3, 3], t.xyz, atol=1e-4)
    rng = np.random.default_rng(0)
    M = scenes.random_motion(rng)
    assert M.shape == (3, 4) and np.allclose(M[:, :3] @ M[:, :3].T, np.eye(3)) and np.linalg.norm(M[:, 3]) <= 2.0
