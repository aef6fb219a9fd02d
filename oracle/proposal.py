"""CPU oracle of the learned pose proposal network (test infrastructure only).

The reference has no learned component: its global registration scores a fixed
rotation grid (get_nearest_init_pose, src/cvo/CvoGPU.cpp:367-398).  This module
restates the definition of the network that stands in for that grid, so that the
device kernels (rkhs_ba_gb300/csrc/cvo_learn.cu) can be checked against it:

* the point sampling hash, the per-cloud mean and the 16-column point input;
* the forward pass (8 -> 64 -> 128 per-point MLP, max-pool, 256 -> 256 -> 72 head);
* the relaxed winner-takes-all loss and every gradient of the backward pass;
* the hypothesis poses (Gram-Schmidt of the 6D rotation, centroid translation).

With ``bf16=True`` every matrix-product operand is rounded to bfloat16
(round-to-nearest-even) exactly where the device stages it for the tensor cores,
and the products are accumulated in float64; with ``bf16=False`` the whole
computation is float64, which ``tests/test_oracle.py`` checks against finite
differences of the loss.  Only tests, the smoke check and the bench's CPU leg
use this module.
"""
from __future__ import annotations

import numpy as np

IN, IN_USED, H1, H2, HEAD, H3, K = 16, 8, 64, 128, 256, 256, 8
OUT = 9 * K
INV_SCALE = 0.1

# parameter block layout (floats), row-major weights [in][out]
_SHAPES = [("W1", (IN, H1)), ("b1", (H1,)), ("W2", (H1, H2)), ("b2", (H2,)), ("W3", (HEAD, H3)), ("b3", (H3,)),
           ("W4", (H3, OUT)), ("b4", (OUT,))]
NUM_PARAMS = int(sum(np.prod(s) for _, s in _SHAPES))


def unpack(flat):
    """Parameter block -> dict of arrays (views of a float64 copy)."""
    flat = np.asarray(flat, np.float64)
    out, o = {}, 0
    for name, shape in _SHAPES:
        n = int(np.prod(shape))
        out[name] = flat[o:o + n].reshape(shape)
        o += n
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], np.float64).reshape(-1) for name, _ in _SHAPES])


def bf16(x):
    """float32 -> bfloat16 -> float32, round to nearest even (finite inputs)."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def _mix32(x):
    x = np.asarray(x, np.uint64) & 0xFFFFFFFF
    x ^= x >> 16
    x = (x * 0x7FEB352D) & 0xFFFFFFFF
    x ^= x >> 15
    x = (x * 0x846CA68B) & 0xFFFFFFFF
    x ^= x >> 16
    return x


def sample_indices(seed, slot, P, n):
    """Indices of the P points the network samples from slot ``slot`` of n points."""
    a = _mix32((int(seed) + 0x9E3779B9 * (slot + 1)) & 0xFFFFFFFF)
    h = _mix32(a ^ np.arange(P, dtype=np.uint64))
    return ((h * np.uint64(n)) >> np.uint64(32)).astype(np.int64)


def slot_input(xyz, feat, T, seed, slot, P):
    """(mean (3,), centroid of the moved cloud (3,), X (P, 16)) of one slot.

    xyz (n, 3), feat (n, F); T row-major 3x4 applied to the points."""
    xyz = np.asarray(xyz, np.float32)
    n = len(xyz)
    T = np.asarray(T, np.float32).reshape(3, 4)
    m = (xyz.astype(np.float64).sum(0) / n).astype(np.float32) if n else np.zeros(3, np.float32)
    cent = (T[:, :3].astype(np.float64) @ m + T[:, 3]).astype(np.float32)
    X = np.zeros((P, IN), np.float32)
    if n:
        j = sample_indices(seed, slot, P, n)
        d = xyz[j] - m
        X[:, 0:3] = ((d.astype(np.float64) @ T[:, :3].T.astype(np.float64)) * INV_SCALE).astype(np.float32)
        nf = min(feat.shape[1] if feat is not None and feat.ndim == 2 else 0, IN_USED - 3)
        if nf:
            X[:, 3:3 + nf] = np.asarray(feat, np.float32)[j, :nf]
    return m, cent, X


def _mm(a, b, rnd):
    if rnd:
        a, b = bf16(a), bf16(b)
    return np.asarray(a, np.float64) @ np.asarray(b, np.float64)


def _f32(x, rnd):
    return np.asarray(x, np.float32) if rnd else np.asarray(x, np.float64)


def forward(params, X, n_pairs, bf16_ops=True):
    """Forward pass.  X: (2 n_pairs, P, 16), slot 2b = source of pair b, 2b + 1 its target.

    Returns a dict of every activation (H1, H2, G, arg, H3, O)."""
    p = unpack(params)
    r = bf16_ops
    S, P, _ = X.shape
    Xf = _f32(X.reshape(S * P, IN), r)
    H1a = _f32(np.maximum(_mm(Xf, p["W1"], r) + p["b1"], 0.0), r)
    H2a = _f32(np.maximum(_mm(H1a, p["W2"], r) + p["b2"], 0.0), r)
    H2v = H2a.reshape(S, P, H2)
    arg = H2v.argmax(axis=1)                                  # first index of the maximum
    G = np.take_along_axis(H2v, arg[:, None, :], axis=1)[:, 0, :]
    Gp = G.reshape(n_pairs, HEAD)
    H3a = _f32(np.maximum(_mm(Gp, p["W3"], r) + p["b3"], 0.0), r)
    O = _f32(_mm(H3a, p["W4"], r) + p["b4"], r)
    return {"X": Xf, "H1": H1a, "H2": H2a, "G": G, "arg": arg, "H3": H3a, "O": O}


def wta_targets(T_label, cent):
    """Per pair y (9,) from the label pose (row-major 3x4) and the slot centroids (2B, 3)."""
    T = np.asarray(T_label, np.float64).reshape(-1, 3, 4)
    B = len(T)
    cent = np.asarray(cent, np.float64).reshape(2 * B, 3)
    y = np.zeros((B, 9))
    for b in range(B):
        R, t = T[b, :, :3], T[b, :, 3]
        y[b, 0:3] = R[:, 0]
        y[b, 3:6] = R[:, 1]
        y[b, 6:9] = (t - (cent[2 * b + 1] - R @ cent[2 * b])) * INV_SCALE
    return y


def wta_loss(O, y):
    """Relaxed winner-takes-all loss: (mean loss, dO (B, 72), best (B,))."""
    B = len(O)
    Ok = np.asarray(O, np.float64).reshape(B, K, 9)
    L = ((Ok - y[:, None, :]) ** 2).sum(-1)
    best = L.argmin(1)
    w = np.full((B, K), 0.05 / (K - 1))
    w[np.arange(B), best] = 0.95
    loss = (w * L).sum(1)
    dO = (w[..., None] / B) * 2.0 * (Ok - y[:, None, :])
    return float(loss.mean()), dO.reshape(B, OUT), best


def backward(params, act, dO, bf16_ops=True):
    """Gradient block (same layout as the parameters) from dL/dO."""
    p = unpack(params)
    r = bf16_ops
    S, P = act["arg"].shape[0], act["H2"].shape[0] // act["arg"].shape[0]
    B = S // 2
    dO = _f32(dO, r)
    g = {}
    g["W4"] = _mm(act["H3"].T, dO, r)
    g["b4"] = dO.sum(0, dtype=np.float64)
    dH3 = _f32(_mm(dO, p["W4"].T, r), r) * (act["H3"] > 0)
    g["W3"] = _mm(act["G"].reshape(B, HEAD).T, dH3, r)
    g["b3"] = dH3.sum(0, dtype=np.float64)
    dG = _f32(_mm(dH3, p["W3"].T, r), r).reshape(S, H2)
    dH2 = np.zeros((S, P, H2), dG.dtype)
    cols = np.arange(H2)
    for c in range(S):
        dH2[c, act["arg"][c], cols] = np.where(act["G"][c] > 0, dG[c], 0.0)
    dH2 = dH2.reshape(S * P, H2)
    g["W2"] = _mm(act["H1"].T, dH2, r)
    g["b2"] = dH2.sum(0, dtype=np.float64)
    dH1 = _f32(_mm(dH2, p["W2"].T, r), r) * (act["H1"] > 0)
    g["W1"] = _mm(act["X"].T, dH1, r)
    g["b1"] = dH1.sum(0, dtype=np.float64)
    return pack(g)


def hypotheses(O, cent):
    """(B, K, 4, 4) row-major poses (target = R source + t) from the outputs."""
    B = len(O)
    Ok = np.asarray(O, np.float64).reshape(B, K, 9)
    cent = np.asarray(cent, np.float64).reshape(2 * B, 3)
    out = np.zeros((B, K, 4, 4))
    for b in range(B):
        for k in range(K):
            a1, a2 = Ok[b, k, 0:3], Ok[b, k, 3:6]
            b1 = a1 / np.linalg.norm(a1)
            b2 = a2 - (b1 @ a2) * b1
            b2 = b2 / np.linalg.norm(b2)
            R = np.stack([b1, b2, np.cross(b1, b2)], 1)
            out[b, k, :3, :3] = R
            out[b, k, :3, 3] = cent[2 * b + 1] - R @ cent[2 * b] + Ok[b, k, 6:9] / INV_SCALE
            out[b, k, 3, 3] = 1.0
    return out


def pool_batch(src_pool, tgt_pool, scene, T_tgt, seed, P):
    """Slot inputs of a pool batch: (X (2B, P, 16), cent (2B, 3))."""
    B = len(scene)
    X = np.zeros((2 * B, P, IN), np.float32)
    cent = np.zeros((2 * B, 3), np.float32)
    I = np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, 0]], np.float32)
    for b, s in enumerate(scene):
        for side, pool in ((0, src_pool), (1, tgt_pool)):
            T = I if (side == 0 or T_tgt is None) else np.asarray(T_tgt[b], np.float32).reshape(3, 4)
            pts = np.asarray(pool[s], np.float32)
            _, c, x = slot_input(pts[:, :3], pts[:, 3:8], T, seed, 2 * b + side, P)
            X[2 * b + side] = x
            cent[2 * b + side] = c
    return X, cent


def train_step_grad(params, src_pool, tgt_pool, scene, T_label, seed, P, bf16_ops=True):
    """(loss, gradient block, outputs O, centroids) of one training batch."""
    X, cent = pool_batch(src_pool, tgt_pool, scene, T_label, seed, P)
    act = forward(params, X, len(scene), bf16_ops)
    y = wta_targets(T_label, cent)
    loss, dO, _ = wta_loss(act["O"], y)
    return loss, backward(params, act, dO, bf16_ops), act["O"], cent


def loss_only(params, X, cent, T_label, bf16_ops=False):
    act = forward(params, X, len(T_label), bf16_ops)
    return wta_loss(act["O"], wta_targets(T_label, cent))[0]
