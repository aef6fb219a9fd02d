"""GPU checks of the learned pose proposal (rkhs_ba_gb300/csrc/cvo_learn.cu):

* forward outputs and hypotheses against the oracle (oracle/proposal.py) with the
  same bfloat16 operand rounding: max |diff| <= 1e-3 of the largest output;
* loss and every gradient block of a training step against the oracle: loss within
  1e-3 relative, gradient blocks within 1e-2 relative L2 (FP32 accumulation order
  and the rare bfloat16 rounding it flips are the only differences);
* the first Adam step against its closed form;
* training is bit-reproducible for one seed (no float atomics in the backward pass);
* training on the device from a scene pool lowers the loss and the hypotheses'
  rotation error on held-out scenes;
* what the trained network gains: registration of held-out 50k-point-like pairs
  (here 8k points) from its hypotheses against the plain 24-rotation grid, at equal
  or better success with a fraction of the align work.
"""
import numpy as np
import pytest

from oracle import proposal as op
from rkhs_ba_gb300 import CvoGPU, CvoParams, params_path, scenes
from rkhs_ba_gb300.proposal import ProposalNet, ScenePool, evaluate, train

pytestmark = pytest.mark.gpu

P_SMALL = 96


@pytest.fixture(scope="module")
def cvo(cuda_device):
    return CvoGPU(params=CvoParams(params_path("color")))


@pytest.fixture(scope="module")
def small_pool(cuda_device):
    return ScenePool(*ScenePool.generate(4, 300, seed0=500, processes=1))


def _batch(rng, n):
    scene = rng.integers(0, 4, size=n)
    T = np.stack([scenes.random_motion(rng) for _ in range(n)]).astype(np.float32)
    return scene, T


def test_forward_matches_oracle(cvo, small_pool):
    net = ProposalNet(cvo, points_per_cloud=P_SMALL, seed=3)
    rng = np.random.default_rng(2)
    scene, T = _batch(rng, 5)
    raw, hyp = net.forward_pool(small_pool, scene, T, seed=11)
    X, cent = op.pool_batch(small_pool.host_src, small_pool.host_tgt, scene, T, 11, P_SMALL)
    act = op.forward(net.weights(), X, len(scene), bf16_ops=True)
    scale = float(np.abs(act["O"]).max())
    assert np.abs(raw - act["O"]).max() <= 1e-3 * scale
    H = op.hypotheses(raw, cent)
    assert np.allclose(hyp[:, :, :3, :3], H[:, :, :3, :3], atol=1e-5)
    assert np.allclose(hyp[:, :, :3, 3], H[:, :, :3, 3], atol=1e-4 * (1 + np.abs(H[:, :, :3, 3]).max()))


def test_identity_motion_and_seed_change(cvo, small_pool):
    net = ProposalNet(cvo, points_per_cloud=P_SMALL, seed=4)
    a, _ = net.forward_pool(small_pool, [0, 1], None, seed=1)
    b, _ = net.forward_pool(small_pool, [0, 1], np.tile(np.eye(4)[:3], (2, 1, 1)), seed=1)
    c, _ = net.forward_pool(small_pool, [0, 1], None, seed=2)
    assert np.array_equal(a, b)
    assert not np.array_equal(a, c)


def test_gradients_match_oracle(cvo, small_pool):
    net = ProposalNet(cvo, points_per_cloud=P_SMALL, seed=5)
    rng = np.random.default_rng(3)
    scene, T = _batch(rng, 6)
    w = net.weights()
    loss = net.train_step(small_pool, scene, T, lr=0.0, seed=7)
    g = net.gradients()
    assert np.array_equal(net.weights(), w)           # lr = 0: gradients only
    loss_o, g_o, _, _ = op.train_step_grad(w, small_pool.host_src, small_pool.host_tgt, scene, T, 7, P_SMALL)
    assert abs(loss - loss_o) <= 1e-3 * loss_o
    gb, ob = op.unpack(g), op.unpack(g_o)
    for name in gb:
        err = np.linalg.norm(gb[name] - ob[name]) / max(np.linalg.norm(ob[name]), 1e-30)
        assert err <= 1e-2, (name, err)
    # the bfloat16 operands are the only approximation: the float64 gradients are close too
    _, g64, _, _ = op.train_step_grad(w, small_pool.host_src, small_pool.host_tgt, scene, T, 7, P_SMALL,
                                      bf16_ops=False)
    assert np.linalg.norm(g - g64) / np.linalg.norm(g64) <= 5e-2


def test_first_adam_step(cvo, small_pool):
    net = ProposalNet(cvo, points_per_cloud=P_SMALL, seed=6)
    rng = np.random.default_rng(4)
    scene, T = _batch(rng, 4)
    w0 = net.weights()
    net.train_step(small_pool, scene, T, lr=0.0, seed=3)
    g = net.gradients()
    lr = 1e-3
    net.train_step(small_pool, scene, T, lr=lr, seed=3)
    w1 = net.weights()
    # first step: m_hat = g, v_hat = g^2 -> w -= lr g / (|g| + 1e-8)
    big = np.abs(g) > 1e-5 * np.abs(g).max()
    expect = w0 - lr * g / (np.abs(g) + 1e-8)
    assert np.allclose(w1[big], expect[big], atol=2e-6)
    assert np.all(np.abs(w1 - w0) <= lr * 1.0001)


def test_training_is_deterministic(cvo, small_pool):
    """Split-K weight gradients and column sums are added in a fixed order: the same
    seeds give bit-identical weights."""
    ws = []
    for _ in range(2):
        net = ProposalNet(cvo, points_per_cloud=P_SMALL, seed=8)
        rng = np.random.default_rng(5)
        for step in range(3):
            scene, T = _batch(rng, 6)
            net.train_step(small_pool, scene, T, lr=1e-3, seed=step)
        ws.append(net.weights())
    assert np.array_equal(ws[0], ws[1])


@pytest.fixture(scope="module")
def trained(cvo):
    pool = ScenePool(*ScenePool.generate(300, 1024, seed0=2_000_000))
    held = ScenePool(*ScenePool.generate(64, 1024, seed0=3_000_000))
    net = ProposalNet(cvo, points_per_cloud=512, seed=0)
    before, _ = evaluate(net, held, 64)
    losses, secs = train(net, pool, steps=1500, batch=64, lr=1e-3, seed=0)
    after, _ = evaluate(net, held, 64)
    return net, losses, before, after, secs


def test_training_on_the_device_learns_the_rotation(trained):
    net, losses, before, after, secs = trained
    assert np.all(np.isfinite(losses))
    assert losses[-100:].mean() < 0.5 * losses[:100].mean()
    assert np.median(after) < 20.0, np.median(after)
    assert (after < 30.0).mean() >= 0.85
    assert np.median(after) < 0.5 * np.median(before)


def test_trained_network_gain_over_the_grid(cvo, trained):
    """Held-out global pairs (uniform rotation, shift <= 2 m): the plain 24-rotation grid
    (nearest grid rotation by cos-angle, then align) against the network's hypotheses
    (best 2 of 8 by cos-angle refined in one batch, grid fallback)."""
    net = trained[0]
    pairs = [scenes.global_pair(n=8000, seed=4_000_000 + k) for k in range(8)]
    gs = [cvo.upload(s) for s, _, _ in pairs]
    gt = [cvo.upload(t) for _, t, _ in pairs]
    p = cvo.get_params()
    # plain grid
    inits = []
    for s, t in zip(gs, gt):
        Tg, _ = cvo.get_nearest_init_pose(s, t, p.ell_init_first_frame, 0, 1)
        inits.append(scenes.inv_T(Tg))
    Tp, _, it_grid, _ = cvo.align_batch(gs, gt, inits)
    ok_grid = [scenes.pose_error(Tp[k], pairs[k][2]) for k in range(len(pairs))]
    # learned
    Tl, cos, fb, it_learn, _ = cvo.register_learned_batch(net, gs, gt, n_refine=2)
    ok_learn = [scenes.pose_error(Tl[k], pairs[k][2]) for k in range(len(pairs))]
    succ = lambda errs: np.mean([r < 2.0 and t < 0.05 for r, t in errs])
    assert succ(ok_learn) >= succ(ok_grid)
    assert succ(ok_learn) >= 0.75
    # the all-24 grid refines 24 hypotheses per pair; the network refines 2 (+ fallback)
    assert fb.sum() <= 2


def test_invalid_arguments_are_rejected(cvo, small_pool):
    from rkhs_ba_gb300._lib import CvoError
    from rkhs_ba_gb300 import CvoPointCloud
    net = ProposalNet(cvo, points_per_cloud=P_SMALL, seed=7)
    T = np.tile(np.eye(4)[:3], (2, 1, 1))
    with pytest.raises(CvoError):
        net.train_step(small_pool, [0, 4], T, lr=0.0, seed=1)       # scene index out of range
    with pytest.raises(CvoError):
        net.forward_pool(small_pool, [-1], None)
    w = net.weights()
    with pytest.raises(ValueError):
        net.set_weights(w[:-1])
    s, t, _ = scenes.global_pair(n=2000, seed=9)
    gs, gt = cvo.upload(s), cvo.upload(t)
    empty = cvo.upload(CvoPointCloud(np.zeros((0, 3), np.float32), np.zeros((0, 5), np.float32)))
    with pytest.raises(CvoError):
        cvo.register_learned_batch(net, [gs], [empty], n_refine=1)  # empty target
    with pytest.raises(CvoError):
        cvo.register_learned_batch(net, [gs], [gt], n_refine=9)     # more refinements than hypotheses
    # hypotheses of an empty cloud are defined (identity rotation block, centroid 0) and finite
    H = net.hypotheses([gs], [empty])
    assert H.shape == (1, 8, 4, 4) and np.all(np.isfinite(H))


def test_cpu_pipeline_hypotheses_equal_device(cvo):
    """The bench's reference arm computes the network's hypotheses on the host
    (bench.CpuLearned: oracle forward with the committed weights); they are the
    device's hypotheses for the same device-resident pair and weights."""
    import argparse
    import os
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import bench
    cl = bench.CpuLearned(argparse.Namespace(refine_ell=0.4, proposal_weights=""))
    net = ProposalNet(cvo, points_per_cloud=512, seed=0)
    net.set_weights(cl.w)
    src, tgt, _ = scenes.global_pair(n=20000, seed=1234)
    H_dev = net.hypotheses([cvo.upload(src)], [cvo.upload(tgt)])[0]
    H_cpu = cl.hypotheses(src, tgt)
    assert np.allclose(H_dev[:, :3, :3], H_cpu[:, :3, :3], atol=1e-4)
    assert np.allclose(H_dev[:, :3, 3], H_cpu[:, :3, 3], atol=1e-3 * (1 + np.abs(H_cpu[:, :3, 3]).max()))


def test_tcgen05_gemm_matches_mma_sync(cvo, small_pool):
    """The network's matrix products on the tcgen05 tensor cores (TMEM accumulators,
    the default) against the warp-level mma.sync kernel kept as a second opinion:
    both round the same FP32 operands to BF16 and accumulate in FP32, so outputs,
    loss and gradients agree to accumulation order."""
    rng = np.random.default_rng(21)
    scene, T = _batch(rng, 7)
    res = {}
    for kind in (1, 0):
        net = ProposalNet(cvo, points_per_cloud=P_SMALL, seed=9)
        net.set_gemm(kind)
        raw, hyp = net.forward_pool(small_pool, scene, T, seed=13)
        loss = net.train_step(small_pool, scene, T, lr=0.0, seed=13)
        res[kind] = (raw, hyp, loss, net.gradients())
    raw1, hyp1, loss1, g1 = res[1]
    raw0, hyp0, loss0, g0 = res[0]
    scale = float(np.abs(raw1).max())
    assert np.abs(raw0 - raw1).max() <= 1e-3 * scale
    assert abs(loss0 - loss1) <= 1e-3 * abs(loss1)
    assert np.linalg.norm(g0 - g1) <= 1e-2 * np.linalg.norm(g1)
    assert np.allclose(hyp0[:, :, :3, :3], hyp1[:, :, :3, :3], atol=1e-3)
