"""The FP64 pose-graph solver (cvo_pose_graph_*, the custom solver standing in for
GTSAM in src/graph_optimizer/PoseGraph.cpp) against closed forms and the scipy oracle
(oracle/posegraph.py).  Host code only: runs without a GPU."""
import numpy as np
import pytest

from oracle import posegraph as opg
from rkhs_ba_gb300.posegraph import BETWEEN_SIGMAS, PRIOR_SIGMAS, PoseGraphSolver


def _rand_pose(rng, ang=0.3, tr=1.0):
    xi = np.concatenate([rng.normal(size=3) * ang, rng.normal(size=3) * tr])
    return opg.exp(xi)


def _perturb(rng, T, ang=0.05, tr=0.1):
    return T @ opg.exp(np.concatenate([rng.normal(size=3) * ang, rng.normal(size=3) * tr]))


def test_log_exp_round_trip_and_near_pi():
    rng = np.random.default_rng(0)
    for _ in range(50):
        xi = np.concatenate([rng.normal(size=3), rng.normal(size=3)])
        assert np.allclose(opg.log(opg.exp(xi)), xi, atol=1e-9) or np.linalg.norm(xi[:3]) > np.pi
    # the native solver's log through a single prior factor's cost: e = Log(P^-1 X)
    for ang in (1e-9, 1e-3, 1.0, np.pi - 1e-4):
        axis = rng.normal(size=3)
        axis /= np.linalg.norm(axis)
        X = opg.exp(np.concatenate([axis * ang, rng.normal(size=3)]))
        g = PoseGraphSolver()
        g.insert(0, X)
        g.add_prior(0, np.eye(4), (1, 1, 1, 1, 1, 1))
        e = opg.log(X)
        assert np.isclose(g.cost(), 0.5 * e @ e, rtol=1e-9, atol=1e-18), ang


def test_chain_recovers_composed_odometry():
    rng = np.random.default_rng(1)
    Z = [_rand_pose(rng) for _ in range(6)]
    truth = [np.eye(4)]
    for z in Z:
        truth.append(truth[-1] @ z)
    g = PoseGraphSolver()
    for k, T in enumerate(truth):
        g.insert(k, _perturb(rng, T))
    g.add_prior(0, truth[0])
    for k, z in enumerate(Z):
        g.add_between(k, k + 1, z)
    c0, c1, it = g.optimize()
    assert c1 < 1e-16 and c1 <= c0
    for k, T in enumerate(truth):
        assert np.allclose(g.get(k), T, atol=1e-7), k


def test_inconsistent_loop_matches_oracle():
    rng = np.random.default_rng(2)
    truth = [np.eye(4)]
    for _ in range(7):
        truth.append(truth[-1] @ _rand_pose(rng, 0.2, 0.8))
    factors = [("prior", 0, truth[0], PRIOR_SIGMAS)]
    g = PoseGraphSolver()
    init = {}
    for k, T in enumerate(truth):
        init[k] = _perturb(rng, T, 0.1, 0.3)
        g.insert(k, init[k])
    g.add_prior(0, truth[0])
    edges = [(k, k + 1) for k in range(7)] + [(0, 4), (2, 7), (1, 6)]
    for i, j in edges:
        Zn = _perturb(rng, opg.inv(truth[i]) @ truth[j], 0.02, 0.05)     # noisy measurements: an inconsistent graph
        g.add_between(i, j, Zn)
        factors.append(("between", i, j, Zn, BETWEEN_SIGMAS))
    c0, c1, it = g.optimize(200)
    ref = opg.optimize(init, factors)
    assert np.isclose(c1, opg.cost(ref, factors), rtol=1e-7, atol=1e-12)
    for k in range(8):
        assert np.allclose(g.get(k), ref[k], atol=1e-6), k
    assert c1 < c0


def test_errors_and_gauge():
    g = PoseGraphSolver()
    g.insert(0, np.eye(4))
    g.insert(1, np.eye(4))
    g.add_between(0, 1, _rand_pose(np.random.default_rng(3)))
    from rkhs_ba_gb300._lib import CvoError
    with pytest.raises(CvoError):
        g.optimize()                                  # no prior: the gauge is free
    with pytest.raises(CvoError):
        g.add_between(0, 7, np.eye(4))                # unknown key
    with pytest.raises(CvoError):
        g.add_prior(0, np.eye(4), (0.1, 0.1, 0.0, 0.1, 0.1, 0.1))   # non-positive sigma
    g.add_prior(0, np.eye(4))
    c0, c1, it = g.optimize()
    assert c1 < 1e-16
    assert g.size() == (2, 2)


def test_more_rejected_inputs():
    from rkhs_ba_gb300._lib import CvoError
    g = PoseGraphSolver()
    bad = np.eye(4)
    bad[0, 3] = np.nan
    with pytest.raises(CvoError):
        g.insert(0, bad)                              # non-finite pose
    g.insert(0, np.eye(4))
    with pytest.raises(CvoError):
        g.add_between(0, 0, np.eye(4))                # a factor needs two poses
    with pytest.raises(CvoError):
        g.add_prior(3, np.eye(4))                     # unknown key
    with pytest.raises(CvoError):
        g.get(3)
    with pytest.raises(CvoError):
        g.add_between(0, 0, bad)
    # re-inserting a key replaces its value; sizes count poses and factors
    g.insert(0, _rand_pose(np.random.default_rng(5)))
    assert g.size() == (1, 0)
    g.add_prior(0, np.eye(4))
    c0, c1, it = g.optimize()
    assert c1 <= c0 and c1 < 1e-16
    assert np.allclose(g.get(0), np.eye(4), atol=1e-9)
