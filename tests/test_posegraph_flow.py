"""Host logic of the keyframe pose graph (rkhs_ba_gb300/posegraph.py, the mirror of
src/graph_optimizer/PoseGraph.cpp:24-569) with a stand-in tracker: registration
returns the true relative motion with a known error, and the quality score falls with
the distance between frames.  Runs without a GPU (the FP64 solver is host code)."""
import numpy as np

from oracle import posegraph as opg
from rkhs_ba_gb300.posegraph import PoseGraph


class _Cloud:
    def __init__(self, fid):
        self.fid = fid
        self.handle = fid

    def __len__(self):
        return 100


class _Params:
    ell_init = 0.5


class FakeCvo:
    """align(ref, new, T_init) returns ref -> new with a fixed rotation error; the cos-angle
    score is exp(-distance / 1 m) between the frames at the tested pose."""

    def __init__(self, gt, err_xi):
        self.gt = gt
        self.err = opg.exp(err_xi)
        self.calls = {"align": 0, "ip": 0}

    def get_params(self):
        return _Params()

    def upload(self, c):
        return c

    def align(self, src, tgt, T_init):
        self.calls["align"] += 1
        rel = opg.inv(self.gt[src.fid]) @ self.gt[tgt.fid]
        return 0, rel @ self.err, None, 0.0, 10

    def inner_product_batch(self, src, tgt, Ts, ell):
        self.calls["ip"] += 1
        T_ab = opg.inv(np.asarray(Ts[0]))                  # the tested ref -> new transform
        true = opg.inv(self.gt[src.fid]) @ self.gt[tgt.fid]
        d = np.linalg.norm(true[:3, 3]) + np.linalg.norm(opg.log(opg.inv(true) @ T_ab))
        return np.array([100.0 * np.exp(-d)])             # divided by sqrt(100 * 100) -> exp(-d)


def _trajectory(n=10, step=0.4):
    gt = [np.eye(4)]
    for k in range(1, n):
        gt.append(gt[-1] @ opg.exp(np.array([0, 0.02, 0, 0, 0, step])))
    return gt


def test_keyframes_follow_the_threshold_and_poses_compose():
    gt = _trajectory()
    cvo = FakeCvo(gt, np.zeros(6))
    pg = PoseGraph(cvo, is_f2f=True, keyframe_threshold=np.exp(-1.0), loop_quality=1e30)
    kfs = [pg.add_new_frame(k, _Cloud(k)) for k in range(len(gt))]
    assert kfs[0]
    # a frame becomes a keyframe once it is more than ~1 m (score exp(-1)) from the last keyframe
    last = 0
    for k in range(1, len(gt)):
        d = np.linalg.norm((opg.inv(gt[last]) @ gt[k])[:3, 3])
        assert kfs[k] == (d > 1.0), (k, d)
        if kfs[k]:
            last = k
    for k, T in enumerate(pg.trajectory()):
        assert np.allclose(T, gt[k], atol=1e-9)
    n, f = pg.solver.size()
    assert n == sum(kfs) and f == n                    # the prior and one odometry factor per later keyframe


def test_loop_closures_pull_a_biased_odometry_back():
    gt = _trajectory(n=8, step=0.3)
    bias = np.array([0, 0.004, 0, 0.01, 0, 0])          # every registration slightly wrong
    odo = PoseGraph(FakeCvo(gt, bias), is_f2f=True, keyframe_threshold=1e30, loop_quality=1e30)
    loop = PoseGraph(FakeCvo(gt, bias), is_f2f=False, keyframe_threshold=1e30, loop_quality=0.0)
    for k in range(len(gt)):
        odo.add_new_frame(k, _Cloud(k))
        loop.add_new_frame(k, _Cloud(k))
    assert len(loop.loop_factors) > 0
    err = lambda pg: np.linalg.norm(pg.trajectory()[-1][:3, 3] - gt[-1][:3, 3])
    assert err(odo) > 0.05                               # the bias accumulates
    assert err(loop) <= err(odo) + 1e-9


def test_write_trajectory(tmp_path):
    gt = _trajectory(n=4)
    pg = PoseGraph(FakeCvo(gt, np.zeros(6)), keyframe_threshold=1e30, loop_quality=1e30)
    for k in range(4):
        pg.add_new_frame(k, _Cloud(k))
    path = tmp_path / "traj.txt"
    pg.write_trajectory(str(path))
    rows = np.loadtxt(path)
    assert rows.shape == (4, 12)
    for k in range(4):
        assert np.allclose(rows[k].reshape(3, 4), gt[k][:3, :], atol=1e-7)
