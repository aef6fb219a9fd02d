"""The keyframe pose graph (cvo::PoseGraph, src/graph_optimizer/PoseGraph.cpp) driven by the
GB300 CVO on a seeded 8-frame trajectory (0.8 m / <= 2 deg per step): frame-to-frame
tracking, cos-angle keyframes, odometry and loop-closure factors, FP64 graph solve."""
import numpy as np
import pytest

from rkhs_ba_gb300 import CvoGPU, CvoParams, params_path, scenes
from rkhs_ba_gb300.posegraph import PoseGraph

pytestmark = pytest.mark.gpu


def _err(A, B):
    E = np.linalg.inv(B) @ A
    c = np.clip((np.trace(E[:3, :3]) - 1) / 2, -1, 1)
    return np.degrees(np.arccos(c)), np.linalg.norm(E[:3, 3])


def _run(cvo, clouds, gt, is_f2f, threshold, loop_quality, loop_accept=0.0):
    pg = PoseGraph(cvo, is_f2f=is_f2f, keyframe_threshold=threshold, loop_quality=loop_quality,
                   loop_accept=loop_accept, first_pose=gt[0], first_motion_guess=np.linalg.inv(gt[0]) @ gt[1])
    kfs = [pg.add_new_frame(k, c) for k, c in enumerate(clouds)]
    return pg, kfs


@pytest.mark.parametrize("is_f2f", [True, False])
def test_pose_graph_tracks_trajectory(cuda_device, is_f2f, tmp_path):
    """irls.yaml tracker (colour CVO at the multi-frame lengthscales), the first pair seeded
    like the reference's tracking init-guess file, constant velocity afterwards."""
    clouds, gt = scenes.irls_window(n_frames=8, seed=5, size_range=(15000, 25000))
    cvo = CvoGPU(params=CvoParams(params_path("irls")))
    gs = [cvo.upload(c) for c in clouds]
    # every frame a keyframe (threshold above any cos-angle): an odometry factor between all
    # consecutive frames; loop closures where re-registration beats half the median quality
    pg, kfs = _run(cvo, gs, gt, is_f2f, float("inf"), 1e30)
    assert all(kfs)
    med = float(np.median(list(pg.kf_cos.values())))
    pg, kfs = _run(cvo, gs, gt, is_f2f, float("inf"), 0.5 * med, 0.5 * med)
    n, f = pg.solver.size()
    assert n == 8 and f == 8 + len(pg.loop_factors)   # the prior, 7 odometry factors, the loop closures
    for k, T in enumerate(pg.trajectory()):
        r, t = _err(T, gt[k])
        assert r < 2.5 and t < 0.15, (k, r, t)
    if not is_f2f:
        return
    # keyframes where the cos-angle against the last keyframe drops below its median
    pg2, kfs2 = _run(cvo, gs, gt, is_f2f, med, 1e30)
    assert kfs2[0] and 2 <= sum(kfs2) < 8
    traj = pg2.trajectory()
    for k in range(8):
        r, t = _err(traj[k], gt[k])
        assert r < 2.5 and t < 0.15, (k, r, t)
    path = tmp_path / "traj.txt"
    pg2.write_trajectory(str(path))
    rows = np.loadtxt(path)
    assert rows.shape == (8, 12) and np.allclose(rows, traj[:, :3, :].reshape(8, 12), atol=1e-6)
