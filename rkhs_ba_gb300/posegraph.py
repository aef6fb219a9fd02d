"""Keyframe pose graph (the Python mirror of cvo::PoseGraph, src/graph_optimizer/PoseGraph.cpp).

``PoseGraphSolver`` binds the native FP64 SE(3) factor-graph solver
(``cvo_pose_graph_*``): prior and between factors with GTSAM's Pose3 error
definitions, Levenberg-Marquardt to the batch optimum.

``PoseGraph`` follows the reference's tracking flow (:24-320).  Every new frame is
registered by the GB300 CVO against the last frame (frame-to-frame, ``is_f2f``) or the
last keyframe, with the constant-velocity initial guess.  A frame becomes a keyframe
when the cos-angle between it and the last keyframe falls below
``keyframe_threshold``.  Each new keyframe adds a between factor from the last
keyframe (sigmas 0.3 rad / 0.1 m, :440-449); the first keyframe carries a prior
(0.1 / 0.1, :321-345).  Older keyframes whose cos-angle against the last keyframe
exceeds ``loop_quality`` are re-registered and give loop-closure factors
(:367-419, 455-466).  The reference registers keyframe *maps* there (BKI mapping,
not part of this library); here the keyframes' own clouds are used.  The graph is
re-optimised after every keyframe.  The reference's inner-product thresholds (3.90,
0.90, 2.0) are for its CPU CVO's unnormalised inner product; this class uses the
approximate cos-angle (inner product / sqrt(n m)), so its thresholds are parameters.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L

_DP = C.POINTER(C.c_double)

PRIOR_SIGMAS = (0.1, 0.1, 0.1, 0.1, 0.1, 0.1)
BETWEEN_SIGMAS = (0.3, 0.3, 0.3, 0.1, 0.1, 0.1)


def _p12(T) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(T, np.float64).reshape(4, 4)[:3, :].reshape(12))


class PoseGraphSolver:
    """Poses are 4x4 frame -> world matrices; a between measurement is Xi^-1 Xj."""

    def __init__(self):
        self._g = C.c_void_p()
        L.check(L.lib().cvo_pose_graph_create(C.byref(self._g)), "cvo_pose_graph_create")

    def __del__(self):
        try:
            if self._g:
                L.lib().cvo_pose_graph_destroy(self._g)
                self._g = C.c_void_p()
        except Exception:
            pass

    def insert(self, key: int, pose) -> None:
        L.check(L.lib().cvo_pose_graph_insert(self._g, int(key), _p12(pose).ctypes.data_as(_DP)), "cvo_pose_graph_insert")

    def add_prior(self, key: int, pose, sigmas=PRIOR_SIGMAS) -> None:
        s = np.ascontiguousarray(sigmas, np.float64)
        L.check(L.lib().cvo_pose_graph_add_prior(self._g, int(key), _p12(pose).ctypes.data_as(_DP), s.ctypes.data_as(_DP)),
                "cvo_pose_graph_add_prior")

    def add_between(self, i: int, j: int, rel, sigmas=BETWEEN_SIGMAS) -> None:
        s = np.ascontiguousarray(sigmas, np.float64)
        L.check(L.lib().cvo_pose_graph_add_between(self._g, int(i), int(j), _p12(rel).ctypes.data_as(_DP),
                                                   s.ctypes.data_as(_DP)), "cvo_pose_graph_add_between")

    def optimize(self, max_iters: int = 100):
        """Returns (initial cost, final cost, iterations)."""
        c0, c1, it = C.c_double(), C.c_double(), C.c_int()
        L.check(L.lib().cvo_pose_graph_optimize(self._g, int(max_iters), C.byref(c0), C.byref(c1), C.byref(it)),
                "cvo_pose_graph_optimize")
        return c0.value, c1.value, it.value

    def get(self, key: int) -> np.ndarray:
        out = np.zeros(12)
        L.check(L.lib().cvo_pose_graph_get(self._g, int(key), out.ctypes.data_as(_DP)), "cvo_pose_graph_get")
        T = np.eye(4)
        T[:3, :] = out.reshape(3, 4)
        return T

    def size(self):
        n, f = C.c_int(), C.c_int()
        L.lib().cvo_pose_graph_size(self._g, C.byref(n), C.byref(f))
        return n.value, f.value

    def cost(self) -> float:
        c = C.c_double()
        L.check(L.lib().cvo_pose_graph_cost(self._g, C.byref(c)), "cvo_pose_graph_cost")
        return c.value


def _inv(T):
    Ti = np.eye(4)
    Ti[:3, :3] = T[:3, :3].T
    Ti[:3, 3] = -T[:3, :3].T @ T[:3, 3]
    return Ti


class PoseGraph:
    """cvo::PoseGraph(is_f2f, optimizer, num_frames_in_window) with the GB300 CVO as its tracker."""

    def __init__(self, cvo, is_f2f: bool = True, keyframe_threshold: float = 0.5, loop_quality: float = 0.6,
                 loop_accept: float = 0.0, ell: float | None = None, first_pose=None, first_motion_guess=None):
        self.cvo = cvo
        self.is_f2f = is_f2f
        self.keyframe_threshold = keyframe_threshold
        self.loop_quality = loop_quality
        self.loop_accept = loop_accept
        self.ell = cvo.get_params().ell_init if ell is None else ell
        self.first_pose = np.eye(4) if first_pose is None else np.asarray(first_pose, float)
        # the first pair's initial guess (the reference reads it from a file, read_tracking_init_guess, :54-72)
        self.first_motion_guess = np.eye(4) if first_motion_guess is None else np.asarray(first_motion_guess, float)
        self.solver = PoseGraphSolver()
        self.clouds = {}           # frame id -> device cloud
        self.ref = {}              # frame id -> (reference keyframe id, ref -> frame)
        self.keyframes = []        # ids, in order
        self.kf_pose = {}          # keyframe id -> pose in graph
        self.order = []            # every frame id, in order
        self.loop_factors = []     # (i, j, cos-angle)
        self.kf_cos = {}           # frame id -> cos-angle against the last keyframe when it was tracked

    # -- poses -----------------------------------------------------------
    def compute_frame_pose_in_graph(self, fid: int) -> np.ndarray:
        """:74-88: keyframes from the graph, other frames through their keyframe."""
        if fid in self.kf_pose:
            return self.kf_pose[fid]
        r, T = self.ref[fid]
        return self.kf_pose[r] @ T

    def trajectory(self) -> np.ndarray:
        return np.stack([self.compute_frame_pose_in_graph(f) for f in self.order])

    def write_trajectory(self, filename: str) -> None:
        """One row-major 3x4 pose per frame (:541-569)."""
        with open(filename, "w") as fh:
            for T in self.trajectory():
                fh.write(" ".join("%.9g" % v for v in T[:3, :].reshape(12)) + "\n")

    # -- tracking ---------------------------------------------------------
    def _align(self, ref_id: int, new_id: int, guess) -> np.ndarray:
        """ref -> new transform by CVO (source = ref frame, target = new frame)."""
        ret, T_out, _, _, _ = self.cvo.align(self.clouds[ref_id], self.clouds[new_id], _inv(guess))
        return np.asarray(T_out, np.float64)

    def _cos(self, a: int, b: int, T_ab) -> float:
        """Approximate cos-angle (inner product / sqrt(n m)) of frame b moved into frame a."""
        ip = self.cvo.inner_product_batch(self.clouds[a], self.clouds[b], [_inv(T_ab)], self.ell)[0]
        return float(ip) / float(np.sqrt(len(self.clouds[a]) * len(self.clouds[b])))

    def add_new_frame(self, fid: int, cloud) -> bool:
        """Tracks a new frame (:226-320); returns whether it became a keyframe."""
        self.clouds[fid] = self.cvo.upload(cloud) if not hasattr(cloud, "handle") else cloud
        if not self.order:
            self.order.append(fid)
            self.keyframes.append(fid)
            self.kf_pose[fid] = self.first_pose.copy()
            self.solver.insert(fid, self.first_pose)
            self.solver.add_prior(fid, self.first_pose)
            return True
        last = self.order[-1]
        last_kf = self.keyframes[-1]
        # constant-velocity guess (:131-137)
        if len(self.order) >= 2:
            slast = self.order[-2]
            v = _inv(self.compute_frame_pose_in_graph(slast)) @ self.compute_frame_pose_in_graph(last)
        else:
            v = self.first_motion_guess
        if self.is_f2f:
            rel = self._align(last, fid, v)
            kf_to_new = _inv(self.kf_pose[last_kf]) @ self.compute_frame_pose_in_graph(last) @ rel
        else:
            guess = _inv(self.kf_pose[last_kf]) @ self.compute_frame_pose_in_graph(last) @ v
            kf_to_new = self._align(last_kf, fid, guess)
        self.order.append(fid)
        cos_kf = self._cos(last_kf, fid, kf_to_new)
        self.kf_cos[fid] = cos_kf
        if cos_kf >= self.keyframe_threshold:
            self.ref[fid] = (last_kf, kf_to_new)
            return False
        # new keyframe: odometry factor from the last keyframe, loop closures, optimise
        pose = self.kf_pose[last_kf] @ kf_to_new
        self.keyframes.append(fid)
        self.kf_pose[fid] = pose
        self.solver.insert(fid, pose)
        self.solver.add_between(last_kf, fid, kf_to_new)
        for kf in self.keyframes[:-2]:
            T = _inv(self.kf_pose[kf]) @ pose
            q = self._cos(kf, fid, T)
            if q > self.loop_quality:
                Tl = self._align(kf, fid, T)
                ql = self._cos(kf, fid, Tl)
                if ql > q and ql > self.loop_accept:
                    self.solver.add_between(kf, fid, Tl)
                    self.loop_factors.append((kf, fid, ql))
        self.solver.optimize()
        for kf in self.keyframes:
            self.kf_pose[kf] = self.solver.get(kf)
        return True
