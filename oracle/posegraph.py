"""CPU oracle of the FP64 pose-graph solver (test infrastructure only).

The reference hands its keyframe graph to GTSAM (src/graph_optimizer/PoseGraph.cpp:
321-495): a PriorFactor<Pose3> on the first keyframe and BetweenFactor<Pose3>
odometry / loop-closure factors with diagonal noise.  GTSAM is not available, so this
module restates the published factor definitions (GTSAM 4, Pose3 with the
exponential-map retraction) independently of the native solver, with scipy's
rotation log / exp and scipy.optimize.least_squares:

    prior    e = Log(P^-1 X),  between  e = Log(Z^-1 Xi^-1 Xj),  e = (omega, rho)
    cost     1/2 sum |e / sigma|^2

Poses are 4x4 homogeneous matrices (frame -> world).  Only tests use this module.
"""
from __future__ import annotations

import numpy as np
from scipy.optimize import least_squares
from scipy.spatial.transform import Rotation


def _V_inv(w):
    th = np.linalg.norm(w)
    W = np.array([[0, -w[2], w[1]], [w[2], 0, -w[0]], [-w[1], w[0], 0]])
    if th < 1e-5:
        k = 1.0 / 12.0 + th * th / 720.0
    else:
        k = (1.0 - th * np.sin(th) / (2.0 * (1.0 - np.cos(th)))) / (th * th)
    return np.eye(3) - 0.5 * W + k * W @ W


def log(T):
    """SE(3) logarithm (omega, rho) of a 4x4 pose."""
    w = Rotation.from_matrix(T[:3, :3]).as_rotvec()
    return np.concatenate([w, _V_inv(w) @ T[:3, 3]])


def exp(xi):
    w, rho = np.asarray(xi[:3], float), np.asarray(xi[3:], float)
    th = np.linalg.norm(w)
    W = np.array([[0, -w[2], w[1]], [w[2], 0, -w[0]], [-w[1], w[0], 0]])
    if th < 1e-5:
        B, C = 0.5 - th * th / 24.0, 1.0 / 6.0 - th * th / 120.0
    else:
        B, C = (1.0 - np.cos(th)) / th ** 2, (th - np.sin(th)) / th ** 3
    T = np.eye(4)
    T[:3, :3] = Rotation.from_rotvec(w).as_matrix()
    T[:3, 3] = (np.eye(3) + B * W + C * W @ W) @ rho
    return T


def inv(T):
    Ti = np.eye(4)
    Ti[:3, :3] = T[:3, :3].T
    Ti[:3, 3] = -T[:3, :3].T @ T[:3, 3]
    return Ti


def residuals(poses, factors):
    """Whitened residuals; factors: ("prior", key, P, sigmas) / ("between", i, j, Z, sigmas)."""
    out = []
    for f in factors:
        if f[0] == "prior":
            _, k, P, s = f
            out.append(log(inv(P) @ poses[k]) / np.asarray(s))
        else:
            _, i, j, Z, s = f
            out.append(log(inv(Z) @ inv(poses[i]) @ poses[j]) / np.asarray(s))
    return np.concatenate(out) if out else np.zeros(0)


def cost(poses, factors):
    r = residuals(poses, factors)
    return 0.5 * float(r @ r)


def optimize(poses, factors, tol=1e-14):
    """Batch optimum over X_k <- X_k Exp(d_k) from the given initial poses (dict key -> 4x4)."""
    keys = sorted(poses)
    base = {k: np.array(poses[k], float) for k in keys}

    def unpack(d):
        return {k: base[k] @ exp(d[6 * n:6 * n + 6]) for n, k in enumerate(keys)}

    res = least_squares(lambda d: residuals(unpack(d), factors), np.zeros(6 * len(keys)), method="lm",
                        xtol=tol, ftol=tol, gtol=tol, max_nfev=20000)
    return unpack(res.x)
