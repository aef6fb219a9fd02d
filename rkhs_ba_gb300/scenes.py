"""Seeded synthetic scenes with the shapes of the five benchmark configurations.

No dataset is available offline, so every workload is generated:
  room_pair      10k geometric points: 20x20x5 m room (6 planes) + 3 spheres
  stereo_pair    50k points in a 1226x370 pinhole frustum (fx=718), depth 2-50 m,
                 procedural RGB texture, kept where the image gradient is high;
                 5 features = RGB in [0,1] + gradient/500 + 0.5 (the reference's
                 image-feature convention, src/utils/CvoPointCloud.cpp:534-538)
  lidar_pair     128k points from a 64-beam ring sensor over a street scene,
                 intensity (F=1) and 19-class label distributions
  irls_window    8 frames of 20k-60k stereo points along a smooth trajectory
  global_pair    stereo points with a uniformly random rotation and <= 2 m shift

Every pair generator returns (source, target, T_gt) with the convention of
CvoGPU::align: source points x and target points y satisfy x ~= T_gt @ y, so a
successful registration returns T_out ~= T_gt.
"""
from __future__ import annotations

import numpy as np

from .cloud import CvoPointCloud


# ------------------------------------------------------------------ SE(3)
def rot_axis_angle(axis, ang) -> np.ndarray:
    a = np.asarray(axis, np.float64)
    a = a / np.linalg.norm(a)
    K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    return np.eye(3) + np.sin(ang) * K + (1 - np.cos(ang)) * K @ K


def random_rotation(rng, max_angle=None) -> np.ndarray:
    """Uniform on SO(3) when max_angle is None, else angle U(0, max_angle) about a uniform axis."""
    if max_angle is None:
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        w, x, y, z = q
        return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                         [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                         [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])
    axis = rng.normal(size=3)
    return rot_axis_angle(axis, rng.uniform(0, max_angle))


def make_T(R, t) -> np.ndarray:
    T = np.eye(4)
    T[:3, :3] = R
    T[:3, 3] = t
    return T


def inv_T(T) -> np.ndarray:
    T = np.asarray(T, np.float64)
    R, t = T[:3, :3], T[:3, 3]
    return make_T(R.T, -R.T @ t)


def pose_error(T_est, T_gt):
    """(rotation error in degrees, translation error in metres) of T_gt^-1 T_est."""
    E = inv_T(T_gt) @ np.asarray(T_est, np.float64)
    R = E[:3, :3]
    s = 0.5 * np.linalg.norm([R[2, 1] - R[1, 2], R[0, 2] - R[2, 0], R[1, 0] - R[0, 1]])
    c = (np.trace(R) - 1) / 2
    return float(np.degrees(np.arctan2(s, c))), float(np.linalg.norm(E[:3, 3]))


def _apply(T, p):
    return (np.asarray(p, np.float64) @ T[:3, :3].T + T[:3, 3])


# -------------------------------------------------------------- room (C1)
def _room_surfaces(rng):
    spheres = []
    for _ in range(3):
        r = rng.uniform(0.5, 1.5)
        c = np.array([rng.uniform(-10 + r, 10 - r), rng.uniform(-10 + r, 10 - r), rng.uniform(r, 5 - r)])
        spheres.append((c, r))
    return spheres


def _sample_room(rng, n, spheres):
    # area-weighted: floor, ceiling (400 m^2 each), 4 walls (100 m^2 each), spheres 4 pi r^2
    areas = [400.0, 400.0, 100.0, 100.0, 100.0, 100.0] + [4 * np.pi * r * r for _, r in spheres]
    areas = np.array(areas)
    which = rng.choice(len(areas), size=n, p=areas / areas.sum())
    pts = np.zeros((n, 3))
    u = rng.uniform(-10, 10, size=n)
    v = rng.uniform(-10, 10, size=n)
    h = rng.uniform(0, 5, size=n)
    pts[which == 0] = np.stack([u, v, np.zeros(n)], 1)[which == 0]
    pts[which == 1] = np.stack([u, v, np.full(n, 5.0)], 1)[which == 1]
    pts[which == 2] = np.stack([np.full(n, -10.0), v, h], 1)[which == 2]
    pts[which == 3] = np.stack([np.full(n, 10.0), v, h], 1)[which == 3]
    pts[which == 4] = np.stack([u, np.full(n, -10.0), h], 1)[which == 4]
    pts[which == 5] = np.stack([u, np.full(n, 10.0), h], 1)[which == 5]
    for k, (c, r) in enumerate(spheres):
        m = which == 6 + k
        d = rng.normal(size=(int(m.sum()), 3))
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        pts[m] = c + r * d
    return pts


def room_pair(n=10000, seed=0, max_angle_deg=10.0, max_trans=0.5, noise=0.01):
    """Config 1: geometric-only pair (source = n room points; target = independent
    resample under a random SE(3) plus N(0, noise) per coordinate)."""
    rng = np.random.default_rng(seed)
    spheres = _room_surfaces(rng)
    src = _sample_room(np.random.default_rng(seed * 7919 + 1), n, spheres)
    tgt_scene = _sample_room(np.random.default_rng(seed * 7919 + 2), n, spheres)
    R = random_rotation(rng, np.radians(max_angle_deg))
    d = rng.normal(size=3)
    t = d / np.linalg.norm(d) * rng.uniform(0, max_trans)
    G = make_T(R, t)                 # target frame = G applied to the scene
    tgt = _apply(G, tgt_scene) + rng.normal(scale=noise, size=(n, 3))
    return CvoPointCloud(src), CvoPointCloud(tgt), inv_T(G)


# ------------------------------------------------------- textured world
class _TexturedWorld:
    """Planar patches with a procedural RGB texture defined in world coordinates."""

    def __init__(self, rng, n_patches=48, depth_range=(2.0, 50.0)):
        self.rng = rng
        lo, hi = np.log(depth_range[0]), np.log(depth_range[1])
        P = []
        # ground plane y = +1.6 (camera y axis points down)
        P.append((np.array([0.0, 1.6, 0.0]), np.array([0.0, -1.0, 0.0]), np.array([1.0, 0, 0]), 1e9, 1e9))
        for _ in range(n_patches):
            z = np.exp(rng.uniform(lo, hi))
            x = rng.uniform(-0.9, 0.9) * z * 0.85
            y = rng.uniform(-0.4, 0.25) * z * 0.25
            nrm = np.array([rng.uniform(-0.5, 0.5), rng.uniform(-0.2, 0.2), -1.0])
            nrm /= np.linalg.norm(nrm)
            ax = np.cross(nrm, [0.0, 1.0, 0.0])
            ax /= np.linalg.norm(ax)
            half_w = rng.uniform(0.15, 0.45) * z
            half_h = rng.uniform(0.08, 0.25) * z
            P.append((np.array([x, y, z]), nrm, ax, half_w, half_h))
        self.patches = P
        # texture: sum of random sinusoids in 3-D plus a value-noise lattice
        scales = np.array([1.5, 1.5, 3.0, 3.0, 6.0, 6.0]).reshape(1, 6, 1)
        self.freq = rng.normal(size=(3, 6, 3)) * scales
        self.phase = rng.uniform(0, 2 * np.pi, size=(3, 6))
        self.amp = rng.uniform(0.3, 1.0, size=(3, 6))

    def color(self, p):
        """RGB in [0, 1] at world points p (n, 3)."""
        out = np.zeros((p.shape[0], 3))
        for c in range(3):
            s = np.zeros(p.shape[0])
            for k in range(6):
                s += self.amp[c, k] * np.sin(p @ self.freq[c, k] + self.phase[c, k])
            out[:, c] = 0.5 + 0.5 * np.tanh(1.2 * s)
        return out

    def raycast(self, o, d):
        """Nearest hit of rays o + s d (world frame); returns points and a hit mask."""
        best = np.full(d.shape[0], np.inf)
        for (c, nrm, ax, hw, hh) in self.patches:
            den = d @ nrm
            with np.errstate(divide="ignore", invalid="ignore"):
                s = ((c - o) @ nrm) / den
            ok = (s > 0.1) & np.isfinite(s) & (s < best)
            if hw < 1e8:
                q = o + s[:, None] * d - c
                ay = np.cross(nrm, ax)
                ok &= (np.abs(q @ ax) <= hw) & (np.abs(q @ ay) <= hh)
            best = np.where(ok, s, best)
        hit = np.isfinite(best) & (best < 80.0)
        return o + np.where(hit, best, 0.0)[:, None] * d, hit


_FX, _FY, _CX, _CY, _W, _H = 718.0, 718.0, 613.0, 185.0, 1226, 370


def _stereo_view(world, cam_T, rng, n, noise=0.0):
    """n points seen by a camera with pose cam_T (camera -> world); returns the
    points in the camera frame and 5 features; keeps high-gradient pixels."""
    cand = 4 * n
    u = rng.uniform(0, _W, size=cand)
    v = rng.uniform(0, _H, size=cand)

    def rays(uu, vv):
        d = np.stack([(uu - _CX) / _FX, (vv - _CY) / _FY, np.ones_like(uu)], 1)
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        dw = d @ cam_T[:3, :3].T
        o = np.broadcast_to(cam_T[:3, 3], dw.shape)
        return o, dw

    o, dw = rays(u, v)
    pw, hit = world.raycast(o, dw)
    ou, du = rays(u + 1.0, v)
    pu, hu = world.raycast(ou, du)
    ov, dv = rays(u, v + 1.0)
    pv, hv = world.raycast(ov, dv)
    ok = hit & hu & hv
    col = world.color(pw)
    I = col.mean(1) * 255.0
    gx = world.color(pu).mean(1) * 255.0 - I
    gy = world.color(pv).mean(1) * 255.0 - I
    mag = np.where(ok, np.hypot(gx, gy), -1.0)
    keep = np.argsort(-mag, kind="stable")[:n]
    keep = keep[ok[keep]]
    keep = np.sort(keep)   # pixel sampling order
    Tinv = inv_T(cam_T)
    pc = _apply(Tinv, pw[keep])
    if noise > 0:
        pc = pc + rng.normal(scale=noise, size=pc.shape)
    feats = np.concatenate([col[keep], np.stack([gx[keep], gy[keep]], 1) / 500.0 + 0.5], 1)
    return pc.astype(np.float32), np.clip(feats, 0, 1).astype(np.float32)


def stereo_pair(n=50000, seed=0, max_yaw_deg=3.0, tz_range=(0.5, 1.5)):
    """Config 2: colour pair under forward motion (t_z ~ U(0.5, 1.5) m, yaw <= 3 deg)."""
    rng = np.random.default_rng(seed)
    world = _TexturedWorld(rng)
    cam0 = np.eye(4)
    yaw = np.radians(rng.uniform(-max_yaw_deg, max_yaw_deg))
    cam1 = make_T(rot_axis_angle([0, 1, 0], yaw), [0.0, 0.0, rng.uniform(*tz_range)])
    xs, fs = _stereo_view(world, cam0, np.random.default_rng(seed * 7919 + 1), n)
    xt, ft = _stereo_view(world, cam1, np.random.default_rng(seed * 7919 + 2), n)
    # x_src = inv(cam0) cam1 y_tgt
    return CvoPointCloud(xs, fs), CvoPointCloud(xt, ft), inv_T(cam0) @ cam1


def _global_views(n, seed):
    """The two camera-frame views of a global pair (source, independent resample),
    both centred on the source centroid, and the generator to draw the motion from."""
    rng = np.random.default_rng(seed)
    world = _TexturedWorld(rng)
    cam0 = np.eye(4)
    xs, fs = _stereo_view(world, cam0, np.random.default_rng(seed * 7919 + 1), n)
    xr, fr = _stereo_view(world, cam0, np.random.default_rng(seed * 7919 + 2), n)
    # centre both clouds on the source centroid, as the reference's global benchmark centres its clouds
    c = xs.mean(0)
    return xs - c, fs, xr - c, fr, rng


def global_views(n=2048, seed=0):
    """Unmoved view pair of a global scene as (n, 8) float32 arrays [xyz, 5 features]
    for the proposal network's training pool; the motion is applied on the device."""
    xs, fs, xr, fr, _ = _global_views(n, seed)
    return (np.concatenate([xs, fs], 1).astype(np.float32), np.concatenate([xr, fr], 1).astype(np.float32))


def random_motion(rng, max_trans=2.0):
    """Row-major 3x4 [R | t] drawn like global_pair's motion (uniform rotation, shift <= max_trans)."""
    R = random_rotation(rng)
    d = rng.normal(size=3)
    t = d / np.linalg.norm(d) * rng.uniform(0, max_trans)
    return np.concatenate([R, t[:, None]], 1)


def global_pair(n=50000, seed=0, max_trans=2.0):
    """Config 5: stereo view resampled and moved by a uniformly random rotation and
    a shift <= 2 m (target = G applied to an independent resample of the source view)."""
    xs, fs, xr, fr, rng = _global_views(n, seed)
    R = random_rotation(rng)
    d = rng.normal(size=3)
    t = d / np.linalg.norm(d) * rng.uniform(0, max_trans)
    G = make_T(R, t)
    xt = _apply(G, xr).astype(np.float32)
    return CvoPointCloud(xs, fs), CvoPointCloud(xt, fr), inv_T(G)


def irls_window(n_frames=8, seed=0, size_range=(20000, 60000), step_m=0.8, step_deg=2.0):
    """Config 4: frames along a smooth trajectory; returns (clouds, gt_poses (n, 4, 4)
    frame -> world)."""
    rng = np.random.default_rng(seed)
    world = _TexturedWorld(rng, n_patches=64)
    poses = [np.eye(4)]
    yaw = 0.0
    for k in range(1, n_frames):
        yaw += np.radians(rng.uniform(-step_deg, step_deg))
        prev = poses[-1]
        fwd = prev[:3, :3] @ np.array([0, 0, 1.0])
        poses.append(make_T(rot_axis_angle([0, 1, 0], yaw), prev[:3, 3] + step_m * fwd))
    clouds = []
    for k in range(n_frames):
        nk = int(rng.integers(size_range[0], size_range[1] + 1))
        p, f = _stereo_view(world, poses[k], np.random.default_rng(seed * 7919 + 10 + k), nk)
        clouds.append(CvoPointCloud(p, f))
    return clouds, np.stack(poses)


# ------------------------------------------------------------ lidar (C3)
def _street(rng):
    boxes = []
    for side in (-1, 1):
        x = -60.0
        while x < 60.0:
            w = rng.uniform(6, 15)
            depth = rng.uniform(6, 12)
            hgt = rng.uniform(4, 15)
            off = rng.uniform(8, 12)
            boxes.append((np.array([x, side * off if side > 0 else -off - depth, -1.8]),
                          np.array([x + w, side * off + depth if side > 0 else -off, -1.8 + hgt])))
            x += w + rng.uniform(1, 4)
    poles = [(np.array([rng.uniform(-60, 60), s * rng.uniform(5, 7)]), rng.uniform(0.1, 0.25)) for s in (-1, 1) for _ in range(15)]
    return boxes, poles


def _lidar_scan(boxes, poles, sensor_T, rng, n_beams=64, n_az=2048):
    el = np.radians(np.linspace(-25.0, 3.0, n_beams))
    az = np.linspace(-np.pi, np.pi, n_az, endpoint=False)
    E, A = np.meshgrid(el, az, indexing="ij")
    d = np.stack([np.cos(E) * np.cos(A), np.cos(E) * np.sin(A), np.sin(E)], -1).reshape(-1, 3)
    dw = d @ sensor_T[:3, :3].T
    o = np.broadcast_to(sensor_T[:3, 3], dw.shape)
    best = np.full(dw.shape[0], np.inf)
    label = np.zeros(dw.shape[0], np.int64)
    # ground z = -1.8
    with np.errstate(divide="ignore", invalid="ignore"):
        s = (-1.8 - o[:, 2]) / dw[:, 2]
    ok = (s > 0) & np.isfinite(s)
    best = np.where(ok, s, best)
    label[ok] = 0
    for (lo, hi) in boxes:
        with np.errstate(divide="ignore", invalid="ignore"):
            t1 = (lo - o) / dw
            t2 = (hi - o) / dw
        tn = np.nanmax(np.minimum(t1, t2), axis=1)
        tf = np.nanmin(np.maximum(t1, t2), axis=1)
        ok = (tn <= tf) & (tn > 0) & (tn < best)
        best = np.where(ok, tn, best)
        label[ok] = 2
    for (c, r) in poles:
        oc = o[:, :2] - c
        a = (dw[:, :2] ** 2).sum(1)
        b = 2 * (oc * dw[:, :2]).sum(1)
        cc = (oc ** 2).sum(1) - r * r
        disc = b * b - 4 * a * cc
        with np.errstate(invalid="ignore", divide="ignore"):
            s = (-b - np.sqrt(disc)) / (2 * a)
        z = o[:, 2] + s * dw[:, 2]
        ok = (disc > 0) & (s > 0) & (s < best) & (z < 6.0)
        best = np.where(ok, s, best)
        label[ok] = 5
    hit = np.isfinite(best) & (best > 2.0) & (best < 80.0)
    pw = o + np.where(hit, best, 0)[:, None] * dw
    return pw[hit], label[hit], best[hit]


def lidar_pair(n=128000, seed=0, max_trans=1.5, max_angle_deg=5.0, n_classes=19):
    """Config 3: ring-sensor scans of a street; intensity (F=1) and 19-class label
    distributions (softmax of N(0,1) logits with +4 on the true class)."""
    rng = np.random.default_rng(seed)
    boxes, poles = _street(rng)
    S0 = make_T(np.eye(3), [0, 0, 0])
    R = random_rotation(rng, np.radians(max_angle_deg))
    d = rng.normal(size=3)
    d[2] *= 0.1
    S1 = make_T(R, d / np.linalg.norm(d) * rng.uniform(0, max_trans))

    def scan(S, r2):
        pw, lab, rng_d = _lidar_scan(boxes, poles, S, r2)
        if pw.shape[0] > n:
            keep = np.sort(r2.choice(pw.shape[0], size=n, replace=False))
            pw, lab, rng_d = pw[keep], lab[keep], rng_d[keep]
        pc = _apply(inv_T(S), pw) + r2.normal(scale=0.01, size=pw.shape)
        inten = np.clip(0.3 + 0.1 * lab + 0.2 * np.sin(pw[:, 0] * 0.7) * np.cos(pw[:, 1] * 0.5), 0, 1)
        logits = r2.normal(size=(pw.shape[0], n_classes))
        logits[np.arange(pw.shape[0]), lab] += 4.0
        e = np.exp(logits - logits.max(1, keepdims=True))
        dist = e / e.sum(1, keepdims=True)
        return CvoPointCloud(pc.astype(np.float32), inten[:, None].astype(np.float32), dist.astype(np.float32))

    src = scan(S0, np.random.default_rng(seed * 7919 + 1))
    tgt = scan(S1, np.random.default_rng(seed * 7919 + 2))
    return src, tgt, inv_T(S0) @ S1
