"""Pins the CPU oracle (oracle/cvo_oracle.c) with independent evidence:
closed-form Lie-group identities, numpy restatements of the kernel matrix on
tiny inputs, finite differences of the inner product, and the reference's own
rotation grid and demo clouds where available."""
import os

import numpy as np
import pytest
import scipy.linalg as sla

from oracle import oracle as orc
from oracle.params import OracleParams, ParamsC, read_yaml_dict
from rkhs_ba_gb300 import CvoGPU, CvoParams, CvoPointCloud, params_path, scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def hat(w):
    return np.array([[0, -w[2], w[1]], [w[2], 0, -w[0]], [-w[1], w[0], 0]])


@pytest.mark.parametrize("seed", range(5))
def test_exp_sek3_matches_matrix_exponential(seed):
    rng = np.random.default_rng(seed)
    v = rng.normal(size=6).astype(np.float32)
    v /= np.linalg.norm(v)
    dt = float(rng.uniform(1e-4, 0.8))
    X = orc.exp_sek3(v, dt)
    tw = np.zeros((4, 4))
    tw[:3, :3] = hat(v[:3].astype(np.float64)) * dt
    tw[:3, 3] = v[3:].astype(np.float64) * dt
    E = sla.expm(tw)
    assert np.allclose(X, E[:3, :], atol=2e-6)


def test_exp_sek3_small_rotation_branch():
    # theta < 1e-6: R = I and Jl = I (LieGroup.cpp:253-256), so t = v regardless of dt
    v = np.array([0, 0, 0, 0.3, -0.2, 0.1], np.float32)
    X = orc.exp_sek3(v, 0.5)
    assert np.allclose(X[:, :3], np.eye(3)) and np.allclose(X[:, 3], v[3:])


@pytest.mark.parametrize("seed", range(5))
def test_dist_se3_is_norm_of_log(seed):
    rng = np.random.default_rng(seed)
    w = rng.normal(size=3) * rng.uniform(0.01, 2.5) / 2
    u = rng.normal(size=3)
    tw = np.zeros((4, 4))
    tw[:3, :3] = hat(w)
    tw[:3, 3] = u
    T = sla.expm(tw)
    d = orc.dist_se3(T[:3, :3], T[:3, 3])
    assert d == pytest.approx(np.sqrt(w @ w + u @ u), rel=1e-9, abs=1e-12)


def test_cubic_roots_match_numpy():
    rng = np.random.default_rng(1)
    for _ in range(200):
        c = rng.normal(size=4)
        ok, re, im = orc.cubic_roots(*c)
        assert ok
        got = np.sort_complex(re + 1j * im)
        want = np.sort_complex(np.roots(c))
        assert np.allclose(got, want, atol=1e-7 * max(1, np.abs(want).max()))
    ok, _, _ = orc.cubic_roots(0.0, 1.0, 2.0, 3.0)
    assert not ok


def test_step_rule():
    p = CvoParams()
    p.min_step, p.max_step = 1e-4, 0.8
    # 4E s^3 + 3D s^2 + 2C s + B with roots 0.1, 0.3, -0.5 -> smallest positive = 0.1
    poly = np.poly([0.1, 0.3, -0.5])
    bcde = [poly[3], poly[2] / 2, poly[1] / 3, poly[0] / 4]
    assert orc.step_from_terms(p, bcde) == pytest.approx(0.1, rel=1e-12)
    # no positive real root -> temp stays max -> clamped to max_step
    poly = np.poly([-0.1, -0.3, -0.5])
    assert orc.step_from_terms(p, [poly[3], poly[2] / 2, poly[1] / 3, poly[0] / 4]) == pytest.approx(0.8, rel=1e-6)
    # tiny root -> min_step
    poly = np.poly([1e-7, 2.0, 3.0])
    assert orc.step_from_terms(p, [poly[3], poly[2] / 2, poly[1] / 3, poly[0] / 4]) == pytest.approx(1e-4, rel=1e-6)
    # degenerate (E == 0) -> max_step
    assert orc.step_from_terms(p, [1.0, 1.0, 1.0, 0.0]) == pytest.approx(0.8, rel=1e-6)


def _numpy_fill_A(p, src, ytr, cap, ell):
    """Independent numpy restatement of fill_in_A_mat_gpu on tiny inputs (float32 ops in
    the canonical order, kernel values with float64 exp)."""
    f32 = np.float32
    n, m = src.num_points(), ytr.shape[0]
    sigma2 = f32(p.sigma) * f32(p.sigma)
    logg = np.log(f32(p.sp_thres) / sigma2, dtype=np.float32)
    out = []
    for i in range(n):
        x = src.xyz[i]
        nrm = np.sqrt((x[0] * x[0] + x[1] * x[1]) + x[2] * x[2], dtype=np.float32)
        l = f32((float(nrm) / 500.0 + 1.0) * float(f32(ell)))
        d2t = f32(-2.0 * float(l) * float(l) * float(logg))
        row = []
        for j in range(m):
            if len(row) == cap:
                break
            y = ytr[j]
            dx, dy, dz = y[0] - x[0], y[1] - x[1], y[2] - x[2]
            d2 = (dx * dx + dy * dy) + dz * dz
            if not d2 < d2t:
                continue
            k = f32(float(sigma2) * np.exp(-float(d2) / (2.0 * float(l) * float(l))))
            a = f32(f32(f32(1.0) * k) * f32(1.0)) * f32(1.0)
            if a > f32(p.sp_thres):
                row.append((j, a))
        out.append(row)
    return out


@pytest.mark.parametrize("cap", [512, 6])
def test_oracle_kernel_matrix_matches_numpy_restatement(cap):
    src, tgt, _ = scenes.room_pair(n=250, seed=4)
    p = CvoParams(params_path("geometric"))
    ell = 0.9
    ytr = orc.transform_target(np.eye(4), tgt)
    ind, val, nnz = orc.association(p, src, tgt, np.eye(4), ell, cap=cap)
    ref = _numpy_fill_A(p, src, ytr, cap, ell)
    total = 0
    for i in range(src.num_points()):
        assert nnz[i] == len(ref[i])
        assert list(ind[i, :nnz[i]]) == [j for j, _ in ref[i]]
        assert np.array_equal(val[i, :nnz[i]], np.array([a for _, a in ref[i]], np.float32))
        total += nnz[i]
    assert total > 0
    if cap == 6:
        assert (nnz == 6).sum() > 10   # truncation exercised


def _numpy_fill_A_aniso(p, src, ytr, cap, K):
    """Independent numpy restatement of the non-isotropic kernel matrix
    (fill_in_A_mat_gpu_dense_mat_kernel + rotate_kernel_and_inverse, src/cvo/CvoGPU.cu:
    135-183, 719-830) on tiny inputs, float32 scalars in the canonical order, geometry only.
    A source point with z = 0 makes -1/z2 infinite, so its row is NaN and keeps no pair,
    as in the reference (the room's floor points exercise this)."""
    f32 = np.float32
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        return _numpy_fill_A_aniso_rows(p, src, ytr, cap, K)


def _numpy_fill_A_aniso_rows(p, src, ytr, cap, K):
    f32 = np.float32
    Ki = orc.kernel_inverse3(K)
    sigma2 = f32(p.sigma) * f32(p.sigma)
    out = []
    for i in range(src.num_points()):
        x = src.xyz[i].astype(f32)
        nrm = np.sqrt((x[0] * x[0] + x[1] * x[1]) + x[2] * x[2], dtype=f32)
        z = [x[0] / nrm, x[1] / nrm, x[2] / nrm]
        t = f32(-1.0) / z[2]
        xv = [f32(1.0), f32(1.0), t * (z[0] + z[1])]
        yv = [z[1] * xv[2] - z[2] * xv[1], z[2] * xv[0] - z[0] * xv[2], z[0] * xv[1] - z[1] * xv[0]]
        U = [[xv[r], yv[r], z[r]] for r in range(3)]
        P = [[(U[r][0] * Ki[0, c] + U[r][1] * Ki[1, c]) + U[r][2] * Ki[2, c] for c in range(3)] for r in range(3)]
        M = [[(P[r][0] * U[c][0] + P[r][1] * U[c][1]) + P[r][2] * U[c][2] for c in range(3)] for r in range(3)]
        row = []
        for j in range(ytr.shape[0]):
            if len(row) == cap:
                break
            y = ytr[j]
            d = [x[0] - y[0], x[1] - y[1], x[2] - y[2]]
            v = [(d[0] * M[0][c] + d[1] * M[1][c]) + d[2] * M[2][c] for c in range(3)]
            d2 = (v[0] * d[0] + v[1] * d[1]) + v[2] * d[2]
            k = f32(float(sigma2) * np.exp(-float(d2) / 2.0))
            a = f32(f32(f32(1.0) * k) * f32(1.0)) * f32(1.0)
            if a > f32(p.sp_thres):
                row.append((j, a))
        out.append(row)
    return out


@pytest.mark.parametrize("cap", [512, 4])
def test_oracle_nonisotropic_matrix_matches_numpy_restatement(cap):
    s0, t0, _ = scenes.room_pair(n=160, seed=6)
    src, tgt = CvoPointCloud(s0.xyz * 0.1), CvoPointCloud(t0.xyz * 0.1)   # a 2 x 2 x 0.5 m room: dense rows
    p = CvoParams(params_path("geometric"))
    K = np.array([[0.5, 0.05, 0.0], [0.05, 0.4, 0.02], [0.0, 0.02, 0.6]], np.float32)
    ytr = orc.transform_target(np.eye(4), tgt)
    ind, val, nnz = orc.association_aniso(p, src, tgt, np.eye(4), K, cap=cap)
    ref = _numpy_fill_A_aniso(p, src, ytr, cap, K)
    total = 0
    for i in range(src.num_points()):
        assert nnz[i] == len(ref[i]), i
        assert list(ind[i, :nnz[i]]) == [j for j, _ in ref[i]]
        assert np.array_equal(val[i, :nnz[i]], np.array([a for _, a in ref[i]], np.float32))
        total += nnz[i]
    assert total > 0
    if cap == 4:
        assert (nnz == 4).sum() > 10   # index-ordered truncation exercised


def test_oracle_kernel_inverse_and_rotated_kernel():
    rng = np.random.default_rng(2)
    A = rng.normal(size=(3, 3))
    K = (A @ A.T + np.eye(3)).astype(np.float32)
    assert np.allclose(orc.kernel_inverse3(K), np.linalg.inv(K.astype(np.float64)), rtol=1e-5, atol=1e-6)
    x = np.array([0.7, -1.3, 2.1], np.float32)
    z = x / np.linalg.norm(x)
    xv = np.array([1.0, 1.0, -(z[0] + z[1]) / z[2]])
    U = np.stack([xv, np.cross(z, xv), z], 1)          # x and y left unnormalised, as the reference
    Ki = orc.kernel_inverse3(K)
    assert np.allclose(orc.aniso_row_matrix(Ki, x), U @ Ki.astype(np.float64) @ U.T, rtol=1e-5, atol=1e-5)


def test_oracle_rgbd_front_end_matches_numpy_restatement():
    """CvoPointCloud(ImageRGBD, Calibration) restated with numpy float32 scalars: BT.601
    14-bit luma, central-difference gradient, back-projection, validity tests and the
    reference's gradient-feature indexing (gradient[v w + u], gradient[v w + u + 1])."""
    rng = np.random.default_rng(9)
    rows, cols = 24, 31
    img = rng.integers(0, 256, size=(rows, cols, 3), dtype=np.uint8)
    depth = rng.uniform(500, 9000, size=(rows, cols)).astype(np.float32)
    depth[3, 4] = 0.0
    depth[5, 6] = np.nan
    depth[7, 8] = 70000.0                     # 70 m: beyond the 55 m limit
    uv = np.array([[u, v] for v in range(rows) for u in range(0, cols, 3)], np.int32)
    uv = np.vstack([uv, [[4, 3], [6, 5], [8, 7]]]).astype(np.int32)
    intr = np.array([300.0, 310.0, 15.2, 11.7], np.float32)
    xyz, feat, lab, geo = orc.cloud_from_rgbd(img, depth, intr, 1000.0, uv)
    f32 = np.float32
    gray = ((img[..., 0].astype(np.int64) * 1868 + img[..., 1].astype(np.int64) * 9617 +
             img[..., 2].astype(np.int64) * 4899 + 8192) >> 14).astype(np.float32).reshape(-1)
    grad = np.zeros(2 * rows * cols, np.float32)
    for idx in range(cols, cols * (rows - 1)):
        if idx % cols in (0, cols - 1):
            continue
        grad[2 * idx] = f32(0.5) * (gray[idx + 1] - gray[idx - 1])
        grad[2 * idx + 1] = f32(0.5) * (gray[idx + cols] - gray[idx - cols])
    exp_xyz, exp_feat = [], []
    for u, v in uv:
        dep = depth[v, u]
        if dep == 0 or np.isnan(dep):
            continue
        z = f32(dep) / f32(1000.0)
        x = (f32(u) - intr[2]) * z / intr[0]
        y = (f32(v) - intr[3]) * z / intr[1]
        if np.sqrt((x * x + y * y) + z * z, dtype=np.float32) > f32(55.0):
            continue
        pix = v * cols + u
        exp_xyz.append([x, y, z])
        exp_feat.append([f32(img[v, u, 0] / 255.0), f32(img[v, u, 1] / 255.0), f32(img[v, u, 2] / 255.0),
                         f32(float(grad[pix]) / 500.0 + 0.5), f32(float(grad[pix + 1]) / 500.0 + 0.5)])
    assert xyz.shape[0] == len(exp_xyz)
    assert len(exp_xyz) <= uv.shape[0] - 3      # the three invalid pixels are dropped
    assert np.array_equal(xyz, np.array(exp_xyz, np.float32))
    assert np.array_equal(feat, np.array(exp_feat, np.float32))


def test_gradient_is_derivative_of_inner_product():
    """d/ds <f(X), f(exp(-s xi) Y')> at s=0 equals sum_ij a_ij / l_i^2 (omega.(x x y) + v.(y - x))."""
    src, tgt, _ = scenes.room_pair(n=400, seed=2)
    p = CvoParams(params_path("geometric"))
    p.sp_thres = 1e-9          # nearly every pair inside the kernel support: smooth objective
    p.nearest_neighbors_max = 400
    ell = 0.5
    ytr = orc.transform_target(np.eye(4), tgt)
    ind, val, nnz = orc.association(p, src, tgt, np.eye(4), ell)
    g = orc.flow(p, src, ytr, ind, val, nnz)
    w, v = g[:3] * p.c, g[3:] * p.d           # undo the 1/c, 1/d scaling
    pred = 0.0
    for i in range(src.num_points()):
        x = src.xyz[i].astype(np.float64)
        l = (np.linalg.norm(x) / 500.0 + 1.0) * ell
        for t in range(nnz[i]):
            y = ytr[ind[i, t]].astype(np.float64)
            pred += val[i, t] / l ** 2 * (w @ np.cross(x, y) + v @ (y - x))

    def F(s):
        tw = np.zeros((4, 4))
        tw[:3, :3] = hat(w)
        tw[:3, 3] = v
        T = sla.expm(s * tw)        # internal pose; the target moves by its inverse
        return orc.inner_product_gpu_semantics(p, src, tgt, T, ell)[0]

    h = 1e-3 / np.sqrt(w @ w + v @ v)
    fd = (F(h) - F(-h)) / (2 * h)
    assert fd == pytest.approx(pred, rel=2e-2)
    assert pred > 0


def test_step_terms_match_taylor_expansion():
    """B is the first Taylor coefficient in s of sum_ij a_ij exp(-(|x - exp(-s xi) y|^2 - |x - y|^2)/(2l^2)).
    (C, D, E follow the reference's own formulas, src/cvo/CvoGPU.cu:420-460, which are not
    the exact higher-order coefficients; they are mirrored, not checked against the expansion.)"""
    src, tgt, _ = scenes.room_pair(n=200, seed=5)
    p = CvoParams(params_path("geometric"))
    p.nearest_neighbors_max = 200
    ell = 0.6
    ytr = orc.transform_target(np.eye(4), tgt)
    ind, val, nnz = orc.association(p, src, tgt, np.eye(4), ell)
    g = orc.flow(p, src, ytr, ind, val, nnz)
    xi = orc.normalize_grad(g).astype(np.float64)
    bcde = orc.step_terms(p, src, ytr, ind, val, nnz, xi.astype(np.float32), ell)
    W = hat(xi[:3])

    def G(s):
        tot = 0.0
        for i in range(src.num_points()):
            x = src.xyz[i].astype(np.float64)
            for t in range(nnz[i]):
                y = ytr[ind[i, t]].astype(np.float64)
                # the target moves by exp(-s xi): z(s) = y - s u + s^2/2 W u - ..., u = W y + v
                u = W @ y + xi[3:]
                zs = y - s * u + s * s / 2 * (W @ u) - s ** 3 / 6 * (W @ W @ u) + s ** 4 / 24 * (W @ W @ W @ u)
                d0 = x - y
                ds = x - zs
                tot += val[i, t] * np.exp(-(ds @ ds - d0 @ d0) / (2 * ell * ell))
        return tot

    ss = np.linspace(-0.02, 0.02, 9)
    vals = np.array([G(s) for s in ss])
    coef = np.polyfit(ss, vals, 4)[::-1]   # a0 + a1 s + ...
    # sum a_ij exp(...) = sum a_ij (1 + B s + C s^2 + D s^3 + E s^4 + ...)
    assert coef[1] == pytest.approx(bcde[0], rel=1e-3)


def test_cpu_inner_product_library_matches_oracle():
    src, tgt, _ = scenes.stereo_pair(n=2000, seed=1)
    p = CvoParams(params_path("color"))
    cvo = CvoGPU(params=p)
    T = scenes.make_T(scenes.rot_axis_angle([0, 1, 0], 0.02), [0.1, 0, 0.3])
    for ell in (0.3, 1.0):
        lib_v = cvo.inner_product_cpu(src, tgt, T, ell)
        orc_v, _ = orc.inner_product_cpu_semantics(p, src, tgt, T, ell)
        assert lib_v == pytest.approx(orc_v, rel=1e-6)
    # non-approximate CPU cos-angle of a cloud with itself is 1
    assert cvo.function_angle(src, src, np.eye(4), 0.3, is_approximate=False, is_gpu=False) == pytest.approx(1.0, rel=1e-5)
    assert orc.function_angle(p, src, src, np.eye(4), 0.3, False, False) == pytest.approx(1.0, rel=1e-5)


def test_cpu_inner_product_library_matches_oracle_full_size():
    """The reference's CPU inner product (radius search, no cap) at the 50,000-point colour
    size: the library's OpenMP implementation and the oracle agree to 1e-6 relative."""
    src, tgt, _ = scenes.stereo_pair(n=50000, seed=2)
    p = CvoParams(params_path("color"))
    cvo = CvoGPU(params=p)
    lib_v = cvo.inner_product_cpu(src, tgt, np.eye(4), 0.4)
    orc_v, _ = orc.inner_product_cpu_semantics(p, src, tgt, np.eye(4), 0.4)
    assert orc_v > 1e5
    assert lib_v == pytest.approx(orc_v, rel=1e-6)


def test_rotation_grids_are_groups():
    for kind, n in ((0, 60), (1, 24)):
        G = CvoGPU.rotation_grid(kind).astype(np.float64)
        assert G.shape == (n, 3, 3)
        for R in G:
            assert np.allclose(R @ R.T, np.eye(3), atol=1e-6) and np.linalg.det(R) == pytest.approx(1, abs=1e-6)
        # closed under composition
        for a in range(0, n, 7):
            for b in range(0, n, 5):
                M = G[a] @ G[b]
                assert np.min(np.abs(G - M).reshape(n, -1).max(1)) < 1e-5
    assert CvoGPU.rotation_grid(2, 3).shape == (27, 3, 3)


def test_icosahedral_grid_equals_reference_set():
    """The 60 rotations regenerated from the icosahedral symmetry are the set that
    gen_icosahedron_init_rots (src/cvo/CvoGPU.cpp:279-342) lists (as a set, to float
    rounding); the reference's table is the fixture tests/golden/icosahedral_rotations.npz
    written by tests/golden/make_golden.py."""
    ref = np.load(os.path.join(GOLDEN, "icosahedral_rotations.npz"))["R"]
    G = CvoGPU.rotation_grid(0).astype(np.float64)
    assert ref.shape == (60, 3, 3)
    for R in ref:
        assert np.min(np.abs(G - R).reshape(60, -1).max(1)) < 2e-6
    for R in G:
        assert np.min(np.abs(ref - R).reshape(60, -1).max(1)) < 2e-6


def test_demo_pcd_fixture_reads_like_reference():
    """tests/golden/demo_pair.npz holds the demo clouds converted by tests/golden/make_golden.py;
    reading them back through our PCD writer/reader round-trips exactly."""
    d = np.load(os.path.join(GOLDEN, "demo_pair.npz"))
    src = CvoPointCloud(d["src_xyz"], d["src_feat"], None, np.tile([[0, 1]], (d["src_xyz"].shape[0], 1)))
    assert src.num_points() == 523 and d["tgt_xyz"].shape[0] == 1080
    assert src.feature_dimensions() == 3
    assert np.all((src.features >= 0) & (src.features <= 1))


def test_pcd_roundtrip(tmp_path):
    rng = np.random.default_rng(0)
    f = (rng.integers(0, 256, size=(40, 3)) / 255.0).astype(np.float32)
    c = CvoPointCloud(rng.normal(size=(40, 3)), f)
    path = str(tmp_path / "a.pcd")
    c.write_pcd(path)
    r = CvoPointCloud.read_pcd(path)
    assert np.array_equal(r.xyz, c.xyz)
    assert np.allclose(r.features, c.features, atol=1e-7)
    assert np.array_equal(r.geom_type, np.tile([[0, 1]], (40, 1)).astype(np.float32))


def test_golden_oracle_outputs_stable():
    """Regression pin of the oracle on the demo clouds (values generated by make_golden.py)."""
    d = np.load(os.path.join(GOLDEN, "demo_pair.npz"))
    g = np.load(os.path.join(GOLDEN, "demo_oracle.npz"))
    src = CvoPointCloud(d["src_xyz"], d["src_feat"])
    tgt = CvoPointCloud(d["tgt_xyz"], d["tgt_feat"])
    p = OracleParams(params_path("color"))
    p.MAX_ITER = int(g["max_iter"])
    v, z = orc.inner_product_gpu_semantics(p, src, tgt, np.eye(4), float(g["ell"]))
    assert z == int(g["ip_nnz"]) and v == pytest.approx(float(g["ip"]), rel=1e-12)
    ret, T, iters, _ = orc.align(p, src, tgt, np.eye(4))
    assert iters == int(g["iters"]) and np.allclose(T, g["T_out"], atol=1e-6)


# ------------------------------------------------------------------ parameters
def _same_params(a, b):
    da, db = a.as_dict(), b.as_dict()
    assert da.keys() == db.keys()
    for k in da:
        assert np.float32(da[k]) == np.float32(db[k]) if isinstance(da[k], float) else da[k] == db[k], k


def test_oracle_params_layout_matches_library():
    """The oracle's parameter structure has the library's layout (both follow
    struct cvo_params of include/cvo_gb300.h, which the C oracle reads)."""
    import ctypes as C
    from rkhs_ba_gb300 import _lib as L
    assert C.sizeof(ParamsC) == C.sizeof(L.CvoParamsC)
    for (fa, ta), (fb, tb) in zip(ParamsC._fields_, L.CvoParamsC._fields_):
        assert fa == fb and ta == tb and getattr(ParamsC, fa).offset == getattr(L.CvoParamsC, fb).offset


@pytest.mark.parametrize("name", ["geometric", "color", "lidar_semantic", "irls", None])
def test_oracle_yaml_reader_agrees_with_library(name):
    """Two independent readers of the parameter files -- the oracle's (Python) and
    the library's (C++, cvo_params_read_yaml) -- give the same values, so the
    parity tests do not rest on one parser (None: the constructor defaults)."""
    path = params_path(name) if name else None
    _same_params(OracleParams(path), CvoParams(path))


def test_oracle_yaml_reader_edge_cases(tmp_path):
    """Comments, quotes, repeated and unknown keys, keys the reference never reads
    from a file, and values yaml-cpp would reject: both readers agree."""
    from rkhs_ba_gb300._lib import CvoError
    f = tmp_path / "p.yaml"
    f.write_text("%YAML:1.0\n---\n# comment line\nsigma: 0.25   # trailing comment\n"
                 "c_ell: '0.05'\nMAX_ITER: 40\nMAX_ITER: 41\nnot_a_field: 3\nstep: 9.0\n"
                 "multiframe_iter_per_ell: 77\nmultiframe_iterations_per_ell: 12\ndl: 1e-3\n"
                 "is_using_intensity: +1\n...\n")
    o, p = OracleParams(str(f)), CvoParams(str(f))
    _same_params(o, p)
    assert o.MAX_ITER == 41 and o.step == 0.0 and o.multiframe_iter_per_ell == 10
    assert o.multiframe_iterations_per_ell == 12 and o.is_using_intensity == 1
    assert np.float32(o.c_ell) == np.float32(0.05) and o.dl == 1e-3
    assert read_yaml_dict(str(f))["sigma"] == 0.25
    bad = tmp_path / "bad.yaml"
    bad.write_text("MAX_ITER: 1.5\n")
    with pytest.raises(ValueError):
        OracleParams(str(bad))
    with pytest.raises(CvoError):
        CvoParams(str(bad))
