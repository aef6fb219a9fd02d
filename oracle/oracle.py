"""ctypes wrapper of the C oracle (oracle/cvo_oracle.c), built by ``build()``.

TEST INFRASTRUCTURE ONLY: the checker for tests/, __graft_entry__.smoke() and
the CPU baseline of bench.py.  Parity is unpinned against the reference binary
(it cannot be compiled here); the oracle restates the reference's arithmetic.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "cvo_oracle.c")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libcvo_oracle.so")
CFLAGS = ["-O2", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-std=c11"]

_L = None


def build(force: bool = False) -> str:
    """Compile the oracle with gcc (no fused multiply-add) into oracle/_build/."""
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cmd = ["gcc"] + CFLAGS + ["-I" + os.path.join(HERE, "..", "include"), SRC, "-o", LIB + ".tmp", "-lm"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


def build_sanitized() -> str:
    """The oracle under AddressSanitizer and UndefinedBehaviorSanitizer, in
    oracle/_build/asan/ (same arithmetic flags)."""
    out = os.path.join(OUT_DIR, "asan", "libcvo_oracle.so")
    os.makedirs(os.path.dirname(out), exist_ok=True)
    flags = [f for f in CFLAGS if f != "-O2"] + ["-O1", "-g", "-fno-omit-frame-pointer", "-fsanitize=address,undefined",
                                                 "-fno-sanitize-recover=undefined"]
    cmd = ["gcc"] + flags + ["-I" + os.path.join(HERE, "..", "include"), SRC, "-o", out, "-lm"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return out


def _lib():
    global _L
    if _L is None:
        build()
        _L = C.CDLL(LIB)
        fp = C.POINTER(C.c_float)
        ip = C.POINTER(C.c_int)
        dp = C.POINTER(C.c_double)
        vp = C.c_void_p
        sig = {
            "orc_fill_A": (C.c_int, [vp, vp, vp, fp, C.c_int, C.c_float, ip, fp, ip]),
            "orc_transform": (None, [fp, fp, vp, fp]),
            "orc_pose_to_rinv": (None, [fp, fp, fp]),
            "orc_flow": (None, [vp, vp, fp, C.c_int, ip, fp, ip, dp]),
            "orc_normalize_grad": (None, [dp, fp]),
            "orc_step_terms": (None, [vp, vp, fp, C.c_int, ip, fp, ip, fp, C.c_float, dp]),
            "orc_cubic_roots": (C.c_int, [C.c_double] * 4 + [dp, dp]),
            "orc_step_from_terms": (C.c_double, [vp, dp]),
            "orc_exp_sek3": (None, [fp, C.c_float, fp]),
            "orc_dist_se3": (C.c_double, [dp, dp]),
            "orc_align": (C.c_int, [vp, vp, vp, fp, fp, ip, vp]),
            "orc_align_adaptive": (C.c_int, [vp, vp, vp, fp, fp, ip, vp]),
            "orc_fill_adaptive": (C.c_int, [vp, fp, fp, fp, C.c_int, fp, fp, fp, C.c_int, C.c_int, C.c_int, C.c_float,
                                            ip, fp, ip]),
            "orc_inner_product_gpu": (C.c_double, [vp, vp, vp, fp, C.c_float, C.POINTER(C.c_int64)]),
            "orc_inner_product_cpu": (C.c_double, [vp, vp, vp, fp, C.c_float, C.POINTER(C.c_int64)]),
            "orc_function_angle": (C.c_double, [vp, vp, vp, fp, C.c_float, C.c_int, C.c_int]),
            "orc_association": (C.c_int, [vp, vp, vp, fp, C.c_float, C.c_int, ip, fp, ip]),
            "orc_association_aniso": (C.c_int, [vp, vp, vp, fp, fp, C.c_int, ip, fp, ip]),
            "orc_kernel_inverse3": (None, [fp, fp]),
            "orc_aniso_row_matrix": (None, [fp, fp, fp]),
            "orc_cloud_from_rgbd": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, fp, fp, C.c_float, ip, C.c_int, vp,
                                              C.c_int, vp, fp, fp, fp, fp]),
            "orc_nearest_init_pose": (C.c_int, [vp, vp, vp, C.c_float, fp, C.c_int, fp, fp]),
            "orc_num_threads": (C.c_int, []),
            "orc_set_num_threads": (None, [C.c_int]),
        }
        for k, (r, a) in sig.items():
            f = getattr(_L, k)
            f.restype = r
            f.argtypes = a
    return _L


class OrcATrace(C.Structure):
    _fields_ = [("ell", C.POINTER(C.c_float)), ("dl", C.POINTER(C.c_double)), ("step", C.POINTER(C.c_double)),
                ("nnz3", C.POINTER(C.c_int64)), ("grad", C.POINTER(C.c_float)), ("max_len", C.c_int)]


ADAPTIVE_CAP = 512


class OrcTrace(C.Structure):
    _fields_ = [("ell", C.POINTER(C.c_float)), ("step", C.POINTER(C.c_double)),
                ("nnz", C.POINTER(C.c_int64)), ("dist", C.POINTER(C.c_double)),
                ("xi", C.POINTER(C.c_float)), ("max_len", C.c_int)]


_fp = C.POINTER(C.c_float)


def _f(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _m16(T):
    return _f(np.asarray(T, np.float32).reshape(4, 4).T.reshape(16))


def _pp(params):
    return C.cast(C.byref(params._c), C.c_void_p)


def _pc(cs):
    return C.cast(C.byref(cs), C.c_void_p)


def set_threads(n: int) -> None:
    _lib().orc_set_num_threads(int(n))


def num_threads() -> int:
    return int(_lib().orc_num_threads())


def transform_target(T, cloud) -> np.ndarray:
    """Target positions moved by inverse(T) in the canonical float order."""
    Ri = np.zeros(9, np.float32)
    Ti = np.zeros(3, np.float32)
    Tm = _m16(T)
    L = _lib()
    L.orc_pose_to_rinv(Tm.ctypes.data_as(_fp), Ri.ctypes.data_as(_fp), Ti.ctypes.data_as(_fp))
    out = np.zeros((cloud.num_points(), 3), np.float32)
    cs = cloud.c_struct()
    L.orc_transform(Ri.ctypes.data_as(_fp), Ti.ctypes.data_as(_fp), _pc(cs), out.ctypes.data_as(_fp))
    return out


def association(params, src, tgt, T, ell, cap=None):
    """ELL kernel matrix with GPU semantics: returns (ind (n, cap), val (n, cap), nnz (n,))."""
    cap = params.nearest_neighbors_max if cap is None else cap
    n = src.num_points()
    ind = np.zeros((n, max(cap, 1)), np.int32)
    val = np.zeros((n, max(cap, 1)), np.float32)
    nnz = np.zeros(n, np.int32)
    s, t = src.c_struct(), tgt.c_struct()
    Tm = _m16(T)
    _lib().orc_association(_pp(params), _pc(s), _pc(t), Tm.ctypes.data_as(_fp), float(ell), int(cap),
                           ind.ctypes.data_as(C.POINTER(C.c_int)), val.ctypes.data_as(_fp),
                           nnz.ctypes.data_as(C.POINTER(C.c_int)))
    return ind[:, :cap], val[:, :cap], nnz


def kernel_inverse3(K):
    """The oracle's float 3x3 inverse (cofactors of column 0, times 1/det); K, result (3, 3)."""
    Kc = np.ascontiguousarray(np.asarray(K, np.float32).T.reshape(9))   # column-major
    out = np.zeros(9, np.float32)
    _lib().orc_kernel_inverse3(Kc.ctypes.data_as(_fp), out.ctypes.data_as(_fp))
    return out.reshape(3, 3).T


def aniso_row_matrix(Ki, x):
    """M = U Ki U^T of rotate_kernel_and_inverse for source point x (row-major (3, 3))."""
    Kc = np.ascontiguousarray(np.asarray(Ki, np.float32).T.reshape(9))
    xv = np.ascontiguousarray(np.asarray(x, np.float32).reshape(3))
    out = np.zeros(9, np.float32)
    _lib().orc_aniso_row_matrix(Kc.ctypes.data_as(_fp), xv.ctypes.data_as(_fp), out.ctypes.data_as(_fp))
    return out.reshape(3, 3)


def association_aniso(params, src, tgt, T, kernel, cap=None):
    """Non-isotropic kernel matrix (compute_association_gpu with a 3x3 kernel) as ELL:
    (ind (n, cap), val (n, cap), nnz (n,)), the first cap kept pairs per row by index."""
    cap = params.nearest_neighbors_max if cap is None else cap
    n = src.num_points()
    ind = np.zeros((n, max(cap, 1)), np.int32)
    val = np.zeros((n, max(cap, 1)), np.float32)
    nnz = np.zeros(n, np.int32)
    s, t = src.c_struct(), tgt.c_struct()
    Tm = _m16(T)
    Kc = np.ascontiguousarray(np.asarray(kernel, np.float32).T.reshape(9))
    _lib().orc_association_aniso(_pp(params), _pc(s), _pc(t), Tm.ctypes.data_as(_fp), Kc.ctypes.data_as(_fp),
                                 int(cap), ind.ctypes.data_as(C.POINTER(C.c_int)), val.ctypes.data_as(_fp),
                                 nnz.ctypes.data_as(C.POINTER(C.c_int)))
    return ind[:, :cap], val[:, :cap], nnz


def cloud_from_rgbd(image, depth, intrinsic, scaling_factor, uv, geom_type=None, semantics=None):
    """RGB-D frame + selected pixels -> (xyz (k, 3), features (k, F), labels (k, C), geom (k, 2) or None)."""
    img = np.ascontiguousarray(image, np.uint8)
    rows, cols = img.shape[:2]
    ch = 1 if img.ndim == 2 else img.shape[2]
    dep = np.ascontiguousarray(depth, np.float32)
    intr = np.ascontiguousarray(intrinsic, np.float32)
    uvc = np.ascontiguousarray(uv, np.int32).reshape(-1, 2)
    n = uvc.shape[0]
    Cn = 0 if semantics is None else semantics.shape[-1]
    sem = None if semantics is None else np.ascontiguousarray(semantics, np.float32)
    geo = None if geom_type is None else np.ascontiguousarray(geom_type, np.float32)
    F = ch + 2
    xyz = np.zeros((max(n, 1), 3), np.float32)
    feat = np.zeros((max(n, 1), F), np.float32)
    lab = np.zeros((max(n, 1), max(Cn, 1)), np.float32)
    og = np.zeros((max(n, 1), 2), np.float32)
    k = _lib().orc_cloud_from_rgbd(img.ctypes.data_as(C.c_void_p), rows, cols, ch, dep.ctypes.data_as(_fp),
                                   intr.ctypes.data_as(_fp), float(scaling_factor), uvc.ctypes.data_as(C.POINTER(C.c_int)),
                                   n, None if geo is None else geo.ctypes.data_as(C.c_void_p), Cn,
                                   None if sem is None else sem.ctypes.data_as(C.c_void_p), xyz.ctypes.data_as(_fp),
                                   feat.ctypes.data_as(_fp), lab.ctypes.data_as(_fp), og.ctypes.data_as(_fp))
    return xyz[:k], feat[:k], lab[:k, :Cn], (og[:k] if geo is not None else None)


def flow(params, src, ytr, ind, val, nnz):
    cap = ind.shape[1]
    out = np.zeros(6, np.float64)
    s = src.c_struct()
    ind = np.ascontiguousarray(ind, np.int32)
    val = np.ascontiguousarray(val, np.float32)
    nnz = np.ascontiguousarray(nnz, np.int32)
    ytr = _f(ytr)
    _lib().orc_flow(_pp(params), _pc(s), ytr.ctypes.data_as(_fp), cap, ind.ctypes.data_as(C.POINTER(C.c_int)),
                    val.ctypes.data_as(_fp), nnz.ctypes.data_as(C.POINTER(C.c_int)),
                    out.ctypes.data_as(C.POINTER(C.c_double)))
    return out


def normalize_grad(g):
    g = np.ascontiguousarray(g, np.float64)
    xi = np.zeros(6, np.float32)
    _lib().orc_normalize_grad(g.ctypes.data_as(C.POINTER(C.c_double)), xi.ctypes.data_as(_fp))
    return xi


def step_terms(params, src, ytr, ind, val, nnz, xi, ell):
    cap = ind.shape[1]
    out = np.zeros(4, np.float64)
    s = src.c_struct()
    ind = np.ascontiguousarray(ind, np.int32)
    val = np.ascontiguousarray(val, np.float32)
    nnz = np.ascontiguousarray(nnz, np.int32)
    ytr = _f(ytr)
    xi = _f(xi)
    _lib().orc_step_terms(_pp(params), _pc(s), ytr.ctypes.data_as(_fp), cap, ind.ctypes.data_as(C.POINTER(C.c_int)),
                          val.ctypes.data_as(_fp), nnz.ctypes.data_as(C.POINTER(C.c_int)), xi.ctypes.data_as(_fp),
                          float(ell), out.ctypes.data_as(C.POINTER(C.c_double)))
    return out


def step_from_terms(params, bcde):
    b = np.ascontiguousarray(bcde, np.float64)
    return float(_lib().orc_step_from_terms(_pp(params), b.ctypes.data_as(C.POINTER(C.c_double))))


def cubic_roots(c3, c2, c1, c0):
    re = np.zeros(3)
    im = np.zeros(3)
    ok = _lib().orc_cubic_roots(c3, c2, c1, c0, re.ctypes.data_as(C.POINTER(C.c_double)),
                                im.ctypes.data_as(C.POINTER(C.c_double)))
    return bool(ok), re, im


def exp_sek3(v, dt):
    v = _f(v)
    X = np.zeros(12, np.float32)
    _lib().orc_exp_sek3(v.ctypes.data_as(_fp), float(dt), X.ctypes.data_as(_fp))
    return X.reshape(3, 4)


def dist_se3(R, t):
    R = np.ascontiguousarray(R, np.float64).reshape(9)
    t = np.ascontiguousarray(t, np.float64).reshape(3)
    return float(_lib().orc_dist_se3(R.ctypes.data_as(C.POINTER(C.c_double)), t.ctypes.data_as(C.POINTER(C.c_double))))


def align(params, src, tgt, T_init, trace_len: int = 0):
    """align_impl restated on the CPU.  Returns (ret, T_out (4x4), iters, trace dict)."""
    s, t = src.c_struct(), tgt.c_struct()
    Ti = _m16(T_init)
    To = np.zeros(16, np.float32)
    iters = C.c_int(0)
    tr = None
    arrays = {}
    if trace_len > 0:
        arrays = dict(ell=np.zeros(trace_len, np.float32), step=np.zeros(trace_len), nnz=np.zeros(trace_len, np.int64),
                      dist=np.zeros(trace_len), xi=np.zeros((trace_len, 6), np.float32))
        tr = OrcTrace(arrays["ell"].ctypes.data_as(_fp), arrays["step"].ctypes.data_as(C.POINTER(C.c_double)),
                      arrays["nnz"].ctypes.data_as(C.POINTER(C.c_int64)),
                      arrays["dist"].ctypes.data_as(C.POINTER(C.c_double)), arrays["xi"].ctypes.data_as(_fp), trace_len)
    ret = _lib().orc_align(_pp(params), _pc(s), _pc(t), Ti.ctypes.data_as(_fp), To.ctypes.data_as(_fp),
                           C.byref(iters), C.cast(C.byref(tr), C.c_void_p) if tr is not None else None)
    return ret, To.reshape(4, 4).T.copy(), iters.value, arrays


def align_adaptive(params, src, tgt, T_init, trace_len: int = 0):
    """AdaptiveCvoGPU::align restated on the CPU.  Returns (ret, T_out (4x4), iters, trace dict
    with per-iteration ell, dl, step, nnz of A / Axx / Ayy and the raw gradient)."""
    s, t = src.c_struct(), tgt.c_struct()
    Ti = _m16(T_init)
    To = np.zeros(16, np.float32)
    iters = C.c_int(0)
    tr = None
    arrays = {}
    if trace_len > 0:
        arrays = dict(ell=np.zeros(trace_len, np.float32), dl=np.zeros(trace_len), step=np.zeros(trace_len),
                      nnz3=np.zeros((trace_len, 3), np.int64), grad=np.zeros((trace_len, 6), np.float32))
        dp = C.POINTER(C.c_double)
        tr = OrcATrace(arrays["ell"].ctypes.data_as(_fp), arrays["dl"].ctypes.data_as(dp),
                       arrays["step"].ctypes.data_as(dp), arrays["nnz3"].ctypes.data_as(C.POINTER(C.c_int64)),
                       arrays["grad"].ctypes.data_as(_fp), trace_len)
    ret = _lib().orc_align_adaptive(_pp(params), _pc(s), _pc(t), Ti.ctypes.data_as(_fp), To.ctypes.data_as(_fp),
                                    C.byref(iters), C.cast(C.byref(tr), C.c_void_p) if tr is not None else None)
    return ret, To.reshape(4, 4).T.copy(), iters.value, arrays


def fill_adaptive(params, xs, fx, lx, ys, fy, ly, ell):
    """Adaptive-path kernel matrix of rows xs (n, 3) against ys (m, 3) (features / labels
    (n, F) / (n, C) or None): (ind (n, 512), val (n, 512), nnz (n,))."""
    xs = np.ascontiguousarray(xs, np.float32)
    ys = np.ascontiguousarray(ys, np.float32)
    n, m = len(xs), len(ys)
    F = 0 if fx is None else fx.shape[1]
    Cn = 0 if lx is None else lx.shape[1]
    f32 = lambda a: None if a is None else np.ascontiguousarray(a, np.float32)
    fx, fy, lx, ly = f32(fx), f32(fy), f32(lx), f32(ly)
    ptr = lambda a: a.ctypes.data_as(_fp) if a is not None else None
    ind = np.zeros((max(n, 1), ADAPTIVE_CAP), np.int32)
    val = np.zeros((max(n, 1), ADAPTIVE_CAP), np.float32)
    nnz = np.zeros(max(n, 1), np.int32)
    ip = C.POINTER(C.c_int)
    _lib().orc_fill_adaptive(_pp(params), ptr(xs), ptr(fx), ptr(lx), n, ptr(ys), ptr(fy), ptr(ly), m, F, Cn,
                             float(ell), ind.ctypes.data_as(ip), val.ctypes.data_as(_fp), nnz.ctypes.data_as(ip))
    return ind[:n], val[:n], nnz[:n]


def inner_product_gpu_semantics(params, src, tgt, T, ell):
    s, t = src.c_struct(), tgt.c_struct()
    Tm = _m16(T)
    z = C.c_int64(0)
    v = _lib().orc_inner_product_gpu(_pp(params), _pc(s), _pc(t), Tm.ctypes.data_as(_fp), float(ell), C.byref(z))
    return float(v), int(z.value)


def inner_product_cpu_semantics(params, src, tgt, T, ell):
    s, t = src.c_struct(), tgt.c_struct()
    Tm = _m16(T)
    z = C.c_int64(0)
    v = _lib().orc_inner_product_cpu(_pp(params), _pc(s), _pc(t), Tm.ctypes.data_as(_fp), float(ell), C.byref(z))
    return float(v), int(z.value)


def function_angle(params, src, tgt, T, ell, is_approximate=True, is_gpu=True):
    s, t = src.c_struct(), tgt.c_struct()
    Tm = _m16(T)
    return float(_lib().orc_function_angle(_pp(params), _pc(s), _pc(t), Tm.ctypes.data_as(_fp), float(ell),
                                           int(is_approximate), int(is_gpu)))


def nearest_init_pose(params, src, tgt, ell, rots):
    rots = _f(np.asarray(rots).reshape(-1, 9))
    nr = rots.shape[0]
    s, t = src.c_struct(), tgt.c_struct()
    To = np.zeros(16, np.float32)
    cos = np.zeros(nr, np.float32)
    bi = _lib().orc_nearest_init_pose(_pp(params), _pc(s), _pc(t), float(ell), rots.ctypes.data_as(_fp), nr,
                                      To.ctypes.data_as(_fp), cos.ctypes.data_as(_fp))
    return bi, To.reshape(4, 4).T.copy(), cos


def align_multi(params, clouds, poses, hold_const, edges):
    """CvoBatchIRLS::solve restated (see oracle/cvo_oracle.c).  poses: (n, 12) row-major
    3x4 frame->world; returns (poses_out, outer_iterations, lm_successful_steps)."""
    L = _lib()
    if not hasattr(L.orc_align_multi, "_bound"):
        L.orc_align_multi.restype = C.c_int
        L.orc_align_multi.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_uint8),
                                      C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.orc_align_multi._bound = True
    from rkhs_ba_gb300._lib import CvoCloudC
    n = len(clouds)
    cs = (CvoCloudC * n)(*[c.c_struct() for c in clouds])
    P = np.ascontiguousarray(np.asarray(poses, np.float64).reshape(n, 12).copy())
    hc = np.ascontiguousarray(np.asarray(hold_const, np.uint8).reshape(n))
    E = np.ascontiguousarray(np.asarray(edges, np.int32).reshape(-1, 2))
    steps = C.c_int(0)
    it = L.orc_align_multi(_pp(params), n, C.cast(cs, C.c_void_p), P.ctypes.data_as(C.POINTER(C.c_double)),
                           hc.ctypes.data_as(C.POINTER(C.c_uint8)), E.shape[0], E.ctypes.data_as(C.POINTER(C.c_int)),
                           C.byref(steps))
    return P, it, steps.value
