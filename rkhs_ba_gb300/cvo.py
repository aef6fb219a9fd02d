"""``CvoGPU``: the Python mirror of the reference's ``cvo::CvoGPU`` class.

Method names, argument meaning, pose conventions and return codes follow
include/UnifiedCvo/cvo/CvoGPU.hpp:43-274; every call goes through the C ABI of
the native library (include/cvo_gb300.h).  4x4 matrices are numpy arrays in
the usual row-major (4, 4) shape; they are passed to the library column-major.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L
from .cloud import CvoPointCloud

_FP = C.POINTER(C.c_float)


def _m16(T) -> np.ndarray:
    T = np.asarray(T, dtype=np.float32).reshape(4, 4)
    return np.ascontiguousarray(T.T.reshape(16))


def _from16(a) -> np.ndarray:
    return np.asarray(a, dtype=np.float32).reshape(4, 4).T.copy()


class CvoParams:
    """cvo::CvoParams (include/UnifiedCvo/cvo/CvoParams.hpp:12-136) as attributes."""

    def __init__(self, yaml_path: str | None = None):
        self._c = L.CvoParamsC()
        L.lib().cvo_params_default(C.byref(self._c))
        if yaml_path is not None:
            self.read_yaml(yaml_path)

    def read_yaml(self, path: str) -> "CvoParams":
        L.check(L.lib().cvo_params_read_yaml(path.encode(), C.byref(self._c)), "cvo_params_read_yaml")
        return self

    def __getattr__(self, k):
        if k.startswith("_"):
            raise AttributeError(k)
        return getattr(self._c, k)

    def __setattr__(self, k, v):
        if k.startswith("_"):
            object.__setattr__(self, k, v)
        else:
            if not any(k == f for f, _ in L.PARAM_FIELDS):
                raise AttributeError("unknown CvoParams field %r" % k)
            setattr(self._c, k, v)

    def as_dict(self) -> dict:
        return {f: getattr(self._c, f) for f, _ in L.PARAM_FIELDS}

    def copy(self) -> "CvoParams":
        p = CvoParams()
        C.memmove(C.byref(p._c), C.byref(self._c), C.sizeof(L.CvoParamsC))
        return p


@dataclass
class Association:
    """cvo::Association (include/UnifiedCvo/cvo/Association.hpp:5-12): CSR rows are
    source indices, columns target indices."""
    rows: int = 0
    cols: int = 0
    row_ptr: np.ndarray = field(default_factory=lambda: np.zeros(1, np.int64))
    col: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    val: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))
    source_inliers: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    target_inliers: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))

    @property
    def nnz(self) -> int:
        return int(self.col.shape[0])

    def to_scipy(self):
        import scipy.sparse as sp
        return sp.csr_matrix((self.val, self.col, self.row_ptr), shape=(self.rows, self.cols))


@dataclass
class CvoResultInfo:
    """cvo::CvoResultInfo (include/UnifiedCvo/cvo/CvoGPU.hpp:34-40)."""
    return_code: int
    T_s2t: np.ndarray
    association: Association | None
    registration_seconds: float
    num_iters: int


class GpuCloud:
    """A cloud resident on the GPU (CvoPointCloudGPU); freed with the object."""

    def __init__(self, cvo: "CvoGPU", cloud: CvoPointCloud):
        self._cvo = cvo
        self.cloud = cloud
        self._h = C.c_void_p()
        cs = cloud.c_struct()
        L.check(L.lib().cvo_cloud_upload(cvo._h, C.byref(cs), C.byref(self._h)), "cvo_cloud_upload", cvo._h)

    @classmethod
    def _wrap(cls, cvo: "CvoGPU", handle: C.c_void_p) -> "GpuCloud":
        g = cls.__new__(cls)
        g._cvo = cvo
        g.cloud = None
        g._h = handle
        return g

    @property
    def handle(self):
        return self._h

    def __len__(self):
        return L.lib().cvo_cloud_size(self._h)

    def download(self) -> CvoPointCloud:
        """The cloud's points, features, labels and geometric types copied back (original order)."""
        F, Cn, hg = C.c_int(), C.c_int(), C.c_int()
        lib = L.lib()
        L.check(lib.cvo_cloud_dims(self._h, C.byref(F), C.byref(Cn), C.byref(hg)), "cvo_cloud_dims")
        n = len(self)
        xyz = np.zeros((n, 3), np.float32)
        feat = np.zeros((n, F.value), np.float32)
        lab = np.zeros((n, Cn.value), np.float32)
        geo = np.zeros((n, 2), np.float32)
        L.check(lib.cvo_cloud_download(self._cvo._h, self._h, xyz.ctypes.data_as(_FP),
                                       feat.ctypes.data_as(_FP) if F.value else None,
                                       lab.ctypes.data_as(_FP) if Cn.value else None,
                                       geo.ctypes.data_as(_FP) if hg.value else None), "cvo_cloud_download",
                self._cvo._h)
        return CvoPointCloud(xyz, feat if F.value else None, lab if Cn.value else None, geo if hg.value else None)

    def free(self):
        if self._h:
            L.lib().cvo_cloud_free(self._cvo._h, self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def _read_assoc(a) -> Association:
    lib = L.lib()
    rows, cols = C.c_int(), C.c_int()
    nnz, ns, nt = C.c_int64(), C.c_int64(), C.c_int64()
    lib.cvo_assoc_info(a, C.byref(rows), C.byref(cols), C.byref(nnz), C.byref(ns), C.byref(nt))
    rp = np.zeros(rows.value + 1, np.int64)
    col = np.zeros(nnz.value, np.int32)
    val = np.zeros(nnz.value, np.float32)
    si = np.zeros(ns.value, np.int32)
    ti = np.zeros(nt.value, np.int32)
    lib.cvo_assoc_copy(a, rp.ctypes.data_as(C.POINTER(C.c_int64)), col.ctypes.data_as(C.POINTER(C.c_int)),
                       val.ctypes.data_as(_FP), si.ctypes.data_as(C.POINTER(C.c_int)),
                       ti.ctypes.data_as(C.POINTER(C.c_int)))
    return Association(rows.value, cols.value, rp, col, val, si, ti)


class _AssocBuf:
    def __init__(self):
        self.h = C.c_void_p()
        L.check(L.lib().cvo_assoc_create(C.byref(self.h)), "cvo_assoc_create")

    def __del__(self):
        if self.h:
            L.lib().cvo_assoc_destroy(self.h)


class CvoGPU:
    """GB300-native drop-in for cvo::CvoGPU."""

    def __init__(self, param_file: str | None = None, params: CvoParams | None = None):
        self._h = C.c_void_p()
        lib = L.lib()
        if params is not None:
            L.check(lib.cvo_create_with_params(C.byref(params._c), C.byref(self._h)), "cvo_create_with_params")
        elif param_file is not None:
            L.check(lib.cvo_create(param_file.encode(), C.byref(self._h)), "cvo_create")
        else:
            L.check(lib.cvo_create_with_params(C.byref(CvoParams()._c), C.byref(self._h)), "cvo_create_with_params")

    def close(self):
        if self._h:
            L.lib().cvo_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- parameters -----------------------------------------------------
    def get_params(self) -> CvoParams:
        p = CvoParams()
        L.check(L.lib().cvo_get_params(self._h, C.byref(p._c)), "cvo_get_params")
        return p

    def write_params(self, p: CvoParams) -> None:
        L.check(L.lib().cvo_write_params(self._h, C.byref(p._c)), "cvo_write_params")

    @property
    def kernel_launches(self) -> int:
        return int(L.lib().cvo_kernel_launch_count(self._h))

    def set_stream(self, stream_ptr: int | None) -> None:
        """Run the handle's work on a caller's CUDA stream (e.g. torch.cuda.current_stream().cuda_stream)."""
        L.check(L.lib().cvo_set_stream(self._h, C.c_void_p(stream_ptr) if stream_ptr else None), "cvo_set_stream")

    def profile(self, on: bool = True) -> None:
        L.check(L.lib().cvo_profile_enable(self._h, int(on)), "cvo_profile_enable")

    def profile_reset(self) -> None:
        L.check(L.lib().cvo_profile_reset(self._h), "cvo_profile_reset")

    def profile_read(self) -> dict:
        ms, n, b, it = C.c_double(), C.c_int64(), C.c_double(), C.c_int64()
        L.check(L.lib().cvo_profile_read(self._h, C.byref(ms), C.byref(n), C.byref(b), C.byref(it)), "cvo_profile_read")
        k = (C.c_double * 5)()
        L.check(L.lib().cvo_profile_kernels(self._h, k), "cvo_profile_kernels")
        names = ("transform", "assoc", "reduce", "step", "iteration")
        sp = (C.c_double * 3)()
        L.check(L.lib().cvo_profile_assoc_split(self._h, sp), "cvo_profile_assoc_split")
        return {"assoc_ms": ms.value, "assoc_launches": n.value, "assoc_bytes": b.value, "iterations": it.value,
                "kernel_ms": {names[i]: k[i] for i in range(5)},
                "assoc_split_ms": {"kernel": sp[0], "select": sp[1], "rowsum": sp[2]}}

    def upload(self, cloud: CvoPointCloud) -> GpuCloud:
        return GpuCloud(self, cloud)

    def cloud_from_rgbd(self, image, depth, intrinsic, scaling_factor, uv, geom_type=None, semantics=None) -> GpuCloud:
        """CvoPointCloud(ImageRGBD, Calibration, ...) built on the device
        (src/utils/CvoPointCloud.cpp:458-560): image (rows, cols[, 3]) uint8 BGR, depth
        (rows, cols) raw units, intrinsic (fx, fy, cx, cy), uv (n, 2) selected pixels."""
        img = np.ascontiguousarray(image, np.uint8)
        rows, cols = img.shape[:2]
        ch = 1 if img.ndim == 2 else img.shape[2]
        dep = np.ascontiguousarray(depth, np.float32)
        intr = np.ascontiguousarray(intrinsic, np.float32)
        uvc = np.ascontiguousarray(uv, np.int32).reshape(-1, 2)
        geo = None if geom_type is None else np.ascontiguousarray(geom_type, np.float32)
        sem = None if semantics is None else np.ascontiguousarray(semantics, np.float32)
        Cn = 0 if sem is None else sem.shape[-1]
        out = C.c_void_p()
        npts = C.c_int()
        rc = L.lib().cvo_cloud_from_rgbd(self._h, img.ctypes.data_as(C.c_void_p), rows, cols, ch, dep.ctypes.data_as(_FP),
                                         intr.ctypes.data_as(_FP), float(scaling_factor),
                                         uvc.ctypes.data_as(C.POINTER(C.c_int)), uvc.shape[0],
                                         None if geo is None else geo.ctypes.data_as(_FP), Cn,
                                         None if sem is None else sem.ctypes.data_as(_FP), C.byref(out), C.byref(npts))
        L.check(rc, "cvo_cloud_from_rgbd", self._h)
        return GpuCloud._wrap(self, out)

    # -- two-view -------------------------------------------------------
    def align(self, source, target, T_init, want_association: bool = False):
        """int CvoGPU::align(src, tgt, T_target_frame_to_source_frame, T_out&, assoc*, secs*, iters*)
        (src/cvo/CvoGPU.cu:1516-1563).  Returns (ret, T_out, association, seconds, iters);
        T_init is the internal initial pose (callers pass init_guess.inverse())."""
        T_out = np.zeros(16, np.float32)
        secs = C.c_double(0)
        iters = C.c_int(0)
        ab = _AssocBuf() if want_association else None
        Ti = _m16(T_init)
        lib = L.lib()
        if isinstance(source, GpuCloud):
            rc = lib.cvo_align_dev(self._h, source.handle, target.handle, Ti.ctypes.data_as(_FP),
                                   T_out.ctypes.data_as(_FP), ab.h if ab else None, C.byref(secs), C.byref(iters))
        else:
            s, t = source.c_struct(), target.c_struct()
            rc = lib.cvo_align(self._h, C.byref(s), C.byref(t), Ti.ctypes.data_as(_FP), T_out.ctypes.data_as(_FP),
                               ab.h if ab else None, C.byref(secs), C.byref(iters))
        L.check(rc, "cvo_align", self._h)
        assoc = _read_assoc(ab.h) if ab else None
        return (0 if rc == L.CVO_OK else -1), _from16(T_out), assoc, secs.value, iters.value

    def align_s2t(self, source: CvoPointCloud, target: CvoPointCloud, T_s2t, is_returning_association=False):
        """CvoResultInfo CvoGPU::align(src, tgt, T_source_frame_to_target_frame, assoc)
        (src/cvo/CvoGPU.cu:1566-1611)."""
        T_out = np.zeros(16, np.float32)
        secs = C.c_double(0)
        iters = C.c_int(0)
        ret = C.c_int(0)
        ab = _AssocBuf() if is_returning_association else None
        s, t = source.c_struct(), target.c_struct()
        Ti = _m16(T_s2t)
        L.check(L.lib().cvo_align_s2t(self._h, C.byref(s), C.byref(t), Ti.ctypes.data_as(_FP), int(bool(ab)),
                                      T_out.ctypes.data_as(_FP), ab.h if ab else None, C.byref(secs), C.byref(iters),
                                      C.byref(ret)), "cvo_align_s2t", self._h)
        return CvoResultInfo(ret.value, _from16(T_out), _read_assoc(ab.h) if ab else None, secs.value, iters.value)

    def align_batch(self, sources, targets, T_inits):
        """Batched two-view align of device clouds (one persistent batch)."""
        n = len(sources)
        S = (C.c_void_p * n)(*[s.handle.value for s in sources])
        Tg = (C.c_void_p * n)(*[t.handle.value for t in targets])
        Ti = np.ascontiguousarray(np.concatenate([_m16(T) for T in T_inits]).astype(np.float32))
        To = np.zeros(16 * n, np.float32)
        rets = np.zeros(n, np.int32)
        its = np.zeros(n, np.int32)
        secs = C.c_double(0)
        L.check(L.lib().cvo_align_batch_dev(self._h, n, S, Tg, Ti.ctypes.data_as(_FP), To.ctypes.data_as(_FP),
                                            rets.ctypes.data_as(C.POINTER(C.c_int)),
                                            its.ctypes.data_as(C.POINTER(C.c_int)), C.byref(secs)),
                "cvo_align_batch_dev", self._h)
        return [_from16(To[16 * i:16 * i + 16]) for i in range(n)], rets, its, secs.value

    # -- inner products -------------------------------------------------
    def inner_product_gpu(self, source, target, T, ell: float) -> float:
        out = C.c_float(0)
        Ti = _m16(T)
        lib = L.lib()
        if isinstance(source, GpuCloud):
            rc = lib.cvo_inner_product_dev(self._h, source.handle, target.handle, Ti.ctypes.data_as(_FP),
                                           float(ell), C.byref(out))
        else:
            s, t = source.c_struct(), target.c_struct()
            rc = lib.cvo_inner_product(self._h, C.byref(s), C.byref(t), Ti.ctypes.data_as(_FP), float(ell),
                                       C.byref(out))
        L.check(rc, "cvo_inner_product", self._h)
        return out.value

    def inner_product_batch(self, source: GpuCloud, target: GpuCloud, Ts, ell: float) -> np.ndarray:
        n = len(Ts)
        Ti = np.ascontiguousarray(np.concatenate([_m16(T) for T in Ts]).astype(np.float32))
        out = np.zeros(n, np.float32)
        L.check(L.lib().cvo_inner_product_batch_dev(self._h, source.handle, target.handle, n, Ti.ctypes.data_as(_FP),
                                                    float(ell), out.ctypes.data_as(_FP)),
                "cvo_inner_product_batch_dev", self._h)
        return out

    def inner_product_cpu(self, source: CvoPointCloud, target: CvoPointCloud, T, ell: float) -> float:
        out = C.c_float(0)
        s, t = source.c_struct(), target.c_struct()
        Ti = _m16(T)
        L.check(L.lib().cvo_inner_product_cpu(self._h, C.byref(s), C.byref(t), Ti.ctypes.data_as(_FP), float(ell),
                                              C.byref(out)), "cvo_inner_product_cpu", self._h)
        return out.value

    def function_angle(self, source: CvoPointCloud, target: CvoPointCloud, T, ell: float,
                       is_approximate: bool = True, is_gpu: bool = True) -> float:
        out = C.c_float(0)
        s, t = source.c_struct(), target.c_struct()
        Ti = _m16(T)
        L.check(L.lib().cvo_function_angle(self._h, C.byref(s), C.byref(t), Ti.ctypes.data_as(_FP), float(ell),
                                           int(is_approximate), int(is_gpu), C.byref(out)),
                "cvo_function_angle", self._h)
        return out.value

    def compute_association_gpu(self, source, target, T, ell_or_kernel) -> Association:
        """CvoGPU::compute_association_gpu, both overloads: a float lengthscale
        (src/cvo/CvoGPU.cu:1836-1871) or a 3x3 non-isotropic geometric kernel
        (:1936-1950, Eigen::Matrix3f; passed here as a (3, 3) array)."""
        ab = _AssocBuf()
        Ti = _m16(T)
        lib = L.lib()
        K = np.asarray(ell_or_kernel, np.float32)
        if K.ndim == 2:
            Kc = np.ascontiguousarray(K.reshape(3, 3).T.reshape(9))   # column-major like Eigen
            if isinstance(source, GpuCloud):
                rc = lib.cvo_compute_association_aniso_dev(self._h, source.handle, target.handle, Ti.ctypes.data_as(_FP),
                                                           Kc.ctypes.data_as(_FP), ab.h)
            else:
                s, t = source.c_struct(), target.c_struct()
                rc = lib.cvo_compute_association_aniso(self._h, C.byref(s), C.byref(t), Ti.ctypes.data_as(_FP),
                                                       Kc.ctypes.data_as(_FP), ab.h)
            L.check(rc, "cvo_compute_association_aniso", self._h)
            return _read_assoc(ab.h)
        s, t = source.c_struct(), target.c_struct()
        L.check(lib.cvo_compute_association(self._h, C.byref(s), C.byref(t), Ti.ctypes.data_as(_FP),
                                            float(ell_or_kernel), ab.h), "cvo_compute_association", self._h)
        return _read_assoc(ab.h)

    # -- global registration --------------------------------------------
    @staticmethod
    def rotation_grid(grid_kind: int = 0, num_guess: int = 0) -> np.ndarray:
        lib = L.lib()
        n = lib.cvo_rotation_grid(grid_kind, num_guess, None, 0)
        L.check(n, "cvo_rotation_grid")
        out = np.zeros(9 * n, np.float32)
        lib.cvo_rotation_grid(grid_kind, num_guess, out.ctypes.data_as(_FP), n)
        return out.reshape(n, 3, 3)

    def get_nearest_init_pose(self, source, target, init_guess_ell: float, num_guess: int = 0, grid_kind: int = 0):
        """CvoGPU::get_nearest_init_pose (src/cvo/CvoGPU.cpp:367-398); returns (T, seconds)."""
        T_out = np.zeros(16, np.float32)
        secs = C.c_double(0)
        lib = L.lib()
        if isinstance(source, GpuCloud):
            rc = lib.cvo_get_nearest_init_pose_dev(self._h, source.handle, target.handle, float(init_guess_ell),
                                                   int(num_guess), int(grid_kind), T_out.ctypes.data_as(_FP),
                                                   C.byref(secs))
        else:
            s, t = source.c_struct(), target.c_struct()
            rc = lib.cvo_get_nearest_init_pose(self._h, C.byref(s), C.byref(t), float(init_guess_ell), int(num_guess),
                                               int(grid_kind), T_out.ctypes.data_as(_FP), C.byref(secs))
        L.check(rc, "cvo_get_nearest_init_pose", self._h)
        return _from16(T_out), secs.value

    def register_hypotheses(self, source: GpuCloud, target: GpuCloud, T_inits, judge_ell: float):
        """Refine every hypothesis with the batched align and keep the best final cos-angle.
        Returns (T_out, best_index, cos_values, seconds)."""
        n = len(T_inits)
        Ti = np.ascontiguousarray(np.concatenate([_m16(T) for T in T_inits]).astype(np.float32))
        To = np.zeros(16, np.float32)
        best = C.c_int(-1)
        cos = np.zeros(n, np.float32)
        secs = C.c_double(0)
        L.check(L.lib().cvo_register_hypotheses_dev(self._h, source.handle, target.handle, n, Ti.ctypes.data_as(_FP),
                                                    float(judge_ell), To.ctypes.data_as(_FP), C.byref(best),
                                                    cos.ctypes.data_as(_FP), C.byref(secs)),
                "cvo_register_hypotheses_dev", self._h)
        return _from16(To), best.value, cos, secs.value

    def register_learned_batch(self, net, sources, targets, n_refine: int = 2, rank_ell: float | None = None,
                               judge_ell: float | None = None, fallback_cos: float = 0.0, seed: int = 0,
                               refine_ell: float = 0.0):
        """Global registration of many pairs from the proposal network's hypotheses
        (ranked, best n_refine refined in one batch, judged by the final cos-angle,
        24-rotation grid fallback below fallback_cos; refine_ell > 0 starts the refinement
        at that lengthscale).  Returns (T_out list of 4x4 in
        align's output convention, cos (B,), used_fallback (B,), iters (B,), seconds)."""
        p = self.get_params()
        rank_ell = p.ell_init_first_frame if rank_ell is None else rank_ell
        judge_ell = p.ell_init_first_frame if judge_ell is None else judge_ell
        n = len(sources)
        S = (C.c_void_p * n)(*[s.handle.value for s in sources])
        Tg = (C.c_void_p * n)(*[t.handle.value for t in targets])
        To = np.zeros(16 * n, np.float32)
        cos = np.zeros(n, np.float32)
        fb = np.zeros(n, np.int32)
        its = np.zeros(n, np.int32)
        secs = C.c_double(0)
        L.check(L.lib().cvo_register_learned_batch_dev(self._h, net.handle, n, S, Tg, int(n_refine), float(rank_ell),
                                                       float(judge_ell), float(fallback_cos), float(refine_ell),
                                                       C.c_uint32(seed & 0xFFFFFFFF), To.ctypes.data_as(_FP),
                                                       cos.ctypes.data_as(_FP),
                                                       fb.ctypes.data_as(C.POINTER(C.c_int)),
                                                       its.ctypes.data_as(C.POINTER(C.c_int)), C.byref(secs)),
                "cvo_register_learned_batch_dev", self._h)
        return [_from16(To[16 * i:16 * i + 16]) for i in range(n)], cos, fb, its, secs.value

    def global_register(self, sources, targets, net=None):
        """cvo_global_register: host pairs in, poses out in one call.  Without net the
        plain grid (nearest of the 24 cube rotations, then one batched align); with net
        the learned proposal (register_learned_batch's defaults).  Returns (list of 4x4
        in align's output convention, iterations (n,), seconds)."""
        n = len(sources)
        if len(targets) != n:
            raise ValueError("one target per source")
        cs = (L.CvoCloudC * max(n, 1))(*[c.c_struct() for c in sources])
        ct = (L.CvoCloudC * max(n, 1))(*[c.c_struct() for c in targets])
        To = np.zeros(16 * max(n, 1), np.float32)
        its = np.zeros(max(n, 1), np.int32)
        secs = C.c_double(0)
        L.check(L.lib().cvo_global_register(self._h, n, cs, ct, 0 if net is None else 1,
                                            None if net is None else net.handle, To.ctypes.data_as(_FP),
                                            its.ctypes.data_as(C.POINTER(C.c_int)), C.byref(secs)),
                "cvo_global_register", self._h)
        return [_from16(To[16 * i:16 * i + 16]) for i in range(n)], its[:n], secs.value

    # -- autotuner -----------------------------------------------------
    def autotune(self, source: GpuCloud, target: GpuCloud, T=None, ell: float = 0.0, reps: int = 3) -> dict:
        """Times the association's cell-size configurations on one pair, then the best one
        with 1-3 resident blocks per SM, and keeps the fastest for later batches of the same
        (F, C, size) key.  Returns {"configs": [(div_r, div_ext, blocks_per_sm, ms), ...],
        "best": index}; blocks_per_sm 0 = as many as the occupancy allows."""
        Ti = _m16(np.eye(4) if T is None else T)
        n = C.c_int()
        dr, de, ms = np.zeros(32, np.float32), np.zeros(32, np.float32), np.zeros(32, np.float32)
        bp = np.zeros(32, np.int32)
        best = C.c_int()
        L.check(L.lib().cvo_autotune_launch_dev(self._h, source.handle, target.handle, Ti.ctypes.data_as(_FP),
                                                float(ell), int(reps), 32, C.byref(n), dr.ctypes.data_as(_FP),
                                                de.ctypes.data_as(_FP), bp.ctypes.data_as(C.POINTER(C.c_int)),
                                                ms.ctypes.data_as(_FP), C.byref(best)),
                "cvo_autotune_launch_dev", self._h)
        return {"configs": [(float(dr[k]), float(de[k]), int(bp[k]), float(ms[k])) for k in range(n.value)],
                "best": best.value}

    def tune_set(self, F: int, Cn: int, rows: int, div_r: float, div_ext: float) -> None:
        L.check(L.lib().cvo_tune_set(self._h, F, Cn, rows, float(div_r), float(div_ext)), "cvo_tune_set", self._h)

    def tune_get(self, F: int, Cn: int, rows: int):
        """(div_r, div_ext, tuned?) for a key."""
        a, b = C.c_float(), C.c_float()
        rc = L.lib().cvo_tune_get(self._h, F, Cn, rows, C.byref(a), C.byref(b))
        return a.value, b.value, rc == 0

    def tune_set_launch(self, F: int, Cn: int, rows: int, div_r: float, div_ext: float, blocks_per_sm: int) -> None:
        L.check(L.lib().cvo_tune_set_launch(self._h, F, Cn, rows, float(div_r), float(div_ext), int(blocks_per_sm)),
                "cvo_tune_set_launch", self._h)

    def tune_get_launch(self, F: int, Cn: int, rows: int):
        """(div_r, div_ext, blocks_per_sm, tuned?) for a key."""
        a, b, c = C.c_float(), C.c_float(), C.c_int()
        rc = L.lib().cvo_tune_get_launch(self._h, F, Cn, rows, C.byref(a), C.byref(b), C.byref(c))
        return a.value, b.value, c.value, rc == 0

    # -- multi-frame ----------------------------------------------------
    def align_multi(self, clouds, poses, hold_const, edges):
        """CvoGPU::align(frames, frames_to_hold_const, edges, secs) (src/cvo/CvoGPU.cu:1615-1670).
        poses: (n, 12) row-major 3x4 frame->world (updated copy returned)."""
        n = len(clouds)
        P = np.ascontiguousarray(np.asarray(poses, np.float64).reshape(n, 12).copy())
        hc = np.ascontiguousarray(np.asarray(hold_const, np.uint8).reshape(n))
        E = np.ascontiguousarray(np.asarray(edges, np.int32).reshape(-1, 2))
        secs = C.c_double(0)
        iters = C.c_int(0)
        lib = L.lib()
        if isinstance(clouds[0], GpuCloud):
            arr = (C.c_void_p * n)(*[c.handle.value for c in clouds])
            rc = lib.cvo_align_multi_dev(self._h, n, arr, P.ctypes.data_as(C.POINTER(C.c_double)),
                                         hc.ctypes.data_as(C.POINTER(C.c_uint8)), E.shape[0],
                                         E.ctypes.data_as(C.POINTER(C.c_int)), C.byref(secs), C.byref(iters))
        else:
            cs = (L.CvoCloudC * n)(*[c.c_struct() for c in clouds])
            rc = lib.cvo_align_multi(self._h, n, cs, P.ctypes.data_as(C.POINTER(C.c_double)),
                                     hc.ctypes.data_as(C.POINTER(C.c_uint8)), E.shape[0],
                                     E.ctypes.data_as(C.POINTER(C.c_int)), C.byref(secs), C.byref(iters))
        L.check(rc, "cvo_align_multi", self._h)
        return P, secs.value, iters.value


class AdaptiveCvoGPU(CvoGPU):
    """cvo::AdaptiveCvoGPU (include/UnifiedCvo/cvo/AdaptiveCvoGPU.hpp:161-180): CVO whose
    lengthscale follows the gradient of the inner product (src/cvo/AdaptiveCvoGPU.cu)."""

    def align(self, source, target, T_init, trace_len: int = 0):
        """int AdaptiveCvoGPU::align(src, tgt, init_guess_transform, transform&, secs*)
        (:1077-1250).  Returns (ret, T_out, seconds, iters) and, with trace_len > 0, a
        (iters, 6) trace {ell, dl, step, nnz A, nnz Axx, nnz Ayy} as a fifth value."""
        T_out = np.zeros(16, np.float32)
        secs = C.c_double(0)
        iters = C.c_int(0)
        Ti = _m16(T_init)
        lib = L.lib()
        tr = np.zeros((max(trace_len, 0), 6)) if trace_len > 0 else None
        if isinstance(source, GpuCloud):
            rc = lib.cvo_align_adaptive_dev(self._h, source.handle, target.handle, Ti.ctypes.data_as(_FP),
                                            T_out.ctypes.data_as(_FP), C.byref(secs), C.byref(iters),
                                            tr.ctypes.data_as(C.POINTER(C.c_double)) if tr is not None else None,
                                            int(max(trace_len, 0)))
        else:
            if tr is not None:
                raise ValueError("a trace needs device clouds (upload them first)")
            s, t = source.c_struct(), target.c_struct()
            rc = lib.cvo_align_adaptive(self._h, C.byref(s), C.byref(t), Ti.ctypes.data_as(_FP),
                                        T_out.ctypes.data_as(_FP), C.byref(secs), C.byref(iters))
        L.check(rc, "cvo_align_adaptive", self._h)
        out = ((0 if rc == L.CVO_OK else -1), _from16(T_out), secs.value, iters.value)
        if tr is not None:
            return out + (tr[:min(trace_len, iters.value + 1)],)
        return out

    def compute_association_gpu(self, source, target, T, ell) -> Association:
        """The adaptive path's kernel matrix A at pose T and lengthscale ell
        (se_kernel -> fill_in_A_mat_gpu, src/cvo/AdaptiveCvoGPU.cu:263-443)."""
        ab = _AssocBuf()
        s, t = source.c_struct(), target.c_struct()
        L.check(L.lib().cvo_compute_association_adaptive(self._h, C.byref(s), C.byref(t), _m16(T).ctypes.data_as(_FP),
                                                         float(ell), ab.h),
                "cvo_compute_association_adaptive", self._h)
        return _read_assoc(ab.h)
