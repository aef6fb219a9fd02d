"""The oracle's own CvoParams: defaults and yaml reader, independent of the product.

TEST INFRASTRUCTURE ONLY.  The product reads parameter files with its own C++
reader (cvo_params_read_yaml in the native library); the oracle must not share
it, or a parser bug would reach both sides of every parity test unseen.  This
module restates, in plain Python:

* the constructor defaults of cvo::CvoParams
  (include/UnifiedCvo/cvo/CvoParams.hpp:80-136), plus max_step = 0.8, which the
  reference constructor leaves uninitialised (the value of its geometric yaml);
* read_CvoParams_yaml (include/UnifiedCvo/cvo/CvoParams.hpp:203-323): a field is
  set only when its key is present; keys the reference does not read are
  ignored; the key multiframe_iterations_per_ell sets that field (the reference
  never reads multiframe_iter_per_ell from a file).

The values are packed into a ctypes structure with the field order of
``cvo_params`` in include/cvo_gb300.h, which the C oracle reads.
"""
from __future__ import annotations

import ctypes as C

_f, _i, _d = C.c_float, C.c_int, C.c_double

# (field, ctype, default) in the order of struct cvo_params (include/cvo_gb300.h);
# defaults from CvoParams::CvoParams() (CvoParams.hpp:80-136)
FIELDS = [
    ("ell_init_first_frame", _f, 0.5), ("ell_init", _f, 0.5), ("ell_min", _f, 0.05),
    ("min_ell_iter_limit", _i, 1), ("ell_max", _f, 1.2), ("dl", _d, 0.0), ("dl_step", _d, 0.3),
    ("sigma", _f, 0.1), ("sp_thres", _f, 0.0006), ("c", _f, 7.0), ("d", _f, 7.0), ("c_ell", _f, 0.15),
    ("c_sigma", _f, 0.6), ("s_ell", _f, 0.1), ("s_sigma", _f, 0.8), ("MAX_ITER", _i, 10000),
    ("eps", _f, 0.00005), ("eps_2", _f, 0.000012), ("min_step", _f, 2e-5), ("max_step", _f, 0.8),
    ("step", _f, 0.0), ("nearest_neighbors_max", _i, 512), ("ell_decay_rate", _f, 0.9),
    ("ell_decay_rate_first_frame", _f, 0.99), ("ell_decay_start", _i, 30),
    ("ell_decay_start_first_frame", _i, 300), ("indicator_window_size", _i, 15),
    ("indicator_stable_threshold", _f, 0.2), ("is_pcl_visualization_on", _i, 0),
    ("is_using_least_square", _i, 0), ("is_ell_adaptive", _i, 0), ("is_full_ip_matrix", _i, 0),
    ("is_using_geometry", _i, 1), ("is_using_intensity", _i, 0), ("is_using_semantics", _i, 0),
    ("is_using_range_ell", _i, 0), ("is_using_kdtree", _i, 0), ("is_exporting_association", _i, 0),
    ("is_using_geometric_type", _i, 0), ("is_global_angle_registration", _i, 0),
    ("multiframe_using_cpu", _i, 1), ("multiframe_max_iters", _i, 200), ("multiframe_ell_init", _f, 0.15),
    ("multiframe_ell_min", _f, 0.05), ("multiframe_ell_max", _f, 5.0), ("multiframe_iter_per_ell", _i, 10),
    ("multiframe_ell_decay_rate", _f, 0.7), ("multiframe_iterations_per_ell", _i, 50),
    ("multiframe_iterations_per_solve", _i, 8), ("multiframe_expected_points", _i, 1000),
    ("multiframe_downsample_voxel_size", _f, 0.5), ("multiframe_num_neighbors", _i, 128),
    ("multiframe_least_squares_num_threads", _i, 24), ("multiframe_min_nonzeros", _i, 300),
    ("multiframe_is_optimizing_ell", _i, 0), ("multiframe_is_sorting_inner_product", _i, 0),
    ("multiframe_is_free_memory_each_iter", _i, 0),
]

# Keys read_CvoParams_yaml looks up (CvoParams.hpp:206-318): every field above except
# step, is_ell_adaptive and multiframe_iter_per_ell, which no file sets.
YAML_KEYS = [f for f, _, _ in FIELDS if f not in ("step", "is_ell_adaptive", "multiframe_iter_per_ell")]


class ParamsC(C.Structure):
    _fields_ = [(f, t) for f, t, _ in FIELDS]


class YamlError(ValueError):
    pass


def _scalar(text: str) -> str:
    """The scalar of a `key: value` line: comment and surrounding quotes removed."""
    v = text.split("#", 1)[0].strip()
    if len(v) >= 2 and v[0] in "\"'" and v[-1] == v[0]:
        v = v[1:-1]
    return v


def _as_int(v: str) -> int:
    try:
        return int(v, 10)
    except ValueError:
        raise YamlError("not an integer: %r" % v) from None


def _as_float(v: str) -> float:
    try:
        return float(v)
    except ValueError:
        raise YamlError("not a number: %r" % v) from None


def read_yaml_dict(path: str) -> dict:
    """The keys read_CvoParams_yaml would set from the file, converted to the field's
    type (ints in base 10, floats and doubles as numbers); later lines win."""
    types = {f: t for f, t, _ in FIELDS}
    out = {}
    with open(path) as fh:
        for raw in fh:
            line = raw.split("#", 1)[0].strip()
            if not line or line.startswith("%") or line in ("---", "..."):
                continue
            if ":" not in line:
                continue
            key, val = line.split(":", 1)
            key = key.strip()
            if key not in YAML_KEYS:
                continue
            v = _scalar(val)
            out[key] = _as_int(v) if types[key] is _i else _as_float(v)
    return out


class OracleParams:
    """cvo::CvoParams for the oracle: attribute access like the product's CvoParams,
    values held in a ctypes structure the C oracle reads."""

    def __init__(self, yaml_path: str | None = None):
        object.__setattr__(self, "_c", ParamsC())
        for f, _, dv in FIELDS:
            setattr(self._c, f, dv)
        if yaml_path is not None:
            for k, v in read_yaml_dict(yaml_path).items():
                setattr(self._c, k, v)

    def __getattr__(self, k):
        if k.startswith("_"):
            raise AttributeError(k)
        return getattr(self._c, k)

    def __setattr__(self, k, v):
        if not any(k == f for f, _, _ in FIELDS):
            raise AttributeError("unknown CvoParams field %r" % k)
        setattr(self._c, k, v)

    def as_dict(self) -> dict:
        return {f: getattr(self._c, f) for f, _, _ in FIELDS}

    def copy(self) -> "OracleParams":
        p = OracleParams()
        C.memmove(C.byref(p._c), C.byref(self._c), C.sizeof(ParamsC))
        return p
