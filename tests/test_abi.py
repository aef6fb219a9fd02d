"""The C-ABI library loads, exports every symbol of include/cvo_gb300.h, and its
structures have the layout the header declares (no GPU needed)."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import numpy as np
import pytest

from rkhs_ba_gb300 import CvoGPU, CvoParams, CvoPointCloud, params_path
from rkhs_ba_gb300 import _lib as L

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "cvo_gb300.h")


def _declared():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(cvo_[a-z0-9_]+)\s*\(", txt)))


def test_every_declared_symbol_is_exported_and_bound():
    lib = L.lib()
    names = _declared()
    assert len(names) >= 30
    for n in names:
        assert hasattr(lib, n), n
        assert n in L.SIGNATURES, "no ctypes binding for %s" % n


def test_struct_layout_matches_header():
    """Compile a probe with gcc that prints sizeof/offsetof of the header's structs."""
    fields = [f for f, _ in L.PARAM_FIELDS]
    src = ['#include <stdio.h>', '#include <stddef.h>', '#include "cvo_gb300.h"', 'int main(void){',
           'printf("%zu %zu\\n", sizeof(cvo_params), sizeof(cvo_cloud));']
    for f in fields:
        src.append('printf("%%zu\\n", offsetof(cvo_params, %s));' % f)
    for f in ("n", "F", "C", "xyz_stride", "xyz", "features", "labels", "geom_type"):
        src.append('printf("%%zu\\n", offsetof(cvo_cloud, %s));' % f)
    src.append("return 0;}")
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "probe.c")
        open(c, "w").write("\n".join(src))
        exe = os.path.join(d, "probe")
        subprocess.run(["gcc", "-I" + os.path.dirname(HEADER), c, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()
    vals = [int(v) for v in out]
    assert vals[0] == C.sizeof(L.CvoParamsC)
    assert vals[1] == C.sizeof(L.CvoCloudC)
    for k, f in enumerate(fields):
        assert vals[2 + k] == getattr(L.CvoParamsC, f).offset, f
    for k, f in enumerate(("n", "F", "C", "xyz_stride", "xyz", "features", "labels", "geom_type")):
        assert vals[2 + len(fields) + k] == getattr(L.CvoCloudC, f).offset, f


def test_defaults_follow_reference_constructor():
    p = CvoParams()
    # CvoParams::CvoParams() (include/UnifiedCvo/cvo/CvoParams.hpp:80-136)
    assert p.ell_init == pytest.approx(0.5)
    assert p.sp_thres == pytest.approx(0.0006)
    assert p.MAX_ITER == 10000
    assert p.nearest_neighbors_max == 512
    assert p.indicator_window_size == 15
    assert p.is_using_geometry == 1 and p.is_using_intensity == 0
    assert p.multiframe_iter_per_ell == 10


def test_yaml_reader_sets_only_present_keys(tmp_path):
    y = tmp_path / "p.yaml"
    y.write_text("%YAML:1.0\n---\nell_init: 0.7 # comment\nMAX_ITER: 12\nis_ell_adaptive: False\n"
                 "multiframe_iterations_per_ell: 33\nunknown_key: 5\n")
    p = CvoParams(str(y))
    assert p.ell_init == pytest.approx(0.7)
    assert p.MAX_ITER == 12
    assert p.sigma == pytest.approx(0.1)          # untouched default
    assert p.multiframe_iterations_per_ell == 33  # the reference reads this key ...
    assert p.multiframe_iter_per_ell == 10        # ... and never sets this field


def test_yaml_reader_rejects_bad_values(tmp_path):
    y = tmp_path / "bad.yaml"
    y.write_text("MAX_ITER: 1.5\n")
    with pytest.raises(L.CvoError) as e:
        CvoParams(str(y))
    assert e.value.code == L.CVO_ERR_BAD_YAML
    with pytest.raises(L.CvoError) as e:
        CvoParams(str(tmp_path / "missing.yaml"))
    assert e.value.code == L.CVO_ERR_IO


def test_bundled_param_files_parse():
    for name in ("geometric", "color", "lidar_semantic", "irls"):
        p = CvoParams(params_path(name))
        assert p.MAX_ITER > 0
    assert CvoParams(params_path("color")).nearest_neighbors_max == 256


def test_status_strings():
    lib = L.lib()
    assert lib.cvo_status_string(0) == b"ok"
    assert lib.cvo_status_string(L.CVO_ERR_BAD_YAML) == b"bad yaml parameter file"


def test_handle_without_gpu_host_paths_work():
    """Host entry points work on a handle; GPU entry points fail loudly when no GPU exists."""
    cvo = CvoGPU(params=CvoParams())
    a = CvoPointCloud(np.random.default_rng(0).uniform(0, 1, (50, 3)))
    v = cvo.inner_product_cpu(a, a, np.eye(4), 0.1)
    assert v > 0
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if not has_gpu:
        with pytest.raises(L.CvoError) as e:
            cvo.inner_product_gpu(a, a, np.eye(4), 0.1)
        assert e.value.code == L.CVO_ERR_CUDA


def test_empty_clouds_follow_reference_returns():
    cvo = CvoGPU(params=CvoParams())
    e = CvoPointCloud(np.zeros((0, 3)))
    a = CvoPointCloud(np.ones((5, 3)))
    # CvoGPU::align returns 0 on empty input, function_angle returns 0 (CvoGPU.cu:1492-1495,1773-1775)
    ret, T, _, _, iters = cvo.align(e, a, np.eye(4))
    assert ret == 0 and iters == 0
    assert cvo.function_angle(e, a, np.eye(4), 0.1) == 0.0
    assert cvo.inner_product_cpu(a, e, np.eye(4), 0.1) == 0.0
    r = cvo.align_s2t(e, a, np.eye(4))
    assert r.return_code == -1


_NULL_OK = {                                  # defined results for NULL / zero arguments
    "cvo_params_default": None,               # void; ignores NULL
    "cvo_cloud_size": 0,
    "cvo_assoc_destroy": 0, "cvo_pose_graph_destroy": 0, "cvo_proposal_destroy": 0,   # free(NULL)
    "cvo_rotation_grid": 60,                  # count query of the icosahedral grid
    "cvo_proposal_dims": 0,                   # p may be NULL: the fixed dimensions
    "cvo_status_string": b"ok", "cvo_kernel_launch_count": 0, "cvo_last_error": b"", "cvo_get_stream": None,
}

_NULL_CHILD = r"""
import ctypes as C, json, sys
sys.path.insert(0, sys.argv[1])
from rkhs_ba_gb300 import _lib as L
lib = L.lib()
out = {}
for name, (res, args) in L.SIGNATURES.items():
    vals = [0 if a in (C.c_int, C.c_int64, C.c_uint32, C.c_float, C.c_double) else None for a in args]
    r = getattr(lib, name)(*vals)
    out[name] = r.decode() if isinstance(r, bytes) else r
print(json.dumps(out))
"""


def test_every_entry_point_rejects_null_arguments():
    """All entry points called with NULL pointers and zero sizes (no GPU work is reached):
    each returns CVO_ERR_INVALID_ARG, except the calls whose NULL behaviour is defined."""
    import json
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", _NULL_CHILD, root], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    got = json.loads(r.stdout.strip().splitlines()[-1])
    assert set(got) == set(L.SIGNATURES)
    for name, v in got.items():
        if name in _NULL_OK:
            want = _NULL_OK[name]
            assert v == (want.decode() if isinstance(want, bytes) else want), (name, v)
        else:
            assert v == L.CVO_ERR_INVALID_ARG, (name, v)


_C_CLIENT = r"""
#include <math.h>
#include <stdio.h>
#include "cvo_gb300.h"

int main(void) {
  cvo_params p;
  cvo_params_default(&p);
  cvo_handle *h = NULL;
  if (cvo_create_with_params(&p, &h) != CVO_OK) return 1;
  float xyz[3 * 4] = {0, 0, 0, 0.1f, 0, 0, 0, 0.1f, 0, 0, 0, 0.1f};
  cvo_cloud c = {4, 0, 0, 3, xyz, NULL, NULL, NULL};
  float T[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
  float ip = 0.f;
  if (cvo_inner_product_cpu(h, &c, &c, T, 0.1f, &ip) != CVO_OK || !(ip > 0.f)) return 2;
  cvo_pose_graph *g = NULL;
  double I[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0}, Z[12] = {1, 0, 0, 1, 0, 1, 0, 0, 0, 0, 1, 0};
  double sig[6] = {0.1, 0.1, 0.1, 0.1, 0.1, 0.1}, c0, c1, X[12];
  int it;
  if (cvo_pose_graph_create(&g) || cvo_pose_graph_insert(g, 0, I) || cvo_pose_graph_insert(g, 1, I) ||
      cvo_pose_graph_add_prior(g, 0, I, sig) || cvo_pose_graph_add_between(g, 0, 1, Z, sig) ||
      cvo_pose_graph_optimize(g, 50, &c0, &c1, &it) || cvo_pose_graph_get(g, 1, X)) return 3;
  if (fabs(X[3] - 1.0) > 1e-9 || c1 > 1e-16) return 4;
  cvo_pose_graph_destroy(g);
  if (cvo_inner_product_cpu(NULL, &c, &c, T, 0.1f, &ip) != CVO_ERR_INVALID_ARG) return 5;
  printf("%s %.6g\n", cvo_status_string(CVO_OK), (double)ip);
  cvo_destroy(h);
  return 0;
}
"""


def test_plain_c_client_links_and_runs():
    """A C99 program built against the header (-Wall -Wextra -Werror) links the library
    and runs its host paths; the header also compiles as C++."""
    lib_dir = os.path.dirname(L.LIB_PATH)
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "client.c")
        open(src, "w").write(_C_CLIENT)
        exe = os.path.join(d, "client")
        subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-I" + os.path.dirname(HEADER), src, "-o",
                        exe, "-L" + lib_dir, "-lcvo_gb300", "-Wl,-rpath," + lib_dir, "-lm"], check=True)
        out = subprocess.run([exe], capture_output=True, text=True)
        assert out.returncode == 0, (out.returncode, out.stderr[-2000:])
        assert out.stdout.startswith("ok ")
        cpp = os.path.join(d, "client.cpp")
        open(cpp, "w").write('#include "cvo_gb300.h"\nint main() { return cvo_status_string(0) ? 0 : 1; }\n')
        subprocess.run(["g++", "-std=c++11", "-Wall", "-Wextra", "-Werror", "-I" + os.path.dirname(HEADER), cpp, "-o",
                        exe + "_cpp", "-L" + lib_dir, "-lcvo_gb300", "-Wl,-rpath," + lib_dir], check=True)
        assert subprocess.run([exe + "_cpp"]).returncode == 0


_OOM_CHILD = r"""
import resource, sys
sys.path.insert(0, sys.argv[1])
from rkhs_ba_gb300 import _lib as L
lib = L.lib()
assert lib.cvo_rotation_grid(2, 3, None, 0) == 27
vm_kb = [int(l.split()[1]) for l in open("/proc/self/status") if l.startswith("VmSize:")][0]
soft, hard = resource.getrlimit(resource.RLIMIT_AS)
resource.setrlimit(resource.RLIMIT_AS, (vm_kb * 1024 + (256 << 20), hard))
print(lib.cvo_rotation_grid(2, 300, None, 0))      # 27 M rotations, about 1 GB: cannot fit
"""


def test_host_allocation_failure_returns_a_status():
    """A host allocation that fails inside an entry point (address space capped in a
    child process) returns CVO_ERR_OUT_OF_MEMORY instead of ending the process."""
    import sys
    env = {k: v for k, v in os.environ.items() if k != "LD_PRELOAD"}   # a sanitizer runtime cannot map its shadow
    r = subprocess.run([sys.executable, "-c", _OOM_CHILD, ROOT], capture_output=True, text=True, timeout=300, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    assert int(r.stdout.strip().splitlines()[-1]) == L.CVO_ERR_OUT_OF_MEMORY


def test_global_register_host_checks():
    """cvo_global_register: argument checks and the no-GPU status, on the host."""
    cvo = CvoGPU(params=CvoParams())
    a = CvoPointCloud(np.random.default_rng(1).uniform(-1, 1, (60, 3)))
    T = np.zeros(16, np.float32)
    lib = L.lib()
    S = (L.CvoCloudC * 1)(a.c_struct())
    assert lib.cvo_global_register(cvo._h, 0, None, None, 0, None, None, None, None) == L.CVO_OK
    assert lib.cvo_global_register(cvo._h, 1, S, S, 1, None, T.ctypes.data_as(C.POINTER(C.c_float)), None,
                                   None) == L.CVO_ERR_INVALID_ARG          # learned without a proposal
    assert lib.cvo_global_register(cvo._h, -1, S, S, 0, None, T.ctypes.data_as(C.POINTER(C.c_float)), None,
                                   None) == L.CVO_ERR_INVALID_ARG
    with pytest.raises(ValueError):
        cvo.global_register([a], [])
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if not has_gpu:
        with pytest.raises(L.CvoError) as e:
            cvo.global_register([a], [a])
        assert e.value.code == L.CVO_ERR_CUDA
