"""Host code under AddressSanitizer and UndefinedBehaviorSanitizer, without a GPU.

Opt-in (about two minutes of nvcc): RKHS_SANITIZE=1 python -m pytest tests/test_host_sanitizers.py

Builds the oracle (oracle.build_sanitized) and the library's host code
(rkhs_ba_gb300._build.build_sanitized) with both sanitizers, then runs the CPU suites
that exercise them in a child process with the sanitizer runtimes preloaded:

* the oracle's known-answer, restatement and edge-case tests;
* the C ABI's host paths: parameter files, the CPU inner product, empty clouds, every
  entry point with NULL arguments, the FP64 pose-graph solver and the keyframe flow.

Any sanitizer report ends the child with a non-zero status.
"""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

pytestmark = pytest.mark.skipif(os.environ.get("RKHS_SANITIZE") != "1", reason="opt-in: RKHS_SANITIZE=1")

_CHILD = r"""
import ctypes as C, sys
root, olib, llib = sys.argv[1:4]
sys.path.insert(0, root)
import oracle.oracle as o
import rkhs_ba_gb300._lib as L
o.LIB = olib
o.build = lambda force=False: olib
L.LIB_PATH = llib
import pytest
rc = pytest.main(["-q", "-x", "-p", "no:cacheprovider", "-m", "not gpu",
                  root + "/tests/test_oracle.py", root + "/tests/test_adaptive_oracle.py",
                  root + "/tests/test_cloud_edges.py", root + "/tests/test_abi.py",
                  root + "/tests/test_posegraph.py", root + "/tests/test_posegraph_flow.py"])
assert o._L._name == olib and L._LIB._name == llib
lib = L.lib()
for name, (res, args) in L.SIGNATURES.items():     # NULL arguments in this process too
    getattr(lib, name)(*[0 if a in (C.c_int, C.c_int64, C.c_uint32, C.c_float, C.c_double) else None for a in args])
sys.exit(rc)
"""


def test_host_code_under_sanitizers():
    sys.path.insert(0, ROOT)
    from oracle import oracle as orc
    from rkhs_ba_gb300 import _build
    olib = orc.build_sanitized()
    llib = _build.build_sanitized()
    env = dict(os.environ)
    env["LD_PRELOAD"] = _build.sanitizer_preload()
    env["ASAN_OPTIONS"] = "detect_leaks=0:halt_on_error=1:protect_shadow_gap=0"
    env["UBSAN_OPTIONS"] = "halt_on_error=1:print_stacktrace=1"
    r = subprocess.run([sys.executable, "-c", _CHILD, ROOT, olib, llib], env=env, capture_output=True, text=True,
                       timeout=3600)
    assert r.returncode == 0, (r.stdout[-3000:], r.stderr[-3000:])
