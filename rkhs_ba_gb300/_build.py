"""Builds the native library ``_lib/libcvo_gb300.so`` in-tree with nvcc (sm_103a).

Each CUDA translation unit is compiled in parallel, then linked into one shared
library exporting the C ABI declared in ``include/cvo_gb300.h``.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG_DIR)
CSRC = os.path.join(PKG_DIR, "csrc")
LIB_DIR = os.path.join(PKG_DIR, "_lib")
LIB_PATH = os.path.join(LIB_DIR, "libcvo_gb300.so")
OBJ_DIR = os.path.join(ROOT, "_build", "obj")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-lineinfo", "-O3", "-std=c++17",
                     "-Xcompiler", "-fPIC,-fopenmp,-ffp-contract=off,-O2",
                     "-I" + os.path.join(ROOT, "include")]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build rkhs_ba_gb300")


def _sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _digest() -> str:
    """Hash of what the library is compiled from: the CUDA sources and the C headers
    (the header-only C++ mirror, include/*.hpp, is not part of the library)."""
    h = hashlib.sha256()
    for d in (CSRC, os.path.join(ROOT, "include")):
        for f in sorted(os.listdir(d)):
            p = os.path.join(d, f)
            if os.path.isfile(p) and not f.endswith(".hpp"):
                h.update(f.encode())
                with open(p, "rb") as fh:
                    h.update(fh.read())
    h.update(" ".join(NVCC_FLAGS).encode())
    return h.hexdigest()


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile and link the library if its sources changed; returns its path."""
    os.makedirs(LIB_DIR, exist_ok=True)
    os.makedirs(OBJ_DIR, exist_ok=True)
    stamp = os.path.join(LIB_DIR, ".build_digest")
    digest = _digest()
    if not force and os.path.exists(LIB_PATH) and os.path.exists(stamp):
        with open(stamp) as fh:
            if fh.read().strip() == digest:
                return LIB_PATH
    nvcc = _nvcc()
    srcs = _sources()

    def compile_one(src: str) -> str:
        obj = os.path.join(OBJ_DIR, os.path.basename(src)[:-3] + ".o")
        cmd = [nvcc] + NVCC_FLAGS + ["-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB_PATH + ".tmp"
    cmd = [nvcc, "-shared", "-Xcompiler", "-fopenmp"] + ARCH + ["-o", tmp] + objs + ["-ldl"]   # NVTX3 loads its tool
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB_PATH)
    with open(stamp, "w") as fh:
        fh.write(digest)
    return LIB_PATH


SAN_DIR = os.path.join(ROOT, "_build", "asan")
SAN_LIB_PATH = os.path.join(SAN_DIR, "libcvo_gb300.so")
SAN_FLAGS = ["-Xcompiler", "-fsanitize=address", "-Xcompiler", "-fsanitize=undefined",
             "-Xcompiler", "-fno-sanitize-recover=undefined", "-Xcompiler", "-fno-omit-frame-pointer"]


def sanitizer_preload() -> str:
    """LD_PRELOAD value with gcc's AddressSanitizer and UBSan runtimes (a sanitized
    shared library loaded into an unsanitized Python needs them first)."""
    libs = []
    for name in ("libasan.so", "libubsan.so"):
        r = subprocess.run(["gcc", "-print-file-name=" + name], capture_output=True, text=True, check=True)
        libs.append(r.stdout.strip())
    return " ".join(libs)


def build_sanitized() -> str:
    """The same library with its HOST code (parameter reader, CPU inner product, pose-graph
    solver, argument checks) under AddressSanitizer and UndefinedBehaviorSanitizer, in
    _build/asan/; device code is compiled as usual.  For checks of the host paths without
    a GPU; load it with sanitizer_preload() in LD_PRELOAD."""
    obj_dir = os.path.join(SAN_DIR, "obj")
    os.makedirs(obj_dir, exist_ok=True)
    nvcc = _nvcc()
    flags = ARCH + ["-O1", "-g", "-std=c++17", "-Xcompiler", "-fPIC,-fopenmp,-ffp-contract=off"] + SAN_FLAGS + \
        ["-I" + os.path.join(ROOT, "include")]

    def compile_one(src: str) -> str:
        obj = os.path.join(obj_dir, os.path.basename(src)[:-3] + ".o")
        r = subprocess.run([nvcc] + flags + ["-c", src, "-o", obj], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
        return obj

    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(compile_one, srcs))
    cmd = [nvcc, "-shared", "-Xcompiler", "-fopenmp"] + SAN_FLAGS[:4] + ARCH + ["-o", SAN_LIB_PATH] + objs + ["-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    return SAN_LIB_PATH


if __name__ == "__main__":
    print(build(verbose=True))
