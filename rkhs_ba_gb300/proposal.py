"""Learned pose proposal for global registration (C ABI ``cvo_proposal_*``).

The reference initialises a global registration from a fixed rotation grid
(get_nearest_init_pose, src/cvo/CvoGPU.cpp:367-398).  ``ProposalNet`` is a small
point-set network that proposes K = 8 poses per pair instead; ``train`` fits it on
the device from a pool of synthetic view pairs moved by random SE(3) labels, and
``CvoGPU.register_learned_batch`` refines its hypotheses with the batched align and
keeps the grid as the fallback.  Every forward and backward product runs in the
native library's BF16 tensor-core kernels; this module only moves arrays.
"""
from __future__ import annotations

import ctypes as C
import os
import time

import numpy as np

from . import _lib as L

_FP = C.POINTER(C.c_float)
_IP = C.POINTER(C.c_int)

K = 8


def _m16(T) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(T, np.float32).reshape(4, 4).T.reshape(16))


class ScenePool:
    """Device-resident training pool: sources and targets as (n_scenes, n_pts, 8) float32
    (x, y, z and 5 features), unmoved; a training step moves the targets by its labels."""

    def __init__(self, src: np.ndarray, tgt: np.ndarray, device="cuda"):
        import torch
        src = np.ascontiguousarray(src, np.float32)
        tgt = np.ascontiguousarray(tgt, np.float32)
        if src.shape != tgt.shape or src.ndim != 3 or src.shape[2] != 8:
            raise ValueError("pool arrays must both be (n_scenes, n_pts, 8)")
        self.host_src, self.host_tgt = src, tgt
        self.src = torch.from_numpy(src).to(device)
        self.tgt = torch.from_numpy(tgt).to(device)
        self.n_scenes, self.n_pts = src.shape[0], src.shape[1]

    @staticmethod
    def generate(n_scenes: int, n_pts: int = 2048, seed0: int = 1_000_000, processes: int | None = None):
        """Seeded view pairs drawn like the global-registration scenes (host arrays)."""
        from concurrent.futures import ProcessPoolExecutor
        from multiprocessing import get_context
        from .scenes import global_views
        seeds = list(range(seed0, seed0 + n_scenes))
        procs = processes or min(16, os.cpu_count() or 1)
        if procs > 1 and n_scenes > 8:
            # spawned workers (never forked after CUDA is up); a worker that fails to
            # start raises instead of being restarted forever
            with ProcessPoolExecutor(procs, mp_context=get_context("spawn")) as ex:
                views = list(ex.map(global_views, [n_pts] * n_scenes, seeds, chunksize=8))
        else:
            views = [global_views(n_pts, s) for s in seeds]
        return np.stack([a for a, _ in views]), np.stack([b for _, b in views])


class ProposalNet:
    """The network's weights and training state on the device of ``cvo``."""

    def __init__(self, cvo, points_per_cloud: int = 512, seed: int = 0):
        self._cvo = cvo
        self._p = C.c_void_p()
        L.check(L.lib().cvo_proposal_create(cvo._h, int(points_per_cloud), C.c_uint32(seed), C.byref(self._p)),
                "cvo_proposal_create", cvo._h)
        npar, pts, nh = C.c_int(), C.c_int(), C.c_int()
        L.lib().cvo_proposal_dims(self._p, C.byref(npar), C.byref(pts), C.byref(nh))
        self.num_params, self.points_per_cloud, self.num_hyp = npar.value, pts.value, nh.value

    def close(self):
        if getattr(self, "_p", None) and self._p.value:
            L.lib().cvo_proposal_destroy(self._p)
            self._p = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._p

    # -- parameters -------------------------------------------------------
    def _get(self, which: int) -> np.ndarray:
        out = np.zeros(self.num_params, np.float32)
        L.check(L.lib().cvo_proposal_get(self._cvo._h, self._p, which, out.ctypes.data_as(_FP)), "cvo_proposal_get",
                self._cvo._h)
        return out

    def weights(self) -> np.ndarray:
        return self._get(0)

    def gradients(self) -> np.ndarray:
        """Gradients of the last ``train_step``."""
        return self._get(1)

    def set_weights(self, w) -> None:
        w = np.ascontiguousarray(w, np.float32)
        if w.size != self.num_params:
            raise ValueError("expected %d weights" % self.num_params)
        L.check(L.lib().cvo_proposal_set(self._cvo._h, self._p, w.ctypes.data_as(_FP)), "cvo_proposal_set",
                self._cvo._h)

    def set_gemm(self, kind: int) -> None:
        """Kernel of the matrix products: 0 the tcgen05 tensor-core GEMM (default), 1 the
        mma.sync GEMM (a second opinion for tests)."""
        L.check(L.lib().cvo_proposal_set_gemm(self._p, int(kind)), "cvo_proposal_set_gemm")

    def save(self, path: str) -> None:
        np.save(path, self.weights())

    def load(self, path: str) -> None:
        self.set_weights(np.load(path))

    # -- training ---------------------------------------------------------
    def train_step(self, pool: ScenePool, scene, T_label, lr: float, seed: int) -> float:
        """One step on pool pairs: scene (B,) indices, T_label (B, 3, 4) target = R source + t."""
        sc = np.ascontiguousarray(scene, np.int32)
        Tl = np.ascontiguousarray(np.asarray(T_label, np.float32).reshape(len(sc), 12))
        loss = C.c_float()
        L.check(L.lib().cvo_proposal_train_pool_dev(self._cvo._h, self._p, pool.n_scenes, pool.n_pts,
                                                    C.c_void_p(pool.src.data_ptr()), C.c_void_p(pool.tgt.data_ptr()),
                                                    len(sc), sc.ctypes.data_as(_IP), Tl.ctypes.data_as(_FP),
                                                    float(lr), C.c_uint32(seed & 0xFFFFFFFF), C.byref(loss)),
                "cvo_proposal_train_pool_dev", self._cvo._h)
        return loss.value

    def forward_pool(self, pool: ScenePool, scene, T_tgt=None, seed: int = 0):
        """(raw outputs (B, 72), hypotheses (B, 8, 4, 4) row-major, target = R source + t)."""
        sc = np.ascontiguousarray(scene, np.int32)
        B = len(sc)
        Tp = None
        if T_tgt is not None:
            Tp = np.ascontiguousarray(np.asarray(T_tgt, np.float32).reshape(B, 12))
        raw = np.zeros((B, 9 * K), np.float32)
        To = np.zeros(B * K * 16, np.float32)
        L.check(L.lib().cvo_proposal_forward_pool_dev(self._cvo._h, self._p, pool.n_scenes, pool.n_pts,
                                                      C.c_void_p(pool.src.data_ptr()), C.c_void_p(pool.tgt.data_ptr()),
                                                      B, sc.ctypes.data_as(_IP),
                                                      Tp.ctypes.data_as(_FP) if Tp is not None else None,
                                                      C.c_uint32(seed & 0xFFFFFFFF), raw.ctypes.data_as(_FP),
                                                      To.ctypes.data_as(_FP)),
                "cvo_proposal_forward_pool_dev", self._cvo._h)
        return raw, To.reshape(B, K, 4, 4).transpose(0, 1, 3, 2).copy()

    def hypotheses(self, sources, targets, seed: int = 0) -> np.ndarray:
        """(B, 8, 4, 4) row-major hypotheses (cvo_align's T_init convention) for GpuClouds."""
        B = len(sources)
        S = (C.c_void_p * B)(*[s.handle.value for s in sources])
        T = (C.c_void_p * B)(*[t.handle.value for t in targets])
        To = np.zeros(B * K * 16, np.float32)
        L.check(L.lib().cvo_proposal_hypotheses_dev(self._cvo._h, self._p, B, S, T, C.c_uint32(seed & 0xFFFFFFFF),
                                                    To.ctypes.data_as(_FP)),
                "cvo_proposal_hypotheses_dev", self._cvo._h)
        return To.reshape(B, K, 4, 4).transpose(0, 1, 3, 2).copy()


def rotation_error_deg(Ra, Rb) -> np.ndarray:
    c = (np.einsum("...ij,...ij->...", Ra, Rb) - 1.0) / 2.0
    return np.degrees(np.arccos(np.clip(c, -1.0, 1.0)))


def train(net: ProposalNet, pool: ScenePool, steps: int, batch: int = 64, lr: float = 1e-3, seed: int = 0,
          max_trans: float = 2.0, log_every: int = 0):
    """Adam on random pool pairs, each target moved by a fresh motion drawn like the
    global-registration pairs.  Returns (per-step losses, seconds)."""
    from .scenes import random_motion
    rng = np.random.default_rng(seed)
    losses = np.zeros(steps, np.float32)
    t0 = time.perf_counter()
    for it in range(steps):
        scene = rng.integers(0, pool.n_scenes, size=batch)
        T = np.stack([random_motion(rng, max_trans) for _ in range(batch)])
        losses[it] = net.train_step(pool, scene, T, lr, int(rng.integers(0, 2 ** 32)))
        if log_every and (it % log_every == 0 or it == steps - 1):
            print("step %d loss %.4f" % (it, losses[it]), flush=True)
    return losses, time.perf_counter() - t0


def evaluate(net: ProposalNet, pool: ScenePool, n_pairs: int, seed: int = 1, max_trans: float = 2.0):
    """Best-of-K rotation error (degrees) of the hypotheses on random moved pool pairs."""
    from .scenes import random_motion
    rng = np.random.default_rng(seed)
    scene = np.arange(n_pairs) % pool.n_scenes
    T = np.stack([random_motion(rng, max_trans) for _ in range(n_pairs)])
    _, hyp = net.forward_pool(pool, scene, T, seed=seed)
    err = rotation_error_deg(hyp[:, :, :3, :3], T[:, None, :3, :3])
    return err.min(1), err
