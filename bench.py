"""Benchmark: global registration of 50k-point pairs on one GB300.

Workload (one "step"): B seeded 50k-point pairs drawn like the colour/stereo
configuration but with a uniformly random rotation and a shift <= 2 m.  Every pair
is registered from the learned proposal: the network proposes 8 poses per pair, all
pairs' hypotheses are ranked by the cos-angle in one batch, the best --refine of
each pair are refined together by the batched CVO align (one persistent batch,
CUDA-graph chunks) and judged by the final cos-angle, with the 24-rotation grid as
the fallback below --fallback-cos.  The network is trained on the device before the
timed region (or loaded with --proposal-weights).  The plain grid (nearest of the 24
rotations by cos-angle, then the batched align) runs on the same pairs in the same
process, and the grid with all 24 rotations refined runs on the first --all24-pairs.
The metric is registrations/s; success = rotation error < 2 deg and translation
error < 5 cm against the generated ground truth.

value : device-resident clouds (inputs already in HBM), whole-job registrations/s
e2e   : the same through the C ABI from host buffers (cloud upload inside the timed region)
roofline : the association phase of the CVO iteration, algorithmic bytes / event-timed duration
cpu_baseline : the CPU oracle (a restatement of the reference's CPU inner product and
               align loop) on a bounded sample, scaled to registrations/s

usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "registrations/s @50k pts: batched+learned vs plain grid, equal accuracy; HBM GB/s"
UNIT = "registrations/s"


def _capture_value(key):
    """A per-pair figure of the committed association capture
    (profiles/k_assoc_cta_global50k.json, written by rkhs_ba_gb300.profiling), or None."""
    from rkhs_ba_gb300 import profiling
    d = profiling.load("k_assoc_cta_global50k.json")
    return None if d is None else d.get(key)


def issue_roofline(inst_per_pair, pair_passes, launches, avg_launch_s, sms, sm_mhz):
    """Instruction-issue bound of the association phase: k_assoc_cta's warp instructions
    per launch (the ncu capture's count per pair-launch times this run's mean pairs per
    launch) over the event-timed phase duration, against one warp instruction per
    cycle on each of an SM's 4 schedulers at the sampled SM clock.  None when an input
    is missing."""
    if not inst_per_pair or pair_passes <= 0 or launches <= 0 or not avg_launch_s or avg_launch_s <= 0 \
            or not sms or not sm_mhz:
        return None
    inst = inst_per_pair * pair_passes / launches
    achieved = inst / avg_launch_s / 1e9
    peak = sms * 4 * sm_mhz * 1e6 / 1e9
    return {"achieved": round(achieved, 2), "peak": round(peak, 2), "unit": "G warp instructions/s",
            "frac": round(achieved / peak, 4), "warp_instructions_per_launch": round(inst),
            "note": "k_assoc_cta instructions per pair from the committed ncu capture summary over the whole "
                    "association phase's duration; peak = SMs x 4 schedulers x SM clock"}


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons while the timed region runs."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None
        self.th = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.th = threading.Thread(target=self._read, daemon=True)
        self.th.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 8:
                self.rows.append(parts)

    def stop(self):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        if self.th is not None:
            self.th.join(timeout=2)
        sm = []
        reasons = set()
        smax = None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[0]))
                smax = float(r[1])
            except ValueError:
                continue
            for k, n in enumerate(names):
                if r[4 + k].lower() in ("active", "1"):
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def make_pairs(n_pairs, n_points, seed0=1000, gen=None):
    """Seeded pairs (global pairs unless gen is another scenes generator taking (n, seed);
    n_points may be a list of sizes), generated by spawned worker processes (never forked
    after CUDA is up)."""
    from rkhs_ba_gb300 import scenes
    gen = gen or scenes.global_pair
    sizes = list(n_points) if isinstance(n_points, (list, tuple)) else [n_points] * n_pairs
    if n_pairs <= 1:
        return [gen(sizes[k], seed0 + k) for k in range(n_pairs)]
    from concurrent.futures import ProcessPoolExecutor
    from multiprocessing import get_context
    with ProcessPoolExecutor(min(n_pairs, os.cpu_count() or 1), mp_context=get_context("spawn")) as ex:
        return list(ex.map(gen, sizes[:n_pairs], [seed0 + k for k in range(n_pairs)]))


def _proposal(args, cvo):
    """The learned proposal for the timed workload: weights from --proposal-weights when
    given, else trained here on the device from a seeded scene pool (untimed setup)."""
    from rkhs_ba_gb300.proposal import ProposalNet, ScenePool, evaluate, train
    net = ProposalNet(cvo, points_per_cloud=512, seed=0)
    info = {"points_per_cloud": 512, "hypotheses": net.num_hyp, "params": net.num_params}
    if args.proposal_weights and os.path.exists(args.proposal_weights):
        net.load(args.proposal_weights)
        info["weights"] = os.path.basename(args.proposal_weights)
        return net, info
    t0 = time.perf_counter()
    pool = ScenePool(*ScenePool.generate(args.train_scenes, 2048, seed0=1_000_000))
    held = ScenePool(*ScenePool.generate(64, 2048, seed0=3_000_000))
    info["pool_s"] = round(time.perf_counter() - t0, 2)
    losses, secs = train(net, pool, steps=args.train_steps, batch=64, lr=1e-3, seed=0)
    best, _ = evaluate(net, held, 64)
    info.update({"train_scenes": args.train_scenes, "train_steps": args.train_steps, "batch": 64,
                 "train_pairs": args.train_steps * 64, "train_s": round(secs, 2),
                 "ms_per_train_step": round(1000.0 * secs / max(1, args.train_steps), 3),
                 "loss_first_100": round(float(losses[:100].mean()), 4),
                 "loss_last_100": round(float(losses[-100:].mean()), 4),
                 "held_out_best_of_k_rot_err_deg_median": round(float(np.median(best)), 2),
                 "held_out_best_of_k_within_30deg": round(float((best < 30).mean()), 3)})
    if args.save_proposal:
        net.save(args.save_proposal)
    return net, info


def workload_config(args):
    """The `config` of both arms' JSON lines (the same workload)."""
    return {"workload": "global registration, learned proposal (8 hypotheses, best %d refined) + CVO refinement, "
                        "24-rotation grid fallback" % args.refine,
            "points_per_cloud": args.points, "pairs_per_step": args.pairs, "params": "color.yaml",
            "rotation": "uniform SO(3)", "translation_max_m": 2.0, "fallback_cos": args.fallback_cos,
            "refine_ell": args.refine_ell,
            "l2": "256 MB buffer written between timed steps",
            "parallelism": "replicas"}


def _success(Ts, pairs):
    errs = [scenes_pose_error(Ts[k], pairs[k][2]) for k in range(len(pairs))]
    return [bool(r < 2.0 and t < 0.05) for r, t in errs]


def scenes_pose_error(T, T_gt):
    from rkhs_ba_gb300 import scenes
    return scenes.pose_error(T, T_gt)


def replica_rate(units_per_rank, ms, dist=None, device="cpu"):
    """Whole-job rate of independent replicas: the units of all ranks divided by the
    slowest rank's milliseconds (a MAX all-reduce over the process group; dist None
    means one process).  Returns (units/s, slowest ms)."""
    world = 1
    if dist is not None:
        import torch
        t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
        world = dist.get_world_size()
    return units_per_rank * world / (ms / 1000.0), ms


def run_ours(args):
    import torch
    from rkhs_ba_gb300 import CvoGPU, CvoParams, params_path, scenes

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    p = CvoParams(params_path("color"))
    if args.max_iter > 0:
        p.MAX_ITER = args.max_iter
    cvo = CvoGPU(params=p)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    cvo.set_stream(stream.cuda_stream)
    net, prop_info = _proposal(args, cvo)
    pairs = make_pairs(args.pairs, args.points, seed0=1000 + 100 * rank)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")   # > L2 (129 MB)

    def register_learned(gs, gt):
        Ts, cos, fb, its, _ = cvo.register_learned_batch(net, gs, gt, n_refine=args.refine,
                                                         fallback_cos=args.fallback_cos, refine_ell=args.refine_ell)
        return Ts, its, fb

    def register_grid(gs, gt):
        inits = []
        for s, t in zip(gs, gt):
            T, _ = cvo.get_nearest_init_pose(s, t, p.ell_init_first_frame, 0, 1)
            inits.append(scenes.inv_T(T))        # CvoGPU::align(int overload) inverts the grid pose
        Ts, rets, its, _ = cvo.align_batch(gs, gt, inits)
        return Ts, its, np.zeros(len(gs), np.int32)

    def timed(fn, gs, gt, steps):
        ms, res = [], []
        for k in range(steps):
            flush.fill_(float(k))
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            res.append(fn(gs, gt))
            e1.record(stream)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        return ms, res

    gs = [cvo.upload(s) for s, _, _ in pairs]
    gt = [cvo.upload(t) for _, t, _ in pairs]
    # association cell size picked by the autotuner on the first pair (untimed setup)
    tune = None
    if not args.no_autotune:
        # at the pose and lengthscale the refinement starts from: the network's first hypothesis
        hyp0 = net.hypotheses([gs[0]], [gt[0]])[0, 0]
        r = cvo.autotune(gs[0], gt[0], hyp0, ell=args.refine_ell if args.refine_ell > 0 else p.ell_init, reps=2)
        b = r["configs"][r["best"]]
        tune = {"div_r": b[0], "div_ext": b[1], "blocks_per_sm": b[2] if b[2] > 0 else "occupancy",
                "blocks_per_sm_applies_to": "batches with the tuned pair's work items (the 8-pair steps keep the "
                                            "occupancy default)",
                "ms": round(b[3], 3), "configs": len(r["configs"]),
                "default_ms": round(next(ms for a, e, bp, ms in r["configs"] if (a, e, bp) == (4.0, 8.0, 0)), 3)}

    for _ in range(args.warmup):
        register_learned(gs, gt)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()

    # ---- device-resident timed region: learned proposal + batched CVO
    cvo.profile(True)
    cvo.profile_reset()
    launches0 = cvo.kernel_launches
    clocks = ClockSampler(local)
    clocks.start()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    t_wall0 = time.perf_counter()
    step_ms, results = timed(register_learned, gs, gt, args.steps)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    wall = time.perf_counter() - t_wall0
    clk = clocks.stop()
    launches = cvo.kernel_launches - launches0
    prof = cvo.profile_read()
    cvo.profile(False)
    value, total_ms = replica_rate(args.pairs * args.steps, float(np.sum(step_ms)), dist, "cuda")
    Ts, its, fb = results[-1]
    succ = _success(Ts, pairs)

    # ---- the plain 24-rotation grid (nearest grid rotation by cos-angle, then align) on the same pairs
    register_grid(gs, gt)
    grid_ms, grid_res = timed(register_grid, gs, gt, max(1, args.grid_steps))
    grid_value = args.pairs * len(grid_ms) / (float(np.sum(grid_ms)) / 1000.0)
    grid_succ = _success(grid_res[-1][0], pairs)
    # ---- the plain grid with every one of its 24 rotations refined and judged (the
    # grid's best accuracy), on the first --all24-pairs pairs
    all24 = None
    if args.all24_pairs > 0:
        grid = CvoGPU.rotation_grid(1)
        T24 = []
        for R in grid:
            T = np.eye(4)
            T[:3, :3] = R.T                      # internal pose of grid rotation R
            T24.append(T)
        k24 = min(args.all24_pairs, args.pairs)
        ms24, ok24, it24 = [], [], []
        all24_err = None
        for k in range(k24):
            flush.fill_(float(k))
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            try:
                To, bi, cosv, _ = cvo.register_hypotheses(gs[k], gt[k], T24, p.ell_init_first_frame)
            except RuntimeError as e:                 # reported in the line, not fatal to it
                all24_err = str(e)
                break
            e1.record(stream)
            e1.synchronize()
            ms24.append(e0.elapsed_time(e1))
            r, tr = scenes.pose_error(To, pairs[k][2])
            ok24.append(bool(r < 2.0 and tr < 0.05))
        if ms24:
            all24 = {"value": round(len(ms24) / (float(np.sum(ms24)) / 1000.0), 4), "unit": UNIT,
                     "pairs": len(ms24), "success_rate": float(np.mean(ok24)),
                     "note": "24 aligns per pair in one batch, judged by the final cos-angle"}
        if all24_err:
            all24 = dict(all24 or {}, error=all24_err)

    # ---- end-to-end through the C ABI from host buffers (learned pipeline)
    h2d = sum(s.xyz.nbytes + s.features.nbytes + t.xyz.nbytes + t.features.nbytes for s, t, _ in pairs)
    d2h = args.pairs * (16 * 4 + 4 + 4 + 4)
    torch.cuda.synchronize()
    e2e_ms = []
    for k in range(max(1, min(args.steps, 2))):
        flush.fill_(float(k))
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        hs = [cvo.upload(s) for s, _, _ in pairs]
        ht = [cvo.upload(t) for _, t, _ in pairs]
        register_learned(hs, ht)
        e1.record(stream)
        e1.synchronize()
        e2e_ms.append(e0.elapsed_time(e1))
        for c in hs + ht:
            c.free()
    e2e_value, _ = replica_rate(args.pairs, float(np.mean(e2e_ms)), dist, "cuda")

    # ---- like-for-like units the reference arm also reports, on the same pairs
    H0 = net.hypotheses([gs[0]], [gt[0]])[0]
    cos_ms = []
    for k in range(3):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        cvo.inner_product_batch(gs[0], gt[0], list(H0), p.ell_init_first_frame)
        e1.record(stream)
        e1.synchronize()
        cos_ms.append(e0.elapsed_time(e1))
    pair_iters = sum(int(i) for r in results for i in r[1])
    like = {"cos_angles_per_s": round(len(H0) / (float(np.median(cos_ms)) / 1000.0), 2),
            "cos_angles_note": "the 8 hypotheses of the first pair in one batched call (GPU cap semantics)",
            "align_iterations_per_s": round(pair_iters / (float(np.sum(step_ms)) / 1000.0), 2),
            "align_iterations_note": "pair iterations of the timed learned steps over their whole duration "
                                     "(ranking and judging included, so a lower bound on the align rate)"}
    weights_match = None
    if os.path.exists(WEIGHTS) and not args.proposal_weights:
        weights_match = bool(np.array_equal(np.load(WEIGHTS).astype(np.float32), net.weights().astype(np.float32)))

    # ---- roofline of the association kernel
    peak, peak_kind = _peaks()
    roof = None
    if prof["assoc_launches"] > 0 and prof["assoc_ms"] > 0:
        per_launch_bytes = prof["assoc_bytes"] / prof["assoc_launches"]
        avg_s = prof["assoc_ms"] / prof["assoc_launches"] / 1000.0
        achieved = per_launch_bytes / avg_s / 1e9
        # DRAM bytes of one association launch: the committed ncu capture's bytes per
        # pair times the mean number of pairs a launch of this run served (pair
        # iterations / launches)
        traffic = None
        pair_passes = sum(int(i) for r in results for i in r[1])
        per_pair = _capture_value("dram_bytes_per_pair_launch")
        if per_pair is not None and pair_passes > 0:
            traffic = round(per_pair * pair_passes / prof["assoc_launches"])
        roof = {"bound": "hbm", "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 5), "traffic": traffic, "peak_source": peak_kind,
                "kernel": "k_assoc_cta + k_select + k_rescan + k_rowsum", "launches": prof["assoc_launches"],
                "avg_launch_us": round(avg_s * 1e6, 3), "algorithmic_bytes_per_launch": round(per_launch_bytes),
                "iteration_kernel_ms": {k: round(v, 3) for k, v in prof["kernel_ms"].items()},
                "association_phase_ms": {k: round(v, 3) for k, v in prof.get("assoc_split_ms", {}).items()}}
        try:
            sms = torch.cuda.get_device_properties(local).multi_processor_count
        except Exception:
            sms = None
        roof["issue"] = issue_roofline(_capture_value("warp_instructions_per_pair_launch"),
                                       pair_passes, prof["assoc_launches"], avg_s, sms,
                                       clk.get("sm_mhz") or clk.get("sm_max_mhz"))

    out = {
        "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 (network: bf16 operands, f32 accumulation)",
        "data": "synthetic (seeded scenes)",
        "config": workload_config(args),
        "accuracy": {"success_rate": float(np.mean(succ)), "criterion": "rot<2deg, trans<5cm",
                     "mean_iters": float(np.mean(its)), "fallbacks": int(np.sum(fb))},
        "plain_grid": {"value": round(grid_value, 4), "unit": UNIT, "success_rate": float(np.mean(grid_succ)),
                       "mean_iters": float(np.mean(grid_res[-1][1])), "steps": len(grid_ms),
                       "note": "nearest of the 24 grid rotations by cos-angle, then one batched align"},
        "plain_grid_all24": all24,
        "proposal": dict(prop_info, weights_equal_committed=weights_match),
        "like_for_like": like,
        "autotune": tune,
        "e2e": {"value": round(e2e_value, 4), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": int(launches),
        "roofline": roof,
        "clocks": clk,
        "wall_s": round(wall, 3),
    }
    if rank == 0 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(args, pairs[0], net.weights())
    if rank == 0:
        print(json.dumps(out))
    if dist:
        dist.destroy_process_group()


WEIGHTS = os.path.join(ROOT, "rkhs_ba_gb300", "weights", "proposal_color50k.npy")


class CpuLearned:
    """The learned global registration of the timed workload, run on the host cores
    with the oracle (the CPU restatement of the reference's path): the proposal
    network's forward pass (oracle/proposal.py, numpy), the ranking of its 8
    hypotheses by the approximate cos-angle with the reference's CPU inner product
    (inner_product_cpu semantics: radius search, no cap, CvoGPU.cpp:113-231), the
    refinement of the best one by the oracle's align loop (align_impl,
    CvoGPU.cu:1239-1477) from --refine-ell, and the final cos-angle that judges it.
    Loads nothing from the product library: parameters come from the oracle's own
    yaml reader and the network weights from the committed file WEIGHTS (the
    deterministic output of the device training the GPU arm runs)."""

    def __init__(self, args, weights=None):
        from oracle import oracle as orc
        from oracle import proposal as op
        from oracle.params import OracleParams
        from rkhs_ba_gb300 import params_path
        self.orc, self.op = orc, op
        self.p = OracleParams(params_path("color"))
        self.refine_ell = args.refine_ell if args.refine_ell > 0 else self.p.ell_init
        if weights is None:
            weights = np.load(args.proposal_weights or WEIGHTS)
        self.w = np.asarray(weights, np.float32)
        self.cores = os.cpu_count() or 1
        orc.set_threads(self.cores)

    def hypotheses(self, src, tgt, seed=0, P=512):
        op = self.op
        I = np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, 0]], np.float32)
        X = np.zeros((2, P, op.IN), np.float32)
        cent = np.zeros((2, 3), np.float32)
        for side, c in ((0, src), (1, tgt)):
            _, cent[side], X[side] = op.slot_input(c.xyz, c.features, I, seed, side, P)
        act = op.forward(self.w, X, 1, bf16_ops=True)
        return op.hypotheses(act["O"], cent)[0].astype(np.float32)

    def cos(self, src, tgt, T, ell):
        ip, _ = self.orc.inner_product_cpu_semantics(self.p, src, tgt, T, ell)
        return ip / np.sqrt(float(src.num_points()) * float(tgt.num_points()))

    def register(self, pair, max_iter=None):
        """One registration (max_iter limits the refinement: a bounded sample).  Returns
        (pose, iterations, {phase: seconds})."""
        src, tgt, _ = pair
        t = {}
        t0 = time.perf_counter()
        H = self.hypotheses(src, tgt)
        t["network"] = time.perf_counter() - t0
        t0 = time.perf_counter()
        cosv = [self.cos(src, tgt, H[k], self.p.ell_init_first_frame) for k in range(len(H))]
        t["rank"] = time.perf_counter() - t0
        q = self.p.copy()
        q.ell_init = self.refine_ell
        if max_iter is not None:
            q.MAX_ITER = max_iter
        t0 = time.perf_counter()
        ret, T, iters, _ = self.orc.align(q, src, tgt, H[int(np.argmax(cosv))])
        t["refine"] = time.perf_counter() - t0
        t0 = time.perf_counter()
        self.cos(src, tgt, np.linalg.inv(T.astype(np.float64)).astype(np.float32), self.p.ell_init_first_frame)
        t["judge"] = time.perf_counter() - t0
        return T, int(iters), t


def cpu_baseline(args, pair, weights=None):
    """One complete registration of one pair of the workload by the same pipeline on the
    host cores (CpuLearned, with the network weights the GPU arm trained), timed end to
    end: about half a minute of CPU work on a 16-core host."""
    cl = CpuLearned(args, weights)
    t0 = time.perf_counter()
    _, iters, t = cl.register(pair)
    sec = time.perf_counter() - t0
    src = pair[0]
    return {"value": round(1.0 / sec, 6), "unit": UNIT, "cores": cl.cores, "kind": "port",
            "sample": "one complete registration of the first %d-point pair of the workload by the same pipeline "
                      "(network forward, 8 CPU cos-angles, CPU align from ell %.2f: %d iterations, CPU judge)"
                      % (src.num_points(), cl.refine_ell, iters),
            "seconds_per_registration": round(sec, 3), "iterations": iters,
            "phase_s": {k: round(v, 3) for k, v in t.items()},
            "cos_angles_per_s": round(9.0 / (t["rank"] + t["judge"]), 4),
            "align_iterations_per_s": round(iters / t["refine"], 4)}


def run_component(args):
    """Timing of one component beside the main workload (one JSON line): the multi-frame
    window solve (8 frames of 20k-60k points, all 28 edges), the association with a
    non-isotropic kernel (50k x 50k), the RGB-D front-end (a 1226 x 370 frame, 50k
    selected pixels), adaptive-ell CVO, the proposal network, or the held-out evaluation
    of global registration (global-eval: learned vs plain grid over --eval-pairs pairs).
    Each call is timed end to end after warm-up; where the oracle has the same path it is
    timed on a bounded sample of the same input."""
    import torch
    from oracle import oracle as orc
    from rkhs_ba_gb300 import CvoGPU, CvoParams, params_path, scenes

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    cores = os.cpu_count() or 1
    orc.set_threads(cores)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        ts = []
        for k in range(args.steps):
            flush.fill_(float(k))
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - t0)
        return float(np.mean(ts))

    out = {"component": args.component, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
           "higher_is_better": True, "data": "synthetic (seeded scenes)", "dtype": "f32"}
    if args.component == "irls":
        clouds, gt = scenes.irls_window(n_frames=8, seed=0)
        rng = np.random.default_rng(7)
        P0 = []
        for k in range(8):
            T = gt[k].copy()
            if k > 0:
                T = T @ scenes.make_T(scenes.rot_axis_angle(rng.normal(size=3), np.radians(1.0)), rng.normal(size=3) * 0.03)
            P0.append(T[:3, :].reshape(12))
        P0 = np.stack(P0)
        edges = [(a, b) for a in range(8) for b in range(a + 1, 8)]
        hold = [1] + [0] * 7
        p = CvoParams(params_path("irls"))
        cvo = CvoGPU(params=p)
        res = {}

        def solve():
            res["P"], res["s"], res["it"] = cvo.align_multi(clouds, P0, hold, edges)
        sec = timed(solve)
        q = p.copy()
        q.multiframe_max_iters = 1
        t0 = time.perf_counter()
        orc.align_multi(q, clouds, P0, hold, edges)
        t_outer = time.perf_counter() - t0
        cpu_sec = t_outer * max(res["it"], 1)
        out.update({"metric": "window solves/s (8 frames, 28 edges)", "unit": "solves/s", "value": round(1.0 / sec, 4),
                    "ms_per_call": round(sec * 1000, 3),
                    "config": {"frames": 8, "points_per_frame": [c.num_points() for c in clouds], "edges": 28,
                               "params": "irls.yaml", "outer_iterations": int(res["it"])},
                    "cpu_baseline": {"value": round(1.0 / cpu_sec, 6), "unit": "solves/s", "cores": cores, "kind": "port",
                                     "sample": "one outer iteration of the oracle's window solve, scaled to the GPU "
                                               "run's %d outer iterations" % res["it"]}})
    elif args.component == "aniso":
        src, tgt, _ = scenes.global_pair(n=args.points, seed=1000)
        p = CvoParams(params_path("color"))
        cvo = CvoGPU(params=p)
        K = np.diag([0.5, 0.5, 0.6]).astype(np.float32)
        T = np.eye(4, dtype=np.float32)
        gs, gtc = cvo.upload(src), cvo.upload(tgt)
        sec = timed(lambda: cvo.compute_association_gpu(gs, gtc, T, K))
        nsub = min(2000, src.num_points())
        from rkhs_ba_gb300 import CvoPointCloud
        sub = CvoPointCloud(src.xyz[:nsub], src.features[:nsub])
        t0 = time.perf_counter()
        orc.association_aniso(p, sub, tgt, T, K)
        cpu_sec = (time.perf_counter() - t0) * src.num_points() / nsub
        out.update({"metric": "non-isotropic associations/s (50k x 50k)", "unit": "associations/s",
                    "value": round(1.0 / sec, 4), "ms_per_call": round(sec * 1000, 3),
                    "config": {"points": args.points, "kernel": "diag(0.5, 0.5, 0.6)", "params": "color.yaml",
                               "device_clouds": True},
                    "cpu_baseline": {"value": round(1.0 / cpu_sec, 6), "unit": "associations/s", "cores": cores,
                                     "kind": "port", "sample": "%d source rows against all targets, scaled to %d rows"
                                                               % (nsub, src.num_points())}})
    elif args.component == "frontend":
        rng = np.random.default_rng(3)
        rows, cols = 370, 1226
        yy, xx = np.mgrid[0:rows, 0:cols]
        base = 127 + 80 * np.sin(xx / 9.0) * np.cos(yy / 7.0)
        img = np.clip(base[..., None] + rng.normal(0, 25, size=(rows, cols, 3)), 0, 255).astype(np.uint8)
        depth = np.exp(rng.uniform(np.log(2000.0), np.log(50000.0), size=(rows, cols))).astype(np.float32)
        flat = rng.choice(rows * cols, size=50000, replace=False)
        uv = np.stack([flat % cols, flat // cols], 1).astype(np.int32)
        intr = np.array([718.0, 718.0, 613.0, 185.0], np.float32)
        cvo = CvoGPU(params=CvoParams(params_path("color")))
        sec = timed(lambda: cvo.cloud_from_rgbd(img, depth, intr, 1000.0, uv))
        t0 = time.perf_counter()
        orc.cloud_from_rgbd(img, depth, intr, 1000.0, uv)
        cpu_sec = time.perf_counter() - t0
        out.update({"metric": "RGB-D frames to clouds/s (1226 x 370, 50k points)", "unit": "frames/s",
                    "value": round(1.0 / sec, 4), "ms_per_call": round(sec * 1000, 3),
                    "config": {"rows": rows, "cols": cols, "selected": 50000, "host_inputs": True},
                    "cpu_baseline": {"value": round(1.0 / cpu_sec, 6), "unit": "frames/s", "cores": 1, "kind": "port",
                                     "sample": "the whole frame (the oracle is single-threaded here)"}})
    elif args.component == "adaptive":
        from rkhs_ba_gb300 import AdaptiveCvoGPU
        s, t, T_gt = scenes.room_pair(n=10000, seed=0)
        p = CvoParams(params_path("geometric"))
        cvo = AdaptiveCvoGPU(params=p)
        res = {}

        def reg():
            res["r"] = cvo.align(s, t, np.eye(4))
        sec = timed(reg)
        ret, T, _, iters = res["r"]
        rerr, terr = scenes.pose_error(T, T_gt)
        # the oracle on a bounded sample: its first --cpu-iters iterations, scaled to the GPU's count
        q = p.copy()
        q.MAX_ITER = max(1, args.cpu_iters)
        t0 = time.perf_counter()
        orc.align_adaptive(q, s, t, np.eye(4))
        per_iter = (time.perf_counter() - t0) / q.MAX_ITER
        cpu_sec = per_iter * max(iters, 1)
        out.update({"metric": "adaptive-ell registrations/s (10k-point room pair, geometric kernel)",
                    "unit": "registrations/s", "value": round(1.0 / sec, 4), "ms_per_call": round(sec * 1000, 3),
                    "iterations": int(iters), "ms_per_iteration": round(sec * 1000 / max(iters, 1), 3),
                    "accuracy": {"rot_err_deg": round(rerr, 4), "trans_err_m": round(terr, 4)},
                    "config": {"points": 10000, "params": "geometric.yaml", "kernel_matrices_per_iteration": 3,
                               "cap": 512, "host_inputs": True},
                    "cpu_baseline": {"value": round(1.0 / cpu_sec, 6), "unit": "registrations/s", "cores": cores,
                                     "kind": "port", "sample": "%d oracle iterations scaled to the GPU's %d"
                                                                % (q.MAX_ITER, iters)}})
    elif args.component == "global-eval":
        # success and registrations/s of the learned pipeline and of the plain grid (nearest
        # of the 24 rotations by cos-angle, then align) over --eval-pairs seeded held-out
        # pairs (seeds disjoint from the training pool and the default line's pairs),
        # registered in batches of --pairs; clouds resident on the device
        p = CvoParams(params_path("color"))
        cvo = CvoGPU(params=p)
        net, prop_info = _proposal(args, cvo)
        n_total = max(1, args.eval_pairs)
        pairs = make_pairs(n_total, args.points, seed0=args.eval_seed0)
        errs = {"learned": [], "grid": []}
        iters = {"learned": [], "grid": []}
        secs = {"learned": 0.0, "grid": 0.0}
        fallbacks = 0

        def learned(gs, gt):
            return cvo.register_learned_batch(net, gs, gt, n_refine=args.refine, fallback_cos=args.fallback_cos,
                                              refine_ell=args.refine_ell)

        def grid(gs, gt):
            inits = []
            for s, t in zip(gs, gt):
                Tg, _ = cvo.get_nearest_init_pose(s, t, p.ell_init_first_frame, 0, 1)
                inits.append(scenes.inv_T(Tg))
            return cvo.align_batch(gs, gt, inits)

        # the grid with all 24 rotations refined and judged (its best accuracy), on the first
        # --all24-pairs pairs
        T24 = []
        for R in CvoGPU.rotation_grid(1):
            T = np.eye(4)
            T[:3, :3] = R.T                   # internal pose of grid rotation R
            T24.append(T)
        errs["all24"], secs["all24"], n24 = [], 0.0, min(max(0, args.all24_pairs), n_total)
        for b0 in range(0, n_total, args.pairs):
            batch = pairs[b0:b0 + args.pairs]
            gs = [cvo.upload(s) for s, _, _ in batch]
            gt = [cvo.upload(t) for _, t, _ in batch]
            if b0 == 0:                       # warm-up of both paths (graphs, grid levels)
                learned(gs, gt)
                grid(gs, gt)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            Ts, _, fb, its, _ = learned(gs, gt)
            torch.cuda.synchronize()
            secs["learned"] += time.perf_counter() - t0
            fallbacks += int(np.sum(fb))
            t0 = time.perf_counter()
            Tp, _, itp, _ = grid(gs, gt)
            torch.cuda.synchronize()
            secs["grid"] += time.perf_counter() - t0
            for k, (_, _, T_gt) in enumerate(batch):
                errs["learned"].append(scenes.pose_error(Ts[k], T_gt))
                errs["grid"].append(scenes.pose_error(Tp[k], T_gt))
                if b0 + k < n24:
                    torch.cuda.synchronize()
                    t0 = time.perf_counter()
                    To, _, _, _ = cvo.register_hypotheses(gs[k], gt[k], T24, p.ell_init_first_frame)
                    torch.cuda.synchronize()
                    secs["all24"] += time.perf_counter() - t0
                    errs["all24"].append(scenes.pose_error(To, T_gt))
            iters["learned"] += [int(i) for i in its]
            iters["grid"] += [int(i) for i in itp]
            for c in gs + gt:
                c.free()
        ok = {m: [bool(r < 2.0 and t < 0.05) for r, t in errs[m]] for m in errs}
        counts = {"learned": n_total, "grid": n_total, "all24": len(errs["all24"])}
        rate = {m: counts[m] / secs[m] for m in secs if secs[m] > 0}
        out.update({"metric": "global registrations/s and success over held-out 50k-point pairs, learned vs plain grid",
                    "unit": "registrations/s", "value": round(rate["learned"], 4), "pairs": n_total,
                    "learned": {"value": round(rate["learned"], 4), "success_rate": float(np.mean(ok["learned"])),
                                "mean_iters": float(np.mean(iters["learned"])), "fallbacks": fallbacks},
                    "plain_grid": {"value": round(rate["grid"], 4), "success_rate": float(np.mean(ok["grid"])),
                                   "mean_iters": float(np.mean(iters["grid"]))},
                    "plain_grid_all24": ({"value": round(rate["all24"], 4), "pairs": counts["all24"],
                                          "success_rate": float(np.mean(ok["all24"])),
                                          "successes": int(np.sum(ok["all24"]))} if counts["all24"] else None),
                    "successes": {"learned": int(np.sum(ok["learned"])), "grid": int(np.sum(ok["grid"]))},
                    "both_succeed": float(np.mean([a and b for a, b in zip(ok["learned"], ok["grid"])])),
                    "learned_over_plain_grid": round(rate["learned"] / rate["grid"], 3),
                    "learned_over_all24": (round(rate["learned"] / rate["all24"], 3) if counts["all24"] else None),
                    "config": {"points_per_cloud": args.points, "batch": args.pairs, "params": "color.yaml",
                               "seeds": [args.eval_seed0, args.eval_seed0 + n_total - 1],
                               "rotation": "uniform SO(3)", "translation_max_m": 2.0,
                               "criterion": "rot<2deg, trans<5cm", "refine_ell": args.refine_ell,
                               "timing": "host clock around synchronised batches, clouds resident"},
                    "proposal": prop_info})
    elif args.component == "batching":
        # one persistent batch for all registrations against one call per registration (the
        # reference's way): (a) --pairs colour pairs of uneven size (20k-60k points), identity
        # start; (b) the 24 grid rotations of one global pair as 24 starts of the same pair
        p = CvoParams(params_path("color"))
        cvo = CvoGPU(params=p)
        sizes = [int(x) for x in np.random.default_rng(7).integers(20000, 60001, size=args.pairs)]
        pairs = make_pairs(args.pairs, sizes, seed0=300, gen=scenes.stereo_pair)
        gs = [cvo.upload(s) for s, _, _ in pairs]
        gt = [cvo.upload(t) for _, t, _ in pairs]
        gp_s, gp_t, _ = make_pairs(1, args.points, seed0=args.eval_seed0)[0]
        hs, ht = cvo.upload(gp_s), cvo.upload(gp_t)
        T24 = []
        for R in CvoGPU.rotation_grid(1):
            T = np.eye(4)
            T[:3, :3] = R.T                   # internal pose of grid rotation R
            T24.append(T)
        legs = {"pairs": (gs, gt, [np.eye(4)] * len(gs)), "hypotheses": ([hs] * len(T24), [ht] * len(T24), T24)}
        res, out_legs = {}, {}
        for name, (S, Tt, inits) in legs.items():
            def batched():
                res["b"] = cvo.align_batch(S, Tt, inits)

            def one_by_one():
                res["s"] = [cvo.align_batch([a], [b], [T]) for a, b, T in zip(S, Tt, inits)]
            sec_b = timed(batched)
            sec_s = timed(one_by_one)
            Tb, _, itb, _ = res["b"]
            same = all(np.allclose(Tb[k], r[0][0], atol=1e-6) and int(itb[k]) == int(r[2][0])
                       for k, r in enumerate(res["s"]))
            out_legs[name] = {"registrations": len(S), "batched_s": round(sec_b, 4), "one_by_one_s": round(sec_s, 4),
                              "speedup": round(sec_s / sec_b, 3), "mean_iters": float(np.mean(itb)),
                              "max_iters": int(np.max(itb)), "identical_results": bool(same)}
        out.update({"metric": "registrations/s, one persistent batch against one call per registration",
                    "unit": "registrations/s", "value": round(len(gs) / out_legs["pairs"]["batched_s"], 4),
                    "legs": out_legs,
                    "config": {"pairs_points": sizes, "hypotheses_points": args.points, "params": "color.yaml",
                               "hypotheses": "24-rotation grid, one global pair", "timing": "host clock, synchronised"}})
    elif args.component == "align":
        # the refinement stage of the learned pipeline on its own: one batched align of
        # --pairs global pairs, each started 5 deg / 10 cm from its ground truth, from
        # ell = --refine-ell (the workload whose association kernel the profiles capture)
        p = CvoParams(params_path("color"))
        p.ell_init = args.refine_ell if args.refine_ell > 0 else p.ell_init
        if args.max_iter > 0:
            p.MAX_ITER = args.max_iter
        cvo = CvoGPU(params=p)
        pairs = make_pairs(args.pairs, args.points)
        gs = [cvo.upload(s) for s, _, _ in pairs]
        gt = [cvo.upload(t) for _, t, _ in pairs]
        dT = scenes.make_T(scenes.rot_axis_angle([0.3, 1.0, 0.2], np.radians(5.0)), [0.1, 0.0, 0.0])
        inits = [np.asarray(T_gt, np.float64) @ dT for _, _, T_gt in pairs]
        res = {}

        def run():
            res["r"] = cvo.align_batch(gs, gt, inits)
        sec = timed(run)
        its = res["r"][2]
        out.update({"metric": "batched refinement registrations/s (%d pairs x %d points)" % (args.pairs, args.points),
                    "unit": "registrations/s", "value": round(args.pairs / sec, 4), "ms_per_call": round(sec * 1000, 3),
                    "iterations": [int(i) for i in its],
                    "config": {"pairs": args.pairs, "points_per_cloud": args.points, "params": "color.yaml",
                               "ell_init": p.ell_init, "max_iter": p.MAX_ITER, "start": "ground truth x (5 deg, 10 cm)"}})
    elif args.component == "proposal":
        from oracle import proposal as op
        from rkhs_ba_gb300.proposal import ProposalNet, ScenePool
        cvo = CvoGPU(params=CvoParams(params_path("color")))
        pool = ScenePool(*ScenePool.generate(64, 2048, seed0=1_000_000))
        net = ProposalNet(cvo, points_per_cloud=512, seed=0)
        net.set_gemm(1 if args.gemm == "mma" else 0)
        B, P = 64, 512
        rng = np.random.default_rng(0)
        batches = [(rng.integers(0, pool.n_scenes, size=B), np.stack([scenes.random_motion(rng) for _ in range(B)]),
                    int(rng.integers(0, 2 ** 32))) for _ in range(args.warmup + args.steps)]
        it = iter(batches)

        def step():
            sc, T, seed = next(it)
            net.train_step(pool, sc, T, 1e-3, seed)
        sec = timed(step)
        pairs = make_pairs(args.pairs, args.points)
        gs = [cvo.upload(a) for a, _, _ in pairs]
        gt = [cvo.upload(b) for _, b, _ in pairs]
        sec_inf = timed(lambda: net.hypotheses(gs, gt))
        rows = 2 * B * P
        enc = op.IN * op.H1 + op.H1 * op.H2
        head = op.HEAD * op.H3 + op.H3 * op.OUT
        # forward 2 m n k per product; backward: the input gradient and the weight gradient
        # of every layer except the first layer's input gradient
        fwd = 2.0 * (rows * enc + B * head)
        bwd = 2.0 * (rows * (2 * enc - op.IN * op.H1) + 2 * B * head)
        peak = None
        pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
        if os.path.exists(pk):
            with open(pk) as fh:
                peak = float(json.load(fh)["bf16_tflops"])
        tflops = (fwd + bwd) / sec / 1e12
        out.update({"metric": "proposal training pairs/s (64 pairs x 2 clouds x 512 points per step)",
                    "unit": "pairs/s", "value": round(B / sec, 2), "ms_per_step": round(sec * 1000, 3),
                    "dtype": "bf16 operands, f32 accumulation",
                    "inference_ms": round(sec_inf * 1000, 3),
                    "inference_config": {"pairs": args.pairs, "points_per_cloud": args.points},
                    "flops_per_step": fwd + bwd,
                    "roofline": {"bound": "tensor", "achieved": round(tflops, 3), "peak": peak, "unit": "TFLOP/s",
                                 "frac": round(tflops / peak, 6) if peak else None,
                                 "note": "kernel launches and host synchronisation dominate: each product is small"},
                    "config": {"batch": B, "points_per_cloud": P, "pool_scenes": 64,
                               "gemm": "tcgen05 (TMEM accumulators)" if args.gemm != "mma" else "mma.sync"}})
    print(json.dumps(out))


def run_reference(args):
    """The reference arm: the workload's learned global registration on the host cores
    (CpuLearned), on the GPU arm's config, metric and unit.

    value: registrations/s of --ref-full-pairs complete registrations of the workload's
    first pairs, each timed end to end (network, ranking, refinement to convergence,
    judge).  The --warmup and --steps steps are bounded samples of the 8-pair step: pair
    (step mod 8) goes through the whole pipeline with its refinement limited to
    --ref-sample-iters iterations; ms_per_step is their measured wall time, and the
    cos-angles/s and align iterations/s they measure are the like-for-like units the GPU
    arm also reports."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    t_all = time.perf_counter()
    pairs = make_pairs(args.pairs, args.points, seed0=1000)
    cl = CpuLearned(args)
    full = []
    for k in range(max(1, min(args.ref_full_pairs, len(pairs)))):
        t0 = time.perf_counter()
        _, it, ph = cl.register(pairs[k])
        full.append({"pair": k, "seconds": round(time.perf_counter() - t0, 3), "iterations": it,
                     "phase_s": {n: round(v, 3) for n, v in ph.items()}})
    value = len(full) / sum(f["seconds"] for f in full)
    S = max(1, args.ref_sample_iters)
    for k in range(max(0, args.warmup)):
        cl.register(pairs[k % len(pairs)], max_iter=S)
    cos_s, iter_s, iters, step_s = 0.0, 0.0, 0, []
    for k in range(max(1, args.steps)):
        t0 = time.perf_counter()
        _, it, t = cl.register(pairs[k % len(pairs)], max_iter=S)
        step_s.append(time.perf_counter() - t0)
        cos_s += t["rank"] + t["judge"]
        iter_s += t["refine"]
        iters += it
    out = {"metric": METRIC, "value": round(value, 6), "unit": UNIT, "impl": "reference", "n_gpus": 1,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1000.0 * float(np.mean(step_s)), 3),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic (seeded scenes)", "config": workload_config(args),
           "full_registrations": full,
           "measured": {"cos_angles_per_s": round(9 * len(step_s) / cos_s, 4),
                        "align_iterations_per_s": round(iters / iter_s, 4),
                        "note": "from the timed sample steps: 9 CPU cos-angles and %d align iterations (from ell "
                                "%.2f, the most expensive part of a refinement) per step" % (S, cl.refine_ell)},
           "cpu_baseline": {"kind": "port", "cores": cl.cores, "value": round(value, 6), "unit": UNIT,
                            "sample": "%d complete registrations of the workload's first pairs on all host threads "
                                      "(value); per step one of the 8 pairs through network, ranking, %d align "
                                      "iterations and judge (ms_per_step)" % (len(full), S)},
           "e2e": {"value": round(value, 6), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "wall_s": round(time.perf_counter() - t_all, 3)}
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--pairs", type=int, default=8)
    ap.add_argument("--points", type=int, default=50000)
    ap.add_argument("--cpu-iters", type=int, default=2, help="oracle iterations timed by --component adaptive")
    ap.add_argument("--ref-sample-iters", type=int, default=2,
                    help="align iterations of the refinement in each step of the reference arm's sample")
    ap.add_argument("--ref-full-pairs", type=int, default=2,
                    help="complete CPU registrations the reference arm's value is measured on")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--refine", type=int, default=1, help="hypotheses refined per pair (1..8)")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default association cell size")
    ap.add_argument("--refine-ell", type=float, default=0.4,
                    help="lengthscale the hypotheses' refinement starts at (0: ell_init of the yaml)")
    ap.add_argument("--fallback-cos", type=float, default=0.0,
                    help="judged cos-angle below which a pair falls back to the grid")
    ap.add_argument("--train-scenes", type=int, default=600)
    ap.add_argument("--train-steps", type=int, default=3000)
    ap.add_argument("--proposal-weights", default="", help="load the proposal network instead of training it")
    ap.add_argument("--save-proposal", default="", help="save the trained proposal network (.npy)")
    ap.add_argument("--grid-steps", type=int, default=1, help="timed steps of the plain grid")
    ap.add_argument("--all24-pairs", type=int, default=2, help="pairs registered by the all-24 grid")
    ap.add_argument("--max-iter", type=int, default=0, help="override MAX_ITER (profiling runs only)")
    ap.add_argument("--eval-pairs", type=int, default=200, help="held-out pairs of --component global-eval")
    ap.add_argument("--eval-seed0", type=int, default=5000, help="first seed of --component global-eval's pairs")
    ap.add_argument("--gemm", default="tcgen05", choices=["tcgen05", "mma"],
                    help="matrix-product kernel of --component proposal")
    ap.add_argument("--component", default="",
                    choices=["", "irls", "aniso", "frontend", "proposal", "adaptive", "global-eval", "batching",
                             "align"],
                    help="time one component instead of the main workload")
    args = ap.parse_args()
    from rkhs_ba_gb300 import _build
    _build.build()
    if args.component:
        run_component(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
