"""Benchmark: GPS-aided bundle adjustment solve throughput on one GB300.

Workload (default ``single500``): one synthetic lawnmower survey with 500
cameras, 400k points and ~3M observations (seeded, see
aerial-3d-model_gb300/stitch_ba/survey.py), Cauchy loss at 1 px, GPS priors,
refine_intrinsics, max_iter 60 (the reference's own test call, ba.rs:482).
A step is one full ``bundle_adjust`` solve of that survey from its perturbed
initial state.

* ``value``  — solves/s with the problem already resident in HBM
  (``ba_context_solve``: structure build, every LM iteration, PCG, updates),
  timed with CUDA events on the solver's stream, L2 flushed between steps.
* ``e2e``    — solves/s through the reference-facing C ABI ``ba_solve`` with
  host (pinned) buffers: H2D of the problem, the solve and D2H of the state
  are inside the timed region.
* ``forms``  — FP64 plain form (the reference's block-Jacobi PCG, 400
  iterations), FP32/FP64 mixed form (two-level PCG: block Jacobi plus the
  similarity motions of camera groups, 40 iterations; 60 above 1000 cameras
  per model; stop after two consecutive small decreases) and, as an
  ablation, the mixed form with the reference's block-Jacobi PCG alone (200
  iterations), side by side: final cost of each,
  relative difference from the FP64 form, and the error of every result
  (centres, rotations, intrinsics, points) against the FP64 form and against
  the CPU solver.  The mixed form is the headline when it reaches the FP64
  final cost (for a batch: every model does).
* ``parity_vs_cpu`` — the FP64 GPU solve against the CPU solver's solve of
  the same survey (single-model workloads): iterations, accept sequence,
  per-iteration trial cost, final cost and every result.
* ``roofline`` — the dominant kernel phase (by device time, from the
  solver's own CUDA-event phase timing) against measured HBM bandwidth.
* ``cpu_baseline`` — the oracle (a CPU restatement of the reference solver,
  same data structures, OpenMP on all host cores): complete solves, timed
  end to end (the survey; for a batch, whole models in index order until
  about 20 s of CPU time, scaled by observations).

``--impl reference`` times that CPU solver alone as the reference arm: every
timed step is one complete solve of the workload (a batch: complete solves of
a fixed sample of its models, scaled by observations); warm-up steps run one
LM iteration each.

Multi-GPU (torchrun, one process per GPU): a single survey runs as
independent replicas (each rank solves its own seeded survey, weak scaling);
the batched workload is partitioned, each rank solving a disjoint subset of
the same models balanced by observations (strong scaling), with no
collective on the data path.

``--stage triangulate|ransac|pair_fits|summary`` measures one of the sparse
stage's steps around the solve on the same survey instead (one JSON line with
the GPU call's throughput through its C ABI entry point, host buffers in and
out, against the oracle on all host cores on a bounded sample, and the
agreement of the two on that sample):
  triangulate — one round's triangulation + gating of every track (tracks/s);
  ransac      — fundamental-matrix RANSAC of every photo pair's putative
                matches, 600 hypotheses, 1.5 px (pairs/s);
  pair_fits   — median Sampson error of every pair under the poses (pairs/s);
  summary     — neighbours, depth ranges and f32 points of the problem
                (observations/s).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "aerial-3d-model_gb300"))

import numpy as np  # noqa: E402

METRIC = "BA solve time & kernel HBM GB/s, mixed vs FP64 GPU at equal final cost"
UNIT = "solves/s"
SIGMA_PX = 1.0
MAX_ITER = 60
# The mixed form solves each LM step with the two-level preconditioner (block
# Jacobi plus the similarity motions of camera groups) and caps its FP32 PCG
# at this many iterations (the FP64 form keeps the reference's block-Jacobi
# PCG and its 400): 40 up to 1000 cameras per model, 60 above, where the
# groups (at most 27 per model) get larger and the coarse space weaker.
MIXED_PCG_ITERS = 40
MIXED_PCG_ITERS_LARGE = 60
MIXED_LARGE_CAMS = 1000
# The mixed forms stop after two consecutive accepted steps with a relative
# decrease below 1e-6 (the reference's rule, ba.rs:372-374, stops after one):
# an FP32 inner solve can give one small decrease before the minimum.
# Measured with 40 PCG iterations: the 500-camera survey takes one LM
# iteration more (12 -> 13) and ends 2.1e-6 below the FP64 form; on the
# 64-model batch 7 models ended up to 1.1e-5 above their FP64 cost with one
# step, none (at most +8.4e-7) with two, at 7% more time.
MIXED_STOP_PATIENCE = 2
# End game of the mixed form: once an accepted step decreases a model's cost by
# less than 1e-5 (relative), its PCG cap rises to 100 for the rest of the solve
# (an inexact-Newton forcing rule: tighter inner solves as the outer iteration
# converges).  Measured (median of two solves, GB300): without it the 77-camera
# survey stops 5.5e-6 above its FP64 cost (11.7 ms) and one of the 64 batched
# models 1.07e-6 above; with it every model of the 77- and 500-camera surveys,
# the 2000-camera survey and the batch ends at or below its FP64 cost, at
# 21.4 / 35.2 / 196 / 305 ms against 11.7 / 32.8 / 188 / 273 ms without.
MIXED_END_PCG_ITERS = 100
MIXED_END_REL = 1e-5
# Ablation: the mixed form's FP32 records, Schur sums and PCG vectors with the
# reference's block-Jacobi preconditioner alone, capped at 200 PCG iterations.
ABLATION_PCG_ITERS = 200
# CPU sample of a batched workload: whole models until this much CPU time.
CPU_SAMPLE_S = 20.0
# Per LM iteration, algorithmic bytes of each phase, written as a function of
# the problem sizes and the storage width s (8 FP64 / 4 FP32): reads and writes
# each kernel must make at minimum.
#   point : obs (cam u32, pt u32, uv 2 f64) + params (cams 12 f64, points 3 f64)
#           → lin record 28 s + Z 18 s + gsub 9 s per obs, L 6 s + zv 3 s per point
#   camera: read lin 28 s + gsub 9 s + index 4 per obs → 63 f64 per camera
#   schur : per pair contribution 2 entries read (18 s each) + 8 B pair → 36 s per sub-segment
#   pcg   : per product S (36 s per block + col 4 B) + p gather 6 s per block
#           + vectors (x, r, z, p, q: ~10 vector passes of 6 s per row) + pre 36·8 per row


def algorithmic_bytes(phase: str, sz: dict, s: int, pcg_iters: float = 0.0) -> float:
    no, np_, nc, nz, nb = sz["n_obs"], sz["n_points"], sz["n_cams"], sz["nz_blocks"], sz["nb"]
    npairs, nsub = sz["pairs"], sz["subsegments"]
    if phase == "point":
        return no * (4 + 4 + 16 + (28 + 18 + 9) * s) + nc * 96 + np_ * (24 + 9 * s)
    if phase == "camera":
        return no * (4 + 4 + 37 * s) + nc * 63 * 8
    if phase == "schur":
        return npairs * (8 + 36 * s) + nsub * 36 * s
    if phase == "pcg":
        per = nz * (36 * s + 4 + 6 * s) + nb * (10 * 6 * s + 36 * 8)
        return per * pcg_iters
    return 0.0


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self):
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            p = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                  "-lms", "200", "-i", os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0]],
                                 stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            return
        while not self._stop.is_set():
            line = p.stdout.readline()
            if not line:
                break
            self.samples.append([x.strip() for x in line.split(",")])
        p.terminate()
        try:
            p.wait(timeout=5)
        except Exception:
            p.kill()

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        try:
            sm = [float(s[0]) for s in self.samples]
            mx = float(self.samples[0][1])
        except ValueError:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unparsed"]}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4)
                          if len(s) > 3 + i and s[3 + i].lower().startswith("active")})
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(sm)}


# --matrix-free: the mixed form applies S without forming it ("recompute" with
# --jtj-recompute: J^T J recomputed in the PCG, no Schur factors stored)
MIXED_MATRIX_FREE = False
MIXED_PCG_CAP = MIXED_PCG_ITERS  # set per workload by set_mixed_cap


def set_mixed_cap(ps):
    global MIXED_PCG_CAP
    big = max(p.n_cams for p in ps) > MIXED_LARGE_CAMS
    MIXED_PCG_CAP = MIXED_PCG_ITERS_LARGE if big else MIXED_PCG_ITERS


def form_options(form: str, **kw):
    """Options of a measured form.  The PCG layout is picked by the solver's
    autotuner on the first (warm-up) solve of the form and reused by the
    timed solves.  Forms: "fp64", "mixed" (two-level PCG), "mixed_bj" (the
    mixed form with block-Jacobi PCG alone: the ablation)."""
    from stitch_ba import Options
    kw.setdefault("autotune", True)
    if form != "fp64":
        kw.setdefault("point_kernel", POINT_KERNEL)
        kw.setdefault("pcg_kernel", PCG_KERNEL)
    if form == "mixed":
        mf = ("recompute" if MIXED_MATRIX_FREE == "recompute"
              else "matrix_free" if MIXED_MATRIX_FREE else "auto")
        kw.setdefault("coarse", not MIXED_MATRIX_FREE)
        kw.setdefault("stop_patience", MIXED_STOP_PATIENCE)
        if MIXED_END_PCG_ITERS > 0:
            kw.setdefault("pcg_end_max_iter", max(MIXED_END_PCG_ITERS, MIXED_PCG_CAP))
            kw.setdefault("pcg_end_rel", MIXED_END_REL)
        return Options(precision="mixed", pcg_max_iter=MIXED_PCG_CAP, matrix_free=mf, **kw)
    if form == "mixed_bj":
        kw.setdefault("stop_patience", MIXED_STOP_PATIENCE)
        return Options(precision="mixed", pcg_max_iter=ABLATION_PCG_ITERS, coarse=False, **kw)
    return Options(precision="fp64", **kw)


def max_over_ranks(x: float, ws: int, device: str = "cuda") -> float:
    """Timing of the slowest rank."""
    if ws <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x: float, ws: int, device: str = "cuda") -> float:
    if ws <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def rank_seed(seed: int, rank: int) -> int:
    """Each replica of a single-survey workload solves its own survey (weak
    scaling: fixed work per GPU)."""
    return seed + rank


def partition_models(sizes, ws: int):
    """Disjoint subsets of model indices, one per rank, balanced by `sizes`
    (observations): largest model first, each to the least-loaded rank (ties
    to the lower rank).  Every model is in exactly one subset; each subset is
    in index order."""
    parts = [[] for _ in range(ws)]
    load = [0] * ws
    for i in sorted(range(len(sizes)), key=lambda k: (-sizes[k], k)):
        r = min(range(ws), key=lambda k: (load[k], k))
        parts[r].append(i)
        load[r] += sizes[i]
    return [sorted(p) for p in parts]


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    return ws, rank


# Batched workload: 64 independent lawnmower models of uneven size (cameras
# ~U[20, 800], 500-1000 points per camera), solved together.
BATCH_MODELS = 64


# Points of a single survey (0: the workload's own count).  A smaller count
# keeps the camera network, hence the reduced system and the PCG kernels, of
# the full workload: the small case for full ncu captures of those kernels.
N_POINTS = 0
# Mixed forms' per-observation passes ("auto": the autotuner's choice).  Under
# ncu the autotuner's timings are distorted (every launch is serialised and
# instrumented, which penalises the three-kernel variant), so the launch-list
# command fixes the variant the plain run chose.
POINT_KERNEL = "auto"
# Mixed forms' PCG layout ("auto": the autotuner's choice; same caveat).
PCG_KERNEL = "auto"


def make_workload(name: str, seed: int):
    """A list of problems: one for a single survey, BATCH_MODELS for batch64."""
    from stitch_ba import survey
    if name == "batch64":
        return [m[0] for m in survey.batched_models(BATCH_MODELS, seed=seed)]
    kw = {"n_points": N_POINTS} if N_POINTS > 0 else {}
    p, truth = survey.generate(name, seed=seed, **kw)
    return [p]


def rank_workload(name: str, seed: int, ws: int, rank: int):
    """(problems of this rank, their indices in the workload or None,
    models solved by all ranks together).  The batch is partitioned across
    ranks; a single survey is replicated with a per-rank seed."""
    if name == "batch64":
        ps = make_workload(name, seed)
        part = partition_models([p.n_obs for p in ps], ws)[rank]
        return [ps[i] for i in part], part, len(ps)
    return make_workload(name, rank_seed(seed, rank)), None, ws


def totals(ps):
    return dict(n_cams=sum(q.n_cams for q in ps), n_points=sum(q.n_points for q in ps),
                n_obs=sum(q.n_obs for q in ps))


def pin_problem(p):
    """Copy a Problem's arrays into page-locked host memory (for e2e)."""
    import torch
    from stitch_ba import Problem

    def pin(a):
        return torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()

    return Problem(intr=pin(p.intr), rot=pin(p.rot), center=pin(p.center),
                   cam_group=pin(p.cam_group), points=pin(p.points), obs_cam=pin(p.obs_cam),
                   obs_pt=pin(p.obs_pt), obs_uv=pin(p.obs_uv), prior_mask=pin(p.prior_mask),
                   prior=pin(p.prior), refine_intrinsics=p.refine_intrinsics)


def reaches(cost: float, ref: float) -> bool:
    """Equal final cost: within 1e-6 relative of the reference cost, or below."""
    return cost <= ref * (1.0 + 1e-6)


def gpu_arm(args, ws, rank):
    import torch
    import stitch_ba
    from stitch_ba import compare, native

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    native.load()
    ps, part, units_all = rank_workload(args.workload, args.seed, ws, rank)
    set_mixed_cap(ps)
    nmod = len(ps)
    tot = totals(ps)
    stream = torch.cuda.current_stream()
    flush = torch.empty(int(256 * 2**20) // 4, dtype=torch.float32, device="cuda")

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    forms = {}
    chosen = args.precision
    names = ["fp64", "mixed", "mixed_bj"] if args.precision == "both" else [args.precision]
    if args.no_ablation and "mixed_bj" in names:
        names.remove("mixed_bj")
    profile_info = {}
    infos_by_form = {}
    solutions = {}
    with stitch_ba.Context(device=dev, stream=stream.cuda_stream) as ctx:
        ctx.upload(ps)
        for form in names:
            opts = form_options(form)
            for _ in range(args.warmup):
                ctx.solve(args.max_iter, SIGMA_PX, opts)
            torch.cuda.synchronize()
            times = []
            info = None
            with ClockSampler() as clk:
                barrier()
                for _ in range(args.steps):
                    flush.zero_()
                    a = torch.cuda.Event(enable_timing=True)
                    b = torch.cuda.Event(enable_timing=True)
                    a.record(stream)
                    infos = ctx.solve(args.max_iter, SIGMA_PX, opts)
                    info = infos[0]
                    b.record(stream)
                    b.synchronize()
                    times.append(a.elapsed_time(b))
                barrier()
            ms = max_over_ranks(float(np.sum(times)) / len(times), ws)
            sol = [q.copy() for q in ps]
            ctx.download(sol)
            solutions[form] = sol
            forms[form] = dict(ms_per_solve=ms, final_cost=sum(i.final_cost for i in infos),
                               initial_cost=sum(i.initial_cost for i in infos),
                               iterations=max(i.iterations for i in infos),
                               pcg_iterations=sum(i.pcg_iterations for i in infos),
                               final_rms=info.final_rms,
                               kernel_launches=sum(i.kernel_launches for i in infos[:1]),
                               clocks=clk.summary())
            forms[form]["model_final_costs"] = [i.final_cost for i in infos] if nmod > 1 else None
            forms[form]["model_iterations"] = [i.iterations for i in infos] if nmod > 1 else None
            # one profiled solve with the per-iteration log (phase timing; not
            # part of the timed region)
            prof = ctx.solve(args.max_iter, SIGMA_PX, form_options(form, profile=True),
                             log=(nmod == 1))[0]
            profile_info[form] = prof
            infos_by_form[form] = infos
            forms[form]["pcg_kernel"] = prof.pcg_kernel
            forms[form]["pcg_ctas"] = int(prof.pcg_ctas)
            forms[form]["pcg_threads_per_cta"] = int(prof.pcg_threads)
            forms[form]["pcg_autotuned_us_per_iter"] = prof.pcg_tuned_us
            forms[form]["schur_sub_len"] = int(prof.schur_sub_len)
            forms[form]["schur_autotuned_us"] = prof.schur_tuned_us
            forms[form]["device_bytes"] = int(prof.device_bytes)
            forms[form]["pcg_max_iter"] = opts.pcg_max_iter
            forms[form]["pcg_end_max_iter"] = opts.pcg_end_max_iter
            forms[form]["coarse_dim"] = int(prof.coarse_dim)
            forms[form]["graph"] = bool(info.graph)
    if "fp64" in forms:
        f64 = forms["fp64"]["final_cost"]
        for form in [f for f in forms if f != "fp64"]:
            F = forms[form]
            F["rel_final_cost_vs_fp64"] = (F["final_cost"] - f64) / abs(f64)
            F["speedup_vs_fp64"] = forms["fp64"]["ms_per_solve"] / F["ms_per_solve"]
            F["error_vs_fp64"] = [compare.state_errors(a, b) for a, b in
                                  zip(solutions[form], solutions["fp64"])][0] if nmod == 1 else None
            if nmod > 1:
                a, b = forms["fp64"]["model_final_costs"], F["model_final_costs"]
                miss = [[int(part[k]) if part else k, (y - x) / abs(x)]
                        for k, (x, y) in enumerate(zip(a, b)) if not reaches(y, x)]
                F["models_reaching_fp64_cost"] = nmod - len(miss)
                F["models_missing_fp64_cost"] = miss  # [model index, relative difference]
                F["reaches_fp64_final_cost"] = not miss
            else:
                F["reaches_fp64_final_cost"] = bool(reaches(F["final_cost"], f64))
            # First LM iteration whose accepted cost is within 1e-6 of the FP64
            # final cost.
            log = profile_info[form]
            hit = None
            for i in range(int(log.iterations) if nmod == 1 else 0):
                if log.accepted[i] and reaches(log.new_cost[i], f64):
                    hit = i
                    break
            if hit is not None:
                F["iteration_reaching_fp64_cost"] = hit + 1
                F["ms_to_fp64_cost_est"] = F["ms_per_solve"] * (hit + 1) / max(int(log.iterations), 1)
        # Per LM iteration of the profiled solve: trial cost relative to the
        # FP64 final cost, accepted (1/0), PCG iterations.
        for form in forms:
            lg = profile_info[form]
            if nmod == 1 and lg.new_cost is not None:
                forms[form]["lm_trace"] = [
                    [float("%.3g" % (lg.new_cost[i] / f64 - 1.0)), int(lg.accepted[i]),
                     int(lg.pcg_iters[i])] for i in range(int(lg.iterations))]
        if "mixed" in forms:
            chosen = "mixed" if forms["mixed"]["reaches_fp64_final_cost"] else "fp64"
            forms["chosen"] = chosen
    head = forms[chosen]

    # End to end through the reference-facing C ABI (host buffers, H2D + D2H inside).
    pps = [pin_problem(q) for q in ps]
    inits = [q.state() for q in pps]
    e2e_times = []
    e2e_info = None
    opts = form_options(chosen, stream=stream.cuda_stream)
    for i in range(args.warmup + args.steps):
        for q, st0 in zip(pps, inits):
            q.set_state(st0)
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        if nmod == 1:
            st, e2e_info = stitch_ba.bundle_adjust(pps[0], args.max_iter, SIGMA_PX, opts,
                                                   return_info=True)
        else:
            e2e_info = stitch_ba.bundle_adjust_batch(pps, args.max_iter, SIGMA_PX, opts)[0]
        torch.cuda.synchronize()
        if i >= args.warmup:
            e2e_times.append(time.perf_counter() - t0)
    e2e_s = max_over_ranks(float(np.mean(e2e_times)), ws)
    h2d = sum_over_ranks(float(e2e_info.h2d_bytes), ws)
    d2h = sum_over_ranks(float(e2e_info.d2h_bytes), ws)

    if rank != 0:
        return None
    # Roofline of the dominant phase.
    prof = profile_info[chosen]
    phases = {k: v for k, v in prof.phases.items() if k != "setup"}
    dom = max(phases, key=lambda k: phases[k][0])
    dom_ms, dom_n = phases[dom]
    zs = prof.sizes
    sz = dict(n_obs=tot["n_obs"], n_points=tot["n_points"], n_cams=tot["n_cams"], nb=zs["blocks"],
              nz_blocks=zs["nonzero_blocks"], pairs=zs["schur_pairs"],
              subsegments=zs["schur_pairs"] // max(int(prof.schur_sub_len), 1)
              + (zs["nonzero_blocks"] + zs["blocks"]) // 2)
    s = 8 if chosen == "fp64" else 4
    per_launch_ms = dom_ms / max(dom_n, 1)
    if dom == "pcg":
        bytes_per_launch = algorithmic_bytes("pcg", sz, s, prof.pcg_iterations / max(dom_n, 1))
    else:
        bytes_per_launch = algorithmic_bytes(dom, sz, s)
    peak, peak_kind = load_peaks()
    achieved = bytes_per_launch / (per_launch_ms * 1e-3) / 1e9 if per_launch_ms > 0 else 0.0
    traffic = None
    tr_path = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tr_path):
        try:
            with open(tr_path) as f:
                traffic = json.load(f).get(f"{args.workload}:{chosen}:{dom}")
        except Exception:
            traffic = None

    value = units_all * 1000.0 / head["ms_per_solve"]
    partitioned = part is not None
    out = {
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": head["ms_per_solve"],
        "higher_is_better": True,
        "scaling": "strong" if partitioned else "weak",
        "vs_baseline": None,
        "dtype": "f64" if chosen == "fp64" else "f32+f64",
        "data": "synthetic (seeded survey generator, reference camera model)",
        "config": {"workload": args.workload, "models": units_all if partitioned else nmod,
                   "cameras": tot["n_cams"], "points": tot["n_points"],
                   "observations": tot["n_obs"], "max_iter": args.max_iter,
                   "sigma_px": SIGMA_PX, "loss": "cauchy", "precision": chosen,
                   "parallelism": (f"models partitioned over {ws} ranks" if partitioned
                                   else f"replicas{ws}"),
                   "l2": "flushed between steps (256 MiB write)"},
        "forms": {k: {kk: vv for kk, vv in v.items() if kk != "clocks"} if isinstance(v, dict) else v
                  for k, v in forms.items()},
        "e2e": {"value": units_all / e2e_s, "unit": UNIT,
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "ms_per_step": e2e_s * 1000.0},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                     "peak_source": peak_kind, "bytes_per_launch": bytes_per_launch,
                     "ms_per_launch": per_launch_ms,
                     "phases_ms_per_solve": {
                         f: {k: round(v[0], 3) for k, v in pi.phases.items()}
                         for f, pi in profile_info.items()}},
        "clocks": head["clocks"],
        "gpu_launches": int(head["kernel_launches"]) * args.steps,
    }
    if partitioned:
        out["config"]["rank0_models"] = [int(i) for i in part]
    if not args.no_cpu and ws == 1:
        cpu = cpu_solves(ps, args.max_iter, budget_s=CPU_SAMPLE_S)
        out["cpu_baseline"] = cpu["baseline"]
        if nmod == 1 and "fp64" in solutions:
            out["parity_vs_cpu"] = parity_record(profile_info["fp64"], forms["fp64"],
                                                 solutions["fp64"][0], cpu["results"][0],
                                                 cpu["solutions"][0])
            for form in forms:
                if form in solutions and form != "fp64":
                    forms_out = out["forms"][form]
                    forms_out["error_vs_cpu"] = compare.state_errors(solutions[form][0],
                                                                     cpu["solutions"][0])
                    forms_out["rel_final_cost_vs_cpu"] = (
                        (forms[form]["final_cost"] - cpu["results"][0].final_cost)
                        / abs(cpu["results"][0].final_cost))
    return out


def parity_record(log, fp64_form, gpu_sol, cpu_res, cpu_sol):
    """FP64 GPU solve against the CPU solver's solve of the same problem:
    iterations, accept sequence, per-iteration trial cost, final cost and
    the per-result differences (ba.rs:198-391)."""
    from stitch_ba import compare
    n = min(int(log.iterations), int(cpu_res.iterations))
    rel = (np.abs(log.new_cost[:n] - cpu_res.new_cost[:n]) / np.abs(cpu_res.new_cost[:n])
           if n else np.zeros(0))
    acc = np.asarray(log.accepted[:n], bool)
    return {
        "iterations_gpu": int(log.iterations), "iterations_cpu": int(cpu_res.iterations),
        "accept_sequence_equal": bool(np.array_equal(acc, np.asarray(cpu_res.accepted[:n], bool))),
        "trial_cost_rel_max": float(rel.max()) if n else 0.0,
        "trial_cost_rel_max_accepted": float(rel[acc].max()) if acc.any() else 0.0,
        "trial_cost_rel": [float("%.2g" % v) for v in rel],
        "final_cost_rel": (fp64_form["final_cost"] - cpu_res.final_cost) / abs(cpu_res.final_cost),
        "state": compare.state_errors(gpu_sol, cpu_sol),
    }


def cpu_solves(ps, max_iter: int, budget_s: float = CPU_SAMPLE_S):
    """Complete oracle solves (CPU restatement of the reference, OpenMP on all
    host cores) of whole models: the survey, or for a batch the models in
    index order until `budget_s` of CPU time, scaled to the whole batch by
    observations.  Returns the baseline line, and the results and solved
    states of the models solved."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import ba_oracle
    ba_oracle.build()
    threads = os.cpu_count() or 1
    results, sols = [], []
    t_all = 0.0
    obs_done = 0
    for p in ps:
        q = p.copy()
        t0 = time.perf_counter()
        r = ba_oracle.bundle_adjust(q, max_iter, SIGMA_PX, n_threads=threads)
        t_all += time.perf_counter() - t0
        obs_done += p.n_obs
        results.append(r)
        sols.append(q)
        if t_all >= budget_s:
            break
    total_obs = sum(p.n_obs for p in ps)
    est = t_all * total_obs / max(obs_done, 1)
    k = len(results)
    what = ("one complete solve of the survey" if len(ps) == 1 else
            f"complete solves of {k} of {len(ps)} models (models 0..{k - 1}), scaled by observations")
    # Per-phase wall time of the CPU solves (seconds, summed over the models
    # solved): linearise / point systems / assembly / Schur / PCG /
    # back-substitution / cost, as the oracle times them.
    phases = {}
    for r in results:
        for k, v in (r.phases or {}).items():
            phases[k] = phases.get(k, 0.0) + float(v)
    return {"baseline": {"value": len(ps) / est, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{what} ({t_all:.1f} s, {max(r.iterations for r in results)} "
                                   f"LM iterations max)",
                         "iterations": [int(r.iterations) for r in results],
                         "phases_s": {k: round(v, 3) for k, v in phases.items()}},
            "results": results, "solutions": sols}


def reference_arm(args, ws, rank):
    """CPU reference solver (oracle port, all host cores), same workload and
    unit.  Warm-up steps run one LM iteration of the first model; every
    timed step is a complete solve of the survey (a batch: complete solves of
    a fixed sample of its models — chosen by the first step, about
    CPU_SAMPLE_S of work — scaled to the batch by observations)."""
    if rank != 0:
        return None
    ps = make_workload(args.workload, args.seed)
    tot = totals(ps)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import ba_oracle
    ba_oracle.build()
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        ba_oracle.bundle_adjust(ps[0].copy(), 1, SIGMA_PX, n_threads=threads)
    times = []
    sample = None
    last = None
    for _ in range(args.steps):
        t0 = time.perf_counter()
        res = []
        for i, p in enumerate(ps if sample is None else ps[:sample]):
            res.append(ba_oracle.bundle_adjust(p.copy(), args.max_iter, SIGMA_PX, n_threads=threads))
            if sample is None and len(ps) > 1 and time.perf_counter() - t0 >= CPU_SAMPLE_S:
                break
        dt = time.perf_counter() - t0
        if sample is None:
            sample = len(res)
        times.append(dt)
        last = res
    obs_sample = sum(p.n_obs for p in ps[:sample])
    per_step = float(np.mean(times)) * tot["n_obs"] / obs_sample
    v = len(ps) / per_step
    r0 = last[0]
    what = ("one complete solve of the survey" if len(ps) == 1 else
            f"complete solves of models 0..{sample - 1} of {len(ps)}, scaled by observations")
    return {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": per_step * 1000.0,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded survey generator, reference camera model)",
        "config": {"workload": args.workload, "models": len(ps), "cameras": tot["n_cams"],
                   "points": tot["n_points"], "observations": tot["n_obs"],
                   "max_iter": args.max_iter, "sigma_px": SIGMA_PX,
                   "loss": "cauchy", "precision": "fp64", "parallelism": "cpu"},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"each step = {what}; warm-up steps = one LM iteration"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "solution": {"iterations": int(r0.iterations), "final_cost": r0.final_cost,
                     "final_rms": r0.final_rms, "accepted": [int(a) for a in r0.accepted],
                     "step_seconds": [round(t, 3) for t in times],
                     # the last step's per-phase wall time, summed over its models
                     "phases_s": {k: round(sum(float((r.phases or {}).get(k, 0.0)) for r in last), 3)
                                  for k in (r0.phases or {})}},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="single500")
    ap.add_argument("--precision", default="both", choices=["both", "fp64", "mixed"])
    ap.add_argument("--max-iter", type=int, default=MAX_ITER)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline and parity legs")
    ap.add_argument("--no-ablation", action="store_true",
                    help="skip the mixed form with block-Jacobi PCG alone")
    ap.add_argument("--stage", default="ba",
                    choices=["ba", "triangulate", "ransac", "pair_fits", "summary"])
    ap.add_argument("--matrix-free", action="store_true",
                    help="mixed form: S p applied from the stored Schur factors, S not formed")
    ap.add_argument("--jtj-recompute", action="store_true",
                    help="mixed form: matrix-free with J^T J recomputed in every PCG product "
                         "from the stored FP32 Jacobians (no Schur factors stored)")
    ap.add_argument("--mixed-patience", type=int, default=0,
                    help="mixed forms: consecutive small decreases before stopping (0: default)")
    ap.add_argument("--mixed-end-iters", type=int, default=-1,
                    help="mixed form: end-game PCG cap (-1: default 100, 0: off)")
    ap.add_argument("--pcg-kernel", default="auto", choices=["auto", "cluster", "cluster_wide"],
                    help="mixed forms: PCG layout (auto: the autotuner's choice; cluster / "
                         "cluster_wide: one cluster per model of 512- / 1024-thread CTAs)")
    ap.add_argument("--point-kernel", default="auto",
                    choices=["auto", "three_pass", "fused128", "fused256"],
                    help="mixed forms: per-observation passes (auto: the autotuner's choice)")
    ap.add_argument("--n-points", type=int, default=0,
                    help="points of a single survey (0: the workload's own); a smaller case "
                         "with the same camera network, for profiling")
    args = ap.parse_args()
    global MIXED_MATRIX_FREE, MIXED_STOP_PATIENCE, MIXED_END_PCG_ITERS, N_POINTS, POINT_KERNEL
    global PCG_KERNEL
    N_POINTS = args.n_points
    POINT_KERNEL = args.point_kernel
    PCG_KERNEL = args.pcg_kernel
    MIXED_MATRIX_FREE = "recompute" if args.jtj_recompute else args.matrix_free
    if args.mixed_patience > 0:
        MIXED_STOP_PATIENCE = args.mixed_patience
    if args.mixed_end_iters >= 0:
        MIXED_END_PCG_ITERS = args.mixed_end_iters
    ws, rank = dist_env()
    if args.stage != "ba":
        out = stage_arm(args, ws, rank)
    elif args.impl == "reference":
        out = reference_arm(args, ws, rank)
    else:
        out = gpu_arm(args, ws, rank)
    if out is not None and rank == 0:
        print(json.dumps(out))


def stage_arm(args, ws, rank):
    """One sparse-stage step on the workload's survey: GPU through the C ABI
    (host arrays in and out, timed with perf_counter around the call, which
    returns after its device-to-host copies), and the oracle on all host
    cores on a bounded sample of the same units."""
    if rank != 0:
        return None
    import stitch_ba
    from stitch_ba import Tracks, native, survey
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import ba_oracle as O
    O.build()
    native.load()
    p, _ = survey.generate(args.workload, seed=args.seed)
    threads = os.cpu_count() or 1
    cnt = np.bincount(p.obs_pt, minlength=p.n_points)
    tp = np.concatenate([[0], np.cumsum(cnt)]).astype(np.uint32)
    if args.stage == "triangulate":
        tr = Tracks(tp, p.obs_cam, p.obs_uv, p.cam_group, 1)
        units, unit = p.n_points, "tracks/s"
        gpu = lambda: stitch_ba.triangulate(tr, p.rot, p.center, p.intr, 10.0)  # noqa: E731
        k = min(units, 200000)
        sub = tp[:k + 1]

        def cpu():
            return O.triangulate(sub, p.obs_cam[:sub[-1]], p.obs_uv[:sub[-1]], p.rot, p.center,
                                 p.intr, p.cam_group, 10.0, n_threads=threads)

        def agree(g, c):
            return {"kept_equal": float((g[0][:k] == c[0]).mean())}
    elif args.stage in ("ransac", "pair_fits"):
        pm = survey.pair_matches(p, seed=args.seed)
        units, unit = len(pm.pair_cam), "pairs/s"
        npairs = len(pm.pair_cam)
        seeds = pm.pair_cam[:, 0].astype(np.uint64) * np.uint64(7919) + pm.pair_cam[:, 1]
        if args.stage == "ransac":
            gpu = lambda: stitch_ba.ransac_fundamental(pm, 1.5, 600)  # noqa: E731
            k = min(npairs, 400)

            def cpu():
                return O.ransac_fundamental(pm.match_ptr[:k + 1], pm.uv, seeds[:k], 1.5, 600,
                                            n_threads=threads)

            def agree(g, c):
                return {"best_hypothesis_equal": float((g[2][:k] == c[2]).mean()),
                        "inlier_flags_equal": float((g[0][:pm.match_ptr[k]] == c[0]).mean())}
        else:
            gpu = lambda: stitch_ba.pair_fits(pm, p.rot, p.center, p.intr, p.cam_group)  # noqa: E731
            k = npairs

            def cpu():
                return O.pair_fits(pm.pair_cam, pm.match_ptr, pm.uv, p.rot, p.center, p.intr,
                                   p.cam_group, n_threads=threads)

            def agree(g, c):
                return {"max_rel_diff": float(np.abs(g - c).max() / np.abs(c).max())}
    else:
        units, unit = p.n_obs, "observations/s"
        gpu = lambda: stitch_ba.sparse_summary(p, 80.0)  # noqa: E731
        k = units

        def cpu():
            return O.sparse_summary(p.obs_cam, p.obs_pt, p.rot, p.center, p.points, 80.0)

        def agree(g, c):
            return {"neighbours_equal": bool(np.array_equal(g.neighbours, c[0])),
                    "depth_range_equal": bool(np.array_equal(g.depth_range, c[3]))}
    for _ in range(args.warmup):
        g = gpu()
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        g = gpu()
        times.append(time.perf_counter() - t0)
    dt = float(np.median(times))
    t0 = time.perf_counter()
    c = cpu()
    tc = time.perf_counter() - t0
    return {"metric": f"sparse stage: {args.stage}", "value": units / dt, "unit": unit,
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3,
            "higher_is_better": True, "dtype": "f64",
            "data": "synthetic (seeded survey generator, reference camera model)",
            "config": {"workload": args.workload, "cameras": p.n_cams, "points": p.n_points,
                       "observations": p.n_obs, "units": units},
            "cpu_baseline": {"value": k / tc, "unit": unit, "cores": threads, "kind": "port",
                             "sample": f"{k} of {units} units ({tc:.2f} s)"},
            "agreement_on_sample": agree(g, c)}



if __name__ == "__main__":
    main()
