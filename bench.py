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
  iterations) and FP32/FP64 mixed form (two-level PCG: block Jacobi plus the
  similarity motions of camera groups, 40 iterations; 60 above 1000 cameras
  per model) side by side, with the final cost of each and their relative
  difference; the mixed form is the headline when it reaches the FP64 final
  cost.
* ``roofline`` — the dominant kernel phase (by device time, from the
  solver's own CUDA-event phase timing) against measured HBM bandwidth.
* ``cpu_baseline`` — the oracle (a CPU restatement of the reference solver,
  same data structures, OpenMP on all host cores) on a bounded sample: the
  first LM iterations of the same solve, scaled to solves/s by the full
  solve's iteration count.

``--impl reference`` times that CPU solver alone as the reference arm.

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


MIXED_MATRIX_FREE = False  # --matrix-free: the mixed form applies S without forming it
MIXED_PCG_CAP = MIXED_PCG_ITERS  # set per workload by set_mixed_cap


def set_mixed_cap(ps):
    global MIXED_PCG_CAP
    big = max(p.n_cams for p in ps) > MIXED_LARGE_CAMS
    MIXED_PCG_CAP = MIXED_PCG_ITERS_LARGE if big else MIXED_PCG_ITERS


def form_options(prec: str, **kw):
    """Per form: the PCG layout is picked by the solver's autotuner on the
    first (warm-up) solve of the form and reused by the timed solves."""
    from stitch_ba import Options
    kw.setdefault("autotune", True)
    if prec == "mixed":
        mf = "matrix_free" if MIXED_MATRIX_FREE else "auto"
        kw.setdefault("coarse", not MIXED_MATRIX_FREE)
        return Options(precision="mixed", pcg_max_iter=MIXED_PCG_CAP, matrix_free=mf, **kw)
    return Options(precision="fp64", **kw)


def max_over_ranks(x: float, ws: int, device: str = "cuda") -> float:
    """Timing of the slowest rank (replicas: every rank solves its own models)."""
    if ws <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def rank_seed(seed: int, rank: int) -> int:
    """Each replica solves its own survey (weak scaling: fixed work per GPU)."""
    return seed + rank


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    return ws, rank


# Batched workload: 64 independent lawnmower models of uneven size (cameras
# ~U[20, 800], 500-1000 points per camera), solved together.
BATCH_MODELS = 64


def make_workload(name: str, seed: int):
    """A list of problems: one for a single survey, BATCH_MODELS for batch64."""
    from stitch_ba import survey
    if name == "batch64":
        return [m[0] for m in survey.batched_models(BATCH_MODELS, seed=seed)]
    p, truth = survey.generate(name, seed=seed)
    return [p]


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


def gpu_arm(args, ws, rank):
    import torch
    import stitch_ba
    from stitch_ba import Options, native

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    native.load()
    ps = make_workload(args.workload, rank_seed(args.seed, rank))
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
    precisions = ["fp64", "mixed"] if args.precision == "both" else [args.precision]
    profile_info = {}
    infos_by_form = {}
    with stitch_ba.Context(device=dev, stream=stream.cuda_stream) as ctx:
        ctx.upload(ps)
        for prec in precisions:
            opts = form_options(prec)
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
            forms[prec] = dict(ms_per_solve=ms, final_cost=sum(i.final_cost for i in infos),
                               initial_cost=sum(i.initial_cost for i in infos),
                               iterations=max(i.iterations for i in infos),
                               pcg_iterations=sum(i.pcg_iterations for i in infos),
                               final_rms=info.final_rms,
                               kernel_launches=info.kernel_launches, clocks=clk.summary())
            forms[prec]["model_final_costs"] = [i.final_cost for i in infos] if nmod > 1 else None
            forms[prec]["model_iterations"] = [i.iterations for i in infos] if nmod > 1 else None
            # one profiled solve with the per-iteration log (phase timing; not
            # part of the timed region)
            prof = ctx.solve(args.max_iter, SIGMA_PX, form_options(prec, profile=True),
                             log=(nmod == 1))[0]
            profile_info[prec] = prof
            infos_by_form[prec] = infos
            forms[prec]["pcg_kernel"] = prof.pcg_kernel
            forms[prec]["pcg_ctas"] = int(prof.pcg_ctas)
            forms[prec]["pcg_autotuned_us_per_iter"] = prof.pcg_tuned_us
            forms[prec]["device_bytes"] = int(prof.device_bytes)
            forms[prec]["pcg_max_iter"] = opts.pcg_max_iter
            forms[prec]["coarse_dim"] = int(prof.coarse_dim)
            forms[prec]["graph"] = bool(info.graph)
    if "fp64" in forms and "mixed" in forms:
        # Equal final cost: the mixed solve reaches the FP64 solve's final cost
        # to within 1e-6 relative (or ends below it).
        f64, fm = forms["fp64"]["final_cost"], forms["mixed"]["final_cost"]
        forms["mixed"]["rel_final_cost_vs_fp64"] = (fm - f64) / abs(f64)
        reaches = fm <= f64 * (1.0 + 1e-6)
        forms["mixed"]["reaches_fp64_final_cost"] = bool(reaches)
        # First LM iteration whose accepted cost is within 1e-6 of the FP64
        # final cost, and the share of the solve's time spent until then.
        log = profile_info["mixed"]
        hit = None
        for i in range(int(log.iterations) if nmod == 1 else 0):
            if log.accepted[i] and log.new_cost[i] <= f64 * (1.0 + 1e-6):
                hit = i
                break
        # Per LM iteration of the profiled solve: trial cost relative to the
        # FP64 final cost, accepted (1/0), PCG iterations.
        for prec in ("fp64", "mixed"):
            lg = profile_info[prec]
            if nmod == 1 and lg.new_cost is not None:
                forms[prec]["lm_trace"] = [
                    [float("%.3g" % (lg.new_cost[i] / f64 - 1.0)), int(lg.accepted[i]),
                     int(lg.pcg_iters[i])] for i in range(int(lg.iterations))]
        if hit is not None:
            forms["mixed"]["iteration_reaching_fp64_cost"] = hit + 1
            forms["mixed"]["ms_to_fp64_cost_est"] = forms["mixed"]["ms_per_solve"] * (hit + 1) / max(
                int(log.iterations), 1)
        if nmod > 1:
            a, b = forms["fp64"]["model_final_costs"], forms["mixed"]["model_final_costs"]
            forms["mixed"]["models_reaching_fp64_cost"] = int(sum(
                1 for x, y in zip(a, b) if y <= x * (1.0 + 1e-6)))
        forms["mixed"]["speedup_vs_fp64"] = forms["fp64"]["ms_per_solve"] / forms["mixed"]["ms_per_solve"]
        chosen = "mixed" if reaches else "fp64"
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
              subsegments=zs["schur_pairs"] // 512 + (zs["nonzero_blocks"] + zs["blocks"]) // 2)
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

    value = ws * nmod * 1000.0 / head["ms_per_solve"]
    out = {
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": head["ms_per_solve"],
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64" if chosen == "fp64" else "f32+f64",
        "data": "synthetic (seeded survey generator, reference camera model)",
        "config": {"workload": args.workload, "models": nmod, "cameras": tot["n_cams"],
                   "points": tot["n_points"], "observations": tot["n_obs"],
                   "max_iter": args.max_iter, "sigma_px": SIGMA_PX,
                   "loss": "cauchy", "precision": chosen, "parallelism": f"replicas{ws}",
                   "l2": "flushed between steps (256 MiB write)"},
        "forms": {k: {kk: vv for kk, vv in v.items() if kk != "clocks"} if isinstance(v, dict) else v
                  for k, v in forms.items()},
        "e2e": {"value": ws * nmod / e2e_s, "unit": UNIT,
                "h2d_bytes_per_step": int(e2e_info.h2d_bytes),
                "d2h_bytes_per_step": int(e2e_info.d2h_bytes),
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
    if not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline(ps, [i.iterations for i in infos_by_form[chosen]],
                                           args.cpu_sample_iters)
    return out


def cpu_baseline(ps, full_iters, sample_iters: int):
    """Oracle (CPU restatement of the reference, OpenMP on all host cores) on
    the first `sample_iters` LM iterations of one model (the largest), scaled
    to the whole job by observations x LM iterations."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import ba_oracle
    ba_oracle.build()
    k = max(range(len(ps)), key=lambda i: ps[i].n_obs)
    q = ps[k].copy()
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    r = ba_oracle.bundle_adjust(q, sample_iters, SIGMA_PX, n_threads=threads)
    dt = time.perf_counter() - t0
    per_iter = dt / max(r.iterations, 1)
    work = sum(p.n_obs * max(it, 1) for p, it in zip(ps, full_iters))
    est = per_iter * work / ps[k].n_obs
    solves = len(ps)
    what = "the survey" if solves == 1 else f"the largest of {solves} models"
    return {"value": solves / est, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"first {r.iterations} LM iterations of {what} ({dt:.1f} s), scaled by "
                      f"observations x the GPU solve's LM iterations ({max(full_iters)} max)",
            "s_per_lm_iteration": per_iter}


def reference_arm(args, ws, rank):
    """CPU reference solver (oracle port, all host cores), same workload and unit.
    A step solves the first `cpu_sample_iters` LM iterations of the survey (of
    the largest model for batch64), scaled to whole solves by the LM
    iteration count of the full solve and, for batch64, by observations."""
    if rank != 0:
        return None
    ps = make_workload(args.workload, args.seed)
    tot = totals(ps)
    k = max(range(len(ps)), key=lambda i: ps[i].n_obs)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import ba_oracle
    ba_oracle.build()
    threads = os.cpu_count() or 1
    times = []
    iters = 0
    for i in range(args.warmup + args.steps):
        q = ps[k].copy()
        t0 = time.perf_counter()
        r = ba_oracle.bundle_adjust(q, args.cpu_sample_iters, SIGMA_PX, n_threads=threads)
        dt = time.perf_counter() - t0
        iters = r.iterations
        if i >= args.warmup:
            times.append(dt / max(r.iterations, 1))
    per_iter = float(np.mean(times))
    est = per_iter * args.full_iters * tot["n_obs"] / ps[k].n_obs
    v = len(ps) / est
    return {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": est * 1000.0,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded survey generator, reference camera model)",
        "config": {"workload": args.workload, "models": len(ps), "cameras": tot["n_cams"],
                   "points": tot["n_points"], "observations": tot["n_obs"],
                   "max_iter": args.max_iter, "sigma_px": SIGMA_PX,
                   "loss": "cauchy", "precision": "fp64", "parallelism": "cpu"},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"each step = first {iters} LM iterations of the "
                                   f"{'survey' if len(ps) == 1 else 'largest model'}, scaled by "
                                   f"{args.full_iters} LM iterations per solve"
                                   + ("" if len(ps) == 1 else " and by observations")},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
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
    ap.add_argument("--cpu-sample-iters", type=int, default=2)
    ap.add_argument("--full-iters", type=int, default=int(os.environ.get("BA_FULL_ITERS", "0")) or None)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--stage", default="ba",
                    choices=["ba", "triangulate", "ransac", "pair_fits", "summary"])
    ap.add_argument("--matrix-free", action="store_true",
                    help="mixed form: matrix-free PCG (S p from per-observation factors)")
    args = ap.parse_args()
    global MIXED_MATRIX_FREE
    MIXED_MATRIX_FREE = args.matrix_free
    ws, rank = dist_env()
    if args.stage != "ba":
        out = stage_arm(args, ws, rank)
    elif args.impl == "reference":
        if args.full_iters is None:
            args.full_iters = FULL_ITERS.get(args.workload, MAX_ITER)
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


# LM iterations the full solve of each workload takes (FP64, measured on the
# GPU plain form, which matches the CPU solver's iteration count); used to
# scale the CPU reference arm's per-iteration sample to solves/s.
FULL_ITERS = {"single500": 17, "lawnmower77": 43}

if __name__ == "__main__":
    main()
