"""``bundle_adjust`` — the drop-in for stitch-core's entry point
``pub fn bundle_adjust(p: &mut Problem, max_iter: usize, sigma_px: f64) -> BaStats``
(crates/stitch-core/src/recon/ba.rs:198), running on the GPU through the C
ABI of ``libba_gb300.so``.

Same argument meaning and the same in-place update of the problem's state as
the reference.  Unlike the reference (which cannot fail), invalid input raises
``BaError`` with status BAD_INPUT, and a missing GPU raises instead of falling
back to the CPU.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import native
from .problem import BaStats, Problem


# ba_options.point_kernel / ba_stats.point_kernel numbering
POINT_KERNELS = ["auto", "three_pass", "fused128", "fused256"]


@dataclass
class Options:
    """Solver options beyond the reference's (max_iter, sigma_px).

    Defaults reproduce the reference: Cauchy loss (ba.rs:99,114), FP64, PCG
    with at most 400 products (ba.rs:334) and |r|² < 1e-20 |b|² (ba.rs:182)."""
    loss: str = "cauchy"          # "cauchy" | "huber"
    precision: str = "fp64"       # "fp64" | "mixed"
    pcg_max_iter: int = 400
    pcg_tol: float = 1e-20
    matrix_free: str = "auto"     # "auto" | "stored" | "matrix_free" | "recompute" (mixed form:
                                  # matrix-free with J^T J recomputed in the PCG)
    memory_cap_bytes: int = 0
    stream: int | None = None     # cudaStream_t as an integer handle
    profile: bool = False         # per-phase CUDA-event timing (SolveInfo.phases)
    pcg_kernel: str = "auto"      # "auto" | "grid" | "cluster" | "cluster_wide" (mixed form;
                                  # cluster_wide: 1024 threads per CTA)
    graph: bool = True            # replay a CUDA graph per LM iteration
    autotune: bool = False        # time PCG configurations on the first solve of a form
    stop_patience: int = 0        # consecutive small accepted steps before stopping (0/1: ba.rs rule)
    coarse: bool = False          # mixed form, cluster PCG: two-level preconditioner
    wait_limit_cycles: int = 0    # spin limit of device-side waits (0: ~2 s)
    workspace_limit_bytes: int = 0  # device memory the call may hold (0: no limit) -> BA_OOM
    pcg_end_max_iter: int = 0     # PCG cap once a step's relative decrease < pcg_end_rel (0: off)
    pcg_end_rel: float = 0.0      # <= 0: 1e-5
    fault_hold_pcg_cta: int = 0   # tests of the timeout path: grid PCG CTA k-1 skips its exchanges
    point_kernel: str = "auto"    # mixed form's per-observation passes: "auto" | "three_pass" |
                                  # "fused128" | "fused256" (bit-identical results)


@dataclass
class SolveInfo:
    """Everything ba_stats reports, plus the per-iteration log (model 0)."""
    iterations: int
    initial_rms: float
    final_rms: float
    initial_cost: float
    final_cost: float
    pcg_iterations: int
    kernel_launches: int
    ms_total: float
    ms_h2d: float
    ms_d2h: float
    h2d_bytes: int
    d2h_bytes: int
    device_bytes: int
    new_cost: np.ndarray = field(default=None, repr=False)
    lam: np.ndarray = field(default=None, repr=False)
    pcg_iters: np.ndarray = field(default=None, repr=False)
    accepted: np.ndarray = field(default=None, repr=False)
    phases: dict = field(default_factory=dict, repr=False)  # name -> (ms, launches)
    sizes: dict = field(default_factory=dict, repr=False)   # reduced-system sizes
    pcg_kernel: str = "none"      # PCG kernel that ran: "grid" | "cluster" | "matrix_free"
    pcg_cluster: int = 0          # CTAs per cluster when the cluster kernel ran
    graph: bool = False           # LM iterations replayed a CUDA graph
    pcg_ctas: int = 0             # CTAs of the PCG launch
    pcg_tuned_us: float = 0.0     # autotuned time per PCG iteration (0: not tuned)
    coarse_dim: int = 0           # coarse unknowns of the two-level preconditioner
    schur_sub_len: int = 0        # Schur pairs per warp sub-segment
    schur_tuned_us: float = 0.0   # autotuned Schur kernel time (0: not tuned)
    pcg_threads: int = 0          # threads per CTA of the PCG launch
    point_kernel: str = "none"    # mixed form's per-observation passes that ran
    point_tuned_us: float = 0.0   # autotuned time of those passes (0: not tuned)

    def stats(self) -> BaStats:
        return BaStats(self.iterations, self.initial_rms, self.final_rms)


_MF = {"auto": 0, "stored": 1, "matrix_free": 2, "recompute": 3}


def _c_options(max_iter: int, sigma_px: float, o: Options | None, log=None) -> native.BaOptions:
    o = o or Options()
    c = native.BaOptions()
    native.load().ba_default_options(C.byref(c))
    c.max_iter = int(max_iter)
    c.sigma_px = float(sigma_px)
    c.loss = native.LOSS[o.loss]
    c.precision = native.PRECISION[o.precision]
    c.pcg_max_iter = int(o.pcg_max_iter)
    c.pcg_tol = float(o.pcg_tol)
    c.matrix_free = _MF[o.matrix_free]
    c.memory_cap_bytes = int(o.memory_cap_bytes)
    c.stream = o.stream
    c.profile = 1 if o.profile else 0
    c.pcg_kernel = {"auto": 0, "grid": 1, "cluster": 2, "cluster_wide": 3}[o.pcg_kernel]
    c.no_graph = 0 if o.graph else 1
    c.autotune = 1 if o.autotune else 0
    c.stop_patience = int(o.stop_patience)
    c.coarse = 1 if o.coarse else 0
    c.wait_limit_cycles = int(o.wait_limit_cycles)
    c.workspace_limit_bytes = int(o.workspace_limit_bytes)
    c.pcg_end_max_iter = int(o.pcg_end_max_iter)
    c.pcg_end_rel = float(o.pcg_end_rel)
    c.fault_hold_pcg_cta = int(o.fault_hold_pcg_cta)
    c.point_kernel = POINT_KERNELS.index(o.point_kernel)
    c.log = C.cast(C.pointer(log), C.c_void_p) if log is not None else None
    return c


def _arr(a, dtype):
    if a is None:
        return None
    if not (isinstance(a, np.ndarray) and a.dtype == dtype and a.flags.c_contiguous):
        raise TypeError(f"expected a C-contiguous {np.dtype(dtype)} array")
    return a.ctypes.data


def c_views(p: Problem):
    """(ba_problem, ba_state) views of a Problem's arrays (no copies)."""
    for name, dt in (("rot", np.float64), ("center", np.float64), ("intr", np.float64),
                     ("points", np.float64)):
        a = getattr(p, name)
        if not (a.dtype == dt and a.flags.c_contiguous and a.flags.writeable):
            raise TypeError(f"Problem.{name} must be a writeable C-contiguous float64 array")
    prob = native.BaProblem(
        p.n_cams, p.n_points, p.n_obs, p.n_groups, _arr(p.obs_cam, np.uint32),
        _arr(p.obs_pt, np.uint32), _arr(p.obs_uv, np.float64), _arr(p.cam_group, np.uint32),
        _arr(p.prior_mask, np.uint8), _arr(p.prior, np.float64) if p.prior_mask is not None else None,
        1 if p.refine_intrinsics else 0)
    st = native.BaState(p.rot.ctypes.data, p.center.ctypes.data, p.intr.ctypes.data,
                        p.points.ctypes.data)
    return prob, st


def _info(s: native.BaStatsC) -> SolveInfo:
    info = SolveInfo(s.iterations, s.initial_rms, s.final_rms, s.initial_cost, s.final_cost,
                     s.pcg_iterations, s.kernel_launches, s.ms_total, s.ms_h2d, s.ms_d2h,
                     s.h2d_bytes, s.d2h_bytes, s.device_bytes)
    info.phases = {n: (s.ms_phase[i], s.n_phase[i]) for i, n in enumerate(native.PHASES)
                   if s.n_phase[i]}
    info.sizes = dict(blocks=s.n_blocks, nonzero_blocks=s.n_nonzero_blocks,
                      schur_pairs=s.n_schur_pairs, lens_entries=s.n_lens_entries)
    info.pcg_kernel = {1: "grid", 2: "cluster", 3: "matrix_free"}.get(s.pcg_kernel, "none")
    info.pcg_cluster = s.pcg_cluster
    info.graph = bool(s.graph)
    info.pcg_ctas = s.pcg_ctas
    info.pcg_tuned_us = s.pcg_tuned_us
    info.coarse_dim = s.pcg_coarse_dim
    info.schur_sub_len = s.schur_sub_len
    info.schur_tuned_us = s.schur_tuned_us
    info.pcg_threads = s.pcg_threads
    info.point_kernel = POINT_KERNELS[s.point_kernel] if s.point_kernel > 0 else "none"
    info.point_tuned_us = s.point_tuned_us
    return info


class _Log:
    def __init__(self, cap: int):
        self.new_cost = np.zeros(cap)
        self.lam = np.zeros(cap)
        self.pcg = np.zeros(cap, np.int32)
        self.acc = np.zeros(cap, np.int32)
        self.c = native.BaLog(cap, self.new_cost.ctypes.data, self.lam.ctypes.data,
                              self.pcg.ctypes.data, self.acc.ctypes.data)

    def attach(self, info: SolveInfo):
        n = int(info.iterations)
        info.new_cost, info.lam = self.new_cost[:n].copy(), self.lam[:n].copy()
        info.pcg_iters, info.accepted = self.pcg[:n].copy(), self.acc[:n].astype(bool)


def bundle_adjust(p: Problem, max_iter: int, sigma_px: float, options: Options | None = None,
                  *, return_info: bool = False):
    """ba.rs:198.  Mutates p.rot, p.center, p.points (and p.intr when
    refining) in place; returns BaStats (and SolveInfo if asked)."""
    L = native.load()
    log = _Log(max(int(max_iter), 1))
    opt = _c_options(max_iter, sigma_px, options, log.c)
    prob, st = c_views(p)
    out = native.BaStatsC()
    native.check(L.ba_solve(C.byref(prob), C.byref(st), C.byref(opt), C.byref(out)))
    info = _info(out)
    log.attach(info)
    return (info.stats(), info) if return_info else info.stats()


def bundle_adjust_batch(problems: list[Problem], max_iter: int, sigma_px: float,
                        options: Options | None = None) -> list[SolveInfo]:
    """Solve independent problems in one batched launch sequence."""
    L = native.load()
    n = len(problems)
    views = [c_views(p) for p in problems]
    probs = (native.BaProblem * n)(*[v[0] for v in views])
    states = (native.BaState * n)(*[v[1] for v in views])
    stats = (native.BaStatsC * n)()
    opt = _c_options(max_iter, sigma_px, options)
    native.check(L.ba_solve_batch(probs, states, n, C.byref(opt), stats))
    return [_info(s) for s in stats]


class Context:
    """Device-resident problems: upload once, solve repeatedly from the
    uploaded initial state, download the solution."""

    def __init__(self, device: int = -1, stream: int | None = None):
        self._L = native.load()
        h = C.c_void_p()
        native.check(self._L.ba_context_create(device, stream, C.byref(h)))
        self._h = h
        self._n = 0
        self._problems = []

    def close(self):
        if self._h:
            self._L.ba_context_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, problems: list[Problem] | Problem):
        if isinstance(problems, Problem):
            problems = [problems]
        views = [c_views(p) for p in problems]
        n = len(problems)
        probs = (native.BaProblem * n)(*[v[0] for v in views])
        states = (native.BaState * n)(*[v[1] for v in views])
        native.check(self._L.ba_context_upload(self._h, probs, states, n))
        self._n = n
        self._problems = list(problems)

    def solve(self, max_iter: int, sigma_px: float, options: Options | None = None,
              log: bool = False) -> list[SolveInfo]:
        lg = _Log(max(int(max_iter), 1)) if log else None
        opt = _c_options(max_iter, sigma_px, options, lg.c if lg else None)
        stats = (native.BaStatsC * self._n)()
        native.check(self._L.ba_context_solve(self._h, C.byref(opt), stats))
        infos = [_info(s) for s in stats]
        if lg:
            lg.attach(infos[0])
        return infos

    def download(self, problems: list[Problem] | Problem | None = None):
        problems = self._problems if problems is None else problems
        if isinstance(problems, Problem):
            problems = [problems]
        states = (native.BaState * len(problems))(*[c_views(p)[1] for p in problems])
        native.check(self._L.ba_context_download(self._h, states, len(problems)))

    def cost(self, sigma_px: float, options: Options | None = None):
        c = np.zeros(self._n)
        r = np.zeros(self._n)
        n = np.zeros(self._n, np.int64)
        opt = _c_options(0, sigma_px, options)
        native.check(self._L.ba_context_cost(self._h, C.byref(opt), c.ctypes.data, r.ctypes.data,
                                             n.ctypes.data))
        return c, r, n

    def linearise(self, sigma_px: float, options: Options | None = None):
        no = sum(p.n_obs for p in self._problems)
        e = np.zeros((no, 2))
        jc = np.zeros((no, 2, 6))
        jg = np.zeros((no, 2, 3))
        jp = np.zeros((no, 2, 3))
        w = np.zeros(no)
        valid = np.zeros(no, np.uint8)
        opt = _c_options(0, sigma_px, options)
        native.check(self._L.ba_context_linearise(
            self._h, C.byref(opt), e.ctypes.data, jc.ctypes.data, jg.ctypes.data, jp.ctypes.data,
            w.ctypes.data, valid.ctypes.data))
        return dict(e=e, jc=jc, jg=jg, jp=jp, w=w, valid=valid.astype(bool))

    def vjp(self, sigma_px: float, cot_obs=None, cot_prior=None, options: Options | None = None):
        nc = sum(p.n_cams for p in self._problems)
        npt = sum(p.n_points for p in self._problems)
        ng = sum(p.n_groups for p in self._problems)
        gc, gp, gi = np.zeros((nc, 6)), np.zeros((npt, 3)), np.zeros((ng, 5))
        co = None if cot_obs is None else np.ascontiguousarray(cot_obs, np.float64)
        cp = None if cot_prior is None else np.ascontiguousarray(cot_prior, np.float64)
        opt = _c_options(0, sigma_px, options)
        native.check(self._L.ba_context_vjp(
            self._h, C.byref(opt), None if co is None else co.ctypes.data,
            None if cp is None else cp.ctypes.data, gc.ctypes.data, gp.ctypes.data,
            gi.ctypes.data))
        return gc, gp, gi

    def debug_step(self, lam: float, sigma_px: float, options: Options | None = None,
                   dense: bool = True):
        """One LM system at damping `lam` from the uploaded state (single
        model): dense S, g, dx, PCG iterations, trial cost."""
        p = self._problems[0]
        nb = p.n_cams + p.n_groups
        S = np.zeros((6 * nb, 6 * nb)) if dense else None
        g, dx = np.zeros(6 * nb), np.zeros(6 * nb)
        it, tc = C.c_int32(), C.c_double()
        opt = _c_options(1, sigma_px, options)
        native.check(self._L.ba_context_debug_step(
            self._h, C.byref(opt), float(lam), None if S is None else S.ctypes.data,
            g.ctypes.data, dx.ctypes.data, C.byref(it), C.byref(tc)))
        return dict(S=S, g=g, dx=dx, pcg_iters=it.value, trial_cost=tc.value)

    def upload_tracks(self, tracks: "Tracks", rot, center, intr, thr_px: float,
                      prior_mask=None, prior=None, refine_intrinsics: bool = True):
        """Triangulate and gate a round's tracks on the device and make the
        kept tracks the context's problem (sparse.rs:389-449), without a host
        round trip.  Returns (n_points, n_obs)."""
        R, Cc, K = _f64(rot), _f64(center), _f64(intr)
        st = native.BaState(R.ctypes.data, Cc.ctypes.data, K.ctypes.data, None)
        pm = None if prior_mask is None else np.ascontiguousarray(prior_mask, np.uint8)
        pr = None if prior is None else _f64(prior)
        n_pts, n_obs = C.c_int64(), C.c_int64()
        tv = tracks.c_view()
        native.check(self._L.ba_context_upload_tracks(
            self._h, C.byref(tv), C.byref(st), None if pm is None else pm.ctypes.data,
            None if pr is None else pr.ctypes.data, 1 if refine_intrinsics else 0, float(thr_px),
            C.byref(n_pts), C.byref(n_obs)))
        nc, ng = len(tracks.cam_group), int(tracks.n_groups)
        # A host mirror for download(): the state arrays the context solves.
        self._problems = [Problem.empty(nc, n_pts.value, n_obs.value, ng,
                                        refine_intrinsics=refine_intrinsics)]
        self._n = 1
        return n_pts.value, n_obs.value

    def sparse_summary(self, agl: float, max_neighbours: int = 8) -> "SparseSummary":
        """sparse_summary() of the context's single model with its current
        (solved) state, computed where the state lives."""
        p = self._problems[0]
        out = SparseSummary.alloc(p.n_cams, p.n_points, max_neighbours)
        native.check(self._L.ba_context_sparse_summary(self._h, int(max_neighbours), float(agl),
                                                        *out.pointers()))
        return out

    def intrinsics_grad(self, sigma_px: float, options: Options | None = None) -> np.ndarray:
        ng = sum(p.n_groups for p in self._problems)
        g = np.zeros((ng, 5))
        opt = _c_options(0, sigma_px, options)
        native.check(self._L.ba_context_intrinsics_grad(self._h, C.byref(opt), g.ctypes.data))
        return g


@dataclass
class Tracks:
    """Feature tracks of one sparse-stage round (sparse.rs:389): track t is
    observed by obs_cam / obs_uv[track_ptr[t]:track_ptr[t + 1]] (full
    resolution, distorted pixels); cam_group gives each camera's lens group."""
    track_ptr: np.ndarray  # u32[n_tracks + 1]
    obs_cam: np.ndarray    # u32[n_obs]
    obs_uv: np.ndarray     # f64[n_obs, 2]
    cam_group: np.ndarray  # u32[n_cams]
    n_groups: int = 1

    def c_view(self) -> native.BaTracks:
        for name, dt in (("track_ptr", np.uint32), ("obs_cam", np.uint32), ("obs_uv", np.float64),
                         ("cam_group", np.uint32)):
            a = getattr(self, name)
            if not (isinstance(a, np.ndarray) and a.dtype == dt and a.flags.c_contiguous):
                raise TypeError(f"Tracks.{name} must be a C-contiguous {np.dtype(dt)} array")
        return native.BaTracks(len(self.track_ptr) - 1, len(self.obs_cam), len(self.cam_group),
                               int(self.n_groups), self.track_ptr.ctypes.data,
                               self.obs_cam.ctypes.data, self.obs_uv.ctypes.data,
                               self.cam_group.ctypes.data)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def triangulate(tracks: Tracks, rot, center, intr, thr_px: float):
    """One round's triangulation and reprojection gating (sparse.rs:389-421).
    Returns (kept bool[n_tracks], points f64[n_tracks, 3], good bool[n_obs])."""
    L = native.load()
    nt, no = len(tracks.track_ptr) - 1, len(tracks.obs_cam)
    kept = np.zeros(max(nt, 0), np.uint8)
    pts = np.zeros((max(nt, 0), 3))
    good = np.zeros(no, np.uint8)
    nk = C.c_int64()
    R, Cc, K = _f64(rot), _f64(center), _f64(intr)
    tv = tracks.c_view()
    native.check(L.ba_triangulate(C.byref(tv), R.ctypes.data, Cc.ctypes.data, K.ctypes.data,
                                  float(thr_px), None, kept.ctypes.data, pts.ctypes.data,
                                  good.ctypes.data, C.byref(nk)))
    return kept.astype(bool), pts, good.astype(bool)


@dataclass
class SparseSummary:
    """Per-camera fields of cameras.json and the f32 points of sparse.ply
    (sparse.rs:470-483, 515-533; mod.rs:31-35).  Row a of `neighbours` holds
    camera a's n_neighbours[a] best co-observing cameras, most shared points
    first (equal counts by ascending index), padded with UINT32_MAX."""
    neighbours: np.ndarray    # u32[n_cams, max_neighbours]
    shared: np.ndarray        # u32[n_cams, max_neighbours]
    n_neighbours: np.ndarray  # i32[n_cams]
    depth_range: np.ndarray   # f64[n_cams, 2]
    points_f32: np.ndarray    # f32[n_points, 3]

    @staticmethod
    def alloc(nc: int, npts: int, k: int) -> "SparseSummary":
        return SparseSummary(np.zeros((nc, k), np.uint32), np.zeros((nc, k), np.uint32),
                             np.zeros(nc, np.int32), np.zeros((nc, 2)),
                             np.zeros((npts, 3), np.float32))

    def pointers(self):
        return (self.neighbours.ctypes.data, self.shared.ctypes.data,
                self.n_neighbours.ctypes.data, self.depth_range.ctypes.data,
                self.points_f32.ctypes.data)

    def neighbour_lists(self) -> list[list[int]]:
        return [self.neighbours[a, :n].tolist() for a, n in enumerate(self.n_neighbours)]


def sparse_summary(problem: Problem, agl: float, max_neighbours: int = 8) -> SparseSummary:
    """Neighbours, depth ranges and f32 points of a bundle-adjusted problem
    on the device (replaces the host loops at sparse.rs:470-483, 515-533 and
    the conversion at mod.rs:31-35).  `agl` is the flying height above
    ground, the depth range of cameras with fewer than ten points."""
    L = native.load()
    prob, st = c_views(problem)
    out = SparseSummary.alloc(problem.n_cams, problem.n_points, max_neighbours)
    native.check(L.ba_sparse_summary(C.byref(prob), C.byref(st), int(max_neighbours), float(agl),
                                     None, *out.pointers()))
    return out


@dataclass
class PairMatches:
    """Matches of photo pairs: pair p joins cameras pair_cam[p] = (i, j) and
    owns uv[match_ptr[p]:match_ptr[p + 1]], rows (u_i, v_i, u_j, v_j) in
    pixels.  seed: per-pair RANSAC seeds (default i * 7919 + j,
    sparse.rs:290)."""
    pair_cam: np.ndarray   # u32[n_pairs, 2]
    match_ptr: np.ndarray  # u32[n_pairs + 1]
    uv: np.ndarray         # f64[n_matches, 4]
    seed: np.ndarray | None = None  # u64[n_pairs]

    def c_view(self) -> native.BaPairMatches:
        for name, dt in (("pair_cam", np.uint32), ("match_ptr", np.uint32), ("uv", np.float64),
                         ("seed", np.uint64)):
            a = getattr(self, name)
            if a is None and name == "seed":
                continue
            if not (isinstance(a, np.ndarray) and a.dtype == dt and a.flags.c_contiguous):
                raise TypeError(f"PairMatches.{name} must be a C-contiguous {np.dtype(dt)} array")
        return native.BaPairMatches(len(self.match_ptr) - 1, len(self.uv.reshape(-1, 4)),
                                    self.pair_cam.ctypes.data, self.match_ptr.ctypes.data,
                                    self.uv.ctypes.data,
                                    None if self.seed is None else self.seed.ctypes.data)


def ransac_fundamental(pairs: PairMatches, thresh_px: float = 1.5, iters: int = 600):
    """Fundamental-matrix RANSAC of every pair on the device (geometry.rs:
    248-300 as sparse.rs:290 calls it).  Returns (inlier bool[n_matches],
    n_inliers i32[n_pairs], best_hypothesis i32[n_pairs], refit bool[n_pairs])."""
    L = native.load()
    v = pairs.c_view()
    inl = np.zeros(v.n_matches, np.uint8)
    n = np.zeros(v.n_pairs, np.int32)
    best = np.zeros(v.n_pairs, np.int32)
    refit = np.zeros(v.n_pairs, np.uint8)
    native.check(L.ba_ransac_fundamental(C.byref(v), float(thresh_px), int(iters), None,
                                         inl.ctypes.data, n.ctypes.data, best.ctypes.data,
                                         refit.ctypes.data))
    return inl.astype(bool), n, best, refit.astype(bool)


def pair_fits(pairs: PairMatches, rot, center, intr, cam_group) -> np.ndarray:
    """Median Sampson error (pixels) of every pair's matches under the given
    poses, on the device (sparse.rs:620-645)."""
    L = native.load()
    v = pairs.c_view()
    R, Cc, K = _f64(rot), _f64(center), _f64(intr)
    cg = np.ascontiguousarray(cam_group, np.uint32)
    med = np.zeros(v.n_pairs)
    native.check(L.ba_pair_fits(C.byref(v), R.ctypes.data, Cc.ctypes.data, K.ctypes.data,
                                cg.ctypes.data, len(cg), len(K.reshape(-1, 5)), None,
                                med.ctypes.data))
    return med
