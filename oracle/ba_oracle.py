"""ORACLE — test infrastructure only.

ctypes wrapper of ``oracle/_build/libba_oracle.so``, the CPU FP64
restatement of stitch-core's bundle adjustment
(crates/stitch-core/src/recon/ba.rs:56-391).  Only the tests, the smoke check
and the CPU-baseline leg of the benchmark load it, and only as the checker or
the timed CPU baseline; the product library never does.

Problems and states are duck-typed: any object with the SoA attributes
``obs_cam, obs_pt, obs_uv, cam_group, prior_mask, prior, refine_intrinsics``
(problem) and ``rot, center, intr, points`` (state) works, which is how the
product's ``stitch_ba.Problem`` is passed in.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libba_oracle.so")

LOSS_CAUCHY = 0
LOSS_HUBER = 1


class _Problem(C.Structure):
    _fields_ = [
        ("n_cams", C.c_int32), ("n_points", C.c_int32), ("n_obs", C.c_int32),
        ("n_groups", C.c_int32),
        ("obs_cam", C.c_void_p), ("obs_pt", C.c_void_p), ("obs_uv", C.c_void_p),
        ("cam_group", C.c_void_p), ("prior_mask", C.c_void_p), ("prior", C.c_void_p),
        ("refine_intrinsics", C.c_int32),
    ]


class _State(C.Structure):
    _fields_ = [("rot", C.c_void_p), ("center", C.c_void_p), ("intr", C.c_void_p),
                ("points", C.c_void_p)]


class _Stats(C.Structure):
    _fields_ = [
        ("iterations", C.c_int64), ("initial_rms", C.c_double), ("final_rms", C.c_double),
        ("initial_cost", C.c_double), ("final_cost", C.c_double),
        ("log_cap", C.c_int32),
        ("log_new_cost", C.c_void_p), ("log_lambda", C.c_void_p),
        ("log_pcg", C.c_void_p), ("log_accept", C.c_void_p),
        ("t_linearise", C.c_double), ("t_point", C.c_double), ("t_assembly", C.c_double),
        ("t_schur", C.c_double), ("t_pcg", C.c_double), ("t_backsub", C.c_double),
        ("t_cost", C.c_double), ("t_total", C.c_double),
    ]


_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (seconds)."""
    if force or not os.path.exists(LIB_PATH) or (
            os.path.getmtime(LIB_PATH) < os.path.getmtime(os.path.join(HERE, "ba_oracle.cpp"))):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        L.oracle_bundle_adjust.argtypes = [C.POINTER(_Problem), C.POINTER(_State), C.c_int32,
                                           C.c_double, C.c_int32, C.c_int32, C.c_int32,
                                           C.POINTER(_Stats)]
        L.oracle_robust_cost.argtypes = [C.POINTER(_Problem), C.POINTER(_State), C.c_double,
                                         C.c_int32, C.POINTER(C.c_double),
                                         C.POINTER(C.c_double), C.POINTER(C.c_int64)]
        L.oracle_linearise.argtypes = [C.POINTER(_Problem), C.POINTER(_State), C.c_double,
                                       C.c_int32] + [C.c_void_p] * 6
        L.oracle_lm_step.argtypes = [C.POINTER(_Problem), C.POINTER(_State), C.c_double,
                                     C.c_double, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p,
                                     C.c_void_p, C.c_void_p, C.POINTER(C.c_int32),
                                     C.POINTER(_State), C.POINTER(C.c_double)]
        L.oracle_exp_so3.argtypes = [C.c_void_p, C.c_void_p]
        L.oracle_from_angles.argtypes = [C.c_double, C.c_double, C.c_double, C.c_void_p]
        L.oracle_project.argtypes = [C.c_void_p] * 5
        L.oracle_undistort.argtypes = [C.c_void_p] * 3
        L.oracle_make_ref_survey.argtypes = [C.c_void_p] * 5 + [
            C.POINTER(_State), C.POINTER(C.c_int32), C.POINTER(C.c_int32),
            C.POINTER(C.c_double)]
        L.oracle_max_threads.restype = C.c_int
        L.oracle_set_spmv_shuffle.argtypes = [C.c_uint64]
        L.oracle_set_spmv_shuffle.restype = None
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data


def _check(a, dtype, n):
    assert isinstance(a, np.ndarray) and a.dtype == dtype and a.flags.c_contiguous, \
        (a.dtype if isinstance(a, np.ndarray) else type(a), dtype)
    assert a.size == n, (a.size, n)
    return a


def _problem(p) -> _Problem:
    nc = p.rot.shape[0]
    ng = p.intr.shape[0]
    npt = p.points.shape[0]
    no = p.obs_cam.shape[0]
    _check(p.obs_cam, np.uint32, no)
    _check(p.obs_pt, np.uint32, no)
    _check(p.obs_uv, np.float64, 2 * no)
    _check(p.cam_group, np.uint32, nc)
    if p.prior_mask is not None:
        _check(p.prior_mask, np.uint8, nc)
        _check(p.prior, np.float64, 6 * nc)
    return _Problem(nc, npt, no, ng, _ptr(p.obs_cam), _ptr(p.obs_pt), _ptr(p.obs_uv),
                    _ptr(p.cam_group), _ptr(p.prior_mask),
                    _ptr(p.prior) if p.prior_mask is not None else None,
                    1 if p.refine_intrinsics else 0)


def _state(s) -> _State:
    nc = s.rot.shape[0]
    _check(s.rot, np.float64, 9 * nc)
    _check(s.center, np.float64, 3 * nc)
    _check(s.intr, np.float64, s.intr.size)
    _check(s.points, np.float64, s.points.size)
    return _State(_ptr(s.rot), _ptr(s.center), _ptr(s.intr), _ptr(s.points))


@dataclass
class OracleResult:
    iterations: int
    initial_rms: float
    final_rms: float
    initial_cost: float
    final_cost: float
    new_cost: np.ndarray = field(repr=False)
    lam: np.ndarray = field(repr=False)
    pcg_iters: np.ndarray = field(repr=False)
    accepted: np.ndarray = field(repr=False)
    phases: dict = field(default_factory=dict)


def bundle_adjust(p, max_iter: int, sigma_px: float, *, loss: int = LOSS_CAUCHY,
                  pcg_max_iter: int = 400, n_threads: int = 0) -> OracleResult:
    """ba.rs:198 `bundle_adjust`; mutates the state arrays of `p` in place."""
    L = lib()
    cap = max(int(max_iter), 1)
    nc_log = np.zeros(cap, np.float64)
    lam = np.zeros(cap, np.float64)
    pcg = np.zeros(cap, np.int32)
    acc = np.zeros(cap, np.int32)
    st = _Stats()
    st.log_cap = cap
    st.log_new_cost, st.log_lambda = nc_log.ctypes.data, lam.ctypes.data
    st.log_pcg, st.log_accept = pcg.ctypes.data, acc.ctypes.data
    P = _problem(p)
    S = _state(p)
    L.oracle_bundle_adjust(C.byref(P), C.byref(S), int(max_iter), float(sigma_px), int(loss),
                           int(pcg_max_iter), int(n_threads), C.byref(st))
    n = int(st.iterations)
    return OracleResult(
        n, st.initial_rms, st.final_rms, st.initial_cost, st.final_cost,
        nc_log[:n].copy(), lam[:n].copy(), pcg[:n].copy(), acc[:n].copy(),
        dict(linearise=st.t_linearise, point=st.t_point, assembly=st.t_assembly,
             schur=st.t_schur, pcg=st.t_pcg, backsub=st.t_backsub, cost=st.t_cost,
             total=st.t_total))


def set_spmv_shuffle(seed: int) -> None:
    """Permute each row's block order in the PCG product (seeded), emulating
    the reference's per-run HashMap order; 0 restores the fixed order."""
    lib().oracle_set_spmv_shuffle(int(seed))


def robust_cost(p, sigma_px: float, loss: int = LOSS_CAUCHY):
    """ba.rs:103 `robust_cost` → (cost incl. priors, rms, n in front)."""
    c, r, n = C.c_double(), C.c_double(), C.c_int64()
    P, S = _problem(p), _state(p)
    lib().oracle_robust_cost(C.byref(P), C.byref(S), float(sigma_px), int(loss), C.byref(c),
                             C.byref(r), C.byref(n))
    return c.value, r.value, n.value


def linearise(p, sigma_px: float, loss: int = LOSS_CAUCHY):
    """ba.rs:56 `linearise` for every observation."""
    no = p.obs_cam.shape[0]
    e = np.zeros((no, 2))
    jc = np.zeros((no, 2, 6))
    jg = np.zeros((no, 2, 3))
    jp = np.zeros((no, 2, 3))
    w = np.zeros(no)
    valid = np.zeros(no, np.uint8)
    P, S = _problem(p), _state(p)
    lib().oracle_linearise(C.byref(P), C.byref(S), float(sigma_px), int(loss), e.ctypes.data,
                           jc.ctypes.data, jg.ctypes.data, jp.ctypes.data, w.ctypes.data,
                           valid.ctypes.data)
    return dict(e=e, jc=jc, jg=jg, jp=jp, w=w, valid=valid.astype(bool))


class _OwnedState:
    def __init__(self, p):
        self.rot = np.empty_like(p.rot)
        self.center = np.empty_like(p.center)
        self.intr = np.empty_like(p.intr)
        self.points = np.empty_like(p.points)


def lm_step(p, lam: float, sigma_px: float, *, loss: int = LOSS_CAUCHY,
            pcg_max_iter: int = 400, dense: bool = True):
    """One LM system at damping `lam` (ba.rs:221-366) without acceptance.

    Returns S (dense, if asked), g, dx, has_sys, pcg iterations, the trial
    state and its cost; `p` is not modified."""
    nc, ng = p.rot.shape[0], p.intr.shape[0]
    nb = nc + ng
    S = np.zeros((6 * nb, 6 * nb)) if dense else None
    g = np.zeros(6 * nb)
    dx = np.zeros(6 * nb)
    has = np.zeros(p.points.shape[0], np.uint8)
    it = C.c_int32()
    trial = _OwnedState(p)
    tc = C.c_double()
    P, St, T = _problem(p), _state(p), _state(trial)
    lib().oracle_lm_step(C.byref(P), C.byref(St), float(lam), float(sigma_px), int(loss),
                         int(pcg_max_iter), _ptr(S), g.ctypes.data, dx.ctypes.data,
                         has.ctypes.data, C.byref(it), C.byref(T), C.byref(tc))
    return dict(S=S, g=g, dx=dx, has_sys=has.astype(bool), pcg_iters=it.value, trial=trial,
                trial_cost=tc.value)


def exp_so3(w) -> np.ndarray:
    w = np.ascontiguousarray(w, np.float64)
    R = np.zeros((3, 3))
    lib().oracle_exp_so3(w.ctypes.data, R.ctypes.data)
    return R


def from_angles(yaw, pitch, roll=0.0) -> np.ndarray:
    R = np.zeros((3, 3))
    lib().oracle_from_angles(float(yaw), float(pitch), float(roll), R.ctypes.data)
    return R


def project(R, Cc, K, X):
    R, Cc, K, X = (np.ascontiguousarray(a, np.float64) for a in (R, Cc, K, X))
    u = np.zeros(2)
    ok = lib().oracle_project(R.ctypes.data, Cc.ctypes.data, K.ctypes.data, X.ctypes.data,
                              u.ctypes.data)
    return u if ok else None


def undistort(K, u):
    K, u = np.ascontiguousarray(K, np.float64), np.ascontiguousarray(u, np.float64)
    p = np.zeros(2)
    lib().oracle_undistort(K.ctypes.data, u.ctypes.data, p.ctypes.data)
    return p


class RefSurvey:
    """The problem of ba.rs:400-481 (`recovers_perturbed_survey`)."""

    def __init__(self):
        L = lib()
        cap_o = 18000
        self.obs_cam = np.zeros(cap_o, np.uint32)
        self.obs_pt = np.zeros(cap_o, np.uint32)
        self.obs_uv = np.zeros((cap_o, 2))
        self.prior_mask = np.zeros(12, np.uint8)
        self.prior = np.zeros((12, 6))
        self.rot = np.zeros((12, 3, 3))
        self.center = np.zeros((12, 3))
        self.intr = np.zeros((1, 5))
        pts = np.zeros((1500, 3))
        self.points = pts
        st = _State(self.rot.ctypes.data, self.center.ctypes.data, self.intr.ctypes.data,
                    pts.ctypes.data)
        npt, no, ft = C.c_int32(), C.c_int32(), C.c_double()
        L.oracle_make_ref_survey(self.obs_cam.ctypes.data, self.obs_pt.ctypes.data,
                                 self.obs_uv.ctypes.data, self.prior_mask.ctypes.data,
                                 self.prior.ctypes.data, C.byref(st), C.byref(npt),
                                 C.byref(no), C.byref(ft))
        n, m = npt.value, no.value
        self.points = np.ascontiguousarray(pts[:n])
        self.obs_cam = np.ascontiguousarray(self.obs_cam[:m])
        self.obs_pt = np.ascontiguousarray(self.obs_pt[:m])
        self.obs_uv = np.ascontiguousarray(self.obs_uv[:m])
        self.cam_group = np.zeros(12, np.uint32)
        self.refine_intrinsics = True
        self.f_true = ft.value


def triangulate(track_ptr, obs_cam, obs_uv, rot, center, intr, cam_group, thr: float,
                n_threads: int = 0):
    """sparse.rs:389-421 restated: (kept bool[nt], points [nt, 3], good bool[no])."""
    L = lib()
    nt = len(track_ptr) - 1
    kept = np.zeros(nt, np.uint8)
    pts = np.zeros((nt, 3))
    good = np.zeros(len(obs_cam), np.uint8)
    f = L.oracle_triangulate
    f.restype = C.c_int64
    f.argtypes = [C.c_int64] + [C.c_void_p] * 7 + [C.c_double, C.c_void_p, C.c_void_p,
                                                    C.c_void_p, C.c_int]
    tp = np.ascontiguousarray(track_ptr, np.uint32)
    oc = np.ascontiguousarray(obs_cam, np.uint32)
    uv = np.ascontiguousarray(obs_uv, np.float64)
    R = np.ascontiguousarray(rot, np.float64)
    Cc = np.ascontiguousarray(center, np.float64)
    K = np.ascontiguousarray(intr, np.float64)
    cg = np.ascontiguousarray(cam_group, np.uint32)
    f(nt, tp.ctypes.data, oc.ctypes.data, uv.ctypes.data, R.ctypes.data, Cc.ctypes.data,
      K.ctypes.data, cg.ctypes.data, float(thr), kept.ctypes.data, pts.ctypes.data,
      good.ctypes.data, int(n_threads or L.oracle_max_threads()))
    return kept.astype(bool), pts, good.astype(bool)


def sparse_summary(obs_cam, obs_pt, rot, center, points, agl: float, max_neighbours: int = 8):
    """sparse.rs:470-483, 515-533 and mod.rs:31-35 restated: (neighbours
    u32[nc, k], shared u32[nc, k], n_neighbours i32[nc], depth_range [nc, 2],
    points_f32 [np, 3])."""
    L = lib()
    f = L.oracle_sparse_summary
    f.restype = None
    f.argtypes = [C.c_int64] * 3 + [C.c_void_p] * 5 + [C.c_int, C.c_double] + [C.c_void_p] * 5
    oc = np.ascontiguousarray(obs_cam, np.uint32)
    op = np.ascontiguousarray(obs_pt, np.uint32)
    R = np.ascontiguousarray(rot, np.float64)
    Cc = np.ascontiguousarray(center, np.float64)
    X = np.ascontiguousarray(points, np.float64)
    nc, npts, k = len(Cc.reshape(-1, 3)), len(X.reshape(-1, 3)), int(max_neighbours)
    nb = np.zeros((nc, k), np.uint32)
    sh = np.zeros((nc, k), np.uint32)
    n_nb = np.zeros(nc, np.int32)
    rng = np.zeros((nc, 2))
    p32 = np.zeros((npts, 3), np.float32)
    f(nc, npts, len(oc), oc.ctypes.data, op.ctypes.data, R.ctypes.data, Cc.ctypes.data,
      X.ctypes.data, k, float(agl), nb.ctypes.data, sh.ctypes.data, n_nb.ctypes.data,
      rng.ctypes.data, p32.ctypes.data)
    return nb, sh, n_nb, rng, p32


def ransac_fundamental(match_ptr, uv, seed, thresh: float, iters: int = 600, n_threads: int = 0):
    """geometry.rs:248-300 per pair: (inlier bool[n_matches], n_inliers
    i32[n_pairs], best hypothesis i32[n_pairs] (-1: none), refit bool)."""
    L = lib()
    f = L.oracle_ransac_fundamental
    f.restype = None
    f.argtypes = [C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_int,
                  C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
    mp = np.ascontiguousarray(match_ptr, np.uint32)
    U = np.ascontiguousarray(uv, np.float64)
    sd = np.ascontiguousarray(seed, np.uint64)
    npairs = len(mp) - 1
    inl = np.zeros(int(mp[-1]) if npairs >= 0 else 0, np.uint8)
    n_inl = np.zeros(npairs, np.int32)
    best = np.zeros(npairs, np.int32)
    refit = np.zeros(npairs, np.uint8)
    f(npairs, mp.ctypes.data, U.ctypes.data, sd.ctypes.data, float(thresh), int(iters),
      inl.ctypes.data, n_inl.ctypes.data, best.ctypes.data, refit.ctypes.data,
      int(n_threads or L.oracle_max_threads()))
    return inl.astype(bool), n_inl, best, refit.astype(bool)


def pair_fits(pair_cam, match_ptr, uv, rot, center, intr, cam_group, n_threads: int = 0):
    """sparse.rs:620-645 per pair: median Sampson error in pixels."""
    L = lib()
    f = L.oracle_pair_fits
    f.restype = None
    f.argtypes = [C.c_int64] + [C.c_void_p] * 8 + [C.c_int]
    pc = np.ascontiguousarray(pair_cam, np.uint32)
    mp = np.ascontiguousarray(match_ptr, np.uint32)
    U = np.ascontiguousarray(uv, np.float64)
    R = np.ascontiguousarray(rot, np.float64)
    Cc = np.ascontiguousarray(center, np.float64)
    K = np.ascontiguousarray(intr, np.float64)
    cg = np.ascontiguousarray(cam_group, np.uint32)
    npairs = len(mp) - 1
    med = np.zeros(npairs)
    f(npairs, pc.ctypes.data, mp.ctypes.data, U.ctypes.data, R.ctypes.data, Cc.ctypes.data,
      K.ctypes.data, cg.ctypes.data, med.ctypes.data, int(n_threads or L.oracle_max_threads()))
    return med


def ransac_kat_correspondences():
    """The correspondences of geometry.rs:355-381 (`fundamental_ransac_
    separates_inliers`): two cameras over a 60 x 50 x 15 m volume, LCG from
    seed 7 (s = s * 6364136223846793005 + 1, value (s >> 33) / 2^31 - 0.5),
    every fourth candidate's second view replaced by a random pixel.
    Returns (uv [n, 4], true-inlier mask)."""
    K = np.array([3000.0, 2000.0, 1500.0, -0.02, 0.005])
    Ra, Ca = from_angles(0.0, -90.0, 0.0), np.array([0.0, 0.0, 80.0])
    Rb, Cb = from_angles(5.0, -88.0, 0.0), np.array([25.0, 3.0, 81.0])
    s = [7]
    M = (1 << 64) - 1

    def r():
        s[0] = (s[0] * 6364136223846793005 + 1) & M
        return (s[0] >> 33) / float(1 << 31) - 0.5

    rows, true = [], []
    for i in range(200):
        x0 = r() * 60.0 + 12.0
        x1 = r() * 50.0
        x2 = r() * 15.0
        X = np.array([x0, x1, x2])
        ua, ub = project(Ra, Ca, K, X), project(Rb, Cb, K, X)
        if ua is None or ub is None:
            continue
        if i % 4 == 0:
            b0 = r() * 4000.0 + 2000.0
            b1 = r() * 3000.0 + 1500.0
            rows.append([ua[0], ua[1], b0, b1])
        else:
            rows.append([ua[0], ua[1], ub[0], ub[1]])
        true.append(i % 4 != 0)
    return np.array(rows), np.array(true)
