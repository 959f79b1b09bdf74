"""Seeded synthetic aerial surveys (libba_survey.so) and the benchmark presets.

The presets are the workloads the solver is measured on:

* ``lawnmower77``  — 77 nadir cameras at 80 m, 5472x3648 px, f ≈ 3650 px,
  40k points on a ±5 m sinusoidal heightfield, ≈250k observations,
  N(0, 0.5 px) noise plus 5% uniform outliers, GPS priors σ = (2, 2, 4) m,
  poses perturbed by 0.5° / 1 m.  Tracks with fewer than two inlier
  observations are not emitted (the sparse stage's gating, sparse.rs:389-421,
  drops them before bundle adjustment); outliers in kept tracks stay.
* ``single500``    — 500 cameras, 400k points, ≈3M observations.
* ``oblique2000``  — 2,000 cameras (30% on a 45° oblique edge ring), 2M
  points, ≈15M observations.
* ``batched64``    — 64 independent models, cameras ~ U[20, 800], each
  camera observing ~U[500, 1000] points.
* ``large5000``    — 5,000 cameras, 6M points, ≈45M observations.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, fields, replace

import numpy as np

from . import _build
from .problem import Problem


class _Params(C.Structure):
    _fields_ = [
        ("seed", C.c_uint64), ("n_cams", C.c_int32), ("n_points", C.c_int32),
        ("altitude", C.c_double), ("width", C.c_int32), ("height", C.c_int32),
        ("f", C.c_double), ("cx", C.c_double), ("cy", C.c_double), ("k_range", C.c_double),
        ("along_overlap", C.c_double), ("across_overlap", C.c_double),
        ("oblique_frac", C.c_double), ("oblique_pitch", C.c_double),
        ("tilt_jitter_deg", C.c_double), ("terrain_amp", C.c_double),
        ("terrain_wavelength", C.c_double), ("noise_px", C.c_double),
        ("outlier_frac", C.c_double), ("prior_sigma_h", C.c_double),
        ("prior_sigma_v", C.c_double), ("rot_perturb_deg", C.c_double),
        ("centre_perturb_m", C.c_double), ("point_perturb_m", C.c_double),
        ("f_scale_init", C.c_double), ("refine_intrinsics", C.c_int32),
        ("min_inlier_views", C.c_int32),
    ]


class _Arrays(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in (
        "obs_cam", "obs_pt", "obs_uv", "cam_group", "prior_mask", "prior", "rot", "center",
        "intr", "points", "true_rot", "true_center", "true_intr", "true_points")]


@dataclass(frozen=True)
class SurveyParams:
    seed: int = 1
    n_cams: int = 77
    n_points: int = 40_000
    altitude: float = 80.0
    width: int = 5472
    height: int = 3648
    f: float = 3650.0
    cx: float = 2736.0
    cy: float = 1824.0
    k_range: float = 0.05
    along_overlap: float = 0.75
    across_overlap: float = 0.45
    oblique_frac: float = 0.0
    oblique_pitch: float = -45.0
    tilt_jitter_deg: float = 1.0
    terrain_amp: float = 5.0
    terrain_wavelength: float = 100.0
    noise_px: float = 0.5
    outlier_frac: float = 0.05
    prior_sigma_h: float = 2.0
    prior_sigma_v: float = 4.0
    rot_perturb_deg: float = 0.5
    centre_perturb_m: float = 1.0
    point_perturb_m: float = 1.0
    f_scale_init: float = 1.03
    refine_intrinsics: bool = True
    # A track reaches bundle adjustment only if the round's gating keeps two
    # or more of its observations (sparse.rs:389-421); tracks with fewer
    # inlier observations are not emitted (0: emit every track).
    min_inlier_views: int = 2


PRESETS = {
    "lawnmower77": SurveyParams(n_cams=77, n_points=40_000, along_overlap=0.79,
                                across_overlap=0.45),
    "single500": SurveyParams(n_cams=500, n_points=400_000, along_overlap=0.795,
                              across_overlap=0.44),
    "oblique2000": SurveyParams(n_cams=2000, n_points=2_000_000, along_overlap=0.5,
                                across_overlap=0.2, oblique_frac=0.30),
    "large5000": SurveyParams(n_cams=5000, n_points=6_000_000, along_overlap=0.79,
                              across_overlap=0.42),
}

_lib = None


def _survey_lib():
    global _lib
    if _lib is None:
        L = C.CDLL(_build.build_survey())
        L.survey_generate.restype = C.c_void_p
        L.survey_generate.argtypes = [C.POINTER(_Params)]
        L.survey_sizes.argtypes = [C.c_void_p] + [C.POINTER(C.c_int64)] * 3
        L.survey_copy.argtypes = [C.c_void_p, C.POINTER(_Arrays)]
        L.survey_free.argtypes = [C.c_void_p]
        _lib = L
    return _lib


@dataclass
class Truth:
    rot: np.ndarray
    center: np.ndarray
    intr: np.ndarray
    points: np.ndarray


def generate(params: SurveyParams | str = "lawnmower77", **overrides) -> tuple[Problem, Truth]:
    """Generate a survey; returns (problem with the perturbed initial state, truth)."""
    if isinstance(params, str):
        params = PRESETS[params]
    if overrides:
        params = replace(params, **overrides)
    L = _survey_lib()
    P = _Params(**{f.name: (int(getattr(params, f.name))
                            if f.name in ("refine_intrinsics", "min_inlier_views")
                            else getattr(params, f.name)) for f in fields(params)})
    h = L.survey_generate(C.byref(P))
    if not h:
        raise ValueError(f"survey generation failed for {params}")
    try:
        nc, npt, no = C.c_int64(), C.c_int64(), C.c_int64()
        L.survey_sizes(h, C.byref(nc), C.byref(npt), C.byref(no))
        nc, npt, no = nc.value, npt.value, no.value
        p = Problem.empty(nc, npt, no, 1, refine_intrinsics=params.refine_intrinsics)
        t = Truth(np.zeros((nc, 3, 3)), np.zeros((nc, 3)), np.zeros((1, 5)), np.zeros((npt, 3)))
        A = _Arrays(*[a.ctypes.data for a in (
            p.obs_cam, p.obs_pt, p.obs_uv, p.cam_group, p.prior_mask, p.prior, p.rot, p.center,
            p.intr, p.points, t.rot, t.center, t.intr, t.points)])
        L.survey_copy(h, C.byref(A))
    finally:
        L.survey_free(h)
    return p, t


def batched_models(n_models: int = 64, seed: int = 1, cam_range=(20, 800),
                   ppc_range=(500, 1000), views_per_point: float = 6.5,
                   base: SurveyParams | None = None):
    """Independent models of uneven size (the batched workload).

    Model m has cameras ~ U[cam_range] and each camera observes ~U[ppc_range]
    points, i.e. points ≈ cameras × ppc / views_per_point."""
    base = base or PRESETS["single500"]
    rs = np.random.default_rng(seed)
    out = []
    for m in range(n_models):
        nc = int(rs.integers(cam_range[0], cam_range[1] + 1))
        ppc = int(rs.integers(ppc_range[0], ppc_range[1] + 1))
        npt = max(50, int(math.ceil(nc * ppc / views_per_point)))
        out.append(generate(replace(base, seed=seed * 1000 + m, n_cams=nc, n_points=npt)))
    return out


def pair_matches(p: Problem, min_shared: int = 30, outlier_frac: float = 0.25, seed: int = 0,
                 max_pairs: int | None = None, width: int = 5472, height: int = 3648):
    """Putative matches of the photo pairs of a survey (the input of the
    sparse stage's per-pair RANSAC, sparse.rs:262-300): every pair of cameras
    (i < j) sharing at least `min_shared` points, with one correspondence
    per shared point (the two observations, in point order), and a fraction
    `outlier_frac` of them turned into mismatches by a uniformly random
    second pixel.  Returns a PairMatches (seeds default to i * 7919 + j)."""
    from .ba import PairMatches
    rng = np.random.default_rng(seed)
    cnt = np.bincount(p.obs_pt, minlength=p.n_points)
    start = np.concatenate([[0], np.cumsum(cnt)])[:-1]
    ia, ib = [], []
    for m in range(2, int(cnt.max(initial=0)) + 1):
        pts = np.nonzero(cnt == m)[0]
        if len(pts) == 0:
            continue
        r, c = np.triu_indices(m, 1)
        base = start[pts][:, None]
        ia.append((base + r[None, :]).reshape(-1))
        ib.append((base + c[None, :]).reshape(-1))
    ia = np.concatenate(ia) if ia else np.zeros(0, np.int64)
    ib = np.concatenate(ib) if ib else np.zeros(0, np.int64)
    ca, cb = p.obs_cam[ia].astype(np.int64), p.obs_cam[ib].astype(np.int64)
    swap = ca > cb
    ia, ib = np.where(swap, ib, ia), np.where(swap, ia, ib)
    ca, cb = np.minimum(ca, cb), np.maximum(ca, cb)
    key = ca * p.n_cams + cb
    order = np.lexsort((p.obs_pt[ia], key))
    ia, ib, key = ia[order], ib[order], key[order]
    uk, first, counts = np.unique(key, return_index=True, return_counts=True)
    keep = counts >= min_shared
    if max_pairs is not None:
        keep &= np.cumsum(keep) <= max_pairs
    sel = np.repeat(keep, counts)
    ia, ib = ia[sel], ib[sel]
    counts = counts[keep]
    pair_cam = np.stack([uk[keep] // p.n_cams, uk[keep] % p.n_cams], 1).astype(np.uint32)
    uv = np.concatenate([p.obs_uv[ia], p.obs_uv[ib]], 1)
    bad = rng.random(len(uv)) < outlier_frac
    uv[bad, 2] = rng.uniform(0, width, bad.sum())
    uv[bad, 3] = rng.uniform(0, height, bad.sum())
    match_ptr = np.concatenate([[0], np.cumsum(counts)]).astype(np.uint32)
    return PairMatches(np.ascontiguousarray(pair_cam), match_ptr, np.ascontiguousarray(uv))
