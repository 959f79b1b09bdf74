"""Synthetic survey generator: determinism, sizes, invariants.  CPU only."""
import numpy as np
import pytest

import ba_oracle as O
from stitch_ba import survey


def test_deterministic_and_sorted():
    a, ta = survey.generate("lawnmower77", n_points=3000)
    b, tb = survey.generate("lawnmower77", n_points=3000)
    assert np.array_equal(a.obs_uv, b.obs_uv) and np.array_equal(a.points, b.points)
    assert np.all(np.diff(a.obs_pt.astype(np.int64)) >= 0)
    m = np.bincount(a.obs_pt, minlength=a.n_points)
    assert m.min() >= 2


def test_lawnmower77_matches_the_configured_sizes():
    p, t = survey.generate("lawnmower77")
    assert p.n_cams == 77 and p.n_points == 40_000
    assert 200_000 < p.n_obs < 300_000  # ~250k observations


def test_truth_reprojects_inliers_within_noise():
    p, t = survey.generate("lawnmower77", n_points=2000, outlier_frac=0.0)
    res = []
    for k in range(0, p.n_obs, 7):
        c, j = p.obs_cam[k], p.obs_pt[k]
        u = O.project(t.rot[c], t.center[c], t.intr[0], t.points[j])
        res.append(np.linalg.norm(p.obs_uv[k] - u))
    res = np.array(res)
    assert 0.3 < np.sqrt(np.mean(res ** 2)) < 1.2  # N(0, 0.5 px) per axis


def test_initial_perturbation():
    p, t = survey.generate("lawnmower77", n_points=1000)
    d = np.linalg.norm(p.center - t.center, axis=1)
    assert np.allclose(d, 1.0, atol=1e-9)
    D = np.einsum("nij,nkj->nik", p.rot, t.rot)
    ang = np.degrees(np.arccos(np.clip((np.trace(D, axis1=1, axis2=2) - 1) / 2, -1, 1)))
    assert np.allclose(ang, 0.5, atol=1e-6)
    assert abs(p.intr[0, 0] / t.intr[0, 0] - 1.03) < 1e-12 and p.intr[0, 3] == 0.0


def test_oblique_ring():
    p, t = survey.generate("lawnmower77", n_cams=100, n_points=5000, oblique_frac=0.3)
    axes = t.rot[:, 2, :]  # viewing direction (camera +z) in world
    nadir = axes[:, 2] < -0.95
    assert nadir.sum() == 70
    tilt = np.degrees(np.arcsin(-axes[~nadir, 2]))
    assert np.all(np.abs(tilt - 45.0) < 2.0)
