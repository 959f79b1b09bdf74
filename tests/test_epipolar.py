"""Epipolar geometry before bundle adjustment: fundamental-matrix RANSAC
(geometry.rs:159-300, called per pair at sparse.rs:290) and the pair check
pair_fits (sparse.rs:620-645).  The oracle is pinned by the reference's own
known-answer test (geometry.rs:355-381); the GPU path is checked against the
oracle on survey pairs."""
import numpy as np
import pytest

import ba_oracle as O
import stitch_ba
from stitch_ba import PairMatches, survey

F64_MAX = np.finfo(np.float64).max


def kat_pairs():
    uv, true = O.ransac_kat_correspondences()
    return PairMatches(np.zeros((1, 2), np.uint32), np.array([0, len(uv)], np.uint32),
                       np.ascontiguousarray(uv), np.array([3], np.uint64)), true


def survey_pairs(seed=1, **kw):
    p, t = survey.generate("lawnmower77", seed=seed)
    return p, t, survey.pair_matches(p, seed=seed, **kw)


def seeds_of(pm):
    return pm.pair_cam[:, 0].astype(np.uint64) * np.uint64(7919) + pm.pair_cam[:, 1]


# ---- oracle pins -----------------------------------------------------------------

def test_oracle_ransac_known_answer():
    """geometry.rs:375-383: with threshold 2 px, 600 iterations, seed 3, the
    inliers found are within [0.9, 1] x the true inliers + 3."""
    pm, true = kat_pairs()
    inl, n, best, refit = O.ransac_fundamental(pm.match_ptr, pm.uv, pm.seed, 2.0, 600)
    true_inl = int(true.sum())
    assert true_inl * 9 // 10 <= n[0] <= true_inl + 3
    assert (inl & true).sum() >= true_inl * 9 // 10


def test_oracle_ransac_rules():
    pm, _ = kat_pairs()
    uv = pm.uv
    # fewer than 12 correspondences: no model; none at all; zero iterations
    mp = np.array([0, 11, 11, len(uv)], np.uint32)
    inl, n, best, refit = O.ransac_fundamental(mp, uv, np.array([3, 3, 3], np.uint64), 2.0, 600)
    assert n[0] == 0 and best[0] == -1 and not inl[:11].any()
    assert n[1] == 0 and best[1] == -1
    assert n[2] > 100 and best[2] >= 0
    inl, n, best, refit = O.ransac_fundamental(pm.match_ptr, uv, pm.seed, 2.0, 0)
    assert n[0] == 0 and best[0] == -1 and not refit[0]
    # the seed is what changes the sample (seed | 1: 2 and 3 are the same stream)
    a = O.ransac_fundamental(pm.match_ptr, uv, np.array([2], np.uint64), 2.0, 50)
    b = O.ransac_fundamental(pm.match_ptr, uv, np.array([3], np.uint64), 2.0, 50)
    assert a[2][0] == b[2][0] and np.array_equal(a[0], b[0])


def sampson_py(E, x1, x2):
    a = np.array([x1[0], x1[1], 1.0])
    b = np.array([x2[0], x2[1], 1.0])
    fx1, ftx2 = E @ a, E.T @ b
    e = b @ fx1
    d = fx1[0] ** 2 + fx1[1] ** 2 + ftx2[0] ** 2 + ftx2[1] ** 2
    return F64_MAX if d < 1e-18 else e * e / d


def test_oracle_pair_fits_matches_numpy():
    p, t, pm = survey_pairs(max_pairs=6)
    med = O.pair_fits(pm.pair_cam, pm.match_ptr, pm.uv, p.rot, p.center, p.intr, p.cam_group)
    K = p.intr[0]
    for q in range(6):
        a, b = pm.pair_cam[q]
        Ra, Rb = p.rot[a].reshape(3, 3), p.rot[b].reshape(3, 3)
        tt = Rb @ (p.center[a] - p.center[b])
        S = np.array([[0, -tt[2], tt[1]], [tt[2], 0, -tt[0]], [-tt[1], tt[0], 0]])
        E = S @ (Rb @ Ra.T)
        errs = sorted(np.sqrt(sampson_py(E, O.undistort(K, u[:2]), O.undistort(K, u[2:]))) * K[0]
                      for u in pm.uv[pm.match_ptr[q]:pm.match_ptr[q + 1]])
        assert abs(med[q] - errs[len(errs) // 2]) <= 1e-9 * errs[len(errs) // 2]
    # true poses fit to the noise level, perturbed ones do not
    med_t = O.pair_fits(pm.pair_cam, pm.match_ptr, pm.uv, t.rot, t.center, t.intr, p.cam_group)
    assert np.median(med_t) < 1.0 < np.median(med)


def test_pair_matches_generator():
    p, _, pm = survey_pairs(max_pairs=20)
    assert len(pm.pair_cam) == 20 and (pm.pair_cam[:, 0] < pm.pair_cam[:, 1]).all()
    assert (np.diff(pm.match_ptr) >= 30).all() and pm.match_ptr[-1] == len(pm.uv)


# ---- GPU against the oracle ------------------------------------------------------

@pytest.mark.gpu
def test_gpu_ransac_known_answer():
    pm, true = kat_pairs()
    inl, n, best, refit = stitch_ba.ransac_fundamental(pm, 2.0, 600)
    oi, on, ob, orf = O.ransac_fundamental(pm.match_ptr, pm.uv, pm.seed, 2.0, 600)
    true_inl = int(true.sum())
    assert true_inl * 9 // 10 <= n[0] <= true_inl + 3
    assert best[0] == ob[0] and n[0] == on[0] and np.array_equal(inl, oi)


@pytest.mark.gpu
def test_gpu_ransac_matches_oracle_on_survey_pairs():
    _, _, pm = survey_pairs(max_pairs=300)
    inl, n, best, refit = stitch_ba.ransac_fundamental(pm, 1.5, 600)
    oi, on, ob, orf = O.ransac_fundamental(pm.match_ptr, pm.uv, seeds_of(pm), 1.5, 600)
    same = best == ob
    assert same.mean() >= 0.99, (best[~same], ob[~same])
    diff = np.abs(n - on)
    assert (diff[same] <= 1).all()
    # inlier sets agree up to rounding at the threshold
    flips = np.add.reduceat((inl != oi).astype(np.int64), pm.match_ptr[:-1].astype(np.int64))
    assert (flips[same] <= 1).all() and flips.sum() <= 0.001 * len(inl)


@pytest.mark.gpu
def test_gpu_ransac_edge_cases():
    pm, _ = kat_pairs()
    uv = pm.uv
    mp = np.array([0, 11, 11, 23, len(uv)], np.uint32)
    seeds = np.array([3, 3, 5, 3], np.uint64)
    q = PairMatches(np.zeros((4, 2), np.uint32), mp, uv, seeds)
    inl, n, best, refit = stitch_ba.ransac_fundamental(q, 2.0, 600)
    oi, on, ob, orf = O.ransac_fundamental(mp, uv, seeds, 2.0, 600)
    assert n[0] == 0 and best[0] == -1 and n[1] == 0 and best[1] == -1
    assert np.array_equal(best, ob) and np.array_equal(n, on) and np.array_equal(inl, oi)
    inl, n, best, refit = stitch_ba.ransac_fundamental(q, 2.0, 0)
    assert (n == 0).all() and (best == -1).all() and not inl.any()
    with pytest.raises(stitch_ba.BaError):
        stitch_ba.ransac_fundamental(PairMatches(q.pair_cam, mp[::-1].copy(), uv, seeds), 2.0, 10)
    # default seeds are i * 7919 + j of pair_cam
    pc = np.array([[3, 7]], np.uint32)
    a = stitch_ba.ransac_fundamental(PairMatches(pc, pm.match_ptr, uv), 2.0, 100)
    b = stitch_ba.ransac_fundamental(PairMatches(pc, pm.match_ptr, uv,
                                                 np.array([3 * 7919 + 7], np.uint64)), 2.0, 100)
    assert a[2][0] == b[2][0] and np.array_equal(a[0], b[0])


@pytest.mark.gpu
def test_gpu_pair_fits_matches_oracle():
    p, t, pm = survey_pairs()
    for rot, center, intr in ((p.rot, p.center, p.intr), (t.rot, t.center, t.intr)):
        med = stitch_ba.pair_fits(pm, rot, center, intr, p.cam_group)
        ref = O.pair_fits(pm.pair_cam, pm.match_ptr, pm.uv, rot, center, intr, p.cam_group)
        assert np.abs(med - ref).max() <= 1e-9 * np.abs(ref).max()
    # a pair without matches is never kept (f64::MAX)
    q = PairMatches(pm.pair_cam[:2].copy(), np.array([0, 0, 40], np.uint32),
                    np.ascontiguousarray(pm.uv[:40]))
    med = stitch_ba.pair_fits(q, p.rot, p.center, p.intr, p.cam_group)
    assert med[0] == F64_MAX and med[1] < F64_MAX
    with pytest.raises(stitch_ba.BaError):
        bad = PairMatches(np.array([[0, 999]], np.uint32), np.array([0, 40], np.uint32),
                          np.ascontiguousarray(pm.uv[:40]))
        stitch_ba.pair_fits(bad, p.rot, p.center, p.intr, p.cam_group)
