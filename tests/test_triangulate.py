"""Triangulation and reprojection gating of a sparse-stage round
(sparse.rs:389-421, geometry.rs:115-156): the oracle's restatement on the
CPU, and the GPU kernel and on-device problem build against it."""
import numpy as np
import pytest

import ba_oracle as O
import stitch_ba
from stitch_ba import Options, Tracks, survey


def survey_tracks(seed=1, **kw):
    """A survey's observations grouped by point are its tracks."""
    p, t = survey.generate("lawnmower77", seed=seed, **kw)
    cnt = np.bincount(p.obs_pt, minlength=p.n_points)
    tp = np.concatenate([[0], np.cumsum(cnt)]).astype(np.uint32)
    return p, t, tp


def test_oracle_recovers_points_from_true_cameras():
    p, t, tp = survey_tracks()
    k, X, g = O.triangulate(tp, p.obs_cam, p.obs_uv, t.rot, t.center, t.intr, p.cam_group, 4.0)
    assert k.mean() > 0.5
    err = np.linalg.norm(X[k] - t.points[k], axis=1)
    assert np.median(err) < 0.05   # 0.5 px noise at 80 m
    # kept tracks keep at least two observations; dropped tracks keep none
    per = np.add.reduceat(g.astype(np.int64), tp[:-1])
    assert (per[k] >= 2).all() and (per[~k] == 0).all()


def test_oracle_ray_angle_gate():
    """Two views 1 m apart at 80 m (0.7 degrees) fail the 6-degree gate for
    two-view points; 20 m apart (14 degrees) pass (sparse.rs:411-415)."""
    R = O.from_angles(0.0, -90.0, 0.0)
    K = np.array([[3650.0, 2736.0, 1824.0, 0.0, 0.0]])
    X = np.array([1.0, 2.0, 0.0])
    for dx, want in [(1.0, False), (20.0, True)]:
        C = np.array([[0.0, 0.0, 80.0], [dx, 0.0, 80.0]])
        uv = np.array([O.project(R, C[i], K[0], X) for i in range(2)])
        k, Xt, g = O.triangulate(np.array([0, 2], np.uint32), np.array([0, 1], np.uint32), uv,
                                 np.stack([R, R]), C, K, np.zeros(2, np.uint32), 4.0)
        assert k[0] == want
        if want:
            assert np.abs(Xt[0] - X).max() < 1e-6


@pytest.mark.gpu
@pytest.mark.parametrize("thr", [200.0, 10.0])
def test_gpu_triangulation_matches_oracle(thr):
    p, t, tp = survey_tracks()
    tr = Tracks(tp, p.obs_cam, p.obs_uv, p.cam_group, 1)
    k, X, g = stitch_ba.triangulate(tr, p.rot, p.center, p.intr, thr)
    ko, Xo, go = O.triangulate(tp, p.obs_cam, p.obs_uv, p.rot, p.center, p.intr, p.cam_group, thr)
    assert (k == ko).mean() > 1 - 1e-4           # threshold ties aside
    both = k & ko
    scale = np.abs(Xo[both]).max()
    assert np.abs(X[both] - Xo[both]).max() <= 1e-8 * scale
    obs_both = np.repeat(both, np.diff(tp))
    assert (g[obs_both] == go[obs_both]).all()


@pytest.mark.gpu
def test_upload_tracks_builds_the_same_problem():
    """Device triangulation + problem build + solve equals the host path:
    oracle triangulation, host-built Problem (sparse.rs:429-449), solve."""
    p, t, tp = survey_tracks(seed=2, n_cams=24, n_points=6000)
    tr = Tracks(tp, p.obs_cam, p.obs_uv, p.cam_group, 1)
    thr = 40.0
    with stitch_ba.Context() as ctx:
        n_pts, n_obs = ctx.upload_tracks(tr, p.rot, p.center, p.intr, thr,
                                         prior_mask=p.prior_mask, prior=p.prior)
        a = ctx.solve(30, thr / 2.0)[0]
    k, X, g = O.triangulate(tp, p.obs_cam, p.obs_uv, p.rot, p.center, p.intr, p.cam_group, thr)
    assert n_pts == int(k.sum()) and n_obs == int(g.sum())
    kept_idx = np.cumsum(k) - 1
    obs_track = np.repeat(np.arange(len(k)), np.diff(tp))
    sel = g
    q = stitch_ba.Problem(intr=p.intr.copy(), rot=p.rot.copy(), center=p.center.copy(),
                          cam_group=p.cam_group, points=np.ascontiguousarray(X[k]),
                          obs_cam=np.ascontiguousarray(p.obs_cam[sel]),
                          obs_pt=np.ascontiguousarray(kept_idx[obs_track[sel]].astype(np.uint32)),
                          obs_uv=np.ascontiguousarray(p.obs_uv[sel]), prior_mask=p.prior_mask,
                          prior=p.prior, refine_intrinsics=True)
    st, b = stitch_ba.bundle_adjust(q, 30, thr / 2.0, return_info=True)
    assert a.iterations == b.iterations
    assert abs(a.initial_cost - b.initial_cost) <= 1e-9 * b.initial_cost
    assert abs(a.final_cost - b.final_cost) <= 1e-6 * b.final_cost
