"""The oracle (CPU restatement of ba.rs) checked against the reference's own
tests and against independent numerics.  CPU only."""
import numpy as np
import pytest

import ba_oracle as O


def test_reference_known_answer():
    """ba.rs:400-493 `recovers_perturbed_survey`: same generator, same call,
    same assertions."""
    p = O.RefSurvey()
    r = O.bundle_adjust(p, 60, 4.0, n_threads=1)
    assert r.initial_rms > 20.0, r
    assert r.final_rms < 0.8, r
    assert abs(p.intr[0, 0] / p.f_true - 1.0) < 0.025, p.intr


def test_from_angles_convention():
    """geometry.rs:318-332."""
    R = O.from_angles(90.0, -90.0, 0.0)
    axis = R[2]  # Pose::axis = row 2 of R
    assert np.abs(axis - [0, 0, -1]).max() < 1e-9
    r_wc = R.T
    assert np.abs(-r_wc[:, 1] - [1, 0, 0]).max() < 1e-9
    assert np.abs(r_wc[:, 0] - [0, -1, 0]).max() < 1e-9
    K = np.array([3000.0, 2000.0, 1500.0, -0.02, 0.005])
    u = O.project(R, np.array([0.0, 0.0, 100.0]), K, np.array([10.0, 0.0, 0.0]))
    assert u is not None and u[1] < 1500.0 and abs(u[0] - 2000.0) < 1e-6
    Ro = O.from_angles(0.0, -45.0, 0.0)
    assert np.abs(Ro[2] - [0, np.sqrt(0.5), -np.sqrt(0.5)]).max() < 1e-9


def test_distortion_round_trip():
    """geometry.rs:334-339 (undistort(distort(p)) within 1e-9)."""
    K = np.array([3000.0, 2000.0, 1500.0, -0.02, 0.005])
    p = np.array([0.31, -0.22])
    r2 = p @ p
    d = 1 + K[3] * r2 + K[4] * r2 * r2
    u = np.array([K[0] * d * p[0] + K[1], K[0] * d * p[1] + K[2]])
    assert np.abs(O.undistort(K, u) - p).max() < 1e-9


def test_exp_so3_small_angle_branch():
    w = np.array([1e-13, -2e-13, 3e-13])
    R = O.exp_so3(w)
    assert np.abs(R - (np.eye(3) + np.array([[0, -w[2], w[1]], [w[2], 0, -w[0]],
                                               [-w[1], w[0], 0]]))).max() == 0.0
    R = O.exp_so3(np.array([0.3, -0.2, 0.1]))
    assert np.abs(R @ R.T - np.eye(3)).max() < 1e-14


def _residual(p, k):
    cam, pt = p.obs_cam[k], p.obs_pt[k]
    u = O.project(p.rot[cam], p.center[cam], p.intr[p.cam_group[cam]], p.points[pt])
    return p.obs_uv[k] - u


def test_jacobians_match_central_differences():
    """linearise (ba.rs:56-101) against FP64 central differences of the
    residual: rotation as the left perturbation R <- exp(w) R (ba.rs:340),
    centre, point, and (f, k1, k2)."""
    p = O.RefSurvey()
    lin = O.linearise(p, 4.0)
    rng = np.random.default_rng(0)
    for k in rng.choice(len(p.obs_cam), 25, replace=False):
        if not lin["valid"][k]:
            continue
        cam, pt = p.obs_cam[k], p.obs_pt[k]
        Jc, Jp, Jg = lin["jc"][k], lin["jp"][k], lin["jg"][k]
        R0, C0, X0, K0 = p.rot[cam].copy(), p.center[cam].copy(), p.points[pt].copy(), p.intr[0].copy()
        h = 1e-6
        for a in range(3):  # rotation
            w = np.zeros(3)
            w[a] = h
            p.rot[cam] = O.exp_so3(w) @ R0
            ep = _residual(p, k)
            p.rot[cam] = O.exp_so3(-w) @ R0
            em = _residual(p, k)
            p.rot[cam] = R0
            fd = -(ep - em) / (2 * h)  # J = d pred / d param = -d e / d param
            assert np.allclose(fd, Jc[:, a], rtol=1e-5, atol=1e-3), (a, fd, Jc[:, a])
        for a in range(3):  # centre
            p.center[cam, a] = C0[a] + h
            ep = _residual(p, k)
            p.center[cam, a] = C0[a] - h
            em = _residual(p, k)
            p.center[cam] = C0
            assert np.allclose(-(ep - em) / (2 * h), Jc[:, 3 + a], rtol=1e-5, atol=1e-3)
        for a in range(3):  # point
            p.points[pt, a] = X0[a] + h
            ep = _residual(p, k)
            p.points[pt, a] = X0[a] - h
            em = _residual(p, k)
            p.points[pt] = X0
            assert np.allclose(-(ep - em) / (2 * h), Jp[:, a], rtol=1e-5, atol=1e-3)
        for a, idx in enumerate((0, 3, 4)):  # f, k1, k2
            hh = 1e-6 * max(1.0, abs(K0[idx]))
            p.intr[0, idx] = K0[idx] + hh
            ep = _residual(p, k)
            p.intr[0, idx] = K0[idx] - hh
            em = _residual(p, k)
            p.intr[0] = K0
            assert np.allclose(-(ep - em) / (2 * hh), Jg[:, a], rtol=1e-5, atol=1e-3)


def _small_problem():
    p = O.RefSurvey()
    # keep the first 300 points (obs are sorted by point)
    keep = p.obs_pt < 300
    p.obs_cam = np.ascontiguousarray(p.obs_cam[keep])
    p.obs_pt = np.ascontiguousarray(p.obs_pt[keep])
    p.obs_uv = np.ascontiguousarray(p.obs_uv[keep])
    p.points = np.ascontiguousarray(p.points[:300])
    return p


def test_reduced_system_equals_dense_schur_complement():
    """The oracle's reduced system (ba.rs:229-331) against a dense FP64
    construction: the full damped normal matrix, then the Schur complement of
    its point block, built with numpy from the oracle's Jacobians."""
    p = _small_problem()
    lam, sigma = 1e-3, 4.0
    lin = O.linearise(p, sigma)
    nc, npt = p.rot.shape[0], p.points.shape[0]
    ncp = 6 * nc + 3  # cameras + (f, k1, k2)
    H = np.zeros((ncp + 3 * npt, ncp + 3 * npt))
    gvec = np.zeros(ncp + 3 * npt)
    for k in range(len(p.obs_cam)):
        if not lin["valid"][k]:
            continue
        c, j = p.obs_cam[k], p.obs_pt[k]
        J = np.zeros((2, ncp + 3 * npt))
        J[:, 6 * c:6 * c + 6] = lin["jc"][k]
        J[:, 6 * nc:6 * nc + 3] = lin["jg"][k]
        J[:, ncp + 3 * j:ncp + 3 * j + 3] = lin["jp"][k]
        H += lin["w"][k] * J.T @ J
        gvec += lin["w"][k] * J.T @ lin["e"][k]
    for i in range(nc):
        for a in range(3):
            w = 1.0 / p.prior[i, 3 + a] ** 2
            H[6 * i + 3 + a, 6 * i + 3 + a] += w
            gvec[6 * i + 3 + a] += w * (p.prior[i, a] - p.center[i, a])
    d = np.diag(H).copy()
    Hd = H + np.diag(d * lam + 1e-9)
    A = Hd[:ncp, :ncp]
    B = Hd[:ncp, ncp:]
    D = Hd[ncp:, ncp:]
    Dinv = np.linalg.inv(D)  # block diagonal 3x3
    S = A - B @ Dinv @ B.T
    g = gvec[:ncp] - B @ Dinv @ gvec[ncp:]
    r = O.lm_step(p, lam, sigma)
    nb = nc + 1
    So = r["S"].reshape(nb, 6, nb, 6)
    Sd = np.zeros((nb, 6, nb, 6))
    Sd[:nc, :, :nc, :] = S[:6 * nc, :6 * nc].reshape(nc, 6, nc, 6)
    Sd[:nc, :, nc, :3] = S[:6 * nc, 6 * nc:].reshape(nc, 6, 3)
    Sd[nc, :3, :nc, :] = S[6 * nc:, :6 * nc].reshape(3, nc, 6)
    Sd[nc, :3, nc, :3] = S[6 * nc:, 6 * nc:]
    Sd[nc, 3:, nc, 3:] = np.eye(3)  # lens padding (ba.rs:310-314)
    scale = np.abs(Sd).max()
    assert np.abs(So - Sd).max() < 1e-9 * scale
    go = r["g"].reshape(nb, 6)
    assert np.abs(go[:nc].ravel() - g[:6 * nc]).max() < 1e-9 * np.abs(g).max()
    assert np.abs(go[nc, :3] - g[6 * nc:]).max() < 1e-9 * np.abs(g).max()
    assert np.all(go[nc, 3:] == 0.0)


def test_pcg_matches_dense_solve_when_converged():
    p = _small_problem()
    r = O.lm_step(p, 1e-3, 4.0, pcg_max_iter=400)
    S, g, dx = r["S"], r["g"], r["dx"]
    assert r["pcg_iters"] < 400
    xs = np.linalg.solve(S, g)
    assert np.abs(S @ dx - g).max() < 1e-6 * np.abs(g).max()
    assert np.abs(xs - dx).max() < 1e-4 * np.abs(xs).max()


def test_lm_log_is_consistent():
    p = O.RefSurvey()
    r = O.bundle_adjust(p, 60, 4.0, n_threads=1)
    c0 = r.initial_cost
    cost = c0
    for nc, acc in zip(r.new_cost, r.accepted):
        assert bool(acc) == (nc < cost)
        if acc:
            cost = nc
    assert abs(cost - r.final_cost) <= 1e-9 * cost


@pytest.mark.parametrize("threads", [1, 4])
def test_oracle_is_thread_count_stable(threads):
    p = O.RefSurvey()
    r = O.bundle_adjust(p, 8, 4.0, n_threads=threads)
    q = O.RefSurvey()
    r1 = O.bundle_adjust(q, 8, 4.0, n_threads=1)
    assert np.allclose(r.new_cost, r1.new_cost, rtol=1e-9, atol=0)


def test_oracle_self_sensitivity():
    """The reference is not bit-reproducible: its reduced matrix rows are hash
    maps with a per-run random key (ba.rs:132,147), so the PCG product sums
    blocks in a different order every run.  Permuting that order in the
    oracle moves the per-iteration cost of the ill-conditioned `refsurvey`
    solve by ~1e-9 relative: the scale the GPU tolerance is set against."""
    base = O.bundle_adjust(O.RefSurvey(), 60, 4.0, n_threads=1)
    devs = []
    try:
        for seed in (1, 2, 3):
            O.set_spmv_shuffle(seed)
            r = O.bundle_adjust(O.RefSurvey(), 60, 4.0, n_threads=1)
            n = min(len(r.new_cost), len(base.new_cost))
            devs.append(np.max(np.abs(r.new_cost[:n] - base.new_cost[:n]) / base.new_cost[:n]))
            assert r.iterations == base.iterations
    finally:
        O.set_spmv_shuffle(0)
    assert max(devs) > 1e-11, devs   # the order matters at this level ...
    assert max(devs) < 1e-7, devs    # ... and stays small
