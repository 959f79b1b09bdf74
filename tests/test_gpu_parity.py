"""GPU solver (through the C ABI) against the oracle and the golden fixtures.

Tolerances (FP64 plain form vs the CPU restatement of ba.rs):
  * per-iteration trial cost: 1e-9 relative, or 5x the reference's own
    run-to-run spread where that is larger: the reduced systems here have
    cond ~1e10 (nadir-only: focal length and flying height trade off) and PCG
    either stops at 400 products or on a tolerance crossing that moves with
    rounding alone; the oracle with its hash-map summation order permuted
    (the reference's own source of run-to-run differences, ba.rs:147) moves
    by ~1e-9 .. 5e-9 on the fixtures and by up to ~1e-7 on the 77-camera
    survey (reference_spread);
  * final camera centres 1e-6 m and rotations 1e-8 rad, or 5x the
    reference's own spread where that is larger (77 cameras: centres move by
    up to ~4e-4 m between the reference's own runs, along the weak
    directions the GPS priors alone hold); points 1e-3 m on the fixtures.
Every test records the deviation it measured (the `parity_record` fixture),
so the distance to the contract's 1e-9 / 1e-6 m / 1e-8 rad is visible.
"""
import os

import numpy as np
import pytest

import ba_oracle as O
import stitch_ba
from stitch_ba import Options, Problem, compare, survey

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
_SPREAD = {}


def reference_spread(name):
    """How far the reference's own result moves under its run-to-run
    summation order (hash-map rows, ba.rs:132,147): the oracle re-run with
    four permuted row orders, max relative deviation of the per-iteration
    trial cost from the fixture."""
    if name not in _SPREAD:
        p, f = load_fixture(name)
        dev = 0.0
        try:
            for seed in (11, 12, 13, 14):
                O.set_spmv_shuffle(seed)
                q = p.copy()
                r = O.bundle_adjust(q, int(f["max_iter"]), float(f["sigma"]), loss=int(f["loss"]),
                                    n_threads=1)
                n = min(len(r.new_cost), len(f["new_cost"]))
                dev = max(dev, float(np.max(np.abs(r.new_cost[:n] - f["new_cost"][:n]) /
                                            f["new_cost"][:n])))
        finally:
            O.set_spmv_shuffle(0)
        _SPREAD[name] = dev
    return _SPREAD[name]


def cost_tol(name):
    return max(1e-9, 5.0 * reference_spread(name))


def load_fixture(name):
    f = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    p = Problem(intr=f["intr"], rot=f["rot"], center=f["center"], cam_group=f["cam_group"],
                points=f["points"], obs_cam=f["obs_cam"], obs_pt=f["obs_pt"],
                obs_uv=f["obs_uv"], prior_mask=f["prior_mask"], prior=f["prior"],
                refine_intrinsics=bool(f["refine"]))
    return p, f


rot_angle = compare.rot_angle


def check_against(p, info, ref_new_cost, ref_accepted, ref_state, tol):
    """Per-iteration trial cost within `tol`, the same accept sequence and the
    final state within 1e-6 m / 1e-8 rad (points 1e-3 m); returns the
    deviations measured."""
    n = min(len(info.new_cost), len(ref_new_cost))
    assert n > 0
    rel = np.abs(info.new_cost[:n] - ref_new_cost[:n]) / np.abs(ref_new_cost[:n])
    rot, center, intr, points = ref_state
    dev = {"trial_cost_rel_max": float(rel.max()), "tolerance": tol,
           "centre_m_max": float(np.abs(p.center - center).max()),
           "rotation_rad_max": float(rot_angle(p.rot, rot).max()),
           "points_m_max": float(np.abs(p.points - points).max()),
           "intr_rel_max": float(np.abs(p.intr - intr).max() / np.abs(intr).max())}
    assert rel.max() < tol, (rel.max(), rel)
    assert np.array_equal(info.accepted[:n], np.asarray(ref_accepted[:n], bool))
    assert dev["centre_m_max"] < 1e-6
    assert dev["rotation_rad_max"] < 1e-8
    assert dev["points_m_max"] < 1e-3
    assert dev["intr_rel_max"] <= 1e-6
    return dev


@pytest.mark.parametrize("name", ["refsurvey", "refsurvey_fixed_intr", "refsurvey_huber",
                                  "lawnmower24"])
def test_fp64_matches_golden(name, parity_record):
    p, f = load_fixture(name)
    loss = "huber" if int(f["loss"]) == 1 else "cauchy"
    st, info = stitch_ba.bundle_adjust(p, int(f["max_iter"]), float(f["sigma"]),
                                       Options(loss=loss), return_info=True)
    assert st.iterations == int(f["iterations"])
    assert abs(st.initial_rms - float(f["initial_rms"])) <= 1e-12 * float(f["initial_rms"])
    tol = cost_tol(name)
    final_rel = abs(info.final_cost - float(f["final_cost"])) / float(f["final_cost"])
    dev = check_against(p, info, f["new_cost"], f["accepted"],
                        (f["out_rot"], f["out_center"], f["out_intr"], f["out_points"]), tol)
    dev.update(final_cost_rel=final_rel, reference_spread=reference_spread(name),
               iterations=int(st.iterations))
    parity_record["fp64_vs_oracle:" + name] = dev
    assert final_rel <= tol
    assert info.kernel_launches > 0


def _oracle_runs(p, max_iter, sigma, seeds):
    """The oracle's solve of `p` (fixed hash-map order) and its solves with
    the SpMV block order permuted by each seed (the reference's own
    run-to-run variation, ba.rs:147), on all host cores."""
    threads = os.cpu_count() or 1
    base = p.copy()
    r0 = O.bundle_adjust(base, max_iter, sigma, n_threads=threads)
    runs = []
    try:
        for seed in seeds:
            O.set_spmv_shuffle(seed)
            q = p.copy()
            runs.append((O.bundle_adjust(q, max_iter, sigma, n_threads=threads), q))
    finally:
        O.set_spmv_shuffle(0)
    return (r0, base), runs


def test_fp64_matches_cpu_solver_on_lawnmower77(parity_record):
    """The 77-camera lawnmower survey (77 cameras, 40k points, ~246k
    observations, 5% outliers, GPS priors): FP64 GPU solve against the
    oracle's solve (ba.rs:198-391), iteration by iteration.

    The same iterations and accept sequence; per-iteration trial cost, final
    cost, centres and rotations within the contract's 1e-9 / 1e-6 m /
    1e-8 rad, or within 5x the spread of the reference's own runs where
    that is larger (measured here: two permuted-order runs of the oracle)."""
    p, _ = survey.generate("lawnmower77", seed=1)
    (r0, base), runs = _oracle_runs(p, 60, 1.0, (11, 12))
    sp_cost = sp_final = sp_c = sp_r = 0.0
    for r, q in runs:
        assert r.iterations == r0.iterations
        n = r.iterations
        sp_cost = max(sp_cost, float(np.max(np.abs(r.new_cost[:n] - r0.new_cost[:n]) /
                                            r0.new_cost[:n])))
        sp_final = max(sp_final, abs(r.final_cost - r0.final_cost) / r0.final_cost)
        sp_c = max(sp_c, float(np.abs(q.center - base.center).max()))
        sp_r = max(sp_r, float(rot_angle(q.rot, base.rot).max()))
    q = p.copy()
    st, info = stitch_ba.bundle_adjust(q, 60, 1.0, return_info=True)
    n = r0.iterations
    rel = np.abs(info.new_cost[:n] - r0.new_cost[:n]) / r0.new_cost[:n]
    dev = {"iterations": int(info.iterations), "oracle_iterations": int(n),
           "trial_cost_rel_max": float(rel.max()),
           "final_cost_rel": abs(info.final_cost - r0.final_cost) / r0.final_cost,
           "centre_m_max": float(np.abs(q.center - base.center).max()),
           "rotation_rad_max": float(rot_angle(q.rot, base.rot).max()),
           "points_m_max": float(np.abs(q.points - base.points).max()),
           "reference_spread": {"trial_cost_rel": sp_cost, "final_cost_rel": sp_final,
                                "centre_m": sp_c, "rotation_rad": sp_r}}
    parity_record["fp64_vs_oracle:lawnmower77"] = dev
    assert info.iterations == r0.iterations
    assert np.array_equal(info.accepted, np.asarray(r0.accepted, bool))
    assert dev["trial_cost_rel_max"] <= max(1e-9, 5 * sp_cost), dev
    assert dev["final_cost_rel"] <= max(1e-9, 5 * sp_final), dev
    assert dev["centre_m_max"] <= max(1e-6, 5 * sp_c), dev
    assert dev["rotation_rad_max"] <= max(1e-8, 5 * sp_r), dev


def _mixed_vs_fp64(name, parity_record, **opts):
    p, _ = survey.generate(name, seed=1)
    a, b = p.copy(), p.copy()
    _, f64 = stitch_ba.bundle_adjust(a, 60, 1.0, return_info=True)
    _, mix = stitch_ba.bundle_adjust(b, 60, 1.0, Options(precision="mixed", coarse=True, **opts),
                                     return_info=True)
    err = compare.state_errors(b, a)
    err["final_cost_rel"] = (mix.final_cost - f64.final_cost) / f64.final_cost
    err["iterations"] = [int(f64.iterations), int(mix.iterations)]
    parity_record["mixed_vs_fp64:" + name] = err
    return err


def test_mixed_form_error_per_result_on_single500(parity_record):
    """The mixed FP32/FP64 form (two-level PCG, 40 iterations, stop after two
    small decreases) against the FP64 form on the 500-camera survey, every
    result the solve updates (ba.rs:338-366), with stated bounds.

    The final cost matches (within 1e-6 relative, or below).  The states
    differ mostly by a motion of the whole block (translation, rotation,
    scale), which only the GPS priors hold and which neither form has
    converged when the reference's stop rule fires: raw centre and point
    differences reach ~1 m, but after the best similarity fit of the centres
    they are centimetres."""
    err = _mixed_vs_fp64("single500", parity_record, pcg_max_iter=40, stop_patience=2)
    assert err["final_cost_rel"] <= 1e-6, err
    assert err["intrinsics_rel"]["f"] < 2e-4, err
    assert err["centre_m"]["max"] < 2.0 and err["points_m"]["max"] < 2.0, err
    al = err["aligned"]
    assert al["centre_m"]["max"] < 0.1, err
    assert al["rotation_rad"]["max"] < 1e-3, err
    assert al["points_m"]["p99"] < 0.1, err


def test_mixed_form_error_per_result_on_lawnmower77(parity_record):
    """The same on the 77-camera survey, where the mixed form with 40 PCG
    iterations stalls a few 1e-6 above the FP64 final cost (its small FP32
    steps stop decreasing the cost first); 100 iterations reach it."""
    err = _mixed_vs_fp64("lawnmower77", parity_record, pcg_max_iter=40, stop_patience=2)
    assert err["final_cost_rel"] <= 2e-5, err
    err100 = _mixed_vs_fp64("lawnmower77", {}, pcg_max_iter=100, stop_patience=2)
    parity_record["mixed_vs_fp64:lawnmower77:pcg100"] = {
        "final_cost_rel": err100["final_cost_rel"], "iterations": err100["iterations"]}
    assert err100["final_cost_rel"] <= 1e-6, err100
