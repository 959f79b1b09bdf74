"""Generate the golden fixtures used by the parity tests.

Each fixture holds a problem (inputs) and the oracle's solve of it (outputs):
per-iteration trial costs, accept flags, stats and the final state.  The
oracle is the CPU restatement of crates/stitch-core/src/recon/ba.rs, pinned
to the reference by its own known-answer test (ba.rs:400-493, reproduced
exactly as `refsurvey`).  Inputs are stored, not regenerated, so the fixtures
do not depend on the host's libm.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "aerial-3d-model_gb300"))

import ba_oracle as O  # noqa: E402


def save(name, p, max_iter, sigma, loss=0):
    arrays = {k: np.array(getattr(p, k)) for k in (
        "obs_cam", "obs_pt", "obs_uv", "cam_group", "prior_mask", "prior", "rot", "center",
        "intr", "points")}
    q = _clone(p)
    r = O.bundle_adjust(q, max_iter, sigma, loss=loss, n_threads=1)
    out = dict(arrays)
    out.update(
        refine=np.array(bool(p.refine_intrinsics)), max_iter=np.array(max_iter),
        sigma=np.array(sigma), loss=np.array(loss),
        iterations=np.array(r.iterations), initial_rms=np.array(r.initial_rms),
        final_rms=np.array(r.final_rms), initial_cost=np.array(r.initial_cost),
        final_cost=np.array(r.final_cost), new_cost=r.new_cost, accepted=r.accepted,
        out_rot=q.rot, out_center=q.center, out_intr=q.intr, out_points=q.points)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print(name, r)


class _P:
    pass


def _clone(p):
    q = _P()
    for k in ("obs_cam", "obs_pt", "obs_uv", "cam_group", "prior_mask", "prior", "rot", "center",
              "intr", "points"):
        setattr(q, k, np.array(getattr(p, k)))
    q.refine_intrinsics = p.refine_intrinsics
    return q


def main():
    p = O.RefSurvey()
    save("refsurvey", p, 60, 4.0)           # the reference's own test (Cauchy, refine)
    p = O.RefSurvey()
    p.refine_intrinsics = False
    save("refsurvey_fixed_intr", p, 30, 4.0)
    p = O.RefSurvey()
    save("refsurvey_huber", p, 30, 4.0, loss=O.LOSS_HUBER)
    from stitch_ba import survey
    # made before the generator gated tracks by inlier count
    s, _ = survey.generate("lawnmower77", n_cams=24, n_points=4000, min_inlier_views=0)
    save("lawnmower24", s, 25, 1.0)


if __name__ == "__main__":
    main()
