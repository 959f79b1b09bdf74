"""Failure paths of the C ABI, made on the host or by a wait that runs out.

The reference cannot fail (ba.rs:198 returns BaStats); its degenerate cases
are skipped silently (ba.rs:61-63, 159-160, 174).  Through the C ABI:

* non-finite measurements, priors or initial state, and a prior sigma of 0
  (it divides the prior residual, ba.rs:120-126), are rejected as BAD_INPUT
  by the upload check before anything is solved;
* a device-memory budget (`workspace_limit_bytes`) makes an allocation fail
  on the host before it is made: OOM;
* a device-side wait that runs out: one CTA of the grid PCG launch is held
  back (`fault_hold_pcg_cta`, a test hook) so the others' group exchange
  never completes; with a short spin limit (`wait_limit_cycles`, about
  1 ms) every waiter gives up, sets the error flag and returns, and the call
  returns TIMEOUT.  No kernel faults, traps or hangs: every wait is bounded.

Every failed call leaves the caller's state untouched, and the next call on
the device succeeds."""
import os
import time

import numpy as np
import pytest

import stitch_ba
from stitch_ba import Options, Problem, native, survey

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _fixture(name="lawnmower24"):
    f = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    return Problem(intr=f["intr"], rot=f["rot"], center=f["center"], cam_group=f["cam_group"],
                   points=f["points"], obs_cam=f["obs_cam"], obs_pt=f["obs_pt"],
                   obs_uv=f["obs_uv"], prior_mask=f["prior_mask"], prior=f["prior"],
                   refine_intrinsics=bool(f["refine"]))


def _expect(status, p, max_iter=5, opts=None, text=None):
    before = p.state()
    with pytest.raises(stitch_ba.BaError) as e:
        stitch_ba.bundle_adjust(p, max_iter, 1.0, opts)
    assert e.value.status == status, str(e.value)
    if text:
        assert text in str(e.value), str(e.value)
    for a, b in zip(before, p.state()):
        assert np.array_equal(a, b, equal_nan=True)


@pytest.mark.parametrize("where", ["obs_uv", "points", "rot", "center", "intr", "prior",
                                   "prior_sigma"])
def test_non_finite_input_is_rejected(where):
    p = _fixture()
    if where == "obs_uv":
        p.obs_uv[17, 1] = np.nan
    elif where == "points":
        p.points[3, 2] = np.inf
    elif where == "rot":
        p.rot[2, 1, 1] = np.nan
    elif where == "center":
        p.center[5, 0] = -np.inf
    elif where == "intr":
        p.intr[0, 3] = np.nan
    elif where == "prior":
        p.prior[4, 1] = np.nan
    else:
        p.prior[4, 5] = 0.0
    _expect(native.BAD_INPUT, p, text="not finite")
    st = stitch_ba.bundle_adjust(_fixture(), 3, 1.0)  # the device is fine
    assert st.iterations == 3


def test_workspace_limit_gives_oom_and_leaves_the_state():
    p = _fixture()
    _expect(native.OOM, p, opts=Options(workspace_limit_bytes=1 << 20), text="workspace limit")
    # enough room: the same call succeeds
    st = stitch_ba.bundle_adjust(p, 3, 1.0, Options(workspace_limit_bytes=1 << 34))
    assert st.iterations == 3


def test_context_solve_respects_the_workspace_limit():
    p = _fixture()
    with stitch_ba.Context() as ctx:
        ctx.upload(p)
        with pytest.raises(stitch_ba.BaError) as e:
            ctx.solve(3, 1.0, Options(workspace_limit_bytes=4096))
        assert e.value.status == native.OOM
        info = ctx.solve(3, 1.0)[0]  # the context is still usable
        assert info.iterations == 3


def test_a_wait_that_runs_out_returns_timeout():
    p, _ = survey.generate("lawnmower77", seed=1)
    # 78 block rows at 4 rows per CTA: one group of ~20 CTAs, CTA 1 in it
    probe = p.copy()
    _, info = stitch_ba.bundle_adjust(probe, 1, 1.0, Options(pcg_kernel="grid"), return_info=True)
    assert info.pcg_kernel == "grid" and info.pcg_ctas >= 2
    q = p.copy()
    t0 = time.perf_counter()
    _expect(native.TIMEOUT, q, max_iter=10,
            opts=Options(pcg_kernel="grid", wait_limit_cycles=2_000_000, fault_hold_pcg_cta=2),
            text="gave up waiting")
    assert time.perf_counter() - t0 < 30.0
    # the next call on the device solves normally
    r = p.copy()
    st = stitch_ba.bundle_adjust(r, 5, 1.0, Options(pcg_kernel="grid"))
    assert st.iterations == 5 and np.isfinite(r.center).all()


def test_batch_with_one_bad_model_is_rejected_whole():
    good, bad = _fixture(), _fixture()
    bad.obs_uv[0, 0] = np.nan
    before = good.state()
    with pytest.raises(stitch_ba.BaError) as e:
        stitch_ba.bundle_adjust_batch([good, bad], 3, 1.0)
    assert e.value.status == native.BAD_INPUT
    for a, b in zip(before, good.state()):
        assert np.array_equal(a, b)
