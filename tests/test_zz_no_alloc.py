"""ba_robust_cost_noalloc: the cost of a device-resident problem computed
without allocating device memory (for callers whose device memory is all
held by another runtime's allocator, or whose loop must not synchronise the
device through cudaMalloc / cudaFree).

Called through the C ABI on device arrays twice in a row — the second call
reuses the fixed scratch array the first one left behind — and checked
against the allocating entry point ba_context_cost within the tests' cost
tolerance (1e-12 relative).  The device's free memory is the same before
and after the second call (nothing is allocated), and an observation index
out of range is rejected by the kernel's own bounds check.  Collected last
on purpose: it touches a per-process device array."""
import ctypes as C
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _device_views(p, torch):
    """Device copies of a Problem's arrays and the (ba_problem, ba_state)
    views of them (the entry point takes device pointers)."""
    from stitch_ba import native
    dev = {}
    for k in ("obs_cam", "obs_pt", "obs_uv", "cam_group", "prior_mask", "prior", "rot",
              "center", "intr", "points"):
        a = getattr(p, k)
        t = torch.from_numpy(np.ascontiguousarray(a).view(np.int32 if a.dtype == np.uint32 else a.dtype))
        dev[k] = t.cuda()
    torch.cuda.synchronize()
    prob = native.BaProblem(p.n_cams, p.n_points, p.n_obs, p.n_groups,
                            dev["obs_cam"].data_ptr(), dev["obs_pt"].data_ptr(),
                            dev["obs_uv"].data_ptr(), dev["cam_group"].data_ptr(),
                            dev["prior_mask"].data_ptr(), dev["prior"].data_ptr(), 1)
    st = native.BaState(dev["rot"].data_ptr(), dev["center"].data_ptr(),
                        dev["intr"].data_ptr(), dev["points"].data_ptr())
    return dev, prob, st


def _problem(name):
    from stitch_ba import Problem
    f = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    return Problem(intr=f["intr"], rot=f["rot"], center=f["center"], cam_group=f["cam_group"],
                   points=f["points"], obs_cam=f["obs_cam"], obs_pt=f["obs_pt"],
                   obs_uv=f["obs_uv"], prior_mask=f["prior_mask"], prior=f["prior"],
                   refine_intrinsics=bool(f["refine"]))


@pytest.mark.parametrize("name,sigma,loss", [("lawnmower24", 1.0, 0), ("refsurvey", 4.0, 1)])
def test_noalloc_cost_matches_context_cost_twice(name, sigma, loss):
    torch = pytest.importorskip("torch")
    import stitch_ba
    from stitch_ba import native

    L = native.load()
    p = _problem(name)
    dev, prob, st = _device_views(p, torch)
    loss_name = "huber" if loss == 1 else "cauchy"
    with stitch_ba.Context() as ctx:
        ctx.upload(p)
        ref_c, ref_r, ref_n = ctx.cost(sigma, stitch_ba.Options(loss=loss_name))
    stream = torch.cuda.current_stream().cuda_stream
    free = []
    for _ in range(2):
        torch.cuda.synchronize()
        free.append(torch.cuda.mem_get_info()[0])
        c, r, n = C.c_double(), C.c_double(), C.c_int64()
        native.check(L.ba_robust_cost_noalloc(C.byref(prob), C.byref(st), sigma, loss, stream,
                                              C.byref(c), C.byref(r), C.byref(n)))
        assert abs(c.value - ref_c[0]) <= 1e-12 * abs(ref_c[0])
        assert abs(r.value - ref_r[0]) <= 1e-12 * abs(ref_r[0])
        assert n.value == ref_n[0]
    torch.cuda.synchronize()
    # the second call (after the first has set the scratch array up) leaves
    # the device's free memory exactly as it found it
    assert torch.cuda.mem_get_info()[0] == free[1]
    del dev


def test_noalloc_rejects_an_index_out_of_range():
    torch = pytest.importorskip("torch")
    import stitch_ba  # noqa: F401
    from stitch_ba import native

    L = native.load()
    p = _problem("lawnmower24")
    p.obs_pt = p.obs_pt.copy()
    p.obs_pt[-1] = p.n_points  # one past the last point
    dev, prob, st = _device_views(p, torch)
    c = C.c_double()
    status = L.ba_robust_cost_noalloc(C.byref(prob), C.byref(st), 1.0, 0,
                                      torch.cuda.current_stream().cuda_stream, C.byref(c),
                                      None, None)
    assert status == native.BAD_INPUT
    assert b"out of range" in L.ba_last_error()
    # the device is still usable: a valid problem gives a cost afterwards
    q = _problem("lawnmower24")
    dev2, prob2, st2 = _device_views(q, torch)
    native.check(L.ba_robust_cost_noalloc(C.byref(prob2), C.byref(st2), 1.0, 0,
                                          torch.cuda.current_stream().cuda_stream, C.byref(c),
                                          None, None))
    assert c.value > 0.0
    del dev, dev2


def test_noalloc_rejects_oversized_problems():
    import stitch_ba  # noqa: F401
    from stitch_ba import native

    L = native.load()
    prob = native.BaProblem(1, 1, 33_554_433, 1, 1, 1, 1, 1, None, None, 1)
    st = native.BaState(1, 1, 1, 1)
    c = C.c_double()
    status = L.ba_robust_cost_noalloc(C.byref(prob), C.byref(st), 1.0, 0, None, C.byref(c), None,
                                      None)
    assert status == native.BAD_INPUT
    assert b"no-allocation limit" in L.ba_last_error()
