"""The sparse stage's outputs: per-camera neighbours and depth ranges and the
f32 points (sparse.rs:470-483, 515-533; mod.rs:31-35) computed on the
device against the oracle, and the cameras.json / sparse.ply writers
(mod.rs:26-62, ply.rs:8-82)."""
import json
import os

import numpy as np
import pytest

import ba_oracle as O
import stitch_ba
from stitch_ba import Problem, survey
from stitch_ba import sparse_io as S


def py_summary(obs_cam, obs_pt, rot, center, points, agl, k=8):
    """sparse.rs:470-483 and 515-528 as plain Python loops (small cases):
    the independent check of the oracle's C restatement."""
    nc = len(center)
    shared = [dict() for _ in range(nc)]
    depths = [[] for _ in range(nc)]
    by_pt = {}
    for i, p in enumerate(obs_pt):
        by_pt.setdefault(int(p), []).append(int(obs_cam[i]))
    for p, cams in by_pt.items():
        X = points[p]
        for a in cams:
            R = rot[a].reshape(3, 3)
            d = X - center[a]
            depths[a].append(R[2, 0] * d[0] + R[2, 1] * d[1] + R[2, 2] * d[2])
            for b in cams:
                if a != b:
                    shared[a][b] = shared[a].get(b, 0) + 1
    nb, rng = [], []
    for a in range(nc):
        v = sorted(shared[a].items(), key=lambda t: (-t[1], t[0]))[:k]
        nb.append(v)
        d = sorted(depths[a])
        n = len(d)
        rng.append((d[n // 20] * 0.8, d[n * 19 // 20] * 1.25) if n >= 10 else (agl * 0.3, agl * 3.0))
    return nb, np.array(rng).reshape(nc, 2)


def random_problem(nc, npts, seed, max_views=6):
    """Random observation lists (not a geometric survey): every point seen by
    2..max_views distinct cameras, points and cameras anywhere, so equal
    counts, cameras with no observations and negative depths all occur."""
    rng = np.random.default_rng(seed)
    m = rng.integers(2, max_views + 1, npts)
    cams = [rng.choice(nc, size=int(k), replace=False) for k in m]
    obs_cam = np.concatenate(cams).astype(np.uint32)
    obs_pt = np.repeat(np.arange(npts), m).astype(np.uint32)
    q, _ = np.linalg.qr(rng.standard_normal((nc, 3, 3)))
    rot = np.ascontiguousarray(q.reshape(nc, 9))
    center = rng.uniform(-50, 50, (nc, 3))
    points = rng.uniform(-50, 50, (npts, 3))
    return obs_cam, obs_pt, rot, center, points


def problem_of(obs_cam, obs_pt, rot, center, points):
    nc = len(center)
    return Problem(intr=np.array([[3650.0, 2736.0, 1824.0, 0.0, 0.0]]), rot=rot.copy(),
                   center=center.copy(), cam_group=np.zeros(nc, np.uint32), points=points.copy(),
                   obs_cam=obs_cam, obs_pt=obs_pt, obs_uv=np.zeros((len(obs_cam), 2)),
                   prior_mask=None, prior=None, refine_intrinsics=False)


# ---- oracle pins -------------------------------------------------------------

def test_oracle_summary_matches_python_loops():
    oc, op, R, Cc, X = random_problem(40, 600, seed=3)
    nb, sh, n_nb, rng, p32 = O.sparse_summary(oc, op, R, Cc, X, agl=80.0)
    want_nb, want_rng = py_summary(oc, op, R, Cc, X, 80.0)
    for a in range(40):
        assert n_nb[a] == len(want_nb[a])
        assert nb[a, :n_nb[a]].tolist() == [b for b, _ in want_nb[a]]
        assert sh[a, :n_nb[a]].tolist() == [c for _, c in want_nb[a]]
        assert (nb[a, n_nb[a]:] == 0xffffffff).all() and (sh[a, n_nb[a]:] == 0).all()
    assert np.array_equal(rng, want_rng)
    assert np.array_equal(p32, X.astype(np.float32))


def test_oracle_summary_depth_fallback_and_sparse_cameras():
    # camera 5 observes nothing, cameras 0..2 fewer than ten points
    oc, op, R, Cc, X = random_problem(6, 8, seed=4, max_views=3)
    oc = np.where(oc == 5, 4, oc).astype(np.uint32)
    keep = np.ones(len(oc), bool)
    for p in range(8):  # keep cameras distinct within a point
        idx = np.nonzero(op == p)[0]
        _, first = np.unique(oc[idx], return_index=True)
        mask = np.zeros(len(idx), bool)
        mask[first] = True
        keep[idx] = mask
    oc, op = oc[keep], op[keep]
    nb, sh, n_nb, rng, _ = O.sparse_summary(oc, op, R, Cc, X, agl=100.0)
    assert n_nb[5] == 0 and (nb[5] == 0xffffffff).all()
    assert np.array_equal(rng[5], [30.0, 300.0])


# ---- writers (host) -----------------------------------------------------------

@pytest.mark.parametrize("x,text", [
    (1.0, "1.0"), (0.1, "0.1"), (1e-7, "1e-7"), (1.5e300, "1.5e300"),
    (123456789.0, "123456789.0"), (1e16, "1e16"), (1e15, "1000000000000000.0"),
    (1e-5, "0.00001"), (1.234e-5, "0.00001234"), (9.999e-6, "9.999e-6"), (-0.0, "-0.0"),
    (0.0, "0.0"), (float("nan"), "null"), (float("inf"), "null"), (5e-324, "5e-324"),
    (1.7976931348623157e308, "1.7976931348623157e308"), (-2.5, "-2.5"),
    (9007199254740992.0, "9007199254740992.0"), (3650.0000000001, "3650.0000000001"),
])
def test_json_number_layout(x, text):
    """serde_json (ryu) layout: positional for 1e-5 <= |x| < 1e16, else
    d.ddde±x without '+' or padding; integral values keep ".0"."""
    assert S.json_f64(x) == text


def test_json_numbers_round_trip():
    rng = np.random.default_rng(0)
    v = rng.standard_normal(20000) * 10.0 ** rng.integers(-300, 300, 20000)
    t = S._json_array("f64", v, 4)
    back = np.array(json.loads(t)).reshape(-1)
    assert np.array_equal(back, v)
    assert S._json_array("u8", np.array([0, 7, 255], np.uint8)) == "[0,7,255]"
    assert S._json_array("u32", np.array([], np.uint32)) == "[]"


@pytest.mark.parametrize("x,text", [(500000.0, "500000"), (512345.678, "512345.678"),
                                    (0.5, "0.5"), (-0.0, "-0"), (1e21, "1" + "0" * 21),
                                    (1e-7, "0.0000001")])
def test_rust_display(x, text):
    assert S.rust_display_f64(x) == text


def small_sparse(n_points=50, seed=0):
    rng = np.random.default_rng(seed)
    R = O.from_angles(90.0, -90.0, 0.0)
    cams = [S.Camera(i, f"/photos/DJI_{i:04d}.JPG", f"k\"{i}", 0, R, np.array([i * 25.0, 3.5, 80.0]),
                     i == 2, [1, 2] if i == 0 else [], (24.0, 240.0 + i)) for i in range(3)]
    return S.Sparse(S.UtmZone(33, True), 512345.678, 6543210.5, "takeoff",
                    [stitch_ba.Intrinsics(3650.25, 2736.0, 1824.0, -0.0125, 1e-7, 5472, 3648)],
                    cams, rng.uniform(-40, 40, (n_points, 3)),
                    rng.integers(0, 256, (n_points, 3)).astype(np.uint8), 0.4375, [7, 9])


def test_cameras_json_layout_and_round_trip(tmp_path):
    s = small_sparse()
    b = S.sparse_json(s)
    d = json.loads(b)
    assert list(d) == ["zone", "origin_e", "origin_n", "height_ref", "intrinsics", "cameras",
                       "points", "colors", "rms_px", "skipped"]
    assert list(d["cameras"][0]) == ["id", "path", "key", "group", "pose", "oblique",
                                     "neighbours", "depth_range"]
    assert b.startswith(b'{"zone":{"zone":33,"north":true},"origin_e":512345.678,')
    assert b'"k1":-0.0125,"k2":1e-7,"width":5472,"height":3648}' in b
    assert b'"key":"k\\"0"' in b and b" " not in b.replace(b"DJI_", b"")
    # pose.r: the storage (column-major) order of the world->camera matrix
    assert np.array_equal(np.array(d["cameras"][1]["pose"]["r"]), s.cameras[1].rot.T.reshape(-1))
    S.write_sparse(str(tmp_path), s)
    t = S.load_sparse(str(tmp_path))
    assert t.zone == s.zone and t.origin_e == s.origin_e and t.height_ref == s.height_ref
    assert np.array_equal(t.points, s.points) and np.array_equal(t.colors, s.colors)
    for a, c in zip(t.cameras, s.cameras):
        assert np.array_equal(a.rot, c.rot) and np.array_equal(a.center, c.center)
        assert a.neighbours == c.neighbours and a.depth_range == c.depth_range
        assert (a.path, a.key, a.oblique) == (c.path, c.key, c.oblique)
    assert t.intrinsics[0] == s.intrinsics[0] and t.skipped == [7, 9] and t.rms_px == 0.4375


def test_sparse_ply_bytes(tmp_path):
    s = small_sparse(n_points=4)
    S.write_sparse(str(tmp_path), s)
    raw = open(os.path.join(tmp_path, "sparse.ply"), "rb").read()
    head = (b"ply\nformat binary_little_endian 1.0\n"
            b"comment origin EPSG:32633 E 512345.678 N 6543210.5 height takeoff\n"
            b"element vertex 4\nproperty float x\nproperty float y\nproperty float z\n"
            b"property uchar red\nproperty uchar green\nproperty uchar blue\nend_header\n")
    assert raw[:len(head)] == head and len(raw) == len(head) + 4 * 15
    rec = raw[len(head):len(head) + 15]
    assert rec[:12] == s.points[0].astype("<f4").tobytes() and rec[12:] == s.colors[0].tobytes()
    p, c = S.read_ply(os.path.join(tmp_path, "sparse.ply"))
    assert np.array_equal(p, s.points.astype(np.float32)) and np.array_equal(c, s.colors)
    assert not os.path.exists(os.path.join(tmp_path, "sparse.ply.tmp"))
    with pytest.raises(ValueError):
        S.write_ply(os.path.join(tmp_path, "x.ply"), s.points, s.colors[:2], "c")


# ---- the device summary --------------------------------------------------------

def check_summary(out, ref):
    nb, sh, n_nb, rng, p32 = ref
    assert np.array_equal(out.n_neighbours, n_nb)
    assert np.array_equal(out.neighbours, nb)
    assert np.array_equal(out.shared, sh)
    assert np.array_equal(out.depth_range.view(np.uint64), rng.view(np.uint64))  # bit-exact
    assert np.array_equal(out.points_f32, p32)


@pytest.mark.gpu
@pytest.mark.parametrize("nc,npts,seed", [(40, 600, 3), (500, 20000, 5), (30000, 60000, 6)])
def test_gpu_summary_random_matches_oracle(nc, npts, seed):
    """Random observation lists: ties, empty cameras, negative depths; 30000
    cameras takes the global-memory histogram."""
    oc, op, R, Cc, X = random_problem(nc, npts, seed)
    out = stitch_ba.sparse_summary(problem_of(oc, op, R, Cc, X), agl=80.0)
    check_summary(out, O.sparse_summary(oc, op, R, Cc, X, agl=80.0))


@pytest.mark.gpu
def test_gpu_summary_survey_after_solve_matches_oracle():
    p, _ = survey.generate("lawnmower77", seed=1)
    with stitch_ba.Context() as ctx:
        ctx.upload(p)
        ctx.solve(10, 1.0)
        out = ctx.sparse_summary(agl=80.0)
        ctx.download(p)
    ref = O.sparse_summary(p.obs_cam, p.obs_pt, p.rot, p.center, p.points, agl=80.0)
    check_summary(out, ref)
    # neighbours along a lawnmower line share the most points
    assert (out.n_neighbours == 8).all()
    assert ((out.depth_range[:, 0] > 40.0) & (out.depth_range[:, 1] < 140.0)).all()
    out2 = stitch_ba.sparse_summary(p, agl=80.0)
    check_summary(out2, ref)


@pytest.mark.gpu
def test_gpu_summary_edge_cases():
    oc, op, R, Cc, X = random_problem(5, 3, seed=8, max_views=2)
    # no observations at all: every camera falls back to (0.3 agl, 3 agl)
    e = np.zeros(0, np.uint32)
    out = stitch_ba.sparse_summary(problem_of(e, e, R, Cc, X), agl=50.0)
    assert (out.n_neighbours == 0).all() and (out.neighbours == 0xffffffff).all()
    assert np.array_equal(out.depth_range, np.tile([15.0, 150.0], (5, 1)))
    out = stitch_ba.sparse_summary(problem_of(oc, op, R, Cc, X), agl=50.0, max_neighbours=1)
    check_summary(out, O.sparse_summary(oc, op, R, Cc, X, agl=50.0, max_neighbours=1))
    bad = op[::-1].copy()
    with pytest.raises(stitch_ba.BaError):
        stitch_ba.sparse_summary(problem_of(oc, bad, R, Cc, X), agl=50.0)
    with pytest.raises(stitch_ba.BaError):
        stitch_ba.sparse_summary(problem_of(oc, op, R, Cc, X), agl=50.0, max_neighbours=65)


@pytest.mark.gpu
def test_gpu_sparse_outputs_end_to_end(tmp_path):
    """Solve, summarise on the device, write cameras.json + sparse.ply, load."""
    p, _ = survey.generate("lawnmower77", seed=2)
    st = stitch_ba.bundle_adjust(p, 10, 1.0)
    out = stitch_ba.sparse_summary(p, agl=80.0)
    sp = S.build_sparse(p, out, zone=S.UtmZone(17, True), origin_e=500000.0, origin_n=4.5e6,
                        height_ref="takeoff", rms_px=st.final_rms, image_size=[(5472, 3648)])
    S.write_sparse(str(tmp_path), sp, points_f32=out.points_f32)
    back = S.load_sparse(str(tmp_path))
    assert np.array_equal(back.points, p.points)
    assert [c.neighbours for c in back.cameras] == out.neighbour_lists()
    pts, cols = S.read_ply(os.path.join(tmp_path, "sparse.ply"))
    assert np.array_equal(pts, p.points.astype(np.float32)) and (cols == 128).all()
