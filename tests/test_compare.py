"""Per-result solution differences (stitch_ba.compare).  CPU only."""
import numpy as np

from stitch_ba import compare


class _Sol:
    def __init__(self, rot, center, intr, points):
        self.rot, self.center, self.intr, self.points = rot, center, intr, points


def _rotations(n, rng):
    out = []
    for _ in range(n):
        q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        out.append(q * np.sign(np.linalg.det(q)))
    return np.array(out)


def _rodrigues(w):
    th = np.linalg.norm(w)
    k = w / th
    K = np.array([[0, -k[2], k[1]], [k[2], 0, -k[0]], [-k[1], k[0], 0]])
    return np.eye(3) + np.sin(th) * K + (1 - np.cos(th)) * K @ K


def test_a_motion_of_the_whole_block_is_removed_by_the_alignment():
    rng = np.random.default_rng(0)
    b = _Sol(_rotations(40, rng), rng.normal(size=(40, 3)) * 100,
             np.array([[3000.0, 2000, 1500, -0.03, 0.01]]), rng.normal(size=(300, 3)) * 50)
    s, R, t = 1.0005, _rodrigues(np.array([1e-3, -2e-3, 5e-4])), np.array([0.3, -0.2, 0.5])
    a = _Sol(np.einsum("nij,kj->nik", b.rot, R), s * b.center @ R.T + t, b.intr.copy(),
             s * b.points @ R.T + t)
    e = compare.state_errors(a, b)
    assert e["centre_m"]["max"] > 0.1 and e["rotation_rad"]["max"] > 1e-3
    al = e["aligned"]
    assert al["centre_m"]["max"] < 1e-9 and al["points_m"]["max"] < 1e-9
    assert al["rotation_rad"]["max"] < 1e-12
    assert abs(al["similarity"]["scale_minus_1"] - (1 / s - 1)) < 1e-12
    assert e["intrinsics_rel"]["f"] == 0.0


def test_identical_solutions_differ_by_nothing():
    rng = np.random.default_rng(1)
    b = _Sol(_rotations(5, rng), rng.normal(size=(5, 3)), np.ones((1, 5)), rng.normal(size=(9, 3)))
    e = compare.state_errors(b, b)
    assert e["centre_m"]["max"] == 0.0 and e["points_m"]["max"] == 0.0
    assert e["rotation_rad"]["max"] < 1e-15 and e["points_m"]["n_above"] == 0
