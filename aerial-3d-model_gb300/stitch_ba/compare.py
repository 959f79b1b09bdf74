"""Differences between two solutions of one problem, per result.

Used to state how far a solve (the mixed FP32/FP64 form, or the FP64 form on
the GPU) ends from another (the FP64 form, or the CPU solver) for every
quantity bundle adjustment updates (crates/stitch-core/src/recon/ba.rs:
338-366): camera centres (metres), rotations (radians, the angle of
R_a R_b^T), lens intrinsics (f, cx, cy, k1, k2) and points (metres).
"""
from __future__ import annotations

import numpy as np

INTR_NAMES = ("f", "cx", "cy", "k1", "k2")


def rot_angle(Ra: np.ndarray, Rb: np.ndarray) -> np.ndarray:
    """Angle of Ra Rb^T per camera, from its skew part (accurate for small
    angles, where the trace form loses half the digits)."""
    D = np.einsum("nij,nkj->nik", Ra.reshape(-1, 3, 3), Rb.reshape(-1, 3, 3))
    v = np.stack([D[:, 2, 1] - D[:, 1, 2], D[:, 0, 2] - D[:, 2, 0], D[:, 1, 0] - D[:, 0, 1]], 1)
    return np.arcsin(np.clip(np.linalg.norm(v, axis=1) / 2, 0, 1))


def _stats(v: np.ndarray, p99: bool = False) -> dict:
    if v.size == 0:
        return {"max": 0.0, "median": 0.0}
    out = {"max": float(v.max()), "median": float(np.median(v))}
    if p99:
        out["p99"] = float(np.percentile(v, 99))
    return out


def state_errors(a, b, far_m: float = 1.0) -> dict:
    """Per-result differences of solution `a` from solution `b` (objects with
    rot, center, intr, points).  Points: max / median / 99th percentile of
    the distance, and how many points differ by more than `far_m` metres."""
    dc = np.linalg.norm(a.center - b.center, axis=1)
    dr = rot_angle(a.rot, b.rot)
    dp = np.linalg.norm(a.points - b.points, axis=1)
    di = np.abs(np.asarray(a.intr) - np.asarray(b.intr)).reshape(-1, 5)
    scale = np.maximum(np.abs(np.asarray(b.intr)).reshape(-1, 5), 1e-300)
    return {
        "centre_m": _stats(dc),
        "rotation_rad": _stats(dr),
        "points_m": dict(_stats(dp, p99=True), n_above=int((dp > far_m).sum()), above_m=far_m),
        "intrinsics_abs": {n: float(di[:, i].max()) for i, n in enumerate(INTR_NAMES)},
        "intrinsics_rel": {n: float((di[:, i] / scale[:, i]).max())
                           for i, n in enumerate(INTR_NAMES)},
    }
