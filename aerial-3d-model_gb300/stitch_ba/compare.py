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


def similarity_fit(src: np.ndarray, dst: np.ndarray):
    """Least-squares similarity (s, R, t) with dst ≈ s R src + t (Umeyama's
    closed form: SVD of the cross-covariance of the centred point sets)."""
    ms, md = src.mean(0), dst.mean(0)
    xs, xd = src - ms, dst - md
    U, S, Vt = np.linalg.svd(xd.T @ xs / len(src))
    d = np.sign(np.linalg.det(U @ Vt))
    D = np.diag([1.0, 1.0, d])
    R = U @ D @ Vt
    var = (xs ** 2).sum() / len(src)
    s = float(np.trace(np.diag(S) @ D) / var) if var > 0 else 1.0
    return s, R, md - s * R @ ms


def state_errors(a, b, far_m: float = 1.0) -> dict:
    """Per-result differences of solution `a` from solution `b` (objects with
    rot, center, intr, points).  Points: max / median / 99th percentile of
    the distance, and how many points differ by more than `far_m` metres.

    `aligned`: the same centre, rotation and point differences after `a` is
    mapped onto `b` by the similarity that best fits its camera centres —
    the part of the difference that is not a motion of the whole block
    (translation, rotation, scale: the directions that only the GPS priors
    hold, which the reference's stop rule leaves least converged)."""
    dc = np.linalg.norm(a.center - b.center, axis=1)
    dr = rot_angle(a.rot, b.rot)
    dp = np.linalg.norm(a.points - b.points, axis=1)
    di = np.abs(np.asarray(a.intr) - np.asarray(b.intr)).reshape(-1, 5)
    scale = np.maximum(np.abs(np.asarray(b.intr)).reshape(-1, 5), 1e-300)
    out = {
        "centre_m": _stats(dc),
        "rotation_rad": _stats(dr),
        "points_m": dict(_stats(dp, p99=True), n_above=int((dp > far_m).sum()), above_m=far_m),
        "intrinsics_abs": {n: float(di[:, i].max()) for i, n in enumerate(INTR_NAMES)},
        "intrinsics_rel": {n: float((di[:, i] / scale[:, i]).max())
                           for i, n in enumerate(INTR_NAMES)},
    }
    if len(a.center) >= 3:
        s, R, t = similarity_fit(a.center, b.center)
        ca = s * a.center @ R.T + t
        pa = s * a.points @ R.T + t
        ra = np.einsum("nij,kj->nik", a.rot.reshape(-1, 3, 3), R)  # world change: R_cam R^T
        out["aligned"] = {
            "similarity": {"scale_minus_1": s - 1.0,
                           "rotation_rad": float(np.arcsin(min(1.0, np.linalg.norm(
                               [R[2, 1] - R[1, 2], R[0, 2] - R[2, 0], R[1, 0] - R[0, 1]]) / 2))),
                           "translation_m": float(np.linalg.norm(t + (s * R - np.eye(3)) @
                                                                 a.center.mean(0)))},
            "centre_m": _stats(np.linalg.norm(ca - b.center, axis=1)),
            "rotation_rad": _stats(rot_angle(ra, b.rot)),
            "points_m": _stats(np.linalg.norm(pa - b.points, axis=1), p99=True),
        }
    return out
