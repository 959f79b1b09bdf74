"""Host-side mirror of stitch-core's bundle-adjustment types.

``Problem`` and ``BaStats`` carry the fields of the reference's ``Problem``
and ``BaStats`` (crates/stitch-core/src/recon/ba.rs:28-46) in structure-of-
arrays form, the layout the C ABI (``include/ba_gb300.h``) takes:

=================  ==================  =====================================
reference field    here                layout
=================  ==================  =====================================
``intr``           ``intr``            (n_groups, 5) f64: f, cx, cy, k1, k2
``poses[i].r``     ``rot[i]``          (n_cams, 3, 3) f64, row-major, world→camera
``poses[i].c``     ``center[i]``       (n_cams, 3) f64
``group``          ``cam_group``       (n_cams,) u32
``prior``          ``prior_mask``,     (n_cams,) u8 and (n_cams, 6) f64:
                   ``prior``           centre xyz then sigma xyz (metres)
``points``         ``points``          (n_points, 3) f64
``obs``            ``obs_cam``,        (n_obs,) u32, (n_obs,) u32 sorted by point,
                   ``obs_pt``,         (n_obs, 2) f64 pixels
                   ``obs_uv``
``refine_intr…``   ``refine_intrinsics``  bool
=================  ==================  =====================================

Like the reference, ``bundle_adjust`` mutates ``rot``, ``center``, ``points``
and (when refining) ``intr`` in place and leaves the rest untouched.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class Intrinsics:
    """geometry.rs:15-23 (width/height are not used by the solver)."""
    f: float
    cx: float
    cy: float
    k1: float
    k2: float
    width: int = 0
    height: int = 0


@dataclass
class Obs:
    """ba.rs:21-26."""
    cam: int
    pt: int
    u: tuple


@dataclass
class BaStats:
    """ba.rs:41-46."""
    iterations: int
    initial_rms: float
    final_rms: float


class Problem:
    """ba.rs:28-39 in structure-of-arrays form."""

    def __init__(self, *, intr, rot, center, cam_group, points, obs_cam, obs_pt, obs_uv,
                 prior_mask=None, prior=None, refine_intrinsics: bool = True):
        self.intr = np.ascontiguousarray(intr, np.float64).reshape(-1, 5)
        self.rot = np.ascontiguousarray(rot, np.float64).reshape(-1, 3, 3)
        self.center = np.ascontiguousarray(center, np.float64).reshape(-1, 3)
        self.cam_group = np.ascontiguousarray(cam_group, np.uint32).reshape(-1)
        self.points = np.ascontiguousarray(points, np.float64).reshape(-1, 3)
        self.obs_cam = np.ascontiguousarray(obs_cam, np.uint32).reshape(-1)
        self.obs_pt = np.ascontiguousarray(obs_pt, np.uint32).reshape(-1)
        self.obs_uv = np.ascontiguousarray(obs_uv, np.float64).reshape(-1, 2)
        if prior_mask is None:
            self.prior_mask = None
            self.prior = None
        else:
            self.prior_mask = np.ascontiguousarray(prior_mask, np.uint8).reshape(-1)
            self.prior = np.ascontiguousarray(prior, np.float64).reshape(-1, 6)
        self.refine_intrinsics = bool(refine_intrinsics)

    @classmethod
    def empty(cls, n_cams, n_points, n_obs, n_groups, refine_intrinsics=True):
        return cls(intr=np.zeros((n_groups, 5)), rot=np.zeros((n_cams, 3, 3)),
                   center=np.zeros((n_cams, 3)), cam_group=np.zeros(n_cams, np.uint32),
                   points=np.zeros((n_points, 3)), obs_cam=np.zeros(n_obs, np.uint32),
                   obs_pt=np.zeros(n_obs, np.uint32), obs_uv=np.zeros((n_obs, 2)),
                   prior_mask=np.zeros(n_cams, np.uint8), prior=np.zeros((n_cams, 6)),
                   refine_intrinsics=refine_intrinsics)

    @property
    def n_cams(self):
        return self.rot.shape[0]

    @property
    def n_points(self):
        return self.points.shape[0]

    @property
    def n_obs(self):
        return self.obs_cam.shape[0]

    @property
    def n_groups(self):
        return self.intr.shape[0]

    def copy(self) -> "Problem":
        return Problem(intr=self.intr.copy(), rot=self.rot.copy(), center=self.center.copy(),
                       cam_group=self.cam_group.copy(), points=self.points.copy(),
                       obs_cam=self.obs_cam.copy(), obs_pt=self.obs_pt.copy(),
                       obs_uv=self.obs_uv.copy(),
                       prior_mask=None if self.prior_mask is None else self.prior_mask.copy(),
                       prior=None if self.prior is None else self.prior.copy(),
                       refine_intrinsics=self.refine_intrinsics)

    def state(self):
        """Copies of the mutable state: (rot, center, intr, points)."""
        return (self.rot.copy(), self.center.copy(), self.intr.copy(), self.points.copy())

    def set_state(self, st):
        self.rot[...], self.center[...], self.intr[...], self.points[...] = st

    def intrinsics(self, g: int = 0) -> Intrinsics:
        f, cx, cy, k1, k2 = self.intr[g]
        return Intrinsics(f, cx, cy, k1, k2)
