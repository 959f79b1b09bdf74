"""ctypes binding of ``libba_gb300.so`` (the C ABI in ``include/ba_gb300.h``).

There is no CPU fallback: if the library cannot be built or loaded, or no
CUDA device is usable, the calls raise.
"""
from __future__ import annotations

import ctypes as C
import os
import shutil

from . import _build

OK, BAD_INPUT, OOM, CUDA_ERROR, TIMEOUT, NOT_SUPPORTED = range(6)
_STATUS = {0: "OK", 1: "BAD_INPUT", 2: "OOM", 3: "CUDA_ERROR", 4: "TIMEOUT", 5: "NOT_SUPPORTED"}

LOSS = {"cauchy": 0, "huber": 1}
PRECISION = {"fp64": 0, "mixed": 1}


class BaProblem(C.Structure):
    _fields_ = [("n_cams", C.c_int64), ("n_points", C.c_int64), ("n_obs", C.c_int64),
                ("n_groups", C.c_int64), ("obs_cam", C.c_void_p), ("obs_pt", C.c_void_p),
                ("obs_uv", C.c_void_p), ("cam_group", C.c_void_p), ("prior_mask", C.c_void_p),
                ("prior", C.c_void_p), ("refine_intrinsics", C.c_int32)]


class BaState(C.Structure):
    _fields_ = [("rot", C.c_void_p), ("center", C.c_void_p), ("intr", C.c_void_p),
                ("points", C.c_void_p)]


class BaTracks(C.Structure):
    _fields_ = [("n_tracks", C.c_int64), ("n_obs", C.c_int64), ("n_cams", C.c_int64),
                ("n_groups", C.c_int64), ("track_ptr", C.c_void_p), ("obs_cam", C.c_void_p),
                ("obs_uv", C.c_void_p), ("cam_group", C.c_void_p)]


class BaPairMatches(C.Structure):
    _fields_ = [("n_pairs", C.c_int64), ("n_matches", C.c_int64), ("pair_cam", C.c_void_p),
                ("match_ptr", C.c_void_p), ("uv", C.c_void_p), ("seed", C.c_void_p)]


class BaLog(C.Structure):
    _fields_ = [("cap", C.c_int32), ("new_cost", C.c_void_p), ("lam", C.c_void_p),
                ("pcg_iters", C.c_void_p), ("accepted", C.c_void_p)]


class BaOptions(C.Structure):
    _fields_ = [("max_iter", C.c_int32), ("sigma_px", C.c_double), ("loss", C.c_int32),
                ("precision", C.c_int32), ("pcg_max_iter", C.c_int32), ("pcg_tol", C.c_double),
                ("matrix_free", C.c_int32), ("memory_cap_bytes", C.c_int64),
                ("stream", C.c_void_p), ("log", C.c_void_p), ("profile", C.c_int32),
                ("pcg_kernel", C.c_int32), ("no_graph", C.c_int32), ("autotune", C.c_int32),
                ("stop_patience", C.c_int32), ("coarse", C.c_int32),
                ("fault_hold_pcg_cta", C.c_int32), ("wait_limit_cycles", C.c_int64),
                ("workspace_limit_bytes", C.c_int64), ("pcg_end_max_iter", C.c_int32),
                ("pcg_end_rel", C.c_double), ("point_kernel", C.c_int32)]


class BaStatsC(C.Structure):
    _fields_ = [("iterations", C.c_int64), ("initial_rms", C.c_double),
                ("final_rms", C.c_double), ("initial_cost", C.c_double),
                ("final_cost", C.c_double), ("pcg_iterations", C.c_int64),
                ("kernel_launches", C.c_int64), ("ms_total", C.c_double),
                ("ms_h2d", C.c_double), ("ms_d2h", C.c_double), ("h2d_bytes", C.c_int64),
                ("d2h_bytes", C.c_int64), ("device_bytes", C.c_int64),
                ("ms_phase", C.c_double * 9), ("n_phase", C.c_int64 * 9),
                ("n_blocks", C.c_int64), ("n_nonzero_blocks", C.c_int64),
                ("n_schur_pairs", C.c_int64), ("n_lens_entries", C.c_int64),
                ("pcg_kernel", C.c_int32), ("pcg_cluster", C.c_int32), ("graph", C.c_int32),
                ("pcg_ctas", C.c_int32), ("pcg_tuned_us", C.c_double),
                ("pcg_coarse_dim", C.c_int32), ("schur_sub_len", C.c_int32),
                ("schur_tuned_us", C.c_double), ("pcg_threads", C.c_int32),
                ("point_kernel", C.c_int32), ("point_tuned_us", C.c_double)]

PHASES = ["point", "camera", "schur", "assemble", "pcg", "update", "cost", "control", "setup"]


# Every symbol include/ba_gb300.h declares.
EXPORTS = [
    "ba_default_options", "ba_solve", "ba_solve_batch", "ba_context_create",
    "ba_context_destroy", "ba_context_upload", "ba_context_solve", "ba_context_download",
    "ba_context_intrinsics_grad", "ba_context_vjp", "ba_context_linearise", "ba_context_cost",
    "ba_context_debug_step", "ba_robust_cost_noalloc", "ba_triangulate",
    "ba_context_upload_tracks", "ba_sparse_summary", "ba_context_sparse_summary",
    "ba_json_f64", "ba_json_u8", "ba_json_u32", "ba_ransac_fundamental", "ba_pair_fits",
    "ba_last_error",
    "ba_abi_version", "ba_version",
]


class BaError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{_STATUS.get(status, status)}: {msg}")
        self.status = status


_lib = None


def library_path() -> str:
    return _build.SOLVER_LIB


def load(build_if_missing: bool = True):
    """Load libba_gb300.so (building it in-tree if nvcc is present)."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if build_if_missing and (shutil.which("nvcc") or os.path.exists("/usr/local/cuda/bin/nvcc")):
        path = _build.build_solver()
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: the CUDA solver has not been built")
    L = C.CDLL(path)
    P, S, O, T = C.POINTER(BaProblem), C.POINTER(BaState), C.POINTER(BaOptions), C.POINTER(BaStatsC)
    L.ba_default_options.argtypes = [O]
    L.ba_default_options.restype = None
    L.ba_solve.argtypes = [P, S, O, T]
    L.ba_solve_batch.argtypes = [P, S, C.c_int32, O, T]
    L.ba_context_create.argtypes = [C.c_int32, C.c_void_p, C.POINTER(C.c_void_p)]
    L.ba_context_destroy.argtypes = [C.c_void_p]
    L.ba_context_destroy.restype = None
    L.ba_context_upload.argtypes = [C.c_void_p, P, S, C.c_int32]
    L.ba_context_solve.argtypes = [C.c_void_p, O, T]
    L.ba_context_download.argtypes = [C.c_void_p, S, C.c_int32]
    L.ba_context_intrinsics_grad.argtypes = [C.c_void_p, O, C.c_void_p]
    L.ba_context_vjp.argtypes = [C.c_void_p, O] + [C.c_void_p] * 5
    L.ba_context_linearise.argtypes = [C.c_void_p, O] + [C.c_void_p] * 6
    L.ba_context_cost.argtypes = [C.c_void_p, O, C.c_void_p, C.c_void_p, C.c_void_p]
    L.ba_context_debug_step.argtypes = [C.c_void_p, O, C.c_double, C.c_void_p, C.c_void_p,
                                        C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_double)]
    L.ba_robust_cost_noalloc.argtypes = [P, S, C.c_double, C.c_int32, C.c_void_p,
                                         C.POINTER(C.c_double), C.POINTER(C.c_double),
                                         C.POINTER(C.c_int64)]
    L.ba_triangulate.argtypes = [C.POINTER(BaTracks), C.c_void_p, C.c_void_p, C.c_void_p,
                                 C.c_double, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                 C.POINTER(C.c_int64)]
    L.ba_context_upload_tracks.argtypes = [C.c_void_p, C.POINTER(BaTracks), S, C.c_void_p,
                                           C.c_void_p, C.c_int32, C.c_double,
                                           C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
    L.ba_sparse_summary.argtypes = [P, S, C.c_int32, C.c_double, C.c_void_p] + [C.c_void_p] * 5
    L.ba_context_sparse_summary.argtypes = [C.c_void_p, C.c_int32, C.c_double] + [C.c_void_p] * 5
    L.ba_ransac_fundamental.argtypes = [C.POINTER(BaPairMatches), C.c_double, C.c_int32,
                                        C.c_void_p] + [C.c_void_p] * 4
    L.ba_pair_fits.argtypes = [C.POINTER(BaPairMatches)] + [C.c_void_p] * 4 + [
        C.c_int64, C.c_int64, C.c_void_p, C.c_void_p]
    for name in ("ba_json_f64", "ba_json_u8", "ba_json_u32"):
        getattr(L, name).argtypes = [C.c_void_p, C.c_int64, C.c_int32, C.c_char_p, C.c_int64,
                                     C.POINTER(C.c_int64)]
    L.ba_last_error.restype = C.c_char_p
    L.ba_version.restype = C.c_char_p
    for name in ("ba_solve", "ba_solve_batch", "ba_context_create", "ba_context_upload",
                 "ba_context_solve", "ba_context_download", "ba_context_intrinsics_grad",
                 "ba_context_vjp", "ba_context_debug_step", "ba_robust_cost_noalloc",
                 "ba_context_linearise", "ba_context_cost", "ba_triangulate",
                 "ba_context_upload_tracks", "ba_sparse_summary", "ba_context_sparse_summary",
                 "ba_json_f64", "ba_json_u8", "ba_json_u32", "ba_ransac_fundamental",
                 "ba_pair_fits"):
        getattr(L, name).restype = C.c_int
    _lib = L
    return L


def check(status: int):
    if status != OK:
        raise BaError(status, load().ba_last_error().decode(errors="replace"))
