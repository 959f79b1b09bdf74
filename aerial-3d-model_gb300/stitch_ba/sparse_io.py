"""The sparse stage's output files: ``cameras.json`` (the ``Sparse`` result,
serialised with serde_json; sparse.rs:26-54, mod.rs:26-31) and ``sparse.ply``
(binary little-endian xyz f32 + rgb u8; ply.rs:8-82), plus ``load_sparse``
(mod.rs:57-62) and ``origin_comment`` (mod.rs:45-53).

The per-camera fields that come from the bundle-adjusted problem (neighbours,
depth ranges) and the f32 points are computed on the device by
``sparse_summary``; this module lays them out byte for byte as the
reference's writers do.  Numbers in cameras.json are formatted by the native
library (``ba_json_f64``: shortest round-trip digits in serde_json's layout).

Layout notes:
* ``pose.r`` is nalgebra's ``Matrix3`` as serde writes it, the storage order,
  which is column-major: the row-major world->camera matrix transposed.
* Image paths are written as JSON strings (serde's ``PathBuf``).
* Colours default to 128 grey: the reference samples them from the photos
  (sparse.rs:485-512), which need image decoding outside this library.
"""
from __future__ import annotations

import ctypes as C
import json
import math
import os
from dataclasses import dataclass, field

import numpy as np

from . import native
from .problem import Intrinsics


@dataclass
class UtmZone:
    """geo.rs:12-31."""
    zone: int
    north: bool

    def epsg(self) -> int:
        return (32600 if self.north else 32700) + int(self.zone)


@dataclass
class Camera:
    """sparse.rs:26-38.  `rot` is the row-major world->camera rotation."""
    id: int
    path: str
    key: str
    group: int
    rot: np.ndarray
    center: np.ndarray
    oblique: bool = False
    neighbours: list = field(default_factory=list)
    depth_range: tuple = (0.0, 0.0)


@dataclass
class Sparse:
    """sparse.rs:40-54."""
    zone: UtmZone
    origin_e: float
    origin_n: float
    height_ref: str
    intrinsics: list
    cameras: list
    points: np.ndarray  # f64[n, 3]
    colors: np.ndarray  # u8[n, 3]
    rms_px: float
    skipped: list = field(default_factory=list)


# ---- numbers ---------------------------------------------------------------

def _json_array(kind: str, a, group: int = 0) -> str:
    L = native.load()
    dt, w, fn = {"f64": (np.float64, 25, L.ba_json_f64), "u8": (np.uint8, 3, L.ba_json_u8),
                 "u32": (np.uint32, 10, L.ba_json_u32)}[kind]
    v = np.ascontiguousarray(a, dt).reshape(-1)
    n = v.size
    cap = n * (w + 1) + 2 * (n // group if group else 0) + 3
    buf = C.create_string_buffer(cap)
    ln = C.c_int64()
    native.check(fn(v.ctypes.data if n else None, n, int(group), buf, cap, C.byref(ln)))
    return buf.raw[:ln.value].decode()


def json_f64(x: float) -> str:
    """serde_json's text of one f64 (shortest round trip; 1.0, 1e-7)."""
    return _json_array("f64", [x])[1:-1]


def rust_display_f64(x: float) -> str:
    """Rust's ``{}`` of an f64 (used in the PLY origin comment): the shortest
    round-trip digits written positionally, no exponent, no trailing ".0"."""
    if math.isnan(x):
        return "NaN"
    if math.isinf(x):
        return "inf" if x > 0 else "-inf"
    sign = "-" if math.copysign(1.0, x) < 0 else ""
    r = repr(abs(x))
    mant, _, exp = r.partition("e")
    ip, _, fp = mant.partition(".")
    digits = (ip + fp).lstrip("0")
    k = (int(exp) if exp else 0) - len(fp)
    if not digits:
        return sign + "0"
    stripped = digits.rstrip("0")
    k += len(digits) - len(stripped)
    digits = stripped
    if k >= 0:
        return sign + digits + "0" * k
    pos = len(digits) + k
    if pos > 0:
        return sign + digits[:pos] + "." + digits[pos:]
    return sign + "0." + "0" * (-pos) + digits


# ---- cameras.json ----------------------------------------------------------

def _s(x: str) -> str:
    return json.dumps(str(x), ensure_ascii=False)


def _b(x: bool) -> str:
    return "true" if x else "false"


def sparse_json(s: Sparse) -> bytes:
    """`serde_json::to_vec(&Sparse)` (mod.rs:30): compact, fields in
    declaration order."""
    f = json_f64
    intr = ",".join(
        '{"f":%s,"cx":%s,"cy":%s,"k1":%s,"k2":%s,"width":%d,"height":%d}'
        % (f(k.f), f(k.cx), f(k.cy), f(k.k1), f(k.k2), int(k.width), int(k.height))
        for k in s.intrinsics)
    cams = []
    for c in s.cameras:
        r = np.asarray(c.rot, np.float64).reshape(3, 3).T  # column-major storage
        cams.append(
            '{"id":%d,"path":%s,"key":%s,"group":%d,"pose":{"r":%s,"c":%s},"oblique":%s,'
            '"neighbours":%s,"depth_range":[%s,%s]}'
            % (int(c.id), _s(c.path), _s(c.key), int(c.group), _json_array("f64", r),
               _json_array("f64", np.asarray(c.center, np.float64).reshape(3)), _b(c.oblique),
               _json_array("u32", np.asarray(c.neighbours, np.uint32)),
               f(c.depth_range[0]), f(c.depth_range[1])))
    pts = np.asarray(s.points, np.float64).reshape(-1, 3)
    cols = np.asarray(s.colors, np.uint8).reshape(-1, 3)
    text = ('{"zone":{"zone":%d,"north":%s},"origin_e":%s,"origin_n":%s,"height_ref":%s,'
            '"intrinsics":[%s],"cameras":[%s],"points":%s,"colors":%s,"rms_px":%s,"skipped":%s}'
            % (int(s.zone.zone), _b(s.zone.north), f(s.origin_e), f(s.origin_n),
               _s(s.height_ref), intr, ",".join(cams), _json_array("f64", pts, 3),
               _json_array("u8", cols, 3), f(s.rms_px),
               _json_array("u32", np.asarray(s.skipped, np.uint32))))
    return text.encode()


def parse_sparse(data: bytes) -> Sparse:
    """`serde_json::from_slice::<Sparse>` (mod.rs:57-62)."""
    d = json.loads(data)
    nan = float("nan")

    def num(x):
        return nan if x is None else float(x)

    cams = [Camera(c["id"], c["path"], c["key"], c["group"],
                   np.array([num(v) for v in c["pose"]["r"]]).reshape(3, 3).T.copy(),
                   np.array([num(v) for v in c["pose"]["c"]]), c["oblique"],
                   list(c["neighbours"]), (num(c["depth_range"][0]), num(c["depth_range"][1])))
            for c in d["cameras"]]
    intr = [Intrinsics(num(k["f"]), num(k["cx"]), num(k["cy"]), num(k["k1"]), num(k["k2"]),
                       k["width"], k["height"]) for k in d["intrinsics"]]
    pts = np.array(d["points"], np.float64).reshape(-1, 3)
    cols = np.array(d["colors"], np.uint8).reshape(-1, 3)
    return Sparse(UtmZone(d["zone"]["zone"], d["zone"]["north"]), num(d["origin_e"]),
                  num(d["origin_n"]), d["height_ref"], intr, cams, pts, cols, num(d["rms_px"]),
                  list(d["skipped"]))


def origin_comment(s: Sparse) -> str:
    """mod.rs:45-53."""
    return "origin EPSG:%d E %s N %s height %s" % (
        s.zone.epsg(), rust_display_f64(s.origin_e), rust_display_f64(s.origin_n), s.height_ref)


# ---- sparse.ply ------------------------------------------------------------

_PLY_REC = np.dtype([("xyz", "<f4", (3,)), ("rgb", "u1", (3,))])


def write_ply(path: str, points_f32, colors, comment: str) -> None:
    """ply.rs:8-38: header, then 15-byte records, written to
    ``<path>.tmp`` (Path::with_extension("ply.tmp")) and renamed.  Points and
    colours must have the same length (the reference would write a header
    that disagrees with its records)."""
    p = np.asarray(points_f32, np.float32).reshape(-1, 3)
    c = np.asarray(colors, np.uint8).reshape(-1, 3)
    if len(p) != len(c):
        raise ValueError(f"{len(p)} points but {len(c)} colours")
    d = os.path.dirname(path)
    if d:
        os.makedirs(d, exist_ok=True)
    root, ext = os.path.splitext(path)
    tmp = (root if ext else path) + ".ply.tmp"
    rec = np.empty(len(p), _PLY_REC)
    rec["xyz"] = p
    rec["rgb"] = c
    head = ("ply\nformat binary_little_endian 1.0\ncomment %s\nelement vertex %d\n"
            "property float x\nproperty float y\nproperty float z\n"
            "property uchar red\nproperty uchar green\nproperty uchar blue\nend_header\n"
            % (comment, len(p)))
    with open(tmp, "wb") as fh:
        fh.write(head.encode())
        fh.write(rec.tobytes())
    os.replace(tmp, path)


def read_ply(path: str):
    """ply.rs:40-82: (points f32[n, 3], colours u8[n, 3])."""
    with open(path, "rb") as fh:
        n = None
        while True:
            line = fh.readline()
            if not line:
                raise ValueError(f"{path} has no PLY header")
            t = line.decode(errors="replace")
            if t.startswith("element vertex "):
                n = int(t[len("element vertex "):].strip())
            if t.strip() == "end_header":
                break
        n = n or 0
        rec = np.frombuffer(fh.read(15 * n), _PLY_REC, count=n)
    return rec["xyz"].copy(), rec["rgb"].copy()


# ---- the stage's outputs ---------------------------------------------------

def build_sparse(problem, summary, *, zone: UtmZone, origin_e: float, origin_n: float,
                 height_ref: str, rms_px: float, ids=None, paths=None, keys=None,
                 oblique=None, image_size=None, colors=None, skipped=()) -> Sparse:
    """The ``Sparse`` value of sparse.rs:515-554 from a bundle-adjusted
    problem and its device summary (`sparse_summary`).  `image_size`: (width,
    height) per lens group."""
    nc = problem.n_cams
    ids = list(range(nc)) if ids is None else list(ids)
    paths = [""] * nc if paths is None else list(paths)
    keys = [str(i) for i in ids] if keys is None else list(keys)
    oblique = [False] * nc if oblique is None else list(oblique)
    R = np.asarray(problem.rot, np.float64).reshape(nc, 3, 3)
    Cc = np.asarray(problem.center, np.float64).reshape(nc, 3)
    nbl = summary.neighbour_lists()
    cams = [Camera(ids[a], paths[a], keys[a], int(problem.cam_group[a]), R[a].copy(), Cc[a].copy(),
                   bool(oblique[a]), nbl[a], (float(summary.depth_range[a, 0]),
                                              float(summary.depth_range[a, 1])))
            for a in range(nc)]
    K = np.asarray(problem.intr, np.float64).reshape(-1, 5)
    intr = [Intrinsics(*map(float, k)) for k in K]
    for k, wh in zip(intr, image_size or []):
        k.width, k.height = int(wh[0]), int(wh[1])
    pts = np.asarray(problem.points, np.float64).reshape(-1, 3)
    if colors is None:
        colors = np.full((len(pts), 3), 128, np.uint8)
    return Sparse(zone, float(origin_e), float(origin_n), height_ref, intr, cams, pts,
                  np.asarray(colors, np.uint8), float(rms_px), list(skipped))


def write_sparse(out_dir: str, s: Sparse, points_f32=None) -> None:
    """run_sparse's writes (mod.rs:26-43): cameras.json, then sparse.ply with
    the points as f32 (from the device summary when given)."""
    os.makedirs(out_dir, exist_ok=True)
    with open(os.path.join(out_dir, "cameras.json"), "wb") as fh:
        fh.write(sparse_json(s))
    if points_f32 is None:
        points_f32 = np.asarray(s.points, np.float64).astype(np.float32)
    write_ply(os.path.join(out_dir, "sparse.ply"), points_f32, s.colors, origin_comment(s))


def load_sparse(out_dir: str) -> Sparse:
    """mod.rs:57-62."""
    with open(os.path.join(out_dir, "cameras.json"), "rb") as fh:
        return parse_sparse(fh.read())
