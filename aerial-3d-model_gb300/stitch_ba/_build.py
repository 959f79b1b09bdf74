"""In-tree build of the native libraries (no setuptools, no cmake).

* ``_build/libba_gb300.so`` — the CUDA solver behind the C ABI in
  ``include/ba_gb300.h``; every ``.cu`` file under ``csrc/`` compiled for
  sm_103a in parallel, then linked with nvcc.
* ``_build/libba_survey.so`` — the host-side synthetic survey generator.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
REPO = os.path.dirname(PKG)
INCLUDE = os.path.join(REPO, "include")

SOLVER_LIB = os.path.join(OUT, "libba_gb300.so")
SURVEY_LIB = os.path.join(OUT, "libba_survey.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr",
              "-Xcompiler", "-fPIC,-O3", "-I" + CSRC, "-I" + INCLUDE]


def _nvcc() -> str:
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libba_gb300.so")


def _sources(ext):
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(ext))


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def _stale(target, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build_survey(force: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    src = os.path.join(CSRC, "survey.cpp")
    if force or _stale(SURVEY_LIB, [src] + _headers()):
        _run(["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-I" + CSRC,
              "-o", SURVEY_LIB + ".tmp", src])
        os.replace(SURVEY_LIB + ".tmp", SURVEY_LIB)
    return SURVEY_LIB


def build_solver(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    cus = _sources(".cu")
    hdr = _headers()
    objs = []
    jobs = []
    for s in cus:
        o = os.path.join(OUT, os.path.basename(s) + ".o")
        objs.append(o)
        if force or _stale(o, [s] + hdr):
            cmd = [nvcc, *ARCH, *NVCC_FLAGS, "-c", s, "-o", o]
            if verbose:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            logs = list(ex.map(_run, jobs))
        if verbose:
            for lg in logs:
                print(lg)
    if force or jobs or _stale(SOLVER_LIB, objs):
        _run([nvcc, *ARCH, "-shared", "-o", SOLVER_LIB + ".tmp", *objs])
        os.replace(SOLVER_LIB + ".tmp", SOLVER_LIB)
    return SOLVER_LIB


def build_all(force: bool = False) -> None:
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        a = ex.submit(build_survey, force)
        b = ex.submit(build_solver, force)
        a.result()
        b.result()
