"""The C-ABI library: builds, loads without a GPU, and exports exactly what
include/ba_gb300.h declares.  CPU only (no compute calls)."""
import ctypes
import os
import re
import subprocess

import pytest

from stitch_ba import _build, native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "ba_gb300.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(ba_[a-z_0-9]+)\s*\(", src)))


def test_header_matches_binding_list():
    assert declared_functions() == sorted(native.EXPORTS)


def test_library_builds_and_exports_every_declared_symbol():
    path = _build.build_solver()
    lib = ctypes.CDLL(path)  # loads without a GPU
    for name in declared_functions():
        assert hasattr(lib, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (ba_\w+)", out))
    assert set(declared_functions()) <= exported


def test_static_queries_work_without_gpu():
    L = native.load()
    assert L.ba_abi_version() == 1
    assert b"sm_103a" in L.ba_version()
    o = native.BaOptions()
    L.ba_default_options(ctypes.byref(o))
    assert o.max_iter == 60 and o.sigma_px == 1.0 and o.pcg_max_iter == 400
    assert o.pcg_tol == 1e-20


def test_null_context_is_rejected_without_gpu():
    L = native.load()
    assert L.ba_context_solve(None, None, None) == native.BAD_INPUT
    assert b"null context" in L.ba_last_error()


def test_header_compiles_as_c():
    src = '#include "ba_gb300.h"\nint main(void){ ba_options o; ba_default_options(&o); return 0; }\n'
    p = subprocess.run(["gcc", "-std=c99", "-fsyntax-only", "-I", os.path.dirname(HEADER), "-x", "c",
                        "-"], input=src, capture_output=True, text=True)
    assert p.returncode == 0, p.stderr


def c_layout(struct, fields):
    """sizeof and offsetof of a header struct, from a C program built here."""
    body = "".join(f'printf("%zu ", offsetof({struct}, {f}));' for f in fields)
    src = ('#include <stdio.h>\n#include <stddef.h>\n#include "ba_gb300.h"\n'
           f'int main(void){{ printf("%zu ", sizeof({struct})); {body} return 0; }}\n')
    exe = os.path.join(_build.OUT, "layout_probe")
    p = subprocess.run(["gcc", "-std=c99", "-I", os.path.dirname(HEADER), "-x", "c", "-", "-o", exe],
                       input=src, capture_output=True, text=True)
    assert p.returncode == 0, p.stderr
    vals = [int(v) for v in subprocess.run([exe], capture_output=True, text=True).stdout.split()]
    return vals[0], vals[1:]


@pytest.mark.parametrize("cname,py", [
    ("ba_problem", native.BaProblem), ("ba_state", native.BaState), ("ba_log", native.BaLog),
    ("ba_options", native.BaOptions), ("ba_stats", native.BaStatsC), ("ba_tracks", native.BaTracks),
    ("ba_pair_matches", native.BaPairMatches)])
def test_binding_structs_match_the_header_layout(cname, py):
    names = [f[0] for f in py._fields_]
    cnames = ["lambda" if n == "lam" else n for n in names]
    size, offs = c_layout(cname, cnames)
    assert ctypes.sizeof(py) == size
    assert [getattr(py, n).offset for n in names] == offs


def test_default_options_leave_the_extensions_off():
    L = native.load()
    o = native.BaOptions()
    L.ba_default_options(ctypes.byref(o))
    assert (o.coarse, o.autotune, o.stop_patience, o.pcg_kernel, o.no_graph, o.matrix_free) == (0,) * 6
    assert o.precision == 0 and o.loss == 0
    # no fault injection, the default wait limit, no workspace budget
    assert (o.fault_hold_pcg_cta, o.wait_limit_cycles, o.workspace_limit_bytes) == (0, 0, 0)
