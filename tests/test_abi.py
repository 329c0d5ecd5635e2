"""The C-ABI library loads and exports every function include/gdgpu.h declares
(no compute calls: runs without a GPU)."""
import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "gdgpu.h"
LIB = ROOT / "gridapdistributed.jl_gb300" / "lib" / "libgdgpu.so"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gd_[a-z_0-9]+)\s*\(", text)))


def test_header_declares_the_path():
    names = declared_functions()
    for must in ["gd_model_cartesian", "gd_space_create", "gd_space_get_gids", "gd_assembler_create",
                 "gd_assemble_symbolic", "gd_assemble_numeric", "gd_matrix_export", "gd_vector_export",
                 "gd_solve", "gd_spmv", "gd_fe_function_local", "gd_last_error"]:
        assert must in names


def test_library_exports_every_declared_symbol():
    if not LIB.exists():
        import __graft_entry__
        __graft_entry__.build()
    lib = ctypes.CDLL(str(LIB))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header():
    import gridap_gb300._lib as L
    assert set(declared_functions()) <= set(L.SIGNATURES)


def test_no_gpu_context_fails_cleanly():
    """Without a visible GPU, creating a context returns an error status, not a crash."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    import gridap_gb300._lib as L
    lib = L.load()
    h = ctypes.c_void_p()
    st = lib.gd_ctx_create(0, ctypes.byref(h))
    assert st != 0 and lib.gd_last_error()


_NULL_PROBE = r'''
import ctypes as C, json, sys
import gridap_gb300._lib as L
lib = L.load()
ints = (C.c_int, C.c_int32, C.c_int64, C.c_uint32, C.c_uint64, C.c_size_t, C.c_long)
out = {}
for name, types in sorted(L.SIGNATURES.items()):
    if name in ("gd_last_error", "gd_version"):
        continue
    args = [0 if t in ints else 0.0 if t in (C.c_double, C.c_float) else None for t in types]
    out[name] = int(getattr(lib, name)(*args))
print(json.dumps(out))
'''


def test_every_entry_point_rejects_null_arguments():
    """Every C-ABI function called with null handles and pointers (zero sizes) returns
    GD_ERR_ARG instead of crashing, and the destroy functions accept NULL (a no-op, as
    free does), as include/gdgpu.h states.  All calls run in one child process, so a crash
    fails this test instead of the test run."""
    import json
    import os
    import subprocess
    import sys
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    env = dict(os.environ, PYTHONPATH=os.pathsep.join([str(ROOT / "gridapdistributed.jl_gb300"),
                                                       os.environ.get("PYTHONPATH", "")]))
    p = subprocess.run([sys.executable, "-c", _NULL_PROBE], capture_output=True, text=True, env=env, timeout=300)
    assert p.returncode == 0, p.stderr[-2000:]
    status = json.loads(p.stdout.strip().splitlines()[-1])
    assert len(status) >= 80
    for name, st in status.items():
        if name.endswith("_destroy"):
            assert st == 0, name
        else:
            assert st == 1, (name, st)   # GD_ERR_ARG
