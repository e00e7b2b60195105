"""The C-ABI library loads and exports every entry point include/*.h declares."""

import ctypes
import re
from pathlib import Path

from conftest import REPO, gpu_available
from resolve2d_gb300 import _native as N

DECL = re.compile(r"R2D_API\s+[\w\s\*]+?\b(r2d_\w+)\s*\(")


def declared_symbols():
    names = []
    for h in sorted(Path(REPO, "include").glob("*.h")):
        names += DECL.findall(h.read_text())
    return names


def test_every_declared_symbol_is_exported():
    names = declared_symbols()
    assert len(names) >= 20
    lib = ctypes.CDLL(str(N.LIB_PATH))
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, f"declared but not exported: {missing}"


def test_python_binding_covers_the_header():
    assert set(declared_symbols()) <= set(N.SIGNATURES)


def test_no_device_is_an_error_not_a_crash():
    if gpu_available():
        return
    lib = N.load()
    h = ctypes.c_void_p()
    cfg = N.Config()
    assert lib.r2d_solver_create(ctypes.byref(cfg), ctypes.byref(h)) == -8
    assert lib.r2d_version() == 1
