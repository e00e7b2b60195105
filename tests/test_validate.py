"""Host-side validation of body arrays (resolve2d_gb300/csrc/r2d_validate.h).

The check runs inside r2d_solver_set_bodies and r2d_batch_set_worlds, which
need a device.  Here the same header is compiled into a small shim with g++
and called on every benchmark scene's arrays, which must pass, and on planted
duplicates, which must be found.  CPU only.
"""

import ctypes as C
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from conftest import REPO
from resolve2d_gb300 import scenes as S

SHIM = """
#include "r2d_validate.h"
extern "C" long long first_duplicate_id(uint32_t nw, const uint32_t* off, const uint32_t* ids, uint32_t* dup) {
    return (long long)r2d_first_duplicate_id(nw, off, ids, dup);
}
"""


@pytest.fixture(scope="module")
def check(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no g++")
    d = tmp_path_factory.mktemp("validate")
    (d / "shim.cpp").write_text(SHIM)
    so = d / "libshim.so"
    subprocess.run([cxx, "-std=c++17", "-O2", "-shared", "-fPIC", "-Wall", "-Werror",
                    "-I", str(Path(REPO, "resolve2d_gb300", "csrc")), str(d / "shim.cpp"), "-o", str(so)], check=True)
    lib = C.CDLL(str(so))
    u32p = C.POINTER(C.c_uint32)
    lib.first_duplicate_id.argtypes = [C.c_uint32, u32p, u32p, u32p]
    lib.first_duplicate_id.restype = C.c_longlong

    def run(body_off, ids):
        off = np.ascontiguousarray(body_off, np.uint32)
        ids = np.ascontiguousarray(ids, np.uint32)
        dup = C.c_uint32(0)
        w = lib.first_duplicate_id(len(off) - 1, off.ctypes.data_as(u32p), ids.ctypes.data_as(u32p), C.byref(dup))
        return int(w), int(dup.value)

    return run


@pytest.mark.parametrize("cfg", [0, 1, 2, 3])
def test_every_benchmark_scene_passes(check, cfg):
    sc = S.CONFIGS[cfg]()
    assert check(sc.body_off, sc.ids)[0] == -1


def test_ids_may_repeat_across_worlds_and_worlds_may_be_empty(check):
    off = [0, 3, 3, 6, 7]
    ids = [0, 1, 2, 2, 1, 0, 0]
    assert check(off, ids) == (-1, 0)
    assert check([0], []) == (-1, 0)


def test_a_repeated_id_names_its_world(check):
    off = [0, 3, 6, 10]
    ids = [5, 6, 7, 0, 1, 2, 9, 70000, 8, 70000]
    assert check(off, ids) == (2, 70000)
    ids2 = [5, 5, 7, 0, 1, 1, 9, 3, 8, 2]
    assert check(off, ids2) == (0, 5)  # the first world that has one


def test_a_large_world_with_one_planted_duplicate(check):
    rng = np.random.default_rng(0)
    ids = rng.permutation(200_000).astype(np.uint32)
    assert check([0, ids.size], ids) == (-1, 0)
    ids[123_456] = ids[7]
    assert check([0, ids.size], ids) == (0, int(ids[7]))
