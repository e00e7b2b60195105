"""Shared-memory layouts of the fused kernel's size classes (csrc/r2d_world.cuh).

make_layout is host code, so g++ compiles it here into a small program.  The
program prints each class's footprint with the host runtime's default
capacities (caps_for in csrc/r2d_capi.cu: 2.25 manifolds a body, 40 %
rectangles, one substep).  Every class must fit one CTA's 227 KB, in the lean
and the full layout.  Run with -s to see the table.  CPU only.
"""

import shutil
import subprocess
from pathlib import Path

import pytest

from conftest import REPO

PROGRAM = r"""
#define __host__
#define __device__
struct float4 { float x, y, z, w; };
#include <algorithm>
#include <cmath>
#include <cstdio>
#include "r2d_world.cuh"
using namespace r2d;
static uint32_t sz(double v) { return (uint32_t)std::min(65535.0, std::max(4.0, std::ceil(v))); }
int main() {
    const uint32_t bounds[] = {32, 64, 96, 128, 160, 192, 256, 320, 384, 448, 520};
    const double rf = 0.4;
    for (uint32_t nb : bounds) {
        Caps c{};  // caps_for with no boost
        c.nb = nb;
        c.nm = sz(2.25 * nb + 16.0);
        c.npt = sz((2.25 * nb + 16.0) * (1.08 + 0.92 * rf * rf) + 16.0);
        c.ne = sz(2.5 * nb + 64.0);
        c.np = sz(3.25 * nb + 32.0);
        c.hs = c.np;
        c.nt = 2 * nb;
        const Layout lean = make_layout(c, LayoutOpts{true, false, false, false});
        const Layout full = make_layout(c, LayoutOpts{false, false, false, false});
        printf("%u %u %u %u %u\n", nb, c.nm, c.npt, lean.total, full.total);
    }
}
"""

SMEM_PER_CTA = 227 * 1024
SMEM_PER_SM = 228 * 1024
RESERVED_PER_CTA = 1024


@pytest.fixture(scope="module")
def table(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no g++")
    d = tmp_path_factory.mktemp("layout")
    (d / "layout.cpp").write_text(PROGRAM)
    subprocess.run([cxx, "-std=c++17", "-O1", "-I", str(Path(REPO, "resolve2d_gb300", "csrc")),
                    str(d / "layout.cpp"), "-o", str(d / "layout")], check=True)
    out = subprocess.run([str(d / "layout")], check=True, stdout=subprocess.PIPE, text=True).stdout
    return [tuple(int(v) for v in line.split()) for line in out.splitlines()]


def test_every_size_class_fits_one_cta(table):
    assert [row[0] for row in table] == [32, 64, 96, 128, 160, 192, 256, 320, 384, 448, 520]
    print("\nclass  manifolds  points  lean B   full B   CTAs/SM (lean, shared memory)")
    for nb, nm, npt, lean, full in table:
        per_sm = SMEM_PER_SM // (lean + RESERVED_PER_CTA)
        print(f"{nb:5d} {nm:10d} {npt:7d} {lean:8d} {full:8d}   {per_sm}")
        assert lean <= full <= SMEM_PER_CTA
    lean = [row[3] for row in table]
    assert lean == sorted(lean)
    assert SMEM_PER_SM // (lean[-1] + RESERVED_PER_CTA) >= 2  # two of the largest worlds share an SM
