"""The build's rebuild rule and source list (resolve2d_gb300/build.py).  CPU only."""

import os

from resolve2d_gb300 import build as B


def test_a_target_is_stale_when_missing_or_older_than_a_source(tmp_path):
    src, out = tmp_path / "a.cu", tmp_path / "lib.so"
    src.write_text("x")
    assert B._stale(out, [src])  # never built
    out.write_text("y")
    os.utime(src, (1_000, 1_000))
    os.utime(out, (2_000, 2_000))
    assert not B._stale(out, [src])  # built after the source
    os.utime(src, (3_000, 3_000))
    assert B._stale(out, [src])  # the source changed since


def test_every_header_the_kernels_include_is_a_rebuild_dependency():
    deps = {p.name for p in B._deps()}
    for name in ("r2d_world_kernel.cu", "r2d_large.cu", "r2d_capi.cu", "r2d_world.cuh", "r2d_device.cuh",
                 "r2d_solve.cuh", "r2d_sincos.h", "r2d_colour.h", "r2d_sleep.h", "r2d_validate.h", "r2d_gb300.h"):
        assert name in deps, name


def test_the_library_builds_for_sm_103a_only_with_strict_float_flags():
    arch = " ".join(B.ARCH)
    assert "sm_103a" in arch and "sm_100" not in arch
    flags = " ".join(B.NVCC_FLAGS)
    for f in ("--fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ffp-contract=off"):
        assert f in flags
    assert "use_fast_math" not in flags
