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


def test_header_compiles_as_c_and_cpp_and_links(tmp_path):
    """A caller in plain C99 (and in C++) compiles against include/r2d_gb300.h
    and links against the library, using only its types and entry points."""
    import shutil
    import subprocess

    src = tmp_path / "caller.c"
    src.write_text(
        '#include "r2d_gb300.h"\n'
        "#include <stddef.h>\n"
        "int frame(r2d_batch* b, const float* forces, float* pose) {\n"
        "    r2d_config cfg = {0};\n"
        "    cfg.flags = R2D_FLAG_SLEEP | R2D_FLAG_WARM_START;\n"
        "    (void)cfg;\n"
        "    uint32_t launches = 0;\n"
        "    if (r2d_batch_launches_per_step(b, &launches) != R2D_OK) return -1;\n"
        "    return r2d_batch_process_io(b, 1.0f / 60.0f, 1, 8, forces, pose);\n"
        "}\n"
        "int main(void) { return r2d_version() == 1 ? 0 : 1; }\n"
    )
    inc = str(Path(REPO, "include"))
    lib_dir = str(Path(N.LIB_PATH).parent)
    for cc, std in (("gcc", "-std=c99"), ("g++", "-std=c++17")):
        exe = shutil.which(cc)
        if exe is None:
            continue
        lang = ["-x", "c++"] if cc == "g++" else []
        out = tmp_path / f"caller_{cc.replace('+', 'p')}"
        r = subprocess.run([exe, std, "-Wall", "-Werror", *lang, "-I", inc, str(src), "-o", str(out),
                            "-L", lib_dir, "-lr2d_gb300", f"-Wl,-rpath,{lib_dir}"],
                           stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        assert r.returncode == 0, r.stdout
