"""The Zig binding (zig/r2d.zig) agrees with include/r2d_gb300.h, and the C
example (examples/frame_loop.c) compiles and links against the library.

Each `pub extern "r2d_gb300" fn` there must name an entry point the header
declares, with the same parameters in the same order (pointer depth, constness
and base type) and the same return type; the Zig `Config` and the Python
`Config` must lay out the header's `r2d_config` field for field.  CPU only:
the test reads text.
"""

import re
from pathlib import Path

import pytest

from conftest import REPO
from resolve2d_gb300 import _native as N

C_BASE = {
    "uint32_t": "u32", "uint8_t": "u8", "float": "f32", "double": "f64", "int": "c_int",
    "char": "u8", "void": "anyopaque", "r2d_config": "Config", "r2d_solver": "Solver",
    "r2d_batch": "Batch",
}


def c_type(decl: str, has_name: bool = True):
    """(pointer depth, const, base) of a C parameter or return type."""
    decl = decl.strip()
    depth = decl.count("*")
    words = decl.replace("*", " ").split()
    if has_name:
        words = words[:-1]
    const = "const" in words
    base = [w for w in words if w != "const"][-1]
    return depth, const, C_BASE[base]


def zig_type(t: str):
    t = t.strip().replace("?", "").replace("[*:0]", "*").replace("[*]", "*")
    depth = t.count("*")
    words = t.replace("*", " ").split()
    const = "const" in words
    base = [w for w in words if w != "const"][-1]
    return depth, const, "c_int" if base == "Status" else base


def header_decls():
    text = Path(REPO, "include", "r2d_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    out = {}
    for ret, name, params in re.findall(r"R2D_API\s+([\w\s\*]+?)\b(r2d_\w+)\s*\((.*?)\);", text, flags=re.S):
        plist = [] if params.strip() in ("", "void") else [c_type(p) for p in params.split(",")]
        out[name] = (c_type(ret, has_name=False), plist)
    return out


def zig_block():
    return Path(REPO, "zig", "r2d.zig").read_text()


def zig_decls():
    out = {}
    for name, params, ret in re.findall(r'pub extern "r2d_gb300" fn (r2d_\w+)\((.*?)\)\s*([^;]+);', zig_block(), flags=re.S):
        plist = [zig_type(p.split(":", 1)[1]) for p in params.split(",") if p.strip()]
        out[name] = (zig_type(ret), plist)
    return out


def test_zig_externs_match_the_header():
    h, z = header_decls(), zig_decls()
    assert set(z) == set(h), f"not bound in Zig: {sorted(set(h) - set(z))}"
    for name, (ret, params) in z.items():
        assert name in h, f"{name} is bound in Zig but not declared"
        assert ret == h[name][0], f"{name}: return type"
        assert params == h[name][1], f"{name}: parameters {params} vs {h[name][1]}"


def test_config_layouts_agree():
    text = re.sub(r"/\*.*?\*/", "", Path(REPO, "include", "r2d_gb300.h").read_text(), flags=re.S)
    body = re.search(r"typedef struct r2d_config \{(.*?)\} r2d_config;", text, flags=re.S).group(1)
    c_fields = [(f.split()[-1].lstrip("*"), c_type(f)) for f in body.split(";") if f.strip()]
    zbody = re.search(r"pub const Config = extern struct \{(.*?)\};", zig_block(), flags=re.S).group(1)
    z_fields = []
    for line in zbody.splitlines():
        line = line.split("//")[0].strip().rstrip(",")
        if line:
            name, rest = line.split(":", 1)
            z_fields.append((name.strip(), zig_type(rest.split("=")[0])))
    assert z_fields == c_fields
    assert [f for f, _ in N.Config._fields_] == [f for f, _ in c_fields]


def test_status_codes_agree():
    text = Path(REPO, "include", "r2d_gb300.h").read_text()
    header = {f"R2D_{n}": int(v) for n, v in re.findall(r"R2D_(OK|ERR_\w+)\s*=\s*(-?\d+)", text)}
    zig = {f"R2D_{n}": int(v) for n, v in re.findall(r"pub const (OK|ERR_\w+): Status = (-?\d+);", zig_block())}
    assert zig == header
    assert {v: k for k, v in header.items()} == N.STATUS_NAMES


def test_the_c_example_compiles_and_links(tmp_path):
    """examples/frame_loop.c compiles as C99 against the header and links
    against the library."""
    import shutil
    import subprocess

    cc = shutil.which("gcc")
    if cc is None:
        pytest.skip("no gcc")
    src = tmp_path / "example.c"
    src.write_text(Path(REPO, "examples", "frame_loop.c").read_text() + "\nint main(void) { return 0; }\n")
    lib_dir = str(Path(N.LIB_PATH).parent)
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-I", str(Path(REPO, "include")), str(src),
                        "-o", str(tmp_path / "example"), "-L", lib_dir, "-lr2d_gb300", f"-Wl,-rpath,{lib_dir}"],
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout
