"""The C ABI's structs are byte-identical to the reference's data.hpp.

tests/golden/abi_layout.json holds sizeof / offsetof of every field of the
reference structs, measured by compiling the reference's data.hpp
(tests/golden/make_golden.py); here the same program is compiled against
include/ppf_gb300.h and must print the same numbers.
"""
import json
from pathlib import Path

import abi_fields

ROOT = Path(__file__).resolve().parents[1]


def test_struct_layout_matches_reference():
    golden = json.loads((ROOT / "tests/golden/abi_layout.json").read_text())
    mine = abi_fields.measure(['#include "ppf_gb300.h"'], "Ppf", [str(ROOT / "include")])
    diff = {k: (golden[k], mine.get(k)) for k in golden if golden[k] != mine.get(k)}
    assert diff == {}


def test_library_exports_every_declared_symbol(product_lib):
    import re

    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b(\w+)\s*\([^;{]*\)\s*;", text, flags=re.M):
            name = m.group(1)
            if name not in ("if", "sizeof", "return"):
                names.add(name)
    assert len(names) > 20
    missing = [n for n in sorted(names) if not hasattr(product_lib, n)]
    assert missing == []


def test_ctypes_mirrors_match_headers():
    """The Python-side ctypes structs have the C headers' byte layout."""
    import ctypes
    import subprocess
    import tempfile

    from ppf_gb300 import abi

    lines = ['#include "ppf_gb300.h"', '#include "ppf_gb300_ext.h"',
             '#include "ppf_gb300_scene.h"', "#include <cstdio>", "#include <cstddef>",
             "int main() {"]
    expect = {}
    for cname, py in abi.MIRRORS.items():
        lines.append(f'std::printf("{cname} %zu\\n", sizeof({cname}));')
        expect[cname] = ctypes.sizeof(py)
        for fname, _ in py._fields_:
            key = f"{cname}.{fname}"
            lines.append(f'std::printf("{key} %zu\\n", offsetof({cname}, {fname}));')
            expect[key] = getattr(py, fname).offset
    lines += ["return 0; }"]
    with tempfile.TemporaryDirectory() as d:
        src = Path(d) / "m.cpp"
        exe = Path(d) / "m"
        src.write_text("\n".join(lines) + "\n")
        subprocess.run(["g++", "-std=c++17", f"-I{ROOT / 'include'}", str(src), "-o", str(exe)],
                       check=True, capture_output=True)
        out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    got = {k: int(v) for k, v in (line.split() for line in out.strip().splitlines())}
    assert got == expect


def test_host_side_argument_checks(product_lib):
    """Entry points that reject their arguments before touching the device
    (these run without a GPU)."""
    import ctypes as C

    lib = product_lib
    lib.ppf_multi_create.restype = C.c_void_p
    lib.ppf_multi_create.argtypes = [C.c_uint, C.c_void_p, C.c_void_p, C.c_uint]
    assert lib.ppf_multi_create(0, None, None, 4) is None
    assert lib.ppf_fatal_code() != 0
    lib.ppf_multi_advance.argtypes = [C.c_void_p, C.c_void_p]
    assert lib.ppf_multi_advance(None, None) == -1
    lib.ppf_multi_fetch.argtypes = [C.c_void_p, C.c_uint]
    assert lib.ppf_multi_fetch(None, 0) == -1
    lib.ppf_set_pcg_static_share.argtypes = [C.c_uint]
    assert lib.ppf_set_pcg_static_share(17) == -1
    assert lib.ppf_set_pcg_static_share(0) == 0
    stats = (C.c_ulonglong * 4)()
    lib.ppf_iteration_graph_stats(stats)
    assert all(v >= 0 for v in stats)
