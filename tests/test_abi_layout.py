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
