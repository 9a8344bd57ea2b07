"""Freezes golden vectors from the reference's own element code.

Builds oracle/_ref/libppfref.so from the reference sources (oracle/Makefile),
evaluates the seeded cases of tests/element_cases.py through it and writes the
outputs to tests/golden/elements.npz. Run from the repository root:

    python tests/golden/make_golden.py
"""
import ctypes as C
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "tests"))
sys.path.insert(0, str(ROOT / "ppf-contact-solver_gb300"))

import element_cases as ec  # noqa: E402
from ppf_gb300 import build  # noqa: E402


def main():
    lib_path = build.build_reference(force=True)
    if lib_path is None:
        raise SystemExit("reference sources not found")
    ref = C.CDLL(str(lib_path))
    out = ec.evaluate(ref, "ref_")
    np.savez_compressed(Path(__file__).parent / "elements.npz", **out)
    print("wrote", len(out), "arrays")




def layout():
    """Byte layout of the reference's data.hpp, for tests/test_abi_layout.py."""
    import json

    import abi_fields

    cpp = build.reference_root() / "crates/ppf-cts-solver/src/cpp"
    shim = [
        "#include <algorithm>", "#include <cmath>",
        "using std::max; using std::min; using std::isfinite;",
        '#include "data.hpp"',
        'extern "C" { unsigned char g_ppf_fatal_code = 0; char g_ppf_fatal_detail[512]; }',
        'extern "C" void print_rust(const char *) {}',
    ]
    res = abi_fields.measure(shim, "", [str(cpp), "/usr/local/cuda/include"])
    (Path(__file__).parent / "abi_layout.json").write_text(json.dumps(res, indent=0) + "\n")
    print("wrote layout of", len(res), "fields")


if __name__ == "__main__":
    main()
    layout()
