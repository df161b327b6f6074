"""The C-ABI library loads and exports every symbol include/qsgpu.h declares
(no compute calls: no GPU here); the Python binding covers the same set."""
import ctypes
import os
import re
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    text = open(os.path.join(ROOT, "include", "qsgpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return set(re.findall(r"^\s*(?:int|int64_t)\s+(qs_\w+)\s*\(", text, flags=re.M))


def _lib():
    from quspin_gb300 import _lib as L
    if not os.path.exists(L.LIB_PATH):
        subprocess.check_call(["make", "-s", "-j4", "-C", os.path.join(ROOT, "quspin_gb300", "csrc")])
    return L


def test_header_symbols_exported():
    L = _lib()
    lib = ctypes.CDLL(L.LIB_PATH)
    names = _declared()
    assert len(names) >= 38
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_matches_header():
    L = _lib()
    assert set(L.exported_names()) == _declared()
    lib = L.load()
    assert lib.qs_expm_ctl_bytes() == 56
    assert lib.qs_enum_num_candidates(32, 1, 16, 0) == 601080390
    assert lib.qs_enum_num_candidates(32, 2, 5, 5) == 4368 * 4368
    assert lib.qs_scan_scratch_elems(10) >= 1


def test_product_path_has_no_oracle_import():
    """The package must never route through the oracle."""
    pkg = os.path.join(ROOT, "quspin_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith(".py"):
                src = open(os.path.join(dirpath, f)).read()
                assert "oracle" not in src.replace("the oracle", ""), f
