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


def _header_params():
    """name -> list of parameter declarations, parsed from include/qsgpu.h."""
    text = open(os.path.join(ROOT, "include", "qsgpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    out = {}
    for m in re.finditer(r"^\s*(int|int64_t)\s+(qs_\w+)\s*\(([^;]*?)\)\s*;", text, flags=re.M | re.S):
        params = " ".join(m.group(3).split())
        out[m.group(2)] = (m.group(1), [] if params in ("", "void") else [p.strip() for p in params.split(",")])
    return out


def test_binding_argument_counts_and_kinds_match_header():
    """Each ctypes binding declares as many arguments as the header, with a
    pointer where the header has a pointer, a 64-bit integer for int64_t, a
    double for double and a C int for int, and the same return width."""
    import ctypes
    from quspin_gb300 import _lib as L
    hdr = _header_params()
    assert set(hdr) == set(L.exported_names())
    for name, (res, args) in L._SIGS.items():
        ret, params = hdr[name]
        assert len(args) == len(params), (name, len(args), params)
        assert (res is ctypes.c_int64) == (ret == "int64_t"), name
        for a, p in zip(args, params):
            if "*" in p:
                assert a is ctypes.c_void_p or getattr(a, "_type_", None) is not None, (name, p)
            elif p.startswith("int64_t"):
                assert a is ctypes.c_int64, (name, p)
            elif p.startswith("double"):
                assert a is ctypes.c_double, (name, p)
            elif p.startswith("int"):
                assert a is ctypes.c_int, (name, p)
