"""bench.py's own bookkeeping, on the CPU: the algorithmic byte counts of the
roofline, the launch-code decoding, the traffic record's guard against a
stale ncu capture, the clock-sample summary and the workload config that both
arms share."""
import os
import shutil

import numpy as np

import bench


def test_algorithmic_bytes():
    n, nnz = 4707969, 159282583
    # packed operand: 4 bytes per nonzero, indptr, B read and written, F read and written
    assert bench.taylor_term_bytes(n, nnz, vb=0) == nnz * 4 + 4 * (n + 1) + n * 64
    assert abs(bench.taylor_term_bytes(n, nnz, vb=0) / 1e9 - 0.957) < 1e-3
    assert bench.taylor_term_bytes(n, nnz, nvec=3, vb=1) == nnz * 5 + 4 * (n + 1) + 3 * n * 64
    # SpMV: x read once, y written once (16 bytes each per complex element)
    assert bench.spmv_bytes(n, nnz, vb=0) == nnz * 4 + 4 * (n + 1) + n * 32
    assert bench.spmv_bytes(n, nnz, nvec=8, vb=8) == nnz * 12 + 4 * (n + 1) + 8 * n * 32


def test_launch_code_names():
    assert bench.taylor_kernel_name(0x640202) == "taylor_rows_kernel"
    assert bench.taylor_kernel_name(0x440202) == "taylor_rows_kernel"
    assert bench.taylor_kernel_name(0x240204) == "taylor_r32_kernel"
    assert bench.taylor_kernel_name(0x000204) == "taylor_lp_kernel"


def test_traffic_record_matches_current_sources():
    b, note = bench.profile_traffic("taylor_rows_kernel")
    assert b is not None and b > 0, note
    # the record is of this kernel: another kernel gets no number
    b2, note2 = bench.profile_traffic("taylor_lp_kernel")
    assert b2 is None and "covers taylor_rows_kernel" in note2


def test_traffic_record_rejects_changed_sources(tmp_path, monkeypatch):
    """A copy of the tree whose kernel source differs by one byte loses the
    traffic figure."""
    root = tmp_path / "repo"
    (root / "profiles").mkdir(parents=True)
    shutil.copy(os.path.join(bench.ROOT, "profiles", "taylor_term_j1j2.md"), root / "profiles")
    src = root / "quspin_gb300" / "csrc"
    src.mkdir(parents=True)
    for f in bench.KERNEL_SOURCES["taylor_rows_kernel"]:
        shutil.copy(os.path.join(bench.ROOT, "quspin_gb300", "csrc", f), src / f)
    monkeypatch.setattr(bench, "ROOT", str(root))
    assert bench.profile_traffic("taylor_rows_kernel")[0] is not None
    with open(src / "expm_st.cu", "a") as fh:
        fh.write("\n")
    b, note = bench.profile_traffic("taylor_rows_kernel")
    assert b is None and "changed" in note


def test_clock_summary():
    cs = bench.ClockSampler.__new__(bench.ClockSampler)
    cs.out = ("2070, 2070, 900.1, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active\n"
              "2040, 2070, 1200.5, 0x0000000000000004, Not Active, Not Active, Not Active, Active\n"
              "2070, 2070, 1180.0, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active\n")
    s = cs.summary()
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0 and s["samples"] == 3
    assert s["reasons"] == ["sw_power_cap"]
    cs.out = ""
    assert cs.summary()["reasons"] == ["unsampled"]


def test_workload_config_is_shared():
    c1 = bench.workload_config(4707969, 159282583, 1)
    c2 = bench.workload_config(4707969, 159282583, 1)
    assert c1 == c2 and c1["L"] == 32 and c1["J2"] == 0.5 and c1["t"] == 5.0
    assert c1["parallelism"] == "single" and bench.workload_config(1, 1, 2)["parallelism"] == "replicas"
    assert "inputs larger than L2" in c1["l2"]


def test_j1j2_static_terms():
    """S+S- and S-S+ with J/2, SzSz with J, on the L nearest and L next-nearest
    bonds of the periodic chain."""
    L, J1, J2 = 8, 1.0, 0.5
    st = dict((o, t) for o, t in bench.j1j2_static(L, J1, J2))
    assert set(st) == {"+-", "-+", "zz"}
    for o, t in st.items():
        assert len(t) == 2 * L
        scale = 0.5 if o != "zz" else 1.0
        bonds = {(i, j): J for J, i, j in t}
        for i in range(L):
            assert bonds[(i, (i + 1) % L)] == scale * J1
            assert bonds[(i, (i + 2) % L)] == scale * J2
