"""Host side of the C ABI (no device): the library loads and exports every
declared symbol, defaults and the keyword parser follow the reference, the
reference file formats round-trip, and errors come back as status codes."""
import ctypes as C
import os
import re
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "nanofiller_gb300.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(nf_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol(lib):
    from nanofiller_gb300 import _abi
    out = subprocess.run(["nm", "-D", "--defined-only", _abi.LIB_PATH], capture_output=True, text=True,
                         check=True).stdout
    exported = set(re.findall(r"\sT\s(nf_[a-z0-9_]+)$", out, flags=re.M))
    decl = declared_functions()
    assert decl, "no declarations parsed"
    missing = [f for f in decl if f not in exported]
    assert not missing, missing
    assert set(decl) == set(_abi.SIGNATURES), "ctypes mirror out of date"
    L = lib.load()
    assert L.nf_abi_version() == 1
    assert L.nf_status_string(7) == b"solve not converged"


def test_params_struct_layout_matches_oracle_mirror(lib):
    from oracle import nf_oracle as O
    assert C.sizeof(lib.NfParams) == C.sizeof(O.NfParams)
    assert [f for f, _ in lib.NfParams._fields_] == [f for f, _ in O.NfParams._fields_]


def test_defaults_follow_reference(lib):
    p = lib.make_params()
    # src/simPrms.cpp:22-117
    assert p.vf == pytest.approx(0.0005) and p.l == 4.0 and p.a == pytest.approx(0.010)
    assert p.tol == pytest.approx(1e-6) and p.sep == 0 and p.sc_frac == 1.0
    assert p.stat_dist_lim == pytest.approx(0.015) and p.theta_dev == -1 and p.phi_dev == -1
    from oracle import nf_oracle as O
    op = O.make_params({})
    for name, _ in lib.NfParams._fields_:
        a, b = getattr(p, name), getattr(op, name)
        if hasattr(a, "__len__") and not isinstance(a, bytes):
            a, b = list(a), list(b)
        if isinstance(a, float):
            assert a == pytest.approx(b), name
        else:
            assert a == b, name


def test_keyword_file(lib, tmp_path):
    f = tmp_path / "in.txt"
    f.write_text("\n".join([
        "VOLUME_PERCENT 1.5",
        "SPAT_DISTR_FILE NONE 5 5 5 64 64 64",
        "INC_LEN_MED 1.0",
        "INC_RAD_MED 0.005",
        "INC_SEPARATION 0.00034",
        "STAT_DIST_LIM 0.0014",
        "PREF_ORT_THETA 90",
        "DEF_THETA_DEV -1",
        "SELF_ALLIGN_STEP 0",
        "VOLUME_PERCENT_LIST 2 1.0 2.0",
        "SEED 42",
        "CANDIDATES 12345",
        "ORIENT VMF",
        "VMF_KAPPA 4",
        "LEN_LAW LOGNORMAL",
        "LEN_CLIP 0.5 3.0",
        "RAD_RANGE 0.004 0.008",
        "RAD_LAW UNIFORM",
        "TUNNEL_LAMBDA 0.00018",
        "TUBE_LOAD 32",
        "ALIGN_LAW 1",
        "AUTOTUNE 1",
        "SOME_UNKNOWN_KEY 3",
        "",
    ]))
    d, unknown = lib.params_from_file(f)
    assert unknown == 1
    assert d["vf"] == pytest.approx(0.015) and d["box"] == pytest.approx((5, 5, 5))
    assert d["mesh_ext"] == (64, 64, 64) and d["sep"] == pytest.approx(0.00034)
    assert d["pref_ort"][1] == pytest.approx(np.pi / 2, rel=1e-6) and d["theta_dev"] == -1
    assert d["seed"] == 42 and d["n_candidates"] == 12345 and d["orient_mode"] == 1
    assert d["len_mode"] == 1 and d["len_min"] == pytest.approx(0.5) and d["rad_mode"] == 2
    assert d["lambda_"] == pytest.approx(0.00018)
    assert d["tube_load"] == 32 and d["align_law"] == 1 and d["autotune"] == 1
    missing = lib.load().nf_params_from_file(str(tmp_path / "nope.txt").encode(),
                                             C.byref(lib.make_params()), None)
    assert missing == 8  # NF_ERR_IO


def test_target_counts(lib):
    from nanofiller_gb300 import configs
    assert lib.target_count(configs.SMALL) == 510
    assert lib.target_count(configs.MEDIUM) == 15916
    assert 860_000 < lib.target_count(configs.LARGE) < 1_000_000
    from oracle import nf_oracle as O
    # identical formula on both sides (simPrms::set_numCNT)
    rods, _, _ = O.generate(dict(configs.SMALL), batch=4096)
    assert len(rods) == 510


def test_state_bin_roundtrip_and_errors(lib, tmp_path):
    L = lib.load()
    hd = lib.NfStateHeader()
    for d in range(3):
        hd.phys_dim[d] = 2.0
        hd.edge[d] = 1.0
        hd.ext[d] = 2
    hd.l, hd.a, hd.ttl, hd.num, hd.tol = 1.0, 0.005, 5, 5, 1e-6
    occ = np.array([1, 0, 2, 0, 0, 0, 2, 0], np.int16)
    addr = np.cumsum(occ).astype(np.int32)
    planes = np.arange(45, dtype=np.float32)
    path = str(tmp_path / "output.bin").encode()
    assert L.nf_format_write_state_bin(path, C.byref(hd), occ.ctypes.data, addr.ctypes.data,
                                       planes.ctypes.data) == 0
    raw = open(tmp_path / "output.bin", "rb").read()
    assert len(raw) == 3 * 4 + 3 * 4 + 3 * 4 + 4 + 4 + 4 + 4 + 4 + 8 * 2 + 8 * 4 + 45 * 4
    h2 = lib.NfStateHeader()
    assert L.nf_format_read_state_bin(path, C.byref(h2), None, None, None, 0, 0) == 0
    assert list(h2.ext) == [2, 2, 2] and h2.ttl == 5 and h2.l == 1.0
    o2 = np.zeros(8, np.int16)
    a2 = np.zeros(8, np.int32)
    p2 = np.zeros(45, np.float32)
    assert L.nf_format_read_state_bin(path, C.byref(h2), o2.ctypes.data, a2.ctypes.data, p2.ctypes.data,
                                      8, 45) == 0
    assert np.array_equal(o2, occ) and np.array_equal(a2, addr) and np.array_equal(p2, planes)
    assert L.nf_format_read_state_bin(path, C.byref(h2), o2.ctypes.data, a2.ctypes.data, p2.ctypes.data,
                                      4, 45) == 5  # NF_ERR_CAPACITY
    (tmp_path / "trunc.bin").write_bytes(raw[:-20])
    assert L.nf_format_read_state_bin(str(tmp_path / "trunc.bin").encode(), C.byref(h2), o2.ctypes.data,
                                      a2.ctypes.data, p2.ctypes.data, 8, 45) == 9  # NF_ERR_FORMAT
    (tmp_path / "short.bin").write_bytes(raw[:10])
    assert L.nf_format_read_state_bin(str(tmp_path / "short.bin").encode(), C.byref(h2), None, None, None,
                                      0, 0) == 9
    assert L.nf_format_read_state_bin(str(tmp_path / "none.bin").encode(), C.byref(h2), None, None, None,
                                      0, 0) == 8


def test_vtk_format(lib, tmp_path):
    L = lib.load()
    n = 2
    f = [np.array(v, np.float32) for v in ([0.5, 1.25], [1, 2], [3, 4], [1, 0], [0, 1], [0, 0],
                                           [1, 1], [0.005, 0.005], [0, 7])]
    path = str(tmp_path / "rods.vtk").encode()
    assert L.nf_format_write_vtk(path, n, *[a.ctypes.data for a in f]) == 0
    lines = open(tmp_path / "rods.vtk").read().splitlines()
    assert lines[:5] == ["# vtk DataFile Version 2.0", "CUDA generated CNTs", "ASCII",
                         "DATASET UNSTRUCTURED_GRID", "POINTS 2 float"]
    assert lines[5] == "         0.5           1           3"   # setw(12), setprecision(6)
    assert lines[7] == "POINT_DATA 2" and lines[8] == "VECTORS CNT float"
    assert lines[11:13] == ["SCALARS LAK float 3", "LOOKUP_TABLE default"]
    assert lines[14] == "           1       0.005           7"


def test_density_file_reader(lib, tmp_path):
    p = tmp_path / "mesh.dat"
    vals = np.arange(24, dtype=np.float32) / 24
    p.write_text("5 5 5\n2 3 4\n" + " ".join(f"{v:.6f}" for v in vals))
    ext = (C.c_int * 3)()
    dim = (C.c_float * 3)()
    out = np.zeros(24, np.float32)
    L = lib.load()
    assert L.nf_read_density_file(str(p).encode(), ext, dim, out.ctypes.data, 24) == 0
    assert list(ext) == [2, 3, 4] and list(dim) == [5, 5, 5]
    np.testing.assert_allclose(out, vals, atol=1e-6)
    assert L.nf_read_density_file(str(p).encode(), ext, dim, out.ctypes.data, 10) == 5
    (tmp_path / "bad.dat").write_text("5 5\n")
    assert L.nf_read_density_file(str(tmp_path / "bad.dat").encode(), ext, dim, None, 0) == 9


def test_create_reports_status_codes(lib):
    """Invalid parameters are refused before any device work."""
    import ctypes
    L = lib.load()
    h = ctypes.c_void_p()
    bad = lib.make_params(lib.configs.SMALL, box=(0.0, 2.0, 2.0))
    st = L.nf_create(ctypes.byref(bad), ctypes.byref(h))
    assert st in (1, 3)  # NF_ERR_PARAM, or NF_ERR_NO_DEVICE on a host without GPU
    assert L.nf_destroy(None) == 1


STRUCTS = {"NfParams": "nf_params", "NfRods": "nf_rods", "NfContactList": "nf_contact_list",
           "NfGenStats": "nf_gen_stats", "NfContactStats": "nf_contact_stats", "NfSolveStats": "nf_solve_stats",
           "NfBatchResult": "nf_batch_result", "NfBatchStats": "nf_batch_stats",
           "NfInternalStats": "nf_internal_stats", "NfInternalNet": "nf_internal_net",
           "NfReduceStats": "nf_reduce_stats", "NfPairStats": "nf_pair_stats", "NfAcParams": "nf_ac_params",
           "NfAcPoint": "nf_ac_point", "NfAcStats": "nf_ac_stats", "NfAcNet": "nf_ac_net",
           "NfTuneResult": "nf_tune_result", "NfStateHeader": "nf_state_header"}


def test_ctypes_layouts_match_the_header(lib, tmp_path):
    """Every structure of the header, compiled by the C compiler, has the
    size and field offsets of its ctypes mirror (a field appended to one side
    only shows up here)."""
    from nanofiller_gb300 import _abi
    src = tmp_path / "layout.c"
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "nanofiller_gb300.h"', "int main(void) {"]
    want = []
    for py, cname in STRUCTS.items():
        cls = getattr(_abi, py)
        lines.append(f'printf("%zu\\n", sizeof({cname}));')
        want.append(C.sizeof(cls))
        for f, _ in cls._fields_:
            lines.append(f'printf("%zu\\n", offsetof({cname}, {"lambda" if f == "lambda_" else f}));')
            want.append(getattr(cls, f).offset)
    lines += ["return 0;", "}"]
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                   check=True, capture_output=True)
    got = [int(x) for x in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()]
    assert got == want
    assert set(STRUCTS.values()) == set(re.findall(r"\}\s*(nf_[a-z_]+)\s*;", open(HEADER).read())) - {"nf_status"}


def test_no_fallback_without_the_library(tmp_path):
    """With the shared library absent the package raises on first use; nothing
    runs on the CPU in its place."""
    code = (
        "import sys; sys.path.insert(0, %r)\n"
        "import nanofiller_gb300 as nf\n"
        "from nanofiller_gb300 import _abi\n"
        "_abi.LIB_PATH = %r\n"
        "for f in (lambda: nf.Simulation(dict(nf.configs.SMALL)), lambda: nf.batch_run([dict(nf.configs.SMALL)]),\n"
        "          nf.kernel_launches):\n"
        "    try:\n"
        "        f()\n"
        "    except RuntimeError as e:\n"
        "        assert 'no CPU fallback' in str(e), e\n"
        "    else:\n"
        "        raise SystemExit('ran without the library')\n"
        "print('ok')\n" % (ROOT, str(tmp_path / "absent.so")))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stderr[-2000:]
