"""The library's file writers against the reference's own writer code: the
bytes that write_CNTvtk, write_CNT_ORTvtk, write_CNTlmp (src/IO.cpp:38-146)
and save_state_BIN (src/stateSR.cpp:54-89) produced, compiled from the
reference's sources (tests/golden/make_golden_formats.py, oracle/ref_io.cpp),
for a seeded rod set and cell layout; and the state that the reference's
read_state_BIN (src/stateSR.cpp:90-134) read back from this library's
output.bin. Host-only calls: no device needed."""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import GOLDEN


@pytest.fixture(scope="module")
def fx():
    return np.load(os.path.join(GOLDEN, "ref_formats.npz"))


def _cols(rods):
    return [np.ascontiguousarray(rods[:, k], np.float32) for k in range(9)]


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def test_vtk_bytes_equal_reference(lib, fx, tmp_path):
    cols = _cols(fx["rods"])
    st = lib.load().nf_format_write_vtk(str(tmp_path / "rods.vtk").encode(), len(cols[0]), *[_p(c) for c in cols])
    assert st == 0
    assert (tmp_path / "rods.vtk").read_bytes() == fx["vtk"].tobytes()


def test_orientation_vtk_bytes_equal_reference(lib, fx, tmp_path):
    cols = _cols(fx["rods"])
    st = lib.load().nf_format_write_ort_vtk(str(tmp_path / "orient.vtk").encode(), len(cols[0]),
                                            *[_p(c) for c in cols[3:6]])
    assert st == 0
    assert (tmp_path / "orient.vtk").read_bytes() == fx["ort"].tobytes()


def test_lammps_bytes_equal_reference(lib, fx, tmp_path):
    cols = _cols(fx["rods"])
    box = np.array([20.0, 20.0, 20.0], np.float32)
    name = bytes(fx["lmp_name"]).decode()
    st = lib.load().nf_format_write_lmp(str(tmp_path / name).encode(), len(cols[0]), *[_p(c) for c in cols[:8]],
                                        _p(box), C.c_double(float(np.float32(4.579))))
    assert st == 0
    assert (tmp_path / name).read_bytes() == fx["lmp"].tobytes()


def _header(lib, fx):
    from nanofiller_gb300._abi import NfStateHeader
    h = NfStateHeader()
    for k in range(3):
        h.phys_dim[k], h.edge[k], h.ext[k] = fx["hdr_phys"][k], fx["hdr_edge"][k], int(fx["hdr_ext"][k])
    h.l, h.a, h.tol = (float(v) for v in fx["hdr_scalars"])
    h.ttl, h.num = (int(v) for v in fx["hdr_counts"])
    return h


def test_state_bin_bytes_equal_reference(lib, fx, tmp_path):
    h = _header(lib, fx)
    occ, addr = np.ascontiguousarray(fx["occ"]), np.ascontiguousarray(fx["addr"])
    planes = np.ascontiguousarray(fx["planes"])
    st = lib.load().nf_format_write_state_bin(str(tmp_path / "output.bin").encode(), C.byref(h), _p(occ), _p(addr),
                                              _p(planes))
    assert st == 0
    assert (tmp_path / "output.bin").read_bytes() == fx["state"].tobytes()


def test_reference_reads_library_state(lib, fx):
    """What read_state_BIN took from this library's output.bin is the state written."""
    assert np.array_equal(fx["read_phys"], fx["hdr_phys"]) and np.array_equal(fx["read_edge"], fx["hdr_edge"])
    assert np.array_equal(fx["read_ext"], fx["hdr_ext"]) and np.array_equal(fx["read_counts"], fx["hdr_counts"])
    assert np.array_equal(fx["read_scalars"], fx["hdr_scalars"])
    assert np.array_equal(fx["read_occ"], fx["occ"]) and np.array_equal(fx["read_addr"], fx["addr"])
    assert np.array_equal(fx["read_planes"], fx["planes"].reshape(-1))


def test_library_reads_reference_state(lib, fx, tmp_path):
    from nanofiller_gb300._abi import NfStateHeader
    path = tmp_path / "ref.bin"
    path.write_bytes(fx["state"].tobytes())
    h = NfStateHeader()
    cells = int(np.prod(fx["hdr_ext"]))
    occ, addr = np.zeros(cells, np.int16), np.zeros(cells, np.int32)
    planes = np.zeros(fx["planes"].size, np.float32)
    st = lib.load().nf_format_read_state_bin(str(path).encode(), C.byref(h), _p(occ), _p(addr), _p(planes), cells,
                                             planes.size)
    assert st == 0
    assert (h.ttl, h.num) == tuple(int(v) for v in fx["hdr_counts"])
    assert np.array_equal(occ, fx["occ"]) and np.array_equal(addr, fx["addr"])
    assert np.array_equal(planes, fx["planes"].reshape(-1))
