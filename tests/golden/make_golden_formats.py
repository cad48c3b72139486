"""Fixtures that pin the library's file writers to the reference's own ones:

    NANOFILLER_REF=<reference checkout> sh oracle/ref_build.sh
    python tests/golden/make_golden_formats.py

ref_formats.npz -- a seeded set of rods (with values that exercise the
    writers' setw/setprecision formatting: tiny, negative, large, whole) and
    a synthetic cell layout; the bytes that the reference's write_CNTvtk,
    write_CNT_ORTvtk, write_CNTlmp (src/IO.cpp:38-146) and save_state_BIN
    (src/stateSR.cpp:54-89) write for them, compiled from the reference's
    sources in place by oracle/ref_build.sh (oracle/ref_io.cpp); and what the
    reference's read_state_BIN (src/stateSR.cpp:90-134) reads back from the
    output.bin that this library writes for the same state.
"""
import ctypes as C
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, ROOT)


def inputs():
    rng = np.random.default_rng(20261204)
    n = 40
    rods = np.zeros((n, 9), np.float32)
    rods[:, 0:3] = rng.uniform(0, 20, (n, 3))
    c = rng.normal(size=(n, 3))
    rods[:, 3:6] = c / np.linalg.norm(c, axis=1, keepdims=True)
    rods[:, 6] = rng.uniform(0.5, 3.0, n)
    rods[:, 7] = rng.uniform(0.004, 0.008, n)
    rods[:, 8] = rng.integers(0, 1000, n)
    special = [1e-7, -0.5, 12345.678, 0.0, 1e5, 2.0, -1e-30, 0.1, 3.14159265, 999999.5]
    for i, v in enumerate(special):
        rods[i, i % 9] = v
    rods[10, 3:6] = [1.0, 0.0, 0.0]
    rods[11, 3:6] = [-1.0, 0.0, 0.0]
    ext = np.array([2, 3, 2], np.int32)
    cells = int(np.prod(ext))
    occ = rng.integers(0, 6, cells).astype(np.int16)
    ttl = int(occ.sum())
    addr = np.cumsum(occ).astype(np.int32)
    planes = rng.uniform(-1, 20, (9, ttl)).astype(np.float32)
    hdr = dict(phys=np.array([20, 20, 20], np.float32), edge=np.array([10, 6.6666665, 10], np.float32), ext=ext,
               l=np.float32(1.5), a=np.float32(0.006), ttl=ttl, num=ttl - 2, tol=np.float32(1e-6))
    return rods, hdr, occ, addr, planes


def main():
    rods, hdr, occ, addr, planes = inputs()
    L = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libref_io.so"))
    fp = C.POINTER(C.c_float)
    out = {}
    with tempfile.TemporaryDirectory() as d:
        cwd = os.getcwd()
        os.chdir(d)  # the reference writers write "./<base>.<ext>"
        try:
            r = np.ascontiguousarray(rods)
            L.ref_write_vtk(b"rods", len(r), r.ctypes.data_as(fp))
            L.ref_write_ort_vtk(b"orient", len(r), r.ctypes.data_as(fp))
            box = np.array([20.0, 20.0, 20.0], np.float32)
            L.ref_write_lmp.argtypes = [C.c_char_p, C.c_int, fp, fp, C.c_float]
            L.ref_write_lmp(b"output", len(r), r.ctypes.data_as(fp), box.ctypes.data_as(fp), C.c_float(4.579))
            L.ref_save_state.argtypes = [C.c_char_p, fp, fp, C.POINTER(C.c_int), C.c_float, C.c_float, C.c_int,
                                         C.c_int, C.c_float, C.c_void_p, C.c_void_p, C.c_void_p]
            pl = np.ascontiguousarray(planes)
            L.ref_save_state(b"ref_state.bin", hdr["phys"].ctypes.data_as(fp), hdr["edge"].ctypes.data_as(fp),
                             hdr["ext"].ctypes.data_as(C.POINTER(C.c_int)), C.c_float(hdr["l"]), C.c_float(hdr["a"]),
                             hdr["ttl"], hdr["num"], C.c_float(hdr["tol"]), occ.ctypes.data, addr.ctypes.data,
                             pl.ctypes.data)
            for name, f in (("vtk", "rods.vtk"), ("ort", "orient.vtk"), ("state", "ref_state.bin")):
                out[name] = np.frombuffer(open(f, "rb").read(), np.uint8)
            lmp = [f for f in os.listdir(".") if f.startswith("output")]
            out["lmp"] = np.frombuffer(open(lmp[0], "rb").read(), np.uint8)
            out["lmp_name"] = np.frombuffer(lmp[0].encode(), np.uint8)
            # the reference reads the library's output.bin
            import nanofiller_gb300 as nf
            from nanofiller_gb300._abi import NfStateHeader
            h = NfStateHeader()
            for k in range(3):
                h.phys_dim[k], h.edge[k], h.ext[k] = hdr["phys"][k], hdr["edge"][k], hdr["ext"][k]
            h.l, h.a, h.ttl, h.num, h.tol = hdr["l"], hdr["a"], hdr["ttl"], hdr["num"], hdr["tol"]
            st = nf.load().nf_format_write_state_bin(b"lib_state.bin", C.byref(h), occ.ctypes.data, addr.ctypes.data,
                                                      pl.ctypes.data)
            assert st == 0, st
            ph, ed, ex = np.zeros(3, np.float32), np.zeros(3, np.float32), np.zeros(3, np.int32)
            l_, a_, tol_ = C.c_float(), C.c_float(), C.c_float()
            ttl_, num_ = C.c_int(), C.c_int()
            ro, ra, rp = np.zeros(64, np.int16), np.zeros(64, np.int32), np.zeros(9 * hdr["ttl"] + 9, np.float32)
            L.ref_read_state.argtypes = [C.c_char_p, fp, fp, C.POINTER(C.c_int), fp, fp, C.POINTER(C.c_int),
                                         C.POINTER(C.c_int), fp, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int]
            rc = L.ref_read_state(b"lib_state.bin", ph.ctypes.data_as(fp), ed.ctypes.data_as(fp),
                                  ex.ctypes.data_as(C.POINTER(C.c_int)), C.byref(l_), C.byref(a_), C.byref(ttl_),
                                  C.byref(num_), C.byref(tol_), ro.ctypes.data, ra.ctypes.data, rp.ctypes.data, 64,
                                  len(rp))
            assert rc == 0
            cells = int(np.prod(ex))
            out.update(read_phys=ph, read_edge=ed, read_ext=ex,
                       read_scalars=np.array([l_.value, a_.value, tol_.value], np.float32),
                       read_counts=np.array([ttl_.value, num_.value], np.int32), read_occ=ro[:cells],
                       read_addr=ra[:cells], read_planes=rp[:9 * ttl_.value])
        finally:
            os.chdir(cwd)
    out.update(rods=rods, occ=occ, addr=addr, planes=planes, hdr_phys=hdr["phys"], hdr_edge=hdr["edge"],
               hdr_ext=hdr["ext"], hdr_scalars=np.array([hdr["l"], hdr["a"], hdr["tol"]], np.float32),
               hdr_counts=np.array([hdr["ttl"], hdr["num"]], np.int32))
    np.savez_compressed(os.path.join(HERE, "ref_formats.npz"), **out)
    print("wrote ref_formats.npz:", {k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main()
