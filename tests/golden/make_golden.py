"""Regenerates the golden fixtures in this directory.

    python tests/golden/make_golden.py

ref_predicates.npz -- outputs of the reference's OWN geometric routines
    (cnt_intersec_shr, distance_cylinder_capped + if_intersects_cylinder_capped,
    body_intersect_cylinder_capped, surf_to_cylinder_capped, get_relative_crd),
    compiled for the host from the reference's headers by oracle/ref_build.sh,
    on seeded random pairs plus constructed edge cases (parallel, collinear,
    perpendicular crossings, skew, pairs within 1e-6..1e-3 of the thresholds).
    Needs the reference checkout, named by NANOFILLER_REF.
small_oracle.npz -- the oracle's accepted set and contact list for the small
    workload (2 um box, 510 rods), pinning the stream contract and the
    pipeline across machines.
"""
import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, ROOT)

EPS = np.float32(1e-6)
SEP = np.float32(0.00034)
CUT = np.float32(0.0014)


def unit(v):
    v = np.asarray(v, np.float64)
    return v / np.linalg.norm(v)


def rotation(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def rod(r, c, l, a):
    c = unit(c)
    return np.array([r[0], r[1], r[2], c[0], c[1], c[2], l, a, 0.0], np.float32)


def make_pairs(seed=20261203):
    rng = np.random.default_rng(seed)
    A, B = [], []
    # 1) random pairs around contact range
    for _ in range(4000):
        l1, l2 = rng.choice([1.0, 1.5, 0.6]), rng.choice([1.0, 1.5, 0.6])
        a1, a2 = rng.uniform(0.004, 0.008, 2)
        r1 = rng.uniform(0.5, 4.5, 3)
        r2 = r1 + rng.normal(scale=0.4, size=3)
        A.append(rod(r1, rng.normal(size=3), l1, a1))
        B.append(rod(r2, rng.normal(size=3), l2, a2))
    # 2) constructed near-threshold crossings / end contacts / parallels
    for k in range(3000):
        R = rotation(rng)
        t = rng.uniform(0.5, 4.5, 3)
        l1, l2 = 1.0, rng.choice([1.0, 1.5])
        a1, a2 = np.float32(0.005), np.float32(rng.choice([0.005, 0.006]))
        thr = float(np.float32(a1 + a2) + (SEP if k % 2 else CUT) + EPS)
        d = thr * (1 + rng.choice([-1, 1]) * 10 ** rng.uniform(-7, -2))
        kind = k % 6
        if kind == 0:    # perpendicular crossing at distance d
            ra, ca = [0, 0, 0], [1, 0, 0]
            rb, cb = [rng.uniform(-0.4, 0.4) * l1, 0, d], [0, 1, 0]
            rb[1] = rng.uniform(-0.4, 0.4) * l2
        elif kind == 1:  # skew at angle
            ang = rng.uniform(0.05, np.pi / 2)
            ra, ca = [0, 0, 0], [1, 0, 0]
            rb, cb = [0, 0, d], [np.cos(ang), np.sin(ang), 0]
        elif kind == 2:  # collinear end to end
            ra, ca = [0, 0, 0], [1, 0, 0]
            rb, cb = [l1 / 2 + l2 / 2 + d + rng.uniform(-1e-3, 1e-3), 0, 0], [1, 0, 0]
        elif kind == 3:  # exactly parallel side by side, offset along the axis
            ra, ca = [0, 0, 0], [1, 0, 0]
            rb, cb = [rng.uniform(-1, 1) * 0.7, 0, d], [1, 0, 0]
        elif kind == 4:  # nearly parallel (inside the 1e-6 parallel tolerance or just outside)
            e = 10 ** rng.uniform(-5, -2)
            ra, ca = [0, 0, 0], [1, 0, 0]
            rb, cb = [rng.uniform(-0.5, 0.5), 0, d], [1, e, 0]
        else:            # T-shape: end of B near the side of A
            ra, ca = [0, 0, 0], [1, 0, 0]
            rb, cb = [rng.uniform(-0.45, 0.45), 0, l2 / 2 + d], [0, 0, 1]
        A.append(rod(R @ np.asarray(ra, float) + t, R @ np.asarray(ca, float), l1, a1))
        B.append(rod(R @ np.asarray(rb, float) + t, R @ np.asarray(cb, float), l2, a2))
    # 3) axis-aligned exact cases
    for d in (0.0, 0.01, 0.01034, 0.0114, 0.5):
        A.append(rod([1, 1, 1], [1, 0, 0], 1.0, 0.005))
        B.append(rod([1, 1, 1 + d], [0, 1, 0], 1.0, 0.005))
        A.append(rod([1, 1, 1], [0, 0, 1], 1.0, 0.005))
        B.append(rod([1, 1, 1 + 1.0 + d], [0, 0, 1], 1.0, 0.005))
    return np.array(A, np.float32), np.array(B, np.float32)


def ref_outputs(A, B):
    lib_path = subprocess.run([os.path.join(ROOT, "oracle", "ref_build.sh")], check=True,
                              capture_output=True, text=True).stdout.strip().splitlines()[-1]
    L = C.CDLL(lib_path)
    fp = C.POINTER(C.c_float)
    L.ref_hardcore.argtypes = [fp, fp, C.c_float, C.c_float, C.c_float]
    L.ref_contact.argtypes = [fp, fp, C.c_float, C.c_float, fp]
    L.ref_body.argtypes = [fp, C.c_float]
    L.ref_surface.argtypes = [fp, fp, fp, C.c_float]
    L.ref_surface.restype = C.c_float
    L.ref_relative.argtypes = [fp, fp, fp, fp]
    n = len(A)
    hc = np.zeros(n, np.int8)
    ct = np.zeros(n, np.int8)
    out6 = np.zeros((n, 6), np.float32)
    body = np.zeros(n, np.int8)
    surf = np.zeros(n, np.float32)
    rel = np.zeros((n, 3), np.float32)
    box = np.array([5.0, 5.0, 5.0], np.float32)
    for i in range(n):
        a = np.ascontiguousarray(A[i])
        b = np.ascontiguousarray(B[i])
        pa, pb = a.ctypes.data_as(fp), b.ctypes.data_as(fp)
        hc[i] = L.ref_hardcore(pa, pb, EPS, SEP, np.float32(1.0))
        o = np.zeros(6, np.float32)
        ct[i] = L.ref_contact(pa, pb, CUT, np.float32(1.0), o.ctypes.data_as(fp))
        out6[i] = o
        body[i] = L.ref_body(pb, o[5])
        dtt = np.ascontiguousarray(o[3:6])
        surf[i] = L.ref_surface(pa, pb, dtt.ctypes.data_as(fp), CUT)
        r = np.zeros(3, np.float32)
        L.ref_relative(pa, pb, box.ctypes.data_as(fp), r.ctypes.data_as(fp))
        rel[i] = r
    return dict(A=A, B=B, hc=hc, ct=ct, out6=out6, body=body, surf=surf, rel=rel, box=box,
                eps=EPS, sep=SEP, cut=CUT)


def small_fixture():
    from nanofiller_gb300 import configs
    from oracle import nf_oracle as O
    p = configs.SMALL
    rods, idx, st = O.generate(p, batch=1)
    ct = O.contacts(p, rods)
    g, v, info = O.solve(len(rods), ct)
    return dict(stream_index=idx, rods=rods.view(np.float32).reshape(-1, 8), drawn=st["drawn"],
                I=ct["I"], J=ct["J"], tI=ct["tI"], tJ=ct["tJ"], D=ct["D"], G=ct["G"],
                image=ct["image"], n_int=ct["counts"]["internal"], n_snk=ct["counts"]["sink"],
                n_src=ct["counts"]["source"], G_eff=g)


if __name__ == "__main__":
    A, B = make_pairs()
    ref = os.environ.get("NANOFILLER_REF")
    if ref and os.path.isdir(ref):
        np.savez_compressed(os.path.join(HERE, "ref_predicates.npz"), **ref_outputs(A, B))
        print("wrote ref_predicates.npz", len(A))
    np.savez_compressed(os.path.join(HERE, "small_oracle.npz"), **small_fixture())
    print("wrote small_oracle.npz")
