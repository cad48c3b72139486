"""Golden digests of the two workloads too large for the oracle to replay inside
a test, made once on the host cores with the FP64 C++ oracle (test
infrastructure; tens of minutes on 8 cores):

    python tests/golden/make_golden_configs.py [large|batched|all]

large_oracle.json -- the 20 um polydisperse box: lognormal lengths (median
    1.5 um, sigma_ln 0.3, clipped 0.5-3 um), radii uniform on 4-8 nm,
    isotropic, 2 % target, 5 M candidates of Philox seed 7; accepted count,
    candidates drawn, SHA-256 of the accepted stream indices, of the rod floats
    and of the contact list (1.4 nm cutoff, screening, electrodes at z = 0, L).
large_stream_index.npz -- the accepted stream indices themselves (deltas,
    compressed), so that a mismatch can be located.
batched_oracle.json -- the 256-realisation mix (box edge 2-10 um, volume
    fraction log-uniform on 0.2-2 %, seeds 0-255, 1 um x 5 nm isotropic
    rods): the same digests per realisation, its contact counts and the
    oracle's FP64 G_eff.

The digests are taken over the arrays the device path returns (digest_rods,
digest_contacts), so the GPU tests compare bit for bit without the oracle.
"""
import hashlib
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

ROD_F = ("x", "y", "z", "cx", "cy", "cz", "l", "a")


def digest_rods(stream_index, rods):
    """(sha256 of the stream indices as u64, sha256 of the eight rod fields as
    float32, field after field); rods is a record array or a dict of arrays."""
    hi = hashlib.sha256(np.ascontiguousarray(stream_index, np.uint64).tobytes()).hexdigest()
    hr = hashlib.sha256()
    for f in ROD_F:
        hr.update(np.ascontiguousarray(rods[f], np.float32).tobytes())
    return hi, hr.hexdigest()


def digest_contacts(ct):
    """sha256 over I, J (u32), D (f64), image (3 x i8), tI, tJ (f32) of the
    whole list (rod-rod contacts, then sink, then source)."""
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(ct["I"], np.uint32).tobytes())
    h.update(np.ascontiguousarray(ct["J"], np.uint32).tobytes())
    h.update(np.ascontiguousarray(ct["D"], np.float64).tobytes())
    h.update(np.ascontiguousarray(ct["image"], np.int8).tobytes())
    h.update(np.ascontiguousarray(ct["tI"], np.float32).tobytes())
    h.update(np.ascontiguousarray(ct["tJ"], np.float32).tobytes())
    return h.hexdigest()


def oracle_record(O, params, nthreads, batch=65536):
    rods, idx, st = O.generate(params, nthreads=nthreads, batch=batch)
    ct = O.contacts(params, rods, nthreads=nthreads)
    g, _, si = O.solve(len(rods), ct, tol=params.get("solve_tol", 1e-10))
    hi, hr = digest_rods(idx, rods)
    rec = dict(accepted=int(len(idx)), drawn=int(st["drawn"]), density_accepted=int(st["density_accepted"]),
               sha_stream_index=hi, sha_rods=hr, contacts=int(len(ct["I"])),
               counts={k: int(v) for k, v in ct["counts"].items()}, sha_contacts=digest_contacts(ct),
               G_eff=float(g), percolating=bool(si["percolating"]))
    return rec, idx


def make_large(O, nthreads):
    from nanofiller_gb300 import configs
    p = dict(configs.LARGE)
    t0 = time.time()
    rec, idx = oracle_record(O, p, nthreads)
    rec["oracle_s"] = round(time.time() - t0, 1)
    rec["workload"] = "20 um box, lognormal lengths, uniform radii, 2 %, 5 M candidates, seed 7"
    with open(os.path.join(HERE, "large_oracle.json"), "w") as f:
        json.dump(rec, f, indent=1)
    d = np.diff(np.concatenate([[0], idx.astype(np.int64)]))
    np.savez_compressed(os.path.join(HERE, "large_stream_index.npz"), delta=d.astype(np.uint32))
    print("large:", rec, flush=True)


def make_batched(O, nthreads):
    from nanofiller_gb300 import configs
    reals = configs.batched_realisations(256)
    out = []
    t0 = time.time()
    for r, p in enumerate(reals):
        rec, _ = oracle_record(O, p, nthreads)
        rec.update(seed=p["seed"], box=p["box"][0], vf=p["vf"])
        out.append(rec)
        if r % 16 == 0:
            print(f"batched {r}/256 {time.time() - t0:.0f} s", flush=True)
    with open(os.path.join(HERE, "batched_oracle.json"), "w") as f:
        json.dump({"workload": "256 realisations, box 2-10 um, vf 0.2-2 %, seeds 0-255",
                   "oracle_s": round(time.time() - t0, 1), "realisations": out}, f, indent=0)
    print("batched done", time.time() - t0, flush=True)


def main():
    from oracle import nf_oracle as O
    O.build()
    what = sys.argv[1] if len(sys.argv) > 1 else "all"
    nt = os.cpu_count() or 1
    if what in ("batched", "all"):
        make_batched(O, nt)
    if what in ("large", "all"):
        make_large(O, nt)


if __name__ == "__main__":
    main()
