"""The two largest workloads at full size, bit for bit against the oracle's
digests (tests/golden/make_golden_configs.py made them on the host cores):

- the 20 um polydisperse box (5 M candidates, seed 7, ~0.66 M rods), whose
  heavy rounds run the phased old-rod test (centre row, rows beside it, inner
  corners, outer rows, survivors re-binned between phases);
- the 256-realisation batch through one batch handle (nf_create_batch), every
  realisation's accepted stream indices, rod floats and contact list, G_eff
  within 1e-6 of the oracle's FP64 solve; and every realisation of the batch
  equal to the same realisation run alone (nf_create), bit for bit.

Sequential-insertion semantics (src/cudaMain.cu:113-161, restated): candidate
k is accepted iff it passes the density test and hits no earlier accepted rod.
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN
from golden.make_golden_configs import digest_contacts, digest_rods

pytestmark = pytest.mark.gpu


def _fixture(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


def test_large_full_size_matches_oracle(gpu):
    fx = _fixture("large_oracle.json")
    cfg = dict(gpu.configs.LARGE)
    with gpu.Simulation(cfg) as sim:
        g = sim.generate()
        rods = sim.rods()
        c = sim.contacts()
        ct = sim.contact_list()
    assert g["accepted"] == fx["accepted"]
    assert g["candidates_drawn"] == fx["drawn"] and g["density_accepted"] == fx["density_accepted"]
    hi, hr = digest_rods(rods["stream_index"], rods)
    if hi != fx["sha_stream_index"]:
        d = np.load(os.path.join(GOLDEN, "large_stream_index.npz"))["delta"]
        ref = np.cumsum(d.astype(np.int64))
        got = rods["stream_index"].astype(np.int64)
        n = min(len(ref), len(got))
        first = int(np.argmax(ref[:n] != got[:n])) if np.any(ref[:n] != got[:n]) else n
        pytest.fail(f"accepted set differs from the oracle's first at rank {first}")
    assert hr == fx["sha_rods"]
    assert c["contacts"] == fx["counts"]["internal"]
    assert c["n_sink"] == fx["counts"]["sink"] and c["n_source"] == fx["counts"]["source"]
    assert digest_contacts(ct) == fx["sha_contacts"]


@pytest.fixture(scope="module")
def batch256(gpu):
    reals = gpu.configs.batched_realisations(256)
    b = gpu.Batch(reals)
    g = b.generate()
    # a fresh handle's first-guess capacities hold the mix's rounds: no round
    # is run twice for an overflowing work list, FP64 queue or conflict list
    assert g["redone_rounds"] == 0
    b.contacts()
    b.solve(check=False)
    res = b.results()
    digests = []
    for r in range(len(reals)):
        b.select(r)
        rods = b.rods()
        ct = b.contact_list()
        digests.append((digest_rods(rods["stream_index"], rods), digest_contacts(ct), len(rods["x"]), len(ct["I"])))
    b.close()
    return reals, res, digests


def test_batched_256_matches_oracle(gpu, batch256):
    fx = _fixture("batched_oracle.json")["realisations"]
    reals, res, digests = batch256
    assert len(fx) == len(reals) == 256
    bad = []
    for r, (f, o, d) in enumerate(zip(fx, res, digests)):
        (hi, hr), hc, n, m = d
        ok = (o["accepted"] == f["accepted"] == n and hi == f["sha_stream_index"] and hr == f["sha_rods"]
              and m == f["contacts"] and hc == f["sha_contacts"] and o["contacts"] == f["counts"]["internal"]
              and bool(o["percolating"]) == f["percolating"])
        if ok and f["percolating"]:
            ok = abs(o["G_eff"] - f["G_eff"]) <= 1e-6 * abs(f["G_eff"])
        if not ok:
            bad.append(r)
    assert not bad, f"realisations differing from the oracle: {bad[:20]}"
    # the mix spans the stated ranges
    vf = [p["vf"] for p in reals]
    box = [p["box"][0] for p in reals]
    assert min(vf) < 0.0022 and max(vf) > 0.018 and min(box) < 2.2 and max(box) > 9.8


def test_batched_256_equals_plain(gpu, batch256):
    reals, res, digests = batch256
    bad = []
    for r, p in enumerate(reals):
        with gpu.Simulation(p) as sim:
            sim.generate()
            rods = sim.rods()
            sim.contacts()
            ct = sim.contact_list()
            s = sim.solve(check=False)
        d = (digest_rods(rods["stream_index"], rods), digest_contacts(ct), len(rods["x"]), len(ct["I"]))
        if d != digests[r] or abs(s["G_eff"] - res[r]["G_eff"]) > 1e-9 * max(abs(s["G_eff"]), 1e-300):
            bad.append(r)
    assert not bad, f"batched realisations differing from their plain runs: {bad[:20]}"


def test_batch_handle_reruns_and_guards(gpu, tmp_path):
    """A batch handle re-runs its stages with the same result as nf_batch_run;
    calls that write one realisation's files refuse a multi-realisation handle."""
    reals = gpu.configs.batched_realisations(6)
    one, _ = gpu.batch_run(reals)
    with gpu.Batch(reals) as b:
        for _ in range(2):
            b.generate()
            b.contacts()
            b.solve(check=False)
            res = b.results()
            assert [(x["accepted"], x["contacts"], x["G_eff"]) for x in res] == \
                   [(x["accepted"], x["contacts"], x["G_eff"]) for x in one]
        with pytest.raises(gpu.NanoFillerError):
            b.write_vtk(tmp_path / "x.vtk")
        with pytest.raises(gpu.NanoFillerError):
            b.select(6)


def test_block_cache_reuse_and_release(gpu):
    """Blocks of a destroyed handle serve the next one without changing any
    result; nf_release_cached_memory hands them back to the driver."""
    reals = gpu.configs.batched_realisations(8)
    a, _ = gpu.batch_run(reals)
    b, _ = gpu.batch_run(reals)
    assert gpu.load().nf_release_cached_memory() == 0
    c, _ = gpu.batch_run(reals)
    key = lambda res: [(x["accepted"], x["contacts"], x["G_eff"]) for x in res]
    assert key(a) == key(b) == key(c)
