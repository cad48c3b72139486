"""Large workload at full size: 20 um box (periodic x, y), lognormal lengths
(median 1.5 um, sigma_ln 0.3, clipped 0.5-3 um), radii uniform 4-8 nm,
isotropic, target 2 % volume fraction, 5 M candidates from seed 7.

The oracle cannot replay the whole generation in a test, so the GPU result is
checked through properties that hold at any size and pin the sequential
insertion exactly where they look:
- the density stage keeps exactly the candidates with u < rho(x) (stream dump);
- no accepted rod centred in the interior cube [8, 12]^3 um violates the hard
  core with any accepted rod (FP64 oracle predicate);
- sampled rejected candidates each hit an accepted rod of smaller stream index,
  and sampled accepted rods hit none (FP64, brute force over all rods);
- every contact of a rod centred in that cube equals the oracle's contact
  extraction on the same rods, bit for bit.
The interior checks hand the oracle the rods centred within 3.1 um of the cube
(beyond the longest pair reach, 3 um + radii + cutoff), so every partner of an
interior rod is present; the cube lies 8 um from the periodic faces, so no
periodic image reaches it.
"""
import numpy as np
import pytest

from conftest import rods_struct

pytestmark = pytest.mark.gpu

ROD_F = ("x", "y", "z", "cx", "cy", "cz", "l", "a")


@pytest.fixture(scope="module")
def large(gpu):
    cfg = dict(gpu.configs.LARGE)
    sim = gpu.Simulation(cfg)
    g = sim.generate()
    c = sim.contacts()
    out = dict(cfg=cfg, sim=sim, gen=g, cst=c, rods=sim.rods(), ct=sim.contact_list())
    yield out
    sim.close()


def stream_keep(sim, n, chunk=1 << 20):
    keep = []
    for k0 in range(0, n, chunk):
        s = sim.stream(k0, min(chunk, n - k0))
        keep.append(s[:, 8] < s[:, 9])
    return np.concatenate(keep)


def test_large_counts_and_density_stage(gpu, large):
    cfg, g = large["cfg"], large["gen"]
    target = gpu.target_count(cfg)
    assert 860_000 < target < 1_000_000
    assert g["target"] == target and g["accepted"] == len(large["rods"]["x"])
    assert g["accepted"] == target or g["candidates_drawn"] == cfg["n_candidates"]
    assert g["accepted"] > 500_000
    keep = stream_keep(large["sim"], int(g["candidates_drawn"]))
    assert int(keep.sum()) == g["density_accepted"]
    si = large["rods"]["stream_index"].astype(np.int64)
    assert np.all(np.diff(si) > 0) and si[-1] < g["candidates_drawn"]
    assert keep[si].all()


CORE = (8.0, 12.0)
MARGIN = 3.1


def interior(rods):
    c = np.stack([rods["x"], rods["y"], rods["z"]], 1)
    core = np.all((c >= CORE[0]) & (c < CORE[1]), axis=1)
    near = np.all((c >= CORE[0] - MARGIN) & (c < CORE[1] + MARGIN), axis=1)
    return np.flatnonzero(core), np.flatnonzero(near)


def test_large_accepted_set_has_no_overlaps(large, oracle):
    cfg = large["cfg"]
    core, near = interior(large["rods"])
    assert len(core) > 4000
    # the contact routine at cutoff = hard-core gap and soft-core fraction 1 is
    # the hard-core predicate
    hc = dict(cfg, stat_dist_lim=cfg["sep"], screening=0, field_dir=0)
    ct = oracle.contacts(hc, rods_struct(large["rods"])[near])
    assert ct["counts"]["internal"] == 0


def test_large_decisions_sampled(large, oracle):
    cfg, g, rods = large["cfg"], large["gen"], large["rods"]
    si = rods["stream_index"].astype(np.uint64)
    rng = np.random.default_rng(7)
    # rejected: density-passing candidates that are not accepted
    k0 = int(rng.integers(0, int(g["candidates_drawn"]) - 200_000))
    s = large["sim"].stream(k0, 200_000)
    ks = k0 + np.flatnonzero(s[:, 8] < s[:, 9])
    rej = np.setdiff1d(ks, si.astype(np.int64))
    rej = rng.choice(rej, size=min(300, len(rej)), replace=False)
    probes = np.zeros(len(rej), oracle.ROD_DTYPE)
    for i, f in enumerate(ROD_F):
        probes[f] = s[rej - k0, i]
    fh = oracle.first_hits(cfg, probes, rej.astype(np.uint64), rods_struct(rods), si)
    assert np.all(fh >= 0)
    assert np.all(si[fh] < rej.astype(np.uint64))
    # accepted: a sample hits no earlier accepted rod
    acc = rng.choice(len(si), size=300, replace=False)
    fa = oracle.first_hits(cfg, rods_struct(rods)[acc], si[acc], rods_struct(rods), si)
    assert np.all(fa < 0)


def test_large_contacts_match_oracle(large, oracle):
    cfg, cg = large["cfg"], large["ct"]
    n = len(large["rods"]["x"])
    core, near = interior(large["rods"])
    co = oracle.contacts(dict(cfg, field_dir=0), rods_struct(large["rods"])[near])
    incore = np.zeros(n, bool)
    incore[core] = True
    # oracle pairs among the interior rods, in original ids (the map is monotone)
    oi, oj = near[co["I"]], near[co["J"]]
    so = incore[oi] | incore[oj]
    # GPU rod-rod pairs touching the cube
    gi, gj = cg["I"].astype(np.int64), cg["J"].astype(np.int64)
    rr = gj < n
    sg = rr & (incore[gi] | incore[np.where(rr, gj, 0)])
    assert sg.sum() == so.sum() > 500
    assert np.array_equal(gi[sg], oi[so]) and np.array_equal(gj[sg], oj[so])
    assert np.array_equal(cg["D"][sg], co["D"][so])
    assert np.array_equal(cg["image"][sg], co["image"][so])
