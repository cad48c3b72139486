"""Edge cases of the path on the device:

- empty inputs: a zero candidate budget and a density of 0 everywhere (every
  candidate fails the von Neumann test) give no rods, and every later stage (contacts, solve, node network, pruning,
  statistics, AC spectrum) runs on the empty set and reports it;
- a ragged batch: realisations with no rods beside normal ones, each equal to
  its single-realisation run;
- hand-placed geometry through nf_set_rods, compared with the oracle's
  contact extraction bit for bit (tolerance 0: I, J, image and the FP64
  distance): parallel rods 1 nm and 2 nm apart (the cutoff is 1.4 nm),
  crossing rods, collinear rods end to end, a pair that meets only through
  the periodic boundary, rods touching the electrode planes and a pair placed
  at the cutoff to within 1e-9 um on either side;
- a single rod and a duplicated rod (distance at rounding level) through
  contacts.
"""
import numpy as np
import pytest

from conftest import rods_struct

pytestmark = pytest.mark.gpu

SRC, SNK = 0xFFFFFFFF, 0xFFFFFFFE
A = 0.005           # rod radius, um
CUT = 1.4e-3        # tunnelling cutoff, um


def test_empty_rod_set_through_every_stage(gpu):
    for over in (dict(n_candidates=0), dict(density_default=0.0)):
        cfg = dict(gpu.configs.SMALL, **over)
        with gpu.Simulation(cfg) as sim:
            g = sim.generate()
            assert g["accepted"] == 0 and sim.n_rods() == 0
            c = sim.contacts()
            assert c["contacts"] == 0 and len(sim.contact_list()["I"]) == 0
            s = sim.solve()
            assert s["G_eff"] == 0.0 and not s["percolating"] and s["n_active"] == 0
            st = sim.internal_network()
            assert st["nodes"] == 0 and st["segments"] == 0
            assert sim.solve()["G_eff"] == 0.0
            spec = sim.ac_spectrum([1e3, 1e9])
            assert np.all(spec["i_re"] == 0) and np.all(np.isinf(spec["z_re"]))
            assert sim.nematic() == 0.0 and int(sim.phitheta().sum()) == 0
            ps = sim.pair_stats()
            assert ps["pairs"] == 0 and ps["max_per_rod"] == 0
            r = sim.reduce(2)
            assert r["rods_before"] == 0 and r["rods_after"] == 0


def test_ragged_batch(gpu):
    base = dict(gpu.configs.SMALL)
    cfgs = [dict(base, n_candidates=0), dict(base, vf=0.02, seed=3), dict(base, density_default=0.0),
            dict(base, seed=5)]
    res, st = gpu.batch_run(cfgs)
    assert st["n"] == 4
    for c, r in zip(cfgs, res):
        with gpu.Simulation(c) as sim:
            g = sim.generate()
            k = sim.contacts()
            s = sim.solve(check=False)
        assert r["accepted"] == g["accepted"] and r["contacts"] == k["contacts"]
        assert r["G_eff"] == pytest.approx(s["G_eff"], rel=1e-9, abs=0)
    assert res[0]["accepted"] == 0 and res[2]["accepted"] == 0 and res[1]["accepted"] > 0


def rod(x, y, z, c, l=1.0, a=A):
    c = np.asarray(c, np.float64)
    c = c / np.linalg.norm(c)
    return (x, y, z, c[0], c[1], c[2], l, a)


def placed():
    """Hand-placed pairs in a 12 um box (periodic x, y), each in its own
    region; electrodes at z = 0 and z = 12."""
    R = []
    # parallel along x, gap 1 nm (contact) and 2 nm (none)
    R += [rod(2.0, 2.0, 6.0, (1, 0, 0)), rod(2.0, 2.0 + 2 * A + 1.0e-3, 6.0, (1, 0, 0))]
    R += [rod(2.0, 4.0, 6.0, (1, 0, 0)), rod(2.0, 4.0 + 2 * A + 2.0e-3, 6.0, (1, 0, 0))]
    # crossing: x rod and y rod, 0.5 nm apart in z
    R += [rod(6.0, 2.0, 6.0, (1, 0, 0)), rod(6.0, 2.0, 6.0 + 2 * A + 0.5e-3, (0, 1, 0))]
    # collinear end to end along x, caps 1 nm apart
    R += [rod(6.0, 6.0, 6.0, (1, 0, 0)), rod(6.0 + 1.0 + 2 * A + 1.0e-3, 6.0, 6.0, (1, 0, 0))]
    # across the periodic x boundary: ends 1 nm apart through x = 0 = 12
    R += [rod(0.5 - 1e-9, 9.0, 6.0, (1, 0, 0)), rod(12.0 - 0.5 - 2 * A - 1.0e-3, 9.0, 6.0, (1, 0, 0))]
    # electrode planes: a rod reaching z = 0 within 1 nm, one reaching z = 12
    R += [rod(9.0, 9.0, 0.5 + A + 1.0e-3, (0, 0, 1)), rod(9.0, 2.0, 12.0 - 0.5 - A - 0.5e-3, (0, 0, 1))]
    # at the cutoff to within 1e-9 um, on either side
    R += [rod(9.0, 5.0, 3.0, (1, 0, 0)), rod(9.0, 5.0 + 2 * A + CUT - 1e-9, 3.0, (1, 0, 0))]
    R += [rod(9.0, 7.0, 3.0, (1, 0, 0)), rod(9.0, 7.0 + 2 * A + CUT + 1e-5, 3.0, (1, 0, 0))]
    # skew rods, nearly parallel (1e-7 rad)
    R += [rod(3.0, 9.0, 3.0, (1, 0, 0)), rod(3.0, 9.0 + 2 * A + 0.7e-3, 3.0, (1, 1e-7, 0))]
    return R


def as_dict(R):
    arr = np.array(R, np.float64)
    d = {f: arr[:, i].astype(np.float32) for i, f in enumerate(("x", "y", "z", "cx", "cy", "cz", "l", "a"))}
    d["stream_index"] = np.arange(len(R), dtype=np.uint64)
    return d


def test_placed_geometry_matches_oracle(gpu, oracle):
    cfg = dict(gpu.configs.SMALL, box=(12.0, 12.0, 12.0), screening=1)
    rods = as_dict(placed())
    with gpu.Simulation(cfg) as sim:
        sim.set_rods(rods)
        c = sim.contacts()
        ct = sim.contact_list()
    co = oracle.contacts(cfg, rods_struct(rods))
    for k in ("I", "J", "image"):
        assert np.array_equal(ct[k], co[k]), k
    assert np.array_equal(ct["D"], co["D"])
    pairs = {(int(i), int(j)) for i, j in zip(ct["I"], ct["J"])}
    assert (0, 1) in pairs and (2, 3) not in pairs            # 1 nm yes, 2 nm no
    assert (4, 5) in pairs and (6, 7) in pairs                # crossing, end to end
    assert (8, 9) in pairs and np.any(ct["image"][(ct["I"] == 8) & (ct["J"] == 9)] != 0)
    assert (10, SRC) in pairs and (11, SNK) in pairs          # electrode planes
    assert (12, 13) in pairs and (14, 15) not in pairs        # at the cutoff
    assert (16, 17) in pairs                                  # nearly parallel
    assert c["n_source"] >= 1 and c["n_sink"] >= 1


def test_single_and_duplicated_rods(gpu, oracle):
    cfg = dict(gpu.configs.SMALL, box=(4.0, 4.0, 4.0))
    one = as_dict([rod(2.0, 2.0, 2.0, (0.3, 0.4, 0.5))])
    two = as_dict([rod(2.0, 2.0, 2.0, (0.3, 0.4, 0.5))] * 2)
    with gpu.Simulation(cfg) as sim:
        sim.set_rods(one)
        assert sim.contacts()["contacts"] == 0
        sim.set_rods(two)
        sim.contacts()
        ct = sim.contact_list()
    co = oracle.contacts(cfg, rods_struct(two))
    assert np.array_equal(ct["I"], co["I"]) and np.array_equal(ct["D"], co["D"])
    # identical axes take the routine's parallel branch: a distance at rounding level
    assert len(ct["I"]) == 1 and ct["D"][0] < 1e-7


def test_set_orientation_equals_creation_parameters(gpu):
    base = dict(gpu.configs.SMALL, vf=0.02)
    aligned = dict(base, orient_mode=1, vmf_kappa=20.0, pref_ort=(0.0, np.pi / 2))  # about x
    with gpu.Simulation(base) as sim:
        sim.set_orientation(1, 20.0, 0.0, np.pi / 2)
        sim.generate()
        r1 = sim.rods()
        S = sim.nematic((1.0, 0.0, 0.0))
        s1 = sim.stream(0, 1000)
        with pytest.raises(gpu.NanoFillerError) as ei:
            sim.set_orientation(1, 0.0)  # a von Mises-Fisher law needs kappa > 0
        assert ei.value.status == 1
        sim.set_orientation(0)
        s0 = sim.stream(0, 1000)
    with gpu.Simulation(aligned) as ref:
        ref.generate()
        r2 = ref.rods()
        s2 = ref.stream(0, 1000)
    for f in ("x", "y", "z", "cx", "cy", "cz", "stream_index"):
        assert np.array_equal(r1[f], r2[f]), f
    assert np.array_equal(s1, s2) and S > 0.7
    assert np.mean(np.abs(s0[:, 3])) < 0.6 < np.mean(np.abs(s1[:, 3]))  # isotropic again
