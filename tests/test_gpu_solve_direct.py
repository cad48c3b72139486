"""Direct form of the network solve (SOLVE_METHOD 1, and 0 = auto when the
band is narrow): banded LDL^T after reverse Cuthill-McKee with FP64
refinement, against the PCG form (SOLVE_METHOD 2) and the oracle:

- jammed rod network: auto picks the direct form (narrow band), G_eff equal
  to PCG's and to the oracle's FP64 solve within 1e-9 relative, residual at
  the FP64 floor (<= 1e-13), voltages equal to PCG's within 1e-8 V;
- the intra-rod node network (chain links in the band): direct == PCG
  within 1e-9;
- a batch of realisations (one CTA and one band each) equals its PCG run.
"""
import numpy as np
import pytest

from conftest import rods_struct

pytestmark = pytest.mark.gpu


def solve_with(gpu, cfg, method, internal=False):
    with gpu.Simulation(dict(cfg, solve_method=method)) as sim:
        sim.generate()
        sim.contacts()
        if internal:
            sim.internal_network()
        s = sim.solve()
        v = sim.voltages()
        rods = sim.rods()
        ct = sim.contact_list()
    return s, v, rods, ct


def test_direct_matches_pcg_and_oracle_on_jammed(gpu, oracle):
    cfg = dict(gpu.configs.JAMMED)
    sd, vd, rods, ct = solve_with(gpu, cfg, 0)
    sp, vp, _, _ = solve_with(gpu, cfg, 2)
    assert sd["direct"] == 1 and 0 < sd["bandwidth"] <= 512 and sp["direct"] == 0
    assert sd["inner_iters"] == 0 and sp["inner_iters"] > 0
    assert sd["residual"] <= 1e-13
    assert sd["G_eff"] == pytest.approx(sp["G_eff"], rel=1e-9)
    assert np.allclose(vd, vp, atol=1e-8, rtol=0)
    G, _, _ = oracle.solve(len(rods["x"]), oracle.contacts(cfg, rods_struct(rods)), tol=1e-13)
    assert sd["G_eff"] == pytest.approx(G, rel=1e-9)


def test_direct_on_node_network(gpu):
    cfg = dict(gpu.configs.JAMMED)
    sd, vd, _, _ = solve_with(gpu, cfg, 1, internal=True)
    sp, vp, _, _ = solve_with(gpu, cfg, 2, internal=True)
    assert sd["direct"] == 1 and sd["n_active"] > 1000
    assert sd["G_eff"] == pytest.approx(sp["G_eff"], rel=1e-9)
    assert np.allclose(vd, vp, atol=1e-8, rtol=0)


def test_direct_batch_matches_pcg(gpu):
    base = dict(gpu.configs.JAMMED, n_candidates=3_000_000)
    cfgs = [dict(base, seed=s, vf=v) for s, v in ((1, 0.045), (2, 0.05), (3, 0.04))]
    rd, _ = gpu.batch_run([dict(c, solve_method=0) for c in cfgs])
    rp, _ = gpu.batch_run([dict(c, solve_method=2) for c in cfgs])
    for a, b in zip(rd, rp):
        assert a["accepted"] == b["accepted"] and a["contacts"] == b["contacts"]
        assert a["G_eff"] == pytest.approx(b["G_eff"], rel=1e-9, abs=0)
    assert any(a["G_eff"] > 0 for a in rd)
