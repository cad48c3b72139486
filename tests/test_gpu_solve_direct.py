"""Direct forms of the network solve against the PCG form (SOLVE_METHOD 2)
and the oracle. SOLVE_METHOD 0 (auto) and 1 pick block cyclic reduction when
the band after reverse Cuthill-McKee is at most 32 wide (direct = 2), else
the banded LDL^T (direct = 1); SOLVE_METHOD 3 forces the banded form. Both
refine in FP64:

- jammed rod network (band 28): reduction, banded and PCG agree on G_eff
  within 1e-9 relative and with the oracle's FP64 solve, residual at the FP64
  floor (<= 1e-13), voltages within 1e-8 V;
- the intra-rod node network (chain links in the band, band 30): the same;
- small jammed boxes, whose networks fill one to nine blocks of 32 (the
  last block alone, odd block counts, padding rows): reduction == PCG and
  the oracle;
- a batch of realisations (one CTA each) equals its PCG run.
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
    sb, vb, _, _ = solve_with(gpu, cfg, 3)
    sp, vp, _, _ = solve_with(gpu, cfg, 2)
    assert sd["direct"] == 2 and 0 < sd["bandwidth"] <= 32 and sb["direct"] == 1 and sp["direct"] == 0
    assert sd["inner_iters"] == 0 and sp["inner_iters"] > 0
    assert sd["residual"] <= 1e-13 and sb["residual"] <= 1e-13
    assert sd["G_eff"] == pytest.approx(sp["G_eff"], rel=1e-9)
    assert sd["G_eff"] == pytest.approx(sb["G_eff"], rel=1e-9)
    assert np.allclose(vd, vp, atol=1e-8, rtol=0) and np.allclose(vd, vb, atol=1e-8, rtol=0)
    G, _, _ = oracle.solve(len(rods["x"]), oracle.contacts(cfg, rods_struct(rods)), tol=1e-13)
    assert sd["G_eff"] == pytest.approx(G, rel=1e-9)


def test_direct_on_node_network(gpu):
    cfg = dict(gpu.configs.JAMMED)
    sd, vd, _, _ = solve_with(gpu, cfg, 1, internal=True)
    sb, vb, _, _ = solve_with(gpu, cfg, 3, internal=True)
    sp, vp, _, _ = solve_with(gpu, cfg, 2, internal=True)
    assert sd["direct"] == 2 and sb["direct"] == 1 and sd["n_active"] > 1000
    assert sd["residual"] <= 1e-11 and sb["residual"] <= 1e-11  # the refinement's floor on this network
    assert sd["G_eff"] == pytest.approx(sp["G_eff"], rel=1e-9)
    assert sd["G_eff"] == pytest.approx(sb["G_eff"], rel=1e-9)
    assert np.allclose(vd, vp, atol=1e-8, rtol=0) and np.allclose(vd, vb, atol=1e-8, rtol=0)


# (box edge, volume fraction, seed) -> active unknowns of the oracle's network:
# one block (2, 23, 25), three (75), five (129, 158), nine (268)
FEW_BLOCKS = [((1.1, 0.02, 1), 2), ((1.1, 0.03, 2), 25), ((1.3, 0.025, 7), 23), ((1.2, 0.03, 3), 75),
              ((1.4, 0.04, 4), 129), ((1.8, 0.05, 6), 158), ((1.6, 0.05, 5), 268)]


def test_reduction_on_few_blocks(gpu, oracle):
    """Small jammed boxes: networks of one to nine blocks of 32 (the last
    block alone, odd block counts, padding rows) against PCG and the oracle."""
    for (box, vf, seed), n_active in FEW_BLOCKS:
        cfg = dict(gpu.configs.JAMMED, box=(box, box, box), vf=vf, seed=seed, n_candidates=2_000_000)
        sd, vd, rods, _ = solve_with(gpu, cfg, 0)
        sp, vp, _, _ = solve_with(gpu, cfg, 2)
        assert sd["n_active"] == n_active
        assert sd["direct"] == 2 and sd["residual"] <= 1e-12
        assert sd["G_eff"] == pytest.approx(sp["G_eff"], rel=1e-9)
        assert np.allclose(vd, vp, atol=1e-8, rtol=0)
        G, _, _ = oracle.solve(len(rods["x"]), oracle.contacts(cfg, rods_struct(rods)), tol=1e-13)
        assert sd["G_eff"] == pytest.approx(G, rel=1e-9)


def test_direct_batch_matches_pcg(gpu):
    base = dict(gpu.configs.JAMMED, n_candidates=3_000_000)
    cfgs = [dict(base, seed=s, vf=v) for s, v in ((1, 0.045), (2, 0.05), (3, 0.04))]
    rd, _ = gpu.batch_run([dict(c, solve_method=0) for c in cfgs])
    rb, _ = gpu.batch_run([dict(c, solve_method=3) for c in cfgs])
    rp, _ = gpu.batch_run([dict(c, solve_method=2) for c in cfgs])
    for a, b, c in zip(rd, rp, rb):
        assert a["accepted"] == b["accepted"] and a["contacts"] == b["contacts"]
        assert a["G_eff"] == pytest.approx(b["G_eff"], rel=1e-9, abs=0)
        assert c["G_eff"] == pytest.approx(b["G_eff"], rel=1e-9, abs=0)
    assert any(a["G_eff"] > 0 for a in rd)
