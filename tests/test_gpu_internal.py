"""Intra-rod resistor network (stat_conduct ... internal) on the jammed box
(9 481 rods, percolating): each contact end is a node on its rod, ends no more
than one radius past their predecessor along the rod merge into one node at
the mean position, consecutive nodes of a rod are joined by a segment of
length L = dt / a (radii) and conductance rod_sigma pi a / L, and the contacts
join nodes instead of rods.

Node table, segments and contact-end nodes are compared with the oracle's
construction on the same contact list bit for bit (tolerance 0: integer ids,
and FP64 positions and lengths from the same ordered sums and IEEE divisions);
G_eff of the node network against the oracle's FP64 direct solve at rel 1e-6
(the refinement tolerance of the iterative solve is 1e-10 on the residual).
"""
import numpy as np
import pytest

from conftest import rods_struct

pytestmark = pytest.mark.gpu

SRC, SNK = 0xFFFFFFFF, 0xFFFFFFFE
NET = ("node_rod", "node_t", "seg_i", "seg_j", "seg_l", "seg_g", "edge_i", "edge_j")


@pytest.fixture(scope="module")
def jammed(gpu, oracle):
    cfg = dict(gpu.configs.JAMMED)
    sim = gpu.Simulation(cfg)
    sim.generate()
    sim.contacts()
    rod_level = sim.solve()
    rods = sim.rods()
    ct = oracle.contacts(cfg, rods_struct(rods))
    ctg = sim.contact_list()
    assert np.array_equal(ctg["I"], ct["I"]) and np.array_equal(ctg["J"], ct["J"])
    stats = sim.internal_network()
    net = sim.internal_net()
    sol = sim.solve()
    out = dict(cfg=cfg, sim=sim, rods=rods, ct=ct, stats=stats, net=net, sol=sol, rod_level=rod_level)
    yield out
    sim.close()


def test_internal_network_matches_oracle(jammed, oracle):
    net, ct = jammed["net"], jammed["ct"]
    on = oracle.internal_network(jammed["cfg"], rods_struct(jammed["rods"]), ct)
    st = jammed["stats"]
    n_ends = int(np.sum(ct["J"] < len(jammed["rods"]["x"]))) + len(ct["I"])
    assert st["contact_ends"] == n_ends == on["nodes_before_merge"]
    assert st["nodes"] == len(on["node_rod"]) and st["segments"] == len(on["seg_i"])
    assert st["nodes"] < st["contact_ends"]  # some ends merged
    for k in NET:
        assert net[k].dtype == on[k].dtype and np.array_equal(net[k], on[k]), k
    # structure: nodes ordered by (rod, t), segments join neighbours on one rod
    r, t = net["node_rod"].astype(np.int64), net["node_t"]
    assert np.all((np.diff(r) > 0) | ((np.diff(r) == 0) & (np.diff(t) > 0)))
    assert np.all(net["seg_j"] == net["seg_i"] + 1)
    assert np.array_equal(r[net["seg_i"]], r[net["seg_j"]])
    a = jammed["rods"]["a"].astype(np.float64)[r[net["seg_i"]]]
    assert np.all(net["seg_l"] > 1.0 - 1e-12)  # merged ends sit within one radius
    np.testing.assert_allclose(net["seg_l"], (t[net["seg_j"]] - t[net["seg_i"]]) / a, rtol=1e-12)
    assert np.array_equal(r[net["edge_i"]], ct["I"].astype(np.int64))
    rr = ct["J"] < len(jammed["rods"]["x"])
    assert np.array_equal(r[net["edge_j"][rr]], ct["J"][rr].astype(np.int64))
    assert np.array_equal(net["edge_j"][~rr], ct["J"][~rr])


def test_internal_conductance_matches_oracle(jammed, oracle):
    sol, on = jammed["sol"], oracle.internal_network(jammed["cfg"], rods_struct(jammed["rods"]), jammed["ct"])
    G, V, info = oracle.solve_internal(on, jammed["ct"])
    assert sol["percolating"] and sol["n_active"] == info["n_active"]
    assert sol["G_eff"] == pytest.approx(G, rel=1e-6)
    # the rods' own resistance lowers the conductance of the contact network
    assert 0 < sol["G_eff"] < jammed["rod_level"]["G_eff"]
    assert sol["n_nodes"] == len(on["node_rod"])
    np.testing.assert_allclose(jammed["sim"].voltages(), V, atol=1e-7)


def test_internal_mode_stops_at_next_contacts(gpu, jammed):
    sim = jammed["sim"]
    with pytest.raises(gpu.NanoFillerError) as ei:
        sim.adjoint()
    assert ei.value.status == 11
    # new contacts drop the node network: the solve is rod-level again
    sim.contacts()
    assert sim.solve()["G_eff"] == jammed["rod_level"]["G_eff"]
    with pytest.raises(gpu.NanoFillerError) as ei:
        sim.internal_net()
    assert ei.value.status == 10


def test_internal_coo_files(gpu, oracle, tmp_path):
    cfg = dict(gpu.configs.JAMMED)
    with gpu.Simulation(cfg) as sim:
        sim.generate()
        sim.contacts()
        sim.internal_network()
        net = sim.internal_net()
        ct = sim.contact_list()
        sim.write_internal_coo(tmp_path)

    def table(name, cols):
        lines = (tmp_path / name).read_text().splitlines()
        assert lines[0].startswith("#\tI\tJ\tData")
        rows = [ln.split() for ln in lines[1:]]
        assert all(len(x) == cols for x in rows)
        return rows
    nodes = table("Nodes.tbl.dat", 3)
    assert len(nodes) == len(net["node_rod"])
    assert [int(x[0]) for x in nodes] == list(range(len(nodes)))
    assert [int(x[1]) for x in nodes] == net["node_rod"].tolist()
    np.testing.assert_allclose([float(x[2]) for x in nodes], net["node_t"], rtol=1e-5, atol=1e-9)  # 6 digits
    segs = table("segment.LA.coo", 4)
    assert [(int(x[0]), int(x[1])) for x in segs] == list(zip(net["seg_i"].tolist(), net["seg_j"].tolist()))
    rr = ct["J"] < SNK  # rod-rod contacts
    internal = table("internal.DS.coo", 4)
    sink = table("sink.DS.coo", 4)
    source = table("source.DS.coo", 4)
    assert len(internal) == int(rr.sum())
    assert len(sink) == int(np.sum(ct["J"] == SNK)) and len(source) == int(np.sum(ct["J"] == SRC))
    pairs = sorted(zip(net["edge_i"][rr].tolist(), net["edge_j"][rr].tolist()))
    assert sorted((int(x[0]), int(x[1])) for x in internal) == pairs
