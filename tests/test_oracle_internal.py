"""Oracle of the intra-rod resistor network (stat_conduct ... internal) on hand
built contact lists: node merging (a node no more than one radius past its
predecessor merges into it, chains included, mean position), rod segments
(L = dt / a, conductance rod_sigma pi a / L) and the node-network G_eff
against a dense FP64 solve."""
import numpy as np
import pytest

SRC, SNK = 0xFFFFFFFF, 0xFFFFFFFE


def rods2(oracle):
    rods = np.zeros(2, oracle.ROD_DTYPE)
    for f, v in dict(x=0.5, y=0.5, z=0.5, cx=0.0, cy=0.0, cz=1.0, l=1.0, a=0.005).items():
        rods[f] = v
    return rods


def test_internal_nodes_segments_and_conductance(oracle):
    rods = rods2(oracle)
    # rod 0: source at t=-0.5, contact to rod 1 at t=0.1, sink at t=0.5
    # rod 1: contact at t=0.1001 and sink at t=0.1002 (0.1 um apart: one node)
    ct = dict(I=np.array([0, 0, 0, 1], np.uint32), J=np.array([1, SNK, SRC, SNK], np.uint32),
              tI=np.array([0.1, 0.5, -0.5, 0.1002]), tJ=np.array([0.1001, 0.0, 0.0, 0.0]),
              G=np.array([1e-5, 2e-5, 3e-5, 4e-5]))
    sigma = 67.0
    net = oracle.internal_network(dict(rod_sigma=sigma), rods, ct)
    assert net["nodes_before_merge"] == 5
    assert net["node_rod"].tolist() == [0, 0, 0, 1]
    assert net["node_t"][:3].tolist() == [-0.5, 0.1, 0.5]
    assert net["node_t"][3] == pytest.approx(0.10015, abs=1e-15)
    assert net["seg_i"].tolist() == [0, 1] and net["seg_j"].tolist() == [1, 2]
    a = float(np.float32(0.005))  # radii are stored in single precision
    np.testing.assert_allclose(net["seg_l"], [0.6 / a, 0.4 / a], rtol=1e-12)
    np.testing.assert_allclose(net["seg_g"], sigma * np.pi * a / net["seg_l"], rtol=1e-15)
    assert net["edge_i"].tolist() == [1, 2, 0, 3] and net["edge_j"].tolist() == [3, SNK, SRC, SNK]
    # dense solve: K v = b over the four nodes
    g01, g12 = net["seg_g"]
    K = np.zeros((4, 4))
    b = np.zeros(4)

    def edge(i, j, g):
        K[i, i] += g; K[j, j] += g; K[i, j] -= g; K[j, i] -= g
    edge(0, 1, g01); edge(1, 2, g12); edge(1, 3, 1e-5)
    K[2, 2] += 2e-5; K[3, 3] += 4e-5; K[0, 0] += 3e-5; b[0] = 3e-5
    v = np.linalg.solve(K, b)
    G, vo, info = oracle.solve_internal(net, ct)
    assert info["n_active"] == 4
    assert G == pytest.approx(3e-5 * (1 - v[0]), rel=1e-10)


def test_internal_merge_chains_and_order(oracle):
    rods = rods2(oracle)
    # three ends on rod 0 at 0, 0.004, 0.008 (each within a = 0.005 of the
    # previous one: a single node at their mean) and one at 0.3
    ct = dict(I=np.array([0, 0, 0, 0], np.uint32), J=np.array([SRC, SNK, SRC, SNK], np.uint32),
              tI=np.array([0.008, 0.0, 0.3, 0.004]), tJ=np.zeros(4), G=np.full(4, 1e-5))
    net = oracle.internal_network({}, rods, ct)
    assert net["node_rod"].tolist() == [0, 0]
    assert net["node_t"][0] == pytest.approx(0.004, abs=1e-15) and net["node_t"][1] == 0.3
    assert net["edge_i"].tolist() == [0, 0, 1, 0]
    assert len(net["seg_i"]) == 1 and net["seg_l"][0] == pytest.approx((0.3 - 0.004) / float(np.float32(0.005)), rel=1e-12)
