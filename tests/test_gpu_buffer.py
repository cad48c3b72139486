"""Buffer-layer electrodes (ELEC_BUFFER 1, the reference's `expand`):
periodic images of the rods beyond each face of the field axis are the
electrodes; a contact with an image below the box is a source contact, above
it a sink contact, one per image rod; contacts between two images are dropped.

- the contact list equals the oracle's buffer mode bit for bit (tolerance 0:
  ids, images and FP64 distances from the same arithmetic; conductances to
  1e-14, the device's exp against the host's);
- it equals, pair for pair, a literal restatement of the reference's
  expansion: the rods plus float32 copies shifted by -L and +L along the field
  axis, contacts extracted with no electrodes, roles by position, distances
  within 1e-6 um (the copies are rounded to float32 as the reference rounds
  them); pairs within 1e-6 um of the cutoff are left out of the comparison;
- G_eff of the contact network and of the intra-rod network against the
  oracle's solves at rel 1e-6, with rods that carry several source contacts;
- the adjoint reports NF_ERR_UNSUPPORTED, and a batch mixing electrode models
  is refused.
"""
import numpy as np
import pytest

from conftest import rods_struct

pytestmark = pytest.mark.gpu

SRC, SNK = 0xFFFFFFFF, 0xFFFFFFFE


@pytest.fixture(scope="module")
def buf(gpu, oracle):
    cfg = dict(gpu.configs.JAMMED, elec_buffer=1)
    sim = gpu.Simulation(cfg)
    sim.generate()
    c = sim.contacts()
    out = dict(cfg=cfg, sim=sim, cst=c, rods=sim.rods(), ct=sim.contact_list())
    out["co"] = oracle.contacts(cfg, rods_struct(out["rods"]))
    yield out
    sim.close()


def test_buffer_contacts_match_oracle(buf):
    ct, co, c = buf["ct"], buf["co"], buf["cst"]
    for k in ("I", "J", "image"):
        assert np.array_equal(ct[k], co[k]), k
    assert np.array_equal(ct["D"], co["D"])
    np.testing.assert_allclose(ct["G"], co["G"], rtol=1e-14)  # device and host exp differ in the last ulp
    assert np.array_equal(ct["tI"], co["tI"].astype(np.float32))
    assert c["n_source"] == c["n_sink"] > 0  # each pair across a face gives one of each
    src = ct["I"][ct["J"] == SRC]
    assert np.any(np.bincount(src) >= 2)  # rods with several source contacts
    n = len(buf["rods"]["x"])
    internal = ct["J"] < n
    assert np.all(ct["image"][internal][:, 2] == 0)  # no internal pair wraps the field axis


def literal_expansion(oracle, cfg, rods):
    """The reference's expand, restated: float32 copies of the rods shifted by
    -L (source layer) and +L (sink layer) along the field axis, contacts with no
    electrodes in the expanded box, roles by position. Returns
    {(rod, partner or electrode kind): [distances]}."""
    f = {1: 0, 2: 1, 4: 2}[cfg["field_dir"]]
    key = "xyz"[f]
    L = np.float32(cfg["box"][f])
    reach = np.float32(rods["l"].max() + 2 * rods["a"].max() + cfg["stat_dist_lim"] + 1e-3)
    n = len(rods)
    lo = rods[rods[key] >= L - reach].copy()
    hi = rods[rods[key] < reach].copy()
    lo[key] = lo[key] - L
    hi[key] = hi[key] + L
    ids = np.concatenate([np.arange(n), np.flatnonzero(rods[key] >= L - reach), np.flatnonzero(rods[key] < reach)])
    role = np.concatenate([np.zeros(n, int), -np.ones(len(lo), int), np.ones(len(hi), int)])
    ex = np.concatenate([rods, lo, hi])
    ex[key] = ex[key] + reach                   # the expanded box along f is [0, L + 2 reach)
    box = list(cfg["box"])
    box[f] = float(L + 2 * reach)
    p = dict(cfg, box=tuple(box), field_dir=0, elec_buffer=0, gen_periodic=cfg["gen_periodic"] & ~cfg["field_dir"])
    co = oracle.contacts(p, ex)
    out = {}
    for a, b, d in zip(co["I"], co["J"], co["D"]):
        ra, rb = role[a], role[b]
        if ra != 0 and rb != 0:
            continue                            # electrode-electrode contacts are dropped
        if ra == 0 and rb == 0:
            k = (int(ids[a]), int(ids[b]))
        else:
            rod, other = (a, b) if ra == 0 else (b, a)
            k = (int(ids[rod]), SRC if role[other] < 0 else SNK)
        out.setdefault(k, []).append(float(d))
    return out


def test_buffer_matches_literal_expansion(buf, oracle):
    rods = rods_struct(buf["rods"])
    n = len(rods)
    a = rods["a"].astype(np.float64)
    cut = buf["cfg"]["stat_dist_lim"]
    ct = buf["ct"]
    mine = {}
    for i, j, d in zip(ct["I"], ct["J"], ct["D"]):
        k = (int(i), int(j))
        mine.setdefault(k, []).append(float(d))
    lit = literal_expansion(oracle, buf["cfg"], rods)

    def away(k, ds):  # distances not within 1e-6 um of the cutoff (equal radii here)
        return sorted(d for d in ds if abs(d - 2 * a[k[0]] - cut) > 1e-6)
    keys = set(mine) | set(lit)
    n_el = 0
    for k in keys:
        m, t = away(k, mine.get(k, [])), away(k, lit.get(k, []))
        assert len(m) == len(t), (k, m, t)
        assert np.allclose(m, t, atol=1e-6, rtol=0), k
        n_el += len(m) if k[1] >= n else 0
    assert n_el > 0


def test_buffer_solves_match_oracle(buf, oracle):
    sim, co, rods = buf["sim"], buf["co"], rods_struct(buf["rods"])
    sim.contacts()
    s = sim.solve()
    G, v, info = oracle.solve(len(rods), co, tol=1e-13)
    assert s["percolating"] and s["G_eff"] == pytest.approx(G, rel=1e-6)
    sim.internal_network()
    net = sim.internal_net()
    on = oracle.internal_network(buf["cfg"], rods, co)
    for k in ("node_rod", "node_t", "seg_i", "seg_j", "seg_l", "seg_g", "edge_i", "edge_j"):
        assert np.array_equal(net[k], on[k]), k
    si = sim.solve()
    Gi, _, _ = oracle.solve_internal(on, co)
    assert si["G_eff"] == pytest.approx(Gi, rel=1e-6) and 0 < si["G_eff"] < s["G_eff"]


def test_buffer_limits(gpu, buf):
    sim = buf["sim"]
    sim.contacts()
    sim.solve()
    with pytest.raises(gpu.NanoFillerError) as ei:
        sim.adjoint()
    assert ei.value.status == 11
    base = dict(gpu.configs.SMALL)
    with pytest.raises(gpu.NanoFillerError):
        gpu.batch_run([dict(base, elec_buffer=1), dict(base)])
    with pytest.raises(gpu.NanoFillerError):
        gpu.Simulation(dict(base, elec_buffer=2))
