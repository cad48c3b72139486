"""GPU parity: the sm_103a path through the C ABI against the CPU oracle on the
same seeded inputs. Integer/index results and FP64 decisions are bit-exact;
conductances within 1e-12 relative (exp of the host vs the device libm may
differ by an ulp); G_eff within 1e-6 relative."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, rods_struct

pytestmark = pytest.mark.gpu

ROD_F = ("x", "y", "z", "cx", "cy", "cz", "l", "a")


def perc_small(cfg):
    return dict(cfg._COMMON, box=(1.2, 1.2, 1.2), vf=0.06, l=0.5, n_candidates=300000, seed=3)


def run_gpu(nf, params, mesh=None, stages=("generate",)):
    sim = nf.Simulation(params, mesh=mesh)
    out = {}
    if "generate" in stages:
        out["gen"] = sim.generate()
        out["rods"] = sim.rods()
    if "contacts" in stages:
        out["cst"] = sim.contacts()
        out["ct"] = sim.contact_list()
    if "solve" in stages:
        out["sol"] = sim.solve()
        out["v"] = sim.voltages()
    out["sim"] = sim
    return out


def assert_rods_equal(r_gpu, rods_o, idx_o):
    assert len(r_gpu["x"]) == len(rods_o)
    assert np.array_equal(r_gpu["stream_index"], idx_o)
    for f in ROD_F:
        assert np.array_equal(r_gpu[f], rods_o[f]), f


def assert_contacts_equal(cg, co):
    n = len(co["I"])
    assert len(cg["I"]) == n
    assert np.array_equal(cg["I"], co["I"]) and np.array_equal(cg["J"], co["J"])
    assert np.array_equal(cg["tI"], co["tI"].astype(np.float32))
    assert np.array_equal(cg["tJ"], co["tJ"].astype(np.float32))
    assert np.array_equal(cg["D"], co["D"])
    assert np.array_equal(cg["image"], co["image"])
    np.testing.assert_allclose(cg["G"], co["G"], rtol=1e-12, atol=0)
    np.testing.assert_allclose(cg["S"], co["S"], rtol=1e-12, atol=1e-30)


# --------------------------------------------------------------------------- stream
@pytest.mark.parametrize("name", ["SMALL", "MEDIUM", "LARGE"])
def test_stream_bit_exact(gpu, oracle, name):
    cfg = dict(getattr(gpu.configs, name))
    mesh = gpu.configs.gaussian_mesh() if name == "MEDIUM" else None
    sim = gpu.Simulation(cfg, mesh=mesh)
    for k0, n in ((0, 40000), (123456789, 5000)):
        g = sim.stream(k0, n)
        o = oracle.candidates(cfg, k0, n, mesh=mesh)
        assert np.array_equal(g.view(np.uint32), o.view(np.uint32)), name
    sim.close()


# --------------------------------------------------------------------------- generation
def test_generate_small_bit_exact(gpu, oracle):
    cfg = dict(gpu.configs.SMALL)
    g = run_gpu(gpu, cfg)
    rods_o, idx_o, st = oracle.generate(cfg, batch=1)
    assert_rods_equal(g["rods"], rods_o, idx_o)
    assert g["gen"]["accepted"] == 510 and g["gen"]["target_reached"] == 1
    assert g["gen"]["candidates_drawn"] == st["drawn"]
    assert g["gen"]["density_accepted"] == st["density_accepted"]
    fx = np.load(os.path.join(GOLDEN, "small_oracle.npz"))
    assert np.array_equal(g["rods"]["stream_index"], fx["stream_index"])
    g["sim"].close()


def test_generate_agglomerate_vmf_bit_exact(gpu, oracle):
    cfg = dict(gpu.configs.MEDIUM, box=(2.5, 2.5, 2.5), mesh_ext=(32, 32, 32))
    mesh = gpu.configs.gaussian_mesh(box=(2.5, 2.5, 2.5), ext=(32, 32, 32), n_gauss=3, sigma=0.4)
    g = run_gpu(gpu, cfg, mesh=mesh)
    rods_o, idx_o, st = oracle.generate(cfg, mesh=mesh, batch=8192)
    assert_rods_equal(g["rods"], rods_o, idx_o)
    assert g["gen"]["candidates_drawn"] == st["drawn"]
    assert g["gen"]["fp32_would_flip"] >= 0 and g["gen"]["exact_evals"] > 0
    g["sim"].close()


def test_generate_polydisperse_bit_exact(gpu, oracle):
    cfg = dict(gpu.configs.LARGE, box=(7.0, 7.0, 7.0), n_candidates=60000)
    g = run_gpu(gpu, cfg)
    rods_o, idx_o, st = oracle.generate(cfg, batch=8192)
    assert_rods_equal(g["rods"], rods_o, idx_o)
    assert g["gen"]["target_reached"] == 0 and g["gen"]["candidates_drawn"] == 60000
    g["sim"].close()


def test_round_size_does_not_change_the_result(gpu):
    cfg = dict(gpu.configs.SMALL)
    a = run_gpu(gpu, cfg)
    b = run_gpu(gpu, dict(cfg, round_candidates=97))
    assert np.array_equal(a["rods"]["stream_index"], b["rods"]["stream_index"])
    assert b["gen"]["rounds"] > a["gen"]["rounds"]
    a["sim"].close(); b["sim"].close()


def test_reference_parallel_typo_switch(gpu, oracle):
    cfg = dict(gpu.configs.SMALL, ref_parallel_typo=1, n_candidates=3000)
    g = run_gpu(gpu, cfg)
    rods_o, idx_o, _ = oracle.generate(cfg, batch=512)
    assert_rods_equal(g["rods"], rods_o, idx_o)
    g["sim"].close()


def test_medium_full_size_bit_exact(gpu, oracle):
    cfg = dict(gpu.configs.MEDIUM)
    mesh = gpu.configs.gaussian_mesh()
    g = run_gpu(gpu, cfg, mesh=mesh, stages=("generate", "contacts"))
    rods_o, idx_o, st = oracle.generate(cfg, mesh=mesh, batch=16384)
    assert_rods_equal(g["rods"], rods_o, idx_o)
    co = oracle.contacts(cfg, rods_o)
    assert_contacts_equal(g["ct"], co)
    assert g["cst"]["contacts"] == co["counts"]["internal"]
    assert g["cst"]["screened"] == co["counts"]["screened"]
    g["sim"].close()


# --------------------------------------------------------------------------- contacts
def test_contacts_small_bit_exact(gpu, oracle):
    cfg = dict(gpu.configs.SMALL)
    g = run_gpu(gpu, cfg, stages=("generate", "contacts"))
    co = oracle.contacts(cfg, rods_struct(g["rods"]))
    assert_contacts_equal(g["ct"], co)
    fx = np.load(os.path.join(GOLDEN, "small_oracle.npz"))
    assert np.array_equal(g["ct"]["I"], fx["I"]) and np.array_equal(g["ct"]["D"], fx["D"])
    g["sim"].close()


def test_contacts_dense_with_screening(gpu, oracle):
    cfg = perc_small(gpu.configs)
    g = run_gpu(gpu, cfg, stages=("generate", "contacts"))
    co = oracle.contacts(cfg, rods_struct(g["rods"]))
    assert_contacts_equal(g["ct"], co)
    assert g["cst"]["screened"] == co["counts"]["screened"]
    assert g["cst"]["n_sink"] == co["counts"]["sink"] and g["cst"]["n_source"] == co["counts"]["source"]
    g["sim"].close()


# --------------------------------------------------------------------------- solve and adjoint
def test_solve_matches_oracle(gpu, oracle):
    cfg = perc_small(gpu.configs)
    g = run_gpu(gpu, cfg, stages=("generate", "contacts", "solve"))
    co = oracle.contacts(cfg, rods_struct(g["rods"]))
    G, v, info = oracle.solve(len(g["rods"]["x"]), co, tol=1e-13)
    assert info["percolating"] and g["sol"]["percolating"]
    assert g["sol"]["n_active"] == info["n_active"]
    assert g["sol"]["G_eff"] == pytest.approx(G, rel=1e-6)
    assert g["sol"]["residual"] <= 1e-10
    np.testing.assert_allclose(g["v"], v, atol=1e-7)
    g["sim"].close()


def test_adjoint_matches_oracle(gpu, oracle):
    cfg = perc_small(gpu.configs)
    g = run_gpu(gpu, cfg, stages=("generate", "contacts", "solve"))
    rods = rods_struct(g["rods"])
    co = oracle.contacts(cfg, rods)
    G, v, _ = oracle.solve(len(rods), co, tol=1e-13)
    go, dlo, dg0o = oracle.adjoint(cfg, rods, co, v)
    gg, dl, dg0 = g["sim"].adjoint()
    assert dg0 == pytest.approx(dg0o, rel=1e-6) and dg0 == pytest.approx(g["sol"]["G_eff"] / cfg["G0"], rel=1e-6)
    assert dl == pytest.approx(dlo, rel=1e-6)
    scale = np.abs(go).max()
    assert np.abs(gg - go).max() <= 1e-5 * scale
    g["sim"].close()


def test_solve_not_percolating_is_zero(gpu):
    cfg = dict(gpu.configs.SMALL)
    g = run_gpu(gpu, cfg, stages=("generate", "contacts", "solve"))
    assert g["sol"]["G_eff"] == 0.0 and not g["sol"]["percolating"]
    g["sim"].close()


# --------------------------------------------------------------------------- determinism, batching, files
def test_determinism(gpu):
    cfg = perc_small(gpu.configs)
    a = run_gpu(gpu, cfg, stages=("generate", "contacts", "solve"))
    b = run_gpu(gpu, cfg, stages=("generate", "contacts", "solve"))
    for f in ROD_F:
        assert np.array_equal(a["rods"][f], b["rods"][f])
    for k in ("I", "J", "D", "G"):
        assert np.array_equal(a["ct"][k], b["ct"][k])
    assert a["sol"]["G_eff"] == b["sol"]["G_eff"]
    a["sim"].close(); b["sim"].close()


def test_batched_equals_plain(gpu):
    cfgs = [perc_small(gpu.configs), dict(gpu.configs.SMALL), dict(perc_small(gpu.configs), seed=11)]
    res, st = gpu.batch_run(cfgs)
    assert st["n"] == 3
    for c, r in zip(cfgs, res):
        g = run_gpu(gpu, c, stages=("generate", "contacts", "solve"))
        assert r["accepted"] == g["gen"]["accepted"]
        assert r["contacts"] == g["cst"]["contacts"]
        assert r["G_eff"] == pytest.approx(g["sol"]["G_eff"], rel=1e-9, abs=0)
        assert r["status"] == 0
        g["sim"].close()


def test_state_bin_roundtrip_keeps_contacts(gpu, tmp_path):
    """output.bin stores the rods grouped by cell; reading it back gives the same
    rod set and, up to relabelling, the same contacts (distances to 1e-12)."""
    cfg = perc_small(gpu.configs)
    g = run_gpu(gpu, cfg, stages=("generate", "contacts"))
    g["sim"].write_state(tmp_path / "output.bin")
    g["sim"].write_vtk(tmp_path / "rods.vtk")
    g["sim"].write_coo(tmp_path)
    s2 = gpu.Simulation(cfg)
    s2.read_state(tmp_path / "output.bin")
    c2s = s2.contacts()
    c2 = s2.contact_list()
    r1, r2 = g["rods"], s2.rods()
    key = lambda r: sorted(zip(*(r[f].tolist() for f in ROD_F)))
    assert key(r1) == key(r2)
    assert c2s["contacts"] == g["cst"]["contacts"] and c2s["n_sink"] == g["cst"]["n_sink"]
    np.testing.assert_allclose(np.sort(c2["D"]), np.sort(g["ct"]["D"]), rtol=1e-12)
    lines = open(tmp_path / "internal.srt.coo").read().splitlines()
    assert lines[0] == "#\tI\tJ\tD\tS" and len(lines) == 1 + g["cst"]["contacts"]
    assert open(tmp_path / "rods.vtk").readline().strip() == "# vtk DataFile Version 2.0"
    g["sim"].close(); s2.close()


def test_call_order_errors(gpu):
    sim = gpu.Simulation(dict(gpu.configs.SMALL))
    with pytest.raises(gpu.NanoFillerError) as e:
        sim.solve()
    assert e.value.status == 10
    with pytest.raises(gpu.NanoFillerError) as e:
        sim.contacts()
    assert e.value.status == 10
    sim.close()


def test_state_bin_restores_length_radius_and_tol(gpu, tmp_path):
    """read_state_BIN restores l, a and TOL from the file (src/stateSR.cpp:96-103):
    a handle made with other values finds the same contacts after reading it."""
    cfg = perc_small(gpu.configs)
    g = run_gpu(gpu, cfg, stages=("generate", "contacts"))
    g["sim"].write_state(tmp_path / "output.bin")
    other = dict(cfg, l=0.2, a=0.002, tol=1e-5)
    with gpu.Simulation(other) as s2:
        s2.read_state(tmp_path / "output.bin")
        c2 = s2.contacts()
        s2.write_state(tmp_path / "again.bin")
    assert c2["contacts"] == g["cst"]["contacts"] and c2["n_sink"] == g["cst"]["n_sink"]
    assert (tmp_path / "again.bin").read_bytes() == (tmp_path / "output.bin").read_bytes()
    g["sim"].close()
