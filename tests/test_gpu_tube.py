"""The tube sweeps (the default; TUBE_LOAD < 0 selects the stencil sweeps):
the pair tests of the generation, contacts and screening run over the pairs
registered together in the cells of a fine grid along each rod's axis instead
of a stencil of cells around its centre (load 0 = the default, 64
registrations per cell; small cells share packed items). Speed only: the accepted
set and every rod float must equal the oracle's bit for bit, whatever the
load, on every kind of workload (uniform, agglomerate with von Mises-Fisher
orientation, polydisperse, the reference's angle law, jammed to the end of
the stream, open and periodic axes), and on the two full-size workloads
against the oracle's digests."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN
from golden.make_golden_configs import digest_contacts, digest_rods
from test_gpu_parity import assert_contacts_equal, assert_rods_equal

pytestmark = pytest.mark.gpu


def _run(gpu, cfg, mesh=None):
    with gpu.Simulation(cfg, mesh=mesh) as sim:
        g = sim.generate()
        rods = sim.rods()
        sim.contacts()
        ct = sim.contact_list()
    want = 0 if cfg.get("tube_load", 0.0) < 0 else 1
    assert g["tube_grid"] == want, "the tube sweeps did not run" if want else "the stencil sweeps did not run"
    return g, rods, ct


@pytest.mark.parametrize("load", [6.0, 24.0, 0.0, 96.0, -1.0])
def test_tube_small_bit_exact(gpu, oracle, load):
    cfg = dict(gpu.configs.SMALL, tube_load=load)
    g, rods, ct = _run(gpu, cfg)
    rods_o, idx_o, st = oracle.generate(cfg, batch=1)
    assert_rods_equal(rods, rods_o, idx_o)
    assert g["candidates_drawn"] == st["drawn"]
    assert_contacts_equal(ct, oracle.contacts(cfg, rods_o))


def test_tube_agglomerate_vmf_bit_exact(gpu, oracle):
    cfg = dict(gpu.configs.MEDIUM, box=(2.5, 2.5, 2.5), mesh_ext=(32, 32, 32), tube_load=24.0)
    mesh = gpu.configs.gaussian_mesh(box=(2.5, 2.5, 2.5), ext=(32, 32, 32), n_gauss=3, sigma=0.4)
    g, rods, _ = _run(gpu, cfg, mesh)
    rods_o, idx_o, st = oracle.generate(cfg, mesh=mesh, batch=8192)
    assert_rods_equal(rods, rods_o, idx_o)
    assert g["candidates_drawn"] == st["drawn"]


def test_tube_polydisperse_bit_exact(gpu, oracle):
    cfg = dict(gpu.configs.LARGE, box=(7.0, 7.0, 7.0), n_candidates=60000, tube_load=24.0)
    g, rods, _ = _run(gpu, cfg)
    rods_o, idx_o, _ = oracle.generate(cfg, batch=8192)
    assert_rods_equal(rods, rods_o, idx_o)


def test_tube_angle_law_and_periodic_z(gpu, oracle):
    cfg = dict(gpu.configs.SMALL, vf=0.015, n_candidates=200000, gen_periodic=7, theta_dev=0.3, phi_dev=0.5,
               pref_ort=(0.4, 0.7), tube_load=24.0)
    g, rods, _ = _run(gpu, cfg)
    rods_o, idx_o, _ = oracle.generate(cfg, batch=4096)
    assert_rods_equal(rods, rods_o, idx_o)


def test_tube_jammed_bit_exact(gpu, oracle):
    """Filled to jamming: late rounds reject almost every candidate against
    thousands of placed rods; in-round conflicts are dense early on."""
    cfg = dict(gpu.configs.JAMMED, box=(1.5, 1.5, 1.5), n_candidates=3_000_000, tube_load=24.0)
    g, rods, _ = _run(gpu, cfg)
    rods_o, idx_o, st = oracle.generate(cfg, batch=65536)
    assert_rods_equal(rods, rods_o, idx_o)
    assert g["candidates_drawn"] == st["drawn"]


@pytest.mark.parametrize("load", [0.0, 24.0, -1.0])
def test_tube_medium_full_size_bit_exact(gpu, oracle, load):
    cfg = dict(gpu.configs.MEDIUM, tube_load=load)
    mesh = gpu.configs.gaussian_mesh()
    g, rods, ct = _run(gpu, cfg, mesh)
    rods_o, idx_o, _ = oracle.generate(cfg, mesh=mesh, batch=16384)
    assert_rods_equal(rods, rods_o, idx_o)
    assert_contacts_equal(ct, oracle.contacts(cfg, rods_o))


def test_tube_buffer_electrodes_and_stencil_fallback(gpu, oracle):
    """Buffer-layer electrodes (the field axis periodic for contacts) on the
    tube grid; a box too short for one copy per cell falls back to the
    stencil sweeps with the same result."""
    cfg = dict(gpu.configs.SMALL, vf=0.01, n_candidates=100000, elec_buffer=1, tube_load=24.0)
    g, rods, ct = _run(gpu, cfg)
    rods_o, idx_o, _ = oracle.generate(cfg, batch=4096)
    assert_rods_equal(rods, rods_o, idx_o)
    assert_contacts_equal(ct, oracle.contacts(cfg, rods_o))
    tiny = dict(gpu.configs.SMALL, box=(1.05, 1.05, 1.05), vf=0.01, n_candidates=20000, tube_load=24.0)
    with gpu.Simulation(tiny) as sim:
        gt = sim.generate()
        rt = sim.rods()
    assert gt["tube_grid"] == 0
    r2, i2, _ = oracle.generate(tiny, batch=4096)
    assert_rods_equal(rt, r2, i2)


@pytest.mark.parametrize("load", [0.0, 24.0, -1.0])
def test_tube_large_matches_oracle_digest(gpu, load):
    with open(os.path.join(GOLDEN, "large_oracle.json")) as f:
        fx = json.load(f)
    cfg = dict(gpu.configs.LARGE, tube_load=load)
    g, rods, ct = _run(gpu, cfg)
    assert g["accepted"] == fx["accepted"] and g["candidates_drawn"] == fx["drawn"]
    assert digest_rods(rods["stream_index"], rods) == (fx["sha_stream_index"], fx["sha_rods"])
    assert digest_contacts(ct) == fx["sha_contacts"]


@pytest.mark.parametrize("load", [0.0, 24.0, -1.0])
def test_tube_batched_256_matches_oracle_digests(gpu, load):
    with open(os.path.join(GOLDEN, "batched_oracle.json")) as f:
        fx = json.load(f)["realisations"]
    reals = [dict(p, tube_load=load) for p in gpu.configs.batched_realisations(256)]
    bad = []
    with gpu.Batch(reals) as b:
        assert b.generate()["tube_grid"] == (0 if load < 0 else 1)
        b.contacts()
        for r in range(len(reals)):
            b.select(r)
            rods = b.rods()
            ct = b.contact_list()
            (hi, hr), hc = digest_rods(rods["stream_index"], rods), digest_contacts(ct)
            if (hi, hr, hc) != (fx[r]["sha_stream_index"], fx[r]["sha_rods"], fx[r]["sha_contacts"]):
                bad.append(r)
    assert not bad, f"realisations differing from the oracle: {bad[:20]}"
