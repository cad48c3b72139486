"""Tuning settings change speed only: every value of stencil_radius,
round_overshoot and two_phase_work gives the oracle's accepted set and contact
list bit for bit (two_phase_work = 1 forces the two-phase old-rod test on every
round, which the default threshold keeps for heavy rounds only), and
nf_autotune (on the tube grid: tube_load and round_overshoot; on the stencil
sweeps: the three above) leaves the handle, single or batch, holding the same
rods."""
import numpy as np
import pytest

from conftest import rods_struct

pytestmark = pytest.mark.gpu

ROD_F = ("x", "y", "z", "cx", "cy", "cz", "l", "a")

SETTINGS = [dict(stencil_radius=1), dict(stencil_radius=2), dict(round_overshoot=1.5),
            dict(round_overshoot=3.0), dict(two_phase_work=1.0), dict(two_phase_work=-1.0),
            dict(stencil_radius=1, two_phase_work=1.0)]


@pytest.fixture(scope="module")
def medium_oracle(gpu, oracle):
    cfg = dict(gpu.configs.MEDIUM)
    mesh = gpu.configs.gaussian_mesh()
    rods_o, idx_o, _ = oracle.generate(cfg, mesh=mesh, batch=16384)
    return cfg, mesh, rods_o, idx_o, oracle.contacts(cfg, rods_o)


def check(sim, rods_o, idx_o, co):
    r = sim.rods()
    assert np.array_equal(r["stream_index"], idx_o)
    for f in ROD_F:
        assert np.array_equal(r[f], rods_o[f]), f
    ct = sim.contact_list()
    assert np.array_equal(ct["I"], co["I"]) and np.array_equal(ct["J"], co["J"])
    assert np.array_equal(ct["D"], co["D"]) and np.array_equal(ct["image"], co["image"])


@pytest.mark.parametrize("setting", SETTINGS, ids=lambda d: ",".join(f"{k}={v}" for k, v in d.items()))
def test_settings_do_not_change_results(gpu, medium_oracle, setting):
    cfg, mesh, rods_o, idx_o, co = medium_oracle
    with gpu.Simulation(dict(cfg, **setting), mesh=mesh) as sim:
        g = sim.generate()
        sim.contacts()
        check(sim, rods_o, idx_o, co)
        if setting.get("two_phase_work", 0) > 0:
            assert g["work_items"] > 0


@pytest.mark.parametrize("load", [0.0, -1.0])
def test_autotune_keeps_results(gpu, medium_oracle, load):
    """Tube grid (load 0: the default): tube_load and round_overshoot, 8
    trials; stencil sweeps (load -1): stencil_radius, round_overshoot and
    two_phase_work, 9 trials."""
    cfg, mesh, rods_o, idx_o, co = medium_oracle
    with gpu.Simulation(dict(cfg, tube_load=load), mesh=mesh) as sim:
        t = sim.autotune()
        assert t["trials"] == (9 if load < 0 else 8)
        assert 0 < t["ms_best"] <= t["ms_first"] * 1.05
        assert t["stencil_radius"] in (0, 1, 2) and t["round_overshoot"] in (0.0, 1.25, 2.0, 3.0)
        assert t["tube_load"] == load if load < 0 else t["tube_load"] in (0.0, 32.0, 48.0, 96.0, 128.0)
        sim.contacts()
        check(sim, rods_o, idx_o, co)
        # the chosen settings stay on the handle
        g = sim.generate()
        assert g["accepted"] == len(idx_o)


def test_autotune_batch_keeps_results(gpu):
    """A batch handle is tuned as one: every realisation keeps its rods and
    contacts whatever settings the tuner picks."""
    reals = gpu.configs.batched_realisations(16)
    ref, _ = gpu.batch_run(reals)
    with gpu.Batch(reals) as b:
        t = b.autotune()
        assert t["trials"] == 8 and 0 < t["ms_best"] <= t["ms_first"] * 1.05
        b.contacts()
        b.solve(check=False)
        res = b.results()
    assert [(r["accepted"], r["contacts"], r["G_eff"]) for r in res] == \
           [(r["accepted"], r["contacts"], r["G_eff"]) for r in ref]


def test_batch_run_autotune_keeps_results(gpu):
    """AUTOTUNE 1: nf_batch_run tunes its own batch first; the results are
    the untuned call's."""
    reals = gpu.configs.batched_realisations(16)
    ref, _ = gpu.batch_run(reals)
    tuned, st = gpu.batch_run([dict(p, autotune=1) for p in reals])
    assert [(r["accepted"], r["contacts"], r["G_eff"]) for r in tuned] == \
           [(r["accepted"], r["contacts"], r["G_eff"]) for r in ref]
    assert st["rods"] == sum(r["accepted"] for r in ref)


def test_tuning_parameters_validated(gpu):
    for bad in (dict(stencil_radius=3), dict(round_overshoot=-1.0), dict(autotune=2)):
        with pytest.raises(gpu.NanoFillerError) as e:
            gpu.Simulation(dict(gpu.configs.SMALL, **bad))
        assert e.value.status == 1
