"""Dead-end pruning (nf_reduce, the reference's reduce verb) on the jammed
box and the medium agglomerate box:

- the surviving rods are the oracle's min-2-core of the unscreened contact
  graph (electrodes counted and kept), in their original order, every field
  bit for bit (tolerance 0), after the same number of passes;
- dangling trees and isolated rods carry no current: G_eff before and after
  pruning agree to 1e-8 relative (both solves run to a 1e-10 residual), with
  screening off so that the contact set of the surviving rods is unchanged;
- the command line's `reduce 4` writes reduced.bin byte for byte as the
  library does.
"""
import os
import subprocess

import numpy as np
import pytest

from conftest import rods_struct

pytestmark = pytest.mark.gpu

FIELDS = ("x", "y", "z", "cx", "cy", "cz", "l", "a", "stream_index")


@pytest.mark.parametrize("name", ["JAMMED", "MEDIUM"])
def test_reduce_matches_oracle(gpu, oracle, name):
    cfg = dict(getattr(gpu.configs, name))
    mesh = gpu.configs.gaussian_mesh() if name == "MEDIUM" else None
    with gpu.Simulation(cfg, mesh=mesh) as sim:
        sim.generate()
        rods0 = sim.rods()
        st = sim.reduce(2)
        rods1 = sim.rods()
        # the handle works on the reduced set afterwards
        c = sim.contacts()
    n = len(rods0["x"])
    ct = oracle.contacts(dict(cfg, screening=0), rods_struct(rods0))
    keep, rounds = oracle.prune(n, ct)
    assert st["rods_before"] == n and st["contacts"] == len(ct["I"])
    assert st["rods_after"] == int(keep.sum()) and st["rounds"] == rounds
    assert st["rods_after"] < n and (st["rods_after"] > 0 or name != "JAMMED")
    for f in FIELDS:
        assert np.array_equal(rods1[f], rods0[f][keep]), f
    assert c["contacts"] > 0


def test_reduce_keeps_conductance(gpu):
    cfg = dict(gpu.configs.JAMMED, screening=0)
    with gpu.Simulation(cfg) as sim:
        sim.generate()
        sim.contacts()
        full = sim.solve()
        st = sim.reduce(2)
        sim.contacts()
        red = sim.solve()
    assert full["percolating"] and red["percolating"]
    assert st["rods_after"] < st["rods_before"]
    assert red["G_eff"] == pytest.approx(full["G_eff"], rel=1e-8)
    assert red["n_nodes"] == st["rods_after"]


def test_reduce_state_and_limits(gpu):
    with gpu.Simulation(dict(gpu.configs.SMALL)) as sim:
        with pytest.raises(gpu.NanoFillerError):
            sim.reduce(-1)
        sim.generate()
        st = sim.reduce(0)  # nothing has fewer than 0 contacts
        assert st["rods_after"] == st["rods_before"] and st["rounds"] == 0
        with pytest.raises(gpu.NanoFillerError) as ei:
            sim.solve()  # contacts were dropped
        assert ei.value.status == 10


def test_cli_reduce_writes_reduced_bin(gpu, tmp_path):
    from test_cli import SMALL_KEYS, cli, run
    exe = cli(gpu)
    a, b = tmp_path / "cli", tmp_path / "lib"
    a.mkdir()
    b.mkdir()
    # 3 % by volume (~3 000 rods in the 2 um box), so that a network survives
    (a / "in.txt").write_text(SMALL_KEYS.replace("VOLUME_PERCENT 0.5", "VOLUME_PERCENT 3"))
    r = run(exe, ["in.txt", "generate", "expand", "4", "reduce", "4", "stat_conduct", "4"], a)
    assert r.returncode == 0, r.stderr
    assert "Inclusions remained" in r.stdout and "G_eff" in r.stdout
    params, _ = gpu.params_from_file(a / "in.txt")
    params["field_dir"] = 4
    with gpu.Simulation(params) as sim:
        sim.generate()
        sim.reduce(2)
        sim.write_state(b / "reduced.bin")
        sim.contacts()
        sim.write_coo(b)
    for f in ("reduced.bin", "internal.srt.coo", "sink.elec.coo", "source.elec.coo"):
        assert (a / f).read_bytes() == (b / f).read_bytes(), f
    assert os.path.getsize(a / "reduced.bin") < os.path.getsize(a / "output.bin")
