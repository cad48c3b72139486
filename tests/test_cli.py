"""The command-line front end (nanofiller_gb300/_build/nanofiller): the verb
syntax of the reference binary (src/NanoFiller.cpp:37-162) over the C ABI.
Command-line checks run without a GPU; the run itself is compared, file for
file, with the same stages called through the library."""
import os
import subprocess

import numpy as np
import pytest

SMALL_KEYS = """VOLUME_PERCENT 0.5
SPAT_DISTR_FILE NONE 2 2 2 1 1 1
INC_LEN_MED 1.0
INC_RAD_MED 0.005
INC_SEPARATION 0.00034
STAT_DIST_LIM 0.0014
SELF_ALLIGN_STEP 0
DEF_THETA_DEV -1
WRT_BIN 1
SEED 0
CANDIDATES 20000
PERIODIC 3
CELL_EDGE 1.0
TUNNEL_G0 1e-5
TUNNEL_LAMBDA 0.00018
TUNNEL_DC 0.00034
"""


def cli(lib):
    from nanofiller_gb300 import build
    build.build()
    return build.CLI


def run(exe, args, cwd):
    return subprocess.run([exe] + args, cwd=cwd, capture_output=True, text=True, timeout=600)


def test_cli_usage_and_verbs_without_gpu(lib, tmp_path):
    exe = cli(lib)
    r = run(exe, [], tmp_path)
    assert r.returncode == 1 and "usage" in r.stderr
    (tmp_path / "in.txt").write_text(SMALL_KEYS)
    r = run(exe, ["in.txt", "generate", "stat_vdw"], tmp_path)
    assert r.returncode == 2 and "not part of this path" in r.stderr
    r = run(exe, ["in.txt", "generate", "stat_conduct", "3"], tmp_path)
    assert r.returncode == 1 and "direction" in r.stderr
    r = run(exe, ["in.txt", "generate", "bogus"], tmp_path)
    assert r.returncode == 1 and "unknown verb" in r.stderr
    r = run(exe, ["missing.txt", "generate", "write_vtk"], tmp_path)
    assert r.returncode == 1 and "I/O" in r.stderr
    assert not (tmp_path / "output.vtk").exists()


@pytest.mark.gpu
def test_cli_run_matches_library(gpu, tmp_path):
    exe = cli(gpu)
    a, b = tmp_path / "cli", tmp_path / "lib"
    a.mkdir()
    b.mkdir()
    (a / "in.txt").write_text(SMALL_KEYS)
    r = run(exe, ["in.txt", "generate", "write_vtk", "expand", "4", "stat_conduct", "4"], a)
    assert r.returncode == 0, r.stderr
    assert "510 inclusions generated" in r.stdout and "G_eff" in r.stdout
    # the same stages through the library
    params, _ = gpu.params_from_file(a / "in.txt")
    params["field_dir"] = 4
    with gpu.Simulation(params) as sim:
        sim.generate()
        sim.write_vtk(b / "output.vtk")
        sim.write_state(b / "output.bin")
        sim.contacts()
        sim.write_coo(b)
    for f in ("output.vtk", "output.bin", "internal.srt.coo", "sink.elec.coo", "source.elec.coo"):
        assert (a / f).read_bytes() == (b / f).read_bytes(), f
    # without `generate` the rods come back from output.bin
    os.remove(a / "output.vtk")
    r = run(exe, ["in.txt", "write_vtk"], a)
    assert r.returncode == 0, r.stderr
    assert (a / "output.vtk").read_bytes() == (b / "output.vtk").read_bytes()


@pytest.mark.gpu
def test_cli_internal_network_matches_library(gpu, tmp_path):
    exe = cli(gpu)
    a, b = tmp_path / "cli", tmp_path / "lib"
    a.mkdir()
    b.mkdir()
    (a / "in.txt").write_text(SMALL_KEYS)
    r = run(exe, ["in.txt", "generate", "stat_conduct", "4", "internal"], a)
    assert r.returncode == 0, r.stderr
    assert "rod segments" in r.stdout and "G_eff" in r.stdout
    params, _ = gpu.params_from_file(a / "in.txt")
    params["field_dir"] = 4
    with gpu.Simulation(params) as sim:
        sim.generate()
        sim.contacts()
        st = sim.internal_network()
        sim.write_internal_coo(b)
        sol = sim.solve(check=False)
    assert f"{st['nodes']} nodes ({st['contact_ends']} contact ends), {st['segments']} rod segments" in r.stdout
    assert f"G_eff = {sol['G_eff']:.9e} S" in r.stdout
    for f in ("Nodes.tbl.dat", "segment.LA.coo", "internal.DS.coo", "sink.DS.coo", "source.DS.coo"):
        assert (a / f).read_bytes() == (b / f).read_bytes(), f
    assert not (a / "internal.srt.coo").exists()
