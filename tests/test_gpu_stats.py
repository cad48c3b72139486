"""Statistics of the stat_* verbs on the device against the oracle, on the
jammed and medium (von Mises-Fisher kappa = 4 about z) boxes:

- nematic order within 1e-12 (FP64 sums in different orders); the aligned
  box S > 0.3 (S = 0.44 for kappa = 4), the dilute isotropic box |S| < 0.06
  (four standard deviations for 510 rods; the jammed box is not isotropic:
  sequential addition at 5 % in a box open along z prefers z, S ~ 0.1);
- the direction histogram and the mutual-angle histogram equal bit for bit
  (tolerance 0: integer counts from the same FP64 bin arithmetic), contacts
  per rod equal for every rod;
- on a handle whose contacts are screened, the pair statistics run on an
  unscreened sweep and drop the handle's contacts;
- the command line's stat_* and write_* verbs write the same files as the
  library, byte for byte.
"""
import numpy as np
import pytest

from conftest import rods_struct

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["JAMMED", "MEDIUM"])
def test_stats_match_oracle(gpu, oracle, name):
    cfg = dict(getattr(gpu.configs, name))
    mesh = gpu.configs.gaussian_mesh() if name == "MEDIUM" else None
    with gpu.Simulation(cfg, mesh=mesh) as sim:
        sim.generate()
        rods = sim.rods()
        S = sim.nematic()
        Sx = sim.nematic((1.0, 0.0, 0.0))
        h = sim.phitheta()
        ps = sim.pair_stats()
    rs = rods_struct(rods)
    n = len(rs)
    assert S == pytest.approx(oracle.nematic(rs), abs=1e-12)
    assert Sx == pytest.approx(oracle.nematic(rs, (1, 0, 0)), abs=1e-12)
    if name == "MEDIUM":
        assert S > 0.3
    assert np.array_equal(h, oracle.phitheta(rs)) and int(h.sum()) == n
    ct = oracle.contacts(dict(cfg, screening=0), rs)
    po = oracle.pair_stats(cfg, rs, ct)
    assert np.array_equal(ps["per_rod"], po["per_rod"])
    assert np.array_equal(ps["hist"], po["hist"])
    assert ps["pairs"] == po["pairs"] and ps["contacts_total"] == 2 * po["pairs"]
    assert ps["max_per_rod"] == po["per_rod"].max() and ps["rods"] == n
    assert ps["mean_per_rod"] == pytest.approx(2 * po["pairs"] / n)
    assert 0 < ps["angle_pairs"] <= ps["pairs"]


def test_dilute_isotropic_nematic(gpu):
    with gpu.Simulation(dict(gpu.configs.SMALL)) as sim:
        sim.generate()
        assert abs(sim.nematic()) < 0.06


def test_pair_stats_replace_screened_contacts(gpu):
    cfg = dict(gpu.configs.JAMMED)
    assert cfg["screening"]
    with gpu.Simulation(cfg) as sim:
        sim.generate()
        c = sim.contacts()  # screening on: the handle's list is a screened one
        ps = sim.pair_stats()
        assert ps["pairs"] >= c["contacts"] - c["n_source"] - c["n_sink"]
        with pytest.raises(gpu.NanoFillerError) as ei:
            sim.solve()
        assert ei.value.status == 10
    cfg0 = dict(cfg, screening=0)
    with gpu.Simulation(cfg0) as sim:
        sim.generate()
        sim.contacts()
        sim.pair_stats()
        assert sim.solve()["percolating"]  # unscreened contacts are the handle's own: kept


def test_cli_stats_verbs(gpu, tmp_path):
    from test_cli import SMALL_KEYS, cli, run
    exe = cli(gpu)
    a, b = tmp_path / "cli", tmp_path / "lib"
    a.mkdir()
    b.mkdir()
    keys = SMALL_KEYS.replace("VOLUME_PERCENT 0.5", "VOLUME_PERCENT 3")
    (a / "in.txt").write_text(keys)
    r = run(exe, ["in.txt", "generate", "stat_nematic", "stat_phitheta", "stat_mutangle", "stat_contacts",
                  "write_ort", "write_lmp"], a)
    assert r.returncode == 0, r.stderr
    params, _ = gpu.params_from_file(a / "in.txt")
    with gpu.Simulation(params) as sim:
        sim.generate()
        S = sim.nematic()
        gpu.write_rho(b / "rho.dat", sim.phitheta())
        ps = sim.pair_stats()
        gpu.write_gamma(b / "gamma.dat", ps["hist"])
        sim.write_ort(b / "orient.vtk")
        sim.write_lmp(b / "output.lmp.data")
    assert "Estimated nematic order parameter: %f" % S in r.stdout
    assert "Maximum number of contacts per inclusion: %d" % ps["max_per_rod"] in r.stdout
    for f in ("rho.dat", "gamma.dat", "orient.vtk", "output.lmp.data"):
        assert (a / f).read_bytes() == (b / f).read_bytes(), f
    lmp = (a / "output.lmp.data").read_text().splitlines()
    assert lmp[2] == "%d atoms" % ps["rods"] and lmp[4] == "%d ellipsoids" % ps["rods"]
