"""Adaptive generation on the device against the oracle, bit for bit
(tolerance 0: the same FP32 stream, exact integer tensor sums, the same FP64
fits, FP32 snaps with every operation rounded on its own):

- self-alignment + thin-out + clusterisation under a von Mises-Fisher law:
  every rod field and stream index, the epoch / refit / thin-out / snap
  counts and the final per-cell laws (axis, kappa) equal the oracle's;
- the same with small rounds (round_candidates 300): rounds never cross an
  epoch boundary, so the result does not depend on them;
- an isotropic law with thin-out (the fitted laws act only through the
  thin-out) and a dense box with clusterisation alone;
- a batch with adaptive realisations is refused (NF_ERR_UNSUPPORTED) and a
  plain handle has no laws to read (NF_ERR_STATE);
- the medium agglomerate box (density mesh, von Mises-Fisher) with all
  three steps, bit for bit;
- ALIGN_LAW 1, the reference's truncated-normal cell laws and Gaussian
  thin-out with DEF_THETA_* / DEF_PHI_* set, bit for bit in both draw forms;
- the command line reads SELF_ALLIGN_STEP, REDUCE_FLAG, CLUST_FLAG,
  CLUST_ANGL_LIM and the project keys and writes the library's output.bin
  byte for byte.
"""
import numpy as np
import pytest

from conftest import rods_struct

pytestmark = pytest.mark.gpu

NM = 1e-3
FIELDS = ("x", "y", "z", "cx", "cy", "cz", "l", "a", "stream_index")

ADAPT = dict(vf=0.03, box=(2.0, 2.0, 2.0), l=1.0, a=5 * NM, sep=0.34 * NM, stat_dist_lim=1.4 * NM, tol=1e-6,
             sc_frac=1.0, gen_periodic=3, field_dir=4, seed=3, n_candidates=30000, orient_mode=1, vmf_kappa=2.0,
             self_align_step=1, reduce_flag=1, clust_flag=1, epoch_candidates=2000, align_cell=1.0,
             density_default=1.0)


def run_both(gpu, oracle, cfg):
    with gpu.Simulation(cfg) as sim:
        g = sim.generate()
        rods = sim.rods()
        laws = sim.orientation_laws()
    ro, io, so = oracle.generate(cfg)
    return g, rods, laws, ro, io, so


def check_equal(g, rods, laws, ro, io, so):
    n = len(ro)
    assert g["accepted"] == n
    rs = rods_struct(rods)
    for f in ("x", "y", "z", "cx", "cy", "cz", "l", "a"):
        assert np.array_equal(rs[f], ro[f]), f
    assert np.array_equal(rods["stream_index"], io)
    for k, ko in (("candidates_drawn", "drawn"), ("density_accepted", "density_accepted"), ("epochs", "epochs"),
                  ("refits", "refits"), ("thinned", "thinned"), ("snapped", "snapped")):
        assert g[k] == so[ko], k
    assert laws["ext"] == so["law_ext"]
    assert np.array_equal(laws["axis"], so["laws"][:, [2, 5, 8]])
    assert np.array_equal(laws["kappa"], so["laws"][:, 9])


def test_adaptive_vmf_matches_oracle(gpu, oracle):
    out = run_both(gpu, oracle, ADAPT)
    check_equal(*out)
    g = out[0]
    assert g["refits"] > 0 and g["thinned"] > 0 and g["snapped"] > 0
    assert np.any(out[2]["kappa"] != np.float32(2.0))  # refit laws differ from the global one


def test_adaptive_round_size_independent(gpu, oracle):
    with gpu.Simulation(ADAPT) as a, gpu.Simulation(dict(ADAPT, round_candidates=300)) as b:
        ga, gb = a.generate(), b.generate()
        ra, rb = a.rods(), b.rods()
    assert gb["rounds"] > ga["rounds"]
    for f in FIELDS:
        assert np.array_equal(ra[f], rb[f]), f
    for k in ("epochs", "refits", "thinned", "snapped", "candidates_drawn"):
        assert ga[k] == gb[k], k


def test_isotropic_thinout_matches_oracle(gpu, oracle):
    cfg = dict(ADAPT, orient_mode=0, clust_flag=0, vf=0.02, seed=5)
    out = run_both(gpu, oracle, cfg)
    check_equal(*out)
    assert out[0]["thinned"] > 0 and out[0]["snapped"] == 0


def test_reference_cell_law_matches_oracle(gpu, oracle):
    """ALIGN_LAW 1 (the reference's truncated-normal cell laws, its
    Gaussian-likelihood thin-out) with DEF_THETA_* / DEF_PHI_* set, refits,
    thin-out and clusterisation: bit for bit, both forms of the draw."""
    base = dict(ADAPT, orient_mode=0, vmf_kappa=0.0, theta_med=0.5, theta_dev=0.3, phi_med=0.8, phi_dev=0.4,
                align_law=1, seed=11)
    for ref in (0, 1):
        out = run_both(gpu, oracle, dict(base, ref_trunc_normal=ref))
        check_equal(*out)
        g, so = out[0], out[5]
        assert g["refits"] > 0 and g["thinned"] > 0 and g["snapped"] > 0
        assert any(int(f) & 4 for f in so["laws"][:, 11])  # cells drew from their own laws
    with pytest.raises(gpu.NanoFillerError) as ei:  # the von Mises-Fisher refit does not take these laws
        gpu.Simulation(dict(base, align_law=0))
    assert ei.value.status == 11


def test_dense_clusterisation_matches_oracle(gpu, oracle):
    cfg = dict(ADAPT, box=(2.5, 2.5, 2.5), vf=0.04, self_align_step=0, reduce_flag=0, orient_mode=0,
               n_candidates=120000, epoch_candidates=10000, seed=11, clust_angl=0.5, clust_dist=0.02)
    out = run_both(gpu, oracle, cfg)
    check_equal(*out)
    assert out[0]["snapped"] > 100 and out[0]["refits"] == 0


def test_adaptive_limits(gpu):
    with pytest.raises(gpu.NanoFillerError) as ei:
        gpu.batch_run([dict(ADAPT)])
    assert ei.value.status == 11
    with gpu.Simulation(dict(gpu.configs.SMALL)) as sim:
        sim.generate()
        with pytest.raises(gpu.NanoFillerError) as ei:
            sim.orientation_laws()
        assert ei.value.status == 10
    with pytest.raises(gpu.NanoFillerError):
        gpu.Simulation(dict(ADAPT, box=(0.8, 2.0, 2.0)))  # clusterisation needs edges >= the rod length


def test_cli_adaptive_keywords(gpu, tmp_path):
    """The reference's keywords drive the adaptive generation of the command
    line, which writes the library's output.bin byte for byte."""
    from test_cli import SMALL_KEYS, cli, run
    exe = cli(gpu)
    keys = SMALL_KEYS.replace("VOLUME_PERCENT 0.5", "VOLUME_PERCENT 3").replace(
        "SELF_ALLIGN_STEP 0", "SELF_ALLIGN_STEP 1\nREDUCE_FLAG 1\nCLUST_FLAG 1\nCLUST_ANGL_LIM 0.5\n"
        "ORIENT VMF\nVMF_KAPPA 2\nEPOCH_CANDIDATES 2000\nALIGN_CELL 1.0")
    a, b = tmp_path / "cli", tmp_path / "lib"
    a.mkdir()
    b.mkdir()
    (a / "in.txt").write_text(keys)
    r = run(exe, ["in.txt", "generate"], a)
    assert r.returncode == 0, r.stderr
    params, unknown = gpu.params_from_file(a / "in.txt")
    assert unknown == 0 and params["self_align_step"] == 1 and params["clust_flag"] == 1
    assert params["clust_angl"] == pytest.approx(0.5) and params["epoch_candidates"] == 2000
    with gpu.Simulation(params) as sim:
        g = sim.generate()
        sim.write_state(b / "output.bin")
    assert g["refits"] > 0 and g["snapped"] > 0
    assert (a / "output.bin").read_bytes() == (b / "output.bin").read_bytes()


def test_adaptive_with_density_mesh(gpu, oracle):
    """The medium agglomerate box (8-Gaussian density, von Mises-Fisher kappa
    4 about z) with all three steps: the per-cell laws and the density draw
    act together; equal to the oracle bit for bit."""
    cfg = dict(gpu.configs.MEDIUM, self_align_step=2, reduce_flag=1, clust_flag=1, epoch_candidates=50000,
               n_candidates=400000)
    mesh = gpu.configs.gaussian_mesh()
    with gpu.Simulation(cfg, mesh=mesh) as sim:
        g = sim.generate()
        rods = sim.rods()
        laws = sim.orientation_laws()
    ro, io, so = oracle.generate(cfg, mesh=mesh)
    check_equal(g, rods, laws, ro, io, so)
    assert g["refits"] > 0 and g["thinned"] > 0 and g["snapped"] > 0
