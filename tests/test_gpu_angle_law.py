"""The reference's own orientation inputs on the device: DEF_THETA_MED/DEV,
DEF_PHI_MED/DEV and PREF_ORT_PHI/THETA (genCosine, sym_truncNormal and
inc_rotation, inc/cuda_CNTgenerate.h:262-295; keywords src/simPrms.cpp:264-287).
The candidate stream, the accepted set and the contact list are bit-exact
against the oracle under the exact truncated normal and under the reference's
own formula (TRUNC_NORMAL_REF 1), from parameters and from a reference-style
keyword file."""
import numpy as np
import pytest

from test_gpu_parity import assert_contacts_equal, assert_rods_equal

pytestmark = pytest.mark.gpu

LAW = dict(theta_dev=0.3, phi_dev=0.5, theta_med=0.1, phi_med=0.2, pref_ort=(0.4, 0.7))


@pytest.mark.parametrize("ref_form", [0, 1])
def test_angle_law_stream_bit_exact(gpu, oracle, ref_form):
    cfg = dict(gpu.configs.SMALL, ref_trunc_normal=ref_form, **LAW)
    sim = gpu.Simulation(cfg)
    for k0, n in ((0, 60000), (987654321, 4000)):
        g = sim.stream(k0, n)
        o = oracle.candidates(cfg, k0, n)
        assert np.array_equal(g.view(np.uint32), o.view(np.uint32)), ref_form
    # only one of the two angles on the law
    for only in (dict(phi_dev=-1.0), dict(theta_dev=-1.0)):
        c2 = dict(cfg, **only)
        s2 = gpu.Simulation(c2)
        assert np.array_equal(s2.stream(0, 20000).view(np.uint32), oracle.candidates(c2, 0, 20000).view(np.uint32))
        s2.close()
    sim.close()


@pytest.mark.parametrize("ref_form", [0, 1])
def test_angle_law_rods_and_contacts_bit_exact(gpu, oracle, ref_form):
    # an aligned law packs more rods side by side: a 2 um box at 1.5 %
    cfg = dict(gpu.configs.SMALL, vf=0.015, n_candidates=200000, ref_trunc_normal=ref_form, **LAW)
    with gpu.Simulation(cfg) as sim:
        g = sim.generate()
        sim.contacts()
        rods = sim.rods()
        ct = sim.contact_list()
    rods_o, idx_o, st = oracle.generate(cfg, batch=4096)
    assert_rods_equal(rods, rods_o, idx_o)
    assert g["candidates_drawn"] == st["drawn"]
    co = oracle.contacts(cfg, rods_o)
    assert len(co["I"]) > 0
    assert_contacts_equal(ct, co)


def test_reference_keyword_file_runs_the_law(gpu, oracle, tmp_path):
    """A reference-style input (angles in degrees) no longer stops with
    NF_ERR_UNSUPPORTED: the parsed law drives the device and the oracle alike."""
    text = """VOLUME_PERCENT 1.5
SPAT_DISTR_FILE NONE 2 2 2 1 1 1
INC_LEN_MED 1.0
INC_RAD_MED 0.005
INC_SEPARATION 0.00034
STAT_DIST_LIM 0.0014
PREF_ORT_PHI 20
PREF_ORT_THETA 40
DEF_THETA_MED 5
DEF_THETA_DEV 17
DEF_PHI_MED 10
DEF_PHI_DEV 29
SEED 11
CANDIDATES 150000
PERIODIC 3
"""
    (tmp_path / "in.txt").write_text(text)
    params, _ = gpu.params_from_file(tmp_path / "in.txt")
    assert params["theta_dev"] > 0 and params["phi_dev"] > 0 and params["pref_ort"][1] > 0
    with gpu.Simulation(params) as sim:
        sim.generate()
        rods = sim.rods()
    rods_o, idx_o, _ = oracle.generate(params, batch=4096)
    assert_rods_equal(rods, rods_o, idx_o)
    # the law is not isotropic: the order tensor has a clear leading eigenvalue
    d = np.stack([rods["cx"], rods["cy"], rods["cz"]], 1).astype(np.float64)
    Q = d.T @ d / len(d)
    assert np.linalg.eigvalsh(Q)[-1] > 0.6


def test_angle_law_exclusive_with_vmf(gpu):
    cfg = dict(gpu.configs.SMALL, theta_dev=0.3, orient_mode=1, vmf_kappa=4.0)
    with pytest.raises(gpu.NanoFillerError):
        gpu.Simulation(cfg)
