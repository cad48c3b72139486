"""AC admittance model of the Kirchhoff tool (tools/kirchhoff/kirchhoff.py):
the oracle's admittance laws at known points, its spectrum on networks with a
closed-form answer, and the library's frequency grid (host code only, no GPU).
"""
import numpy as np
import pytest

SRC, SNK = 0xFFFFFFFF, 0xFFFFFFFE
RC = 4.75e-3  # um, the tool's R_cnt
DMIN = 0.34e-3


def one(oracle, D, S):
    net = dict(n_nodes=1, seg_i=[], seg_j=[], seg_l=[], seg_a=[], ct_i=[0], ct_j=[SRC], ct_d=[D], ct_s=[S])
    G, C, _, s = oracle.ac_admittances(net, {})
    return G[0], C[0], s


def test_admittance_known_points(oracle):
    smin = np.pi * RC * RC  # um^2
    # gap = delta_min and S = S_min: one resistance and one capacitance unit
    G, C, s = one(oracle, 2 * RC + DMIN, smin)
    assert G == pytest.approx(1.0, rel=1e-12) and C == pytest.approx(1.0, rel=1e-12)
    # a touching pair (gap below the floor) counts as gap = delta_min; S above
    # S_max = 2 R_cnt L_cnt is clamped to it
    G2, C2, _ = one(oracle, 2 * RC, 1.0)
    smax = 2 * RC * 1.5
    assert G2 == pytest.approx(smax / smin, rel=1e-12) and C2 == pytest.approx(smax / smin, rel=1e-12)
    # at the tunnelling range: exp(-B (d - d_min)) d_min / d; beyond it only C
    d = 1.1e-3
    G3, C3, _ = one(oracle, 2 * RC + d, smin)
    assert G3 == pytest.approx(np.exp(-s["B"] * (d - DMIN) * 1e-6) * DMIN / d, rel=1e-9)
    assert C3 == pytest.approx(DMIN / d, rel=1e-12)
    G4, C4, _ = one(oracle, 2 * RC + 1.2e-3, smin)
    assert G4 == 0.0 and C4 == pytest.approx(DMIN / 1.2e-3, rel=1e-12)
    # capacitance below c_min (0.005) is 0; beyond delta_eff (50 nm) the contact is dropped
    G5, C5, _ = one(oracle, 2 * RC + 0.07, smin)
    assert G5 == 0.0 and C5 == 0.0
    G6, C6, _ = one(oracle, 2 * RC + 0.049, smin)
    assert G6 == 0.0 and C6 == pytest.approx(DMIN / 0.049, rel=1e-12)


def test_series_chain_closed_form(oracle):
    # source -> node 0 -segment- node 1 -> sink: I = 1 / (1/Ys + 1/Yseg + 1/Yk)
    smin = np.pi * RC * RC
    net = dict(n_nodes=2, seg_i=[0], seg_j=[1], seg_l=[40.0], seg_a=[0.005],
               ct_i=[0, 1], ct_j=[SRC, SNK], ct_d=[2 * RC + 0.5e-3, 2 * RC + 0.9e-3], ct_s=[smin, 2 * smin])
    G, C, Gs, s = oracle.ac_admittances(net, {})
    assert Gs[0] == pytest.approx(67.0 * np.pi * 0.005 / 40.0 * s["R0"], rel=1e-14)
    freq = np.array([1e-2, 1e6, 1e11, 1e12, 1e13])
    out = oracle.ac_spectrum(net, freq)
    assert out["n_active"] == 2
    for k, f in enumerate(freq):
        w = 2 * np.pi * f / s["omega0"]
        Ys, Yk = G[0] + 1j * w * C[0], G[1] + 1j * w * C[1]
        I = 1.0 / (1.0 / Ys + 1.0 / Gs[0] + 1.0 / Yk)
        assert out["i_re"][k] + 1j * out["i_im"][k] == pytest.approx(I, rel=1e-10)
        z = s["R0"] * 1e-6 / I
        assert out["z_re"][k] == pytest.approx(z.real, rel=1e-10)
        assert out["z_im"][k] == pytest.approx(-z.imag, rel=1e-10)


def test_capacitive_path_and_floating_parts(oracle):
    # source and sink joined only through a capacitive gap (2 nm): I = i w C (series
    # with the two electrode contacts); node 2 floats and node 3 touches only the
    # source, neither enters the solve
    smin = np.pi * RC * RC
    net = dict(n_nodes=4, seg_i=[], seg_j=[], seg_l=[], seg_a=[],
               ct_i=[0, 0, 1, 3, 2], ct_j=[SRC, 1, SNK, SRC, 3],
               ct_d=[2 * RC, 2 * RC + 2e-3, 2 * RC, 2 * RC, 2 * RC + 0.1], ct_s=[smin, smin, smin, smin, smin])
    G, C, _, s = oracle.ac_admittances(net, {})
    assert G[1] == 0.0 and C[1] > 0 and G[4] == 0.0 and C[4] == 0.0
    out = oracle.ac_spectrum(net, [1e9, 1e12])
    assert out["n_active"] == 2
    for k, f in enumerate([1e9, 1e12]):
        w = 2 * np.pi * f / s["omega0"]
        I = 1.0 / (1.0 / (G[0] + 1j * w * C[0]) + 1.0 / (1j * w * C[1]) + 1.0 / (G[2] + 1j * w * C[2]))
        assert out["i_re"][k] + 1j * out["i_im"][k] == pytest.approx(I, rel=1e-10)


def tool_grid(log_df, n_patch, patch_id):
    """kirchhoff.py:72-79,176 written out."""
    nf = int((14 - (-2)) / log_df) + 1
    patch = int(np.ceil(nf * 1.0 / n_patch))
    lo = -2 + patch_id * patch * log_df
    return np.array([10 ** (log_df * x + lo) for x in np.arange(patch)])


@pytest.mark.parametrize("log_df,n_patch,patch_id", [(0.1, 1, 0), (0.25, 1, 0), (0.1, 4, 3), (0.5, 3, 1)])
def test_frequency_grid(lib, log_df, n_patch, patch_id):
    f = lib.ac_frequencies(log_df, n_patch, patch_id)
    np.testing.assert_allclose(f, tool_grid(log_df, n_patch, patch_id), rtol=1e-15)


def test_ac_params_defaults(lib):
    p = lib.ac_params()
    assert (p.r_cnt, p.l_cnt, p.phi_ev, p.eps_r) == (4.75e-3, 1.5, 3.5, 2.9)
    assert (p.delta_min, p.delta_tun, p.c_min, p.tol) == (0.34e-3, 1.1e-3, 0.005, 1e-10)
    with pytest.raises(KeyError):
        lib.ac_params(bogus=1)
