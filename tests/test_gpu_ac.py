"""AC admittance spectrum (nf_ac_spectrum) against the oracle's restatement of
the Kirchhoff tool (refined sparse LU per frequency).

The library solves every frequency by a banded LDL^T after reverse
Cuthill-McKee (method 1, the automatic choice for these networks) or by COCG
(method 2); both are tested. Both sides report the first-order error of the
current, i_err = |V^T r|. On
the jammed box the tool's laws make the network extremely stiff: rod
segments conduct up to ~5e4 R0^-1 while the current at 10^-2 Hz is ~1e-11
R0^-1, below the rounding floor of the node potentials in FP64 for any
node-potential method (the tool's own direct solve included); there i_err
exceeds |I| on both sides. Parity is asserted where both sides resolve I
(i_err <= 1e-8 |I|), at rel 1e-6 of |I| and |Z|, and that set must contain
every frequency from 10^8 Hz up:
- the intra-rod node network and the rod-level network of the handle, the
  tool's radius convention and the rods' own radii, the tool's tunnelling
  range and one widened to 2 nm (every contact conducts);
- a synthetic ladder network handed in as host arrays (rods of 5 nodes,
  tunnelling and capacitive-only contacts, random long-range contacts that
  make its band too wide to factor, so COCG runs), resolvable over the whole
  grid (10^-2 to 10^14 Hz, step 10^0.5);
- the same network handed in as host arrays gives the same spectrum bit for
  bit (tolerance 0: same edge order, same arithmetic);
- the command-line drop-in for the tool on the files the internal mode wrote
  agrees with the oracle run on those files, and its two output files have the
  tool's layout.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC, SNK = 0xFFFFFFFF, 0xFFFFFFFE


@pytest.fixture(scope="module")
def jam(gpu):
    cfg = dict(gpu.configs.JAMMED)
    sim = gpu.Simulation(cfg)
    sim.generate()
    sim.contacts()
    out = dict(cfg=cfg, sim=sim, rods=sim.rods(), ct=sim.contact_list())
    yield out
    sim.close()


def host_net(jam, internal):
    ct, rods = jam["ct"], jam["rods"]
    a = rods["a"].astype(np.float64)
    if internal:
        net = jam["sim"].internal_net()
        return dict(n_nodes=len(net["node_rod"]), seg_i=net["seg_i"], seg_j=net["seg_j"], seg_l=net["seg_l"],
                    seg_a=a[net["node_rod"][net["seg_i"]]], ct_i=net["edge_i"], ct_j=net["edge_j"], ct_d=ct["D"],
                    ct_s=ct["S"])
    z = np.zeros(0)
    return dict(n_nodes=len(a), seg_i=z, seg_j=z, seg_l=z, seg_a=z, ct_i=ct["I"], ct_j=ct["J"], ct_d=ct["D"],
                ct_s=ct["S"])


def radii(jam):
    ct, a = jam["ct"], jam["rods"]["a"].astype(np.float64)
    rr = ct["J"] < len(a)
    return a[ct["I"]], np.where(rr, a[np.where(rr, ct["J"], 0)], 0.0)


def close(a, b, rel=1e-6, keys=("i_re", "i_im")):
    """|X_a - X_b| < rel |X_b| for the complex X given by keys."""
    xa = a[keys[0]] + 1j * a[keys[1]]
    xb = b[keys[0]] + 1j * b[keys[1]]
    err = np.abs(xa - xb) / np.abs(xb)
    assert np.all(err < rel), (err.max(), int(np.argmax(err)))


PERC = dict(delta_tun=2e-3)  # every contact of the jammed box conducts


def resolved(spec):
    return spec["i_err"] <= 1e-8 * np.abs(spec["i_re"] + 1j * spec["i_im"])


def compare(spec, ora, freq, full=False, f_min=1e8):
    ok = resolved(spec) & resolved(ora)
    assert ok[freq >= f_min].all()
    if full:
        assert ok.all()
    sub = lambda d: {k: np.asarray(d[k])[ok] for k in ("i_re", "i_im", "z_re", "z_im")}  # noqa: E731
    close(sub(spec), sub(ora))
    close(sub(spec), sub(ora), keys=("z_re", "z_im"))
    return ok


@pytest.mark.parametrize("internal,own,law", [(True, 0, "tool"), (True, 1, "tool"), (False, 0, "tool"),
                                              (True, 0, "perc")])
def test_spectrum_matches_oracle(gpu, oracle, jam, internal, own, law):
    sim = jam["sim"]
    if internal:
        sim.internal_network()
    else:
        sim.contacts()  # back to the rod-level network
    acp = dict(PERC if law == "perc" else {}, own_radii=own)
    freq = gpu.ac_frequencies(0.5)
    assert len(freq) == 33
    spec = sim.ac_spectrum(freq, check=False, **acp)
    st = spec["stats"]
    # the direct form (banded LDL^T after reverse Cuthill-McKee) converges at
    # every frequency; the flag follows the residual
    assert st["direct"] == 1 and 0 < st["bandwidth"] < 512
    assert np.array_equal(spec["converged"] == 1, spec["residual"] <= 1e-10)
    assert spec["status"] == 0, (spec["residual"], spec["iters"])
    assert st["n_active"] > 1000 and st["n_kept"] == st["n_contacts"] == len(jam["ct"]["I"])
    net = host_net(jam, internal)
    ora = oracle.ac_spectrum(net, freq, acp, radii=radii(jam) if own else None)
    assert ora["n_active"] == st["n_active"]
    assert st["R0"] == pytest.approx(ora["scales"]["R0"], rel=1e-9)
    assert st["omega0"] == pytest.approx(ora["scales"]["omega0"], rel=1e-9)
    compare(spec, ora, freq)
    # physics: |Z| falls with frequency once capacitances conduct
    assert np.abs(spec["z_re"][-1] + 1j * spec["z_im"][-1]) < np.abs(spec["z_re"][0] + 1j * spec["z_im"][0])


def ladder(seed=3, rods=400, per=5):
    """Rods of `per` nodes in a row, each tied to its predecessor by two
    tunnelling contacts, plus random tunnelling and capacitive-only contacts;
    the first rods touch the source, the last the sink (tool convention:
    D = 2 r_cnt + gap)."""
    rng = np.random.default_rng(seed)
    rc = 4.75e-3
    n = rods * per
    node = lambda r, k: r * per + k  # noqa: E731
    si = np.array([node(r, k) for r in range(rods) for k in range(per - 1)], np.uint32)
    ci, cj, gap = [], [], []
    for r in range(1, rods):
        for _ in range(2):
            ci.append(node(r, rng.integers(per))); cj.append(node(r - 1, rng.integers(per)))
            gap.append(rng.uniform(0.34e-3, 0.8e-3))
    for _ in range(3 * rods):
        r1, r2 = rng.choice(rods, 2, replace=False)
        ci.append(node(r1, rng.integers(per))); cj.append(node(r2, rng.integers(per)))
        gap.append(rng.uniform(0.34e-3, 0.8e-3) if rng.random() < 0.5 else rng.uniform(1.2e-3, 5e-3))
    for r in range(5):
        ci.append(node(r, 0)); cj.append(SRC); gap.append(rng.uniform(0.34e-3, 0.6e-3))
        ci.append(node(rods - 1 - r, per - 1)); cj.append(SNK); gap.append(rng.uniform(0.34e-3, 0.6e-3))
    m = len(ci)
    return dict(n_nodes=n, seg_i=si, seg_j=si + 1, seg_l=rng.uniform(2.0, 50.0, len(si)), seg_a=np.full(len(si), 0.005),
                ct_i=np.array(ci, np.uint32), ct_j=np.array(cj, np.uint32), ct_d=2 * rc + np.array(gap),
                ct_s=np.pi * rc * rc * rng.uniform(1.0, 10.0, m))


@pytest.mark.parametrize("method", [0, 2])
def test_ladder_network_full_grid(gpu, oracle, method):
    """Random long-range contacts make the ladder's band wide after reordering:
    the automatic choice falls back to COCG, and the direct form is refused."""
    net = ladder()
    freq = gpu.ac_frequencies(0.5)
    with gpu.Simulation(dict(gpu.configs.SMALL)) as sim:
        spec = sim.ac_spectrum(freq, net=net, method=method)
        if method == 0:
            with pytest.raises(gpu.NanoFillerError) as ei:
                sim.ac_spectrum(freq[:1], net=net, method=1)
            assert ei.value.status == 1
    st = spec["stats"]
    assert spec["status"] == 0 and st["n_active"] == net["n_nodes"]
    assert st["n_segments"] == len(net["seg_i"]) and st["direct"] == 0 and st["bandwidth"] > 512
    ora = oracle.ac_spectrum(net, freq)
    compare(spec, ora, freq, full=True)


def test_iterative_form_on_the_node_network(gpu, oracle, jam):
    """COCG (method 2, the form for bands too wide to factor) on the tool's
    node network: converged at every frequency and equal to the oracle where
    both resolve I."""
    sim = jam["sim"]
    sim.internal_network()
    freq = gpu.ac_frequencies(0.5)
    spec = sim.ac_spectrum(freq, method=2)
    assert spec["stats"]["direct"] == 0 and spec["status"] == 0
    ora = oracle.ac_spectrum(host_net(jam, True), freq)
    compare(spec, ora, freq)
    d = sim.ac_spectrum(freq, method=1)
    ok = resolved(spec) & resolved(d)
    close({k: spec[k][ok] for k in ("i_re", "i_im")}, {k: d[k][ok] for k in ("i_re", "i_im")})


def test_host_network_is_bit_identical(gpu, jam):
    sim = jam["sim"]
    sim.internal_network()
    freq = gpu.ac_frequencies(1.0)
    a = sim.ac_spectrum(freq)
    b = sim.ac_spectrum(freq, net=host_net(jam, True))
    for k in ("i_re", "i_im", "z_re", "z_im", "rms", "residual", "iters"):
        assert np.array_equal(a[k], b[k]), k
    # the handle's network is untouched: the DC solve still runs on it
    assert sim.solve()["percolating"]


def test_host_network_checks(gpu, jam):
    sim = jam["sim"]
    bad = host_net(jam, True)
    bad["seg_j"] = bad["seg_j"].copy()
    bad["seg_j"][0] = bad["n_nodes"]
    with pytest.raises(gpu.NanoFillerError) as ei:
        sim.ac_spectrum([1.0], net=bad)
    assert ei.value.status == 1 and "segment" in str(ei.value)
    with pytest.raises(gpu.NanoFillerError) as ei:
        sim.ac_spectrum([0.0])
    assert ei.value.status == 1
    with pytest.raises(gpu.NanoFillerError) as ei:
        sim.ac_spectrum([1.0], net=host_net(jam, True), own_radii=1)
    assert ei.value.status == 1


def test_tool_command_line_on_internal_files(gpu, oracle, jam, tmp_path):
    sim = jam["sim"]
    sim.contacts()
    sim.internal_network()
    sim.write_internal_coo(tmp_path)
    r = subprocess.run([sys.executable, "-m", "nanofiller_gb300.kirchhoff", "50", "2.0", "0.5", "2", "1", "--coo",
                        "--dir", str(tmp_path)], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    log = (tmp_path / "kirchhoff.1.log").read_text().splitlines()
    assert log[0] == "# Frequency\tZ_real\t(-1)Z_imag\tConverged\tRMSD\tElapsed"
    dat = np.loadtxt(tmp_path / "impedance_rRC.1.dat")
    freq = gpu.ac_frequencies(0.5, 2, 1)
    assert dat.shape == (len(freq), 4) and len(log) == len(freq) + 1
    np.testing.assert_allclose(dat[:, 0], freq, rtol=1e-15)
    assert all(ln.split("\t")[3] == "1" for ln in log[1:])
    net = oracle.read_kirchhoff_inputs(str(tmp_path), ("segment.LA.coo", "internal.DS.coo", "source.DS.coo",
                                                        "sink.DS.coo"))
    ora = oracle.ac_spectrum(net, freq, dict(l_box=2.0, delta_eff=50e-3))
    ok = resolved(ora) & (freq >= 1e6)
    assert ok.sum() >= 8
    close(dict(z_re=dat[ok, 1], z_im=dat[ok, 2]), dict(z_re=ora["z_re"][ok], z_im=ora["z_im"][ok]),
          keys=("z_re", "z_im"))
