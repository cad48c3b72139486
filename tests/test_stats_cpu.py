"""Statistics of the stat_* verbs without a GPU: the oracle on rods with known
directions, and the rho.dat / gamma.dat writers (host-only library code)
against text built from the reference's writers (write_Mathematica2Di and
write_mat, src/IO.cpp): "rho = {" rows of setw(12) integers, and
"gamma={<tab>" values of setw(10) setprecision(7)."""
import numpy as np
import pytest


def rods_with(oracle, dirs):
    r = np.zeros(len(dirs), oracle.ROD_DTYPE)
    d = np.asarray(dirs, np.float64)
    d /= np.linalg.norm(d, axis=1)[:, None]
    r["cx"], r["cy"], r["cz"] = d[:, 0], d[:, 1], d[:, 2]
    r["l"], r["a"] = 1.0, 0.005
    return r


def test_nematic_known_values(oracle):
    assert oracle.nematic(rods_with(oracle, [(0, 0, 1)] * 3)) == pytest.approx(1.0)
    assert oracle.nematic(rods_with(oracle, [(1, 0, 0), (0, 1, 0)])) == pytest.approx(-0.5)
    # a rod along -x (component -1) is left out of the sum, not of the count
    assert oracle.nematic(rods_with(oracle, [(0, 0, 1), (-1, 0, 0)])) == pytest.approx(0.5)


def test_phitheta_bins(oracle):
    h = oracle.phitheta(rods_with(oracle, [(0, 0, 1), (1, 0, 0), (0, 1, 0), (0, 0, -1)]), 4, 4)
    assert h.sum() == 4
    assert h[0, 0] == 1        # theta = 0 (phi set to 0)
    assert h[2, 0] == 1        # theta = pi/2, phi = 0
    assert h[2, 2] == 1        # theta = pi/2, phi = pi/2
    assert h[3, 0] == 1        # theta = pi in the last theta bin


def fmt_g(v, prec):
    """C++ ostream default (general) formatting at the given precision."""
    s = "%.*g" % (prec, v)
    if "e" in s:
        m, e = s.split("e")
        s = "%se%s%02d" % (m, e[0], int(e[1:]))
    return s


def test_rho_and_gamma_writers(lib, tmp_path):
    h = np.array([[1, 2, 3], [40, 50, 600]], np.uint64)  # 2 theta rows x 3 phi bins
    lib.write_rho(tmp_path / "rho.dat", h)
    rows = ["\t{" + ",".join("%12d" % v for v in row) + "}" for row in h]
    assert (tmp_path / "rho.dat").read_text() == "rho = {" + ",\n\t".join(rows) + "}"
    g = np.array([0, 7, 12345678], np.uint64)
    lib.write_gamma(tmp_path / "gamma.dat", g)
    body = "".join("%10s,\n" % fmt_g(float(v), 7) for v in g[:-1]) + "%10s\t}\n" % fmt_g(float(g[-1]), 7)
    assert (tmp_path / "gamma.dat").read_text() == "gamma={\t" + body
