"""Adaptive generation in the oracle (self-alignment, thin-out,
clusterisation; src/cudaMain.cu:112-132,254-273,354-396,
inc/allignment_fit.h, inc/cuda_Clusterize.h):

- the law fit: the axis equals numpy's principal eigenvector of the same
  tensor (to 1e-6), the concentration solves E[(c.mu)^2] = 1 - 2 coth(k)/k +
  2/k^2 for the largest eigenvalue (scipy brentq, rel 1e-9), a von
  Mises-Fisher sample of kappa = 5 drawn by the candidate stream fits back to
  kappa 5 +- 5 % about its axis, an isotropic sample to kappa < 1, and rods
  all along one direction to the cap 500;
- the snap of cuda_Clusterize2Old against a closed form: a candidate 12 nm
  above an older rod and 5 degrees off its axis ends parallel to it, a + a' +
  sep above its axis, with its own foot kept in place along the axis; no move
  past the angle limit, past the distance limit, with centres farther than
  half the longer length, or when the axes meet;
- the generation does not depend on the batch size, the thread count or the
  neighbour search (cells or brute force), refits, thins and snaps;
- with an isotropic law, refits alone change nothing: the rods equal the
  plain generation's;
- REDUCE_FLAG without refits thins nothing, one epoch longer than the budget
  has no boundary, and a rod minimum no cell reaches keeps every law global.
"""
import math

import numpy as np
import pytest

from oracle import nf_oracle as O

NM = 1e-3


def unit(v):
    v = np.asarray(v, np.float64)
    return v / np.linalg.norm(v)


def stream_dirs(n, **kw):
    p = dict(O.DEFAULTS, box=(5.0, 5.0, 5.0), l=1.0, a=0.005, **kw)
    c = O.candidates(p, 0, n)
    return c[:, 3:6].astype(np.float32)


def vmf_m2(k):
    return 1.0 / 3.0 + 2 * k * k / 45 if k < 1e-3 else 1 - 2 / (k * math.tanh(k)) + 2 / (k * k)


def test_fit_axis_and_kappa_match_numpy_and_moment_equation():
    sp = pytest.importorskip("scipy.optimize")
    d = stream_dirs(20000, orient_mode=1, vmf_kappa=5.0, pref_ort=(0.3, 0.7))
    law = O.fit_law(O.law_sums(d))
    T = (d.astype(np.float64).T @ d.astype(np.float64)) / len(d)
    w, V = np.linalg.eigh(T)
    mu = V[:, -1] * np.sign(V[2, -1])
    assert np.allclose(law["axis"], mu, atol=1e-6)
    k = sp.brentq(lambda x: vmf_m2(x) - w[-1], 1e-6, 499.0, xtol=1e-14)
    assert law["kappa"] == pytest.approx(k, rel=1e-6)
    assert law["kappa"] == pytest.approx(5.0, rel=0.05)
    m = law["m"].astype(np.float64)
    assert np.allclose(m.T @ m, np.eye(3), atol=1e-6)  # a rotation taking z to the axis
    assert np.allclose(m @ [0, 0, 1], law["axis"], atol=1e-7)
    assert law["flags"] == 3 and law["E2"] == pytest.approx(math.exp(-2 * law["kappa"]), rel=1e-6)
    assert O.fit_law(O.law_sums(d), sample=False)["flags"] == 0  # fitted for the thin-out only


def test_fit_isotropic_and_aligned_limits():
    iso = O.fit_law(O.law_sums(stream_dirs(20000)))
    assert iso["kappa"] < 1.0
    u = unit([0.2, -0.5, 0.8]).astype(np.float32)
    al = O.fit_law(O.law_sums(np.tile(u, (50, 1))))
    assert al["kappa"] == 500.0 and np.allclose(al["axis"], u, atol=1e-6)
    flipped = O.fit_law(O.law_sums(np.tile(-u, (50, 1))))  # axes are unsigned
    assert np.array_equal(flipped["axis"], al["axis"])


ROD = lambda x, y, z, c, l=1.0, a=5 * NM: (x, y, z, *unit(c), l, a)


def snap_params(**kw):
    return dict(O.DEFAULTS, box=(4.0, 4.0, 4.0), l=1.0, a=5 * NM, sep=0.34 * NM, **kw)


def test_snap_closed_form():
    p = snap_params()
    th = math.radians(5.0)
    older = ROD(1.0, 1.0, 1.0, (1, 0, 0))
    cand = ROD(1.1, 1.0, 1.0 + 12 * NM, (math.cos(th), math.sin(th), 0))
    moved, out = O.clust_snap(p, cand, older)
    assert moved
    # common perpendicular along z: the candidate's foot on its axis is t0
    # from its centre, on the older rod's axis at x = 1.1 - t0 cos th... the
    # feet solve (c - r) = t1 c2 - t0 c1 + dz e_z
    c1 = np.array([math.cos(th), math.sin(th), 0.0])
    r1 = np.array(cand[:3], np.float64)
    r2 = np.array(older[:3], np.float64)
    A = np.stack([c1, -np.array([1.0, 0, 0])], 1)[:2]
    t0, t1 = np.linalg.solve(A, (r2 - r1)[:2])
    sd = 5 * NM + 5 * NM + 0.34 * NM
    want = r2 + np.array([1.0, 0, 0]) * t1 + np.array([0, 0, 1.0]) * sd - np.array([1.0, 0, 0]) * (math.cos(th) * t0)
    got = np.array([out["x"], out["y"], out["z"]], np.float64)
    assert np.allclose(got, want, atol=2e-6)
    assert (out["cx"], out["cy"], out["cz"]) == (np.float32(1.0), np.float32(0.0), np.float32(0.0))
    assert out["z"] - 1.0 == pytest.approx(sd, abs=1e-6)


def test_snap_limits():
    p = snap_params()
    older = ROD(1.0, 1.0, 1.0, (1, 0, 0))
    th = math.radians(20.0)  # beyond pi/12
    assert not O.clust_snap(p, ROD(1.1, 1.0, 1.012, (math.cos(th), math.sin(th), 0)), older)[0]
    th = math.radians(5.0)
    assert not O.clust_snap(p, ROD(1.1, 1.0, 1.0 + 16 * NM, (math.cos(th), math.sin(th), 0)), older)[0]
    assert not O.clust_snap(p, ROD(1.6, 1.0, 1.012, (math.cos(th), math.sin(th), 0)), older)[0]  # centres 0.6 apart
    assert O.clust_snap(dict(p, clust_angl=math.radians(25.0)),
                        ROD(1.1, 1.0, 1.012, (math.cos(math.radians(20)), math.sin(math.radians(20)), 0)), older)[0]
    # axes that meet: no direction to move along
    assert not O.clust_snap(p, ROD(1.1, 1.0, 1.0, (math.cos(th), math.sin(th), 0)), older)[0]
    # through a periodic image
    moved, out = O.clust_snap(p, ROD(0.05, 1.0, 1.012, (math.cos(th), math.sin(th), 0)),
                              ROD(3.95, 1.0, 1.0, (1, 0, 0)), shift=(-4.0, 0.0, 0.0))
    assert moved and out["cx"] == 1.0


ADAPT = dict(O.DEFAULTS, vf=0.03, box=(2.0, 2.0, 2.0), l=1.0, a=5 * NM, sep=0.34 * NM, stat_dist_lim=1.4 * NM,
             gen_periodic=3, field_dir=4, seed=3, n_candidates=30000, orient_mode=1, vmf_kappa=2.0,
             self_align_step=1, reduce_flag=1, clust_flag=1, epoch_candidates=2000, align_cell=1.0)


def test_adaptive_generation_is_batch_and_search_independent():
    ref, ri, st = O.generate(ADAPT, nthreads=1, batch=1)
    assert st["refits"] > 0 and st["thinned"] > 0 and st["snapped"] > 0
    assert st["epochs"] == -(-st["drawn"] // 2000) or st["epochs"] == st["drawn"] // 2000 + 1
    for kw in (dict(nthreads=0, batch=4096), dict(nthreads=3, batch=777), dict(nthreads=0, batch=512, brute_force=True)):
        r, i, s = O.generate(ADAPT, **kw)
        assert np.array_equal(r, ref) and np.array_equal(i, ri), kw
        for k in ("drawn", "density_accepted", "epochs", "refits", "thinned", "snapped"):
            assert s[k] == st[k], (kw, k)
        assert np.array_equal(s["laws"], st["laws"])
    assert np.all(np.diff(ri.astype(np.int64)) > 0)  # stream order kept through the thin-outs


def test_isotropic_refits_alone_change_nothing():
    base = dict(ADAPT, orient_mode=0, reduce_flag=0, clust_flag=0, self_align_step=0)
    r0, i0, s0 = O.generate(base)
    r1, i1, s1 = O.generate(dict(base, self_align_step=1))
    assert s1["refits"] > 0 and s1["thinned"] == 0
    assert np.array_equal(r0, r1) and np.array_equal(i0, i1)
    assert np.any(s1["laws"][:, 9] > 0)  # fitted, for the thin-out only
    assert np.all(s1["laws"][:, 11] == 0)


def test_adaptive_edge_rules():
    base = dict(ADAPT, clust_flag=0)
    plain = dict(base, self_align_step=0, reduce_flag=0)
    r0, i0, _ = O.generate(plain)
    # thin-out only follows a refit (src/cudaMain.cu:128-131): REDUCE_FLAG alone changes nothing
    r1, i1, s1 = O.generate(dict(base, self_align_step=0, reduce_flag=1))
    assert np.array_equal(r0, r1) and np.array_equal(i0, i1) and s1["refits"] == 0 and s1["thinned"] == 0
    # one epoch longer than the budget: no boundary, no refit
    r2, i2, s2 = O.generate(dict(base, epoch_candidates=10 ** 9))
    assert s2["epochs"] == 1 and s2["refits"] == 0 and np.array_equal(r0, r2)
    # a cell needs ALIGN_MIN_RODS rods for a refit: with an impossible minimum every law stays global
    _, _, s3 = O.generate(dict(base, align_min=10 ** 6))
    assert s3["refits"] > 0 and np.all(s3["laws"][:, 9] == np.float32(2.0))
