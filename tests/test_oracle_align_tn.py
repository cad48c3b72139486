"""The reference's cell law of self-alignment in the oracle (ALIGN_LAW 1;
crossMtxBuild / resetOrt / resetAvgVec, inc/allignment_fit.h:154-458, and
randomThinOut / check_probability, :466-578):

- the preferred axis is numpy's eigenvector of <c c^T> of the largest
  eigenvalue for rods about one direction (two small eigenvalues within
  10 %), of the smallest for rods in a plane (disk-like); the rotation is
  inc_rotation(phi_o, -theta_o) of its angles;
- the medians are the box-frame angles (asin |a_xy|, acos(a_x / |a_xy|)) of
  the unit mean direction and the scales the mean squared deviations of the
  rods' own angles from them (numpy, 1e-12);
- a cell whose mean direction is short (norm per rod <= 0.5: isotropic, or
  the two senses of one axis) keeps its truncated-normal laws (flag bit 2
  clear) while its rotation is refitted;
- the constants are tn_angle's for those scales (exact truncated normal, or
  the reference's form);
- a generation with refits and thin-out under this law runs, refits and
  thins, and does not depend on the batch size.
"""
import math

import numpy as np
import pytest

from oracle import nf_oracle as O

NM = 1e-3


def angles(d):
    nxy = np.hypot(d[:, 0], d[:, 1])
    th = np.arcsin(np.minimum(nxy, 1.0))
    ph = np.where(nxy > 1e-6, np.arccos(np.clip(d[:, 0] / np.where(nxy > 0, nxy, 1), -1, 1)), 0.0)
    return th, ph


def about(axis, n, spread, seed):
    rng = np.random.default_rng(seed)
    a = np.asarray(axis, np.float64)
    a /= np.linalg.norm(a)
    d = a + spread * rng.standard_normal((n, 3))
    return (d / np.linalg.norm(d, axis=1)[:, None]).astype(np.float32)


def check_medians(d, law):
    x = d.astype(np.float64)
    a = x.sum(axis=0)
    a /= np.linalg.norm(a)
    th, ph = angles(a[None, :])
    t, p = angles(x)
    assert law["theta"] == pytest.approx(float(np.float32(th[0])), abs=1e-7)
    assert law["phi"] == pytest.approx(float(np.float32(ph[0])), abs=1e-7)
    assert law["theta_scale"] == pytest.approx(float(np.float32(np.mean((t - th[0]) ** 2))), rel=1e-6)
    assert law["phi_scale"] == pytest.approx(float(np.float32(np.mean((p - ph[0]) ** 2))), rel=1e-6)


def rotation(phi_o, theta_o):
    cm, sm = math.cos(phi_o), math.sin(phi_o)
    cx, sx = math.cos(-theta_o), math.sin(-theta_o)
    return np.array([[cm * cx, sm, -sx * cm], [-sm * cx, cm, sx * sm], [sx, 0.0, cx]])


def test_prolate_cell_takes_the_largest_eigenvector():
    d = about((0.3, 0.2, 0.93), 400, 0.05, 1)
    law = O.tn_cell_law(d)
    assert law["flags"] == 6  # rotate, own truncated-normal laws
    w, v = np.linalg.eigh((d.astype(np.float64).T @ d.astype(np.float64)) / len(d))
    ax = v[:, np.argmax(w)] * np.sign(v[2, np.argmax(w)])
    th_o = math.acos(ax[2])
    ph_o = math.acos(ax[0] / math.sin(th_o))
    assert np.allclose(law["m"], rotation(ph_o, th_o), atol=2e-6)
    check_medians(d, law)


def test_disk_cell_takes_the_smallest_eigenvector():
    rng = np.random.default_rng(2)
    phi = rng.uniform(0.2, 1.2, 300)  # rods in the xy plane, one sense
    d = np.stack([np.cos(phi), np.sin(phi), 0.01 * rng.standard_normal(300)], 1)
    d = (d / np.linalg.norm(d, axis=1)[:, None]).astype(np.float32)
    law = O.tn_cell_law(d)
    w, v = np.linalg.eigh((d.astype(np.float64).T @ d.astype(np.float64)) / len(d))
    assert abs((w[1] - w[0]) / w[1]) >= 0.1  # not uniaxial about the largest
    ax = v[:, np.argmin(w)] * np.sign(v[2, np.argmin(w)])
    th_o = math.acos(ax[2]) if abs(ax[2]) <= 1 - 1e-6 else 0.0
    assert th_o < 0.05
    assert law["flags"] == 6
    check_medians(d, law)


def test_short_mean_keeps_the_truncated_normal_laws():
    rng = np.random.default_rng(3)
    iso = rng.standard_normal((600, 3))
    iso = (iso / np.linalg.norm(iso, axis=1)[:, None]).astype(np.float32)
    assert O.tn_cell_law(iso)["flags"] == 2
    d = about((0.0, 0.0, 1.0), 200, 0.05, 4)
    both = np.concatenate([d, -d])  # one axis, both senses: the mean cancels
    law = O.tn_cell_law(both)
    assert law["flags"] == 2 and law["theta_scale"] == 0.0


@pytest.mark.parametrize("ref", [False, True])
def test_constants_are_tn_angle_constants(ref):
    sp = pytest.importorskip("scipy.special")
    d = about((0.5, -0.1, 0.86), 300, 0.1, 5)
    law = O.tn_cell_law(d, ref=ref)
    for s, w, (c1, c2, z) in ((law["theta_scale"], math.pi / 2, law["consts"][:3]),
                              (law["phi_scale"], math.pi, law["consts"][3:])):
        zz = w / s / math.sqrt(2.0)
        if ref:
            assert c1 == pytest.approx(0.5 * sp.erf(zz), rel=1e-12)
            assert c2 == pytest.approx(2 * s * math.sqrt(2.0), rel=1e-12)
        else:
            assert c1 == pytest.approx(sp.erf(zz), rel=1e-12)
            assert c2 == pytest.approx(s * math.sqrt(2.0), rel=1e-12)
            assert z == pytest.approx(zz, rel=1e-12)


def test_generation_with_reference_law_refits_and_thins():
    cfg = dict(O.DEFAULTS, vf=0.03, box=(2.0, 2.0, 2.0), l=1.0, a=5 * NM, sep=0.34 * NM, stat_dist_lim=1.4 * NM,
               gen_periodic=3, seed=11, n_candidates=20000, theta_med=0.5, theta_dev=0.3, phi_med=0.8,
               phi_dev=0.4, self_align_step=1, reduce_flag=1, epoch_candidates=2000, align_cell=1.0,
               align_law=1)
    r1, i1, s1 = O.generate(cfg, batch=512)
    r2, i2, s2 = O.generate(cfg, batch=4096)
    assert s1["refits"] > 0 and s1["thinned"] > 0
    assert np.array_equal(i1, i2) and np.array_equal(r1, r2)
    assert any(int(f) & 4 for f in s1["laws"][:, 11])  # some cell drew from its own law
