"""The reference's truncated-normal angle law (DEF_THETA_MED/DEV, DEF_PHI_MED/DEV;
genCosine and sym_truncNormal, inc/cuda_CNTgenerate.h:262-275) in the oracle:
its FP64 erf / erfinv against scipy, the exact truncated normal and the
reference's own form against their distributions, and the keyword file."""
import math

import numpy as np
import pytest
from scipy import special, stats


def test_erf_matches_scipy(oracle):
    xs = np.concatenate([np.linspace(-6, 6, 4001), [1e-300, 1e-12, 1e-4, 1.9999999, 2.0, 2.0000001]])
    for x in xs:
        ref = special.erf(x)
        got = oracle.erf(x)
        assert abs(got - ref) <= 2e-15 * max(abs(ref), 1e-300), (x, got, ref)
    # erfc form above 2 keeps relative accuracy of 1 - erf in the tail
    for x in np.linspace(2.0, 5.9, 200):
        assert abs((1.0 - oracle.erf(x)) - special.erfc(x)) <= 1e-13 * special.erfc(x) + 2e-16


def test_erfinv_matches_scipy_within_float_ulp(oracle):
    rng = np.random.default_rng(5)
    ys = np.concatenate([rng.uniform(-1, 1, 20000), 1 - 10.0 ** rng.uniform(-16, -1, 2000),
                         -(1 - 10.0 ** rng.uniform(-16, -1, 2000)), 10.0 ** rng.uniform(-300, -3, 500),
                         [0.0, 1e-3, -1e-3, 0.5, 1 - 2.0 ** -24]])
    worst = 0.0
    for y in ys:
        ref = special.erfinv(y)
        got = oracle.erfinv(y)
        if ref == 0.0:
            assert got == 0.0
            continue
        worst = max(worst, abs(got - ref) / abs(ref))
        # the float the generator keeps is within 1 ulp of the correctly rounded
        # one (CUDA documents 2 ulp for erfinvf)
        assert abs(int(np.float32(got).view(np.int32)) - int(np.float32(ref).view(np.int32))) <= 1, y
    assert worst < 5e-14, worst
    # |y| >= 1 and the cap
    assert oracle.erfinv(1.0, 3.5) == 3.5 and oracle.erfinv(-1.0, 3.5) == -3.5
    assert oracle.erfinv(0.9999, 1.0) == 1.0


def test_log_exp_double(oracle):
    for x in np.concatenate([10.0 ** np.linspace(-300, 300, 601), np.linspace(0.5, 2, 301)]):
        assert abs(oracle.log_d(x) - math.log(x)) <= 4e-16 * max(abs(math.log(x)), 1e-300) + 1e-300
    for x in np.linspace(-40, 40, 801):
        assert abs(oracle.exp_d(x) - math.exp(x)) <= 4e-16 * math.exp(x)


def _angles(oracle, params, n=200000):
    c = oracle.candidates(params, 0, n).astype(np.float64)
    return c[:, 3], c[:, 4], c[:, 5]


def test_theta_law_is_the_truncated_normal(oracle, cfg):
    s = 0.6
    p = dict(cfg.SMALL, theta_dev=s, theta_med=0.0)
    cx, cy, cz = _angles(oracle, p)
    theta = np.arccos(np.clip(cz, -1, 1))  # |theta| for theta in (-pi/2, pi/2)
    assert cz.min() >= 0.0  # truncated to +-pi/2 about the axis
    half = stats.truncnorm(-(np.pi / 2) / s, (np.pi / 2) / s, loc=0, scale=s)
    d, pv = stats.kstest(theta, lambda t: 2 * half.cdf(t) - 1)
    assert pv > 1e-3, (d, pv)
    # phi stays uniform while DEF_PHI_DEV is off
    phi = np.arctan2(cy, cx)
    d, pv = stats.kstest(phi, stats.uniform(-np.pi, 2 * np.pi).cdf)
    assert pv > 1e-3, (d, pv)


def test_phi_law_is_the_truncated_normal(oracle, cfg):
    s, med = 0.9, 0.4
    p = dict(cfg.SMALL, phi_dev=s, phi_med=med)
    cx, cy, cz = _angles(oracle, p)
    phi = np.arctan2(cy, cx)
    # truncated to med +- pi: fold the draws back onto [med - pi, med + pi)
    phi = np.where(phi < med - np.pi, phi + 2 * np.pi, phi)
    law = stats.truncnorm(-np.pi / s, np.pi / s, loc=med, scale=s)
    d, pv = stats.kstest(phi, law.cdf)
    assert pv > 1e-3, (d, pv)
    # cos theta stays uniform
    d, pv = stats.kstest(cz, stats.uniform(-1, 2).cdf)
    assert pv > 1e-3, (d, pv)


def test_reference_form_switch(oracle, cfg):
    """TRUNC_NORMAL_REF 1: theta = 2 s sqrt2 erfinv(Fa (1 - 2u)), Fa = erf(-w/s/sqrt2)/2:
    the law of 2 s sqrt2 erfinv(V), V uniform on +-erf(z)/2 (not a normal)."""
    s = 0.3
    p = dict(cfg.SMALL, theta_dev=s, ref_trunc_normal=1)
    cx, cy, cz = _angles(oracle, p)
    theta = np.arccos(np.clip(cz, -1, 1))
    E = special.erf((np.pi / 2) / s / np.sqrt(2))

    def cdf_abs(t):  # P(|T| <= t), T = 2 s sqrt2 erfinv(V)
        return np.clip(special.erf(t / (2 * s * np.sqrt(2))) / (E / 2), 0, 1)

    d, pv = stats.kstest(theta, cdf_abs)
    assert pv > 1e-3, (d, pv)
    # the reference's form is narrower than its nominal support: |T| < 2 s sqrt2 erfinv(E/2)
    assert theta.max() <= 2 * s * np.sqrt(2) * special.erfinv(E / 2) * (1 + 1e-6)
    # and differs from the exact law
    q = dict(p, ref_trunc_normal=0)
    assert not np.array_equal(_angles(oracle, q)[2], cz)


def test_rotation_to_the_preferred_axis(oracle, cfg):
    """inc_rotation (inc/cuda_CNTgenerate.h:289-295) with Mu = PREF_ORT_PHI,
    Xi = -PREF_ORT_THETA takes the law's axis z to (sin th cos ph, sin th sin ph,
    cos th) up to the reference's sign convention: the mean axis of a narrow law."""
    th, ph = 0.7, 0.3
    p = dict(cfg.SMALL, theta_dev=0.05, pref_ort=(ph, th))
    cx, cy, cz = _angles(oracle, p, n=20000)
    m = np.array([cx.mean(), cy.mean(), cz.mean()])
    m /= np.linalg.norm(m)
    # the image of z under the reference's matrix: (-sin Xi cos Mu, sin Xi sin Mu, cos Xi)
    Xi, Mu = -th, ph
    axis = np.array([-np.sin(Xi) * np.cos(Mu), np.sin(Xi) * np.sin(Mu), np.cos(Xi)])
    assert np.dot(m, axis) > 0.998
