"""Workload presets of the benchmark and parity suites (lengths in micrometres).

Each preset is a dict of nf_params field names. The five presets are the
benchmark workloads:

  small       2 um cube, periodic x/y, open z; 1 um x 5 nm rods; 0.5 % volume
              fraction (510 rods); uniform density; isotropic; Philox seed 0,
              20 000 candidates; hard-core gap 0.34 nm; tunnelling cutoff 1.4 nm.
  medium      5 um cube; 1 % (15 916 rods); density 0.01 + 8 Gaussians
              (sigma 0.5 um, centres uniform in the box) normalised to max 1 on
              a 64^3 mesh; von Mises-Fisher orientation about z, kappa = 4;
              G = G0 exp(-(gap - 0.34 nm)/lambda), G0 = 1e-5 S, lambda = 0.18 nm;
              electrodes at z = 0 and z = L.
  large       20 um cube; lognormal lengths (median 1.5 um, sigma_ln 0.3,
              clipped 0.5-3 um); radii uniform 4-8 nm; 2 % (~0.87 M rods);
              5 M candidates, seed 7.
  batched     256 realisations, seeds 0-255, box edge in 2-10 um and volume
              fraction log-uniform in 0.2-2 %, 1 um x 5 nm isotropic rods,
              each solved as in `medium`.
  adjoint     the `medium` network; gradient w.r.t. rod endpoints, lambda, G0.
  jammed      2.5 um cube filled to jamming (~4.8 %), the percolating network
              used for the solve and the adjoint (the `medium` network does not
              percolate with a 1.4 nm cutoff).
"""
import math

import numpy as np

NM = 1e-3  # micrometres per nanometre

_COMMON = dict(
    l=1.0, a=5 * NM, sep=0.34 * NM, stat_dist_lim=1.4 * NM, tol=1e-6, sc_frac=1.0,
    gen_periodic=3, field_dir=4, G0=1e-5, lambda_=0.18 * NM, d_c=0.34 * NM,
    screening=1, solve_tol=1e-10, solve_max_iter=20000, density_default=1.0,
)

SMALL = dict(_COMMON, vf=0.005, box=(2.0, 2.0, 2.0), seed=0, n_candidates=20000,
             cell_edge=1.0, orient_mode=0)

MEDIUM = dict(_COMMON, vf=0.01, box=(5.0, 5.0, 5.0), seed=0, n_candidates=8_000_000,
              orient_mode=1, vmf_kappa=4.0, mesh_ext=(64, 64, 64))

LARGE = dict(_COMMON, vf=0.02, box=(20.0, 20.0, 20.0), seed=7, n_candidates=5_000_000,
             l=1.5, len_mode=1, len_sigma_ln=0.3, len_min=0.5, len_max=3.0,
             rad_mode=2, rad_min=4 * NM, rad_max=8 * NM, a=6 * NM, orient_mode=0)

# Percolating network for the solve and the adjoint: jammed random sequential
# addition (target 5 %, the 20 M-candidate budget stops it near 4.8 %).
JAMMED = dict(_COMMON, vf=0.05, box=(2.5, 2.5, 2.5), seed=0, n_candidates=20_000_000,
              orient_mode=0)

MESH_SEED = 0x6D657368  # key of the Philox sub-stream placing the Gaussian centres


def _philox(ctr, key):
    """Philox4x32-10 block (Salmon et al. 2011) in pure Python."""
    c = list(ctr)
    k0, k1 = key
    for _ in range(10):
        p0 = 0xD2511F53 * c[0]
        p1 = 0xCD9E8D57 * c[2]
        c = [((p1 >> 32) ^ c[1] ^ k0) & 0xFFFFFFFF, p1 & 0xFFFFFFFF,
             ((p0 >> 32) ^ c[3] ^ k1) & 0xFFFFFFFF, p0 & 0xFFFFFFFF]
        k0 = (k0 + 0x9E3779B9) & 0xFFFFFFFF
        k1 = (k1 + 0xBB67AE85) & 0xFFFFFFFF
    return c


def gaussian_mesh(box=(5.0, 5.0, 5.0), ext=(64, 64, 64), n_gauss=8, sigma=0.5,
                  floor=0.01, seed=MESH_SEED):
    """Density mesh in read_density order, shape (nx, ny, nz), float32, max 1.

    Gaussians use minimum-image distances so the mesh is smooth under the
    wrap addressing of the density lookup."""
    box = np.asarray(box, np.float64)
    centres = []
    for g in range(n_gauss):
        u = _philox((g, 0, 0, 0), (seed & 0xFFFFFFFF, seed >> 32))
        centres.append([(u[d] >> 8) * 2.0 ** -24 * box[d] for d in range(3)])
    axes = [(np.arange(ext[d]) + 0.5) / ext[d] * box[d] for d in range(3)]
    X, Y, Z = np.meshgrid(*axes, indexing="ij")
    rho = np.full(X.shape, floor, np.float64)
    for c in centres:
        d2 = 0.0
        for P, cd, Ld in ((X, c[0], box[0]), (Y, c[1], box[1]), (Z, c[2], box[2])):
            d = P - cd
            d = d - Ld * np.round(d / Ld)
            d2 = d2 + d * d
        rho += np.exp(-d2 / (2 * sigma * sigma))
    rho /= rho.max()
    return np.ascontiguousarray(rho.astype(np.float32))


def batched_realisations(n=256):
    """Per-realisation params of the batched workload (deterministic spread)."""
    out = []
    for r in range(n):
        u1 = math.fmod(r * 0.6180339887498949 + 0.5, 1.0)
        u2 = math.fmod(r * 0.7548776662466927 + 0.25, 1.0)
        L = 2.0 + 8.0 * u1
        vf = 0.002 * 10.0 ** u2
        out.append(dict(_COMMON, vf=vf, box=(L, L, L), seed=r, n_candidates=4_000_000,
                        orient_mode=0))
    return out
