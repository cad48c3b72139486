"""ctypes front end of the CPU oracle (TEST INFRASTRUCTURE).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this
module. It builds oracle/_build/libnf_oracle.so on first use (g++, no GPU) and
exposes the oracle's restatement of the reference path on numpy arrays.

Parameters travel as plain dicts of nf_params field names; the ctypes mirror of
nf_params below follows include/nanofiller_gb300.h field for field.
"""
import ctypes as C
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libnf_oracle.so")
_lock = threading.Lock()
_lib = None

SRC_ELEC = 0xFFFFFFFF
SNK_ELEC = 0xFFFFFFFE


class NfParams(C.Structure):
    _fields_ = [
        ("vf", C.c_float), ("vf_precision", C.c_float), ("box", C.c_float * 3),
        ("mesh_ext", C.c_int32 * 3), ("density_file", C.c_char * 256),
        ("pref_ort", C.c_float * 2), ("theta_med", C.c_float), ("theta_dev", C.c_float),
        ("phi_med", C.c_float), ("phi_dev", C.c_float), ("l", C.c_float), ("a", C.c_float),
        ("l_dev", C.c_float), ("a_dev", C.c_float), ("sep", C.c_float), ("sc_frac", C.c_float),
        ("tol", C.c_float), ("stat_dist_lim", C.c_float), ("wrt_bin", C.c_int32),
        ("self_align_step", C.c_int32), ("clust_flag", C.c_int32), ("reduce_flag", C.c_int32),
        ("seed", C.c_uint64), ("n_candidates", C.c_uint64), ("n_target", C.c_int64),
        ("gen_periodic", C.c_int32), ("field_dir", C.c_int32), ("orient_mode", C.c_int32),
        ("vmf_kappa", C.c_float), ("len_mode", C.c_int32), ("len_sigma_ln", C.c_float),
        ("len_min", C.c_float), ("len_max", C.c_float), ("rad_mode", C.c_int32),
        ("rad_min", C.c_float), ("rad_max", C.c_float), ("density_default", C.c_float),
        ("cell_edge", C.c_float), ("G0", C.c_double), ("lambda_", C.c_double), ("d_c", C.c_double),
        ("ref_parallel_typo", C.c_int32), ("screening", C.c_int32),
        ("round_candidates", C.c_int32), ("solve_max_iter", C.c_int32), ("solve_tol", C.c_double),
        ("stencil_radius", C.c_int32), ("round_overshoot", C.c_float), ("two_phase_work", C.c_double),
        ("rod_sigma", C.c_double),
        ("elec_buffer", C.c_int32), ("ref_trunc_normal", C.c_int32),
        ("clust_dist", C.c_float), ("clust_angl", C.c_float), ("align_cell", C.c_float),
        ("align_min", C.c_int32), ("epoch_candidates", C.c_int64),
        ("solve_method", C.c_int32), ("tube_load", C.c_float), ("align_law", C.c_int32),
        ("autotune", C.c_int32),
    ]


# Reference defaults (src/simPrms.cpp:22-117) plus project defaults.
DEFAULTS = dict(
    vf=0.05 / 100.0, vf_precision=0.05, box=(0.0, 0.0, 0.0), mesh_ext=(0, 0, 0), density_file=b"",
    pref_ort=(0.0, 0.0), theta_med=0.0, theta_dev=-1.0, phi_med=0.0, phi_dev=-1.0,
    l=4.0, a=0.010, l_dev=-1.0, a_dev=-1.0, sep=0.0, sc_frac=1.0, tol=1e-6, stat_dist_lim=0.015,
    wrt_bin=0, self_align_step=0, clust_flag=0, reduce_flag=0,
    seed=0, n_candidates=1 << 20, n_target=0, gen_periodic=7, field_dir=4, orient_mode=0,
    vmf_kappa=0.0, len_mode=0, len_sigma_ln=0.0, len_min=0.0, len_max=0.0, rad_mode=0,
    rad_min=0.0, rad_max=0.0, density_default=1.0, cell_edge=0.0, G0=1e-5, lambda_=0.00018,
    d_c=0.00034, ref_parallel_typo=0, screening=1, round_candidates=0, solve_max_iter=20000,
    solve_tol=1e-10, stencil_radius=0, round_overshoot=0.0, two_phase_work=0.0, rod_sigma=67.0, elec_buffer=0,
    clust_dist=0.015, clust_angl=float(np.float32(3.14159265359) / np.float32(12)), align_cell=0.0, align_min=4,
    epoch_candidates=0, solve_method=0,
)


def make_params(d):
    p = NfParams()
    full = dict(DEFAULTS)
    full.update(d)
    for k, v in full.items():
        if k == "lambda":
            k = "lambda_"
        if isinstance(v, (tuple, list)):
            arr = getattr(p, k)
            for i, x in enumerate(v):
                arr[i] = x
        elif k == "density_file":
            setattr(p, k, v if isinstance(v, bytes) else str(v).encode())
        else:
            setattr(p, k, v)
    return p


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < max(
                    os.path.getmtime(os.path.join(HERE, f)) for f in ("nf_oracle.cpp", "nf_oracle.h")):
                build()
            L = C.CDLL(LIB_PATH)
            P = C.POINTER
            L.nfo_philox4x32_10.argtypes = [P(C.c_uint32), P(C.c_uint32), P(C.c_uint32)]
            L.nfo_sincos_turns.argtypes = [C.c_float, P(C.c_float), P(C.c_float)]
            L.nfo_logf.argtypes = [C.c_float]; L.nfo_logf.restype = C.c_float
            L.nfo_expf.argtypes = [C.c_float]; L.nfo_expf.restype = C.c_float
            for nm in ("nfo_erf", "nfo_log_d", "nfo_exp_d"):
                getattr(L, nm).argtypes = [C.c_double]
                getattr(L, nm).restype = C.c_double
            L.nfo_erfinv.argtypes = [C.c_double, C.c_double]; L.nfo_erfinv.restype = C.c_double
            L.nfo_pair_eval.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, P(C.c_double),
                                        C.c_double, C.c_double, C.c_double, C.c_int, P(C.c_double)]
            L.nfo_pair_eval.restype = C.c_int
            L.nfo_screen_eval.argtypes = [C.c_void_p, P(C.c_double), P(C.c_double), C.c_double,
                                          C.c_double, P(C.c_double), C.c_double]
            L.nfo_candidates.argtypes = [P(NfParams), C.c_void_p, C.c_int, C.c_int, C.c_int,
                                         C.c_uint64, C.c_uint64, C.c_void_p]
            L.nfo_generate.argtypes = [P(NfParams), C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int,
                                       C.c_int64, C.c_int, C.c_int64, C.c_void_p, C.c_void_p,
                                       P(C.c_uint64), C.c_void_p, C.c_int64, C.c_void_p]
            L.nfo_generate.restype = C.c_int64
            L.nfo_clust_snap.argtypes = [P(NfParams), C.c_void_p, C.c_void_p, P(C.c_float), C.c_void_p]
            L.nfo_fit_law.argtypes = [P(C.c_int64), C.c_int, P(C.c_float)]
            L.nfo_tn_cell_law.argtypes = [P(C.c_float), C.c_int64, C.c_int, P(C.c_float), P(C.c_double)]
            L.nfo_contacts.argtypes = [P(NfParams), C.c_void_p, C.c_int64, C.c_int, C.c_int,
                                       C.c_int64] + [C.c_void_p] * 8 + [P(C.c_int64)]
            L.nfo_contacts.restype = C.c_int64
            L.nfo_first_hits.argtypes = [P(NfParams), C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p,
                                         C.c_int64, C.c_int, C.c_void_p]
            L.nfo_first_hits.restype = C.c_int64
            L.nfo_internal_network.argtypes = [P(NfParams), C.c_void_p, C.c_int64, C.c_int64] + [C.c_void_p] * 4 + \
                [C.c_int64] + [C.c_void_p] * 8 + [P(C.c_int64)]
            L.nfo_internal_network.restype = C.c_int64
            L.nfo_solve.argtypes = [C.c_int64, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                                    C.c_double, C.c_int, C.c_void_p, P(C.c_double)]
            L.nfo_solve.restype = C.c_double
            L.nfo_adjoint.argtypes = [P(NfParams), C.c_void_p, C.c_int64, C.c_int64] + \
                [C.c_void_p] * 8 + [C.c_void_p, P(C.c_double), P(C.c_double)]
            _lib = L
    return _lib


ROD_DTYPE = np.dtype([(f, np.float32) for f in ("x", "y", "z", "cx", "cy", "cz", "l", "a")])


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def philox(ctr, key):
    L = lib()
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    L.nfo_philox4x32_10(c, k, o)
    return list(o)


def sincos_turns(t):
    c, s = C.c_float(), C.c_float()
    lib().nfo_sincos_turns(t, C.byref(c), C.byref(s))
    return c.value, s.value


def erf(x):
    return lib().nfo_erf(float(x))


def erfinv(y, zmax=1e300):
    return lib().nfo_erfinv(float(y), float(zmax))


def log_d(x):
    return lib().nfo_log_d(float(x))


def exp_d(x):
    return lib().nfo_exp_d(float(x))


def candidates(params, k0, n, mesh=None):
    p = make_params(params)
    out = np.zeros((n, 10), np.float32)
    nx, ny, nz = mesh.shape if mesh is not None else (0, 0, 0)
    m = None if mesh is None else np.ascontiguousarray(mesh, np.float32)
    lib().nfo_candidates(C.byref(p), _ptr(m), nx, ny, nz, k0, n, _ptr(out))
    return out


def pair_eval(A, B, shift=(0.0, 0.0, 0.0), kind=1, use_double=True, eps=1e-6, scf=1.0,
              thr_sep=0.0014, typo=False):
    a = np.array([tuple(A)], ROD_DTYPE)
    b = np.array([tuple(B)], ROD_DTYPE)
    sh = (C.c_double * 3)(*shift)
    out = (C.c_double * 6)()
    hit = lib().nfo_pair_eval(int(use_double), kind, _ptr(a), _ptr(b), sh, eps, scf, thr_sep,
                              int(typo), out)
    return bool(hit), list(out)


def first_hits(params, probes, k, rods, stream_index, nthreads=0):
    """For each probe (rod record) with stream index k: the first accepted rod
    with a smaller stream index that it hits (FP64, all images), or -1."""
    p = make_params(params)
    probes = np.ascontiguousarray(probes, ROD_DTYPE)
    rods = np.ascontiguousarray(rods, ROD_DTYPE)
    k = np.ascontiguousarray(k, np.uint64)
    si = np.ascontiguousarray(stream_index, np.uint64)
    out = np.zeros(len(probes), np.int64)
    r = lib().nfo_first_hits(C.byref(p), _ptr(probes), _ptr(k), len(probes), _ptr(rods), _ptr(si), len(rods),
                             nthreads, _ptr(out))
    if r < 0:
        raise RuntimeError("nfo_first_hits failed")
    return out


def internal_network(params, rods, ct):
    """Nodes, segments and node-level edges of the intra-rod resistor network."""
    p = make_params(params)
    rods = np.ascontiguousarray(rods, ROD_DTYPE)
    m = len(ct["I"])
    arr = [np.ascontiguousarray(ct["I"], np.uint32), np.ascontiguousarray(ct["J"], np.uint32),
           np.ascontiguousarray(ct["tI"], np.float64), np.ascontiguousarray(ct["tJ"], np.float64)]
    cap = 2 * m + 1
    out = dict(node_rod=np.zeros(cap, np.uint32), node_t=np.zeros(cap), seg_i=np.zeros(cap, np.uint32),
               seg_j=np.zeros(cap, np.uint32), seg_l=np.zeros(cap), seg_g=np.zeros(cap),
               edge_i=np.zeros(m, np.uint32), edge_j=np.zeros(m, np.uint32))
    cnt = (C.c_int64 * 3)()
    r = lib().nfo_internal_network(C.byref(p), _ptr(rods), len(rods), m, *[_ptr(a) for a in arr], cap,
                                   *[_ptr(out[k]) for k in ("node_rod", "node_t", "seg_i", "seg_j", "seg_l",
                                                            "seg_g", "edge_i", "edge_j")], cnt)
    if r < 0:
        raise RuntimeError(f"nfo_internal_network failed ({r})")
    n, ns = cnt[0], cnt[1]
    for k in ("node_rod", "node_t"):
        out[k] = out[k][:n]
    for k in ("seg_i", "seg_j", "seg_l", "seg_g"):
        out[k] = out[k][:ns]
    out["nodes_before_merge"] = cnt[2]
    return out


def _laplacian_solve(na, a, c, y, el, b, steps=6, x0=None):
    """Solve (diag(el) + Laplacian of the edges (a, c, y)) x = b by sparse LU
    with iterative refinement. The residual is formed in difference form,
    el_i x_i + sum_j y_ij (x_i - x_j), which does not cancel when strong edges
    (rod segments, 1e4-1e12 times a contact) join nearly equipotential nodes;
    plain LU loses that many digits in its pivots. With x0 the solve is for
    the deviation x = x0 - V of the solution V from x0: K x = K x0 - b, the
    right-hand side formed in difference form; x is returned (V = x0 - x).
    Returns (x, ||b - K V||)."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spl
    diag = np.array(el, dtype=np.result_type(el, y))
    np.add.at(diag, a, y)
    np.add.at(diag, c, y)
    K = sp.coo_matrix((np.concatenate([diag, -y, -y]),
                       (np.concatenate([np.arange(na), a, c]), np.concatenate([np.arange(na), c, a]))),
                      shape=(na, na)).tocsc()
    lu = spl.splu(K)

    def kmul(x):
        kx = el * x
        d = y * (x[a] - x[c])
        np.add.at(kx, a, d)
        np.add.at(kx, c, -d)
        return kx
    rhs = b if x0 is None else kmul(np.asarray(x0, diag.dtype)) - b  # K x0 - b
    x = lu.solve(rhs)
    r = rhs - kmul(x)
    for _ in range(steps):
        x = x + lu.solve(r)
        r2 = rhs - kmul(x)
        if not np.linalg.norm(r2) < np.linalg.norm(r):
            r = r2
            break
        r = r2
    _laplacian_solve.rhs_norm = float(np.linalg.norm(rhs))
    _laplacian_solve.last_r = r
    return x, float(np.linalg.norm(r))


def solve_internal(net, ct):
    """G_eff of the node network (contact edges between nodes plus rod
    segments) by a direct sparse LU factorisation in FP64, as the reference's
    Kirchhoff tool solves its network (tools/kirchhoff/kirchhoff.py:211-269,
    MKL DSS): Norton electrodes (source 1 V, sink 0 V), unknowns only in
    components that touch both electrodes; outside them a component touching
    only the source sits at 1 V, any other at 0 V.
    The LU solve is refined (_laplacian_solve).
    Returns (G_eff, node voltages, info) like solve()."""
    import scipy.sparse as sp
    import scipy.sparse.csgraph as csg
    n = len(net["node_rod"])
    I = np.concatenate([net["edge_i"], net["seg_i"]]).astype(np.int64)
    J = np.concatenate([net["edge_j"], net["seg_j"]]).astype(np.int64)
    G = np.concatenate([np.asarray(ct["G"], np.float64), net["seg_g"]])
    rr = J < SNK_ELEC
    src, snk = J == SRC_ELEC, J == SNK_ELEC
    s = np.zeros(n)
    t = np.zeros(n)
    np.add.at(s, I[src], G[src])
    np.add.at(t, I[snk], G[snk])
    A = sp.coo_matrix((np.ones(int(rr.sum())), (I[rr], J[rr])), shape=(n, n))
    ncomp, lab = csg.connected_components(A, directed=False)
    hs = np.zeros(ncomp, bool)
    ht = np.zeros(ncomp, bool)
    hs[lab[I[src]]] = True
    ht[lab[I[snk]]] = True
    act = (hs & ht)[lab]
    v = (hs & ~ht)[lab].astype(np.float64)
    na = int(act.sum())
    info = dict(iters=0, n_active=na, percolating=na > 0, residual=0.0)
    if na == 0:
        return 0.0, v, info
    idx = -np.ones(n, np.int64)
    idx[act] = np.arange(na)
    e = rr & act[I]
    b = s[act]
    x, res = _laplacian_solve(na, idx[I[e]], idx[J[e]], G[e], s[act] + t[act], b)
    info["residual"] = res / float(np.linalg.norm(b))
    v[act] = x
    return float(np.sum(b * (1.0 - x))), v, info


LAW_F = 14  # floats per law cell (kLawF)


def generate(params, mesh=None, nthreads=0, batch=4096, brute_force=False, cap=None):
    p = make_params(params)
    if cap is None:
        cap = int(params.get("n_target") or 0) or 4 * 10 ** 6
    rods = np.zeros(cap, ROD_DTYPE)
    idx = np.zeros(cap, np.uint64)
    st = (C.c_uint64 * 7)()
    nx, ny, nz = mesh.shape if mesh is not None else (0, 0, 0)
    m = None if mesh is None else np.ascontiguousarray(mesh, np.float32)
    ext = np.zeros(3, np.int32)
    lcap = LAW_F * 256 ** 3 if (p.self_align_step > 0 or p.clust_flag) else 0
    laws = np.zeros(0, np.float32)
    if lcap:
        bx = np.array(p.box[:], np.float64)
        e = p.align_cell if p.align_cell > 0 else p.l
        nc = int(np.prod(np.clip(np.floor(bx / e), 1, 256)))
        laws = np.zeros(LAW_F * nc, np.float32)
        lcap = laws.size
    n = lib().nfo_generate(C.byref(p), _ptr(m), nx, ny, nz, nthreads, batch, int(brute_force),
                           cap, _ptr(rods), _ptr(idx), st, _ptr(laws) if lcap else None, lcap, _ptr(ext))
    if n < 0:
        raise RuntimeError(f"nfo_generate failed ({n})")
    info = dict(drawn=st[0], density_accepted=st[1], exact_evals=st[2], epochs=st[3], refits=st[4],
                thinned=st[5], snapped=st[6])
    if lcap:
        info["laws"] = laws.reshape(-1, LAW_F)
        info["law_ext"] = tuple(int(v) for v in ext)
    return rods[:n].copy(), idx[:n].copy(), info


def clust_snap(params, cand, older, shift=(0.0, 0.0, 0.0)):
    """One clusterisation step; returns (moved, candidate after the step)."""
    c = np.array([tuple(cand)], ROD_DTYPE)
    o = np.array([tuple(older)], ROD_DTYPE)
    out = np.zeros(1, ROD_DTYPE)
    sh = (C.c_float * 3)(*shift)
    r = lib().nfo_clust_snap(C.byref(make_params(params)), _ptr(c), _ptr(o), sh, _ptr(out))
    return bool(r == 1), out[0]


def law_sums(dirs):
    """Tensor sums {n, xx, yy, zz, xy, xz, yz} of unit directions (float32
    rows), each product rounded to 2^-40 units as the generation does."""
    d = np.asarray(dirs, np.float32).astype(np.float64)
    pr = [d[:, 0] * d[:, 0], d[:, 1] * d[:, 1], d[:, 2] * d[:, 2], d[:, 0] * d[:, 1], d[:, 0] * d[:, 2],
          d[:, 1] * d[:, 2]]
    return [len(d)] + [int(np.rint(v * 2.0 ** 40).astype(np.int64).sum()) for v in pr]


def fit_law(sums, sample=True):
    """The law of one cell from its tensor sums: {"m": 3x3, "axis", "kappa", "flags"}."""
    s = (C.c_int64 * 7)(*sums)
    out = (C.c_float * 12)()
    if lib().nfo_fit_law(s, int(sample), out) != 0:
        raise ValueError("empty cell")
    v = np.array(out[:], np.float32)
    return dict(m=v[:9].reshape(3, 3), axis=v[[2, 5, 8]], kappa=float(v[9]), E2=float(v[10]), flags=int(v[11]))


def tn_cell_law(dirs, ref=False):
    """ALIGN_LAW 1 law of one cell from its rods' directions (n x 3):
    {"m": 3x3 rotation, "flags", "theta", "phi" (medians), "theta_scale",
    "phi_scale", "consts": tn_angle (c1, c2, zmax) for theta then phi}."""
    d = np.ascontiguousarray(dirs, np.float32).reshape(-1, 3)
    law = (C.c_float * 14)()
    lawd = (C.c_double * 10)()
    if lib().nfo_tn_cell_law(d.ctypes.data_as(C.POINTER(C.c_float)), len(d), int(ref), law, lawd) != 0:
        raise ValueError("empty cell")
    v = np.array(law[:], np.float32)
    w = np.array(lawd[:])
    return dict(m=v[:9].reshape(3, 3), flags=int(v[11]), theta=float(w[0]), theta_scale=float(w[1]),
                phi=float(w[2]), phi_scale=float(w[3]), consts=w[4:])


def contacts(params, rods, nthreads=0, brute_force=False):
    p = make_params(params)
    rods = np.ascontiguousarray(rods, ROD_DTYPE)
    cnt = (C.c_int64 * 4)()
    L = lib()
    need = L.nfo_contacts(C.byref(p), _ptr(rods), len(rods), nthreads, int(brute_force), 0,
                          *([None] * 9), cnt)
    if need < 0:
        raise RuntimeError("nfo_contacts failed")
    cap = max(int(need), 1)
    out = dict(I=np.zeros(cap, np.uint32), J=np.zeros(cap, np.uint32), tI=np.zeros(cap),
               tJ=np.zeros(cap), D=np.zeros(cap), G=np.zeros(cap), S=np.zeros(cap),
               image=np.zeros((cap, 3), np.int8))
    n = L.nfo_contacts(C.byref(p), _ptr(rods), len(rods), nthreads, int(brute_force), cap,
                       _ptr(out["I"]), _ptr(out["J"]), _ptr(out["tI"]), _ptr(out["tJ"]),
                       _ptr(out["D"]), _ptr(out["G"]), _ptr(out["S"]), _ptr(out["image"]), cnt)
    out = {k: v[:n] for k, v in out.items()}
    out["counts"] = dict(internal=cnt[0], screened=cnt[1], sink=cnt[2], source=cnt[3])
    return out


def solve(n_rods, ct, tol=1e-12, max_iter=200000):
    v = np.zeros(n_rods)
    info = (C.c_double * 4)()
    I = np.ascontiguousarray(ct["I"], np.uint32)
    J = np.ascontiguousarray(ct["J"], np.uint32)
    G = np.ascontiguousarray(ct["G"], np.float64)
    g = lib().nfo_solve(n_rods, len(I), _ptr(I), _ptr(J), _ptr(G), tol, max_iter, _ptr(v), info)
    return g, v, dict(iters=info[0], n_active=int(info[1]), percolating=bool(info[2]), residual=info[3])


def adjoint(params, rods, ct, v):
    p = make_params(params)
    rods = np.ascontiguousarray(rods, ROD_DTYPE)
    n = len(rods)
    g = np.zeros((n, 6))
    dl, dg0 = C.c_double(), C.c_double()
    arr = [np.ascontiguousarray(ct[k]) for k in ("I", "J", "tI", "tJ", "D", "G")]
    img = np.ascontiguousarray(ct["image"], np.int8)
    lib().nfo_adjoint(C.byref(p), _ptr(rods), n, len(arr[0]), *[_ptr(a) for a in arr], _ptr(img),
                      _ptr(np.ascontiguousarray(v, np.float64)), _ptr(g), C.byref(dl), C.byref(dg0))
    return g, dl.value, dg0.value


# ---------------------------------------------------------------------------
# AC admittance spectrum: the offline Kirchhoff tool's sweep
# (tools/kirchhoff/kirchhoff.py:55-286) restated in Python 3 / numpy / scipy.
# ---------------------------------------------------------------------------
AC_DEFAULTS = dict(r_cnt=4.75e-3, l_cnt=1.5, phi_ev=3.5, eps_r=2.9, delta_min=0.34e-3, delta_tun=1.1e-3,
                   delta_eff=50e-3, c_min=0.005, l_box=1.0, own_radii=0)


def ac_scales(p):
    """A, B, R0, C0, omega0, S_min, S_max of kirchhoff.py:66-88 (SI units)."""
    from scipy import constants as K
    p = dict(AC_DEFAULTS, **p)
    rc = p["r_cnt"] * 1e-6
    dmin = p["delta_min"] * 1e-6
    smin = np.pi * rc * rc
    smax = p["l_cnt"] * 1e-6 * 2 * rc
    phi = p["phi_ev"] * K.eV
    A = 1.0 / np.sqrt(2 * K.m_e * phi) * (K.h / K.e) ** 2
    B = 4 * np.pi / K.h * np.sqrt(2 * K.m_e * phi)
    R0 = A * np.exp(B * dmin) * dmin / smin
    C0 = K.epsilon_0 * p["eps_r"] * smin / dmin
    return dict(A=A, B=B, R0=R0, C0=C0, omega0=1.0 / (R0 * C0), smin=smin, smax=smax)


def ac_admittances(net, p, rod_sigma=67.0, radii=None):
    """Scaled (G, C) per contact and G per segment (kirchhoff.py:90-116,139-206).
    radii: (a_I, a_J) per contact in um for own_radii=1 (a_J = 0 at electrodes)."""
    p = dict(AC_DEFAULTS, **p)
    s = ac_scales(p)
    D = np.asarray(net["ct_d"], np.float64)
    S = np.asarray(net["ct_s"], np.float64)
    if p["own_radii"]:
        d = D * 1e-6 - (radii[0] + radii[1]) * 1e-6
    else:
        d = D * 1e-6 - 2 * p["r_cnt"] * 1e-6
    dmin = p["delta_min"] * 1e-6
    d = np.where(d > dmin, d, dmin)
    S = S * 1e-12
    S = np.where(S > s["smin"], S, s["smin"])
    S = np.where(S <= s["smax"], S, s["smax"])
    keep = d < p["delta_eff"] * 1e-6
    sr, dr = S / s["smin"], d / dmin
    tun = d <= p["delta_tun"] * 1e-6
    G = np.zeros(len(d))
    G[tun] = 1.0 / (np.exp(s["B"] * (d[tun] - dmin)) * dr[tun] / sr[tun])
    Cc = sr / dr
    Cc = np.where(Cc < p["c_min"], 0.0, Cc)
    G = np.where(keep, G, 0.0)
    Cc = np.where(keep, Cc, 0.0)
    a = np.asarray(net["seg_a"], np.float64)
    L = np.asarray(net["seg_l"], np.float64)
    Gs = rod_sigma * np.pi * a / L * s["R0"]
    return G, Cc, Gs, s


def ac_spectrum(net, freq, p=None, rod_sigma=67.0, radii=None):
    """Complex current I, impedance columns and RMS per frequency; unknowns
    are the nodes whose component (edges with G > 0 or C > 0) touches both
    electrodes, solved by sparse LU per frequency (kirchhoff.py:224-286,
    solver_type 0) with refinement (_laplacian_solve). The solve runs on
    x = chi - V, chi = 1 on the resistive clusters (G > 0 edges) tied to the
    source by a resistive contact and 0 elsewhere: where the resistive network
    does not join the electrodes, the low-frequency current is ~1e-14 of the
    electrode admittances and 1 - V near the source is below what V carries in
    FP64; x carries it. I = sum_i b_i (1 - chi_i + x_i)."""
    import scipy.sparse as sp
    import scipy.sparse.csgraph as csg
    p = dict(AC_DEFAULTS, **(p or {}))
    G, Cc, Gs, s = ac_admittances(net, p, rod_sigma, radii)
    n = int(net["n_nodes"])
    I = np.concatenate([np.asarray(net["ct_i"], np.int64), np.asarray(net["seg_i"], np.int64)])
    J = np.concatenate([np.asarray(net["ct_j"], np.int64), np.asarray(net["seg_j"], np.int64)])
    EG = np.concatenate([G, Gs])
    EC = np.concatenate([Cc, np.zeros(len(Gs))])
    on = (EG > 0) | (EC > 0)
    rr = (J < SNK_ELEC) & on
    src, snk = (J == SRC_ELEC) & on, (J == SNK_ELEC) & on
    A = sp.coo_matrix((np.ones(int(rr.sum())), (I[rr], J[rr])), shape=(n, n))
    ncomp, lab = csg.connected_components(A, directed=False)
    hs = np.zeros(ncomp, bool)
    ht = np.zeros(ncomp, bool)
    hs[lab[I[src]]] = True
    ht[lab[I[snk]]] = True
    act = (hs & ht)[lab]
    na = int(act.sum())
    idx = -np.ones(n, np.int64)
    idx[act] = np.arange(na)
    e = rr & act[I]
    a, c = idx[I[e]], idx[J[e]]
    # chi: resistive clusters with a resistive source contact
    res = rr & (EG > 0)
    Ar = sp.coo_matrix((np.ones(int(res.sum())), (I[res], J[res])), shape=(n, n))
    _, labr = csg.connected_components(Ar, directed=False)
    srcr = src & (EG > 0)
    chi_all = np.isin(labr, np.unique(labr[I[srcr]])).astype(np.float64)
    chi = chi_all[act]
    out = {k: np.zeros(len(freq)) for k in ("i_re", "i_im", "z_re", "z_im", "rms", "residual", "i_err")}
    out["converged"] = np.ones(len(freq), bool)
    out["freq"] = np.asarray(freq, np.float64)
    zs = s["R0"] * p["l_box"] * 1e-6
    for fi, f in enumerate(out["freq"]):
        w = 2 * np.pi * f / s["omega0"]
        Y = EG + 1j * w * EC
        if na == 0:
            out["z_re"][fi] = out["z_im"][fi] = np.inf
            continue
        bs = np.zeros(na, complex)
        bt = np.zeros(na, complex)
        np.add.at(bs, idx[I[src & act[I]]], Y[src & act[I]])
        np.add.at(bt, idx[I[snk & act[I]]], Y[snk & act[I]])
        x, rms = _laplacian_solve(na, a, c, Y[e], bs + bt, bs, x0=chi.astype(complex))
        cur = np.sum(bs * ((1.0 - chi) + x))  # 1 - V = 1 - chi + x
        cn = _laplacian_solve.rhs_norm
        out["residual"][fi] = rms / cn if cn > 0 else 0.0
        out["converged"][fi] = out["residual"][fi] <= 1e-9
        # first-order error of I: V^T r, V = chi - x, r the residual of x
        out["i_err"][fi] = abs(np.sum((chi - x) * _laplacian_solve.last_r))
        out["i_re"][fi], out["i_im"][fi] = cur.real, cur.imag
        out["rms"][fi] = rms
        zi = zs / cur
        out["z_re"][fi], out["z_im"][fi] = zi.real, -zi.imag
    out["n_active"] = na
    out["scales"] = s
    return out


def read_kirchhoff_inputs(directory, names=("segment.La.dat", "internal.DS.dat", "source.DS.dat", "sink.DS.dat")):
    """The tool's four input tables (kirchhoff.py:118-138): segments (I, J, L,
    a), internal contacts (I, J, D, S), source / sink contacts with the node in
    column 1. Returns a host network dict."""
    seg, internal, src, snk = (os.path.join(directory, x) for x in names)

    def table(path, cols):
        arr = np.loadtxt(path, skiprows=1, usecols=cols, ndmin=2)
        return arr.reshape(-1, len(cols))
    sg = table(seg, (0, 1, 2, 3))
    it = table(internal, (0, 1, 2, 3))
    so = table(src, (1, 2, 3))
    si = table(snk, (1, 2, 3))
    ct_i = np.concatenate([it[:, 0], so[:, 0], si[:, 0]]).astype(np.uint32)
    ct_j = np.concatenate([it[:, 1], np.full(len(so), SRC_ELEC), np.full(len(si), SNK_ELEC)]).astype(np.uint32)
    nodes = np.concatenate([sg[:, 0], sg[:, 1], it[:, 0], it[:, 1], so[:, 0], si[:, 0]])
    return dict(n_nodes=int(nodes.max()) + 1 if len(nodes) else 0,
                seg_i=sg[:, 0].astype(np.uint32), seg_j=sg[:, 1].astype(np.uint32), seg_l=sg[:, 2], seg_a=sg[:, 3],
                ct_i=ct_i, ct_j=ct_j, ct_d=np.concatenate([it[:, 2], so[:, 1], si[:, 1]]),
                ct_s=np.concatenate([it[:, 3], so[:, 2], si[:, 2]]))


def prune(n_rods, ct, min_contacts=2):
    """Dead-end pruning of the reference's reduce verb (src/NanoFiller.cpp:71-91,
    src/conductivity.cu:79-138, inc/conductKernels.h:39-162): contacts per
    rod among the rods still present (an electrode contact counts, electrodes
    stay), every rod below min_contacts removed in the same pass, passes
    repeated until one removes nothing. Returns (keep mask, passes that
    removed rods)."""
    I = np.asarray(ct["I"], np.int64)
    J = np.asarray(ct["J"], np.int64)
    alive = np.ones(n_rods, bool)
    elec = J >= SNK_ELEC
    Jr = np.where(elec, 0, J)
    rounds = 0
    while True:
        on = alive[I] & (elec | alive[Jr])
        deg = np.bincount(I[on], minlength=n_rods) + np.bincount(Jr[on & ~elec], minlength=n_rods)
        drop = alive & (deg < min_contacts)
        if not drop.any():
            return alive, rounds
        alive &= ~drop
        rounds += 1


# ---------------------------------------------------------------------------
# Statistics of the stat_* verbs (src/statistics_collection.cu), restated.
# ---------------------------------------------------------------------------
def nematic(rods, axis=(0.0, 0.0, 1.0)):
    """sum P2(c . n) / N, rods with a direction component <= -1 + 1e-6 left out
    of the sum (nematic_func, statistics_collection.cu:589-614)."""
    n = np.asarray(axis, np.float64)
    n = n / np.linalg.norm(n)
    c = np.stack([rods["cx"], rods["cy"], rods["cz"]], 1)
    lim = np.float32(-1.0) + np.float32(1e-6)
    ok = np.all(c > lim, axis=1)
    ct = c.astype(np.float64) @ n
    return float(np.sum(np.where(ok, (3 * ct * ct - 1) / 2, 0.0)) / len(ct)) if len(ct) else 0.0


def phitheta(rods, bx=32, by=32):
    """Direction histogram (bins_theta, bins_phi) (statKernel_ANGL,
    inc/statKernel_ANGL.h:57-63); phi = pi or theta = pi in the last bin."""
    cz = np.clip(np.asarray(rods["cz"], np.float64), -1, 1)
    cx = np.asarray(rods["cx"], np.float64)
    theta = np.arccos(cz)
    mid = (theta > 1e-3) & (theta < np.pi - 1e-3)
    phi = np.zeros(len(cz))
    phi[mid] = np.arccos(np.clip(cx[mid] / np.sqrt(1 - cz[mid] * cz[mid]), -1, 1))
    ip = np.clip(np.floor(phi / (np.pi / bx)).astype(np.int64), 0, bx - 1)
    it = np.clip(np.floor(theta / (np.pi / by)).astype(np.int64), 0, by - 1)
    h = np.zeros((by, bx), np.uint64)
    np.add.at(h, (it, ip), 1)
    return h


def pair_stats(params, rods, ct, bins=32):
    """Contacts per rod (rod-rod, both ends) and the mutual-angle histogram of
    the pairs with interior closest points and axis gap below stat_dist_lim
    (statKernel_CntctPerInc and statKernel_MUT_ANGLE_weightedFloat,
    inc/statKernel_MUT.h:26-131,452-512), from the oracle's unscreened
    contacts."""
    p = make_params(params)
    n = len(rods)
    I = np.asarray(ct["I"], np.int64)
    J = np.asarray(ct["J"], np.int64)
    rr = J < SNK_ELEC
    I, J = I[rr], J[rr]
    per = np.bincount(I, minlength=n) + np.bincount(J, minlength=n)
    l = rods["l"].astype(np.float64)
    a = rods["a"].astype(np.float64)
    tI, tJ, D = np.asarray(ct["tI"])[rr], np.asarray(ct["tJ"])[rr], np.asarray(ct["D"])[rr]
    interior = (np.abs(tI) < l[I] / 2) & (np.abs(tJ) < l[J] / 2)
    near = (D - a[I] - a[J]) < float(p.stat_dist_lim)
    sel = interior & near
    c = np.stack([rods["cx"], rods["cy"], rods["cz"]], 1).astype(np.float64)
    dot = np.sum(c[I[sel]] * c[J[sel]], axis=1)
    g = np.arccos(np.minimum(np.abs(dot), 1.0))
    step = ((np.pi + float(p.tol)) / 2.0) / bins
    b = np.floor(g / step).astype(np.int64) % bins
    hist = np.bincount(b, minlength=bins).astype(np.uint64)
    return dict(per_rod=per.astype(np.uint32), hist=hist, pairs=int(rr.sum()))
