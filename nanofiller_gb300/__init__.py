"""GB300-native NanoFiller hot path: Python front end of the C ABI.

    import nanofiller_gb300 as nf
    sim = nf.Simulation(nf.configs.SMALL)
    sim.generate(); sim.contacts(); sim.solve()

Parameters are dicts of nf_params field names (lengths in micrometres); any
field not given keeps the library default (nf_params_default). The library is
the CUDA build in nanofiller_gb300/_build/; there is no CPU path.
"""
import ctypes as C

import numpy as np

from . import configs  # noqa: F401
from ._abi import (LIB_PATH, SNK_ELEC, SRC_ELEC, STATUS, NfBatchResult, NfBatchStats,  # noqa: F401
                   NfContactList, NfContactStats, NfGenStats, NfParams, NfRods, NfSolveStats,
                   NfInternalNet, NfInternalStats, NfStateHeader, NfTuneResult, NfAcNet, NfAcParams,
                   NfAcPoint, NfAcStats, NfPairStats, NfReduceStats, load)

__all__ = ["Simulation", "NanoFillerError", "make_params", "params_from_file", "batch_run",
           "target_count", "kernel_launches", "allocations", "configs", "Batch", "SRC_ELEC", "SNK_ELEC", "ac_params", "ac_frequencies",
           "write_impedance", "write_kirchhoff_log"]


def kernel_launches():
    """Kernel launches issued by the library in this process."""
    return int(load().nf_kernel_launches())


def allocations():
    """Device and pinned host blocks the library requested in this process."""
    return int(load().nf_allocations())


class NanoFillerError(RuntimeError):
    def __init__(self, status, msg=""):
        self.status = status
        super().__init__(f"{STATUS.get(status, status)}: {msg}")


def _check(st, h=None, what=""):
    if st != 0:
        msg = what
        if h:
            buf = C.create_string_buffer(512)
            load().nf_last_error(h, buf, 512)
            if buf.value:
                msg = f"{what}: {buf.value.decode()}"
        raise NanoFillerError(st, msg)


def make_params(d=None, **kw):
    p = NfParams()
    _check(load().nf_params_default(C.byref(p)))
    full = dict(d or {})
    full.update(kw)
    for k, v in full.items():
        if k == "lambda":
            k = "lambda_"
        if isinstance(v, (tuple, list)):
            arr = getattr(p, k)
            for i, x in enumerate(v):
                arr[i] = x
        elif k == "density_file":
            p.density_file = v if isinstance(v, bytes) else str(v).encode()
        else:
            setattr(p, k, v)
    return p


def params_to_dict(p):
    out = {}
    for name, _ in NfParams._fields_:
        v = getattr(p, name)
        if hasattr(v, "__len__") and not isinstance(v, (bytes, str)):
            v = tuple(v)
        out[name] = v
    return out


def params_from_file(path, base=None):
    p = make_params(base)
    unk = C.c_int(0)
    _check(load().nf_params_from_file(str(path).encode(), C.byref(p), C.byref(unk)), what=str(path))
    return params_to_dict(p), unk.value


def target_count(params):
    n = C.c_int64()
    _check(load().nf_target_count(C.byref(make_params(params)), C.byref(n)))
    return n.value


def _f32p(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class Simulation:
    """One realisation on the current CUDA device (a C-ABI handle)."""

    def __init__(self, params, mesh=None, stream=None):
        self._L = load()
        self._nv = None  # voltage count of the last solve
        self.params = make_params(params)
        h = C.c_void_p()
        _check(self._L.nf_create(C.byref(self.params), C.byref(h)), what="nf_create")
        self._h = h
        if stream is not None:
            _check(self._L.nf_set_stream(h, C.c_void_p(stream)), h)
        if mesh is not None:
            self.load_density(mesh)

    def close(self):
        if getattr(self, "_h", None):
            self._L.nf_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # inputs
    def load_density(self, mesh):
        m = np.ascontiguousarray(mesh, np.float32)
        nx, ny, nz = m.shape
        _check(self._L.nf_load_density(self._h, nx, ny, nz, m.ctypes.data_as(C.c_void_p)), self._h)

    # stages
    def generate(self):
        s = NfGenStats()
        _check(self._L.nf_generate(self._h, C.byref(s)), self._h, "nf_generate")
        return {k: getattr(s, k) for k, _ in s._fields_}

    def contacts(self):
        s = NfContactStats()
        _check(self._L.nf_contacts(self._h, C.byref(s)), self._h, "nf_contacts")
        return {k: getattr(s, k) for k, _ in s._fields_}

    def solve(self, check=True):
        s = NfSolveStats()
        st = self._L.nf_solve(self._h, C.byref(s))
        if check:
            _check(st, self._h, "nf_solve")
        out = {k: getattr(s, k) for k, _ in s._fields_}
        out["status"] = st
        self._nv = int(s.n_nodes) if st == 0 else None
        return out

    def adjoint(self):
        n = self.n_rods()
        g = np.zeros((n, 6), np.float32)
        dl, dg0 = C.c_double(), C.c_double()
        _check(self._L.nf_adjoint(self._h, g.ctypes.data_as(C.c_void_p), n, C.byref(dl), C.byref(dg0)),
               self._h, "nf_adjoint")
        return g, dl.value, dg0.value

    # outputs
    def n_rods(self):
        r = NfRods()
        r.capacity = 0
        st = self._L.nf_get_rods(self._h, C.byref(r))
        if st not in (0, 5):
            _check(st, self._h, "nf_get_rods")
        return int(r.count)

    def rods(self):
        n = self.n_rods()
        # every element is written by nf_get_rods
        out = {f: np.empty(n, np.float32) for f in ("x", "y", "z", "cx", "cy", "cz", "l", "a")}
        out["stream_index"] = np.empty(n, np.uint64)
        out["cell"] = np.empty(n, np.uint32)
        r = NfRods()
        r.capacity = n
        for f in ("x", "y", "z", "cx", "cy", "cz", "l", "a"):
            setattr(r, f, _f32p(out[f]))
        r.stream_index = out["stream_index"].ctypes.data_as(C.POINTER(C.c_uint64))
        r.cell = out["cell"].ctypes.data_as(C.POINTER(C.c_uint32))
        _check(self._L.nf_get_rods(self._h, C.byref(r)), self._h, "nf_get_rods")
        return out

    def set_rods(self, rods):
        n = len(rods["x"])
        arrs = {f: np.ascontiguousarray(rods[f], np.float32) for f in ("x", "y", "z", "cx", "cy", "cz", "l", "a")}
        r = NfRods()
        r.capacity = n
        r.count = n
        for f, a in arrs.items():
            setattr(r, f, _f32p(a))
        si = None
        if rods.get("stream_index") is not None:
            si = np.ascontiguousarray(rods["stream_index"], np.uint64)
            r.stream_index = si.ctypes.data_as(C.POINTER(C.c_uint64))
        _check(self._L.nf_set_rods(self._h, C.byref(r)), self._h, "nf_set_rods")

    def contact_list(self):
        c = NfContactList()
        c.capacity = 0
        st = self._L.nf_get_contacts(self._h, C.byref(c))
        if st not in (0, 5):
            _check(st, self._h, "nf_get_contacts")
        n = int(c.count)
        # every element is written by nf_get_contacts
        out = dict(I=np.empty(n, np.uint32), J=np.empty(n, np.uint32), tI=np.empty(n, np.float32),
                   tJ=np.empty(n, np.float32), D=np.empty(n), G=np.empty(n), S=np.empty(n),
                   image=np.empty((n, 3), np.int8))
        c.capacity = n
        c.I = out["I"].ctypes.data_as(C.POINTER(C.c_uint32))
        c.J = out["J"].ctypes.data_as(C.POINTER(C.c_uint32))
        c.tI = _f32p(out["tI"])
        c.tJ = _f32p(out["tJ"])
        for f in ("D", "G", "S"):
            setattr(c, f, out[f].ctypes.data_as(C.POINTER(C.c_double)))
        c.image = out["image"].ctypes.data_as(C.POINTER(C.c_int8))
        _check(self._L.nf_get_contacts(self._h, C.byref(c)), self._h, "nf_get_contacts")
        return out

    def voltages(self):
        """Voltages of the last solve: one per rod, or one per node of the
        internal network when that was solved."""
        n = self._nv if self._nv is not None else self.n_rods()
        v = np.zeros(n)
        _check(self._L.nf_get_voltages(self._h, v.ctypes.data_as(C.c_void_p), n), self._h, "nf_get_voltages")
        return v

    def stream(self, k0, n):
        out = np.zeros((10, n), np.float32)
        ptrs = [out[i].ctypes.data_as(C.c_void_p) for i in range(10)]
        _check(self._L.nf_stream_candidates(self._h, k0, n, *ptrs), self._h, "nf_stream_candidates")
        return out.T.copy()

    def internal_network(self):
        """Build the intra-rod resistor network from the current contacts
        (nf_internal_network); nf_solve then solves it."""
        st = NfInternalStats()
        _check(self._L.nf_internal_network(self._h, C.byref(st)), self._h, "nf_internal_network")
        return {k: getattr(st, k) for k, _ in st._fields_}

    def internal_net(self):
        """Nodes, segments and contact-end nodes of the internal network."""
        q = NfInternalNet()
        _check(self._L.nf_get_internal_network(self._h, C.byref(q)), self._h, "nf_get_internal_network")
        nn, ns, ne = q.n_nodes, q.n_segments, q.n_edges
        out = dict(node_rod=np.zeros(nn, np.uint32), node_t=np.zeros(nn), seg_i=np.zeros(ns, np.uint32),
                   seg_j=np.zeros(ns, np.uint32), seg_l=np.zeros(ns), seg_g=np.zeros(ns),
                   edge_i=np.zeros(ne, np.uint32), edge_j=np.zeros(ne, np.uint32))
        q.capacity = max(nn, ns, ne, 1)
        for k, a in out.items():
            setattr(q, k, a.ctypes.data_as(C.c_void_p))
        _check(self._L.nf_get_internal_network(self._h, C.byref(q)), self._h, "nf_get_internal_network")
        return out

    def write_internal_coo(self, path):
        _check(self._L.nf_write_internal_coo(self._h, str(path).encode()), self._h, "nf_write_internal_coo")

    def autotune(self):
        """Pick the speed-only settings by timing generations (nf_autotune):
        tube_load and round_overshoot on the tube grid, stencil_radius,
        round_overshoot and two_phase_work on the stencil sweeps; the handle
        (every realisation of a batch) keeps the fastest settings."""
        r = NfTuneResult()
        _check(self._L.nf_autotune(self._h, C.byref(r)), self._h, "nf_autotune")
        return {k: getattr(r, k) for k, _ in r._fields_}

    def stream_noalloc(self, k0, n):
        """Same rows as stream(k0, n) through nf_stream_candidates_noalloc,
        which stages in a fixed device array (n <= 65536) and allocates no
        device memory."""
        out = np.zeros((10, n), np.float32)
        ptrs = [out[i].ctypes.data_as(C.c_void_p) for i in range(10)]
        _check(self._L.nf_stream_candidates_noalloc(self._h, k0, n, *ptrs), self._h,
               "nf_stream_candidates_noalloc")
        return out.T.copy()

    def set_orientation(self, mode, kappa=1.0, pref_phi=0.0, pref_theta=0.0):
        """Orientation law of the candidates drawn from now on (nf_set_orientation):
        mode 0 isotropic, 1 von Mises-Fisher with concentration kappa about the
        axis (pref_phi, pref_theta)."""
        _check(self._L.nf_set_orientation(self._h, mode, kappa, pref_phi, pref_theta), self._h,
               "nf_set_orientation")

    def orientation_laws(self):
        """Per-cell orientation laws of the adaptive generation after
        generate() (nf_orientation_laws): {"ext": (nx, ny, nz), "axis": (cells, 3),
        "kappa": (cells,)}, cell = i + nx (j + ny k)."""
        ext = np.zeros(3, np.int32)
        n = C.c_size_t()
        _check(self._L.nf_orientation_laws(self._h, 0, ext.ctypes.data_as(C.c_void_p), None, None, C.byref(n)),
               self._h, "nf_orientation_laws")
        axis = np.zeros((n.value, 3), np.float32)
        kappa = np.zeros(n.value, np.float32)
        _check(self._L.nf_orientation_laws(self._h, n.value, ext.ctypes.data_as(C.c_void_p),
                                           axis.ctypes.data_as(C.c_void_p), kappa.ctypes.data_as(C.c_void_p),
                                           C.byref(n)), self._h, "nf_orientation_laws")
        return {"ext": tuple(int(v) for v in ext), "axis": axis, "kappa": kappa}

    def reduce(self, min_contacts=2):
        """Dead-end pruning (nf_reduce): keep the rods with at least
        min_contacts unscreened contacts, repeatedly; electrodes stay."""
        st = NfReduceStats()
        _check(self._L.nf_reduce(self._h, min_contacts, C.byref(st)), self._h, "nf_reduce")
        return {k: getattr(st, k) for k, _ in st._fields_}

    # statistics (the reference's stat_* verbs)
    def nematic(self, axis=(0.0, 0.0, 1.0)):
        """Nematic order parameter S = <P2(c . axis)> (nf_stat_nematic)."""
        ax = np.ascontiguousarray(axis, np.float64)
        S = C.c_double()
        _check(self._L.nf_stat_nematic(self._h, ax.ctypes.data_as(C.c_void_p), C.byref(S)), self._h,
               "nf_stat_nematic")
        return S.value

    def phitheta(self, bins_phi=32, bins_theta=32):
        """Histogram of rod directions, shape (bins_theta, bins_phi) (nf_stat_phitheta)."""
        h = np.zeros((bins_theta, bins_phi), np.uint64)
        _check(self._L.nf_stat_phitheta(self._h, bins_phi, bins_theta, h.ctypes.data_as(C.c_void_p)), self._h,
               "nf_stat_phitheta")
        return h

    def pair_stats(self, bins=32):
        """Contacts per rod and the mutual-angle histogram over the unscreened
        rod-rod contacts (nf_stat_pairs)."""
        n = self.n_rods()
        h = np.zeros(bins, np.uint64)
        per = np.zeros(max(n, 1), np.uint32)
        st = NfPairStats()
        _check(self._L.nf_stat_pairs(self._h, bins, h.ctypes.data_as(C.c_void_p), per.ctypes.data_as(C.c_void_p),
                                     len(per), C.byref(st)), self._h, "nf_stat_pairs")
        out = {k: getattr(st, k) for k, _ in st._fields_}
        out["hist"] = h
        out["per_rod"] = per[:n]
        return out

    def write_ort(self, path):
        _check(self._L.nf_write_ort_vtk(self._h, str(path).encode()), self._h, "nf_write_ort_vtk")

    def write_lmp(self, path, density=4.579):
        _check(self._L.nf_write_lmp(self._h, str(path).encode(), density), self._h, "nf_write_lmp")

    def ac_spectrum(self, freq, net=None, check=True, **ac):
        """AC admittance spectrum (nf_ac_spectrum) at the frequencies freq
        (Hz) of the handle's network (net=None: the intra-rod network after
        internal_network(), else the rod-level one) or of a host network
        given as a dict (n_nodes, seg_i, seg_j, seg_l, seg_a, ct_i, ct_j,
        ct_d, ct_s). Keyword arguments override nf_ac_params fields.
        Returns a dict of per-frequency arrays plus 'stats' and 'status'."""
        f = np.ascontiguousarray(freq, np.float64)
        pts = (NfAcPoint * max(len(f), 1))()
        st = NfAcStats()
        keep = []
        pn = None
        if net is not None:
            q = NfAcNet()
            q.n_nodes = int(net["n_nodes"])
            for k, t in (("seg_i", np.uint32), ("seg_j", np.uint32), ("seg_l", np.float64), ("seg_a", np.float64),
                         ("ct_i", np.uint32), ("ct_j", np.uint32), ("ct_d", np.float64), ("ct_s", np.float64)):
                a = np.ascontiguousarray(net.get(k, np.zeros(0)), t)
                keep.append(a)
                setattr(q, k, a.ctypes.data_as(C.c_void_p) if len(a) else None)
            q.n_segments = len(keep[0])
            q.n_contacts = len(keep[4])
            pn = C.byref(q)
        rc = self._L.nf_ac_spectrum(self._h, pn, C.byref(ac_params(**ac)), f.ctypes.data_as(C.c_void_p), len(f),
                                    C.cast(pts, C.c_void_p), C.byref(st))
        if check:
            _check(rc, self._h, "nf_ac_spectrum")
        out = {k: np.array([getattr(pts[i], k) for i in range(len(f))]) for k, _ in NfAcPoint._fields_}
        out["stats"] = {k: getattr(st, k) for k, _ in st._fields_}
        out["status"] = rc
        return out

    # diagnostics
    def set_kernel_timing(self, on=True):
        _check(self._L.nf_set_kernel_timing(self._h, int(on)), self._h, "nf_set_kernel_timing")

    def kernel_time(self, name):
        ms, b, f = C.c_double(), C.c_double(), C.c_double()
        n = C.c_uint64()
        _check(self._L.nf_kernel_time(self._h, name.encode(), C.byref(ms), C.byref(n), C.byref(b), C.byref(f)),
               self._h, "nf_kernel_time")
        return dict(ms=ms.value, launches=n.value, bytes=b.value, flops=f.value)

    # files
    def write_vtk(self, path):
        _check(self._L.nf_write_vtk(self._h, str(path).encode()), self._h, "nf_write_vtk")

    def write_state(self, path):
        _check(self._L.nf_write_state_bin(self._h, str(path).encode()), self._h, "nf_write_state_bin")

    def read_state(self, path):
        _check(self._L.nf_read_state_bin(self._h, str(path).encode()), self._h, "nf_read_state_bin")

    def write_coo(self, directory):
        _check(self._L.nf_write_coo(self._h, str(directory).encode()), self._h, "nf_write_coo")


class Batch(Simulation):
    """Many realisations in one handle (nf_create_batch): generate(),
    contacts() and solve() run them all in shared launches; select(r) picks
    the realisation that rods(), contact_list(), adjoint() and the solve
    stats report; results() gives every realisation's outcome."""

    def __init__(self, param_list, stream=None):
        self._L = load()
        self._nv = None
        self.n = len(param_list)
        arr = (NfParams * self.n)(*[make_params(p) for p in param_list])
        self.params = arr[0]
        h = C.c_void_p()
        _check(self._L.nf_create_batch(arr, self.n, C.byref(h)), what="nf_create_batch")
        self._h = h
        if stream is not None:
            _check(self._L.nf_set_stream(h, C.c_void_p(stream)), h)

    def select(self, r):
        _check(self._L.nf_select(self._h, int(r)), self._h, "nf_select")

    def results(self):
        res = (NfBatchResult * self.n)()
        _check(self._L.nf_batch_results(self._h, res, self.n), self._h, "nf_batch_results")
        return [{k: getattr(x, k) for k, _ in x._fields_} for x in res]


def batch_run(param_list):
    """All realisations in one engine (shared launches); returns (results, stats)."""
    L = load()
    n = len(param_list)
    arr = (NfParams * n)(*[make_params(p) for p in param_list])
    res = (NfBatchResult * n)()
    st = NfBatchStats()
    _check(L.nf_batch_run(arr, n, res, C.byref(st)), what="nf_batch_run")
    out = [{k: getattr(r, k) for k, _ in r._fields_} for r in res]
    return out, {k: getattr(st, k) for k, _ in st._fields_}


def ac_params(**kw):
    """nf_ac_params with the Kirchhoff tool's defaults, fields overridden by kw."""
    p = NfAcParams()
    load().nf_ac_params_default(C.byref(p))
    for k, v in kw.items():
        if k not in dict(NfAcParams._fields_):
            raise KeyError(k)
        setattr(p, k, v)
    return p


def ac_frequencies(log_df, n_patch=1, patch_id=0):
    """The Kirchhoff tool's frequency grid (Hz) for one patch (nf_ac_frequencies)."""
    L = load()
    n = L.nf_ac_frequencies(log_df, n_patch, patch_id, None, 0)
    f = np.zeros(n)
    L.nf_ac_frequencies(log_df, n_patch, patch_id, f.ctypes.data_as(C.c_void_p), n)
    return f


def write_impedance(path, spec):
    """impedance_rRC.<patch>.dat: frequency, Re Z, -Im Z, RMS per line, as the
    Kirchhoff tool's numpy.savetxt writes it (tools/kirchhoff/kirchhoff.py:284-286)."""
    np.savetxt(path, np.c_[spec["freq"], spec["z_re"], spec["z_im"], spec["rms"]])


def write_kirchhoff_log(path, spec, elapsed=None):
    """kirchhoff.<patch>.log with the tool's header and line format
    (tools/kirchhoff/kirchhoff.py:220-222,273-280)."""
    n = len(spec["freq"])
    el = np.zeros(n) if elapsed is None else np.broadcast_to(np.asarray(elapsed, float), (n,))
    with open(path, "w") as f:
        f.write("# Frequency\tZ_real\t(-1)Z_imag\tConverged\tRMSD\tElapsed\n")
        for i in range(n):
            f.write("{:>10.3e}\t{:>10.3e}\t{:>10.3e}\t{:>d}\t{:>10.3e}\t{:>10.3f}\n".format(
                spec["freq"][i], spec["z_re"][i], spec["z_im"][i], int(spec["converged"][i]), spec["rms"][i], el[i]))


def write_rho(path, hist):
    """rho.dat of the stat_phitheta verb; hist shaped (bins_theta, bins_phi)."""
    h = np.ascontiguousarray(hist, np.uint64)
    _check(load().nf_format_write_rho(str(path).encode(), h.shape[1], h.shape[0], h.ctypes.data_as(C.c_void_p)),
           what="nf_format_write_rho")


def write_gamma(path, hist):
    """gamma.dat of the stat_mutangle verb."""
    h = np.ascontiguousarray(hist, np.uint64)
    _check(load().nf_format_write_gamma(str(path).encode(), len(h), h.ctypes.data_as(C.c_void_p)),
           what="nf_format_write_gamma")
