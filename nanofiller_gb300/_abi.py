"""ctypes mirror of include/nanofiller_gb300.h and the library loader.

The library is built in-tree (nanofiller_gb300/_build/libnanofiller_gb300.so).
Loading fails with an ImportError-like RuntimeError when it is missing: there is
no fallback implementation.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libnanofiller_gb300.so")

SRC_ELEC = 0xFFFFFFFF
SNK_ELEC = 0xFFFFFFFE

STATUS = {
    0: "NF_OK", 1: "NF_ERR_PARAM", 2: "NF_ERR_CUDA", 3: "NF_ERR_NO_DEVICE", 4: "NF_ERR_ALLOC",
    5: "NF_ERR_CAPACITY", 6: "NF_ERR_OVERFLOW", 7: "NF_ERR_NOT_CONVERGED", 8: "NF_ERR_IO",
    9: "NF_ERR_FORMAT", 10: "NF_ERR_STATE", 11: "NF_ERR_UNSUPPORTED", 12: "NF_ERR_TIMEOUT",
}


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


class NfRods(C.Structure):
    _fields_ = [("capacity", C.c_size_t), ("count", C.c_size_t)] + \
        [(f, C.POINTER(C.c_float)) for f in ("x", "y", "z", "cx", "cy", "cz", "l", "a")] + \
        [("stream_index", C.POINTER(C.c_uint64)), ("cell", C.POINTER(C.c_uint32))]


class NfContactList(C.Structure):
    _fields_ = [("capacity", C.c_size_t), ("count", C.c_size_t),
                ("I", C.POINTER(C.c_uint32)), ("J", C.POINTER(C.c_uint32)),
                ("tI", C.POINTER(C.c_float)), ("tJ", C.POINTER(C.c_float)),
                ("D", C.POINTER(C.c_double)), ("G", C.POINTER(C.c_double)),
                ("S", C.POINTER(C.c_double)), ("image", C.POINTER(C.c_int8))]


class NfGenStats(C.Structure):
    _fields_ = [("candidates_drawn", C.c_uint64), ("density_accepted", C.c_uint64),
                ("accepted", C.c_uint64), ("target", C.c_uint64), ("pair_tests", C.c_uint64),
                ("exact_evals", C.c_uint64), ("fp32_would_flip", C.c_uint64),
                ("rounds", C.c_int32), ("target_reached", C.c_int32), ("ms", C.c_double),
                ("work_items", C.c_uint64), ("target_tiles", C.c_uint64), ("marked_pairs", C.c_uint64),
                ("line_pairs", C.c_uint64), ("epochs", C.c_uint64), ("refits", C.c_uint64),
                ("thinned", C.c_uint64), ("snapped", C.c_uint64), ("tube_grid", C.c_int32),
                ("redone_rounds", C.c_int32)]


class NfContactStats(C.Structure):
    _fields_ = [("contacts", C.c_uint64), ("screened", C.c_uint64), ("n_source", C.c_uint64),
                ("n_sink", C.c_uint64), ("pair_tests", C.c_uint64), ("exact_evals", C.c_uint64),
                ("fp32_would_flip", C.c_uint64), ("ms", C.c_double)]


class NfSolveStats(C.Structure):
    _fields_ = [("G_eff", C.c_double), ("residual", C.c_double), ("outer_iters", C.c_int32),
                ("inner_iters", C.c_int32), ("n_nodes", C.c_int64), ("n_active", C.c_int64),
                ("percolating", C.c_int32), ("ms", C.c_double), ("direct", C.c_int32),
                ("bandwidth", C.c_uint32)]


class NfBatchResult(C.Structure):
    _fields_ = [("accepted", C.c_uint64), ("contacts", C.c_uint64), ("G_eff", C.c_double),
                ("residual", C.c_double), ("percolating", C.c_int32), ("status", C.c_int32)]


class NfInternalStats(C.Structure):
    _fields_ = [("contact_ends", C.c_uint64), ("nodes", C.c_uint64), ("segments", C.c_uint64)]


class NfInternalNet(C.Structure):
    _fields_ = [("capacity", C.c_size_t), ("n_nodes", C.c_size_t), ("n_segments", C.c_size_t),
                ("n_edges", C.c_size_t), ("node_rod", C.c_void_p), ("node_t", C.c_void_p), ("seg_i", C.c_void_p),
                ("seg_j", C.c_void_p), ("seg_l", C.c_void_p), ("seg_g", C.c_void_p), ("edge_i", C.c_void_p),
                ("edge_j", C.c_void_p)]


class NfReduceStats(C.Structure):
    _fields_ = [("rods_before", C.c_uint64), ("rods_after", C.c_uint64), ("contacts", C.c_uint64),
                ("rounds", C.c_int32), ("min_contacts", C.c_int32), ("ms", C.c_double)]


class NfPairStats(C.Structure):
    _fields_ = [("rods", C.c_uint64), ("pairs", C.c_uint64), ("contacts_total", C.c_uint64),
                ("angle_pairs", C.c_uint64), ("max_per_rod", C.c_uint32), ("pad", C.c_uint32),
                ("mean_per_rod", C.c_double)]


class NfAcParams(C.Structure):
    _fields_ = [("r_cnt", C.c_double), ("l_cnt", C.c_double), ("phi_ev", C.c_double), ("eps_r", C.c_double),
                ("delta_min", C.c_double), ("delta_tun", C.c_double), ("delta_eff", C.c_double),
                ("c_min", C.c_double), ("l_box", C.c_double), ("own_radii", C.c_int32), ("method", C.c_int32),
                ("tol", C.c_double)]


class NfAcPoint(C.Structure):
    _fields_ = [("freq", C.c_double), ("i_re", C.c_double), ("i_im", C.c_double), ("z_re", C.c_double),
                ("z_im", C.c_double), ("rms", C.c_double), ("residual", C.c_double), ("i_err", C.c_double),
                ("iters", C.c_int32), ("converged", C.c_int32)]


class NfAcStats(C.Structure):
    _fields_ = [("n_nodes", C.c_uint64), ("n_active", C.c_uint64), ("n_contacts", C.c_uint64),
                ("n_kept", C.c_uint64), ("n_segments", C.c_uint64), ("R0", C.c_double), ("C0", C.c_double),
                ("omega0", C.c_double), ("ms", C.c_double), ("bandwidth", C.c_uint32), ("direct", C.c_int32)]


class NfAcNet(C.Structure):
    _fields_ = [("n_nodes", C.c_uint64), ("n_segments", C.c_uint64), ("seg_i", C.c_void_p), ("seg_j", C.c_void_p),
                ("seg_l", C.c_void_p), ("seg_a", C.c_void_p), ("n_contacts", C.c_uint64), ("ct_i", C.c_void_p),
                ("ct_j", C.c_void_p), ("ct_d", C.c_void_p), ("ct_s", C.c_void_p)]


class NfTuneResult(C.Structure):
    _fields_ = [("stencil_radius", C.c_int32), ("round_overshoot", C.c_float), ("two_phase_work", C.c_double),
                ("ms_first", C.c_double), ("ms_best", C.c_double), ("trials", C.c_int32),
                ("tube_load", C.c_float)]


class NfBatchStats(C.Structure):
    _fields_ = [("n", C.c_int32), ("rounds", C.c_int32), ("rods", C.c_uint64),
                ("contacts", C.c_uint64), ("ms", C.c_double)]


class NfStateHeader(C.Structure):
    _fields_ = [("phys_dim", C.c_float * 3), ("edge", C.c_float * 3), ("ext", C.c_int32 * 3),
                ("l", C.c_float), ("a", C.c_float), ("ttl", C.c_int32), ("num", C.c_int32),
                ("tol", C.c_float)]


# Every exported symbol of the header with its ctypes signature.
_P = C.POINTER
_H = C.c_void_p
_st = C.c_int
SIGNATURES = {
    "nf_abi_version": (C.c_int, []),
    "nf_status_string": (C.c_char_p, [C.c_int]),
    "nf_params_default": (_st, [_P(NfParams)]),
    "nf_params_from_file": (_st, [C.c_char_p, _P(NfParams), _P(C.c_int)]),
    "nf_target_count": (_st, [_P(NfParams), _P(C.c_int64)]),
    "nf_create": (_st, [_P(NfParams), _P(_H)]),
    "nf_destroy": (_st, [_H]),
    "nf_set_stream": (_st, [_H, C.c_void_p]),
    "nf_last_error": (_st, [_H, C.c_char_p, C.c_size_t]),
    "nf_load_density": (_st, [_H, C.c_int, C.c_int, C.c_int, C.c_void_p]),
    "nf_read_density_file": (_st, [C.c_char_p, _P(C.c_int), _P(C.c_float), C.c_void_p, C.c_size_t]),
    "nf_generate": (_st, [_H, _P(NfGenStats)]),
    "nf_stream_candidates": (_st, [_H, C.c_uint64, C.c_uint64] + [C.c_void_p] * 10),
    "nf_stream_candidates_noalloc": (_st, [_H, C.c_uint64, C.c_uint64] + [C.c_void_p] * 10),
    "nf_get_rods": (_st, [_H, _P(NfRods)]),
    "nf_set_rods": (_st, [_H, _P(NfRods)]),
    "nf_contacts": (_st, [_H, _P(NfContactStats)]),
    "nf_get_contacts": (_st, [_H, _P(NfContactList)]),
    "nf_solve": (_st, [_H, _P(NfSolveStats)]),
    "nf_get_voltages": (_st, [_H, C.c_void_p, C.c_size_t]),
    "nf_adjoint": (_st, [_H, C.c_void_p, C.c_size_t, _P(C.c_double), _P(C.c_double)]),
    "nf_batch_run": (_st, [_P(NfParams), C.c_int, _P(NfBatchResult), _P(NfBatchStats)]),
    "nf_create_batch": (_st, [_P(NfParams), C.c_int, _P(C.c_void_p)]),
    "nf_select": (_st, [C.c_void_p, C.c_int32]),
    "nf_batch_results": (_st, [C.c_void_p, _P(NfBatchResult), C.c_int32]),
    "nf_write_vtk": (_st, [_H, C.c_char_p]),
    "nf_write_state_bin": (_st, [_H, C.c_char_p]),
    "nf_read_state_bin": (_st, [_H, C.c_char_p]),
    "nf_write_coo": (_st, [_H, C.c_char_p]),
    "nf_kernel_launches": (C.c_uint64, []),
    "nf_allocations": (C.c_uint64, []),
    "nf_release_cached_memory": (_st, []),
    "nf_set_kernel_timing": (_st, [_H, C.c_int]),
    "nf_autotune": (_st, [_H, _P(NfTuneResult)]),
    "nf_internal_network": (_st, [_H, _P(NfInternalStats)]),
    "nf_get_internal_network": (_st, [_H, _P(NfInternalNet)]),
    "nf_write_internal_coo": (_st, [_H, C.c_char_p]),
    "nf_reduce": (_st, [_H, C.c_int32, _P(NfReduceStats)]),
    "nf_set_orientation": (_st, [_H, C.c_int32, C.c_float, C.c_float, C.c_float]),
    "nf_orientation_laws": (_st, [_H, C.c_size_t, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_size_t)]),
    "nf_stat_nematic": (_st, [_H, C.c_void_p, _P(C.c_double)]),
    "nf_stat_phitheta": (_st, [_H, C.c_int32, C.c_int32, C.c_void_p]),
    "nf_stat_pairs": (_st, [_H, C.c_int32, C.c_void_p, C.c_void_p, C.c_size_t, _P(NfPairStats)]),
    "nf_write_ort_vtk": (_st, [_H, C.c_char_p]),
    "nf_format_write_ort_vtk": (_st, [C.c_char_p, C.c_size_t] + [C.c_void_p] * 3),
    "nf_format_write_lmp": (_st, [C.c_char_p, C.c_size_t] + [C.c_void_p] * 9 + [C.c_double]),
    "nf_write_lmp": (_st, [_H, C.c_char_p, C.c_double]),
    "nf_format_write_rho": (_st, [C.c_char_p, C.c_int32, C.c_int32, C.c_void_p]),
    "nf_format_write_gamma": (_st, [C.c_char_p, C.c_int32, C.c_void_p]),
    "nf_ac_params_default": (None, [_P(NfAcParams)]),
    "nf_ac_frequencies": (C.c_size_t, [C.c_double, C.c_int, C.c_int, C.c_void_p, C.c_size_t]),
    "nf_ac_spectrum": (_st, [_H, _P(NfAcNet), _P(NfAcParams), C.c_void_p, C.c_size_t, C.c_void_p,
                             _P(NfAcStats)]),
    "nf_kernel_time": (_st, [_H, C.c_char_p, _P(C.c_double), _P(C.c_uint64), _P(C.c_double),
                             _P(C.c_double)]),
    "nf_format_write_vtk": (_st, [C.c_char_p, C.c_size_t] + [C.c_void_p] * 9),
    "nf_format_write_state_bin": (_st, [C.c_char_p, _P(NfStateHeader), C.c_void_p, C.c_void_p,
                                        C.c_void_p]),
    "nf_format_read_state_bin": (_st, [C.c_char_p, _P(NfStateHeader), C.c_void_p, C.c_void_p,
                                       C.c_void_p, C.c_size_t, C.c_size_t]),
}

_lib = None


def load(path=None):
    """Load the in-tree library (no fallback: raises if it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError(
            f"{path} is missing: build it with `python -m nanofiller_gb300.build` "
            "(this package has no CPU fallback)")
    L = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L
