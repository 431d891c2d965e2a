"""ctypes binding of libgbns.so (the C ABI declared in ``include/gbns.h``).

The shared library is built in-tree by ``jaxns_gb300.build.build_library`` (nvcc,
``-gencode arch=compute_103a,code=sm_103a``).  There is no CPU fallback: if the library
is missing, importing the engine raises.
"""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libgbns.so")

c_int = ctypes.c_int
c_ll = ctypes.c_longlong
c_double = ctypes.c_double
c_void_p = ctypes.c_void_p
c_u32 = ctypes.c_uint32


class TermCond(ctypes.Structure):
    _fields_ = [(n, c_int) for n in ("has_ess", "has_evidence_uncert", "has_dlogZ", "has_max_samples",
                                      "has_max_nlik", "has_log_L_contour", "has_efficiency", "has_rtol",
                                      "has_atol", "has_peak_XL")] + \
               [(n, c_double) for n in ("ess", "evidence_uncert", "dlogZ", "max_samples", "max_nlik",
                                        "log_L_contour", "efficiency_threshold", "rtol", "atol",
                                        "peak_XL_frac")]


class EvCalc(ctypes.Structure):
    _fields_ = [(n, c_double) for n in ("log_L", "log_X_mean", "log_X2_mean", "log_Z_mean", "log_ZX_mean",
                                         "log_Z2_mean", "log_dZ_mean", "log_dZ2_mean")]


class RunDesc(ctypes.Structure):
    _fields_ = [("D", c_int), ("n", c_int), ("s", c_int), ("S", c_int), ("K", c_int), ("family", c_int),
                ("midpoint", c_int), ("uniform_phase", c_int), ("N", c_int), ("ucols", c_int),
                ("init_efficiency_threshold", c_double), ("log_L_offset", c_double), ("cap", c_ll), ("live_off", c_ll),
                ("store_off", c_ll), ("shell_off", c_ll), ("param_off", c_ll), ("prior_off", c_ll),
                ("ustore_off", c_ll), ("liveU_off", c_ll), ("newU_off", c_ll), ("phU_off", c_ll),
                ("phL_off", c_ll), ("tc", TermCond)]


class RunState(ctypes.Structure):
    _fields_ = [("ev", EvCalc), ("ev_rem", EvCalc), ("log_L_contour", c_double), ("efficiency", c_double),
                ("relative_spread", c_double), ("absolute_spread", c_double), ("peak_log_XL", c_double),
                ("num_likelihood_evaluations", c_ll), ("num_samples", c_ll), ("next_sample_idx", c_ll),
                ("iterations", c_ll), ("key", c_u32 * 2), ("plateau", c_int), ("no_seed_points", c_int),
                ("phase", c_int), ("done", c_int), ("termination_reason", c_int), ("parity", c_int),
                ("status", c_int), ("pad1", c_int)]


class Batch(ctypes.Structure):
    _fields_ = [("num_runs", c_int), ("nmax", c_int), ("ncoef_n", c_int), ("runs", c_void_p), ("state", c_void_p),
                ("live_U", c_void_p * 2), ("live_L", c_void_p * 2), ("live_Lc", c_void_p * 2),
                ("live_E", c_void_p * 2), ("live_S", c_void_p * 2),
                ("new_U", c_void_p), ("new_L", c_void_p), ("new_E", c_void_p), ("ph_U", c_void_p),
                ("ph_L", c_void_p), ("store_L", c_void_p), ("store_S", c_void_p), ("store_E", c_void_p),
                ("store_P", c_void_p), ("store_U", c_void_p), ("fparams", c_void_p), ("prior_kind", c_void_p),
                ("prior_a", c_void_p), ("prior_b", c_void_p), ("ncoef", c_void_p), ("items", c_void_p),
                ("num_items", c_int), ("bucket_begin", c_int * 8), ("bucket_end", c_int * 8),
                ("chains_per_item", c_int), ("max_evals_per_slice", c_int), ("gradient_guided", c_int),
                ("gradient_slice", c_int)]


class LGBufs(ctypes.Structure):
    _fields_ = [("j", c_void_p), ("in_slice", c_void_p), ("total", c_void_p), ("flags", c_void_p),
                ("left", c_void_p), ("right", c_void_p), ("t", c_void_p), ("alpha", c_void_p), ("logL0", c_void_p),
                ("ck", c_void_p), ("after_key", c_void_p), ("slices_key", c_void_p), ("dir_key", c_void_p),
                ("u0", c_void_p), ("u0_lo", c_void_p), ("dir", c_void_p), ("W", c_void_p), ("ss", c_void_p), ("chains_left", c_void_p),
                ("items", c_void_p), ("num_items", c_int), ("pmax", c_int), ("total_chains", c_ll),
                ("use_tc", c_int), ("num_items_tc", c_int), ("items_tc", c_void_p), ("W_hi", c_void_p),
                ("W_lo", c_void_p), ("Phi_hi", c_void_p), ("Phi_lo", c_void_p),
                ("row_base", c_void_p), ("total_rows", c_ll), ("num_ctas_tc", c_int), ("num_tiles", c_int),
                ("chain_run", c_void_p), ("tile_base", c_void_p), ("tile_pending", c_void_p), ("tc_done", c_void_p),
                ("items_fused", c_void_p), ("num_items_fused", c_int), ("cluster_size", c_int),
                ("rows_per_cta", c_int), ("pad_fused", c_int), ("max_steps", c_ll),
                ("grad", c_void_p), ("grad_list", c_void_p), ("grad_count", c_void_p)]


class ResultsBufs(ctypes.Structure):
    _fields_ = [("samples_indices", c_void_p), ("num_live_points", c_void_p), ("log_L_samples", c_void_p),
                ("log_dp_mean", c_void_p), ("log_X_mean", c_void_p), ("nevals_sorted", c_void_p),
                ("U_sorted", c_void_p), ("scalars", c_void_p), ("scratch_ll", c_void_p), ("scratch_i", c_void_p)]


class PriorTable(ctypes.Structure):
    _fields_ = [("D", c_int), ("kind", c_void_p), ("a", c_void_p), ("b", c_void_p), ("log_norm", c_void_p),
                ("A", c_void_p), ("row_start", c_void_p), ("c", c_void_p), ("log_det", ctypes.c_double)]


EXPORTED = ("gbns_version", "gbns_last_error", "gbns_abi_sizes", "gbns_threefry2x32", "gbns_threefry_split", "gbns_random_bits64",
            "gbns_uniform", "gbns_normal", "gbns_forward", "gbns_batch_init", "gbns_batch_iterate",
            "gbns_batch_finalize", "gbns_batch_results", "gbns_slice_shell", "gbns_count_crossed_edges",
            "gbns_evidence_stats", "gbns_batch_shell", "gbns_batch_merge", "gbns_record_event",
            "gbns_count_crossed_edges_static", "gbns_lg_shell_begin", "gbns_lg_steps", "gbns_evidence_adjoint",
            "gbns_lg_prepare_tc", "gbns_evidence_adjoint_tc", "gbns_lg_chain_step", "gbns_lg_residual",
            "gbns_sample_evidence", "gbns_lg_shell_fused", "gbns_lg_iterate", "gbns_lg_fused_max_clusters",
            "gbns_prior_transform")

_lib = None


class GBNSError(RuntimeError):
    pass


def load(path: str = LIB_PATH):
    """Load libgbns.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise GBNSError(f"libgbns.so not found at {path}: run jaxns_gb300.build.build_library() "
                        "(there is no CPU fallback)")
    lib = ctypes.CDLL(path)
    lib.gbns_last_error.restype = ctypes.c_char_p
    lib.gbns_version.restype = c_int
    _lib = lib
    return lib


def require_cuda(what: str, **tensors):
    """Raise unless every named tensor lives on one CUDA device: the kernels take device
    pointers, and a host pointer must never reach them (there is no CPU path)."""
    devs = set()
    for name, t in tensors.items():
        if not getattr(t, "is_cuda", False):
            raise GBNSError(f"{what}: {name} is on {getattr(t, 'device', type(t).__name__)}; the kernels need CUDA "
                            "device buffers (there is no CPU path)")
        devs.add(t.device)
    if len(devs) > 1:
        raise GBNSError(f"{what}: tensors on several devices {sorted(map(str, devs))}")


def call(name: str, *args):
    lib = load()
    rc = getattr(lib, name)(*args)
    if rc != 0:
        raise GBNSError(f"{name} failed ({rc}): {lib.gbns_last_error().decode(errors='replace')}")
    return rc
