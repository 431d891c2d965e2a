"""A complete ctypes binding of libgbns.so: every entry point of include/gbns.h with its
argument kinds, for a caller that binds the C ABI directly (the Python package itself goes
through ``jaxns_gb300._ffi``).

    from jaxns_gb300.binding import bind
    lib = bind()                        # jaxns_gb300/_lib/libgbns.so, or bind(path)
    rc = lib.gbns_batch_iterate(ctypes.byref(batch), 16, stream)
    if rc != 0: raise RuntimeError(lib.gbns_last_error().decode())

Device pointers, struct pointers (``ctypes.byref``) and the CUDA stream are all ``c_void_p``.
"""
from __future__ import annotations

import ctypes
import os
from ctypes import c_char_p, c_double, c_int, c_longlong, c_void_p

P = c_void_p

ARGTYPES = {
    "gbns_version": [],
    "gbns_last_error": [],
    "gbns_abi_sizes": [P, c_int],
    "gbns_threefry2x32": [P, P, P, c_longlong, P],
    "gbns_threefry_split": [P, P, c_longlong, P],
    "gbns_random_bits64": [P, P, c_longlong, P],
    "gbns_uniform": [P, P, c_longlong, P],
    "gbns_normal": [P, P, c_longlong, P],
    "gbns_forward": [P, c_int, P, P, c_longlong, P],
    "gbns_batch_init": [P, P],
    "gbns_batch_iterate": [P, c_int, P],
    "gbns_batch_finalize": [P, P],
    "gbns_batch_shell": [P, P],
    "gbns_record_event": [P, P],
    "gbns_batch_merge": [P, P],
    "gbns_batch_results": [P, P, P],
    "gbns_slice_shell": [P, P, P, P],
    "gbns_count_crossed_edges": [P, P, c_longlong, P, P, P, P, P],
    "gbns_count_crossed_edges_static": [P, P, c_longlong, P, P, P],
    "gbns_lg_shell_begin": [P, P, P],
    "gbns_lg_steps": [P, P, c_int, P],
    "gbns_lg_chain_step": [P, P, P],
    "gbns_lg_residual": [P, P, P],
    "gbns_lg_prepare_tc": [P, P, P],
    "gbns_lg_shell_fused": [P, P, P],
    "gbns_lg_iterate": [P, P, c_int, P],
    "gbns_lg_fused_max_clusters": [P, P, P],
    "gbns_evidence_adjoint": [P, P, c_longlong, c_int, P, P, c_int, c_double, c_double, P, P, P, P],
    "gbns_evidence_adjoint_tc": [P, P, c_longlong, c_int, P, P, c_int, c_double, c_double, P, P, P, P, P, P, P],
    "gbns_sample_evidence": [P, P, P, c_longlong, c_int, P, P],
    "gbns_evidence_stats": [P, P, c_longlong, P, c_int, P, P, P, P, P],
    "gbns_prior_transform": [P, P, P, c_longlong, P, P, P, P],
}
RESTYPES = {"gbns_last_error": c_char_p}

DEFAULT_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "libgbns.so")


def bind(path: str = DEFAULT_PATH) -> ctypes.CDLL:
    """Load libgbns.so and declare every entry point's argument and return types."""
    lib = ctypes.CDLL(path)
    for name, args in ARGTYPES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = RESTYPES.get(name, c_int)
    return lib
