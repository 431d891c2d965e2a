"""gbns_count_crossed_edges_static: live-point counting for callers that cannot allocate
device memory (a host runtime that owns all device memory, such as an XLA FFI custom call;
a real-time pipeline that cannot take cudaMalloc's implicit synchronisation).  Its scratch is
a fixed device array inside libgbns.so, so this test checks that two calls in a row, each
reusing that array, give exactly what the allocating entry point gives on the same inputs.

This file is collected last on purpose: it runs after every other test."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

MAX_SAMPLES = 262143


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _cases():
    rng = np.random.default_rng(11)
    N1 = 5000  # unsorted store with ties (+0/-0 and rounded values): the radix-sort path
    s1 = rng.integers(0, N1 // 2, size=N1).astype(np.int32)
    L1 = np.round(rng.standard_normal(N1), 2).astype(np.float32)
    L1[:10] = 0.0
    L1[10:20] = -0.0
    N2 = 200000  # sorted store: the already-sorted path
    L2 = np.sort(rng.standard_normal(N2)).astype(np.float32)
    s2 = np.minimum(np.arange(N2), rng.integers(0, N2, size=N2)).astype(np.int32)
    N3 = MAX_SAMPLES  # unsorted at the capacity: the last elements of the fixed arrays are used
    s3 = rng.integers(0, N3, size=N3).astype(np.int32)
    L3 = np.round(rng.standard_normal(N3), 3).astype(np.float32)
    N4 = 3000  # senders outside [0, N]: negative ones count for the root, too large ones are dropped
    s4 = rng.integers(-5, N4 + 40, size=N4).astype(np.int32)
    s4[:8] = [N4, N4 + 1, 2 ** 31 - 1, -2 ** 31, N4 + 7, -1, 0, N4 - 1]
    L4 = np.round(rng.standard_normal(N4), 2).astype(np.float32)
    return [(s1, L1), (s2, L2), (s3, L3), (s4, L4)]


def _allocating(gpu_lib, sender, L):
    N = len(L)
    si = torch.zeros(N, dtype=torch.int32, device="cuda")
    nl = torch.zeros(N, dtype=torch.int32, device="cuda")
    scratch_ll = torch.zeros(2 * (N + 1), dtype=torch.int64, device="cuda")
    scratch_i = torch.zeros(N + 1, dtype=torch.int32, device="cuda")
    rc = gpu_lib.gbns_count_crossed_edges(_p(sender), _p(L), ctypes.c_longlong(N), _p(si), _p(nl), _p(scratch_ll),
                                          _p(scratch_i), _stream())
    assert rc == 0, gpu_lib.gbns_last_error()
    return si, nl


def _static(gpu_lib, sender, L):
    N = len(L)
    si = torch.full((N,), -7, dtype=torch.int32, device="cuda")
    nl = torch.full((N,), -7, dtype=torch.int32, device="cuda")
    rc = gpu_lib.gbns_count_crossed_edges_static(_p(sender), _p(L), ctypes.c_longlong(N), _p(si), _p(nl), _stream())
    assert rc == 0, gpu_lib.gbns_last_error()
    return si, nl


def test_static_scratch_matches_allocating_entry_point(gpu_lib, oracle_mod):
    gpu_lib.gbns_last_error.restype = ctypes.c_char_p
    host = _cases()
    cases = [(torch.tensor(s, device="cuda"), torch.tensor(L, device="cuda")) for s, L in host]
    # calls in a row on the shared scratch (each sees the previous call's leftovers), then the
    # first input again; both entry points against the oracle's count_crossed_edges
    checked_first = False
    for k in list(range(len(cases))) + [0]:
        sender, L = cases[k]
        si_s, nl_s = _static(gpu_lib, sender, L)
        si_a, nl_a = _allocating(gpu_lib, sender, L)
        torch.cuda.synchronize()
        assert torch.equal(si_s, si_a)
        assert torch.equal(nl_s, nl_a)
        if k != 0 or not checked_first:  # every case once (the large ones run over many CTAs)
            checked_first = checked_first or k == 0
            osi, onl = oracle_mod.count_crossed_edges(host[k][0], host[k][1].astype(np.float64))
            np.testing.assert_array_equal(si_s.cpu().numpy(), osi)
            np.testing.assert_array_equal(nl_s.cpu().numpy(), onl)


def test_static_scratch_empty_set(gpu_lib):
    """N = 0 (buffers keep one element so that no pointer is NULL): both entry points leave the
    outputs untouched and return 0."""
    gpu_lib.gbns_last_error.restype = ctypes.c_char_p
    sender = torch.zeros(1, dtype=torch.int32, device="cuda")
    L = torch.zeros(1, dtype=torch.float32, device="cuda")
    si = torch.full((1,), -7, dtype=torch.int32, device="cuda")
    nl = torch.full((1,), -7, dtype=torch.int32, device="cuda")
    rc = gpu_lib.gbns_count_crossed_edges_static(_p(sender), _p(L), ctypes.c_longlong(0), _p(si), _p(nl), _stream())
    assert rc == 0, gpu_lib.gbns_last_error()
    scratch_ll = torch.zeros(2, dtype=torch.int64, device="cuda")
    scratch_i = torch.zeros(1, dtype=torch.int32, device="cuda")
    si2 = torch.full((1,), -7, dtype=torch.int32, device="cuda")
    nl2 = torch.full((1,), -7, dtype=torch.int32, device="cuda")
    rc = gpu_lib.gbns_count_crossed_edges(_p(sender), _p(L), ctypes.c_longlong(0), _p(si2), _p(nl2), _p(scratch_ll),
                                          _p(scratch_i), _stream())
    assert rc == 0, gpu_lib.gbns_last_error()
    torch.cuda.synchronize()
    assert int(si.item()) == -7 and int(nl.item()) == -7
    assert int(si2.item()) == -7 and int(nl2.item()) == -7


def test_static_scratch_rejects_oversize(gpu_lib):
    gpu_lib.gbns_last_error.restype = ctypes.c_char_p
    out = torch.zeros(4, dtype=torch.int32, device="cuda")
    dummy_L = torch.zeros(4, dtype=torch.float32, device="cuda")
    dummy_s = torch.zeros(4, dtype=torch.int32, device="cuda")
    rc = gpu_lib.gbns_count_crossed_edges_static(_p(dummy_s), _p(dummy_L), ctypes.c_longlong(MAX_SAMPLES + 1), _p(out),
                                                 _p(out), _stream())
    assert rc == -1
    assert b"262143" in gpu_lib.gbns_last_error()
