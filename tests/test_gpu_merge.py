"""Dead-point ordering on the device, word for word: k_merge (gbns_batch_merge) on a fixed
log-likelihood stream against the oracle's stable argsort (jnp.argsort order: -0 == +0,
ties by position) of _collect_shell (sharded_static.py:240-275).

The run's live set and the shell outputs are overwritten with chosen values (ties, signed
zeros, -inf, a plateau; n up to 4096), so the merge sees exactly the stream the test knows;
the permuted live set (log L, U rows, evaluation counts, senders, constraints) and the store
append must equal the oracle's permutation of the same stream."""
import ctypes

import numpy as np
import pytest

from tests.conftest import corr_gauss

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _stream(n, s, seed):
    """Live log L (sorted ascending, as the live set always is) and new shell log L with
    ties, +-0, -inf and a plateau."""
    rng = np.random.default_rng(seed)
    live = np.round(rng.standard_normal(n) * 3, 1).astype(np.float32)
    live[: n // 8] = -np.inf
    live[n // 8: n // 8 + max(1, n // 16)] = -0.0
    live[n // 3: n // 3 + max(1, n // 10)] = 1.5                    # plateau
    live = np.sort(live)
    new = np.round(rng.standard_normal(s) * 3, 1).astype(np.float32)
    new[::7] = 0.0
    new[3::7] = -0.0
    new[5::11] = 1.5                                                # ties with the plateau
    new[1::13] = -np.inf
    return live, new


@pytest.mark.parametrize("n,seed", [(7, 0), (64, 1), (1000, 2), (4096, 3)])
def test_merge_permutation_matches_stable_argsort(gpu_lib, oracle_mod, n, seed):
    from jaxns_gb300 import _ffi
    from jaxns_gb300.engine import NSBatch, RunSpec, mvn_offset, mvn_params
    D = 3
    mu, cov = corr_gauss(D, seed)
    s = n // 2
    cap = 8 * n
    cap = int(np.ceil(cap / s) * s)
    spec = RunSpec(D=D, num_live_points=n, shell_size=s, num_slices=D, family=0, params=mvn_params(mu, cov),
                   prior_kind=np.zeros(D, np.int32), prior_a=np.full(D, -10.0), prior_b=np.full(D, 20.0),
                   max_samples=cap, term_cond={"dlogZ": 1e-4, "max_samples": float(cap)},
                   key=np.asarray(oracle_mod.PRNGKey(seed), np.uint32), log_L_offset=float(mvn_offset(cov)))
    b = NSBatch([spec])
    b.init()
    st = b.state()[0]
    assert st["phase"] == 1 and st["done"] == 0
    p = int(st["parity"])
    live_L, new_L = _stream(n, s, seed)
    # index-coded U rows, evaluation counts, senders and constraints tell the rows apart
    live_U = (np.arange(n * D, dtype=np.float32).reshape(n, D) + 0.25) / (n * D + 1)
    new_U = (np.arange(s * D, dtype=np.float32).reshape(s, D) + 0.75) / (s * D + 1)
    live_E = np.arange(n, dtype=np.int32) + 1000
    new_E = np.arange(s, dtype=np.int32) + 5000
    live_S = np.arange(n, dtype=np.int32) % 17
    live_Lc = (np.arange(n, dtype=np.float32) - n).astype(np.float32)
    b.set_live(0, live_U, live_L)
    b.live_E[p][:n].copy_(torch.from_numpy(live_E))
    b.live_S[p][:n].copy_(torch.from_numpy(live_S))
    b.live_Lc[p][:n].copy_(torch.from_numpy(live_Lc))
    b.new_L[:s].copy_(torch.from_numpy(new_L))
    b.new_U[:s * D].copy_(torch.from_numpy(new_U.ravel()))
    b.new_E[:s].copy_(torch.from_numpy(new_E))
    _ffi.call("gbns_batch_merge", ctypes.byref(b._b), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    st = b.state()[0]
    q = int(st["parity"])
    assert q == 1 - p

    # oracle: _collect_shell replaces slots [0, s) with the new samples, then argsorts stably
    keys = np.concatenate([new_L, live_L[s:]])
    perm = oracle_mod.stable_argsort(keys.astype(np.float64))
    fresh = perm < s
    U_all = np.concatenate([new_U, live_U[s:]])
    E_all = np.concatenate([new_E, live_E[s:]])
    sender_idx = s - 1  # next_sample_idx - 1 after the shell's store append (sharded_static.py:261)
    S_exp = np.where(fresh, sender_idx, np.concatenate([np.zeros(s, np.int32), live_S[s:]])[perm])
    Lc_exp = np.where(fresh, live_L[s - 1], np.concatenate([np.zeros(s, np.float32), live_Lc[s:]])[perm])

    got_L = b.live_L[q][:n].cpu().numpy()
    np.testing.assert_array_equal(got_L.view(np.uint32), keys[perm].view(np.uint32))  # incl. the sign of zeros
    np.testing.assert_array_equal(b.live_U[q][:n * D].view(n, D).cpu().numpy(), U_all[perm])
    np.testing.assert_array_equal(b.live_E[q][:n].cpu().numpy(), E_all[perm])
    np.testing.assert_array_equal(b.live_S[q][:n].cpu().numpy(), S_exp)
    np.testing.assert_array_equal(b.live_Lc[q][:n].cpu().numpy().view(np.uint32),
                                  Lc_exp.astype(np.float32).view(np.uint32))
    # the discarded shell went to the store in live-set order with its senders and counts
    np.testing.assert_array_equal(b.store_L[:s].cpu().numpy().view(np.uint32), live_L[:s].view(np.uint32))
    np.testing.assert_array_equal(b.store_S[:s].cpu().numpy(), live_S[:s])
    np.testing.assert_array_equal(b.store_E[:s].cpu().numpy(), live_E[:s])
    np.testing.assert_array_equal(b.store_P[:s].cpu().numpy(), 0)
    assert int(st["num_likelihood_evaluations"]) == int(new_E.sum())
