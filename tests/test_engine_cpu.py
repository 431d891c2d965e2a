"""Host-side batch layout of NSBatch, built on the CPU (no kernel runs): work items cover every
chain exactly once, the items of each (family, D) bucket are contiguous, packed offsets are
exclusive prefix sums of the per-run sizes, and the linear-Gaussian family stores U as FP64
word pairs."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")


def _specs():
    from jaxns_gb300.engine import FAMILY_LINGAUSS, FAMILY_MVN, FAMILY_SHELLS, RunSpec
    out = []
    rng = np.random.default_rng(0)
    for i, (fam, D, n) in enumerate([(FAMILY_MVN, 4, 64), (FAMILY_MVN, 12, 200), (FAMILY_MVN, 20, 96),
                                     (FAMILY_MVN, 40, 128), (FAMILY_SHELLS, 6, 80), (FAMILY_SHELLS, 50, 100),
                                     (FAMILY_MVN, 9, 60), (FAMILY_MVN, 14, 90)]):
        s = n // 2
        out.append(RunSpec(D=D, num_live_points=n, shell_size=s, num_slices=2 * D, family=fam,
                           params=rng.standard_normal(D + D * D + 1 if fam == FAMILY_MVN else 2 * D + 3).astype(np.float32),
                           prior_kind=np.zeros(D, np.int32), prior_a=np.zeros(D), prior_b=np.ones(D),
                           max_samples=10 * n, term_cond={"dlogZ": 1e-4, "max_samples": 10.0 * n},
                           key=np.array([0, i], np.uint32), store_U=(i % 2 == 0)))
    return out


def test_items_cover_every_chain_once_and_buckets_are_contiguous():
    from jaxns_gb300.engine import NSBatch, _dbucket
    specs = _specs()
    for cpi, cpl, wide, wmin in ((32, 1, 0, 17), (64, 2, 256, 17), (128, 4, 512, 17), (64, 3, 0, 9)):
        b = NSBatch(specs, device="cpu", chains_per_item=cpi, wide_chains_per_item=wide, chains_per_lane=cpl,
                    warp_min_D=wmin)
        items = b.items.numpy()[: b._b.num_items]
        covered = [np.zeros(s.shell_size, np.int32) for s in specs]
        for r, c0, cnt, _ in items:
            covered[r][c0:c0 + cnt] += 1
            wide_run = specs[r].family == 0 and specs[r].D >= wmin
            # thread-per-chain CTAs draw from a pool of cpi * cpl chains
            assert cnt <= (wide or (256 if specs[r].D > 32 else 512)) if wide_run else cnt <= cpi * cpl
        assert all(np.all(c == 1) for c in covered)
        for k in range(8):
            lo, hi = b._b.bucket_begin[k], b._b.bucket_end[k]
            for r, *_ in items[lo:hi]:
                expect = specs[r].family * 4 + _dbucket(specs[r].D)
                if specs[r].family == 0 and specs[r].D >= wmin:
                    expect = max(expect, 2)  # correlated Gaussians on the warp-cooperative kernel
                assert expect == k
            Ds = [specs[r].D for r, *_ in items[lo:hi]]
            assert Ds == sorted(Ds, reverse=True)     # longest (largest D) first in a bucket
        assert sum(b._b.bucket_end[k] - b._b.bucket_begin[k] for k in range(8)) == len(items)


def test_packed_offsets_are_exclusive_prefix_sums():
    from jaxns_gb300.engine import NSBatch
    specs = _specs()
    b = NSBatch(specs, device="cpu")
    ns = np.array([s.num_live_points for s in specs])
    ss = np.array([s.shell_size for s in specs])
    caps = np.array([s.max_samples for s in specs])
    Ds = np.array([s.D for s in specs])
    excl = lambda v: np.concatenate([[0], np.cumsum(v)[:-1]])
    np.testing.assert_array_equal(b.offsets["live"], excl(ns))
    np.testing.assert_array_equal(b.offsets["shell"], excl(ss))
    np.testing.assert_array_equal(b.offsets["store"], excl(caps))
    np.testing.assert_array_equal(b.offsets["liveU"], excl(ns * Ds))
    ustore = np.array([s.store_U for s in specs])
    ucap = np.where(ustore, caps * Ds, 0)
    np.testing.assert_array_equal(b.offsets["ustore"], np.where(ustore, excl(ucap), -1))
    assert b.live_U[0].numel() == int((ns * Ds).sum()) and b.store_L.numel() == int(caps.sum())


def test_lingauss_runs_keep_fp64_U_as_word_pairs():
    from jaxns_gb300.engine import FAMILY_LINGAUSS, NSBatch, RunSpec
    N, P, n = 50, 3, 20
    rng = np.random.default_rng(1)
    spec = RunSpec(D=P, num_live_points=n, shell_size=n // 2, num_slices=2 * P, family=FAMILY_LINGAUSS,
                   params=np.concatenate([rng.standard_normal(N * P), rng.standard_normal(N), [0.5]]).astype(np.float32),
                   prior_kind=np.ones(P, np.int32), prior_a=np.zeros(P), prior_b=np.ones(P), max_samples=200,
                   term_cond={"dlogZ": 1e-4, "max_samples": 200.0}, key=np.array([0, 1], np.uint32), N=N)
    b = NSBatch([spec], device="cpu", lg_tensor_cores=False)
    assert int(b.ucols[0]) == 2 * P
    assert b.live_U[0].numel() == n * 2 * P and b.new_U.numel() == (n // 2) * 2 * P
    assert b.live_view(0)["U"].dtype == torch.float64 and b.live_view(0)["U"].shape == (n, P)
    assert b.lg_t["u0"].numel() == (n // 2) * P and b.lg_t["ss"].dtype == torch.float64
    U = np.random.default_rng(2).random((n, P))
    U[0, 0] = 1e-300                                  # a value fp32 cannot hold
    b.set_live(0, U, np.sort(rng.standard_normal(n)))
    np.testing.assert_array_equal(b.live_view(0)["U"].numpy(), U)


def test_batch_mixing_rules():
    from jaxns_gb300.engine import FAMILY_LINGAUSS, NSBatch
    specs = _specs()
    lg = _specs()[0]
    lg.family, lg.N = FAMILY_LINGAUSS, 10
    with pytest.raises(ValueError):
        NSBatch([specs[0], lg], device="cpu", lg_tensor_cores=False)
    specs[1].gradient_guided = True
    with pytest.raises(ValueError):
        NSBatch(specs, device="cpu")


def test_cpu_batch_refuses_to_launch():
    """A batch built on the CPU (layout only) never hands host buffers to a kernel."""
    from jaxns_gb300 import _ffi
    from jaxns_gb300.engine import NSBatch
    b = NSBatch(_specs(), device="cpu")
    for call in (b.init, lambda: b.iterate(1), b.finalize, lambda: b.results(with_U=False)):
        with pytest.raises(_ffi.GBNSError, match="no CPU path"):
            call()


def test_adjoint_refuses_host_tensors():
    from jaxns_gb300 import _ffi
    from jaxns_gb300.adjoint import DeadSet, evidence_and_grad
    ds = DeadSet(U=torch.rand(10, 3, dtype=torch.float64), log_w=torch.zeros(10, dtype=torch.float64),
                 Phi=torch.randn(20, 3), y=torch.randn(20))
    with pytest.raises(_ffi.GBNSError, match="no CPU path"):
        evidence_and_grad(ds, 0.0, 0.0)
    with pytest.raises(_ffi.GBNSError, match="U is on"):
        _ffi.require_cuda("x", U=np.zeros(3))


def test_hook_shapes_are_checked_on_the_host():
    from jaxns_gb300.engine import NSBatch
    specs = _specs()
    b = NSBatch(specs, device="cpu")
    with pytest.raises(ValueError, match="out of range"):
        b.forward(len(specs), torch.zeros(3, specs[0].D))
    with pytest.raises(ValueError, match=r"U must be \[B, 4\]"):
        b.forward(0, torch.zeros(3, 5))
    with pytest.raises(ValueError, match="one contour and one key"):
        b.slice_shell(torch.zeros(len(specs) - 1), torch.zeros(len(specs), 2, dtype=torch.int32))
    with pytest.raises(ValueError, match="one contour and one key"):
        b.slice_shell(torch.zeros(len(specs)), torch.zeros(len(specs), dtype=torch.int32))


def test_set_live_writes_the_run_slice():
    from jaxns_gb300.engine import NSBatch
    specs = _specs()
    b = NSBatch(specs, device="cpu")
    r = 2
    s = specs[r]
    U = np.random.default_rng(0).random((s.num_live_points, s.D)).astype(np.float32)
    L = np.sort(np.random.default_rng(1).standard_normal(s.num_live_points)).astype(np.float32)
    with pytest.raises(ValueError):
        b.set_live(r, U[:-1], L[:-1])
    b.set_live(r, U, L)
    v = b.live_view(r)
    np.testing.assert_array_equal(v["U"].numpy(), U)
    np.testing.assert_array_equal(v["log_L"].numpy(), L)
    for q in range(len(specs)):      # the other runs' slices are untouched
        if q != r:
            assert not b.live_view(q)["log_L"].any()


def test_shrinkage_coefficient_table():
    """ncoef_table rows are the n-only terms of _update_evidence_calc_op
    (internals/shrinkage_statistics.py:55-73): log T, log t, log T2, log t2, log tT."""
    import math
    from jaxns_gb300.engine import ncoef_table

    def lae(a, b):
        return max(a, b) + math.log1p(math.exp(-abs(a - b)))

    tab = ncoef_table(300)
    assert tab.shape == (301, 16)
    # bytes 64-103: the same five as fp32 pairs hi + lo (the device scans' form), to 2^-48
    pairs = tab[:, 8:].view(np.float32)
    hi, lo = pairs[:, 0:10:2].astype(np.float64), pairs[:, 1:10:2].astype(np.float64)
    assert np.all(hi[1:] == tab[1:, :5].astype(np.float32))
    np.testing.assert_allclose((hi + lo)[1:], tab[1:, :5], rtol=2.0 ** -46, atol=0)
    assert np.all(pairs[:, 10:] == 0)
    for n in (1, 2, 3, 7, 50, 299, 300):
        ln, ln1, ln2 = math.log(n), math.log(n + 1), math.log(n + 2)
        want = [-lae(0.0, -ln), -ln1, -lae(0.0, math.log(2.0) - ln), math.log(2.0) - ln1 - ln2, -lae(0.0, -ln) - ln2]
        np.testing.assert_allclose(tab[n, :5], want, rtol=1e-14, atol=1e-15)
        # and they are the logs of n/(n+1), 1/(n+1), n/(n+2), 2/((n+1)(n+2)), n/((n+1)(n+2))
        np.testing.assert_allclose(np.exp(tab[n, :5]), [n / (n + 1), 1 / (n + 1), n / (n + 2),
                                                        2 / ((n + 1) * (n + 2)), n / ((n + 1) * (n + 2))], rtol=1e-13)


@pytest.mark.parametrize("change,match", [
    ({"shell_size": 0}, "shell size"), ({"shell_size": 65}, "shell size"), ({"num_slices": 0}, "num_slices"),
    ({"num_phantom": 8}, "num_phantom"), ({"max_samples": 0}, "max_samples"), ({"D": 65}, "D=65"),
    ({"params": np.zeros(5, np.float32)}, "parameters"), ({"prior_a": np.zeros(3)}, "prior_a"),
    ({"prior_kind": np.full(4, 7, np.int32)}, "prior kinds"), ({"key": np.zeros(3, np.uint32)}, "key")])
def test_malformed_runs_are_rejected_on_the_host(change, match):
    """Every size a kernel reads from the run descriptor is checked before any buffer exists."""
    import dataclasses
    from jaxns_gb300.engine import NSBatch
    spec = dataclasses.replace(_specs()[0], **change)    # MVN, D = 4, n = 64, s = 32, S = 8
    with pytest.raises(ValueError, match=match):
        NSBatch([spec], device="cpu")


def test_lingauss_needs_data_rows():
    import dataclasses
    from jaxns_gb300.engine import FAMILY_LINGAUSS, NSBatch, param_count
    spec = dataclasses.replace(_specs()[0], family=FAMILY_LINGAUSS, N=0, params=np.zeros(1, np.float32))
    with pytest.raises(ValueError, match="N >= 1"):
        NSBatch([spec], device="cpu", lg_tensor_cores=False)
    assert param_count(FAMILY_LINGAUSS, 4, 10) == 51
