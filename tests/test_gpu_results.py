"""k_results (the batch's _to_results, sharded_static.py:652-773) against the oracle's
_to_results of the very same sample store: sender tree, FP64 log L, evaluation counts and
phantom flags read back from the device, so the comparison isolates the results pass (tree
count, gather, evidence per sample, normalisation, H, ESS, uncertainty, efficiency) from the
sampler.  Stores with phantoms are out of likelihood order, which takes the radix-sort path."""
import numpy as np
import pytest

from tests.conftest import corr_gauss

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _specs(num_phantom):
    import jaxns_gb300 as gb
    from jaxns_gb300.engine import RunSpec, mvn_offset, mvn_params, shells_offset, shells_params
    specs = []
    for r, D in enumerate([3, 6]):
        mu, cov = corr_gauss(D, 40 + r)
        n = 40 * D
        s = n // 2
        cap = int(np.ceil(n * (3 * D + 25) / s)) * s * (1 + num_phantom)
        specs.append(RunSpec(D=D, num_live_points=n, shell_size=s, num_slices=3 * D, family=0,
                             params=mvn_params(mu, cov), prior_kind=np.zeros(D, np.int32),
                             prior_a=np.full(D, -10.0), prior_b=np.full(D, 20.0), max_samples=cap,
                             term_cond={"dlogZ": 1e-4, "max_samples": float(cap)}, num_phantom=num_phantom,
                             key=gb.random.PRNGKey(500 + r), store_U=False, log_L_offset=mvn_offset(cov)))
    D = 4
    c1 = np.zeros(D); c1[0] = 3.5
    n, w = 200, 0.1
    cap = 200 * 60 * (1 + num_phantom)
    specs.append(RunSpec(D=D, num_live_points=n, shell_size=n // 2, num_slices=5 * D, family=1,
                         params=shells_params(c1, -c1, 2.0, w), prior_kind=np.zeros(D, np.int32),
                         prior_a=np.full(D, -6.0), prior_b=np.full(D, 12.0), max_samples=cap,
                         term_cond={"dlogZ": 1e-4, "max_samples": float(cap)}, num_phantom=num_phantom,
                         key=gb.random.PRNGKey(777), store_U=False, log_L_offset=shells_offset(w)))
    return specs


@pytest.mark.parametrize("num_phantom", [0, 2])
def test_results_match_oracle_on_the_same_store(gpu_lib, oracle_mod, num_phantom):
    from jaxns_gb300.engine import NSBatch
    b = NSBatch(_specs(num_phantom))
    b.run(block=8)
    out = b.results(with_U=False)
    unsorted = 0
    for r in range(b.R):
        sv = b.store_view(r)
        L = sv["log_L"].cpu().numpy()
        unsorted += int(np.any(np.diff(sv["log_L_raw"].cpu().numpy()) < 0))
        sc_o, si_o, nl_o, ls_o, dp_o, lx_o = oracle_mod.results_of_store(
            sv["sender"].cpu().numpy(), L, sv["nevals"].cpu().numpy(), sv["phantom"].cpu().numpy())
        v = b.run_slices(r, out)
        # integer and gathered outputs: bit for bit
        np.testing.assert_array_equal(v["samples_indices"].cpu().numpy(), si_o)
        np.testing.assert_array_equal(v["num_live_points"].cpu().numpy(), nl_o)
        np.testing.assert_array_equal(v["log_L_samples"].cpu().numpy(), ls_o)
        np.testing.assert_array_equal(v["nevals_sorted"].cpu().numpy(), sv["nevals"].cpu().numpy()[si_o])
        # the evidence per sample (fp32-pair scan with FP64 carries vs sequential FP64)
        np.testing.assert_allclose(v["log_X_mean"].cpu().numpy(), lx_o, rtol=1e-12, atol=1e-9)
        dp = v["log_dp_mean"].cpu().numpy()
        fin = np.isfinite(dp_o)
        np.testing.assert_array_equal(np.isfinite(dp), fin)
        # log dZ carries the fp32 accuracy of the midpoint log((L_k + L_{k-1}) / 2) (about 1e-7)
        np.testing.assert_allclose(dp[fin], dp_o[fin], rtol=1e-6, atol=1e-6)
        sc = v["scalars"].cpu().numpy()
        print(f"run {r}: |d log dp| {np.max(np.abs(dp[fin] - dp_o[fin])):.2e}, d log Z {sc[0] - sc_o['log_Z_mean']:.2e}, "
              f"d uncert {sc[1] / sc_o['log_Z_uncert'] - 1:.2e}, d ESS {sc[2] / sc_o['ESS'] - 1:.2e}, "
              f"d H {sc[3] - sc_o['H_mean']:.2e}")
        assert abs(sc[0] - sc_o["log_Z_mean"]) < 1e-6, (r, sc[0], sc_o["log_Z_mean"])
        np.testing.assert_allclose(sc[1], sc_o["log_Z_uncert"], rtol=1e-5)
        np.testing.assert_allclose(sc[2], sc_o["ESS"], rtol=1e-5)
        assert abs(sc[3] - sc_o["H_mean"]) < 1e-5 * (1.0 + abs(sc_o["H_mean"])), (r, sc[3], sc_o["H_mean"])
        assert sc[4] == sc_o["total_num_samples"] and sc[5] == sc_o["total_phantom_samples"]
        assert sc[6] == sc_o["total_num_likelihood_evaluations"]
        np.testing.assert_allclose(sc[7], sc_o["log_efficiency"], rtol=1e-14)
    if num_phantom:
        assert unsorted > 0  # the radix-sort path ran
