"""The results' U -> X transform and prior density (Model.transform / Model.log_prob_prior,
framework/model.py:155-187, applied by _to_results at sharded_static.py:744-745).

CPU: the FP64 quantile and log of gbns_fmath.h (through the oracle, which compiles the same
header) against scipy / numpy, and the oracle's restatement of the device transform against
the model's host transform.  GPU: the prior-transform kernel bit for bit against that
restatement, and the results of a run carrying it."""
import numpy as np
import pytest

gb = pytest.importorskip("jaxns_gb300")
sp = pytest.importorskip("scipy.special")
stats = pytest.importorskip("scipy.stats")


def _mixed_model(D_tril=0, seed=0):
    """Uniform and Normal priors of several shapes, optionally a MultivariateNormalTriL block."""
    rng = np.random.default_rng(seed)
    if D_tril:
        A = rng.standard_normal((D_tril, D_tril))
        L = np.linalg.cholesky(A @ A.T / D_tril + 0.3 * np.eye(D_tril))
        loc = rng.standard_normal(D_tril)

    def prior_model():
        a = yield gb.Prior(gb.Uniform(-2.0, 3.0), name="a")
        v = yield gb.Prior(gb.Normal(np.array([0.0, 1.0, -1.0]), 2.0), name="v")
        if D_tril:
            t = yield gb.Prior(gb.MultivariateNormalTriL(loc, L), name="t")
        m = yield gb.Prior(gb.Uniform(np.zeros((2, 2)), np.ones((2, 2)) * 4.0), name="m")
        yield gb.Prior(gb.Normal(5.0, 0.5))
        return a, v, m

    D = 9 + D_tril
    return gb.Model(prior_model, gb.MultivariateNormalLikelihood(np.zeros(D), np.eye(D)))


def _oracle_args(model):
    """The prior table exactly as Model._prior_table builds it, as numpy arrays."""
    normal = model.prior_kind == gb.engine.PRIOR_NORMAL
    log_norm = -np.log(model.prior_b) - np.where(normal, 0.5 * np.log(2.0 * np.pi), 0.0)
    kw = dict(kind=model.prior_kind, a=model.prior_a, b=model.prior_b, log_norm=log_norm)
    aff = model.affine()
    if aff is not None:
        A, c = aff
        row_start = np.arange(model.U_ndims, dtype=np.int32)
        for s0, loc, L in model.tril_blocks:
            row_start[s0:s0 + len(loc)] = s0
        kw.update(A=A, c=c, row_start=row_start,
                  log_det=-float(sum(np.sum(np.log(np.diag(L))) for _, _, L in model.tril_blocks)))
    return kw


def test_ndtri64_and_log64_accuracy(oracle_mod):
    rng = np.random.default_rng(0)
    ps = np.concatenate([rng.uniform(size=4000), 10.0 ** rng.uniform(-300, -1, 1000),
                         1.0 - 10.0 ** rng.uniform(-16, -1, 1000), [0.5, 0.075, 0.925, 0.0749999, 0.425, 1e-320]])
    got = np.array([oracle_mod.fm_ndtri64(p) for p in ps])
    want = sp.ndtri(ps)
    np.testing.assert_allclose(got, want, rtol=2e-15, atol=0)
    assert oracle_mod.fm_ndtri64(0.0) == -np.inf and oracle_mod.fm_ndtri64(1.0) == np.inf
    assert oracle_mod.fm_ndtri64(0.5) == 0.0
    xs = np.concatenate([10.0 ** rng.uniform(-320, 300, 4000), rng.uniform(0.5, 2.0, 4000), [1.0, 2.0, 0.5]])
    np.testing.assert_allclose([oracle_mod.fm_log64(x) for x in xs], np.log(xs), rtol=1e-15, atol=1e-300)
    assert oracle_mod.fm_log64(1.0) == 0.0 and oracle_mod.fm_log64(0.0) == -np.inf


@pytest.mark.parametrize("D_tril", [0, 5])
def test_oracle_transform_matches_host_model(oracle_mod, D_tril):
    model = _mixed_model(D_tril)
    rng = np.random.default_rng(2)
    U = rng.random((40, model.U_ndims)).astype(np.float32)
    lL = rng.standard_normal(40)
    X, lpd = oracle_mod.prior_transform(U=U, log_L=lL, **_oracle_args(model))
    np.testing.assert_allclose(X, model.transform_flat(U.astype(np.float64)), rtol=1e-13, atol=1e-13)
    np.testing.assert_allclose(lpd, lL + model.log_prob_prior(U.astype(np.float64)), rtol=1e-13, atol=1e-12)
    U[3, 0] = 1.5                                           # outside the Uniform's support
    assert np.isneginf(oracle_mod.prior_transform(U=U, **_oracle_args(model))[1][3])


# ----------------------------------------------------------------------------- GPU

@pytest.mark.gpu
@pytest.mark.parametrize("D_tril,dtype", [(0, np.float32), (5, np.float32), (40, np.float32), (5, np.float64)])
def test_device_transform_bit_exact(gpu_lib, oracle_mod, D_tril, dtype):
    """X and the log posterior density of the kernel equal the oracle's bit for bit (D = 49
    strides the dimensions over more than one pass of the warp, the TriL block across lanes)."""
    import torch
    model = _mixed_model(D_tril, seed=D_tril)
    rng = np.random.default_rng(3)
    M = 1000
    U = rng.random((M, model.U_ndims)).astype(dtype)
    U[0, :] = 0.5
    U[1, :] = np.float32(2.0 ** -24)                       # the smallest fp32 uniform step: deep tails
    U[2, 0] = 1.5                                           # outside the Uniform's support
    lL = rng.standard_normal(M)
    X, lpd = model.transform_device(torch.tensor(U, device="cuda"), log_L=torch.tensor(lL, device="cuda"))
    Xo, lpdo = oracle_mod.prior_transform(U=U, log_L=lL, **_oracle_args(model))
    np.testing.assert_array_equal(X.cpu().numpy(), Xo)
    np.testing.assert_array_equal(lpd.cpu().numpy(), lpdo)
    assert np.isneginf(lpdo[2])
    # leading batch axes, prior density alone, and the named views
    Xb, lp = model.transform_device(torch.tensor(U[:12].reshape(3, 4, -1), device="cuda"))
    np.testing.assert_array_equal(Xb.cpu().numpy().reshape(12, -1), Xo[:12])
    np.testing.assert_array_equal(lp.cpu().numpy().reshape(12), oracle_mod.prior_transform(U=U[:12], **_oracle_args(model))[1])
    named = model.transform(torch.tensor(U[:5], device="cuda"))
    np.testing.assert_array_equal(named["m"].cpu().numpy(), Xo[:5, -5:-1].reshape(5, 2, 2))
    assert named["v"].is_cuda and named["v"].dtype == torch.float64


@pytest.mark.gpu
def test_device_transform_empty_and_refusals(gpu_lib):
    import torch
    model = _mixed_model(0)
    X, lp = model.transform_device(torch.zeros((0, model.U_ndims), device="cuda"))
    assert X.shape == (0, model.U_ndims) and lp.shape == (0,)
    with pytest.raises(ValueError):
        model.transform_device(torch.zeros((4, model.U_ndims + 1), device="cuda"))
    with pytest.raises(gb._ffi.GBNSError):
        model.transform_device(torch.zeros((4, model.U_ndims)))  # a host tensor never reaches the kernel


@pytest.mark.gpu
def test_results_samples_and_posterior_density(gpu_lib):
    """A run's samples and log posterior density come from the kernel and equal the host
    transform of its U samples (sharded_static.py:744-745)."""
    import torch
    D = 4

    def prior_model():
        x = yield gb.Prior(gb.Uniform(-3.0 * np.ones(2), 3.0 * np.ones(2)), name="x")
        y = yield gb.Prior(gb.Normal(np.zeros(2), 1.5), name="y")
        return x, y

    model = gb.Model(prior_model, gb.MultivariateNormalLikelihood(np.zeros(D), np.eye(D)))
    ns = gb.NestedSampler(model, num_live_points=100)
    term, state = ns(gb.random.PRNGKey(7))
    res = ns.to_results(term, state)
    U = res.U_samples.double().cpu().numpy()
    X_host = model.transform_flat(U)
    np.testing.assert_allclose(res.samples["x"].cpu().numpy(), X_host[:, :2], rtol=1e-13, atol=1e-13)
    np.testing.assert_allclose(res.samples["y"].cpu().numpy(), X_host[:, 2:], rtol=1e-13, atol=1e-13)
    want = res.log_L_samples.cpu().numpy() + model.log_prob_prior(U)
    np.testing.assert_allclose(res.log_posterior_density.cpu().numpy(), want, rtol=1e-13, atol=1e-11)
    assert res.samples["x"].is_cuda and isinstance(res.log_posterior_density, torch.Tensor)
