"""Modelling front end: ``Prior`` / ``Model`` with jaxns's generator-based prior syntax
(framework/model.py:24-41, framework/prior.py:65, framework/ops.py:89-326).

A fused CUDA likelihood cannot be an arbitrary Python callable, so ``log_likelihood`` is
one of the registered likelihood families of :mod:`jaxns_gb300.likelihoods`; priors are
Uniform or Normal quantile transforms per U dimension, or a MultivariateNormalTriL block (the
standard normal quantile per dimension followed by the affine bijector loc + L z), as jaxns
applies them through WrappedTFPDistribution._forward (framework/wrapped_tfp_distribution.py:77-84).
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Callable, List, Optional, Sequence

import numpy as np

from .engine import PRIOR_NORMAL, PRIOR_UNIFORM


class InvalidPriorName(Exception):
    def __init__(self, name: Optional[str] = None):
        super().__init__(f'Prior name {name} already taken by another prior.')


class Uniform:
    """Uniform(low, high) distribution (quantile: low + (high - low) * u)."""

    def __init__(self, low, high):
        self.low = np.asarray(low, np.float64)
        self.high = np.asarray(high, np.float64)
        self.shape = np.broadcast(self.low, self.high).shape

    def table(self):
        size = int(np.prod(self.shape)) if self.shape else 1
        a = np.broadcast_to(self.low, self.shape).ravel() if self.shape else np.array([float(self.low)])
        b = (np.broadcast_to(self.high, self.shape).ravel() - a) if self.shape else \
            np.array([float(self.high) - float(self.low)])
        return np.full(size, PRIOR_UNIFORM, np.int32), a, b


class Normal:
    """Normal(loc, scale) distribution (quantile: loc + scale * ndtri(u))."""

    def __init__(self, loc, scale):
        self.loc = np.asarray(loc, np.float64)
        self.scale = np.asarray(scale, np.float64)
        self.shape = np.broadcast(self.loc, self.scale).shape

    def table(self):
        size = int(np.prod(self.shape)) if self.shape else 1
        a = np.broadcast_to(self.loc, self.shape).ravel() if self.shape else np.array([float(self.loc)])
        b = np.broadcast_to(self.scale, self.shape).ravel() if self.shape else np.array([float(self.scale)])
        return np.full(size, PRIOR_NORMAL, np.int32), a, b


class MultivariateNormalTriL:
    """MultivariateNormalTriL(loc, scale_tril): a D-dimensional Gaussian prior block.  Its U->X
    map is the reference's: the base distribution's quantile per dimension (standard normal,
    z = ndtri(u)) followed by the bijector X = loc + L z (tfp's MultivariateNormalTriL is a
    transformed Sample(Normal(0, 1), D))."""

    def __init__(self, loc, scale_tril):
        self.loc = np.asarray(loc, np.float64).reshape(-1)
        L = np.asarray(scale_tril, np.float64)
        D = self.loc.shape[0]
        if L.shape != (D, D):
            raise ValueError(f"scale_tril must be [{D}, {D}], got {L.shape}")
        if not np.all(np.diag(L) > 0):
            raise ValueError("scale_tril must have a positive diagonal")
        self.scale_tril = np.tril(L)
        self.shape = (D,)

    def table(self):
        D = self.shape[0]
        return np.full(D, PRIOR_NORMAL, np.int32), np.zeros(D), np.ones(D)


class Prior:
    """A named prior over a block of U dimensions (framework/prior.py:65)."""

    def __init__(self, dist_or_value, name: Optional[str] = None):
        if not isinstance(dist_or_value, (Uniform, Normal, MultivariateNormalTriL)):
            raise ValueError("Prior supports Uniform, Normal and MultivariateNormalTriL distributions on the fused "
                             "GPU path")
        self.dist = dist_or_value
        self.name = name

    @property
    def base_shape(self):
        return self.dist.shape

    @property
    def size(self) -> int:
        return int(np.prod(self.dist.shape)) if self.dist.shape else 1


@dataclass
class _ParsedPrior:
    name: str
    shape: tuple
    start: int
    size: int


class Model:
    """Model(prior_model, log_likelihood) (framework/model.py:24)."""

    def __init__(self, prior_model: Callable, log_likelihood, params=None):
        self.prior_model = prior_model
        self.log_likelihood = log_likelihood
        self._params = params
        priors: List[_ParsedPrior] = []
        kinds, a_s, b_s = [], [], []
        tril_blocks = []
        gen = prior_model()
        names = set()
        start = 0
        try:
            p = next(gen)
            while True:
                if not isinstance(p, Prior):
                    raise ValueError("prior_model must yield Prior objects")
                name = p.name or f"__prior_{len(priors)}"
                if name in names:
                    raise InvalidPriorName(name)
                names.add(name)
                k, a, b = p.dist.table()
                priors.append(_ParsedPrior(name, p.dist.shape, start, p.size))
                if isinstance(p.dist, MultivariateNormalTriL):
                    tril_blocks.append((start, p.dist.loc, p.dist.scale_tril))
                kinds.append(k)
                a_s.append(a)
                b_s.append(b)
                start += p.size
                p = gen.send(np.zeros(p.dist.shape))
        except StopIteration:
            pass
        self.priors = priors
        self.tril_blocks = tril_blocks  # (first dimension, loc, L) of every MultivariateNormalTriL block
        self.U_ndims = start
        self.prior_kind = np.concatenate(kinds) if kinds else np.zeros(0, np.int32)
        self.prior_a = np.concatenate(a_s) if a_s else np.zeros(0)
        self.prior_b = np.concatenate(b_s) if b_s else np.zeros(0)
        if self.U_ndims < 1:
            raise ValueError("model has no sampled dimensions")
        log_likelihood.check(self.U_ndims)

    def __call__(self, params):
        return Model(self.prior_model, self.log_likelihood, params=params)

    def transform(self, U):
        """U -> X (dict of prior name -> value), vectorised over leading axes."""
        return self.unflatten(self.transform_flat(U))

    def unflatten(self, X):
        """The named priors' views of a flat X [..., D]."""
        return {p.name: X[..., p.start:p.start + p.size].reshape(X.shape[:-1] + tuple(p.shape))
                for p in self.priors if not p.name.startswith("__prior_")}

    def _quantiles(self, Ut):
        """Per-dimension quantile outputs q (X for Uniform / Normal dimensions, the standard
        normal z of MultivariateNormalTriL dimensions) and X."""
        import torch
        a = torch.as_tensor(self.prior_a, dtype=Ut.dtype, device=Ut.device)
        b = torch.as_tensor(self.prior_b, dtype=Ut.dtype, device=Ut.device)
        normal = torch.as_tensor(self.prior_kind == PRIOR_NORMAL, device=Ut.device)
        q = a + b * torch.where(normal, np.sqrt(2.0) * torch.erfinv(2.0 * Ut - 1.0), Ut)
        X = q
        if self.tril_blocks:
            X = q.clone()
            for s0, loc, L in self.tril_blocks:
                D = len(loc)
                Lt = torch.as_tensor(L, dtype=Ut.dtype, device=Ut.device)
                X[..., s0:s0 + D] = torch.as_tensor(loc, dtype=Ut.dtype, device=Ut.device) + q[..., s0:s0 + D] @ Lt.T
        return q, X

    def transform_flat(self, U):
        import torch
        if isinstance(U, torch.Tensor) and U.is_cuda:
            return self.transform_device(U)[0]
        is_t = isinstance(U, torch.Tensor)
        Ut = U if is_t else torch.as_tensor(np.asarray(U, np.float64))
        X = self._quantiles(Ut)[1]
        return X if is_t else X.numpy()

    def _prior_table(self, device):
        """The per-dimension prior table of gbns_prior_transform, as device tensors (cached)."""
        import torch
        cache = getattr(self, "_table_cache", None)
        if cache is not None and cache[0] == device:
            return cache[1]
        D = self.U_ndims
        normal = self.prior_kind == PRIOR_NORMAL
        log_norm = -np.log(self.prior_b) - np.where(normal, 0.5 * np.log(2.0 * np.pi), 0.0)
        t = {"kind": torch.as_tensor(self.prior_kind.astype(np.int32), device=device),
             "a": torch.as_tensor(self.prior_a, dtype=torch.float64, device=device),
             "b": torch.as_tensor(self.prior_b, dtype=torch.float64, device=device),
             "log_norm": torch.as_tensor(log_norm, dtype=torch.float64, device=device),
             "log_det": 0.0}
        aff = self.affine()
        if aff is not None:
            A, c = aff
            row_start = np.arange(D, dtype=np.int32)
            for s0, loc, L in self.tril_blocks:
                row_start[s0:s0 + len(loc)] = s0
            t.update(A=torch.as_tensor(A, dtype=torch.float64, device=device),
                     c=torch.as_tensor(c, dtype=torch.float64, device=device),
                     row_start=torch.as_tensor(row_start, device=device),
                     log_det=-float(sum(np.sum(np.log(np.diag(L))) for _, _, L in self.tril_blocks)))
        self._table_cache = (device, t)
        return t

    def transform_device(self, U, log_L=None, with_X: bool = True):
        """(X, log density) of the rows of a CUDA tensor U [..., D] (fp32, or FP64 for the
        linear-Gaussian family) by the prior-transform kernel: X FP64 [..., D] (None unless
        with_X) and log L + log p(X) (log_L given) or log p(X), FP64 [...]."""
        import ctypes
        import torch
        from . import _ffi
        _ffi.require_cuda("Model.transform_device", U=U)
        D = self.U_ndims
        if U.shape[-1] != D:
            raise ValueError(f"U has {U.shape[-1]} columns, the model {D} dimensions")
        if U.dtype not in (torch.float32, torch.float64):
            raise ValueError(f"U must be float32 or float64, not {U.dtype}")
        lead = tuple(U.shape[:-1])
        Uc = U.reshape(-1, D).contiguous()
        M = Uc.shape[0]
        t = self._prior_table(U.device)
        X = torch.empty((M, D), dtype=torch.float64, device=U.device) if with_X else None
        out = torch.empty(M, dtype=torch.float64, device=U.device)
        lL = None
        if log_L is not None:
            _ffi.require_cuda("Model.transform_device", log_L=log_L)
            lL = log_L.reshape(-1).to(torch.float64).contiguous()
            if lL.numel() != M:
                raise ValueError(f"log_L has {lL.numel()} entries for {M} rows")
        p = lambda x: ctypes.c_void_p(x.data_ptr() if x is not None else 0)
        tab = _ffi.PriorTable(D=D, kind=t["kind"].data_ptr(), a=t["a"].data_ptr(), b=t["b"].data_ptr(),
                              log_norm=t["log_norm"].data_ptr(), A=t["A"].data_ptr() if "A" in t else None,
                              row_start=t["row_start"].data_ptr() if "A" in t else None,
                              c=t["c"].data_ptr() if "A" in t else None, log_det=t["log_det"])
        f32 = Uc.dtype == torch.float32
        stream = ctypes.c_void_p(torch.cuda.current_stream(U.device).cuda_stream)
        _ffi.call("gbns_prior_transform", ctypes.byref(tab), p(Uc if f32 else None), p(None if f32 else Uc),
                  ctypes.c_longlong(M), p(lL), p(X), p(out), stream)
        return (X.view(lead + (D,)) if X is not None else None), out.view(lead)

    def log_prob_prior(self, U):
        """log prior density of the X that U maps to (per sample); a tensor for a tensor U, a
        numpy array otherwise."""
        import torch
        if isinstance(U, torch.Tensor) and U.is_cuda:
            return self.transform_device(U, with_X=False)[1]
        is_t = isinstance(U, torch.Tensor)
        Ut = U if is_t else torch.as_tensor(np.asarray(U, np.float64))
        q, X = self._quantiles(Ut)
        a = torch.as_tensor(self.prior_a, dtype=X.dtype, device=X.device)
        b = torch.as_tensor(self.prior_b, dtype=X.dtype, device=X.device)
        normal = torch.as_tensor(self.prior_kind == PRIOR_NORMAL, device=X.device)
        inside = (q >= a) & (q <= a + b)
        lp_u = torch.where(inside, -torch.log(b), torch.full_like(q, -float("inf")))
        lp_n = -0.5 * ((q - a) / b) ** 2 - torch.log(b) - 0.5 * np.log(2.0 * np.pi)
        lp = torch.where(normal, lp_n, lp_u).sum(-1)
        # a MultivariateNormalTriL block: log N(X; loc, L L^T) = sum over its z of the standard
        # normal density - sum log L_ii
        for s0, loc, L in self.tril_blocks:
            lp = lp - float(np.sum(np.log(np.diag(L))))
        return lp if is_t else lp.numpy()

    def affine(self):
        """(A, c) with X = A q + c over all dimensions (A lower triangular: identity except the
        MultivariateNormalTriL blocks), or None when the model has no such block."""
        if not self.tril_blocks:
            return None
        D = self.U_ndims
        A, c = np.eye(D), np.zeros(D)
        for s0, loc, L in self.tril_blocks:
            k = len(loc)
            A[s0:s0 + k, s0:s0 + k] = L
            c[s0:s0 + k] = loc
        return A, c

    @property
    def U_placeholder(self):
        return np.zeros(self.U_ndims)

    def family_params(self) -> np.ndarray:
        return self.log_likelihood.params(self)

    @property
    def family(self) -> int:
        return self.log_likelihood.family
