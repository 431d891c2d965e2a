"""Registered likelihood families for the fused GPU path.

Each family supplies an enum (matching ``enum gbns_family`` in include/gbns.h), the
packed float32 parameter block the kernels read, and a float64 numpy reference
(``__call__``) of the same log-likelihood on X.
"""
from __future__ import annotations

import numpy as np

from .engine import FAMILY_LINGAUSS, FAMILY_MVN, FAMILY_SHELLS, mvn_offset, mvn_params, shells_offset, shells_params


class MultivariateNormalLikelihood:
    """log N(x; mu, cov) -- tfpd.MultivariateNormalTriL(mu, chol(cov)).log_prob(x)."""
    family = FAMILY_MVN

    def __init__(self, mu, cov):
        self.mu = np.asarray(mu, np.float64)
        self.cov = np.asarray(cov, np.float64)
        self.L = np.linalg.cholesky(self.cov)

    def check(self, D):
        if D != len(self.mu):
            raise ValueError(f"likelihood has dimension {len(self.mu)}, model has {D}")

    def params(self, model) -> np.ndarray:
        aff = model.affine() if model is not None else None
        if aff is None:
            return mvn_params(self.mu, self.cov)
        # a MultivariateNormalTriL prior X = A q + c folds into the likelihood's triangular
        # factor: Linv (X - mu) = (Linv A) (q - A^-1 (mu - c)), so the kernels see a correlated
        # Gaussian in q with mean A^-1 (mu - c) and factor Linv A (lower triangular)
        A, c = aff
        Linv = np.linalg.inv(self.L)
        mu_q = np.linalg.solve(A, self.mu - c)
        M = np.tril(Linv @ A)
        D = len(self.mu)
        c0 = -np.sum(np.log(np.diag(self.L))) - 0.5 * D * np.log(2.0 * np.pi)
        return np.concatenate([mu_q, M.ravel(), [c0]]).astype(np.float32)

    def log_L_offset(self) -> float:
        return mvn_offset(self.cov)

    def __call__(self, x):
        x = np.asarray(x, np.float64)
        z = np.linalg.solve(self.L, (x - self.mu).T).T
        return -0.5 * np.sum(z * z, -1) - np.sum(np.log(np.diag(self.L))) - 0.5 * len(self.mu) * np.log(2 * np.pi)


class GaussianShellsLikelihood:
    """logaddexp of two Gaussian shells: -0.5((|x-c_k| - R)/w)^2 - log sqrt(2 pi w^2)."""
    family = FAMILY_SHELLS

    def __init__(self, c1, c2, radius, width):
        self.c1 = np.asarray(c1, np.float64)
        self.c2 = np.asarray(c2, np.float64)
        self.radius = float(radius)
        self.width = float(width)

    def check(self, D):
        if D != len(self.c1) or D != len(self.c2):
            raise ValueError("shell centres must have the model's dimension")

    def params(self, model) -> np.ndarray:
        if model is not None and model.affine() is not None:
            raise NotImplementedError("MultivariateNormalTriL priors are supported with the correlated-Gaussian "
                                      "likelihood")
        return shells_params(self.c1, self.c2, self.radius, self.width)

    def log_L_offset(self) -> float:
        return shells_offset(self.width)

    def __call__(self, x):
        x = np.asarray(x, np.float64)
        norm = np.log(np.sqrt(2 * np.pi * self.width ** 2))
        s = [-0.5 * ((np.linalg.norm(x - c, axis=-1) - self.radius) / self.width) ** 2 - norm
             for c in (self.c1, self.c2)]
        return np.logaddexp(s[0], s[1])


class LinearGaussianLikelihood:
    """log N(y; Phi w, sigma^2 I) -- the linear-Gaussian (Phi w) likelihood."""
    family = FAMILY_LINGAUSS

    def __init__(self, Phi, y, sigma):
        self.Phi = np.asarray(Phi, np.float64)
        self.y = np.asarray(y, np.float64)
        self.sigma = float(sigma)

    def check(self, D):
        if D != self.Phi.shape[1]:
            raise ValueError("Phi must have one column per model dimension")

    def params(self, model) -> np.ndarray:
        if model is not None and model.affine() is not None:
            raise NotImplementedError("MultivariateNormalTriL priors are supported with the correlated-Gaussian "
                                      "likelihood")
        return np.concatenate([self.Phi.ravel(), self.y, [self.sigma]]).astype(np.float32)

    def log_L_offset(self) -> float:
        return float(-0.5 * len(self.y) * np.log(2.0 * np.pi * self.sigma ** 2))

    def __call__(self, w):
        r = self.y - np.asarray(w, np.float64) @ self.Phi.T
        N = len(self.y)
        return -0.5 * N * np.log(2 * np.pi * self.sigma ** 2) - 0.5 * np.sum(r * r, -1) / self.sigma ** 2
