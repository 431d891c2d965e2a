"""Evidence gradient of the linear-Gaussian model by reweighting a fixed dead-point set.

EvidenceMaximisation (experimental/evidence_maximisation.py:151-160, weights :213) fixes the
dead points U_i of one nested-sampling run and maximises
    log Z(theta) = logsumexp_i(log L_theta(U_i) + log w_i),
    log w_i = log_dp_mean_i - log L_i + log Z_mean,
over the hyperparameters theta = (log tau, log sigma) of y ~ N(Phi w, sigma^2 I),
w = tau * ndtri(U).  gbns_evidence_adjoint returns log Z(theta) and its exact gradient
sum_i softmax_i * d log L_theta(U_i) / d theta, recomputing each point's residual from U.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _ffi


@dataclass
class DeadSet:
    """The fixed dead points of one run (device tensors)."""
    U: torch.Tensor        # [M, P] float64 (U space)
    log_w: torch.Tensor    # [M] float64
    Phi: torch.Tensor      # [N, P] float32
    y: torch.Tensor        # [N] float32

    @staticmethod
    def from_results(results, Phi, y) -> "DeadSet":
        log_w = (results.log_dp_mean - results.log_L_samples + results.log_Z_mean).contiguous()
        dev = results.U_samples.device
        return DeadSet(U=results.U_samples.to(torch.float64).contiguous(), log_w=log_w.to(torch.float64),
                       Phi=torch.as_tensor(np.asarray(Phi, np.float32), device=dev).contiguous(),
                       y=torch.as_tensor(np.asarray(y, np.float32), device=dev).contiguous())


def evidence_and_grad(ds: DeadSet, log_tau: float, log_sigma: float, tensor_cores: bool = True,
                      check: bool = True):
    """(log Z(theta), d log Z / d log tau, d log Z / d log sigma) on the device, FP64.
    tensor_cores: the per-point residuals |y - Phi w|^2 as a 3xTF32 tcgen05 GEMM
    (gbns_evidence_adjoint_tc) instead of fp32 CUDA-core tiles (gbns_evidence_adjoint).
    check: synchronise and raise if a tensor-core wait timed out."""
    _ffi.require_cuda("evidence_and_grad", U=ds.U, log_w=ds.log_w, Phi=ds.Phi, y=ds.y)
    M, P = ds.U.shape
    N = ds.Phi.shape[0]
    dev = ds.U.device
    out = torch.zeros(3, dtype=torch.float64, device=dev)
    ss = torch.empty(max(M, 1), dtype=torch.float64, device=dev)
    ry = torch.empty(max(M, 1), dtype=torch.float64, device=dev)
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    args = [p(ds.U), p(ds.log_w), ctypes.c_longlong(M), ctypes.c_int(P), p(ds.Phi), p(ds.y), ctypes.c_int(N),
            ctypes.c_double(float(log_tau)), ctypes.c_double(float(log_sigma)), p(out), p(ss), p(ry)]
    if not tensor_cores:
        _ffi.call("gbns_evidence_adjoint", *args, stream)
        return out
    ld = 32 if P <= 32 else 64
    ws = torch.empty(max(2 * M * ld, 1), dtype=torch.float32, device=dev)
    ps = torch.empty(2 * N * ld, dtype=torch.float32, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    _ffi.call("gbns_evidence_adjoint_tc", *args, p(ws), p(ps), p(status), stream)
    if check and int(status.item()) != 0:
        raise _ffi.GBNSError(f"gbns_evidence_adjoint_tc: device status {int(status.item())} (wait timed out)")
    return out


def batch_evidence_and_grad(batch, results, thetas, tensor_cores: bool = True, check: bool = True):
    """Reweighted evidence and gradient of every linear-Gaussian run of an NSBatch from one
    device results pass (NSBatch.results(with_U=True)); thetas: [R, 2] (log tau, log sigma).
    Phi and y are read in place from the batch's parameter buffer.  Returns [R, 3] FP64 on
    the device: log Z(theta), d/d log tau, d/d log sigma."""
    if batch.device.type != "cuda":
        raise _ffi.GBNSError(f"batch_evidence_and_grad: the batch is on {batch.device} (there is no CPU path)")
    st = batch.state()
    R = batch.R
    dev = batch.device
    out = torch.zeros(R, 3, dtype=torch.float64, device=dev)
    sizes = []
    for r, s in enumerate(batch.specs):
        sizes.append((int(min(st["num_samples"][r], s.max_samples)), s.D, s.N))
    Mmax = max(m for m, _, _ in sizes)
    Nmax = max(n for _, _, n in sizes)
    ss = torch.empty(max(Mmax, 1), dtype=torch.float64, device=dev)
    ry = torch.empty(max(Mmax, 1), dtype=torch.float64, device=dev)
    ws = torch.empty(max(2 * Mmax * 64, 1), dtype=torch.float32, device=dev)
    ps = torch.empty(2 * Nmax * 64, dtype=torch.float32, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    log_Z = results["scalars"][:, 0]
    log_w_all = results["log_dp_mean"] - results["log_L_samples"]
    thetas = np.asarray(thetas, np.float64).reshape(R, 2)
    for r, s in enumerate(batch.specs):
        M, P, N = sizes[r]
        o = int(batch.offsets["store"][r])
        uo = int(batch.offsets["ustore"][r])
        if uo < 0:
            raise ValueError("the batch was built without a U store (store_U=False)")
        log_w = (log_w_all[o:o + M] + log_Z[r]).contiguous()
        U = results["U_sorted"][uo:uo + 2 * M * P]  # FP64 U as pairs of 32-bit words
        po = int(batch.offsets["param"][r])
        Phi = batch.fparams[po:po + N * P]
        y = batch.fparams[po + N * P:po + N * P + N]
        args = [p(U), p(log_w), ctypes.c_longlong(M), ctypes.c_int(P), p(Phi), p(y), ctypes.c_int(N),
                ctypes.c_double(thetas[r, 0]), ctypes.c_double(thetas[r, 1]), p(out[r]), p(ss), p(ry)]
        if tensor_cores:
            _ffi.call("gbns_evidence_adjoint_tc", *args, p(ws), p(ps), p(status), stream)
        else:
            _ffi.call("gbns_evidence_adjoint", *args, stream)
        batch.kernel_launches += 5 if tensor_cores else 2
    if check and tensor_cores and int(status.item()) != 0:
        raise _ffi.GBNSError(f"gbns_evidence_adjoint_tc: device status {int(status.item())} (wait timed out)")
    return out


class EvidenceFn(torch.autograd.Function):
    """log Z(theta) of a fixed dead set as a differentiable function of theta = (log tau, log sigma).
    The backward pass recomputes the per-point likelihood gradients (nothing per point is
    stored by the forward pass)."""

    @staticmethod
    def forward(ctx, theta: torch.Tensor, ds: DeadSet):
        th = theta.detach().to(torch.float64).cpu().numpy()
        out = evidence_and_grad(ds, th[0], th[1])
        ctx.ds = ds
        ctx.save_for_backward(theta)
        return out[0].to(device=theta.device, dtype=theta.dtype)

    @staticmethod
    def backward(ctx, grad_out):
        (theta,) = ctx.saved_tensors
        th = theta.detach().to(torch.float64).cpu().numpy()
        out = evidence_and_grad(ctx.ds, th[0], th[1])
        g = out[1:].to(device=theta.device, dtype=theta.dtype)
        return grad_out.to(theta.device) * g, None


def blr_log_evidence(Phi, y, log_tau, log_sigma):
    """Analytic log N(y; 0, sigma^2 I + tau^2 Phi Phi^T) and its gradient in (log tau, log sigma),
    FP64 (Woodbury / matrix-determinant lemma)."""
    Phi = np.asarray(Phi, np.float64)
    y = np.asarray(y, np.float64)
    N, P = Phi.shape
    t2, s2 = np.exp(2 * log_tau), np.exp(2 * log_sigma)
    A = np.eye(P) / t2 + Phi.T @ Phi / s2           # P x P
    L = np.linalg.cholesky(A)
    Pty = Phi.T @ y
    b = np.linalg.solve(A, Pty)
    alpha = y / s2 - Phi @ b / s2 ** 2                # C^{-1} y
    logdetC = N * np.log(s2) + P * np.log(t2) + 2 * np.sum(np.log(np.diag(L)))
    logZ = -0.5 * (N * np.log(2 * np.pi) + logdetC + y @ alpha)
    # d/dtheta: 0.5 (alpha^T dC alpha - tr(C^{-1} dC));  dC/dlog sigma = 2 s2 I, dC/dlog tau = 2 t2 Phi Phi^T
    Ainv = np.linalg.inv(A)
    trCinv = N / s2 - np.trace(Ainv @ (Phi.T @ Phi)) / s2 ** 2
    PtP = Phi.T @ Phi
    trCinvPP = np.trace(PtP) / s2 - np.trace(Ainv @ PtP @ PtP) / s2 ** 2
    Pa = Phi.T @ alpha
    g_sigma = 0.5 * (2 * s2 * (alpha @ alpha) - 2 * s2 * trCinv)
    g_tau = 0.5 * (2 * t2 * (Pa @ Pa) - 2 * t2 * trCinvPP)
    return logZ, np.array([g_tau, g_sigma])
