"""The differentiable expected-histogram chi-square as a torch.autograd.Function
(parameter-server side of the gradient path).

    chi2 = expected_chi2(E, logK, engine, samples=64, seed=1)   # (P,)
    chi2.sum().backward()                                        # E.grad, logK.grad

E is (P, n) and logK (P, n(n-1)) in the reference's off-diagonal order
(K(i,j) = rate j->i, row-major over i skipping i == j); V = 0. The forward is
gpda_expected_hist, the backward gpda_expected_hist_adjoint on the same
engine, both on the GPU; the tensors themselves are tiny and live on the host.
With `anchor` (a (P, n(n+1)) parameter array) the state skeleton is drawn
under the anchor and weighted by the likelihood ratio, which makes chi2 a
smooth function of (E, logK) around the anchor for finite differences.
"""
import numpy as np
import torch

__all__ = ["ExpectedChi2", "expected_chi2", "pack", "unpack"]


def pack(E, logK):
    """(P, n), (P, n(n-1)) -> (P, n(n+1)) float32 parameter vectors, V = 0."""
    E = np.atleast_2d(np.asarray(E, dtype=np.float64))
    lk = np.atleast_2d(np.asarray(logK, dtype=np.float64))
    P, n = E.shape
    if lk.shape != (P, n * (n - 1)):
        raise ValueError("logK must be (P, n(n-1))")
    out = np.zeros((P, n * (n + 1)), dtype=np.float64)
    out[:, :n] = E
    out[:, n:n * n] = np.exp(lk)
    return out.astype(np.float32)


def unpack(args, n):
    """(P, n(n+1)) parameter vectors -> E (P, n), logK (P, n(n-1))."""
    a = np.atleast_2d(np.asarray(args, dtype=np.float64))
    return a[:, :n].copy(), np.log(a[:, n:n * n])


class ExpectedChi2(torch.autograd.Function):
    @staticmethod
    def forward(ctx, E, logK, engine, samples, seed, anchor):
        n = E.shape[-1]
        args = pack(E.detach().cpu().numpy(), logK.detach().cpu().numpy())
        _, chi2 = engine.expected_hist(n, args, samples, seed, anchor=anchor)
        ctx.engine, ctx.args, ctx.anchor = engine, args, anchor
        ctx.samples, ctx.seed, ctx.n = samples, seed, n
        ctx.shape_E, ctx.shape_K = E.shape, logK.shape
        return torch.as_tensor(chi2, dtype=E.dtype, device=E.device).reshape(E.shape[:-1])

    @staticmethod
    def backward(ctx, grad_out):
        up = grad_out.detach().cpu().double().numpy().reshape(-1)
        dE, dK = ctx.engine.expected_adjoint(ctx.n, ctx.args, ctx.samples, ctx.seed,
                                             anchor=ctx.anchor, dchi2=up)
        gE = torch.as_tensor(dE, dtype=grad_out.dtype, device=grad_out.device).reshape(ctx.shape_E)
        gK = torch.as_tensor(dK, dtype=grad_out.dtype, device=grad_out.device).reshape(ctx.shape_K)
        return gE, gK, None, None, None, None


def expected_chi2(E, logK, engine, samples=64, seed=1, anchor=None):
    """Reduced chi-square of the expected histogram for each parameter set;
    differentiable in E and logK."""
    squeeze = E.dim() == 1
    if squeeze:
        E, logK = E.unsqueeze(0), logK.unsqueeze(0)
    out = ExpectedChi2.apply(E, logK, engine, samples, seed, anchor)
    return out[0] if squeeze else out
