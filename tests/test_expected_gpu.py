"""GPU parity of the differentiable expected histogram: gpda_expected_hist and
gpda_expected_hist_adjoint against the FP64 oracle (same skeleton and
background draws), against common-random-number central differences of the
device forward (h = 1e-4), and through the torch.autograd.Function.

Tolerances: normalised bin masses within 1e-5 absolute (device masses are
FP32 with the Loader/recurrence evaluation, the oracle's exact FP64); reduced
chi-square within 1e-5 relative; gradients within 1e-3 relative, component
by component, for every component above a floor of 1e-3 of the largest (a
component below the floor is held to 1e-3 of the largest instead), and
within 1e-3 of the largest component as a second bar."""

GRAD_RTOL = 1e-3      # per component, relative to the reference value
GRAD_FLOOR = 1e-3     # components below GRAD_FLOOR * max |reference| are compared absolutely


def _assert_grad_close(g, ref, what):
    """|g_k - ref_k| <= GRAD_RTOL |ref_k| for |ref_k| >= GRAD_FLOOR max|ref|,
    and |g_k - ref_k| <= GRAD_RTOL max|ref| for every k."""
    g = np.asarray(g, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    scale = np.abs(ref).max()
    err = np.abs(g - ref)
    big = np.abs(ref) >= GRAD_FLOOR * scale
    rel = np.where(big, err / np.maximum(np.abs(ref), 1e-300), 0.0)
    assert np.all(rel <= GRAD_RTOL), f"{what}: per-component relative error {rel} (g={g}, ref={ref})"
    assert err.max() <= GRAD_RTOL * scale, f"{what}: error {err} vs scale {scale}"
import numpy as np
import pytest

from gsmfretda_gb300 import synth
from gsmfretda_gb300.api import Engine

pytestmark = pytest.mark.gpu


def _vec(args, n):
    a = np.asarray(args, dtype=np.float64).reshape(-1)
    return np.concatenate([a[:n], np.log(a[n:n * n])])


def _args(v, n, base):
    a = np.array(base, dtype=np.float64).reshape(-1).copy()
    a[:n] = v[:n]
    a[n:n * n] = np.exp(v[n:])
    return a.astype(np.float32)


def _setup(orc, n, B):
    bs, n, truth, md, S = synth.expected_bursts(B=B, n=n, seed=4)
    m = orc.model(**md)
    h_obs, _ = orc.run_pda(bs.N, bs.T, n, truth, m, 0, 1, 999)
    return bs, n, truth, md, m, h_obs[0].astype(np.float32), S


@pytest.mark.parametrize("n", [2, 3])
def test_forward_and_adjoint_match_the_oracle(orc, gpda_lib, n):
    bs, n, truth, md, m, obs, S = _setup(orc, n, B=2000)
    th = synth.perturb_args(truth, n, seed=1)
    Ho, co, eo, ko = orc.expected(bs.N, bs.T, n, th, m, S, 21, obs)
    with Engine(0, **md) as eng:
        eng.upload(bs)
        eng.set_observed(obs)
        H, c = eng.expected_hist(n, th, S, 21)
        dE, dK = eng.expected_adjoint(n, th, S, 21)
        H2, c2, dE2, dK2 = eng.expected_grad(n, th, S, 21)
    units = Ho.sum()
    assert np.abs(H - Ho).max() / units < 1e-5
    assert abs(c[0] - co[0]) <= 1e-5 * abs(co[0])
    g, go = np.concatenate([dE[0], dK[0]]), np.concatenate([eo[0], ko[0]])
    _assert_grad_close(g, go, "adjoint vs FP64 oracle")
    # the fused call gives the same numbers (same kernels, fixed summation order)
    np.testing.assert_array_equal(H2, H)
    np.testing.assert_array_equal(c2, c)
    np.testing.assert_array_equal(np.concatenate([dE2[0], dK2[0]]), g)


def test_full_size_gradient_vs_oracle_and_central_differences(orc, gpda_lib):
    """20,000 bursts, 64 dwell samples, 3 states: the device adjoint against
    the FP64 host gradient and against central differences (h = 1e-4) of the
    device forward with the skeleton held at the evaluation point."""
    bs, n, truth, md, m, obs, S = _setup(orc, 3, B=20000)
    th = synth.perturb_args(truth, n, seed=3)
    _, co, eo, ko = orc.expected(bs.N, bs.T, n, th, m, S, 5, obs)
    go = np.concatenate([eo[0], ko[0]])
    h = 1e-4
    with Engine(0, **md) as eng:
        eng.upload(bs)
        eng.set_observed(obs)
        _, c, dE, dK = eng.expected_grad(n, th, S, 5)
        g = np.concatenate([dE[0], dK[0]])
        v0 = _vec(th, n)
        fd = np.zeros_like(g)
        for k in range(v0.size):
            ap = _args(v0 + h * np.eye(v0.size)[k], n, th)
            am = _args(v0 - h * np.eye(v0.size)[k], n, th)
            step = (_vec(ap, n) - _vec(am, n))[k]
            _, cp = eng.expected_hist(n, ap, S, 5, anchor=th)
            _, cm = eng.expected_hist(n, am, S, 5, anchor=th)
            fd[k] = (cp[0] - cm[0]) / step
    assert abs(c[0] - co[0]) <= 1e-5 * abs(co[0])
    _assert_grad_close(g, go, "adjoint vs FP64 oracle")
    _assert_grad_close(g, fd, "adjoint vs central differences")


def test_population_batch_matches_the_oracle(orc, gpda_lib):
    bs, n, truth, md, m, obs, S = _setup(orc, 2, B=1500)
    P = 5
    args = np.stack([synth.perturb_args(truth, n, seed=10 + p) for p in range(P)])
    Ho, co, eo, ko = orc.expected(bs.N, bs.T, n, args, m, 16, 8, obs)
    with Engine(0, **md) as eng:
        eng.upload(bs)
        eng.set_observed(obs)
        H, c, dE, dK = eng.expected_grad(n, args, 16, 8)
    assert np.abs(H - Ho).max() / Ho[0].sum() < 1e-5
    np.testing.assert_allclose(c, co, rtol=1e-5)
    g, go = np.concatenate([dE, dK], 1), np.concatenate([eo, ko], 1)
    for p in range(P):
        _assert_grad_close(g[p], go[p], f"set {p}: adjoint vs FP64 oracle")


def test_autograd_function(orc, gpda_lib):
    torch = pytest.importorskip("torch")
    from gsmfretda_gb300.expected import expected_chi2, unpack
    bs, n, truth, md, m, obs, S = _setup(orc, 3, B=1000)
    th = synth.perturb_args(truth, n, seed=4)
    E0, K0 = unpack(th, n)
    with Engine(0, **md) as eng:
        eng.upload(bs)
        eng.set_observed(obs)
        E = torch.tensor(E0[0], dtype=torch.float64, requires_grad=True)
        lk = torch.tensor(K0[0], dtype=torch.float64, requires_grad=True)
        chi = expected_chi2(E, lk, eng, samples=S, seed=2)
        (3.0 * chi).backward()
        _, c, dE, dK = eng.expected_grad(n, th, S, 2)
    assert float(chi.detach()) == c[0]
    np.testing.assert_allclose(E.grad.numpy(), 3.0 * dE[0], rtol=1e-12)
    np.testing.assert_allclose(lk.grad.numpy(), 3.0 * dK[0], rtol=1e-12)


def test_limits_and_invalid_parameters(gpda_lib):
    from gsmfretda_gb300._lib import GpdaError
    bs, n, truth, md, S = synth.expected_bursts(B=100, n=2, seed=4)
    with Engine(0, **md) as eng:
        eng.upload(bs)
        with pytest.raises(GpdaError):               # no observed histogram yet
            eng.expected_hist(n, truth, 4, 1)
        eng.set_observed(np.ones(md["nbins"], dtype=np.float32))
        a = np.array(truth, dtype=np.float32).copy()
        a[n * n] = 0.5                               # distance broadening: not in this form
        with pytest.raises(GpdaError):
            eng.expected_hist(n, a, 4, 1)
        with pytest.raises(GpdaError):               # more than 4 states
            eng.expected_hist(5, np.full(30, 100.0, dtype=np.float32), 4, 1)


def test_mass_tape_and_recompute_agree(orc, gpda_lib):
    """The adjoint reads the forward's mass tape, or walks the binomial again
    when the tape is turned off: the same gradient up to FP32 summation order."""
    bs, n, truth, md, m, obs, S = _setup(orc, 3, B=3000)
    th = synth.perturb_args(truth, n, seed=6)
    with Engine(0, **md) as eng:
        eng.upload(bs)
        eng.set_observed(obs)
        H1, c1, e1, k1 = eng.expected_grad(n, th, S, 4)          # with the tape
        eng.expected_tape_limit(0)
        H0, c0, e0, k0 = eng.expected_grad(n, th, S, 4)          # recomputed
    # (the two forwards differ only in grid size, hence in summation order)
    np.testing.assert_allclose(H1, H0, rtol=1e-7)
    np.testing.assert_allclose(c1, c0, rtol=1e-7)
    g1, g0 = np.concatenate([e1[0], k1[0]]), np.concatenate([e0[0], k0[0]])
    assert np.abs(g1 - g0).max() <= 1e-5 * np.abs(g0).max()
