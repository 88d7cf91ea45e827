"""Fitting drivers on the GPU engine: the gradient fit (Adam on the
differentiable expected-histogram chi-square, gradients from the adjoint) and
the evolutionary baseline (separable CMA-ES on the sampled Monte-Carlo
chi-square, as a parameter server drives the reference's workers).

Coordinates: z = [logit(E_s) for each state, ln k for each free rate], where
the free rates are the nonzero off-diagonals of a template parameter vector in
the reference layout (K(i,j) = rate j->i, row-major over i skipping i == j);
the other rates stay zero and V = 0.

    prob = FitProblem(engine, n, template_args)
    res = adam(prob, z0, steps=300, lr=0.05, samples=16)          # gradient fit
    res = sep_cma_es(prob, z0, sigma0=0.3, popsize=64,
                     evaluate=prob.sampled_batched, samples=10)     # evolutionary fit

Each driver records (wall seconds, best z) after every iteration, so that a
common yardstick (the expected chi-square at a fixed seed and many samples)
can place both on one time axis.
"""
import math
import time

import numpy as np

from .api import MODE_OCCUPANCY

__all__ = ["FitProblem", "FitResult", "adam", "sep_cma_es", "ParamServerEvaluator"]


def _sigmoid(x):
    return 1.0 / (1.0 + np.exp(-x))


class FitProblem:
    def __init__(self, engine, n, template_args):
        self.eng = engine
        self.n = n
        t = np.asarray(template_args, dtype=np.float64).reshape(-1)
        self.template = t
        self.free = np.nonzero(t[n:n * n] > 0.0)[0]
        self.D = n + self.free.size
        if engine is not None:
            m = engine.model
            dof = m.nbins - m.left_pad - n * (n + 1)
            if dof <= 0:
                raise ValueError(f"the reduced chi-square has {dof} degrees of freedom "
                                 f"({m.nbins} bins, left pad {m.left_pad}, {n} states): use more bins")

    # ---------------------------------------------------------------- coordinates
    def to_args(self, Z):
        Z = np.atleast_2d(np.asarray(Z, dtype=np.float64))
        n = self.n
        out = np.zeros((Z.shape[0], n * (n + 1)), dtype=np.float64)
        out[:, :n] = np.clip(_sigmoid(Z[:, :n]), 1e-6, 1.0 - 1e-6)
        out[:, n + self.free] = np.exp(Z[:, n:])
        return out.astype(np.float32)

    def from_args(self, args):
        a = np.atleast_2d(np.asarray(args, dtype=np.float64))
        n = self.n
        E = np.clip(a[:, :n], 1e-6, 1.0 - 1e-6)
        return np.concatenate([np.log(E / (1.0 - E)), np.log(a[:, n + self.free])], axis=1)

    # ---------------------------------------------------------------- objectives
    def expected(self, Z, samples, seed, grad=True):
        """Expected-histogram chi-square (P,) and its gradient in z (P, D)."""
        args = self.to_args(Z)
        if not grad:
            _, chi2 = self.eng.expected_hist(self.n, args, samples, seed)
            return chi2, None
        _, chi2, dE, dK = self.eng.expected_grad(self.n, args, samples, seed)
        E = args[:, :self.n].astype(np.float64)
        gz = np.concatenate([dE * E * (1.0 - E), dK[:, self.free]], axis=1)
        return chi2, gz

    def sampled_batched(self, Z, samples, seed):
        """Sampled Monte-Carlo chi-square of all rows in one batched launch."""
        _, chi2 = self.eng.run_batched(MODE_OCCUPANCY, self.n, self.to_args(Z), samples, seed)
        return chi2

    def sampled_plain(self, Z, samples, seed):
        """Sampled Monte-Carlo chi-square, one launch and read-back per row (the
        reference's shape: one parameter set per kernel launch)."""
        args = self.to_args(Z)
        return np.array([self.eng.run_plain(MODE_OCCUPANCY, self.n, a, samples, seed + 7919 * i)[1]
                         for i, a in enumerate(args)])


class FitResult:
    def __init__(self):
        self.times = []      # wall seconds since the start
        self.best_z = []     # best point so far (by the driver's own objective)
        self.values = []     # the driver's objective at that point
        self.evals = 0       # parameter sets evaluated

    def record(self, t, z, v):
        self.times.append(t)
        self.best_z.append(np.array(z, dtype=np.float64))
        self.values.append(float(v))

    @property
    def z(self):
        return self.best_z[-1]


def adam(prob, z0, steps, lr=0.05, samples=16, seed=1, betas=(0.9, 0.999), eps=1e-8,
         stop=None):
    """Adam on the expected chi-square; z0 is (D,) or (P, D) (P independent
    starts in one launch per step). The uniforms are fixed across steps
    (common random numbers), so the objective is deterministic. stop(t, z)
    ends the run early when it returns True."""
    Z = np.atleast_2d(np.asarray(z0, dtype=np.float64)).copy()
    m = np.zeros_like(Z)
    v = np.zeros_like(Z)
    res = FitResult()
    best_v, best_z = math.inf, Z[0].copy()
    t0 = time.perf_counter()
    for t in range(1, steps + 1):
        chi2, g = prob.expected(Z, samples, seed)
        res.evals += Z.shape[0]
        k = int(np.argmin(chi2))
        if chi2[k] < best_v:
            best_v, best_z = float(chi2[k]), Z[k].copy()
        g = np.where(np.isfinite(g), g, 0.0)
        m = betas[0] * m + (1.0 - betas[0]) * g
        v = betas[1] * v + (1.0 - betas[1]) * g * g
        mh = m / (1.0 - betas[0] ** t)
        vh = v / (1.0 - betas[1] ** t)
        Z = Z - lr * mh / (np.sqrt(vh) + eps)
        now = time.perf_counter() - t0
        res.record(now, best_z, best_v)
        if stop is not None and stop(now, best_z):
            break
    return res


def sep_cma_es(prob, z0, sigma0, popsize, evaluate, samples, seed=1, generations=100,
               stop=None, rng_seed=0):
    """Separable CMA-ES (diagonal covariance; Ros and Hansen, "A simple
    modification in CMA-ES achieving linear time and space complexity", 2008)
    with cumulative step-size adaptation. evaluate(Z, samples, seed) returns
    the chi-square of each row; every generation draws fresh Monte-Carlo
    seeds, as a parameter server does."""
    rng = np.random.default_rng(rng_seed)
    D = prob.D
    lam = popsize
    mu = lam // 2
    w = np.log(mu + 0.5) - np.log(np.arange(1, mu + 1))
    w = w / w.sum()
    mueff = 1.0 / np.sum(w * w)
    cs = (mueff + 2.0) / (D + mueff + 5.0)
    ds = 1.0 + 2.0 * max(0.0, math.sqrt((mueff - 1.0) / (D + 1.0)) - 1.0) + cs
    cc = (4.0 + mueff / D) / (D + 4.0 + 2.0 * mueff / D)
    c1 = 2.0 / ((D + 1.3) ** 2 + mueff)
    cmu = min(1.0 - c1, 2.0 * (mueff - 2.0 + 1.0 / mueff) / ((D + 2.0) ** 2 + mueff))
    # the separable variant may learn faster: scale by (D + 2) / 3
    c1s = min(1.0, c1 * (D + 2.0) / 3.0)
    cmus = min(1.0 - c1s, cmu * (D + 2.0) / 3.0)
    chiN = math.sqrt(D) * (1.0 - 1.0 / (4.0 * D) + 1.0 / (21.0 * D * D))
    mean = np.asarray(z0, dtype=np.float64).reshape(D).copy()
    sigma = float(sigma0)
    C = np.ones(D)
    ps = np.zeros(D)
    pc = np.zeros(D)
    res = FitResult()
    best_v, best_z = math.inf, mean.copy()
    t0 = time.perf_counter()
    for g in range(generations):
        Zs = rng.standard_normal((lam, D))
        Y = Zs * np.sqrt(C)
        X = mean + sigma * Y
        f = np.asarray(evaluate(X, samples, seed + 104729 * (g + 1)), dtype=np.float64)
        res.evals += lam
        f = np.where(np.isfinite(f), f, np.inf)
        order = np.argsort(f)
        if f[order[0]] < best_v:
            best_v, best_z = float(f[order[0]]), X[order[0]].copy()
        yw = w @ Y[order[:mu]]
        mean = mean + sigma * yw
        ps = (1.0 - cs) * ps + math.sqrt(cs * (2.0 - cs) * mueff) * (yw / np.sqrt(C))
        hs = np.linalg.norm(ps) / math.sqrt(1.0 - (1.0 - cs) ** (2 * (g + 1))) < (1.4 + 2.0 / (D + 1.0)) * chiN
        pc = (1.0 - cc) * pc + (math.sqrt(cc * (2.0 - cc) * mueff) * yw if hs else 0.0)
        C = ((1.0 - c1s - cmus) * C + c1s * (pc * pc + (0.0 if hs else cc * (2.0 - cc)) * C)
             + cmus * (w @ (Y[order[:mu]] ** 2)))
        sigma *= math.exp((cs / ds) * (np.linalg.norm(ps) / chiN - 1.0))
        now = time.perf_counter() - t0
        # the population mean is the ES's estimate; record it with the best draw's value
        res.record(now, mean, best_v)
        if stop is not None and stop(now, mean):
            break
    return res


class ParamServerEvaluator:
    """Evaluates a population through a parameter server
    (gsmfretda_gb300.ps.server.ParamServer) and whatever workers are attached
    to it: the distributed shape of the reference's fit."""

    def __init__(self, prob, server, timeout=600.0):
        self.prob = prob
        self.server = server
        self.timeout = timeout

    def __call__(self, Z, samples, seed):
        return self.server.evaluate(list(self.prob.to_args(Z)), timeout=self.timeout)
