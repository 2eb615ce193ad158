"""Calibration callers of the pricing path (src/calibration.rs,
src/optimizer.rs): fit_gbm_volatility (damped Gauss-Newton on sigma),
fit_heston_parameters (trust-region gradient descent), calibrate_heston_cmaes
(CMA-ES in the normalised box [0, 1]^5) and the optimizer cmaes_minimize.

The optimizers are host logic, restated step for step. Their Monte-Carlo
work is what runs on the GPU: every price an iteration needs — each quote
at sigma and sigma + delta, the six parameter vectors of a gradient step, the
whole population of a CMA-ES generation — comes from ONE path launch
(kx_calib_gbm_prices, kx_calib_heston_objective), all on the same normals
(common random numbers: seed 42, 252 steps a year, as calibration.rs:156-162
and :303-311). The reference prices those one call at a time.

Precision: FP64 paths by default, so that the prices, and therefore the
optimizer's trajectory, are the reference's (the FP64 engine matches the
oracle to about 1e-12); `precision="fp32"` trades that for speed.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field
from typing import Callable, Sequence

import numpy as np

from . import _abi, _check, _cfg, _lib, _lock, Contract, KontractError

# ---------------------------------------------------------------------------
# configuration and results (calibration.rs:20-60, optimizer.rs:39-105)
# ---------------------------------------------------------------------------


@dataclass
class FastCalibrationConfig:
    """calibration.rs:20-46 (defaults :35-45), plus the path precision."""
    n_paths: int = 1000
    trust_radius: float = 0.1
    max_iterations: int = 50
    tol_param: float = 1e-4
    tol_obj: float = 1e-6
    precision: str = "fp64"


@dataclass
class CalibrationResult:
    """calibration.rs:48-55."""
    parameters: list
    objective: float
    iterations: int
    converged: bool


@dataclass
class Bounds:
    """optimizer.rs:39-61: a box; points are clamped onto it before every
    evaluation."""
    lower: list
    upper: list

    def clamp(self, x) -> np.ndarray:
        return np.minimum(np.maximum(np.asarray(x, dtype=np.float64), self.lower), self.upper)


@dataclass
class CmaesConfig:
    """optimizer.rs:63-95 (defaults :85-95). `population_size` None means
    4 + floor(3 ln n)."""
    population_size: int | None = None
    sigma0: float = 0.3
    max_generations: int = 200
    tol_x: float = 1e-9
    tol_fun: float = 1e-12
    seed: int = 42


@dataclass
class OptimizeResult:
    """optimizer.rs:97-107."""
    best_params: list
    best_objective: float
    generations: int
    converged: bool = field(default=False)


# ---------------------------------------------------------------------------
# CMA-ES (optimizer.rs:109-400; Hansen, "The CMA Evolution Strategy: A
# Tutorial", 2016)
# ---------------------------------------------------------------------------


class _Strategy:
    """The strategy constants of dimension n and population lambda
    (optimizer.rs:113-170): log-decreasing weights of the mu = lambda / 2 best,
    mu_eff, c_sigma, d_sigma, c_c, c_1, c_mu and E||N(0, I)||."""

    def __init__(self, n: int, lam: int):
        mu = lam // 2
        raw = np.array([math.log(mu + 0.5) - math.log(i + 1) for i in range(mu)])
        w = raw / raw.sum()
        mu_eff = 1.0 / float(np.sum(w * w))
        nf = float(n)
        self.n, self.mu, self.weights, self.mu_eff = n, mu, w, mu_eff
        self.c_sigma = (mu_eff + 2.0) / (nf + mu_eff + 5.0)
        self.d_sigma = 1.0 + 2.0 * max(math.sqrt((mu_eff - 1.0) / (nf + 1.0)) - 1.0, 0.0) + self.c_sigma
        self.c_c = (4.0 + mu_eff / nf) / (nf + 4.0 + 2.0 * mu_eff / nf)
        self.c_1 = 2.0 / ((nf + 1.3) ** 2 + mu_eff)
        self.c_mu = max(min(1.0 - self.c_1, 2.0 * (mu_eff - 2.0 + 1.0 / mu_eff) / ((nf + 2.0) ** 2 + mu_eff)), 0.0)
        self.chi_n = math.sqrt(nf) * (1.0 - 1.0 / (4.0 * nf) + 1.0 / (21.0 * nf * nf))


def _generation_normals(seed: int, gen: int, lam: int, n: int) -> np.ndarray:
    """The lambda x n standard normals of generation `gen`, from a generator
    keyed by (seed, gen + 1): reproducible, and independent across
    generations as the reference's per-generation reseeding
    (optimizer.rs:224). The reference draws them from ChaCha8 (rand_chacha)
    with rand_distr's ziggurat; this draws from numpy's Philox."""
    bitgen = np.random.Philox(key=np.array([seed & (2**64 - 1), gen + 1], dtype=np.uint64))
    return np.random.Generator(bitgen).standard_normal((lam, n))


def cmaes_minimize(objective: Callable | None, x0: Sequence[float], bounds: Bounds, cfg: CmaesConfig, *,
                   objective_batch: Callable | None = None) -> OptimizeResult:
    """cmaes_minimize (optimizer.rs:177-332): minimise `objective(x) -> float`
    over `bounds` from x0. `objective_batch(list of x) -> list of float`, when
    given, evaluates a whole generation at once (the GPU calibration objective
    prices a population in one launch); the reference evaluates the population
    in parallel (optimizer.rs:239-243)."""
    if objective_batch is None:
        if objective is None:
            raise ValueError("an objective is required")
        objective_batch = lambda xs: [objective(x) for x in xs]  # noqa: E731
    x0 = np.asarray(x0, dtype=np.float64)
    n = len(x0)
    lam = max(cfg.population_size if cfg.population_size is not None else 4 + int(math.floor(3.0 * math.log(n))), 4)
    st = _Strategy(n, lam)
    mean = x0.copy()
    sigma = float(cfg.sigma0)
    p_sigma = np.zeros(n)
    p_c = np.zeros(n)
    cov = np.eye(n)
    best_x = bounds.clamp(x0)
    best_f = float(objective_batch([best_x])[0])
    converged = False
    generations = 0
    for gen in range(cfg.max_generations):
        generations = gen + 1
        # C = B diag(d^2) B^T (optimizer.rs:213-217), eigenvalues floored at 1e-18
        eigvals, eigvecs = np.linalg.eigh(cov)
        d = np.sqrt(np.maximum(eigvals, 1e-18))
        # z ~ N(0, I), y = B D z ~ N(0, C), x = m + sigma y (optimizer.rs:222-237)
        z = _generation_normals(cfg.seed, gen, lam, n)
        y = (z * d) @ eigvecs.T
        x = mean + sigma * y
        fitness = np.asarray(objective_batch([bounds.clamp(xi) for xi in x]), dtype=np.float64)
        # ascending fitness; NaN compares as equal (optimizer.rs:246-252): a stable sort
        # that keeps NaN where partial_cmp leaves it is approximated by sorting NaN last
        order = sorted(range(lam), key=lambda i: (math.isnan(fitness[i]), fitness[i]))
        b = order[0]
        if fitness[b] < best_f:
            best_f = float(fitness[b])
            best_x = bounds.clamp(x[b])
        sel = np.array(order[: st.mu])
        y_w = st.weights @ y[sel]
        new_mean = mean + sigma * y_w
        # p_sigma <- (1 - c_s) p_sigma + sqrt(c_s (2 - c_s) mu_eff) C^{-1/2} y_w
        c_inv_sqrt_yw = eigvecs @ ((eigvecs.T @ y_w) / d)
        p_sigma = (1.0 - st.c_sigma) * p_sigma + math.sqrt(st.c_sigma * (2.0 - st.c_sigma) * st.mu_eff) * c_inv_sqrt_yw
        ps_norm = float(np.linalg.norm(p_sigma))
        denom = math.sqrt(1.0 - (1.0 - st.c_sigma) ** (2 * (gen + 1)))
        h_sigma = 1.0 if ps_norm / denom < (1.4 + 2.0 / (st.n + 1.0)) * st.chi_n else 0.0
        p_c = (1.0 - st.c_c) * p_c + h_sigma * math.sqrt(st.c_c * (2.0 - st.c_c) * st.mu_eff) * y_w
        # rank-1 + rank-mu update (optimizer.rs:368-400)
        delta = (1.0 - h_sigma) * st.c_c * (2.0 - st.c_c)
        ys = y[sel]
        rank_mu = (ys * st.weights[:, None]).T @ ys
        cov = (1.0 - st.c_1 - st.c_mu) * cov + st.c_1 * (np.outer(p_c, p_c) + delta * cov) + st.c_mu * rank_mu
        sigma *= math.exp((st.c_sigma / st.d_sigma) * (ps_norm / st.chi_n - 1.0))
        mean = new_mean
        d_max = float(d.max())
        f_spread = abs(fitness[order[min(st.mu, lam - 1)]] - fitness[order[0]])
        if sigma * d_max < cfg.tol_x or f_spread < cfg.tol_fun:
            converged = True
            break
        if not math.isfinite(sigma):
            break
    return OptimizeResult(best_params=[float(v) for v in best_x], best_objective=best_f, generations=generations,
                          converged=converged)


# ---------------------------------------------------------------------------
# the batched objectives (one path launch each)
# ---------------------------------------------------------------------------


def _mc(n_paths: int, rate: float, precision: str) -> _abi.KxMcConfig:
    # McConfig { n_paths, seed: 42, steps_per_year: 252, rate } (calibration.rs:156-162, :303-311)
    return _cfg(n_paths, 42, 252, rate, precision, False)


def contract_asset(contract: Contract) -> str:
    """calibration.rs:62-68: the first asset of the compiled plan, else
    "underlying"."""
    try:
        assets = contract.plan()["assets"]
    except KontractError:
        return "underlying"
    return assets[0] if assets else "underlying"


def gbm_prices(contract: Contract, asset: str, market_prices: Sequence[tuple], sigmas: Sequence[float], rate: float,
               n_paths: int, precision: str = "fp64") -> np.ndarray:
    """gbm_prices (calibration.rs:72-90) at several volatilities in one
    launch: [len(sigmas), len(market_prices)], NaN where a price fails."""
    spots = (C.c_double * max(1, len(market_prices)))(*[float(s) for s, _ in market_prices])
    sg = (C.c_double * max(1, len(sigmas)))(*[float(v) for v in sigmas])
    out = (C.c_double * max(1, len(sigmas) * len(market_prices)))()
    cfg = _mc(n_paths, rate, precision)
    with _lock:
        _check(_lib().kx_calib_gbm_prices(contract._handle().h, asset.encode(), spots, len(market_prices), sg,
                                          len(sigmas), C.byref(cfg), out))
    return np.array(out[: len(sigmas) * len(market_prices)], dtype=np.float64).reshape(len(sigmas),
                                                                                       len(market_prices))


def heston_objective(contract: Contract, market_prices: Sequence[tuple], params: Sequence[Sequence[float]],
                     rate: float, n_paths: int, precision: str = "fp64", asset: str = "underlying") -> np.ndarray:
    """eval_obj_heston (calibration.rs:103-126) for each parameter vector
    (v0, kappa, theta, sigma_v, rho), all in one launch. The reference
    simulates the asset "underlying" whatever the contract names
    (calibration.rs:115); quotes whose price fails are left out of the sum."""
    q = [float(v) for s, p in market_prices for v in (s, p)]
    pv = [float(v) for row in params for v in row]
    if len(pv) != 5 * len(params):
        raise ValueError("each parameter vector has 5 entries (v0, kappa, theta, sigma_v, rho)")
    qa = (C.c_double * max(1, len(q)))(*q)
    pa = (C.c_double * max(1, len(pv)))(*pv)
    obj = (C.c_double * max(1, len(params)))()
    cfg = _mc(n_paths, rate, precision)
    with _lock:
        _check(_lib().kx_calib_heston_objective(contract._handle().h, asset.encode(), qa, len(market_prices), pa,
                                                len(params), C.byref(cfg), obj, None))
    return np.array(obj[: len(params)], dtype=np.float64)


def _mse(prices, market_prices) -> float:
    """calibration.rs:92-101: mean squared error over max(1, n) quotes."""
    n = float(max(len(market_prices), 1))
    s = 0.0
    for p, (_, mkt) in zip(prices, market_prices):
        d = p - mkt
        s += d * d
    return s / n


# ---------------------------------------------------------------------------
# the optimizers, on any batched price / objective function
# ---------------------------------------------------------------------------


def _gauss_newton_sigma(prices_at: Callable, market_prices, config: FastCalibrationConfig) -> CalibrationResult:
    """The loop of fit_gbm_volatility (calibration.rs:164-236);
    prices_at(sigmas) -> [len(sigmas), n_quotes]."""
    delta = 1e-3
    sigma = 0.20
    converged = False
    iters = config.max_iterations
    for it in range(config.max_iterations):
        both = prices_at([sigma, sigma + delta])  # price and price(sigma + delta): one launch
        num = den = 0.0
        for p, p_up, (_, mkt) in zip(both[0], both[1], market_prices):
            vega = (p_up - p) / delta
            resid = p - mkt
            num, den = num + vega * resid, den + vega * vega
        if den < 1e-12:
            converged = True
            iters = it + 1
            break
        raw_step = -num / den
        step = min(max(raw_step, -config.trust_radius), config.trust_radius)
        sigma_next = min(max(sigma + step, 0.01), 3.0)
        if abs(sigma_next - sigma) < config.tol_param:
            sigma = sigma_next
            converged = True
            iters = it + 1
            break
        sigma = sigma_next
    final = prices_at([sigma])[0]
    return CalibrationResult(parameters=[sigma], objective=_mse(final, market_prices), iterations=iters,
                             converged=converged)


def _clamp_heston(params) -> list:
    """calibration.rs:128-141."""
    lo_hi = [(0.001, None), (0.01, None), (0.001, None), (0.01, 2.0), (-0.99, 0.99)]
    out = []
    for p, (lo, hi) in zip(params, lo_hi):
        p = max(p, lo)
        out.append(min(p, hi) if hi is not None else p)
    return out


def _heston_descent(objective_batch: Callable, config: FastCalibrationConfig) -> CalibrationResult:
    """The loop of fit_heston_parameters (calibration.rs:246-300);
    objective_batch(list of 5-vectors) -> objectives. The objective and its
    five forward bumps come from one batch."""
    params = [0.04, 2.0, 0.04, 0.3, -0.5]
    deltas = [0.001, 0.01, 0.001, 0.01, 0.01]
    obj_prev = math.inf
    converged = False
    for _ in range(config.max_iterations):
        batch = [params] + [[p + (deltas[i] if j == i else 0.0) for j, p in enumerate(params)] for i in range(5)]
        objs = objective_batch(batch)
        obj = float(objs[0])
        if abs(obj_prev - obj) < config.tol_obj:
            converged = True
            break
        obj_prev = obj
        new = []
        for i, p in enumerate(params):
            grad = (float(objs[i + 1]) - obj) / deltas[i]
            step = -min(max(grad * config.trust_radius * 0.1, -0.02), 0.02)
            new.append(min(max(p + step, 0.001), 5.0))  # as the reference, rho included
        params = _clamp_heston(new)
    return CalibrationResult(parameters=params, objective=obj_prev, iterations=config.max_iterations,
                             converged=converged)


def _cmaes_calibration(objective_batch: Callable, x0, lower, upper, max_generations: int) -> CalibrationResult:
    """run_cmaes_calibration (calibration.rs:319-384): CMA-ES over u in
    [0, 1]^n mapped to lower + u (upper - lower), population max(8 n, 16),
    sigma0 0.4, seed 42."""
    lower = np.asarray(lower, dtype=np.float64)
    width = np.maximum(np.asarray(upper, dtype=np.float64) - lower, 1e-12)
    n = len(x0)
    u0 = np.clip((np.asarray(x0, dtype=np.float64) - lower) / width, 0.0, 1.0)
    cfg = CmaesConfig(population_size=max(8 * n, 16), sigma0=0.4, max_generations=max_generations, seed=42)
    res = cmaes_minimize(None, u0, Bounds([0.0] * n, [1.0] * n), cfg,
                         objective_batch=lambda us: objective_batch([lower + np.asarray(u) * width for u in us]))
    params = [float(lo + u * w) for u, lo, w in zip(res.best_params, lower, width)]
    return CalibrationResult(parameters=params, objective=res.best_objective, iterations=res.generations,
                             converged=res.converged)


# ---------------------------------------------------------------------------
# the reference's entry points
# ---------------------------------------------------------------------------


def fit_gbm_volatility(contract: Contract, times: Sequence[float], market_prices: Sequence[tuple], rate: float,
                       config: FastCalibrationConfig | None = None) -> CalibrationResult:
    """fit_gbm_volatility (calibration.rs:149-237): sigma from (spot, price)
    quotes by damped Gauss-Newton with a CRN finite-difference vega; each
    iteration prices every quote at sigma and sigma + 1e-3 in one launch."""
    config = config or FastCalibrationConfig()
    asset = contract_asset(contract)
    return _gauss_newton_sigma(
        lambda sigmas: gbm_prices(contract, asset, market_prices, sigmas, rate, config.n_paths, config.precision),
        market_prices, config)


def fit_heston_parameters(contract: Contract, times: Sequence[float], market_prices: Sequence[tuple], rate: float,
                          config: FastCalibrationConfig | None = None) -> CalibrationResult:
    """fit_heston_parameters (calibration.rs:239-301): [v0, kappa, theta,
    sigma_v, rho] by gradient descent in a trust region; each iteration's
    objective and its five forward bumps are one launch."""
    config = config or FastCalibrationConfig()
    return _heston_descent(
        lambda ps: heston_objective(contract, market_prices, ps, rate, config.n_paths, config.precision), config)


HESTON_X0 = [0.04, 2.0, 0.04, 0.3, -0.5]
HESTON_LOWER = [0.001, 0.1, 0.001, 0.01, -0.99]
HESTON_UPPER = [1.0, 10.0, 1.0, 2.0, 0.99]


def calibrate_heston_cmaes(contract: Contract, market_prices: Sequence[tuple], rate: float,
                           config: FastCalibrationConfig | None = None) -> CalibrationResult:
    """calibrate_heston_cmaes (calibration.rs:441-465): the five Heston
    parameters by CMA-ES within v0, theta in [1e-3, 1], kappa in [0.1, 10],
    sigma_v in [0.01, 2], rho in [-0.99, 0.99], config.max_iterations
    generations; each generation's 40 candidates x all quotes are one launch."""
    config = config or FastCalibrationConfig()
    return _cmaes_calibration(
        lambda ps: heston_objective(contract, market_prices, ps, rate, config.n_paths, config.precision),
        HESTON_X0, HESTON_LOWER, HESTON_UPPER, config.max_iterations)


__all__ = ["FastCalibrationConfig", "CalibrationResult", "Bounds", "CmaesConfig", "OptimizeResult",
           "cmaes_minimize", "contract_asset", "gbm_prices", "heston_objective", "fit_gbm_volatility",
           "fit_heston_parameters", "calibrate_heston_cmaes"]
