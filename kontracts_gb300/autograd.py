"""torch.autograd binding of the pathwise adjoint.

    import torch, kontracts_gb300 as kx
    from kontracts_gb300.autograd import heston_price
    p = torch.tensor([100., 0.04, 2.0, 0.04, 0.3, -0.5, 0.05], dtype=torch.float64, requires_grad=True)
    price = heston_price(kx.european_call("X", 100., 1.), p, asset="X", n_paths=2_000_000)
    price.backward()        # p.grad = (d/ds0, d/dv0, d/dkappa, d/dtheta, d/dsigma_v, d/drho, d/dr)

The forward pass runs kx_greeks_adjoint once; it returns the price and keeps
the sensitivities, and backward multiplies them by the incoming gradient.
heston_book_price / gbm_book_price do the same for a book of Europeans on
one shared simulation (kx_price_batch_sens: every contract's sensitivities
from one forward pass), returning the vector of prices; backward contracts
the incoming gradient with the per-contract sensitivities. Tensors are only
the interface here: the work is done by the engine's CUDA kernels through
the C ABI.
"""
from __future__ import annotations

import torch

from . import GBM, heston, price_batch

GBM_FIELDS = ("d_s0", "d_sigma", "d_r")
HESTON_FIELDS = ("d_s0", "d_v0", "d_kappa", "d_theta", "d_sigma_v", "d_rho", "d_r")


class PathwisePrice(torch.autograd.Function):
    @staticmethod
    def forward(ctx, params, contract, kind, asset, q, opts):
        vals = [float(x) for x in params.detach().cpu().tolist()]
        if kind == "gbm":
            s0, sigma, r = vals
            model = GBM(s0=s0, sigma=sigma, r=r, q=q, asset=asset)
            fields = GBM_FIELDS
        else:
            s0, v0, kappa, theta, sigma_v, rho, r = vals
            model = heston(s0, v0, kappa, theta, sigma_v, rho, r, asset=asset, scheme=opts.get("scheme", "reference"))
            fields = HESTON_FIELDS
        kw = {k: v for k, v in opts.items() if k != "scheme"}
        sens = contract.adjoint(model, **kw)
        grads = torch.tensor([getattr(sens, f) for f in fields], dtype=params.dtype, device=params.device)
        ctx.save_for_backward(grads)
        ctx.sens = sens
        return torch.tensor(sens.price, dtype=params.dtype, device=params.device)

    @staticmethod
    def backward(ctx, grad_out):
        (grads,) = ctx.saved_tensors
        return grad_out * grads, None, None, None, None, None


def gbm_price(contract, params: torch.Tensor, asset: str = "ASSET", q: float = 0.0, **opts) -> torch.Tensor:
    """Price of `contract` under GBM with params = (s0, sigma, r), differentiable."""
    return PathwisePrice.apply(params, contract, "gbm", asset, q, opts)


def heston_price(contract, params: torch.Tensor, asset: str = "ASSET", **opts) -> torch.Tensor:
    """Price under Heston with params = (s0, v0, kappa, theta, sigma_v, rho, r), differentiable."""
    return PathwisePrice.apply(params, contract, "heston", asset, 0.0, opts)


class PathwiseBookPrices(torch.autograd.Function):
    @staticmethod
    def forward(ctx, params, contracts, kind, asset, q, opts):
        vals = [float(x) for x in params.detach().cpu().tolist()]
        if kind == "gbm":
            s0, sigma, r = vals
            model = GBM(s0=s0, sigma=sigma, r=r, q=q, asset=asset)
            fields = GBM_FIELDS
        else:
            s0, v0, kappa, theta, sigma_v, rho, r = vals
            model = heston(s0, v0, kappa, theta, sigma_v, rho, r, asset=asset, scheme=opts.get("scheme", "reference"))
            fields = HESTON_FIELDS
        kw = {k: v for k, v in opts.items() if k != "scheme"}
        res, sens = price_batch(list(contracts), model, greeks=True, **kw)
        jac = torch.tensor([[getattr(s, f) for f in fields] for s in sens], dtype=params.dtype, device=params.device)
        ctx.save_for_backward(jac)
        return torch.tensor([r.price for r in res], dtype=params.dtype, device=params.device)

    @staticmethod
    def backward(ctx, grad_out):
        (jac,) = ctx.saved_tensors  # [contract][parameter]
        return grad_out @ jac, None, None, None, None, None


def gbm_book_price(contracts, params: torch.Tensor, asset: str = "ASSET", q: float = 0.0, **opts) -> torch.Tensor:
    """Prices of a book of Europeans on one shared GBM simulation, params =
    (s0, sigma, r), differentiable (price_batch(..., greeks=True))."""
    return PathwiseBookPrices.apply(params, tuple(contracts), "gbm", asset, q, opts)


def heston_book_price(contracts, params: torch.Tensor, asset: str = "ASSET", **opts) -> torch.Tensor:
    """Prices of a book of Europeans on one shared Heston simulation, params =
    (s0, v0, kappa, theta, sigma_v, rho, r), differentiable."""
    return PathwiseBookPrices.apply(params, tuple(contracts), "heston", asset, 0.0, opts)
