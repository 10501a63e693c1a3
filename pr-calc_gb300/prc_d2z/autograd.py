"""delta2zreion as a differentiable torch operation.

The forward is the GPU step (prc_d2z_forward with the argmax recorded); the
backward is prc_d2z_backward: dL/d delta_lin and dL/dB_r for the barrier
offsets.  Because z = A (delta_R + B_r) - 1 is linear in delta_R for the
winning radius r*(cell), the gradient needs only the argmax, not delta_R.

The barrier offsets depend on the model parameters through
    B_r = sqrt(2 (sigma_min^2 - sigma_r^2)) * erfizeta,
    erfizeta = erfc^-1(1/zeta),  sigma_min = sigma(M_min)
(delta2zreion_d2z.C:24-26, 97-100, 206-216), so dL/dzeta and dL/dM_min follow
from dL/dB_r on the host (param_gradients).

    engine = Delta2Zreion.from_parameters(p, cl, argmax=True)
    z = delta2zreion_fn(delta, engine)            # delta: CUDA float32, requires_grad
    loss = ((z - z_t) ** 2).mean(); loss.backward()
    dzeta, dmmin = param_gradients(engine.tables, p, cl, engine.last_dB)
"""
from __future__ import annotations

import math

import numpy as np

from . import CLParameters, Delta2Zreion, Parameters, Tables, compute_tables

__all__ = ["delta2zreion_fn", "Delta2ZreionFunction", "param_gradients", "barrier_derivatives"]


def _function():
    import torch

    class Delta2ZreionFunction(torch.autograd.Function):
        """(delta_lin, barrier_b) -> zreion.  barrier_b (float64, n_radii, any
        device) is installed in the engine before the forward when given; its
        gradient is dL/dB_r."""

        @staticmethod
        def forward(ctx, delta_lin, barrier_b, engine):
            if barrier_b is not None:
                engine.set_barrier(barrier_b.detach().double().cpu().numpy(), engine.barrier_a)
            z, am, _ = engine.forward(delta_lin.detach().contiguous(), want_argmax=True)
            ctx.engine = engine
            ctx.has_b = barrier_b is not None
            ctx.b_device = barrier_b.device if barrier_b is not None else None
            ctx.save_for_backward(am)
            ctx.mark_non_differentiable(am)
            return z, am

        @staticmethod
        def backward(ctx, gz, _gam):
            (am,) = ctx.saved_tensors
            dd, dB = ctx.engine.backward(gz.contiguous(), am, want_dB=True)
            ctx.engine.last_dB = dB
            gb = None
            if ctx.has_b and ctx.needs_input_grad[1]:
                gb = torch.from_numpy(dB).to(ctx.b_device)
            return dd, gb, None

    return Delta2ZreionFunction


_FN = None


def Delta2ZreionFunction():  # noqa: N802  (class factory: torch is imported lazily)
    global _FN
    if _FN is None:
        _FN = _function()
    return _FN


def delta2zreion_fn(delta_lin, engine: Delta2Zreion, barrier_b=None):
    """zreion of a CUDA float32 delta_lin (N^3, file order), differentiable in
    delta_lin (and in barrier_b when given).  The argmax of the call is kept in
    engine.last_argmax; dL/dB_r of the last backward in engine.last_dB."""
    z, am = Delta2ZreionFunction().apply(delta_lin, barrier_b, engine)
    engine.last_argmax = am
    return z


def barrier_derivatives(t: Tables, zeta: float):
    """(dB_r/dzeta, dB_r/dsigma_min) for the tables t.

    dB/dzeta = sqrt(2(smin^2 - s_r^2)) * d erfc^-1(y)/dy * dy/dzeta with
    d erfc^-1(y)/dy = -(sqrt(pi)/2) exp(erfizeta^2) and y = 1/zeta;
    dB/dsigma_min = 2 sigma_min erfizeta / sqrt(2(smin^2 - s_r^2)).
    Radii whose B_r is NaN (sigma_r > sigma_min) get 0."""
    e = float(t.erfizeta)
    smin = float(t.sigma_min)
    B = np.asarray(t.barrier_b, np.float64)
    ok = np.isfinite(B) & (B != 0)
    s = np.where(ok, B / e, 0.0) if e != 0 else np.zeros_like(B)  # sqrt(2(smin^2 - s_r^2))
    derf = (math.sqrt(math.pi) / 2.0) * math.exp(e * e) / (zeta * zeta)
    dB_dzeta = np.where(ok, s * derf, 0.0)
    with np.errstate(divide="ignore", invalid="ignore"):
        dB_dsmin = np.where(ok & (s > 0), 2.0 * smin * e / s, 0.0)
    return dB_dzeta, dB_dsmin


def _sigma_of_mass(p: Parameters, cl: CLParameters, mass: float) -> float:
    q = CLParameters(Rmax=cl.Rmax, zeta=cl.zeta, M_min=float(mass))
    return float(compute_tables(p, q).sigma_min)


def param_gradients(t: Tables, p: Parameters, cl: CLParameters, dL_dB, dlnm: float = 0.01):
    """(dL/dzeta, dL/dM_min) from dL/dB_r (n_radii).  dsigma_min/dM_min is a
    central difference of the host sigma(M) in ln M (step dlnm)."""
    dB_dzeta, dB_dsmin = barrier_derivatives(t, float(cl.zeta))
    g = np.nan_to_num(np.asarray(dL_dB, np.float64))
    dzeta = float(np.dot(g, dB_dzeta))
    m = float(cl.M_min)
    s_hi = _sigma_of_mass(p, cl, m * math.exp(dlnm))
    s_lo = _sigma_of_mass(p, cl, m * math.exp(-dlnm))
    dsmin_dm = (s_hi - s_lo) / (2.0 * dlnm * m)
    dmmin = float(np.dot(g, dB_dsmin)) * dsmin_dm
    return dzeta, dmmin
