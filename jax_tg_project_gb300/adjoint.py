"""Gradient of the final enstrophy with respect to the initial velocity and nu.

``final_enstrophy(u0, nu, dt, nsteps)`` is differentiable with torch.autograd:
its backward is the hand-written discrete adjoint of the integrating-factor RK4
step (tg_adjoint in libtgdns.so: transposed transforms, adjoint cross products,
self-adjoint projection and curl, states checkpointed every ~sqrt(nsteps) steps
and recomputed).  The reference has no gradient code; its counterpart would be
jax.grad through jax/taylor_green_jax.py:188-196.
"""
from __future__ import annotations

import torch

from . import _runtime as rt


def spectral_inner(plan, a, b):
    """sum_half w Re(a conj b): the inner product the state gradient refers to."""
    K = plan.K
    w = torch.full((plan.Hz,), 2.0, dtype=torch.float64, device=a.device)
    w[0] = 1.0
    w[K + 1:] = 0.0
    prod = (a * b.conj()).real.to(torch.float64)
    return float((prod * w).sum())


def enstrophy_gradient(plan, state0, dt, nu, nsteps, checkpoint_every=0):
    """(loss, grad_state, grad_nu) from the discrete adjoint."""
    return plan.adjoint(state0, dt, nu, nsteps, checkpoint_every)


class _FinalEnstrophy(torch.autograd.Function):
    @staticmethod
    def forward(ctx, u0, nu, dt, nsteps, checkpoint_every, precision):
        n = int(u0.shape[-1])
        plan = rt.get_plan(n, precision=precision)
        s0 = plan.forward(rt.as_physical(u0.detach(), plan, 3))
        ck = checkpoint_every if checkpoint_every == "tape" else int(checkpoint_every)
        loss, grad, gnu = plan.adjoint(s0, float(dt), float(nu), int(nsteps), ck)
        # d loss / d u0 on the grid: the state gradient mapped back through the
        # dealiased forward transform, (1/n^3) F^-1 grad
        gu = plan.inverse(grad)[0] / float(n) ** 3
        ctx.save_for_backward(gu.to(u0.dtype), gnu.to(torch.float64))
        return loss.to(torch.float64)

    @staticmethod
    def backward(ctx, gout):
        gu, gnu = ctx.saved_tensors
        gu = gu.to(gout.device)
        return gout * gu, (gout * gnu).to(torch.float64), None, None, None, None


def final_enstrophy(u0, nu, dt, nsteps, checkpoint_every=0, precision=None):
    """Enstrophy after nsteps RK4 steps from the physical field u0 (3, n, n, n), as a
    differentiable scalar in u0 and nu (a 0-d tensor)."""
    if not isinstance(nu, torch.Tensor):
        nu = torch.tensor(float(nu), dtype=torch.float64, device=u0.device)
    return _FinalEnstrophy.apply(u0, nu, dt, nsteps, checkpoint_every, precision)
