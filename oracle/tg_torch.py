"""PyTorch (CPU, FP64) restatement of the reference JAX hydro step (oracle, test-only).

The same arithmetic as ``oracle/tg_numpy.py`` (jax/taylor_green_jax.py:158-201:
advective form, raw u times gradients of the dealiased u_hat, explicit RK4,
enstrophy from the 9 spectral gradients) written with torch.fft so that
torch.autograd can differentiate it.  It is the independent reverse-mode
reference the hand-written GPU adjoint is checked against (jax.grad of the
reference solver cannot run here: jax is not installed).
"""
from __future__ import annotations

import math

import torch


def _grid(N):
    k = 2.0 * math.pi * torch.fft.fftfreq(N, d=2.0 * math.pi / N, dtype=torch.float64)
    kx, ky, kz = torch.meshgrid(k, k, k, indexing="ij")
    cutoff = (N // 3) * 1.0
    m1 = k.abs() <= cutoff
    mask = m1[:, None, None] & m1[None, :, None] & m1[None, None, :]
    return kx, ky, kz, mask.to(torch.float64)


def _ifft(x):
    return torch.fft.ifftn(x, dim=(-3, -2, -1)).real


def spectral_rhs(u, nu, kx, ky, kz, mask):
    """jax/taylor_green_jax.py:158-185."""
    u_hat = torch.fft.fftn(u, dim=(-3, -2, -1)) * mask
    k2 = kx * kx + ky * ky + kz * kz
    k2s = torch.where(k2 == 0.0, torch.ones_like(k2), k2)
    grads = [[_ifft(1j * k * u_hat[c]) for k in (kx, ky, kz)] for c in range(3)]
    nlin = torch.stack([u[0] * g[0] + u[1] * g[1] + u[2] * g[2] for g in grads])
    nh = torch.fft.fftn(nlin, dim=(-3, -2, -1)) * mask
    kd = kx * nh[0] + ky * nh[1] + kz * nh[2]
    proj = nh - torch.stack([kx * kd / k2s, ky * kd / k2s, kz * kd / k2s])
    return _ifft(-proj - nu * k2 * u_hat)


def advance_one_step(u, dt, nu, kx, ky, kz, mask):
    """jax/taylor_green_jax.py:188-196."""
    r1 = spectral_rhs(u, nu, kx, ky, kz, mask)
    r2 = spectral_rhs(u + 0.5 * dt * r1, nu, kx, ky, kz, mask)
    r3 = spectral_rhs(u + 0.5 * dt * r2, nu, kx, ky, kz, mask)
    r4 = spectral_rhs(u + dt * r3, nu, kx, ky, kz, mask)
    return u + (dt / 6.0) * (r1 + 2.0 * r2 + 2.0 * r3 + r4)


def enstrophy(u, kx, ky, kz):
    """jax/taylor_green_jax.py:99-115."""
    uh = torch.fft.fftn(u, dim=(-3, -2, -1))
    d = [[_ifft(1j * k * uh[c]) for k in (kx, ky, kz)] for c in range(3)]
    om = torch.stack([d[2][1] - d[1][2], d[0][2] - d[2][0], d[1][0] - d[0][1]])
    return 0.5 * torch.mean(torch.sum(om * om, dim=0))


def final_enstrophy(u0, nu, dt, nsteps):
    """Enstrophy after nsteps reference RK4 steps, differentiable in u0 and nu."""
    N = u0.shape[-1]
    kx, ky, kz, mask = _grid(N)
    u = u0
    for _ in range(nsteps):
        u = advance_one_step(u, dt, nu, kx, ky, kz, mask)
    return enstrophy(u, kx, ky, kz)
