"""Drop-in for the CuPy HD solver's functional API (cuda/taylor_green_cuda.py).

The state is the full complex spectrum ``fftn(u)`` of shape (3, n, n, n), as in
the CuPy package; it is converted to and from the compact half spectrum of the
kernels by two CUDA kernels (tg_to_full_spectrum / tg_from_full_spectrum).
Viscosity follows the CuPy convention nu = L / Re
(cuda/taylor_green_cuda/config.py:28-30).
"""
from __future__ import annotations

import math
import time

import torch

from . import _runtime as rt
from .config import TaylorGreenConfig
from .taylor_green import make_dealias_mask as _mask
from .taylor_green import make_wavenumbers as _waves

TWO_PI = 2.0 * math.pi


def make_wavenumbers(n, length=TWO_PI):
    """cuda/taylor_green_cuda.py:12-14."""
    return _waves(n, length)


def make_dealias_mask(n, length=TWO_PI):
    """cuda/taylor_green_cuda.py:17-18."""
    return _mask(n, length)


def initial_taylor_green(n, length=TWO_PI):
    """Physical TG velocity (cuda/taylor_green_cuda.py:21-22)."""
    p = rt.get_plan(n)
    return p.inverse(p.initial_condition("taylor_green"))[0]


def initial_taylor_green_spectral(n, length=TWO_PI):
    """fftn of the TG velocity, dealiased (cuda/taylor_green_cuda.py:25-27)."""
    p = rt.get_plan(n)
    return p.to_full(p.initial_condition("taylor_green"))[0]


def _from_full(velocity_hat):
    p = rt.get_plan(rt.grid_size(velocity_hat))
    return p, p.from_full(rt.as_full_spectrum(velocity_hat, p, 3))


def spectral_rhs(velocity_hat, nu, kx, ky, kz, dealias_mask):
    """CupySpectralOperator.rhs (cuda/taylor_green_cuda.py:34-37)."""
    p, s = _from_full(velocity_hat)
    return p.to_full(p.rhs(s, nu=float(nu)))[0]


def advance_one_step(velocity_hat, dt, nu, kx, ky, kz, dealias_mask):
    """RK4 step then dealias (cuda/taylor_green_cuda.py:40-46)."""
    p, s = _from_full(velocity_hat)
    p.step(s, dt=float(dt), nu=float(nu), nsteps=1)
    return p.to_full(s)[0]


def kinetic_energy(velocity):
    """cuda/taylor_green_cuda.py:49-50."""
    p = rt.get_plan(int(velocity.shape[-1]))
    return p.physical_energy(rt.as_physical(velocity, p, 3))[0, 0]


def enstrophy(velocity, kx, ky, kz):
    """Diagnostics.record enstrophy of a physical field (cuda/taylor_green_cuda.py:53-60)."""
    p = rt.get_plan(int(velocity.shape[-1]))
    s = p.forward(rt.as_physical(velocity, p, 3))
    return p.diagnostics(s, nu=0.0)[0, 1]


def run_simulation(n=128, dt=0.005, reynolds=1000.0, total_time=1.0, save_every_time=0.05,
                   verbose=True, make_plots=False, plot_dir="."):
    """TaylorGreenSimulation.run (cuda/taylor_green_cuda.py:63-69): returns
    (u, times, energies, enstrophies); ``make_plots`` writes taylor_green_cuda_slice.png and
    taylor_green_cuda_diagnostics.png (cuda/taylor_green_cuda/plotting.py:7-31)."""
    cfg = TaylorGreenConfig(n, dt, reynolds, total_time, save_every_time)
    p = rt.get_plan(cfg.n)
    s = p.initial_condition("taylor_green")
    t0 = time.perf_counter()
    series = p.run(s, dt=cfg.dt, nu=cfg.viscosity, nsteps=cfg.steps, save_every=cfg.save_every)
    torch.cuda.synchronize()
    elapsed = time.perf_counter() - t0
    host = series[:, 0].cpu().numpy()
    times, step = [0.0], 0
    while step < cfg.steps:
        step = min(step + cfg.save_every - (step % cfg.save_every), cfg.steps)
        times.append(step * cfg.dt)
    energies = [float(v) for v in host[:, 0]]
    enstrophies = [float(v) for v in host[:, 1]]
    if verbose:
        for t, e in zip(times[1:], enstrophies[1:]):
            print(f"Save time step: {int(round(t / cfg.dt))}, time: {t:.6f}, enstrophy: {e:.8e}")
        print(f"CUDA device: {torch.cuda.get_device_name()}")
        print(f"Reynolds number: {cfg.reynolds:.1f}")
        print(f"Simulated time: {cfg.total_time:.3f} ({cfg.steps} steps) in {elapsed:.3f} s")
        print(f"Energy trace: {energies[0]:.6f} -> {energies[-1]:.6f}")
    if make_plots:
        from .plots import save_plots
        save_plots(p, s, times, series.cpu().numpy(), kind="hydro", directory=plot_dir)
    return p.inverse(s)[0], times, energies, enstrophies
