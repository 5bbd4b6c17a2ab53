"""Drop-in for the reference JAX solver's function API (jax/taylor_green_jax.py).

Same names, arguments, defaults, return shapes and error messages; every
computation runs in the sm_103a kernels of libtgdns.so.  Fields are returned as
CUDA tensors (the JAX functions return device arrays); inputs may be CUDA or
host tensors or NumPy arrays.  The wavenumber and mask arrays are accepted for
signature compatibility: the kernels derive k from the grid index, so only
their size is used (L must be 2 pi, as in every reference call).

Differences from the reference, by design: the state is dealiased before the
nonlinear product (identical for the band-limited fields the solver produces,
cf. jax/taylor_green_jax.py:160-168), the nonlinear term is evaluated in
rotational form u x omega (equal after projection), and the default RK4 is the
integrating-factor (Lawson) form (``set_default_scheme('explicit')`` selects the
reference's explicit-viscosity RK4).  Plots are not produced.
"""
from __future__ import annotations

import math
import time

import numpy as np
import torch

from . import _runtime as rt
from .config import (reynolds_to_viscosity, step_counts, validate_timestep,  # noqa: F401
                     viscosity_to_reynolds, wavenumber_axis)
from .plan import Plan  # noqa: F401

TWO_PI = 2.0 * math.pi


def _check_L(L):
    if abs(float(L) - TWO_PI) > 1e-12:
        raise NotImplementedError("the GB300 kernels assume the periodic box [0, 2pi)^3 (L = 2 pi)")


def make_wavenumbers(N, L=TWO_PI):
    """Full N^3 'ij' meshgrids of 2 pi fftfreq(N, L/N) (jax/taylor_green_jax.py:55-59)."""
    k = torch.from_numpy(wavenumber_axis(N, L)).to("cuda")
    kx, ky, kz = torch.meshgrid(k, k, k, indexing="ij")
    return kx, ky, kz


def make_dealias_mask(N, L=TWO_PI):
    """Per-axis 2/3 rule, outer product (jax/taylor_green_jax.py:62-67)."""
    k = wavenumber_axis(N, L)
    m = torch.from_numpy(np.abs(k) <= (N // 3) * (2.0 * np.pi / L)).to("cuda")
    return m[:, None, None] & m[None, :, None] & m[None, None, :]


def initial_taylor_green(N, L=TWO_PI, amp=1.0, precision=None):
    """(3, N, N, N) Taylor-Green velocity (jax/taylor_green_jax.py:70-79)."""
    _check_L(L)
    p = rt.get_plan(N, precision=precision)
    u = p.inverse(p.initial_condition("taylor_green"))[0]
    return u * amp if amp != 1.0 else u


def _state(u, precision=None):
    p = rt.get_plan(int(u.shape[-1]), precision=precision)
    return p, p.forward(rt.as_physical(u, p, 3))


def spectral_gradient(field_hat, kx, ky, kz):
    """(d/dx, d/dy, d/dz) in physical space of a scalar's full spectrum
    (jax/taylor_green_jax.py:82-87); the spectrum is dealiased first."""
    N = rt.grid_size(field_hat, kx)
    p = rt.get_plan(N)
    f = torch.as_tensor(field_hat).to(device=p.device, dtype=p.complex_dtype)
    full = torch.zeros((1, 3, N, N, N), dtype=p.complex_dtype, device=p.device)
    full[0, 0] = f
    s = p.from_full(full)
    # grad f = (d/dx, d/dy, d/dz) f: built from curls of (0, 0, f) and (0, f, 0)
    s2 = torch.zeros_like(s)
    s2[0, 2] = s[0, 0]
    c1 = p.derived(s2, "vorticity")[0]  # curl(0,0,f) = (df/dy, -df/dx, 0)
    s3 = torch.zeros_like(s)
    s3[0, 1] = s[0, 0]
    c2 = p.derived(s3, "vorticity")[0]  # curl(0,f,0) = (-df/dz, 0, df/dx)
    return -c1[1], c1[0], -c2[0]


def spectral_divergence(u, kx, ky, kz):
    """Physical div u via spectral derivatives (jax/taylor_green_jax.py:90-96)."""
    p, s = _state(u)
    return p.derived(s, "divergence")[0, 0]


def vorticity(u, kx, ky, kz):
    """curl u (jax/taylor_green_jax.py:99-109)."""
    p, s = _state(u)
    return p.derived(s, "vorticity")[0]


def enstrophy(u, kx, ky, kz):
    """0.5 <|curl u|^2> (jax/taylor_green_jax.py:112-115), FP64 reduction."""
    p, s = _state(u)
    return float(p.diagnostics(s, nu=0.0)[0, 1])


def viscous_dissipation(u, nu, kx, ky, kz):
    """nu sum |k|^2 |u_k|^2 / N^6 (jax/taylor_green_jax.py:118-128)."""
    p, s = _state(u)
    return float(p.diagnostics(s, nu=float(nu))[0, 2])


def kinetic_energy(u):
    """0.5 <|u|^2> of the grid values (jax/taylor_green_jax.py:199-201), FP64 reduction."""
    p = rt.get_plan(int(u.shape[-1]))
    return float(p.physical_energy(rt.as_physical(u, p, 3))[0, 0])


def spectral_rhs(u, nu, kx, ky, kz, dealias_mask):
    """Physical-space RHS -P[mask F(u.grad u)] - nu k^2 u_hat (jax/taylor_green_jax.py:158-185)."""
    p, s = _state(u)
    return p.inverse(p.rhs(s, nu=float(nu)))[0]


def advance_one_step(u, dt, nu, kx, ky, kz, dealias_mask):
    """One RK4 step of a physical field (jax/taylor_green_jax.py:188-196)."""
    p, s = _state(u)
    p.step(s, dt=float(dt), nu=float(nu), nsteps=1)
    return p.inverse(s)[0]


def run_simulation(N=16, dt=0.005, nu=None, reynolds=None, total_time=0.5, save_every_time=0.05,
                   cfl=0.5, return_diagnostics=False, precision=None, verbose=True, u0=None,
                   make_plots=False, plot_dir="."):
    """Decaying Taylor-Green run (jax/taylor_green_jax.py:204-317).

    Returns (u, energies) or (u, energies, diagnostics) with the reference's keys
    time, energy, divergence_max, enstrophy and dissipation.  ``u0`` optionally
    replaces the Taylor-Green initial field.  ``make_plots`` writes the reference's
    taylor_green_slice.png / taylor_green_diagnostics.png into ``plot_dir``.
    """
    if N < 4 or total_time <= 0.0 or save_every_time <= 0.0:
        raise ValueError("N must be at least 4, total_time and save_every_time must be positive")
    if dt <= 0.0:
        raise ValueError("dt must be positive")
    n_steps, save_every = step_counts(total_time, dt, save_every_time)
    L = TWO_PI
    if reynolds is not None:
        nu = reynolds_to_viscosity(reynolds, 1.0, L)
    elif nu is None:
        reynolds = 100
        nu = reynolds_to_viscosity(reynolds, 1.0, L)
    actual_re = viscosity_to_reynolds(nu, 1.0, L)
    p = rt.get_plan(N, precision=precision)
    if u0 is None:
        s = p.initial_condition("taylor_green")
    else:
        s = p.forward(rt.as_physical(u0, p, 3))
    umax = float(p.absmax(s, "velocity").max())
    kx = wavenumber_axis(N, L)
    validate_timestep(dt, nu, kx, kx, kx, cfl, max_velocity=umax)
    t0 = time.time()
    series = p.run(s, dt=dt, nu=nu, nsteps=n_steps, save_every=save_every)
    host = series[:, 0].cpu().numpy()
    elapsed = time.time() - t0
    times = [0.0]
    step = 0
    while step < n_steps:
        step = min(step + save_every - (step % save_every), n_steps)
        times.append(step * dt)
    energies = [float(v) for v in host[:, 0]]
    diag = {"time": times, "energy": energies, "divergence_max": [float(v) for v in host[:, 6]],
            "enstrophy": [float(v) for v in host[:, 1]],
            "dissipation": [float(v) for v in host[:, 2]]}
    if verbose:
        step = 0
        for i in range(1, len(times)):
            step = int(round(times[i] / dt))
            print(f"Save time step: {step}, Enstrophy: {diag['enstrophy'][i]:.6e}")
        print(f"Reynolds number: Re = {actual_re:.1f}")
        print(f"Simulated time: {total_time:.3f} ({n_steps} steps) in {elapsed:.3f} s")
        print(f"Energy trace: {energies[0]:.6f} -> {energies[-1]:.6f}")
        print(f"Max divergence: {max(diag['divergence_max']):.3e}")
    if make_plots:
        from .plots import save_plots
        out = save_plots(p, s, times, series.cpu().numpy(), kind="jax", directory=plot_dir)
        if verbose:
            print(f"Saved: {out['slice']}")
            print(f"Saved: {out['diagnostics']}")
    u = p.inverse(s)[0]
    if return_diagnostics:
        return u, energies, diag
    return u, energies
