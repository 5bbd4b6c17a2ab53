"""Drop-in for the CuPy MHD solver's functional API (cuda/taylor_green_mhd.py).

Spectral fields are full complex fftn arrays (3, n, n, n) as in the CuPy
package.  The momentum equation uses the physical Lorentz force +(j x b)
by default; ``lorentz_sign=-1`` reproduces the reference code, which subtracts
it (cuda/taylor_green_mhd/operators.py:88-92).  nu = L/Re and eta = L/Rm
(cuda/taylor_green_mhd/config.py:40-46).
"""
from __future__ import annotations

import math
import time
from types import SimpleNamespace

import torch

from . import _runtime as rt
from .config import (TaylorGreenMhdConfig, magnetic_reynolds_to_resistivity,  # noqa: F401
                     resistivity_to_magnetic_reynolds, validate_timestep_mhd, wavenumber_axis)
from .taylor_green import make_dealias_mask as _mask
from .taylor_green import make_wavenumbers as _waves

TWO_PI = 2.0 * math.pi


def make_wavenumbers(n, length=TWO_PI):
    """cuda/taylor_green_mhd.py:12-15."""
    return _waves(n, length)


def make_dealias_mask(n, length=TWO_PI):
    """cuda/taylor_green_mhd.py:18-20."""
    return _mask(n, length)


def _plan(n, lorentz_sign=1.0):
    return rt.get_plan(n, physics="mhd", lorentz_sign=lorentz_sign)


def initial_taylor_green_mhd(n, length=TWO_PI, magnetic_amplitude=0.5):
    """Physical (u, b) with b = amp (u_x, u_y, 0) (cuda/taylor_green_mhd.py:22-24)."""
    p = _plan(n)
    f = p.inverse(p.initial_condition("mhd_reference", b_amp=magnetic_amplitude))[0]
    return f[:3], f[3:]


def initial_taylor_green_mhd_spectral(n, length=TWO_PI, magnetic_amplitude=0.5):
    """(u_hat, b_hat) full spectra (cuda/taylor_green_mhd.py:27-32)."""
    p = _plan(n)
    f = p.to_full(p.initial_condition("mhd_reference", b_amp=magnetic_amplitude))[0]
    return f[:3], f[3:]


def initial_equal_energy(n):
    """TG velocity and b = (cos x sin y sin z, sin x cos y sin z, -2 sin x sin y cos z)/sqrt(3):
    the MHD field of the 128^3 workload (E_m = E_k = 1/8).  Not in the reference."""
    p = _plan(n)
    f = p.inverse(p.initial_condition("mhd_equal_energy"))[0]
    return f[:3], f[3:]


def _state(u_hat, b_hat, lorentz_sign):
    n = rt.grid_size(u_hat)
    p = _plan(n, lorentz_sign)
    full = torch.cat([rt.as_full_spectrum(u_hat, p, 3), rt.as_full_spectrum(b_hat, p, 3)], dim=1)
    return p, p.from_full(full.contiguous())


def spectral_rhs_mhd(velocity_hat, magnetic_field_hat, viscosity, resistivity, kx, ky, kz,
                     dealias_mask, lorentz_sign=1.0):
    """MhdSpectralOperator.rhs (cuda/taylor_green_mhd.py:40-46)."""
    p, s = _state(velocity_hat, magnetic_field_hat, lorentz_sign)
    r = p.to_full(p.rhs(s, nu=float(viscosity), eta=float(resistivity)))[0]
    return r[:3], r[3:]


def advance_one_step(velocity_hat, magnetic_field_hat, dt, viscosity, resistivity, kx, ky, kz,
                     dealias_mask, lorentz_sign=1.0):
    """RK4 step of (u_hat, b_hat) then dealias (cuda/taylor_green_mhd.py:49-59)."""
    p, s = _state(velocity_hat, magnetic_field_hat, lorentz_sign)
    p.step(s, dt=float(dt), nu=float(viscosity), eta=float(resistivity), nsteps=1)
    f = p.to_full(s)[0]
    return f[:3], f[3:]


def kinetic_energy(velocity):
    """cuda/taylor_green_mhd.py:62-64."""
    p = _plan(int(velocity.shape[-1]))
    phys = torch.cat([rt.as_physical(velocity, p, 3), torch.zeros_like(rt.as_physical(velocity, p, 3))],
                     dim=1).contiguous()
    return p.physical_energy(phys)[0, 0]


def magnetic_energy(magnetic_field):
    """cuda/taylor_green_mhd.py:67-69."""
    return kinetic_energy(magnetic_field)


_DIAG_ATTRS = ("times", "kinetic_energies", "magnetic_energies", "total_energies",
               "cross_helicities", "enstrophies", "divergence_u_max", "divergence_b_max")


def run_simulation(n=128, dt=0.005, reynolds=1000.0, magnetic_reynolds=1000.0,
                   magnetic_amplitude=0.5, total_time=1.0, save_every_time=0.05, make_plots=False,
                   lorentz_sign=1.0, initial="reference", verbose=True, plot_dir="."):
    """TaylorGreenMhdSimulation.run (cuda/taylor_green_mhd.py:72-99): returns
    (u, b, diagnostics) with the MhdDiagnostics list attributes.  ``make_plots`` writes
    taylor_green_mhd_slice.png / taylor_green_mhd_diagnostics.png
    (cuda/taylor_green_mhd/plotting.py:9-48) into ``plot_dir``.
    ``initial='equal_energy'`` selects the equal-energy b field."""
    cfg = TaylorGreenMhdConfig(n=n, dt=dt, reynolds=reynolds, magnetic_reynolds=magnetic_reynolds,
                               magnetic_amplitude=magnetic_amplitude, total_time=total_time,
                               save_every_time=save_every_time)
    p = _plan(cfg.n, lorentz_sign)
    if initial == "equal_energy":
        s = p.initial_condition("mhd_equal_energy")
        max_field = float(p.absmax(s, "velocity")[0, 3:].max())
    else:
        s = p.initial_condition("mhd_reference", b_amp=cfg.magnetic_amplitude)
        max_field = cfg.magnetic_amplitude
    k = wavenumber_axis(cfg.n)
    validate_timestep_mhd(cfg.dt, cfg.viscosity, cfg.resistivity, k, k, k, max_velocity=1.0,
                          max_field=max_field)
    t0 = time.perf_counter()
    series = p.run(s, dt=cfg.dt, nu=cfg.viscosity, eta=cfg.resistivity, nsteps=cfg.steps,
                   save_every=cfg.save_every)
    h = series[:, 0].cpu().numpy()
    elapsed = time.perf_counter() - t0
    times, step = [0.0], 0
    while step < cfg.steps:
        step = min(step + cfg.save_every - (step % cfg.save_every), cfg.steps)
        times.append(step * cfg.dt)
    cols = {"kinetic_energies": 0, "magnetic_energies": 3, "total_energies": 5,
            "cross_helicities": 4, "enstrophies": 1, "divergence_u_max": 6, "divergence_b_max": 7}
    d = SimpleNamespace(times=times, **{k: [float(v) for v in h[:, c]] for k, c in cols.items()})
    if verbose:
        for i in range(1, len(times)):
            print(f"Save time step: {int(round(times[i] / cfg.dt))}, time: {times[i]:.6f}, "
                  f"E_k: {d.kinetic_energies[i]:.8e}, E_m: {d.magnetic_energies[i]:.8e}, "
                  f"H_c: {d.cross_helicities[i]:.8e}, enstrophy: {d.enstrophies[i]:.8e}")
        print(f"CUDA device: {torch.cuda.get_device_name()}")
        print(f"Reynolds number: Re = {cfg.reynolds:.1f}")
        print(f"Magnetic Reynolds number: Rm = {cfg.magnetic_reynolds:.1f}")
        print(f"Simulated time: {cfg.total_time:.3f} ({cfg.steps} steps) in {elapsed:.3f} s")
        print(f"Max divergence u: {max(d.divergence_u_max):.3e}, B: {max(d.divergence_b_max):.3e}")
    if make_plots:
        from .plots import save_plots
        save_plots(p, s, times, series.cpu().numpy(), kind="mhd", directory=plot_dir)
    f = p.inverse(s)[0]
    return f[:3], f[3:], d
