"""Host-side parameters and validation with the reference's rules and messages.

Re <-> nu conversions and hydro time-step validation follow
jax/taylor_green_jax.py:17-52,131-155; the MHD conversions and validation follow
cuda/taylor_green_mhd/config.py:53-118; the configuration dataclasses follow
cuda/taylor_green_cuda/config.py:5-38 and cuda/taylor_green_mhd/config.py:7-50.
Error messages are identical so that callers matching on them keep working.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

TWO_PI = 2.0 * math.pi


def reynolds_to_viscosity(reynolds, velocity_amplitude=1.0, domain_length=TWO_PI):
    """nu = u_amp * L / Re (jax/taylor_green_jax.py:17-33)."""
    if reynolds <= 0:
        raise ValueError("Reynolds number must be positive")
    return float((velocity_amplitude * domain_length) / reynolds)


def viscosity_to_reynolds(nu, velocity_amplitude=1.0, domain_length=TWO_PI):
    """Re = u_amp * L / nu; inf for nu == 0 (jax/taylor_green_jax.py:36-52)."""
    if nu < 0.0:
        raise ValueError("Viscosity must be nonnegative")
    if nu == 0.0:
        return float("inf")
    return float((velocity_amplitude * domain_length) / nu)


def magnetic_reynolds_to_resistivity(magnetic_reynolds, velocity_amplitude=1.0,
                                     domain_length=TWO_PI):
    """eta = u_amp * L / Rm (cuda/taylor_green_mhd/config.py:53-60)."""
    if magnetic_reynolds <= 0.0:
        raise ValueError("magnetic_reynolds must be positive")
    return float((velocity_amplitude * domain_length) / magnetic_reynolds)


def resistivity_to_magnetic_reynolds(resistivity, velocity_amplitude=1.0, domain_length=TWO_PI):
    """Rm = u_amp * L / eta (cuda/taylor_green_mhd/config.py:63-72)."""
    if resistivity < 0.0:
        raise ValueError("resistivity must be nonnegative")
    if resistivity == 0.0:
        return float("inf")
    return float((velocity_amplitude * domain_length) / resistivity)


def wavenumber_axis(N, L=TWO_PI):
    """2 pi fftfreq(N, L/N) in FP64, the 1-D axis of the reference's meshgrids."""
    return 2.0 * np.pi * np.fft.fftfreq(N, d=L / N)


def dealias_cutoff(N, L=TWO_PI):
    """Largest |mode index| kept by the reference's 2/3 mask (jax/taylor_green_jax.py:62-67)."""
    k = wavenumber_axis(N, L)
    keep = np.abs(k) <= (N // 3) * (2.0 * np.pi / L)
    idx = np.rint(np.fft.fftfreq(N, d=1.0 / N)).astype(np.int64)
    return int(np.abs(idx[keep]).max())


def _kmax_k2max(kx, ky, kz):
    """max |k| over the three arrays and max |k|^2, as the reference computes them."""
    vals = []
    for k in (kx, ky, kz):
        if hasattr(k, "detach"):
            k = k.detach()
            vals.append(float(k.abs().max()))
        else:
            vals.append(float(np.max(np.abs(np.asarray(k)))))
    kmax = max(vals)
    try:
        k2 = kx * kx + ky * ky + kz * kz
        k2max = float(k2.max())
    except Exception:  # noqa: BLE001 - non-array inputs
        k2max = 3.0 * kmax * kmax
    return kmax, k2max


def validate_timestep(dt, nu, kx, ky, kz, cfl=0.5, max_velocity=1.0):
    """Advective and diffusive stability limits (jax/taylor_green_jax.py:131-155)."""
    if dt <= 0.0:
        raise ValueError("dt must be positive")
    if nu < 0.0:
        raise ValueError("nu must be nonnegative")
    if cfl <= 0.0:
        raise ValueError("cfl must be positive")
    if max_velocity <= 0.0:
        raise ValueError("max_velocity must be positive")
    kmax, k2max = _kmax_k2max(kx, ky, kz)
    if kmax == 0.0:
        raise ValueError("wavenumber arrays must contain nonzero modes")
    advective = cfl * (np.pi / kmax) / max_velocity
    diffusive = np.inf if nu == 0.0 else 2.0 / (nu * k2max)
    limit = float(min(advective, diffusive))
    if dt > limit:
        raise ValueError(f"dt={dt:g} exceeds stability limit {limit:g}; reduce dt or increase cfl")
    return limit


def validate_timestep_mhd(dt, viscosity, resistivity, kx, ky, kz, max_velocity=1.0, max_field=0.5,
                          cfl=0.5):
    """Adds the Alfven and resistive limits (cuda/taylor_green_mhd/config.py:75-118)."""
    if dt <= 0.0:
        raise ValueError("dt must be positive")
    if viscosity < 0.0:
        raise ValueError("viscosity must be nonnegative")
    if resistivity < 0.0:
        raise ValueError("resistivity must be nonnegative")
    if cfl <= 0.0:
        raise ValueError("cfl must be positive")
    if max_velocity <= 0.0:
        raise ValueError("max_velocity must be positive")
    if max_field <= 0.0:
        raise ValueError("max_field must be positive")
    kmax, k2max = _kmax_k2max(kx, ky, kz)
    if kmax == 0.0:
        raise ValueError("wavenumber arrays must contain nonzero modes")
    h = np.pi / kmax
    limit = float(min(cfl * h / max_velocity, cfl * h / max_field,
                      np.inf if viscosity == 0.0 else 2.0 / (viscosity * k2max),
                      np.inf if resistivity == 0.0 else 2.0 / (resistivity * k2max)))
    if dt > limit:
        raise ValueError(f"dt={dt:g} exceeds stability limit {limit:g}; reduce dt or increase cfl")
    return limit


def step_counts(total_time, dt, save_every_time):
    """int(T/dt) steps, saving every max(1, int(save_every_time/dt)) (jax/taylor_green_jax.py:238-239)."""
    return int(total_time / dt), max(1, int(save_every_time / dt))


@dataclass(frozen=True)
class TaylorGreenConfig:
    """cuda/taylor_green_cuda/config.py:5-38."""
    n: int = 128
    dt: float = 0.005
    reynolds: float = 1000.0
    total_time: float = 1.0
    save_every_time: float = 0.05
    domain_length: float = TWO_PI

    def __post_init__(self):
        if self.n < 4:
            raise ValueError("n must be at least 4")
        if self.dt <= 0.0:
            raise ValueError("dt must be positive")
        if self.reynolds <= 0.0:
            raise ValueError("reynolds must be positive")
        if self.total_time <= 0.0:
            raise ValueError("total_time must be positive")
        if self.save_every_time <= 0.0:
            raise ValueError("save_every_time must be positive")
        if self.domain_length <= 0.0:
            raise ValueError("domain_length must be positive")

    @property
    def viscosity(self):
        return self.domain_length / self.reynolds

    @property
    def steps(self):
        return int(self.total_time / self.dt)

    @property
    def save_every(self):
        return max(1, int(self.save_every_time / self.dt))


@dataclass(frozen=True)
class TaylorGreenMhdConfig:
    """cuda/taylor_green_mhd/config.py:7-50."""
    n: int = 128
    dt: float = 0.005
    reynolds: float = 1000.0
    magnetic_reynolds: float = 1000.0
    magnetic_amplitude: float = 0.5
    total_time: float = 1.0
    save_every_time: float = 0.05
    domain_length: float = TWO_PI

    def __post_init__(self):
        if self.n < 4:
            raise ValueError("n must be at least 4")
        if self.dt <= 0.0:
            raise ValueError("dt must be positive")
        if self.reynolds <= 0.0:
            raise ValueError("reynolds must be positive")
        if self.magnetic_reynolds <= 0.0:
            raise ValueError("magnetic_reynolds must be positive")
        if self.magnetic_amplitude < 0.0:
            raise ValueError("magnetic_amplitude must be nonnegative")
        if self.total_time <= 0.0:
            raise ValueError("total_time must be positive")
        if self.save_every_time <= 0.0:
            raise ValueError("save_every_time must be positive")
        if self.domain_length <= 0.0:
            raise ValueError("domain_length must be positive")

    @property
    def viscosity(self):
        return self.domain_length / self.reynolds

    @property
    def resistivity(self):
        return self.domain_length / self.magnetic_reynolds

    @property
    def steps(self):
        return int(self.total_time / self.dt)

    @property
    def save_every(self):
        return max(1, int(self.save_every_time / self.dt))
