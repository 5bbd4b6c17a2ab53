"""FP64 NumPy restatement of the reference CuPy MHD solver (oracle, test-only).

Follows ``cuda/taylor_green_mhd/`` of the reference (mahanr/jax_tg_project):
operator ``operators.py:16-107``, RK4 ``integrator.py:14-32``, diagnostics
``diagnostics.py:20-49``, configuration and time-step validation
``config.py:53-118``, initial condition ``initial_conditions.py:9-21`` and the
run loop ``simulation.py:49-100`` (plots omitted).  All fields are spectral
(full complex ``fftn`` layout, shape (3, N, N, N)).

``lorentz_sign`` selects the sign of the Lorentz term in the momentum RHS:
``-1`` reproduces the reference code (``rhs_u = -P(u.grad u) - P(j x b) - nu k^2 u``,
operators.py:88-92), ``+1`` is the physical ``+ j x b`` of the equations the
reference README states.  The default is the reference's ``-1``.
"""
from __future__ import annotations

import math
import time

import numpy as np

from .tg_numpy import (TWO_PI, fftn, ifftn, make_dealias_mask, make_wavenumbers,
                       step_counts)


class Grid:
    """Arrays of ``SpectralGrid`` (cuda/taylor_green_cuda/grid.py:4-29)."""

    def __init__(self, n, length=TWO_PI):
        self.n = n
        self.kx, self.ky, self.kz = make_wavenumbers(n, length)
        self.mask = make_dealias_mask(n, length)
        self.k2 = self.kx * self.kx + self.ky * self.ky + self.kz * self.kz

    def to_spectral(self, f):
        return fftn(f) * self.mask

    @staticmethod
    def to_real(f_hat):
        return ifftn(f_hat).real

    def dealias(self, f_hat):
        return f_hat * self.mask


# ---------------------------------------------------------------- operators
def _gradients(g, f_hat):
    """Dealiased i k_d f_c (operators.py:8-14), indexed [component][direction]."""
    return [[g.dealias(1j * k * f_hat[c]) for k in (g.kx, g.ky, g.kz)] for c in range(3)]


def spectral_curl_hat(g, f_hat):
    """operators.py:16-22."""
    d = _gradients(g, f_hat)
    return g.dealias(np.stack([d[2][1] - d[1][2], d[0][2] - d[2][0], d[1][0] - d[0][1]]))


def leray_project(g, v_hat):
    """operators.py:27-38."""
    k2s = np.where(g.k2 == 0.0, 1.0, g.k2)
    kd = g.kx * v_hat[0] + g.ky * v_hat[1] + g.kz * v_hat[2]
    return v_hat - np.stack([g.kx * kd / k2s, g.ky * kd / k2s, g.kz * kd / k2s])


def divergence_from_hat(g, v_hat):
    """operators.py:40-51: physical div of a spectral vector."""
    return g.to_real(1j * (g.kx * v_hat[0] + g.ky * v_hat[1] + g.kz * v_hat[2]))


def _cross(a, b):
    return np.stack([a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2],
                     a[0] * b[1] - a[1] * b[0]])


def spectral_rhs_mhd(g, u_hat, b_hat, nu, eta, lorentz_sign=-1.0):
    """MhdSpectralOperator.rhs (operators.py:70-107)."""
    u_hat = g.dealias(u_hat)
    b_hat = g.dealias(b_hat)
    u = g.to_real(u_hat)
    b = g.to_real(b_hat)
    d = _gradients(g, u_hat)  # advection (operators.py:57-68)
    nlin = np.stack([sum(u[dd] * g.to_real(d[c][dd]) for dd in range(3)) for c in range(3)])
    adv = leray_project(g, fftn(nlin) * g.mask)
    j = g.to_real(spectral_curl_hat(g, b_hat))  # Lorentz (operators.py:78-86)
    lor = leray_project(g, fftn(_cross(j, b)) * g.mask)
    rhs_u = -adv + lorentz_sign * lor - nu * g.k2 * u_hat
    ind = spectral_curl_hat(g, fftn(_cross(u, b)) * g.mask) * g.mask  # induction (:94-99)
    rhs_b = leray_project(g, ind) - eta * g.k2 * b_hat
    return rhs_u, rhs_b


def rk4_step(g, u_hat, b_hat, dt, nu, eta, lorentz_sign=-1.0):
    """MhdRK4Integrator.step (integrator.py:14-32)."""
    f = lambda u, b: spectral_rhs_mhd(g, u, b, nu, eta, lorentz_sign)  # noqa: E731
    k1u, k1b = f(u_hat, b_hat)
    k2u, k2b = f(u_hat + 0.5 * dt * k1u, b_hat + 0.5 * dt * k1b)
    k3u, k3b = f(u_hat + 0.5 * dt * k2u, b_hat + 0.5 * dt * k2b)
    k4u, k4b = f(u_hat + dt * k3u, b_hat + dt * k3b)
    u_new = u_hat + (dt / 6.0) * (k1u + 2.0 * k2u + 2.0 * k3u + k4u)
    b_new = b_hat + (dt / 6.0) * (k1b + 2.0 * k2b + 2.0 * k3b + k4b)
    return u_new, b_new


def advance_one_step(g, u_hat, b_hat, dt, nu, eta, lorentz_sign=-1.0):
    """Step then dealias both fields (cuda/taylor_green_mhd.py:49-59)."""
    u_new, b_new = rk4_step(g, u_hat, b_hat, dt, nu, eta, lorentz_sign)
    return g.dealias(u_new), g.dealias(b_new)


# ---------------------------------------------------------------- diagnostics
def record(g, u_hat, b_hat):
    """MhdDiagnostics.record (diagnostics.py:20-49), returned as a dict."""
    u = g.to_real(u_hat)
    b = g.to_real(b_hat)
    ek = 0.5 * np.mean(np.sum(u * u, axis=0))
    em = 0.5 * np.mean(np.sum(b * b, axis=0))
    hc = np.mean(u[0] * b[0] + u[1] * b[1] + u[2] * b[2])
    om = g.to_real(spectral_curl_hat(g, u_hat))
    ens = 0.5 * np.mean(np.sum(om * om, axis=0))
    return {
        "kinetic_energy": float(ek), "magnetic_energy": float(em),
        "total_energy": float(ek + em), "cross_helicity": float(hc),
        "enstrophy": float(ens),
        "divergence_u_max": float(np.max(np.abs(divergence_from_hat(g, u_hat)))),
        "divergence_b_max": float(np.max(np.abs(divergence_from_hat(g, b_hat)))),
    }


# ---------------------------------------------------------------- config (config.py:53-118)
def magnetic_reynolds_to_resistivity(magnetic_reynolds, velocity_amplitude=1.0,
                                     domain_length=TWO_PI):
    if magnetic_reynolds <= 0.0:
        raise ValueError("magnetic_reynolds must be positive")
    return float((velocity_amplitude * domain_length) / magnetic_reynolds)


def resistivity_to_magnetic_reynolds(resistivity, velocity_amplitude=1.0,
                                     domain_length=TWO_PI):
    if resistivity < 0.0:
        raise ValueError("resistivity must be nonnegative")
    if resistivity == 0.0:
        return float("inf")
    return float((velocity_amplitude * domain_length) / resistivity)


def validate_timestep(dt, viscosity, resistivity, g, max_velocity=1.0, max_field=0.5,
                      cfl=0.5):
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
    kmax = float(np.max(np.abs(np.stack((g.kx, g.ky, g.kz)))))
    if kmax == 0.0:
        raise ValueError("wavenumber arrays must contain nonzero modes")
    h = np.pi / kmax
    k2max = float(np.max(g.k2))
    limit = float(min(cfl * h / max_velocity, cfl * h / max_field,
                      np.inf if viscosity == 0.0 else 2.0 / (viscosity * k2max),
                      np.inf if resistivity == 0.0 else 2.0 / (resistivity * k2max)))
    if dt > limit:
        raise ValueError(
            f"dt={dt:g} exceeds stability limit {limit:g}; reduce dt or increase cfl"
        )
    return limit


# ---------------------------------------------------------------- initial conditions
def initial_taylor_green_mhd(n, length=TWO_PI, magnetic_amplitude=0.5, dtype=np.float64):
    """Reference IC: TG velocity, b = amp * (u, v, 0) (initial_conditions.py:9-21).

    The reference builds the grid in float32; ``dtype`` selects it here.
    """
    x = np.linspace(0.0, length, n, endpoint=False, dtype=dtype)
    X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
    u = np.sin(X) * np.cos(Y) * np.cos(Z)
    v = -np.cos(X) * np.sin(Y) * np.cos(Z)
    vel = np.stack((u, v, np.zeros_like(u)))
    a = dtype(magnetic_amplitude)
    return vel, np.stack((a * u, a * v, np.zeros_like(u)))


def initial_mhd_equal_energy(n, length=TWO_PI):
    """TG velocity and b = (cos x sin y sin z, sin x cos y sin z, -2 sin x sin y cos z)
    scaled so that the magnetic energy equals the kinetic energy (1/8).

    This field is not in the reference; it is the MHD case of the 128^3 workload.
    The unscaled b has energy 3/8, so the scale is 1/sqrt(3).
    """
    x = np.linspace(0.0, length, n, endpoint=False)
    X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
    sx, cx, sy, cy, sz, cz = np.sin(X), np.cos(X), np.sin(Y), np.cos(Y), np.sin(Z), np.cos(Z)
    vel = np.stack((sx * cy * cz, -cx * sy * cz, np.zeros_like(X)))
    s = 1.0 / math.sqrt(3.0)
    mag = np.stack((s * cx * sy * sz, s * sx * cy * sz, -2.0 * s * sx * sy * cz))
    return vel, mag


# ---------------------------------------------------------------- run loop
def run_simulation(n=16, dt=0.005, reynolds=1000.0, magnetic_reynolds=1000.0,
                   magnetic_amplitude=0.5, total_time=0.05, save_every_time=0.01,
                   lorentz_sign=-1.0, fields=None, nu=None, eta=None, verbose=False):
    """TaylorGreenMhdSimulation.run (simulation.py:49-100) returning
    (u_hat, b_hat, series) with the MhdDiagnostics lists as a dict.

    ``nu``/``eta`` override the Re/Rm conversions (nu = L/Re, config.py:40-46);
    ``fields`` = (u, b) physical fields override the initial condition.
    """
    g = Grid(n)
    if nu is None:
        nu = TWO_PI / reynolds
    if eta is None:
        eta = TWO_PI / magnetic_reynolds
    steps, save_every = step_counts(total_time, dt, save_every_time)
    if fields is None:
        vel, mag = initial_taylor_green_mhd(n, magnetic_amplitude=magnetic_amplitude)
    else:
        vel, mag = fields
    max_field = magnetic_amplitude if fields is None else float(np.max(np.abs(mag)))
    validate_timestep(dt, nu, eta, g, max_velocity=1.0, max_field=max_field)
    u_hat, b_hat = g.to_spectral(vel), g.to_spectral(mag)
    keys = ("kinetic_energy", "magnetic_energy", "total_energy", "cross_helicity",
            "enstrophy", "divergence_u_max", "divergence_b_max")
    series = {"time": []}
    series.update({k: [] for k in keys})

    def rec(t):
        d = record(g, u_hat, b_hat)
        series["time"].append(t)
        for k in keys:
            series[k].append(d[k])

    rec(0.0)
    t0 = time.perf_counter()
    for step in range(1, steps + 1):
        u_hat, b_hat = advance_one_step(g, u_hat, b_hat, dt, nu, eta, lorentz_sign)
        if step % save_every == 0 or step == steps:
            rec(step * dt)
    if verbose:
        print(f"Simulated time: {total_time:.3f} ({steps} steps) in "
              f"{time.perf_counter() - t0:.3f} s")
    return u_hat, b_hat, series
