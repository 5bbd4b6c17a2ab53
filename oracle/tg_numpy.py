"""FP64 NumPy restatement of the reference JAX hydro solver (oracle, test-only).

Every public function follows ``jax/taylor_green_jax.py`` of the reference
(mahanr/jax_tg_project); the line numbers are given per function.  The
arithmetic is the reference's: full complex ``fftn``, advective form
``u . grad u`` built from the raw (un-dealiased) physical ``u`` times gradients
of the dealiased ``u_hat``, explicit-viscosity classical RK4 in physical space,
and the same diagnostics.  Plotting is not restated.

Two optional knobs exist only so that tests can separate scheme differences
from implementation errors of the GPU path:

* ``form="rotational"`` evaluates ``-P[F(u x omega)]`` instead of
  ``P[F(u . grad u)]`` (identical after projection for band-limited fields);
* ``integrator="lawson"`` uses the integrating-factor RK4 of the GPU path.

The defaults reproduce the reference.  The spectral-state helpers at the end
restate the CuPy HD package (``cuda/taylor_green_cuda/operators.py`` and
``cuda/taylor_green_cuda/integrator.py``), whose arithmetic is the same.
"""
from __future__ import annotations

import math
import time

import numpy as np

try:  # scipy's pocketfft accepts a worker count; numpy's is single-threaded
    import scipy.fft as _sfft

    def _fftn(a, workers=None):
        return _sfft.fftn(a, axes=(-3, -2, -1), workers=workers)

    def _ifftn(a, workers=None):
        return _sfft.ifftn(a, axes=(-3, -2, -1), workers=workers)
except ImportError:  # pragma: no cover - numpy fallback for the oracle only
    def _fftn(a, workers=None):
        return np.fft.fftn(a, axes=(-3, -2, -1))

    def _ifftn(a, workers=None):
        return np.fft.ifftn(a, axes=(-3, -2, -1))

#: worker threads for the oracle's FFTs (``-1`` = all host cores)
WORKERS = -1

TWO_PI = 2.0 * math.pi


def fftn(a):
    return _fftn(a, WORKERS)


def ifftn(a):
    return _ifftn(a, WORKERS)


# --------------------------------------------------------------------------
# Re <-> nu  (jax/taylor_green_jax.py:17-52)
# --------------------------------------------------------------------------
def reynolds_to_viscosity(reynolds, velocity_amplitude=1.0, domain_length=TWO_PI):
    """nu = u_amp * L / Re  (jax/taylor_green_jax.py:17-33)."""
    if reynolds <= 0:
        raise ValueError("Reynolds number must be positive")
    return float((velocity_amplitude * domain_length) / reynolds)


def viscosity_to_reynolds(nu, velocity_amplitude=1.0, domain_length=TWO_PI):
    """Re = u_amp * L / nu, inf for nu == 0  (jax/taylor_green_jax.py:36-52)."""
    if nu < 0.0:
        raise ValueError("Viscosity must be nonnegative")
    if nu == 0.0:
        return float("inf")
    return float((velocity_amplitude * domain_length) / nu)


# --------------------------------------------------------------------------
# grid  (jax/taylor_green_jax.py:55-67)
# --------------------------------------------------------------------------
def wavenumbers_1d(N, L=TWO_PI):
    """2*pi*fftfreq(N, L/N), the 1-D wavenumber axis (jax/taylor_green_jax.py:57)."""
    return 2.0 * np.pi * np.fft.fftfreq(N, d=L / N)


def make_wavenumbers(N, L=TWO_PI):
    """Full N^3 ``ij`` meshgrids of the wavenumbers (jax/taylor_green_jax.py:55-59)."""
    k = wavenumbers_1d(N, L)
    kx, ky, kz = np.meshgrid(k, k, k, indexing="ij")
    return kx, ky, kz


def dealias_keep_1d(N, L=TWO_PI):
    """Per-axis 2/3 rule: |k| <= (N//3)*2*pi/L (jax/taylor_green_jax.py:62-67).

    The comparison is done on the floating-point axis exactly as the reference
    does; for some N this drops the mode |i| == N//3 (see ``dealias_cutoff``).
    """
    cutoff = (N // 3) * (2.0 * np.pi / L)
    return np.abs(wavenumbers_1d(N, L)) <= cutoff


def dealias_cutoff(N, L=TWO_PI):
    """Largest integer mode index kept by the reference's mask along one axis."""
    keep = dealias_keep_1d(N, L)
    idx = np.rint(np.fft.fftfreq(N, d=1.0 / N)).astype(np.int64)
    return int(np.abs(idx[keep]).max())


def make_dealias_mask(N, L=TWO_PI):
    """Outer product of the per-axis masks (a cube, jax/taylor_green_jax.py:62-67)."""
    m = dealias_keep_1d(N, L)
    return m[:, None, None] * m[None, :, None] * m[None, None, :]


# --------------------------------------------------------------------------
# initial condition  (jax/taylor_green_jax.py:70-79)
# --------------------------------------------------------------------------
def initial_taylor_green(N, L=TWO_PI, amp=1.0):
    """u = amp sin x cos y cos z, v = -amp cos x sin y cos z, w = 0 on x_i = L i / N."""
    x = np.linspace(0.0, L, N, endpoint=False)
    X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
    u = amp * np.sin(X) * np.cos(Y) * np.cos(Z)
    v = -amp * np.cos(X) * np.sin(Y) * np.cos(Z)
    w = np.zeros_like(u)
    return np.stack([u, v, w], axis=0)


# --------------------------------------------------------------------------
# spectral operators and diagnostics  (jax/taylor_green_jax.py:82-128)
# --------------------------------------------------------------------------
def spectral_gradient(field_hat, kx, ky, kz):
    """(d/dx, d/dy, d/dz) of one scalar, returned in physical space (:82-87)."""
    return tuple(ifftn(1j * k * field_hat).real for k in (kx, ky, kz))


def spectral_divergence(u, kx, ky, kz):
    """Physical-space div u via spectral derivatives (:90-96)."""
    u_hat = fftn(u)
    div_hat = 1j * (kx * u_hat[0] + ky * u_hat[1] + kz * u_hat[2])
    return ifftn(div_hat).real


def vorticity(u, kx, ky, kz):
    """omega = curl u from the 9 spectral gradients (:99-109)."""
    u_hat = fftn(u)
    du = spectral_gradient(u_hat[0], kx, ky, kz)
    dv = spectral_gradient(u_hat[1], kx, ky, kz)
    dw = spectral_gradient(u_hat[2], kx, ky, kz)
    return np.stack([dw[1] - dv[2], du[2] - dw[0], dv[0] - du[1]], axis=0)


def enstrophy(u, kx, ky, kz):
    """0.5 * mean |omega|^2 (:112-115)."""
    omega = vorticity(u, kx, ky, kz)
    return 0.5 * np.mean(np.sum(omega * omega, axis=0))


def viscous_dissipation(u, nu, kx, ky, kz):
    """nu * sum_k |k|^2 |u_hat|^2 / N^6 (:118-128)."""
    u_hat = fftn(u)
    g2 = np.sum(
        np.abs(1j * kx * u_hat) ** 2
        + np.abs(1j * ky * u_hat) ** 2
        + np.abs(1j * kz * u_hat) ** 2,
        axis=0,
    )
    return nu * np.sum(g2) / (u.shape[-1] ** 6)


def kinetic_energy(u):
    """0.5 * mean |u|^2 (:199-201)."""
    return 0.5 * np.mean(u[0] ** 2 + u[1] ** 2 + u[2] ** 2)


# --------------------------------------------------------------------------
# timestep validation  (jax/taylor_green_jax.py:131-155)
# --------------------------------------------------------------------------
def validate_timestep(dt, nu, kx, ky, kz, cfl=0.5, max_velocity=1.0):
    """Advective (cfl*pi/k_max/u_max) and diffusive (2/(nu k2_max)) limits."""
    if dt <= 0.0:
        raise ValueError("dt must be positive")
    if nu < 0.0:
        raise ValueError("nu must be nonnegative")
    if cfl <= 0.0:
        raise ValueError("cfl must be positive")
    if max_velocity <= 0.0:
        raise ValueError("max_velocity must be positive")
    kmax = float(np.max(np.abs(np.stack([kx, ky, kz]))))
    if kmax == 0.0:
        raise ValueError("wavenumber arrays must contain nonzero modes")
    advective = cfl * (np.pi / kmax) / max_velocity
    k2max = float(np.max(kx * kx + ky * ky + kz * kz))
    diffusive = np.inf if nu == 0.0 else 2.0 / (nu * k2max)
    limit = float(min(advective, diffusive))
    if dt > limit:
        raise ValueError(
            f"dt={dt:g} exceeds stability limit {limit:g}; "
            "reduce dt or increase cfl"
        )
    return limit


# --------------------------------------------------------------------------
# RHS and RK4  (jax/taylor_green_jax.py:158-196)
# --------------------------------------------------------------------------
def _leray(v_hat, kx, ky, kz, k2_safe):
    kdot = kx * v_hat[0] + ky * v_hat[1] + kz * v_hat[2]
    return v_hat - np.stack([kx * kdot / k2_safe, ky * kdot / k2_safe,
                             kz * kdot / k2_safe], axis=0)


def _nonlinear_hat(u, u_hat, kx, ky, kz, mask, form):
    if form == "advective":  # reference: raw u times gradients of masked u_hat (:166-174)
        grads = [spectral_gradient(u_hat[c], kx, ky, kz) for c in range(3)]
        nlin = np.stack([u[0] * g[0] + u[1] * g[1] + u[2] * g[2] for g in grads], axis=0)
        return fftn(nlin) * mask
    if form == "rotational":  # -(u x omega); differs from u.grad u by a gradient
        om_hat = 1j * np.stack([ky * u_hat[2] - kz * u_hat[1],
                                kz * u_hat[0] - kx * u_hat[2],
                                kx * u_hat[1] - ky * u_hat[0]], axis=0)
        om = ifftn(om_hat).real
        uu = ifftn(u_hat).real
        cross = np.stack([uu[1] * om[2] - uu[2] * om[1],
                          uu[2] * om[0] - uu[0] * om[2],
                          uu[0] * om[1] - uu[1] * om[0]], axis=0)
        return -fftn(cross) * mask
    raise ValueError(f"unknown form {form!r}")


def spectral_rhs_hat(u, u_hat, nu, kx, ky, kz, mask, form="advective", viscous=True):
    """Spectral RHS -P[mask F(N)] - nu k^2 u_hat for masked ``u_hat`` (:158-184)."""
    k2 = kx * kx + ky * ky + kz * kz
    k2_safe = np.where(k2 == 0.0, 1.0, k2)
    nl = _leray(_nonlinear_hat(u, u_hat, kx, ky, kz, mask, form), kx, ky, kz, k2_safe)
    if viscous:
        return -nl - nu * k2 * u_hat
    return -nl


def spectral_rhs(u, nu, kx, ky, kz, dealias_mask, form="advective"):
    """Physical-space RHS of the reference (jax/taylor_green_jax.py:158-185)."""
    u_hat = fftn(u) * dealias_mask
    rhs_hat = spectral_rhs_hat(u, u_hat, nu, kx, ky, kz, dealias_mask, form)
    return ifftn(rhs_hat).real


def advance_one_step(u, dt, nu, kx, ky, kz, dealias_mask, form="advective",
                     integrator="explicit"):
    """Classical RK4 in physical space (jax/taylor_green_jax.py:188-196)."""
    if integrator == "lawson":
        return _advance_lawson(u, dt, nu, kx, ky, kz, dealias_mask, form)
    r1 = spectral_rhs(u, nu, kx, ky, kz, dealias_mask, form)
    r2 = spectral_rhs(u + 0.5 * dt * r1, nu, kx, ky, kz, dealias_mask, form)
    r3 = spectral_rhs(u + 0.5 * dt * r2, nu, kx, ky, kz, dealias_mask, form)
    r4 = spectral_rhs(u + dt * r3, nu, kx, ky, kz, dealias_mask, form)
    return u + (dt / 6.0) * (r1 + 2.0 * r2 + 2.0 * r3 + r4)


def _advance_lawson(u, dt, nu, kx, ky, kz, mask, form):
    """Integrating-factor (Lawson) RK4 of the GPU path, in spectral space.

    With E(h) = exp(-nu k^2 h) and N(v) = -P[mask F(nonlinear(v))]:
    a = E(h/2)(v + h/2 N(v)), b = E(h/2) v + h/2 N(a), c = E(h) v + h E(h/2) N(b),
    v' = E(h) v + h/6 (E(h) N(v) + 2 E(h/2) (N(a) + N(b)) + N(c)).
    """
    k2 = kx * kx + ky * ky + kz * kz
    e1 = np.exp(-nu * k2 * dt)
    eh = np.exp(-nu * k2 * 0.5 * dt)

    def nl(v_hat):
        vv = ifftn(v_hat).real
        return spectral_rhs_hat(vv, v_hat, nu, kx, ky, kz, mask, form, viscous=False)

    v = fftn(u) * mask
    n1 = nl(v)
    a = eh * (v + 0.5 * dt * n1)
    n2 = nl(a)
    b = eh * v + 0.5 * dt * n2
    n3 = nl(b)
    c = e1 * v + dt * eh * n3
    n4 = nl(c)
    v_new = e1 * v + (dt / 6.0) * (e1 * n1 + 2.0 * eh * (n2 + n3) + n4)
    return ifftn(v_new).real


# --------------------------------------------------------------------------
# run loop  (jax/taylor_green_jax.py:204-317, plotting omitted)
# --------------------------------------------------------------------------
def step_counts(total_time, dt, save_every_time):
    """int(T/dt) steps, save every max(1, int(save_every_time/dt)) (:238-239)."""
    return int(total_time / dt), max(1, int(save_every_time / dt))


def run_simulation(N=16, dt=0.005, nu=None, reynolds=None, total_time=0.5,
                   save_every_time=0.05, cfl=0.5, return_diagnostics=False,
                   u0=None, verbose=False, form="advective", integrator="explicit"):
    """The reference run loop and its diagnostics series (:204-317).

    ``u0`` (optional) replaces the Taylor-Green initial condition; it is an
    extension used by the perturbed-field parity cases.
    """
    if N < 4 or total_time <= 0.0 or save_every_time <= 0.0:
        raise ValueError(
            "N must be at least 4, total_time and save_every_time must be positive"
        )
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
    kx, ky, kz = make_wavenumbers(N, L)
    mask = make_dealias_mask(N, L)
    u = initial_taylor_green(N, L=L, amp=1.0) if u0 is None else np.array(u0, dtype=np.float64)
    validate_timestep(dt, nu, kx, ky, kz, cfl, max_velocity=float(np.max(np.abs(u))))

    def record(t):
        times.append(t)
        energies.append(float(kinetic_energy(u)))
        divergence_max.append(float(np.max(np.abs(spectral_divergence(u, kx, ky, kz)))))
        enstrophies.append(float(enstrophy(u, kx, ky, kz)))
        dissipations.append(float(viscous_dissipation(u, nu, kx, ky, kz)))

    times, energies, divergence_max, enstrophies, dissipations = [], [], [], [], []
    record(0.0)
    t0 = time.time()
    for step in range(n_steps):
        u = advance_one_step(u, dt, nu, kx, ky, kz, mask, form, integrator)
        if (step + 1) % save_every == 0 or step == n_steps - 1:
            record((step + 1) * dt)
            if verbose:
                print(f"Save time step: {step + 1}, Enstrophy: {enstrophies[-1]:.6e}")
    if verbose:
        print(f"Reynolds number: Re = {actual_re:.1f}")
        print(f"Simulated time: {total_time:.3f} ({n_steps} steps) in {time.time() - t0:.3f} s")
    diagnostics = {"time": times, "energy": energies, "divergence_max": divergence_max,
                   "enstrophy": enstrophies, "dissipation": dissipations}
    if return_diagnostics:
        return u, energies, diagnostics
    return u, energies


# --------------------------------------------------------------------------
# spectral-state (CuPy HD) variants: cuda/taylor_green_cuda/{grid,operators,integrator}.py
# --------------------------------------------------------------------------
def to_spectral(field, mask):
    """fftn then mask (cuda/taylor_green_cuda/grid.py:31-34)."""
    return fftn(field) * mask


def to_real(field_hat):
    """ifftn(...).real (cuda/taylor_green_cuda/grid.py:36-37)."""
    return ifftn(field_hat).real


def spectral_rhs_spectral(velocity_hat, nu, kx, ky, kz, mask):
    """CupySpectralOperator.rhs (cuda/taylor_green_cuda/operators.py:24-48).

    Dealiases the state first, so ``u`` in the product is the dealiased field.
    """
    v_hat = velocity_hat * mask
    v = to_real(v_hat)
    return spectral_rhs_hat(v, v_hat, nu, kx, ky, kz, mask)


def advance_one_step_spectral(velocity_hat, dt, nu, kx, ky, kz, mask):
    """RK4Integrator.step then dealias (cuda/taylor_green_cuda/integrator.py:7-12,
    cuda/taylor_green_cuda.py:40-46)."""
    f = lambda s: spectral_rhs_spectral(s, nu, kx, ky, kz, mask)  # noqa: E731
    r1 = f(velocity_hat)
    r2 = f(velocity_hat + 0.5 * dt * r1)
    r3 = f(velocity_hat + 0.5 * dt * r2)
    r4 = f(velocity_hat + dt * r3)
    return (velocity_hat + (dt / 6.0) * (r1 + 2.0 * r2 + 2.0 * r3 + r4)) * mask


def spectral_curl_hat(field_hat, kx, ky, kz, mask):
    """Dealiased i k x f_hat (cuda/taylor_green_cuda/operators.py:15-21)."""
    g = [[(1j * k * field_hat[c]) * mask for k in (kx, ky, kz)] for c in range(3)]
    return np.stack([g[2][1] - g[1][2], g[0][2] - g[2][0], g[1][0] - g[0][1]]) * mask


# --------------------------------------------------------------------------
# compact half-spectrum helpers shared by the tests
# --------------------------------------------------------------------------
def kept_indices(N, L=TWO_PI):
    """Indices of kept modes on a full axis, ordered 0..K, N-K..N-1."""
    K = dealias_cutoff(N, L)
    return np.concatenate([np.arange(0, K + 1), np.arange(N - K, N)]).astype(np.int64)


def compact_from_physical(u, L=TWO_PI):
    """Masked Fourier coefficients F(u)/N^3 on the kept half-spectrum.

    Shape (C, 2K+1, 2K+1, K+1), complex128: the layout of the GPU state
    without row padding.
    """
    N = u.shape[-1]
    K = dealias_cutoff(N, L)
    idx = kept_indices(N, L)
    uh = np.fft.rfftn(u, axes=(-3, -2, -1)) / float(N) ** 3
    return uh[:, idx][:, :, idx][:, :, :, : K + 1]


def physical_from_compact(c, N, L=TWO_PI):
    """Inverse of ``compact_from_physical`` (real field of shape (C, N, N, N))."""
    K = dealias_cutoff(N, L)
    idx = kept_indices(N, L)
    full = np.zeros((c.shape[0], N, N, N // 2 + 1), dtype=np.complex128)
    full[np.ix_(np.arange(c.shape[0]), idx, idx, np.arange(K + 1))] = c
    return np.fft.irfftn(full * float(N) ** 3, s=(N, N, N), axes=(-3, -2, -1))


def compact_diagnostics(c, nu=0.0):
    """KE, enstrophy and dissipation from compact coefficients (Parseval)."""
    N_half = c.shape[-1]
    K = N_half - 1
    ks = np.concatenate([np.arange(0, K + 1), np.arange(-K, 0)]).astype(np.float64)
    kx = ks[:, None, None]
    ky = ks[None, :, None]
    kz = np.arange(0, K + 1, dtype=np.float64)[None, None, :]
    w = np.where(kz == 0, 1.0, 2.0)
    e2 = np.abs(c[0]) ** 2 + np.abs(c[1]) ** 2 + np.abs(c[2]) ** 2
    ke = 0.5 * np.sum(w * e2)
    om = np.stack([ky * c[2] - kz * c[1], kz * c[0] - kx * c[2], kx * c[1] - ky * c[0]])
    ens = 0.5 * np.sum(w * np.sum(np.abs(om) ** 2, axis=0))
    k2 = kx * kx + ky * ky + kz * kz
    diss = nu * np.sum(w * k2 * e2)
    return ke, ens, diss
