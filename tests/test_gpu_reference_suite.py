"""The reference's own unit tests, ported to the GB300 package's drop-in APIs.

jax/test_taylor_green_jax.py runs against jax_tg_project_gb300.taylor_green in
FP64 (the reference runs JAX with x64 enabled); cuda/test_taylor_green_cuda.py
and cuda/test_taylor_green_mhd.py run against jax_tg_project_gb300.spectral and
jax_tg_project_gb300.mhd in FP32 (the CuPy packages' float32 grids).
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LENGTH = 2.0 * math.pi


@pytest.fixture
def tgx():
    from jax_tg_project_gb300 import _runtime, taylor_green
    _runtime.set_default_precision("f64")
    yield taylor_green
    _runtime.set_default_precision("f32")


# ---------------------------------------------------------------- jax/test_taylor_green_jax.py
def test_initial_condition_is_divergence_free(tgx):
    kx, ky, kz = tgx.make_wavenumbers(16, LENGTH)
    velocity = tgx.initial_taylor_green(16, LENGTH)
    divergence = tgx.spectral_divergence(velocity, kx, ky, kz)
    assert float(divergence.abs().max()) < 1e-12


def test_dealias_mask_keeps_two_thirds_of_each_axis(tgx):
    mask = tgx.make_dealias_mask(16, LENGTH)
    assert tuple(mask.shape) == (16, 16, 16)
    assert int(mask.sum()) == 11 ** 3
    assert not bool(mask[8, 0, 0]) and bool(mask[5, 0, 0])


def test_timestep_validation_rejects_unstable_values(tgx):
    kx, ky, kz = tgx.make_wavenumbers(16, LENGTH)
    with pytest.raises(ValueError, match="stability limit"):
        tgx.validate_timestep(1.0, 0.01, kx, ky, kz)
    with pytest.raises(ValueError, match="positive"):
        tgx.validate_timestep(0.0, 0.01, kx, ky, kz)


def test_zero_mode_is_not_viscously_damped(tgx):
    import torch
    N = 8
    kx, ky, kz = tgx.make_wavenumbers(N, LENGTH)
    mask = tgx.make_dealias_mask(N, LENGTH)
    rhs = tgx.spectral_rhs(torch.ones((3, N, N, N)), 0.01, kx, ky, kz, mask)
    assert float(rhs.abs().max()) < 1e-12


def test_short_run_is_finite_divergence_free_and_decays(tgx):
    velocity, energies, diagnostics = tgx.run_simulation(
        N=8, dt=0.005, nu=0.01, total_time=0.02, save_every_time=0.01, return_diagnostics=True)
    assert bool(velocity.isfinite().all())
    assert diagnostics["time"] == [0.0, 0.01, 0.02]
    assert max(diagnostics["divergence_max"]) < 1e-10
    assert all(a >= b for a, b in zip(energies, energies[1:]))


def test_step_preserves_finite_values(tgx):
    N = 8
    kx, ky, kz = tgx.make_wavenumbers(N, LENGTH)
    mask = tgx.make_dealias_mask(N, LENGTH)
    velocity = tgx.initial_taylor_green(N, LENGTH)
    updated = tgx.advance_one_step(velocity, 0.005, 0.01, kx, ky, kz, mask)
    assert bool(updated.isfinite().all())


def test_reynolds_number_conversion(tgx):
    nu = tgx.reynolds_to_viscosity(100.0, 1.0, LENGTH)
    assert tgx.viscosity_to_reynolds(nu, 1.0, LENGTH) == pytest.approx(100.0, abs=1e-10)


def test_run_with_reynolds_number(tgx):
    u, energies = tgx.run_simulation(N=8, dt=0.005, reynolds=100, total_time=0.02,
                                     save_every_time=0.01)
    assert bool(u.isfinite().all())
    assert all(a >= b for a, b in zip(energies, energies[1:]))


def test_reynolds_must_be_positive(tgx):
    with pytest.raises(ValueError, match="Reynolds number must be positive"):
        tgx.reynolds_to_viscosity(-100)


def test_jax_api_values_match_oracle(tgx, golden_hydro):
    g = golden_hydro
    kx, ky, kz = tgx.make_wavenumbers(16)
    mask = tgx.make_dealias_mask(16)
    u0 = tgx.initial_taylor_green(16)
    assert tgx.kinetic_energy(u0) == pytest.approx(float(g["ic16_energy"]), rel=1e-13)
    assert tgx.enstrophy(u0, kx, ky, kz) == pytest.approx(float(g["ic16_enstrophy"]), rel=1e-13)
    assert tgx.viscous_dissipation(u0, 0.01, kx, ky, kz) == pytest.approx(
        float(g["ic16_dissipation"]), rel=1e-13)
    r = tgx.spectral_rhs(g["rhs16_in"], 0.01, kx, ky, kz, mask).cpu().numpy()
    assert np.linalg.norm(r - g["rhs16_out"]) / np.linalg.norm(g["rhs16_out"]) < 1e-12
    from oracle import tg_numpy as T
    w = tgx.vorticity(g["rhs16_in"], kx, ky, kz).cpu().numpy()
    wo = T.vorticity(g["rhs16_in"], *T.make_wavenumbers(16))
    assert np.abs(w - wo).max() < 1e-12
    gx = tgx.spectral_gradient(np.fft.fftn(g["rhs16_in"][0]), kx, ky, kz)
    go = T.spectral_gradient(np.fft.fftn(g["rhs16_in"][0]) * T.make_dealias_mask(16), *T.make_wavenumbers(16))
    for a, b in zip(gx, go):
        assert np.abs(a.cpu().numpy() - b).max() < 1e-12
    u, e, d = tgx.run_simulation(N=16, dt=0.005, reynolds=100, total_time=0.05,
                                 save_every_time=0.01, return_diagnostics=True, verbose=False)
    np.testing.assert_allclose(d["energy"], g["run16_energy"], rtol=1e-8)
    np.testing.assert_allclose(d["enstrophy"], g["run16_enstrophy"], rtol=1e-8)


# ---------------------------------------------------------------- cuda/test_taylor_green_cuda.py
def test_spectral_step_preserves_finite_values():
    from jax_tg_project_gb300 import spectral as S
    kx, ky, kz = S.make_wavenumbers(8, LENGTH)
    mask = S.make_dealias_mask(8, LENGTH)
    v = S.advance_one_step(S.initial_taylor_green_spectral(8, LENGTH), 0.005, LENGTH / 100.0,
                           kx, ky, kz, mask)
    assert bool(v.isfinite().all())


def test_spectral_short_run_is_finite(golden_cupy):
    from jax_tg_project_gb300 import spectral as S
    u, times, energies, enstrophies = S.run_simulation(n=8, dt=0.005, reynolds=100.0,
                                                       total_time=0.02, save_every_time=0.01,
                                                       verbose=False)
    assert bool(u.isfinite().all())
    assert len(times) == 3
    np.testing.assert_allclose(energies, golden_cupy["hdrun8_energies"], rtol=1e-6)
    np.testing.assert_allclose(enstrophies, golden_cupy["hdrun8_enstrophies"], rtol=1e-6)


def test_spectral_api_matches_reference(golden_cupy):
    from jax_tg_project_gb300 import spectral as S
    g = golden_cupy
    kx, ky, kz = S.make_wavenumbers(16)
    mask = S.make_dealias_mask(16)
    r = S.spectral_rhs(g["u_hat"], 0.02, kx, ky, kz, mask).cpu().numpy()
    assert np.linalg.norm(r - g["hd_rhs"]) / np.linalg.norm(g["hd_rhs"]) < 1e-5
    s = S.advance_one_step(g["u_hat"], 0.004, 0.02, kx, ky, kz, mask).cpu().numpy()
    assert np.linalg.norm(s - g["hd_step"]) / np.linalg.norm(g["hd_step"]) < 1e-5


# ---------------------------------------------------------------- cuda/test_taylor_green_mhd.py
def test_mhd_initial_condition_is_divergence_free():
    import torch

    from jax_tg_project_gb300 import mhd
    from jax_tg_project_gb300 import taylor_green as tgm
    u, b = mhd.initial_taylor_green_mhd(16, LENGTH, 0.5)
    kx, ky, kz = tgm.make_wavenumbers(16)
    assert float(tgm.spectral_divergence(u, kx, ky, kz).abs().max()) < 1e-5
    assert float(tgm.spectral_divergence(b.contiguous(), kx, ky, kz).abs().max()) < 1e-5
    assert isinstance(u, torch.Tensor)


def test_mhd_timestep_validation_rejects_unstable_values():
    from jax_tg_project_gb300 import mhd
    k = mhd.make_wavenumbers(16)
    nu = eta = LENGTH / 100.0
    with pytest.raises(ValueError, match="stability limit"):
        mhd.validate_timestep_mhd(1.0, nu, eta, *k)
    with pytest.raises(ValueError, match="positive"):
        mhd.validate_timestep_mhd(0.0, nu, eta, *k)


def test_mhd_short_run_is_finite_and_divergence_free(golden_cupy):
    from jax_tg_project_gb300 import mhd
    u, b, d = mhd.run_simulation(n=8, dt=0.005, reynolds=100.0, magnetic_reynolds=100.0,
                                 magnetic_amplitude=0.5, total_time=0.02, save_every_time=0.01,
                                 make_plots=False, lorentz_sign=-1.0, verbose=False)
    assert bool(u.isfinite().all()) and bool(b.isfinite().all())
    assert len(d.times) == 3
    assert max(d.divergence_u_max) < 1e-4 and max(d.divergence_b_max) < 1e-4
    np.testing.assert_allclose(d.kinetic_energies, golden_cupy["mhdrun8_kinetic_energies"], rtol=2e-6)
    np.testing.assert_allclose(d.magnetic_energies, golden_cupy["mhdrun8_magnetic_energies"], rtol=2e-6)


def test_mhd_step_preserves_finite_values():
    from jax_tg_project_gb300 import mhd
    uh, bh = mhd.initial_taylor_green_mhd_spectral(8, LENGTH, 0.5)
    k = mhd.make_wavenumbers(8)
    u2, b2 = mhd.advance_one_step(uh, bh, 0.005, LENGTH / 100.0, LENGTH / 100.0, *k,
                                  mhd.make_dealias_mask(8))
    assert bool(u2.isfinite().all()) and bool(b2.isfinite().all())


def test_mhd_rhs_api_matches_reference(golden_cupy):
    from jax_tg_project_gb300 import mhd
    g = golden_cupy
    k = mhd.make_wavenumbers(16)
    ru, rb = mhd.spectral_rhs_mhd(g["u_hat"], g["b_hat"], 0.02, 0.03, *k, mhd.make_dealias_mask(16),
                                  lorentz_sign=-1.0)
    assert np.linalg.norm(ru.cpu().numpy() - g["mhd_rhs_u"]) / np.linalg.norm(g["mhd_rhs_u"]) < 1e-5
    assert np.linalg.norm(rb.cpu().numpy() - g["mhd_rhs_b"]) / np.linalg.norm(g["mhd_rhs_b"]) < 1e-5


def test_magnetic_reynolds_conversion():
    from jax_tg_project_gb300 import mhd
    eta = mhd.magnetic_reynolds_to_resistivity(100.0)
    assert mhd.resistivity_to_magnetic_reynolds(eta) == pytest.approx(100.0, abs=1e-6)
    with pytest.raises(ValueError, match="magnetic_reynolds must be positive"):
        mhd.magnetic_reynolds_to_resistivity(-100.0)
