"""Pin the NumPy oracle against the reference's own outputs (CPU only).

The fixtures in tests/golden/ were produced by the reference's Python code
(jax/taylor_green_jax.py and the CuPy packages) with NumPy standing in for
jax.numpy / cupy; see tests/golden/make_golden.py.  The invariant tests at the
end port jax/test_taylor_green_jax.py, cuda/test_taylor_green_cuda.py and
cuda/test_taylor_green_mhd.py to the oracle.
"""
import math

import numpy as np
import pytest

from conftest import rel_l2, unpack_sparse
from oracle import mhd_numpy as M
from oracle import perturb
from oracle import tg_numpy as T

L = 2.0 * math.pi


# ------------------------------------------------------------------ hydro pins
def test_ic_diagnostics_match_reference(golden_hydro):
    g = golden_hydro
    N = 16
    kx, ky, kz = T.make_wavenumbers(N)
    u0 = T.initial_taylor_green(N)
    assert T.kinetic_energy(u0) == pytest.approx(float(g["ic16_energy"]), rel=1e-14)
    assert T.enstrophy(u0, kx, ky, kz) == pytest.approx(float(g["ic16_enstrophy"]), rel=1e-13)
    assert T.viscous_dissipation(u0, 0.01, kx, ky, kz) == pytest.approx(
        float(g["ic16_dissipation"]), rel=1e-13)
    assert int(T.make_dealias_mask(N).sum()) == int(g["mask16_count"]) == 11 ** 3
    assert T.validate_timestep(0.005, 0.01, kx, ky, kz) == pytest.approx(float(g["limit16"]))
    # analytic known answers: E0 = 1/8, enstrophy0 = 3/8
    assert T.kinetic_energy(u0) == pytest.approx(0.125, rel=1e-14)
    assert T.enstrophy(u0, kx, ky, kz) == pytest.approx(0.375, rel=1e-13)


def test_rhs_and_step_match_reference(golden_hydro):
    g = golden_hydro
    N = 16
    kx, ky, kz = T.make_wavenumbers(N)
    mask = T.make_dealias_mask(N)
    uin = g["rhs16_in"]
    assert rel_l2(T.spectral_rhs(uin, 0.01, kx, ky, kz, mask), g["rhs16_out"]) < 1e-13
    assert rel_l2(T.advance_one_step(uin, 0.005, 0.01, kx, ky, kz, mask), g["step16_out"]) < 1e-14
    k8 = T.make_wavenumbers(8)
    const = T.spectral_rhs(np.ones((3, 8, 8, 8)), 0.01, *k8, T.make_dealias_mask(8))
    assert np.max(np.abs(const)) < 1e-12 and np.max(np.abs(g["rhs8_const"])) < 1e-12


@pytest.mark.parametrize("form,integrator,tol", [
    ("rotational", "explicit", 1e-12), ("advective", "lawson", 1e-9),
    ("rotational", "lawson", 1e-9)])
def test_scheme_variants_agree_with_reference(golden_hydro, form, integrator, tol):
    """The rotational form and Lawson RK4 used on the GPU differ from the
    reference only at round-off / truncation level for band-limited fields."""
    g = golden_hydro
    N = 16
    kx, ky, kz = T.make_wavenumbers(N)
    mask = T.make_dealias_mask(N)
    out = T.advance_one_step(g["rhs16_in"], 0.005, 0.01, kx, ky, kz, mask, form, integrator)
    assert rel_l2(out, g["step16_out"]) < tol


@pytest.mark.parametrize("case,kw", [
    ("run8", dict(N=8, dt=0.005, nu=0.01, total_time=0.02, save_every_time=0.01)),
    ("run16", dict(N=16, dt=0.005, reynolds=100, total_time=0.05, save_every_time=0.01)),
])
def test_run_simulation_matches_reference(golden_hydro, case, kw):
    g = golden_hydro
    u, e, d = T.run_simulation(return_diagnostics=True, **kw)
    assert rel_l2(u, g[f"{case}_u"]) < 1e-13
    assert d["time"] == list(g[f"{case}_time"])
    for key in ("energy", "enstrophy", "dissipation"):
        np.testing.assert_allclose(d[key], g[f"{case}_{key}"], rtol=1e-13)
    assert max(d["divergence_max"]) < 1e-12


def test_tg64_first_saves_match_reference(golden_tg64):
    """First 20 steps of the 64^3 nu=1/1600 run reproduce the reference series."""
    g = golden_tg64
    _, _, d = T.run_simulation(N=64, dt=1e-3, nu=1 / 1600, total_time=0.02,
                               save_every_time=0.01, return_diagnostics=True)
    for key in ("energy", "enstrophy", "dissipation"):
        np.testing.assert_allclose(d[key], g[f"series_{key}"][:3], rtol=1e-13)
    # the sparse 100/200-step fields are consistent with the series
    c200 = unpack_sparse(g, "c200")
    ke, ens, diss = T.compact_diagnostics(c200, nu=1 / 1600)
    assert ke == pytest.approx(g["series_energy"][-1], rel=1e-12)
    assert ens == pytest.approx(g["series_enstrophy"][-1], rel=1e-12)
    assert diss == pytest.approx(g["series_dissipation"][-1], rel=1e-12)


# ------------------------------------------------------------------ CuPy HD / MHD pins
def test_cupy_hd_rhs_and_step_match_reference(golden_cupy):
    g = golden_cupy
    N = 16
    kx, ky, kz = T.make_wavenumbers(N)
    mask = T.make_dealias_mask(N)
    assert rel_l2(T.spectral_rhs_spectral(g["u_hat"], 0.02, kx, ky, kz, mask), g["hd_rhs"]) < 1e-13
    assert rel_l2(T.advance_one_step_spectral(g["u_hat"], 0.004, 0.02, kx, ky, kz, mask),
                  g["hd_step"]) < 1e-14


def test_cupy_mhd_rhs_step_record_match_reference(golden_cupy):
    g = golden_cupy
    G = M.Grid(16)
    ru, rb = M.spectral_rhs_mhd(G, g["u_hat"], g["b_hat"], 0.02, 0.03, lorentz_sign=-1.0)
    assert rel_l2(ru, g["mhd_rhs_u"]) < 1e-13
    assert rel_l2(rb, g["mhd_rhs_b"]) < 1e-13
    su, sb = M.rk4_step(G, g["u_hat"], g["b_hat"], 0.004, 0.02, 0.03, lorentz_sign=-1.0)
    assert rel_l2(su, g["mhd_step_u"]) < 1e-14
    assert rel_l2(sb, g["mhd_step_b"]) < 1e-14
    rec = M.record(G, g["u_hat"], g["b_hat"])
    got = [rec["kinetic_energy"], rec["magnetic_energy"], rec["cross_helicity"], rec["enstrophy"]]
    np.testing.assert_allclose(got, g["mhd_record"], rtol=1e-13)
    # the physical sign differs from the reference's by twice the Lorentz term
    ru_p, _ = M.spectral_rhs_mhd(G, g["u_hat"], g["b_hat"], 0.02, 0.03, lorentz_sign=1.0)
    assert rel_l2(ru_p, g["mhd_rhs_u"]) > 1e-3


def test_cupy_runs_match_reference(golden_cupy):
    g = golden_cupy
    # HD package run: n=8, Re=100 (nu = L/Re), float32 initial grid
    G = M.Grid(8)
    kx, ky, kz, mask = G.kx, G.ky, G.kz, G.mask
    vel, _ = M.initial_taylor_green_mhd(8, dtype=np.float32)
    s = T.to_spectral(vel, mask)
    nu = L / 100.0
    for _ in range(4):
        s = T.advance_one_step_spectral(s, 0.005, nu, kx, ky, kz, mask)
    assert rel_l2(s, g["hdrun8_state"]) < 1e-6  # float32 IC rounding in the reference
    u_hat, b_hat, series = M.run_simulation(n=8, dt=0.005, reynolds=100.0,
                                            magnetic_reynolds=100.0, total_time=0.02,
                                            save_every_time=0.01)
    assert series["time"] == list(g["mhdrun8_times"])
    for k, rk in (("kinetic_energy", "kinetic_energies"), ("magnetic_energy", "magnetic_energies"),
                  ("cross_helicity", "cross_helicities"), ("enstrophy", "enstrophies")):
        np.testing.assert_allclose(series[k], g[f"mhdrun8_{rk}"], rtol=1e-6)


# ------------------------------------------------------------------ ported reference invariants
def test_initial_condition_is_divergence_free():  # jax/test_taylor_green_jax.py:22-26
    kx, ky, kz = T.make_wavenumbers(16)
    assert np.max(np.abs(T.spectral_divergence(T.initial_taylor_green(16), kx, ky, kz))) < 1e-12


def test_dealias_mask_keeps_two_thirds():  # jax/test_taylor_green_jax.py:29-34
    m = T.make_dealias_mask(16)
    assert m.shape == (16, 16, 16) and int(m.sum()) == 11 ** 3
    assert not bool(m[8, 0, 0]) and bool(m[5, 0, 0])


def test_timestep_validation_messages():  # jax/test_taylor_green_jax.py:37-42
    kx, ky, kz = T.make_wavenumbers(16)
    with pytest.raises(ValueError, match="stability limit"):
        T.validate_timestep(1.0, 0.01, kx, ky, kz)
    with pytest.raises(ValueError, match="positive"):
        T.validate_timestep(0.0, 0.01, kx, ky, kz)


def test_reynolds_conversions():  # jax/test_taylor_green_jax.py:77-83,96-98
    assert T.viscosity_to_reynolds(T.reynolds_to_viscosity(100.0)) == pytest.approx(100.0, abs=1e-10)
    with pytest.raises(ValueError, match="Reynolds number must be positive"):
        T.reynolds_to_viscosity(-100)


def test_mhd_config_invariants():  # cuda/test_taylor_green_mhd.py:42-49,80-88
    G = M.Grid(16)
    with pytest.raises(ValueError, match="stability limit"):
        M.validate_timestep(1.0, L / 100, L / 100, G)
    with pytest.raises(ValueError, match="positive"):
        M.validate_timestep(0.0, L / 100, L / 100, G)
    eta = M.magnetic_reynolds_to_resistivity(100.0)
    assert M.resistivity_to_magnetic_reynolds(eta) == pytest.approx(100.0, abs=1e-6)
    with pytest.raises(ValueError, match="magnetic_reynolds must be positive"):
        M.magnetic_reynolds_to_resistivity(-100.0)


def test_equal_energy_mhd_field():
    vel, mag = M.initial_mhd_equal_energy(16)
    G = M.Grid(16)
    rec = M.record(G, G.to_spectral(vel), G.to_spectral(mag))
    assert rec["kinetic_energy"] == pytest.approx(0.125, rel=1e-13)
    assert rec["magnetic_energy"] == pytest.approx(0.125, rel=1e-13)
    assert rec["divergence_b_max"] < 1e-12


# ------------------------------------------------------------------ perturbation definition
@pytest.mark.parametrize("N", [16, 32, 24])
def test_perturbation_properties(N):
    c = perturb.perturbation_compact(N, seed=5, amp=1e-3, k0=4.0)
    u = T.physical_from_compact(c, N)
    assert np.sqrt(np.mean(np.sum(u * u, axis=0)) / 3.0) == pytest.approx(1e-3, rel=1e-12)
    kx, ky, kz = T.make_wavenumbers(N)
    assert np.max(np.abs(T.spectral_divergence(u, kx, ky, kz))) < 1e-15
    # band-limited: round trip through the compact layout is exact
    assert rel_l2(T.compact_from_physical(u), c) < 1e-13
    c2 = perturb.perturbation_compact(N, seed=6, amp=1e-3, k0=4.0)
    assert rel_l2(c, c2) > 0.5


def test_splitmix64_known_answers():
    # SplitMix64 stream from state 0 (Vigna's reference generator): the first
    # outputs are splitmix64(k * golden_gamma) for k = 0, 1, 2
    out = perturb.splitmix64(np.array([0, 0x9E3779B97F4A7C15, 0x3C6EF372FE94F82A], dtype=np.uint64))
    assert [int(x) for x in out] == [0xE220A8397B1DCDAF, 0x6E789E6AA1B965F4, 0x06C45D188009454F]


def _band_limited(N, seed):
    """A real, solenoidal, dealiased random field: the compact layout holds it exactly."""
    rng = np.random.default_rng(seed)
    kx, ky, kz = T.make_wavenumbers(N)
    mask = T.make_dealias_mask(N)
    uh = np.fft.fftn(rng.standard_normal((3, N, N, N)), axes=(-3, -2, -1)) * mask
    k2 = kx * kx + ky * ky + kz * kz
    k2[0, 0, 0] = 1.0
    div = (kx * uh[0] + ky * uh[1] + kz * uh[2]) / k2
    uh = uh - np.stack([kx, ky, kz]) * div
    return np.real(np.fft.ifftn(uh, axes=(-3, -2, -1))), kx, ky, kz


@pytest.mark.parametrize("N", [12, 16, 24])
def test_compact_layout_round_trip_and_parseval(N):
    """The oracle's compact half-spectrum helpers (the reference layout of the GPU state tests):
    physical -> compact -> physical is the identity on dealiased real fields, and Parseval on the
    compact coefficients equals the reference's physical-space diagnostics."""
    u, kx, ky, kz = _band_limited(N, seed=N)
    c = T.compact_from_physical(u)
    K = N // 3
    assert c.shape == (3, 2 * K + 1, 2 * K + 1, K + 1)
    np.testing.assert_allclose(T.physical_from_compact(c, N), u, rtol=0, atol=1e-12)
    ke, ens, diss = T.compact_diagnostics(c, nu=0.01)[:3]
    assert ke == pytest.approx(T.kinetic_energy(u), rel=1e-12)
    assert ens == pytest.approx(T.enstrophy(u, kx, ky, kz), rel=1e-12)
    assert diss == pytest.approx(T.viscous_dissipation(u, 0.01, kx, ky, kz), rel=1e-12)


# ------------------------------------------------------------------ torch restatement pins
def test_torch_restatement_matches_reference(golden_hydro):
    """oracle/tg_torch.py (the reverse-mode reference for the adjoint tests) against the
    reference's own outputs: RHS and one RK4 step at 16^3, the enstrophy of the Taylor-Green
    state, and the run series (jax/taylor_green_jax.py:158-201, run8 / run16 cases)."""
    import torch

    from oracle import tg_torch as TT
    g = golden_hydro
    kx, ky, kz, mask = TT._grid(16)
    uin = torch.from_numpy(np.asarray(g["rhs16_in"], dtype=np.float64))
    assert rel_l2(TT.spectral_rhs(uin, 0.01, kx, ky, kz, mask).numpy(), g["rhs16_out"]) < 1e-13
    assert rel_l2(TT.advance_one_step(uin, 0.005, 0.01, kx, ky, kz, mask).numpy(),
                  g["step16_out"]) < 1e-14
    u0 = torch.from_numpy(T.initial_taylor_green(16))
    assert float(TT.enstrophy(u0, kx, ky, kz)) == pytest.approx(float(g["ic16_enstrophy"]), rel=1e-13)
    for case, N, nu, nsteps in (("run8", 8, 0.01, 4), ("run16", 16, 2 * np.pi / 100, 10)):
        kx, ky, kz, mask = TT._grid(N)
        u = torch.from_numpy(T.initial_taylor_green(N))
        ens = [float(TT.enstrophy(u, kx, ky, kz))]
        for s in range(nsteps):
            u = TT.advance_one_step(u, 0.005, nu, kx, ky, kz, mask)
            if (s + 1) % 2 == 0:
                ens.append(float(TT.enstrophy(u, kx, ky, kz)))
        np.testing.assert_allclose(ens, g[f"{case}_enstrophy"], rtol=1e-12)
        assert rel_l2(u.numpy(), g[f"{case}_u"]) < 1e-12
    # final_enstrophy is the composition of the two pinned pieces
    L = TT.final_enstrophy(torch.from_numpy(T.initial_taylor_green(8)), 0.01, 0.005, 4)
    assert float(L) == pytest.approx(float(g["run8_enstrophy"][-1]), rel=1e-12)
