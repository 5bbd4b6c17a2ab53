"""MHD RHS, RK4 step and diagnostics on the GPU against the reference fixtures
(cuda/taylor_green_mhd run with NumPy standing in for CuPy) and the oracle."""
import numpy as np
import pytest

from conftest import from_state, full_to_compact, rel_l2, to_state
from oracle import mhd_numpy as M
from oracle import tg_numpy as T

pytestmark = pytest.mark.gpu


def _plan(N, prec="f32", **kw):
    import jax_tg_project_gb300 as tg
    return tg.Plan(N, physics="mhd", precision=prec, **kw)


def _mhd_state(p, uh, bh):
    N = p.n
    c = np.concatenate([full_to_compact(uh, N), full_to_compact(bh, N)], axis=0)
    return to_state(p, c)


@pytest.mark.parametrize("prec,tol", [("f32", 1e-5), ("f64", 1e-12)])
def test_mhd_rhs_matches_reference(golden_cupy, prec, tol):
    g = golden_cupy
    p = _plan(16, prec, lorentz_sign=-1.0)
    s = _mhd_state(p, g["u_hat"], g["b_hat"])
    got = from_state(p, p.rhs(s, nu=0.02, eta=0.03))[0]
    want = np.concatenate([full_to_compact(g["mhd_rhs_u"], 16), full_to_compact(g["mhd_rhs_b"], 16)])
    assert rel_l2(got[:3], want[:3]) < tol
    assert rel_l2(got[3:], want[3:]) < tol


@pytest.mark.parametrize("prec,tol", [("f32", 1e-5), ("f64", 1e-12)])
def test_mhd_rhs_physical_sign_matches_oracle(golden_cupy, prec, tol):
    g = golden_cupy
    p = _plan(16, prec)  # physical +j x b
    s = _mhd_state(p, g["u_hat"], g["b_hat"])
    got = from_state(p, p.rhs(s, nu=0.02, eta=0.03))[0]
    ru, rb = M.spectral_rhs_mhd(M.Grid(16), g["u_hat"], g["b_hat"], 0.02, 0.03, lorentz_sign=1.0)
    assert rel_l2(got[:3], full_to_compact(ru, 16)) < tol
    assert rel_l2(got[3:], full_to_compact(rb, 16)) < tol


@pytest.mark.parametrize("prec,explicit,tol", [("f32", True, 1e-5), ("f32", False, 1e-5),
                                               ("f64", True, 1e-12), ("f64", False, 1e-8)])
def test_mhd_step_matches_reference(golden_cupy, prec, explicit, tol):
    g = golden_cupy
    p = _plan(16, prec, lorentz_sign=-1.0, explicit_viscosity=explicit)
    s = _mhd_state(p, g["u_hat"], g["b_hat"])
    p.step(s, dt=0.004, nu=0.02, eta=0.03, nsteps=1)
    got = from_state(p, s)[0]
    assert rel_l2(got[:3], full_to_compact(g["mhd_step_u"], 16)) < tol
    assert rel_l2(got[3:], full_to_compact(g["mhd_step_b"], 16)) < tol


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_mhd_diagnostics_match_reference(golden_cupy, prec):
    g = golden_cupy
    p = _plan(16, prec)
    s = _mhd_state(p, g["u_hat"], g["b_hat"])
    d = p.diagnostics(s, nu=0.02, eta=0.03).cpu().numpy()[0]
    ek, em, hc, ens = g["mhd_record"]
    tol = 1e-6 if prec == "f32" else 1e-12
    assert d[0] == pytest.approx(ek, rel=tol)
    assert d[3] == pytest.approx(em, rel=tol)
    assert d[4] == pytest.approx(hc, rel=tol)
    assert d[1] == pytest.approx(ens, rel=tol)
    assert d[5] == pytest.approx(ek + em, rel=tol)


def test_mhd_initial_conditions():
    p = _plan(16, "f64")
    s = p.initial_condition("mhd_equal_energy")
    d = p.diagnostics(s, nu=0.0, eta=0.0).cpu().numpy()[0]
    assert d[0] == pytest.approx(0.125, rel=1e-13) and d[3] == pytest.approx(0.125, rel=1e-13)
    vel, mag = M.initial_mhd_equal_energy(16)
    u = p.inverse(s)[0].cpu().numpy()
    assert np.abs(u[:3] - vel).max() < 1e-13 and np.abs(u[3:] - mag).max() < 1e-13
    s = p.initial_condition("mhd_reference", b_amp=0.5)
    vel, mag = M.initial_taylor_green_mhd(16, magnetic_amplitude=0.5)
    u = p.inverse(s)[0].cpu().numpy()
    assert np.abs(u[:3] - vel).max() < 1e-13 and np.abs(u[3:] - mag).max() < 1e-13


def test_mhd_run_matches_reference_run(golden_cupy):
    """TaylorGreenMhdSimulation n=8, Re=Rm=100 (cuda/test_taylor_green_mhd.py:51-67)."""
    g = golden_cupy
    p = _plan(8, "f64", lorentz_sign=-1.0, explicit_viscosity=True)
    s = p.initial_condition("mhd_reference", b_amp=0.5)
    nu = 2 * np.pi / 100
    series = p.run(s, dt=0.005, nu=nu, eta=nu, nsteps=4, save_every=2).cpu().numpy()[:, 0]
    # the reference samples its initial grid in float32, hence 1e-6
    np.testing.assert_allclose(series[:, 0], g["mhdrun8_kinetic_energies"], rtol=1e-6)
    np.testing.assert_allclose(series[:, 3], g["mhdrun8_magnetic_energies"], rtol=1e-6)
    np.testing.assert_allclose(series[:, 4], g["mhdrun8_cross_helicities"], rtol=1e-6)
    np.testing.assert_allclose(series[:, 1], g["mhdrun8_enstrophies"], rtol=1e-6)
    assert series[:, 6].max() < 1e-4 and series[:, 7].max() < 1e-4


@pytest.mark.parametrize("N", [16, 32, 64, 128])
def test_mhd_register_and_shared_memory_passes_agree(N, monkeypatch):
    """Register-resident MHD z pass against the shared-memory one (FP32 round-off)."""
    outs = []
    for variant in ("0", "3"):
        monkeypatch.setenv("TG_PASS_VARIANT", variant)
        p = _plan(N, "f32")
        s = p.initial_condition("mhd_equal_energy", seed=2, pert_amp=0.05, k0=3.0)
        p.step(s, dt=1e-3, nu=2e-3, eta=3e-3, nsteps=3)
        outs.append(from_state(p, s)[0])
    assert rel_l2(outs[0], outs[1]) < 2e-6


def test_autotuned_batched_mhd_plan_matches_runs_one_at_a_time():
    """An autotuned batched MHD plan (per-run nu, eta) equals plain single-run plans."""
    import jax_tg_project_gb300 as tg
    nus, etas = [2e-3, 4e-3], [3e-3, 1e-3]
    pb = tg.Plan(32, batch=2, physics="mhd", precision="f32", autotune=True)
    sb = pb.initial_condition("mhd_equal_energy", seed=5, pert_amp=0.02, k0=3.0)
    pb.set_run_params(nu=nus, eta=etas, dt=[1e-3, 1e-3])
    pb.step(sb, nsteps=4)
    for r in range(2):
        p1 = tg.Plan(32, physics="mhd", precision="f32")
        s1 = p1.initial_condition("mhd_equal_energy", seed=5 + r, pert_amp=0.02, k0=3.0)
        p1.step(s1, dt=1e-3, nu=nus[r], eta=etas[r], nsteps=4)
        assert rel_l2(from_state(p1, s1)[0], from_state(pb, sb)[r]) < 2e-6
