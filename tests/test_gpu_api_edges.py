"""Edge cases of the C entry points through the Plan wrapper: zero-step calls, record counts
of the run loop, argument errors (TG_E_INVALID / TG_E_UNSUPPORTED with the plan still
usable afterwards) and reduced dealiasing cutoffs."""
import pytest

pytestmark = pytest.mark.gpu


def _plan(n=16, **kw):
    import jax_tg_project_gb300 as tg
    return tg.Plan(n, precision="f32", **kw)


def test_zero_steps_leave_the_state_unchanged():
    import torch
    p = _plan()
    s = p.initial_condition("taylor_green", seed=2, pert_amp=0.05, k0=3.0)
    before = s.clone()
    p.step(s, dt=0.005, nu=0.01, nsteps=0)
    assert torch.equal(s, before)
    series = p.run(s, dt=0.005, nu=0.01, nsteps=0, save_every=3)
    assert series.shape[0] == 1
    assert torch.equal(s, before)
    assert torch.equal(series[0], p.diagnostics(s, nu=0.01))


@pytest.mark.parametrize("nsteps,save_every", [(5, 10), (6, 3), (7, 3), (1, 1)])
def test_run_records_follow_the_save_cadence(nsteps, save_every):
    """Records: the initial state, every save_every steps, and the last step (the reference's
    run loop, jax/taylor_green_jax.py:266-275)."""
    import torch
    p = _plan()
    a = p.initial_condition("taylor_green", seed=3, pert_amp=0.05, k0=3.0)
    b = a.clone()
    series = p.run(a, dt=0.005, nu=0.01, nsteps=nsteps, save_every=save_every)
    expect = 1 + nsteps // save_every + (1 if nsteps % save_every else 0)
    assert series.shape[0] == expect
    # record r holds the state after min(r * save_every, nsteps) steps
    done = 0
    for r in range(1, expect):
        target = min(r * save_every, nsteps)
        p.step(b, dt=0.005, nu=0.01, nsteps=target - done)
        done = target
        assert torch.equal(series[r], p.diagnostics(b, nu=0.01)), r
    assert torch.equal(a, b)


def test_argument_errors_leave_the_plan_usable():
    from jax_tg_project_gb300 import _abi
    p = _plan()
    s = p.initial_condition("taylor_green")
    cases = [
        lambda: p.step(s, dt=0.005, nu=0.01, nsteps=-1),   # negative step count
        lambda: p.step(s, dt=0.005, nu=-0.01, nsteps=1),   # negative viscosity
        lambda: p.step(s, nsteps=1),                       # dt <= 0 and no per-run table set
        lambda: p.run(s, dt=0.005, nu=0.01, nsteps=2, save_every=0),
    ]
    for case in cases:
        with pytest.raises(_abi.TgError) as e:
            case()
        assert e.value.code == _abi.TG_E_INVALID
    p.step(s, dt=0.005, nu=0.01, nsteps=2)  # still works
    d = p.diagnostics(s, nu=0.01).cpu().numpy()[0]
    assert 0.0 < d[0] < 0.125


def test_plan_creation_errors():
    import jax_tg_project_gb300 as tg
    from jax_tg_project_gb300 import _abi
    with pytest.raises(_abi.TgError) as e:
        tg.Plan(20)
    assert e.value.code == _abi.TG_E_UNSUPPORTED
    with pytest.raises(_abi.TgError) as e:
        tg.Plan(32, cutoff=11)  # above n/3
    assert e.value.code == _abi.TG_E_INVALID


@pytest.mark.parametrize("cutoff", [1, 4])
def test_reduced_cutoff_keeps_taylor_green_modes(cutoff):
    """A plan with a cutoff below n/3 stores |k_i| <= cutoff only; the Taylor-Green modes
    (|k_i| = 1) fit every cutoff >= 1, so E0 = 0.125 and enstrophy0 = 0.375, and with cutoff 1
    the nonlinear transfer to |k_i| = 2 is removed: the energy then decays as exp(-6 nu t)."""
    import math
    p = _plan(32, cutoff=cutoff)
    s = p.initial_condition("taylor_green")
    d0 = p.diagnostics(s, nu=0.01).cpu().numpy()[0]
    assert d0[0] == pytest.approx(0.125, rel=1e-7) and d0[1] == pytest.approx(0.375, rel=1e-7)
    p.step(s, dt=0.01, nu=0.01, nsteps=10)
    e = float(p.diagnostics(s, nu=0.01).cpu().numpy()[0, 0])
    if cutoff == 1:
        assert e == pytest.approx(0.125 * math.exp(-6 * 0.01 * 0.1), rel=1e-5)
    else:
        assert e < 0.125 * math.exp(-6 * 0.01 * 0.1) * (1 + 1e-6)


def test_each_coefficient_argument_applies_on_its_own():
    """A call that passes only eta (dt <= 0 and nu < 0: keep the per-run dt and nu) still
    applies eta: the MHD RHS with the table's nu and an explicit eta equals the one with both
    given."""
    import torch

    import jax_tg_project_gb300 as tg
    p = tg.Plan(16, physics="mhd", precision="f64")
    s = p.initial_condition("mhd_equal_energy", seed=3, pert_amp=0.05, k0=3.0)
    p.set_run_params(nu=0.01, eta=0.02, dt=1e-3)
    r_only_eta = p.rhs(s, nu=-1.0, eta=0.05)
    r_both = p.rhs(s, nu=0.01, eta=0.05)
    r_table = p.rhs(s, nu=0.01, eta=0.02)
    assert torch.equal(r_only_eta, r_both)
    assert not torch.equal(r_only_eta, r_table)
