"""Hydro RHS, RK4 step and run loop on the GPU against the reference fixtures.

Fixtures come from the reference's own jax/taylor_green_jax.py (see
tests/golden/make_golden.py).  Tolerances: FP32 kernels 1e-5 relative L2 on
fields and 1e-6 relative on diagnostics (the parity bar of the hot path);
FP64 kernels 1e-12.
"""
import numpy as np
import pytest

from conftest import from_state, rel_l2, to_state, unpack_sparse
from oracle import tg_numpy as T

pytestmark = pytest.mark.gpu


def _plan(N, prec="f32", **kw):
    import jax_tg_project_gb300 as tg
    return tg.Plan(N, precision=prec, **kw)


def _phys_to_state(p, u):
    import torch
    return p.forward(torch.from_numpy(np.asarray(u)[None]).to(p.real_dtype).cuda().contiguous())


@pytest.mark.parametrize("prec,tol", [("f32", 1e-5), ("f64", 1e-12)])
def test_rhs_matches_reference(golden_hydro, prec, tol):
    g = golden_hydro
    p = _plan(16, prec)
    s = _phys_to_state(p, g["rhs16_in"])
    r = p.rhs(s, nu=0.01)
    got = p.inverse(r)[0].double().cpu().numpy()
    assert rel_l2(got, g["rhs16_out"]) < tol


def test_zero_mode_is_not_damped():  # jax/test_taylor_green_jax.py:45-51
    p = _plan(8, "f64")
    s = _phys_to_state(p, np.ones((3, 8, 8, 8)))
    r = p.inverse(p.rhs(s, nu=0.01))[0].cpu().numpy()
    assert np.abs(r).max() < 1e-12


@pytest.mark.parametrize("prec,explicit,tol", [("f32", False, 1e-5), ("f32", True, 1e-5),
                                               ("f64", False, 1e-9), ("f64", True, 1e-12)])
def test_step_matches_reference(golden_hydro, prec, explicit, tol):
    g = golden_hydro
    p = _plan(16, prec, explicit_viscosity=explicit)
    s = _phys_to_state(p, g["rhs16_in"])
    p.step(s, dt=0.005, nu=0.01, nsteps=1)
    got = p.inverse(s)[0].double().cpu().numpy()
    assert rel_l2(got, g["step16_out"]) < tol


@pytest.mark.parametrize("case,N,nu,nsteps", [("run8", 8, 0.01, 4), ("run16", 16, 2 * np.pi / 100, 10)])
def test_run_series_matches_reference(golden_hydro, case, N, nu, nsteps):
    g = golden_hydro
    for prec, tol in (("f32", 1e-6), ("f64", 1e-12)):
        p = _plan(N, prec, explicit_viscosity=True)
        s = p.initial_condition("taylor_green")
        series = p.run(s, dt=0.005, nu=nu, nsteps=nsteps, save_every=2).cpu().numpy()[:, 0]
        np.testing.assert_allclose(series[:, 0], g[f"{case}_energy"], rtol=tol)
        np.testing.assert_allclose(series[:, 1], g[f"{case}_enstrophy"], rtol=tol)
        np.testing.assert_allclose(series[:, 2], g[f"{case}_dissipation"], rtol=tol)
        assert series[:, 6].max() < (1e-5 if prec == "f32" else 1e-10)
        u = p.inverse(s)[0].double().cpu().numpy()
        assert rel_l2(u, g[f"{case}_u"]) < (1e-6 if prec == "f32" else 1e-12)


def test_tg64_100_steps_velocity_parity(golden_tg64):
    """The parity bar: 64^3, nu=1/1600, dt=1e-3, 100 steps, FP32 kernels vs FP64 reference."""
    c100 = unpack_sparse(golden_tg64, "c100")
    for explicit in (False, True):
        p = _plan(64, "f32", explicit_viscosity=explicit)
        s = p.initial_condition("taylor_green")
        p.step(s, dt=1e-3, nu=1 / 1600, nsteps=100)
        err = rel_l2(from_state(p, s)[0], c100)
        assert err < 1e-5, err


def test_tg64_series_parity(golden_tg64):
    g = golden_tg64
    p = _plan(64, "f32")
    s = p.initial_condition("taylor_green")
    series = p.run(s, dt=1e-3, nu=1 / 1600, nsteps=200, save_every=10).cpu().numpy()[:, 0]
    for col, key in ((0, "energy"), (1, "enstrophy"), (2, "dissipation")):
        np.testing.assert_allclose(series[:, col], g[f"series_{key}"], rtol=1e-6)
    assert rel_l2(from_state(p, s)[0], unpack_sparse(g, "c200")) < 1e-5
    assert all(a >= b for a, b in zip(series[:, 0], series[1:, 0]))  # energy decays


def test_fp64_tracks_reference_to_roundoff(golden_tg64):
    p = _plan(64, "f64", explicit_viscosity=True)
    s = p.initial_condition("taylor_green")
    p.step(s, dt=1e-3, nu=1 / 1600, nsteps=100)
    assert rel_l2(from_state(p, s)[0], unpack_sparse(golden_tg64, "c100")) < 1e-12


def test_batched_runs_are_independent():
    """A batch of runs with different nu equals the runs done one at a time."""
    import torch
    nus = [0.01, 0.002, 0.0005]
    pb = _plan(32, "f32", batch=3)
    sb = pb.initial_condition("taylor_green", seed=3, pert_amp=1e-2, k0=4.0)
    pb.set_run_params(nu=nus, eta=[0.0] * 3, dt=[2e-3] * 3)
    pb.step(sb, nsteps=5)
    for r, nu in enumerate(nus):
        p1 = _plan(32, "f32")
        s1 = p1.initial_condition("taylor_green", seed=3 + r, pert_amp=1e-2, k0=4.0)
        p1.step(s1, dt=2e-3, nu=nu, nsteps=5)
        assert torch.equal(s1[0], sb[r])


@pytest.mark.parametrize("N", [16, 32, 64, 96, 128])
def test_register_and_shared_memory_passes_agree(N, monkeypatch):
    """The register-resident x/z passes and the shared-memory passes are two
    implementations of the same step; every mix of them (TG_PASS_VARIANT bit 0: z, bit 1:
    x, bit 2: the x stage with a shared-memory stash, built at 64 ... 256) agrees with the
    register-resident step to FP32 round-off."""
    steps, rhss = [], []
    for variant in ("0", "1", "2", "3", "4", "5"):
        monkeypatch.setenv("TG_PASS_VARIANT", variant)
        p = _plan(N, "f32")
        assert p.variant == int(variant)
        s = p.initial_condition("taylor_green", seed=9, pert_amp=0.05, k0=3.0)
        p.step(s, dt=2e-3, nu=2e-3, nsteps=3)
        steps.append(from_state(p, s)[0])
        r = p.rhs(p.initial_condition("taylor_green", seed=9, pert_amp=0.05, k0=3.0), nu=2e-3)
        rhss.append(from_state(p, r)[0])
    for k in range(1, 6):
        assert rel_l2(steps[0], steps[k]) < 2e-6, k
        assert rel_l2(rhss[0], rhss[k]) < 2e-6, k


@pytest.mark.parametrize("N,physics", [(32, "hydro"), (96, "hydro"), (128, "hydro"), (64, "mhd")])
def test_autotuned_plan_matches_default(N, physics, monkeypatch):
    """TG_FLAG_AUTOTUNE picks one of the variants by timing; the step it runs agrees with
    the default plan's to FP32 round-off."""
    import jax_tg_project_gb300 as tg
    monkeypatch.delenv("TG_PASS_VARIANT", raising=False)
    ic = "mhd_equal_energy" if physics == "mhd" else "taylor_green"
    outs = []
    for auto in (False, True):
        p = tg.Plan(N, physics=physics, precision="f32", autotune=auto)
        assert p.variant in ((0, 1, 2, 3, 4, 5) if auto else (0,))
        s = p.initial_condition(ic, seed=4, pert_amp=0.05, k0=3.0)
        p.step(s, dt=1e-3, nu=2e-3, eta=2e-3, nsteps=3)
        outs.append(from_state(p, s)[0])
    assert rel_l2(outs[0], outs[1]) < 2e-6


def test_fp32_step_tracks_fp64_gpu_run_at_256():
    """The 256^3 throughput workload checked against an FP64 GPU run of the same steps."""
    p32 = _plan(256, "f32")
    p64 = _plan(256, "f64")
    s32 = p32.initial_condition("taylor_green")
    s64 = p64.initial_condition("taylor_green")
    d32 = p32.run(s32, dt=2.5e-4, nu=1 / 1600, nsteps=20, save_every=10).cpu().numpy()[:, 0]
    d64 = p64.run(s64, dt=2.5e-4, nu=1 / 1600, nsteps=20, save_every=10).cpu().numpy()[:, 0]
    for col in (0, 1, 2):  # energy, enstrophy, dissipation
        np.testing.assert_allclose(d32[:, col], d64[:, col], rtol=1e-6)
    a = from_state(p32, s32)[0]
    b = from_state(p64, s64)[0]
    assert rel_l2(a, b) < 1e-5
    del p32, p64


def test_run_reports_non_finite_state():
    """Failure detection without a GPU fault: a NaN placed in a host-built state makes
    tg_run return TG_E_NONFINITE, and the plan keeps working afterwards."""
    import torch

    from jax_tg_project_gb300 import _abi
    p = _plan(16, "f32")
    s = p.initial_condition("taylor_green")
    host = s.cpu()
    host[0, 0, 1, 1, 1] = complex(float("nan"), 0.0)
    bad = host.to(p.device)
    with pytest.raises(_abi.TgError) as e:
        p.run(bad, dt=0.005, nu=0.01, nsteps=4, save_every=2)
    assert e.value.code == _abi.TG_E_NONFINITE and "record 0" in str(e.value)
    good = p.initial_condition("taylor_green")
    series = p.run(good, dt=0.005, nu=0.01, nsteps=4, save_every=2)
    assert torch.isfinite(series).all()


def test_512_transforms_and_early_steps_match_256():
    """512^3 (shared-memory passes): the forward / inverse transforms round-trip, and a few
    early steps of Taylor-Green agree with the 256^3 run on the modes both keep (the flow is
    still band-limited far below both cutoffs, so only round-off separates them)."""
    import torch

    import jax_tg_project_gb300 as tg
    p5 = tg.Plan(512, precision="f32")
    s5 = p5.initial_condition("taylor_green")
    u = p5.inverse(s5)
    back = p5.forward(u)
    assert rel_l2(from_state(p5, back)[0], from_state(p5, s5)[0]) < 1e-6
    p2 = tg.Plan(256, precision="f32")
    s2 = p2.initial_condition("taylor_green")
    for p, s in ((p5, s5), (p2, s2)):
        p.step(s, dt=2e-3, nu=1 / 1600, nsteps=3)
    d5 = p5.diagnostics(s5, nu=1 / 1600).cpu().numpy()[0]
    d2 = p2.diagnostics(s2, nu=1 / 1600).cpu().numpy()[0]
    np.testing.assert_allclose(d5[:3], d2[:3], rtol=1e-6)
    # the coefficients |k| <= 4 (compact index ranges of both grids)
    c5, c2 = from_state(p5, s5)[0], from_state(p2, s2)[0]
    k5 = [i for i in range(c5.shape[1]) if min(i, c5.shape[1] - i) <= 4]
    k2 = [i for i in range(c2.shape[1]) if min(i, c2.shape[1] - i) <= 4]
    lo5 = c5[:, k5][:, :, k5][..., :5]
    lo2 = c2[:, k2][:, :, k2][..., :5]
    assert rel_l2(lo5, lo2) < 1e-5
    del p5, p2
    torch.cuda.empty_cache()


@pytest.mark.parametrize("physics", ["hydro", "mhd"])
def test_run_in_chunks_matches_step(physics):
    """Plan.run loads the state once and carries the inverse-x fields across its diagnostics
    records (which go through other scratch): the final state equals Plan.step's bit for bit."""
    import torch

    import jax_tg_project_gb300 as tg
    p = tg.Plan(32, physics=physics, precision="f32")
    kind = "taylor_green" if physics == "hydro" else "mhd_equal_energy"
    a = p.initial_condition(kind, seed=5, pert_amp=0.03, k0=3.0)
    b = a.clone()
    series = p.run(a, dt=2e-3, nu=0.004, eta=0.003, nsteps=7, save_every=3)
    p.step(b, dt=2e-3, nu=0.004, eta=0.003, nsteps=7)
    assert series.shape[0] == 4
    assert torch.equal(a, b)
    d = p.diagnostics(b, nu=0.004, eta=0.003)
    assert torch.equal(series[-1], d)


@pytest.mark.parametrize("N", [32, 64, 128, 256])
def test_y_configurations_agree(N, monkeypatch):
    """Every y-pass configuration (radix plan, kz columns per CTA) the autotuner may pick
    gives the default configuration's step to FP32 round-off."""
    import jax_tg_project_gb300 as tg
    monkeypatch.delenv("TG_PASS_VARIANT", raising=False)
    count = tg.Plan(N, precision="f32").y_config[1]
    assert count >= 2
    outs = []
    for y in range(count):
        monkeypatch.setenv("TG_Y_CONF", str(y))
        p = tg.Plan(N, precision="f32")
        assert p.y_config == (y, count)
        s = p.initial_condition("taylor_green", seed=9, pert_amp=0.05, k0=3.0)
        p.step(s, dt=2e-3, nu=2e-3, nsteps=2)
        outs.append(from_state(p, s)[0])
    for y in range(1, count):
        assert rel_l2(outs[0], outs[y]) < 2e-6, y


def test_autotune_cache_is_written_and_read(tmp_path, monkeypatch):
    """TG_AUTOTUNE_CACHE: a tuned plan appends its choice; a later plan of the same key takes
    the cached choice instead of timing (shown by editing the cached values)."""
    import jax_tg_project_gb300 as tg
    monkeypatch.delenv("TG_PASS_VARIANT", raising=False)
    monkeypatch.delenv("TG_Y_CONF", raising=False)
    cache = tmp_path / "tune.txt"
    monkeypatch.setenv("TG_AUTOTUNE_CACHE", str(cache))
    p = tg.Plan(64, batch=2, precision="f32", autotune=True)
    lines = cache.read_text().splitlines()
    assert len(lines) == 1 and " n=64 batch=2 " in lines[0]
    assert lines[0].endswith(f"variant={p.variant} yconf={p.y_config[0]}")
    forced_v, forced_y = (p.variant + 1) % 4, (p.y_config[0] + 1) % p.y_config[1]
    key = lines[0][: lines[0].index(" variant=")]
    cache.write_text(lines[0] + "\n" + f"{key} variant={forced_v} yconf={forced_y}\n")
    q = tg.Plan(64, batch=2, precision="f32", autotune=True)
    assert (q.variant, q.y_config[0]) == (forced_v, forced_y)
    assert len(cache.read_text().splitlines()) == 2  # a cache hit appends nothing
    r = tg.Plan(64, batch=3, precision="f32", autotune=True)  # another key: tuned and appended
    assert len(cache.read_text().splitlines()) == 3
    del p, q, r


@pytest.mark.parametrize("explicit", [False, True])
def test_stashed_x_stage_matches_register_x_stage_at_256(explicit, monkeypatch):
    """The stashed x stage (variant bit 2) and the register-resident one run the same
    arithmetic on the 256^3 workload: three steps of a perturbed field agree to round-off,
    for the integrating-factor and the explicit-viscosity RK4."""
    import jax_tg_project_gb300 as tg
    outs = []
    for variant in ("0", "4"):
        monkeypatch.setenv("TG_PASS_VARIANT", variant)
        p = tg.Plan(256, precision="f32", explicit_viscosity=explicit)
        s = p.initial_condition("taylor_green", seed=12, pert_amp=0.02, k0=4.0)
        p.step(s, dt=2.5e-4, nu=1 / 1600, nsteps=3)
        outs.append(from_state(p, s)[0])
        del p, s
    assert rel_l2(outs[0], outs[1]) < 1e-6
