"""Host-side modules of the package that need no GPU: the parameter conversions and time-step
validation (checked against the oracle's restatement of jax/taylor_green_jax.py:17-52,131-155
and the reference's messages), the dealias cutoff of every built size, the run-loop step
counts, the ensemble's seeded draw and its rank sharding, and the CLI's argument parser."""
import math

import numpy as np
import pytest

from oracle import tg_numpy as T


def test_conversions_match_the_oracle():
    from jax_tg_project_gb300 import config as C
    for re in (1.0, 100.0, 1600.0, 3.2e4):
        assert C.reynolds_to_viscosity(re) == T.reynolds_to_viscosity(re)
        nu = C.reynolds_to_viscosity(re)
        assert C.viscosity_to_reynolds(nu) == pytest.approx(re, rel=1e-15)
        assert C.viscosity_to_reynolds(nu) == T.viscosity_to_reynolds(nu)
    assert C.viscosity_to_reynolds(0.0) == math.inf
    for bad, fn, msg in ((0.0, C.reynolds_to_viscosity, "Reynolds number must be positive"),
                         (-1.0, C.viscosity_to_reynolds, "Viscosity must be nonnegative"),
                         (0.0, C.magnetic_reynolds_to_resistivity, "magnetic_reynolds must be positive"),
                         (-1.0, C.resistivity_to_magnetic_reynolds, "resistivity must be nonnegative")):
        with pytest.raises(ValueError, match=msg):
            fn(bad)
    eta = C.magnetic_reynolds_to_resistivity(500.0, velocity_amplitude=0.5)
    assert C.resistivity_to_magnetic_reynolds(eta, velocity_amplitude=0.5) == pytest.approx(500.0)


@pytest.mark.parametrize("N", [8, 12, 16, 24, 32, 48, 64, 96, 128, 256, 512])
def test_dealias_cutoff_is_n_over_3_for_every_built_size(N):
    from jax_tg_project_gb300 import config as C
    assert C.dealias_cutoff(N) == N // 3 == T.dealias_cutoff(N)
    np.testing.assert_array_equal(C.wavenumber_axis(N), T.wavenumbers_1d(N))


@pytest.mark.parametrize("N,dt,nu", [(16, 0.005, 0.01), (16, 0.2, 0.01), (32, 0.05, 0.5), (64, 1e-3, 0.0),
                                     (64, 0.05, 0.0), (128, 2e-2, 1 / 1600)])
def test_validate_timestep_agrees_with_the_oracle(N, dt, nu):
    from jax_tg_project_gb300 import config as C
    kx, ky, kz = T.make_wavenumbers(N)
    try:
        want = T.validate_timestep(dt, nu, kx, ky, kz)
    except ValueError as e:
        with pytest.raises(ValueError) as got:
            C.validate_timestep(dt, nu, kx, ky, kz)
        assert str(got.value) == str(e)
    else:
        assert C.validate_timestep(dt, nu, kx, ky, kz) == pytest.approx(want, rel=1e-15)


def test_validate_timestep_mhd_limits():
    from jax_tg_project_gb300 import config as C
    kx, ky, kz = T.make_wavenumbers(32)
    kmax = float(np.abs(kx).max())
    k2max = float((kx * kx + ky * ky + kz * kz).max())
    lim = C.validate_timestep_mhd(1e-4, 0.01, 0.02, kx, ky, kz, max_velocity=1.0, max_field=2.0)
    want = min(0.5 * math.pi / kmax, 0.5 * math.pi / kmax / 2.0, 2.0 / (0.01 * k2max), 2.0 / (0.02 * k2max))
    assert lim == pytest.approx(want, rel=1e-15)
    with pytest.raises(ValueError, match="exceeds stability limit"):
        C.validate_timestep_mhd(1.0, 0.01, 0.02, kx, ky, kz)
    with pytest.raises(ValueError, match="resistivity must be nonnegative"):
        C.validate_timestep_mhd(1e-4, 0.01, -1.0, kx, ky, kz)


@pytest.mark.parametrize("T_,dt,save", [(0.5, 0.005, 0.05), (0.02, 0.005, 0.01), (1.0, 0.3, 0.1),
                                         (0.2, 1e-3, 0.01)])
def test_step_counts_match_the_oracle(T_, dt, save):
    from jax_tg_project_gb300 import config as C
    assert C.step_counts(T_, dt, save) == T.step_counts(T_, dt, save)


def test_ensemble_draw_is_seeded_and_in_range():
    pytest.importorskip("torch")
    from jax_tg_project_gb300 import ensemble as E
    a, b = E.draw_runs(64, seed=7), E.draw_runs(64, seed=7)
    assert [(r.n, r.reynolds) for r in a] == [(r.n, r.reynolds) for r in b]
    assert {r.n for r in a} <= {32, 64, 96}
    assert all(100.0 <= r.reynolds <= 3200.0 for r in a)
    assert all(r.nu == pytest.approx(2 * math.pi / r.reynolds) for r in a)
    assert [r.n for r in E.draw_runs(64, seed=8)] != [r.n for r in a]


@pytest.mark.parametrize("world", [1, 2, 3, 8])
def test_shard_runs_partitions_the_runs(world):
    pytest.importorskip("torch")
    from jax_tg_project_gb300 import ensemble as E
    runs = E.draw_runs(64, seed=2024)
    parts = [E.shard_runs(runs, r, world) for r in range(world)]
    flat = sorted(i for p in parts for i in p)
    assert flat == list(range(len(runs)))  # every run exactly once
    loads = [sum(runs[i].n ** 3 for i in p) for p in parts]
    biggest = max(r.n ** 3 for r in runs)
    assert max(loads) - min(loads) <= biggest  # longest-first balancing bound


def test_cli_parser_accepts_the_reference_flags():
    from jax_tg_project_gb300 import cli
    with pytest.raises(SystemExit) as e:
        cli.main(["--help"])
    assert e.value.code == 0
    with pytest.raises(SystemExit) as e:
        cli.main(["hydro", "--no-such-flag"])
    assert e.value.code != 0


def test_product_modules_never_import_the_oracle():
    """The oracle is test infrastructure: importing every module of the package (in a fresh
    interpreter) must not load it."""
    import subprocess
    import sys
    mods = ["jax_tg_project_gb300", "jax_tg_project_gb300.plan", "jax_tg_project_gb300.taylor_green",
            "jax_tg_project_gb300.spectral", "jax_tg_project_gb300.mhd", "jax_tg_project_gb300.config",
            "jax_tg_project_gb300.ensemble", "jax_tg_project_gb300.adjoint", "jax_tg_project_gb300.cli",
            "jax_tg_project_gb300.plots", "jax_tg_project_gb300._abi", "jax_tg_project_gb300._runtime"]
    code = ("import importlib, sys\n"
            f"for m in {mods!r}: importlib.import_module(m)\n"
            "bad = [m for m in sys.modules if m == 'oracle' or m.startswith('oracle.')]\n"
            "assert not bad, bad\n")
    import os
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", code], cwd=root, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
