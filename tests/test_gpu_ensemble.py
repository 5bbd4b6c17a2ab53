"""Batched ensembles: every run of a batched ensemble (groups in order on one stream, or on
concurrent streams) equals the same run done alone, and matches the NumPy oracle."""
import numpy as np
import pytest

from conftest import from_state, rel_l2
from oracle import perturb
from oracle import tg_numpy as T

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("concurrent", [False, True])
def test_ensemble_runs_equal_single_runs(monkeypatch, concurrent):
    """Bit-identical: each single run uses the pass variant its autotuned group chose."""
    import torch

    import jax_tg_project_gb300 as tg
    from jax_tg_project_gb300.ensemble import Ensemble, RunSpec
    runs = [RunSpec(32, 400.0), RunSpec(24, 150.0), RunSpec(32, 2000.0), RunSpec(16, 900.0),
            RunSpec(24, 3000.0), RunSpec(32, 120.0)]
    ens = Ensemble(runs, dt=2e-3, pert_amp=1e-2, k0=3.0, seed=5, concurrent=concurrent)
    ens.step(6)
    torch.cuda.synchronize()
    for i, r in enumerate(runs):
        plan_b, sb = ens.state_of(i)
        grp = next(g for g in ens.groups if g["n"] == r.n)
        monkeypatch.setenv("TG_PASS_VARIANT", str(grp["plan"].variant))
        p1 = tg.Plan(r.n)
        s1 = p1.initial_condition("taylor_green", seed=5 + 1000 * r.n + grp["idx"].index(i),
                                  pert_amp=1e-2, k0=3.0)
        p1.step(s1, dt=2e-3, nu=r.nu, nsteps=6)
        assert torch.equal(s1[0], sb), i


def test_ensemble_run_matches_oracle():
    from jax_tg_project_gb300.ensemble import Ensemble, RunSpec
    runs = [RunSpec(24, 300.0), RunSpec(16, 500.0)]
    ens = Ensemble(runs, dt=2e-3, pert_amp=5e-2, k0=3.0, seed=11)
    ens.step(5)
    for i, r in enumerate(runs):
        plan, s = ens.state_of(i)
        got = from_state(plan, s[None].contiguous())[0]
        c0 = T.compact_from_physical(T.initial_taylor_green(r.n)) + \
            perturb.perturbation_compact(r.n, seed=11 + 1000 * r.n, amp=5e-2, k0=3.0)
        u = T.physical_from_compact(c0, r.n)
        kx, ky, kz = T.make_wavenumbers(r.n)
        mask = T.make_dealias_mask(r.n)
        for _ in range(5):
            u = T.advance_one_step(u, 2e-3, r.nu, kx, ky, kz, mask)
        assert rel_l2(got, T.compact_from_physical(u)) < 1e-5


def test_draw_runs_is_seeded():
    from jax_tg_project_gb300.ensemble import draw_runs
    a, b = draw_runs(64, seed=3), draw_runs(64, seed=3)
    assert a == b and len({r.n for r in a}) == 3
    assert all(100.0 <= r.reynolds <= 3200.0 for r in a)
