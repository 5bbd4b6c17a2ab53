"""Transforms and initial conditions on the GPU against the NumPy oracle."""
import numpy as np
import pytest

from conftest import from_state, rel_l2, to_state
from oracle import perturb
from oracle import tg_numpy as T

pytestmark = pytest.mark.gpu

SIZES_F32 = [8, 12, 16, 24, 32, 48, 64, 96, 128]
SIZES_F64 = [8, 16, 32, 64, 96]


def _plan(N, prec, **kw):
    import jax_tg_project_gb300 as tg
    return tg.Plan(N, precision=prec, **kw)


def _tol(prec):
    return 2e-6 if prec == "f32" else 1e-13


@pytest.mark.parametrize("prec,N", [("f32", n) for n in SIZES_F32] + [("f64", n) for n in SIZES_F64])
def test_forward_inverse_match_oracle(prec, N):
    import torch
    p = _plan(N, prec)
    c = perturb.perturbation_compact(N, seed=N, amp=0.3, k0=3.0)
    u = T.physical_from_compact(c, N)
    uu = torch.from_numpy(u[None]).to(p.real_dtype).cuda().contiguous()
    s = p.forward(uu)
    got = from_state(p, s)[0]
    assert rel_l2(got, c) < _tol(prec) * 5
    back = p.inverse(to_state(p, c))[0].double().cpu().numpy()
    assert rel_l2(back, u) < _tol(prec) * 5


@pytest.mark.parametrize("prec,N", [("f32", 16), ("f32", 64), ("f64", 32)])
def test_taylor_green_initial_condition(prec, N):
    p = _plan(N, prec)
    s = p.initial_condition("taylor_green")
    u = p.inverse(s)[0].double().cpu().numpy()
    assert np.abs(u - T.initial_taylor_green(N)).max() < (1e-6 if prec == "f32" else 1e-14)
    d = p.diagnostics(s, nu=0.01).cpu().numpy()[0]
    assert d[0] == pytest.approx(0.125, rel=1e-7)
    assert d[1] == pytest.approx(0.375, rel=1e-7)
    assert d[2] == pytest.approx(0.01 * 0.75, rel=1e-7)
    assert d[6] < (1e-6 if prec == "f32" else 1e-13)
    m = p.absmax(s, "velocity").cpu().numpy()[0]
    u0 = T.initial_taylor_green(N)
    np.testing.assert_allclose(m, np.abs(u0).reshape(3, -1).max(axis=1), atol=1e-6)


@pytest.mark.parametrize("prec,N,batch", [("f64", 16, 1), ("f64", 32, 3), ("f32", 64, 2), ("f32", 96, 1)])
def test_perturbation_matches_oracle(prec, N, batch):
    p = _plan(N, prec, batch=batch)
    s = p.initial_condition("taylor_green", seed=11, pert_amp=1e-3, k0=4.0)
    got = from_state(p, s)
    tg0 = T.compact_from_physical(T.initial_taylor_green(N))
    for r in range(batch):
        want = tg0 + perturb.perturbation_compact(N, seed=11 + r, amp=1e-3, k0=4.0)
        assert rel_l2(got[r], want) < (2e-7 if prec == "f32" else 1e-14)
        # the perturbation part alone
        assert rel_l2(got[r] - tg0, want - tg0) < (5e-4 if prec == "f32" else 1e-11)
