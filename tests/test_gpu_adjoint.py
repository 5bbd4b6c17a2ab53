"""Hand-written discrete adjoint (tg_adjoint): central finite differences along
seeded divergence-free directions, and torch.autograd through a PyTorch FP64
restatement of the reference JAX solver (oracle/tg_torch.py)."""
import numpy as np
import pytest

from conftest import from_state, rel_l2, to_state
from oracle import perturb
from oracle import tg_numpy as T

pytestmark = pytest.mark.gpu


def _plan(N, prec):
    import jax_tg_project_gb300 as tg
    return tg.Plan(N, precision=prec)


def _loss(plan, s0, dt, nu, nsteps):
    s = s0.clone()
    plan.step(s, dt=dt, nu=nu, nsteps=nsteps)
    return float(plan.diagnostics(s, nu=nu)[0, 1])


@pytest.mark.parametrize("N,nsteps,ck", [(16, 12, 4), (32, 7, 0)])
def test_adjoint_matches_central_differences_fp64(N, nsteps, ck):
    from jax_tg_project_gb300.adjoint import spectral_inner
    p = _plan(N, "f64")
    dt, nu = 5e-3, 0.01
    s0 = p.initial_condition("taylor_green", seed=3, pert_amp=0.1, k0=3.0)
    loss, grad, gnu = p.adjoint(s0, dt, nu, nsteps, ck)
    assert float(loss) == pytest.approx(_loss(p, s0, dt, nu, nsteps), rel=1e-13)
    for seed in range(4):
        d = to_state(p, perturb.perturbation_compact(N, seed=100 + seed, amp=1.0, k0=3.0))
        eps = 1e-5
        fd = (_loss(p, s0 + eps * d, dt, nu, nsteps) - _loss(p, s0 - eps * d, dt, nu, nsteps)) / (2 * eps)
        ad = spectral_inner(p, grad, d)
        assert ad == pytest.approx(fd, rel=1e-6, abs=1e-12), (seed, ad, fd)
    e = 1e-6
    fdn = (_loss(p, s0, dt, nu + e, nsteps) - _loss(p, s0, dt, nu - e, nsteps)) / (2 * e)
    assert float(gnu) == pytest.approx(fdn, rel=1e-6)


def test_adjoint_matches_autograd_of_reference_solver():
    """torch.autograd through the reference algorithm (explicit RK4, advective form,
    FP64, CPU) against the GPU adjoint of the integrating-factor step."""
    import torch

    from jax_tg_project_gb300 import _runtime
    from jax_tg_project_gb300.adjoint import final_enstrophy
    from oracle import tg_torch
    N, dt, nu, nsteps = 32, 4e-3, 0.01, 10
    c = T.compact_from_physical(T.initial_taylor_green(N)) + \
        perturb.perturbation_compact(N, seed=21, amp=0.1, k0=3.0)
    u0 = T.physical_from_compact(c, N)
    ut = torch.tensor(u0, dtype=torch.float64, requires_grad=True)
    nut = torch.tensor(nu, dtype=torch.float64, requires_grad=True)
    Lr = tg_torch.final_enstrophy(ut, nut, dt, nsteps)
    Lr.backward()
    _runtime.set_default_precision("f64")
    try:
        ug = torch.tensor(u0, dtype=torch.float64, device="cuda", requires_grad=True)
        nug = torch.tensor(nu, dtype=torch.float64, device="cuda", requires_grad=True)
        Lg = final_enstrophy(ug, nug, dt, nsteps, checkpoint_every=3)
        Lg.backward()
    finally:
        _runtime.set_default_precision("f32")
    assert float(Lg) == pytest.approx(float(Lr), rel=1e-9)
    # The reference multiplies the raw (un-dealiased) u in u.grad u, so its map also
    # depends on modes outside the 2/3 band; this solver dealiases the state first.
    # On band-limited directions the two gradients must agree: compare projections.
    ref = T.physical_from_compact(T.compact_from_physical(ut.grad.numpy()), N)
    ours = ug.grad.cpu().numpy()
    assert rel_l2(ours, ref) < 1e-6
    assert rel_l2(T.physical_from_compact(T.compact_from_physical(ours), N), ours) < 1e-12
    assert float(nug.grad) == pytest.approx(float(nut.grad), rel=1e-6)


def test_fp32_adjoint_tracks_fp64():
    p32, p64 = _plan(32, "f32"), _plan(32, "f64")
    s32 = p32.initial_condition("taylor_green", seed=4, pert_amp=0.05, k0=3.0)
    s64 = p64.initial_condition("taylor_green", seed=4, pert_amp=0.05, k0=3.0)
    l32, g32, n32 = p32.adjoint(s32, 2e-3, 1 / 400, 16, 4)
    l64, g64, n64 = p64.adjoint(s64, 2e-3, 1 / 400, 16, 4)
    assert float(l32) == pytest.approx(float(l64), rel=1e-6)
    assert rel_l2(from_state(p32, g32), from_state(p64, g64)) < 2e-5
    assert float(n32) == pytest.approx(float(n64), rel=1e-4)


def test_adjoint_128_fp32_finite_differences():
    """The 128^3 gradient configuration (TG + 1e-2 perturbation, nu = 1/1600, dt = 1e-3)
    on a shortened horizon, FP32 kernels: central differences with eps = 1e-4 along
    seeded unit directions agree to the FP32 noise level of the differenced losses."""
    from jax_tg_project_gb300.adjoint import spectral_inner
    p = _plan(128, "f32")
    dt, nu, nsteps = 1e-3, 1 / 1600, 16
    s0 = p.initial_condition("taylor_green", seed=9, pert_amp=1e-2, k0=4.0)
    loss, grad, gnu = p.adjoint(s0, dt, nu, nsteps, 4)
    rel = []
    for seed in range(3):
        d = perturb.perturbation_compact(128, seed=500 + seed, amp=1.0, k0=4.0)
        d /= np.sqrt(np.sum(np.where(np.arange(d.shape[-1]) == 0, 1.0, 2.0) * np.abs(d) ** 2))
        dd = to_state(p, d)
        eps = 1e-4
        fd = (_loss(p, s0 + eps * dd, dt, nu, nsteps) - _loss(p, s0 - eps * dd, dt, nu, nsteps)) / (2 * eps)
        ad = spectral_inner(p, grad, dd)
        rel.append(abs(ad - fd) / max(abs(fd), 1e-30))
    assert max(rel) < 3e-2, rel


@pytest.mark.parametrize("N,nsteps,ck", [(16, 5, 2), (32, 9, 0), (32, 8, 3), (128, 6, 4)])
def test_host_tape_adjoint_matches_checkpointed(N, nsteps, ck):
    """The whole-run stage tape (one forward sweep, stage data in pinned host memory) and
    sqrt(n) checkpointing (each segment recomputed from its checkpoint with its tape
    recorded, segments of ck steps, 0: ceil(sqrt n), the last one shorter when ck does not
    divide nsteps) run the same kernels on the same states: identical results."""
    p = _plan(N, "f32")
    dt, nu = 2e-3, 1 / 400
    s0 = p.initial_condition("taylor_green", seed=6, pert_amp=0.05, k0=3.0)
    lc, gc, nc = p.adjoint(s0, dt, nu, nsteps, ck)
    lt, gt, nt = p.adjoint(s0, dt, nu, nsteps, "tape")
    assert float(lt) == float(lc) and float(nt) == float(nc)
    assert bool((gt == gc).all())
    # a second call reuses the plan's host tape; after a release the next call pins it again
    lt2, gt2, nt2 = p.adjoint(s0, dt, nu, nsteps, "tape")
    assert float(lt2) == float(lt) and float(nt2) == float(nt)
    assert bool((gt2 == gt).all())
    p.release_tape()
    lt3, gt3, nt3 = p.adjoint(s0, dt, nu, nsteps, "tape")
    assert float(nt3) == float(nt) and bool((gt3 == gt).all())


def test_host_tape_tracks_fp64_adjoint():
    p32, p64 = _plan(32, "f32"), _plan(32, "f64")
    s32 = p32.initial_condition("taylor_green", seed=4, pert_amp=0.05, k0=3.0)
    s64 = p64.initial_condition("taylor_green", seed=4, pert_amp=0.05, k0=3.0)
    l32, g32, n32 = p32.adjoint(s32, 2e-3, 1 / 400, 16, "tape")
    l64, g64, n64 = p64.adjoint(s64, 2e-3, 1 / 400, 16, "tape")  # FP64: checkpointed instead
    assert float(l32) == pytest.approx(float(l64), rel=1e-6)
    assert rel_l2(from_state(p32, g32), from_state(p64, g64)) < 2e-5
    assert float(n32) == pytest.approx(float(n64), rel=1e-4)


@pytest.mark.parametrize("N,cutoff,nsteps", [(32, 0, 1), (32, 7, 4), (64, 15, 3)])
def test_host_tape_edge_cases(N, cutoff, nsteps):
    """One step (the backward runs eagerly, no step graph) and cutoffs below N/3 (the
    kernels' masks follow K): tape and checkpointed adjoints agree."""
    import jax_tg_project_gb300 as tg
    p = tg.Plan(N, precision="f32", cutoff=cutoff)
    s0 = p.initial_condition("taylor_green", seed=11, pert_amp=0.05, k0=3.0)
    lc, gc, nc = p.adjoint(s0, 2e-3, 1 / 300, nsteps, 1)
    lt, gt, nt = p.adjoint(s0, 2e-3, 1 / 300, nsteps, "tape")
    assert float(lt) == float(lc) and float(nt) == float(nc)
    assert bool((gt == gc).all())


@pytest.mark.parametrize("N,nsteps,ck", [(32, 9, 3), (128, 5, 2)])
def test_tape_adjoint_matches_recomputing_adjoint(N, nsteps, ck, monkeypatch):
    """The stage-tape kernels against the recomputing adjoint (stage terms recomputed per
    step by separate nonlinear-term and stage kernels; the path FP64 plans and the
    shared-memory pass variants take): the same discrete gradient up to FP32 rounding."""
    dt, nu = 2e-3, 1 / 400
    p = _plan(N, "f32")
    s0 = p.initial_condition("taylor_green", seed=8, pert_amp=0.05, k0=3.0)
    lt, gt, nt = p.adjoint(s0, dt, nu, nsteps, ck)
    monkeypatch.setenv("TG_PASS_VARIANT", "1")  # shared-memory z passes: no tape kernels
    q = _plan(N, "f32")
    assert q.variant == 1
    lr, gr, nr = q.adjoint(s0, dt, nu, nsteps, ck)
    assert float(lt) == pytest.approx(float(lr), rel=1e-6)
    assert rel_l2(from_state(p, gt), from_state(q, gr)) < 2e-5
    assert float(nt) == pytest.approx(float(nr), rel=1e-4)


def test_tape_adjoint_with_stashed_x_stage(monkeypatch):
    """The stage tape written by the stashed x stage (variant bit 2) drives the same adjoint:
    it agrees with the tape of the register x stage to FP32 rounding."""
    dt, nu, nsteps = 2e-3, 1 / 400, 6
    outs = []
    for variant in ("0", "4"):
        monkeypatch.setenv("TG_PASS_VARIANT", variant)
        p = _plan(128, "f32")
        s0 = p.initial_condition("taylor_green", seed=13, pert_amp=0.05, k0=3.0)
        loss, grad, gnu = p.adjoint(s0, dt, nu, nsteps, 3)
        assert p.adjoint_profile()["record"] > 0.0  # the stage-tape schedule ran
        outs.append((float(loss), from_state(p, grad), float(gnu)))
    assert outs[1][0] == pytest.approx(outs[0][0], rel=1e-6)
    assert rel_l2(outs[1][1], outs[0][1]) < 2e-5
    assert outs[1][2] == pytest.approx(outs[0][2], rel=1e-4)
