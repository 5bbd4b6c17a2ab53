"""Parity at the sizes of the measured configurations (GPU).

* 96^3: the mixed-radix (4.4.6) transforms of the ensemble's largest size -- RHS and
  five Lawson-RK4 steps of a perturbed Taylor-Green field against the FP64 oracle
  (oracle/tg_numpy.py, the reference JAX algorithm), for every pass variant and y-pass
  configuration built at 96 and for a batched, autotuned 96^3 group;
* 128^3 MHD: the register-resident MHD z pass against the oracle's restatement of
  cuda/taylor_green_mhd/operators.py:70-107 (one RHS), and the full 400-step MHD
  workload (nu = eta = 1/800, dt = 5e-4, equal kinetic and magnetic energy) in FP32
  against the same run in FP64 on the GPU;
* 256^3: the full 500-step hydro workload (nu = 1/1600, dt = 2.5e-4) in FP32 against
  FP64, every diagnostics record.

Tolerances are the parity bar of the hot path: fields 1e-5 relative L2, energies and
the other positive diagnostics 1e-6 relative (FP32 kernels against FP64).  Each test
prints the errors it observed (``PARITY`` lines, visible with ``pytest -s``).
"""
import numpy as np
import pytest

from conftest import from_state, full_to_compact, rel_l2, to_state
from oracle import mhd_numpy as M
from oracle import perturb
from oracle import tg_numpy as T

pytestmark = pytest.mark.gpu

N96, NU96, DT96, STEPS96, SEED96, AMP96 = 96, 1e-3, 1e-3, 5, 21, 5e-2


def _report(name, **errs):
    print("PARITY " + name + " " + " ".join(f"{k}={v:.3e}" for k, v in errs.items()))


def _tg_pert(N, seed, amp, k0=4.0):
    return T.compact_from_physical(T.initial_taylor_green(N)) + \
        perturb.perturbation_compact(N, seed=seed, amp=amp, k0=k0)


@pytest.fixture(scope="module")
def oracle96():
    """RHS and five Lawson-RK4 steps of the perturbed field at 96^3 (FP64 oracle)."""
    c0 = _tg_pert(N96, SEED96, AMP96)
    u = T.physical_from_compact(c0, N96)
    kx, ky, kz = T.make_wavenumbers(N96)
    mask = T.make_dealias_mask(N96)
    rhs = T.compact_from_physical(T.spectral_rhs(u, NU96, kx, ky, kz, mask))
    for _ in range(STEPS96):
        u = T.advance_one_step(u, DT96, NU96, kx, ky, kz, mask, integrator="lawson")
    return {"rhs": rhs, "step": T.compact_from_physical(u), "c0": c0}


@pytest.mark.parametrize("variant,autotune", [("0", False), ("1", False), ("2", False), ("3", False),
                                              ("4", False), ("5", False), (None, True)])
def test_n96_rhs_and_steps_match_oracle(oracle96, variant, autotune, monkeypatch):
    """Every pass variant at 96 (bit 0: shared-memory instead of register-resident z pass,
    bit 1: the same for the x stage, bit 2: the x stage with a shared-memory stash) and the
    autotuned plan."""
    import jax_tg_project_gb300 as tg
    if variant is None:
        monkeypatch.delenv("TG_PASS_VARIANT", raising=False)
    else:
        monkeypatch.setenv("TG_PASS_VARIANT", variant)
    p = tg.Plan(N96, precision="f32", autotune=autotune)
    s = p.initial_condition("taylor_green", seed=SEED96, pert_amp=AMP96, k0=4.0)
    assert rel_l2(from_state(p, s)[0], oracle96["c0"]) < 2e-7
    e_rhs = rel_l2(from_state(p, p.rhs(s, nu=NU96))[0], oracle96["rhs"])
    p.step(s, dt=DT96, nu=NU96, nsteps=STEPS96)
    e_step = rel_l2(from_state(p, s)[0], oracle96["step"])
    _report(f"n96 variant={p.variant} autotune={autotune}", rhs=e_rhs, step5=e_step)
    assert e_rhs < 1e-5
    assert e_step < 1e-5


@pytest.mark.parametrize("yconf", ["0", "1", "2", "3"])
def test_n96_y_configurations_match_oracle(oracle96, yconf, monkeypatch):
    """Every y-pass configuration the autotuner chooses among at 96 (4.4.6 plan with 8, 12
    or 16 kz columns per CTA, 8.12 plan with 12)."""
    import jax_tg_project_gb300 as tg
    monkeypatch.setenv("TG_Y_CONF", yconf)
    p = tg.Plan(N96, precision="f32")
    assert p.y_config == (int(yconf), 4)
    s = p.initial_condition("taylor_green", seed=SEED96, pert_amp=AMP96, k0=4.0)
    p.step(s, dt=DT96, nu=NU96, nsteps=STEPS96)
    e_step = rel_l2(from_state(p, s)[0], oracle96["step"])
    _report(f"n96 yconf={yconf}", step5=e_step)
    assert e_step < 1e-5


def test_n96_batched_group_matches_oracle():
    """A batched 96^3 group as the ensemble builds it (autotuned plan, per-run nu and dt
    from the device table, seeds seed + 1000 n + r) against the oracle run by run."""
    from jax_tg_project_gb300.ensemble import Ensemble, RunSpec
    runs = [RunSpec(96, 300.0), RunSpec(96, 2500.0)]
    ens = Ensemble(runs, dt=1e-3, pert_amp=AMP96, k0=4.0, seed=3)
    ens.step(4)
    kx, ky, kz = T.make_wavenumbers(N96)
    mask = T.make_dealias_mask(N96)
    for i, r in enumerate(runs):
        plan, s = ens.state_of(i)
        got = from_state(plan, s[None].contiguous())[0]
        u = T.physical_from_compact(_tg_pert(N96, 3 + 1000 * N96 + i, AMP96), N96)
        for _ in range(4):
            u = T.advance_one_step(u, 1e-3, r.nu, kx, ky, kz, mask, integrator="lawson")
        err = rel_l2(got, T.compact_from_physical(u))
        _report(f"n96 batched run={i} variant={plan.variant}", step4=err)
        assert err < 1e-5


def test_mhd128_rhs_matches_oracle():
    """kz_reg_mhd_kernel / the MHD x stage at 128^3 against the restated CuPy MHD operator
    (physical sign of the Lorentz force), FP32 kernels against the FP64 oracle."""
    import jax_tg_project_gb300 as tg
    N, nu, eta = 128, 1 / 800, 1 / 800
    p = tg.Plan(N, physics="mhd", precision="f32")
    s = p.initial_condition("mhd_equal_energy", seed=4, pert_amp=2e-2, k0=4.0)
    c = from_state(p, s)[0]  # the FP32 state's values, exactly, in FP64
    uh = T.fftn(T.physical_from_compact(c[:3], N)) * T.make_dealias_mask(N)
    bh = T.fftn(T.physical_from_compact(c[3:], N)) * T.make_dealias_mask(N)
    ru, rb = M.spectral_rhs_mhd(M.Grid(N), uh, bh, nu, eta, lorentz_sign=1.0)
    got = from_state(p, p.rhs(s, nu=nu, eta=eta))[0]
    eu, eb = rel_l2(got[:3], full_to_compact(ru, N)), rel_l2(got[3:], full_to_compact(rb, N))
    _report("mhd128 rhs", u=eu, b=eb)
    assert eu < 1e-5 and eb < 1e-5


def _series_errors(d32, d64, cols):
    return {name: float(np.max(np.abs(d32[:, c] - d64[:, c]) / np.abs(d64[:, c]))) for name, c in cols}


def test_mhd128_full_run_fp32_tracks_fp64():
    """The 128^3 MHD workload in full (400 steps), FP32 kernels against FP64 kernels."""
    import torch

    import jax_tg_project_gb300 as tg
    N, nu, eta, dt, steps, every = 128, 1 / 800, 1 / 800, 5e-4, 400, 50
    out = {}
    for prec in ("f32", "f64"):
        p = tg.Plan(N, physics="mhd", precision=prec)
        s = p.initial_condition("mhd_equal_energy")
        series = p.run(s, dt=dt, nu=nu, eta=eta, nsteps=steps, save_every=every).cpu().numpy()[:, 0]
        out[prec] = (series, from_state(p, s)[0])
        del p
        torch.cuda.empty_cache()
    (d32, c32), (d64, c64) = out["f32"], out["f64"]
    errs = _series_errors(d32, d64, (("E_k", 0), ("enstrophy", 1), ("E_m", 3), ("E_total", 5)))
    # H_c = <u . b> stays zero for this initial condition (it is odd under a symmetry of
    # the flow): compare it on the scale of the energies
    errs["H_c_abs_over_E"] = float(np.max(np.abs(d32[:, 4] - d64[:, 4]) / d64[:, 5]))
    errs["u"] = rel_l2(c32[:3], c64[:3])
    errs["b"] = rel_l2(c32[3:], c64[3:])
    _report("mhd128 400 steps fp32-vs-fp64", **errs)
    for k in ("E_k", "E_m", "E_total", "enstrophy", "H_c_abs_over_E"):
        assert errs[k] < 1e-6, (k, errs[k])
    assert errs["u"] < 1e-5 and errs["b"] < 1e-5


def test_hydro256_full_run_fp32_tracks_fp64():
    """The 256^3 throughput workload in full (500 steps, every record), FP32 against FP64:
    the energy error bar of the workload is 1e-6."""
    import torch

    import jax_tg_project_gb300 as tg
    N, nu, dt, steps, every = 256, 1 / 1600, 2.5e-4, 500, 10
    out = {}
    for prec in ("f32", "f64"):
        p = tg.Plan(N, precision=prec)
        s = p.initial_condition("taylor_green")
        series = p.run(s, dt=dt, nu=nu, nsteps=steps, save_every=every).cpu().numpy()[:, 0]
        out[prec] = (series, from_state(p, s)[0])
        del p, s
        torch.cuda.empty_cache()
    (d32, c32), (d64, c64) = out["f32"], out["f64"]
    errs = _series_errors(d32, d64, (("energy", 0), ("enstrophy", 1), ("dissipation", 2)))
    errs["u"] = rel_l2(c32, c64)
    errs["divergence_max_f32"] = float(d32[:, 6].max())
    _report("hydro256 500 steps fp32-vs-fp64", **errs)
    assert errs["energy"] < 1e-6
    assert errs["enstrophy"] < 1e-6 and errs["dissipation"] < 1e-6
    assert errs["u"] < 1e-5
    assert errs["divergence_max_f32"] < 1e-5


def _full_spectrum(c, N):
    """Full fftn-layout coefficients (C, N, N, N) of compact half-spectrum coefficients c:
    the kept modes and their Hermitian mirrors, placed exactly (no transform)."""
    K = T.dealias_cutoff(N)
    idx = T.kept_indices(N)
    full = np.zeros((c.shape[0], N, N, N), dtype=np.complex128)
    for kz in range(K + 1):
        full[:, idx[:, None], idx[None, :], kz] = c[..., kz]
        if kz > 0:
            full[:, ((-idx) % N)[:, None], ((-idx) % N)[None, :], N - kz] = np.conj(c[..., kz])
    return full


@pytest.mark.parametrize("N,physics", [(16, "hydro"), (32, "hydro"), (32, "mhd")])
def test_energy_spectrum_matches_oracle(N, physics):
    """tg_energy_spectrum bin by bin against shell sums over the full spectrum,
    E(k) = 1/2 sum over round(|k|) = k of |c_k|^2 (kinetic, and magnetic for MHD), with the
    wavenumbers of the oracle's make_wavenumbers."""
    import jax_tg_project_gb300 as tg
    p = tg.Plan(N, physics=physics, precision="f64")
    kind = "mhd_equal_energy" if physics == "mhd" else "taylor_green"
    s = p.initial_condition(kind, seed=8, pert_amp=0.1, k0=3.0)
    got = p.energy_spectrum(s).cpu().numpy()[0]
    c = from_state(p, s)[0]
    kx, ky, kz = T.make_wavenumbers(N)
    shell = np.floor(np.sqrt(kx * kx + ky * ky + kz * kz) + 0.5).astype(int)
    nb = got.shape[-1]

    def shells(cc):
        e = 0.5 * np.sum(np.abs(_full_spectrum(cc, N)) ** 2, axis=0)
        return np.bincount(shell.ravel(), weights=e.ravel(), minlength=nb)[:nb]

    want = shells(c[:3])
    if physics == "mhd":
        want = np.stack([want, shells(c[3:])])
    np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-300)
    # every kinetic shell is populated (the perturbation fills the band; b has only |k| = sqrt 3)
    assert np.all(want.reshape(-1, nb)[0, 1:] > 0)
    d = p.diagnostics(s, nu=0.0).cpu().numpy()[0]
    assert np.sum(got[0] if physics == "mhd" else got) == pytest.approx(d[0], rel=1e-12)
