"""The allocation-free diagnostics entry point (tg_diagnostics_noalloc).

Callers such as a framework that owns every device buffer (an XLA custom call,
an operator that must not bypass the framework's allocator) cannot create a
plan, because a plan allocates its scratch.  tg_diagnostics_noalloc keeps its
only scratch in a static device array instead.  This file checks, through the
C ABI, that it gives the same energies as tg_diagnostics on two calls in a row,
that it matches the oracle's Parseval sums at the largest batch its fixed scratch
allows, that a call changes the device's free memory by nothing, and that it rejects
a batch larger than its fixed scratch, grid sizes no plan lays out, and a negative nu.
It is named so that pytest collects it last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _call(lib, plan, state, nu, eta, out):
    import torch

    from jax_tg_project_gb300 import _abi
    phys = _abi.TG_PHYS_MHD if plan.physics == "mhd" else _abi.TG_PHYS_HYDRO
    prec = _abi.TG_PREC_F64 if plan.precision == "f64" else _abi.TG_PREC_F32
    stream = torch.cuda.current_stream(plan.device).cuda_stream
    return lib.tg_diagnostics_noalloc(ctypes.c_void_p(state.data_ptr()), plan.n, plan.batch, phys, prec,
                                      float(nu), float(eta), ctypes.c_void_p(out.data_ptr()),
                                      ctypes.c_void_p(stream))


def _noalloc(lib, plan, state, nu, eta):
    import torch

    from jax_tg_project_gb300 import _abi
    out = torch.full((plan.batch, _abi.TG_DIAG_WIDTH), float("nan"), dtype=torch.float64,
                     device=plan.device)
    rc = _call(lib, plan, state, nu, eta, out)
    assert rc == _abi.TG_OK, lib.tg_last_error()
    return out.cpu().numpy()


@pytest.mark.parametrize("n,batch,physics,precision,kind,tol", [
    (32, 3, "hydro", "f32", "taylor_green", 1e-12),
    (32, 2, "hydro", "f64", "taylor_green", 1e-13),
    (16, 2, "mhd", "f32", "mhd_equal_energy", 1e-12),
])
def test_noalloc_matches_tg_diagnostics(n, batch, physics, precision, kind, tol):
    import jax_tg_project_gb300 as tg
    from jax_tg_project_gb300 import _abi

    lib = _abi.load()
    plan = tg.Plan(n, batch=batch, physics=physics, precision=precision)
    state = plan.initial_condition(kind, seed=7, pert_amp=0.05, k0=3.0)
    nu, eta = 0.003, 0.002
    ref = plan.diagnostics(state, nu=nu, eta=eta).cpu().numpy()
    first = _noalloc(lib, plan, state, nu, eta)
    second = _noalloc(lib, plan, state, nu, eta)
    for got in (first, second):
        np.testing.assert_allclose(got[:, :6], ref[:, :6], rtol=tol, atol=1e-300)
        assert np.all(got[:, 6:] == -1.0)


def test_noalloc_rejects_batch_beyond_its_static_scratch():
    import torch

    from jax_tg_project_gb300 import _abi

    lib = _abi.load()
    too_many = _abi.TG_NOALLOC_MAX_RUNS + 1
    dummy = torch.zeros(1, dtype=torch.float64, device="cuda")
    rc = lib.tg_diagnostics_noalloc(ctypes.c_void_p(dummy.data_ptr()), 16, too_many, 0, 0, 0.0, 0.0,
                                    ctypes.c_void_p(dummy.data_ptr()), None)
    assert rc == _abi.TG_E_INVALID
    assert b"outside 1..64" in lib.tg_last_error()


def test_noalloc_full_batch_matches_oracle_and_allocates_nothing():
    """The documented maximum batch (TG_NOALLOC_MAX_RUNS runs of 16^3, perturbed states that
    differ per run): every record against the oracle's Parseval sums of the same FP32
    coefficients (oracle/tg_numpy.py compact_diagnostics), on two calls in a row, and the
    device's free memory is the same before and after a call."""
    import torch

    import jax_tg_project_gb300 as tg
    from conftest import from_state
    from jax_tg_project_gb300 import _abi
    from oracle import tg_numpy as T

    lib = _abi.load()
    batch, nu = _abi.TG_NOALLOC_MAX_RUNS, 0.004
    plan = tg.Plan(16, batch=batch, precision="f32")
    state = plan.initial_condition("taylor_green", seed=31, pert_amp=0.2, k0=3.0)
    coef = from_state(plan, state)
    want = np.array([T.compact_diagnostics(coef[r], nu) for r in range(batch)])
    for _ in range(2):
        got = _noalloc(lib, plan, state, nu, 0.0)
        # per-mode terms of an FP32 state are formed in FP32 (~1e-7 each), summed in FP64
        np.testing.assert_allclose(got[:, 0], want[:, 0], rtol=1e-6)  # E_k
        np.testing.assert_allclose(got[:, 1], want[:, 1], rtol=1e-6)  # enstrophy
        np.testing.assert_allclose(got[:, 2], want[:, 2], rtol=1e-6)  # nu sum w k^2 |u|^2
        np.testing.assert_allclose(got[:, 5], got[:, 0], rtol=0)      # E_k + E_m with E_m = 0
        assert np.all(got[:, 3:5] == 0.0) and np.all(got[:, 6:] == -1.0)
        assert len(np.unique(got[:, 0])) == batch  # every run summed on its own
    out = torch.empty((batch, _abi.TG_DIAG_WIDTH), dtype=torch.float64, device=plan.device)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    assert _call(lib, plan, state, nu, 0.0, out) == _abi.TG_OK, lib.tg_last_error()
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0


def test_noalloc_rejects_unbuilt_sizes_and_negative_nu():
    import torch

    from jax_tg_project_gb300 import _abi

    lib = _abi.load()
    dummy = torch.zeros(64, dtype=torch.float64, device="cuda")
    ptr = ctypes.c_void_p(dummy.data_ptr())
    for n, prec in ((100, _abi.TG_PREC_F32), (24, _abi.TG_PREC_F64), (4, _abi.TG_PREC_F32)):
        rc = lib.tg_diagnostics_noalloc(ptr, n, 1, _abi.TG_PHYS_HYDRO, prec, 0.0, 0.0, ptr, None)
        assert rc == _abi.TG_E_UNSUPPORTED, (n, prec, rc)
        assert b"not built" in lib.tg_last_error()
    rc = lib.tg_diagnostics_noalloc(ptr, 16, 1, _abi.TG_PHYS_HYDRO, _abi.TG_PREC_F32, -1.0, 0.0, ptr, None)
    assert rc == _abi.TG_E_INVALID and b"nu must be nonnegative" in lib.tg_last_error()
