"""The allocation-free diagnostics entry point (tg_diagnostics_noalloc).

Callers such as a framework that owns every device buffer (an XLA custom call,
an operator that must not bypass the framework's allocator) cannot create a
plan, because a plan allocates its scratch.  tg_diagnostics_noalloc keeps its
only scratch in a static device array instead.  This file checks, through the
C ABI, that it gives the same energies as tg_diagnostics on two calls in a row,
and that it rejects a batch larger than its fixed scratch.  It is named so that
pytest collects it last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(lib, plan, state, nu, eta):
    import torch

    from jax_tg_project_gb300 import _abi
    out = torch.full((plan.batch, _abi.TG_DIAG_WIDTH), float("nan"), dtype=torch.float64,
                     device=plan.device)
    phys = _abi.TG_PHYS_MHD if plan.physics == "mhd" else _abi.TG_PHYS_HYDRO
    prec = _abi.TG_PREC_F64 if plan.precision == "f64" else _abi.TG_PREC_F32
    stream = torch.cuda.current_stream(plan.device).cuda_stream
    rc = lib.tg_diagnostics_noalloc(ctypes.c_void_p(state.data_ptr()), plan.n, plan.batch, phys, prec,
                                    float(nu), float(eta), ctypes.c_void_p(out.data_ptr()),
                                    ctypes.c_void_p(stream))
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
