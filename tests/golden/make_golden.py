"""Generate the golden fixtures in this directory from the REFERENCE's own code.

The reference (mahanr/jax_tg_project) is Python on JAX (hydro) and CuPy (HD and
MHD packages).  Neither jax nor cupy (nor matplotlib) is installed here, so this
script imports the reference modules unchanged with small stand-ins:

* ``jax``: ``jax.numpy`` is NumPy with ``jnp.fft`` routed to SciPy's pocketfft
  (FP64, multi-threaded); ``jax.jit`` is the identity; ``jax.config.update`` is a
  no-op (NumPy is FP64 already, matching ``jax_enable_x64``);
* ``cupy``: NumPy plus a ``cupy.cuda`` namespace with no-op synchronisation;
  the two ``_host`` helpers that call ``.get()`` become ``float(value)``;
* ``matplotlib``: plots are swallowed.

The arithmetic that runs is therefore the reference's, with NumPy/SciPy FP64
FFTs in place of XLA/cuFFT.  Inputs are seeded.  Usage (writes *.npz here):

    python tests/golden/make_golden.py --reference <reference checkout> [--skip-64]

(or set TG_REFERENCE_DIR to the checkout instead of passing --reference)
"""
from __future__ import annotations

import argparse
import functools
import os
import sys
import types
from unittest import mock

import numpy as np
import scipy.fft as sfft

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from oracle import perturb, tg_numpy  # noqa: E402  (inputs only)


def _install_stand_ins():
    fft = types.SimpleNamespace(
        fftn=functools.partial(sfft.fftn, workers=-1),
        ifftn=functools.partial(sfft.ifftn, workers=-1),
        fftfreq=np.fft.fftfreq,
    )
    jnp = types.ModuleType("jax.numpy")
    jnp.__dict__.update({k: getattr(np, k) for k in dir(np) if not k.startswith("__")})
    jnp.fft = fft
    jax = types.ModuleType("jax")
    jax.numpy = jnp
    jax.jit = lambda f: f
    jax.config = types.SimpleNamespace(update=lambda *a, **k: None)
    jax.devices = lambda *a, **k: []
    sys.modules["jax"] = jax
    sys.modules["jax.numpy"] = jnp

    cp = types.ModuleType("cupy")
    cp.__dict__.update({k: getattr(np, k) for k in dir(np) if not k.startswith("__")})
    cp.fft = fft
    cp.cuda = types.SimpleNamespace(
        Stream=types.SimpleNamespace(null=types.SimpleNamespace(synchronize=lambda: None)),
        runtime=types.SimpleNamespace(getDeviceProperties=lambda i: {"name": "numpy"}),
        Device=lambda *a: types.SimpleNamespace(id=0),
    )
    sys.modules["cupy"] = cp

    def subplots(nrows=1, ncols=1, **kw):
        return mock.MagicMock(), [mock.MagicMock() for _ in range(nrows * ncols)]

    plt = mock.MagicMock()
    plt.subplots = subplots
    mpl = types.ModuleType("matplotlib")
    mpl.use = lambda *a, **k: None
    mpl.pyplot = plt
    sys.modules["matplotlib"] = mpl
    sys.modules["matplotlib.pyplot"] = plt


def _seeded_field(N, seed, amp):
    """TG plus a seeded band-limited solenoidal field (physical, FP64)."""
    c = perturb.perturbation_compact(N, seed, amp=amp, k0=3.0)
    return tg_numpy.initial_taylor_green(N) + tg_numpy.physical_from_compact(c, N)


def hydro(ref_root, skip_64):
    sys.path.insert(0, os.path.join(ref_root, "jax"))
    import taylor_green_jax as R  # the reference module, unchanged

    out = {}
    L = 2.0 * np.pi
    N = 16
    kx, ky, kz = R.make_wavenumbers(N, L)
    mask = R.make_dealias_mask(N, L)
    u0 = R.initial_taylor_green(N, L)
    out["ic16_energy"] = float(R.kinetic_energy(u0))
    out["ic16_enstrophy"] = float(R.enstrophy(u0, kx, ky, kz))
    out["ic16_dissipation"] = float(R.viscous_dissipation(u0, 0.01, kx, ky, kz))
    out["ic16_divmax"] = float(np.max(np.abs(R.spectral_divergence(u0, kx, ky, kz))))
    out["mask16_count"] = int(np.asarray(mask).sum())
    out["limit16"] = float(R.validate_timestep(0.005, 0.01, kx, ky, kz))

    uin = _seeded_field(N, seed=1234, amp=0.3)
    out["rhs16_in"] = uin
    out["rhs16_out"] = np.asarray(R.spectral_rhs(uin, 0.01, kx, ky, kz, mask))
    out["step16_out"] = np.asarray(R.advance_one_step(uin, 0.005, 0.01, kx, ky, kz, mask))
    # zero mode / constant field (jax/test_taylor_green_jax.py:45-51)
    out["rhs8_const"] = np.asarray(R.spectral_rhs(
        np.ones((3, 8, 8, 8)), 0.01, *R.make_wavenumbers(8, L), R.make_dealias_mask(8, L)))

    u, e, d = R.run_simulation(N=8, dt=0.005, nu=0.01, total_time=0.02,
                               save_every_time=0.01, return_diagnostics=True)
    out["run8_u"] = np.asarray(u)
    for k, v in d.items():
        out[f"run8_{k}"] = np.asarray(v)
    u, e, d = R.run_simulation(N=16, dt=0.005, reynolds=100, total_time=0.05,
                               save_every_time=0.01, return_diagnostics=True)
    out["run16_u"] = np.asarray(u)
    for k, v in d.items():
        out[f"run16_{k}"] = np.asarray(v)
    np.savez_compressed(os.path.join(HERE, "reference_hydro.npz"), **out)
    print("wrote reference_hydro.npz")

    if not skip_64:
        # 64^3 TG, nu=1/1600, dt=1e-3: 100 steps (field) and 200 steps (series)
        nu = 1.0 / 1600.0
        u100, _, d100 = R.run_simulation(N=64, dt=1e-3, nu=nu, total_time=0.1,
                                         save_every_time=0.01, return_diagnostics=True)
        c100 = tg_numpy.compact_from_physical(np.asarray(u100))
        u200, _, d200 = R.run_simulation(N=64, dt=1e-3, nu=nu, total_time=0.2,
                                         save_every_time=0.01, return_diagnostics=True)
        c200 = tg_numpy.compact_from_physical(np.asarray(u200))
        o = {}
        for name, c in (("c100", c100), ("c200", c200)):
            # sparse: modes below 1e-16 of the largest are round-off noise
            flat = c.ravel()
            keep = np.nonzero(np.abs(flat) > 1e-16 * np.abs(flat).max())[0]
            o[f"{name}_shape"] = np.array(c.shape)
            o[f"{name}_idx"] = keep.astype(np.int32)
            o[f"{name}_val"] = flat[keep]
        for k, v in d200.items():
            o[f"series_{k}"] = np.asarray(v)
        np.savez_compressed(os.path.join(HERE, "reference_tg64.npz"), **o)
        print("wrote reference_tg64.npz")


def cupy_packages(ref_root):
    sys.path.insert(0, os.path.join(ref_root, "cuda"))
    from taylor_green_cuda.grid import SpectralGrid
    from taylor_green_cuda.operators import CupySpectralOperator
    from taylor_green_cuda.integrator import RK4Integrator
    from taylor_green_cuda import diagnostics as hd_diag
    from taylor_green_cuda.simulation import TaylorGreenSimulation
    from taylor_green_cuda.config import TaylorGreenConfig
    from taylor_green_mhd.operators import MhdSpectralOperator
    from taylor_green_mhd.integrator import MhdRK4Integrator
    from taylor_green_mhd import diagnostics as mhd_diag
    from taylor_green_mhd.simulation import TaylorGreenMhdSimulation
    from taylor_green_mhd.config import TaylorGreenMhdConfig

    hd_diag.Diagnostics._host = staticmethod(lambda v: float(v))
    mhd_diag.MhdDiagnostics._host = staticmethod(lambda v: float(v))

    L = 2.0 * np.pi
    N = 16
    g = SpectralGrid(N, L)
    out = {}
    u = _seeded_field(N, 77, 0.3)
    b = 0.5 * _seeded_field(N, 78, 0.3)
    uh = np.fft.fftn(u, axes=(-3, -2, -1)) * g.dealias_mask
    bh = np.fft.fftn(b, axes=(-3, -2, -1)) * g.dealias_mask
    out["u_hat"], out["b_hat"] = uh, bh
    out["hd_rhs"] = CupySpectralOperator(g).rhs(uh, 0.02)
    out["hd_step"] = g.dealias(RK4Integrator(CupySpectralOperator(g), 0.004, 0.02).step(uh))
    op = MhdSpectralOperator(g)
    ru, rb = op.rhs(uh, bh, 0.02, 0.03)
    out["mhd_rhs_u"], out["mhd_rhs_b"] = ru, rb
    su, sb = MhdRK4Integrator(op, 0.004, 0.02, 0.03).step((uh, bh))
    out["mhd_step_u"], out["mhd_step_b"] = su, sb
    rec = mhd_diag.MhdDiagnostics(op)
    out["mhd_record"] = np.array(rec.record(0.0, uh, bh))
    out["mhd_record_divu"] = rec.divergence_u_max[0]
    out["mhd_record_divb"] = rec.divergence_b_max[0]

    sim = TaylorGreenSimulation(TaylorGreenConfig(n=8, dt=0.005, reynolds=100.0,
                                                  total_time=0.02, save_every_time=0.01),
                                make_plots=False)
    state, d = sim.run()
    out["hdrun8_state"] = state
    out["hdrun8_times"] = np.array(d.times)
    out["hdrun8_energies"] = np.array(d.energies)
    out["hdrun8_enstrophies"] = np.array(d.enstrophies)

    cfg = TaylorGreenMhdConfig(n=8, dt=0.005, reynolds=100.0, magnetic_reynolds=100.0,
                               magnetic_amplitude=0.5, total_time=0.02, save_every_time=0.01)
    sim = TaylorGreenMhdSimulation(cfg, make_plots=False)
    vh, bh2, d = sim.run()
    out["mhdrun8_u_hat"], out["mhdrun8_b_hat"] = vh, bh2
    for k in ("times", "kinetic_energies", "magnetic_energies", "total_energies",
              "cross_helicities", "enstrophies", "divergence_u_max", "divergence_b_max"):
        out[f"mhdrun8_{k}"] = np.array(getattr(d, k))
    np.savez_compressed(os.path.join(HERE, "reference_cupy.npz"), **out)
    print("wrote reference_cupy.npz")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("TG_REFERENCE_DIR"),
                    help="root of the reference checkout (default: $TG_REFERENCE_DIR)")
    ap.add_argument("--skip-64", action="store_true")
    a = ap.parse_args()
    if not a.reference:
        ap.error("the reference checkout is required: --reference DIR or TG_REFERENCE_DIR")
    _install_stand_ins()
    os.chdir(HERE)  # run_simulation prints; nothing is written by the stand-in plots
    hydro(a.reference, a.skip_64)
    cupy_packages(a.reference)


if __name__ == "__main__":
    main()
