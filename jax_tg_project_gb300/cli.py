"""Command line front-end (python -m jax_tg_project_gb300 ...).

Subcommands mirror the reference's entry points:

  hydro   --n --dt --reynolds | --nu --total-time --save-every-time --no-plots
          (cuda/taylor_green_cuda/cli.py:7-23 and jax/taylor_green_jax.py run_simulation)
  mhd     --n --dt --reynolds --magnetic-reynolds --magnetic-amplitude --total-time
          --save-every-time --no-plots  (cuda/taylor_green_mhd/cli.py:7-29)
  native  N dt Re total_time save_time  (the positional form of cuda/taylor_green_cuda.cu:125)

Extensions: --precision f32|f64, --save PATH (final state + series to .npz), --resume PATH
(start from a saved state, continuing its step count and time), --spectrum (print E(k) at the
end), --plot-dir DIR.  Like the reference CLIs, the hydro and mhd subcommands write the slice
and diagnostics PNGs (headless, plots.py) unless --no-plots is given.
"""
from __future__ import annotations

import argparse
import json
import math
import sys
import time

import numpy as np


def _run(physics, n, dt, nu, eta, total_time, save_every_time, precision, save, resume,
         spectrum, b_amp, lorentz_sign, out=None, plots=False, plot_dir="."):
    import torch

    out = out or sys.stdout
    from .config import step_counts, validate_timestep, validate_timestep_mhd, wavenumber_axis
    from .plan import DIAG_KEYS, Plan

    plan = Plan(n, physics=physics, precision=precision, lorentz_sign=lorentz_sign)
    step0, t0 = 0, 0.0
    if resume:
        state, meta = plan.load(resume)
        step0 = int(meta.get("step", 0))
        t0 = float(meta.get("time", 0.0))
    elif physics == "mhd":
        state = plan.initial_condition("mhd_reference", b_amp=b_amp)
    else:
        state = plan.initial_condition("taylor_green")
    steps, save_every = step_counts(total_time, dt, save_every_time)
    k = wavenumber_axis(n)
    umax = plan.absmax(state, "velocity").cpu().numpy()[0]
    if physics == "mhd":
        validate_timestep_mhd(dt, nu, eta, k, k, k, max_velocity=float(umax[:3].max()),
                              max_field=max(float(umax[3:].max()), 1e-30))
    else:
        validate_timestep(dt, nu, k, k, k, 0.5, max_velocity=float(umax.max()))
    t_start = time.perf_counter()
    series = plan.run(state, dt=dt, nu=nu, eta=eta, nsteps=steps, save_every=save_every)
    torch.cuda.synchronize()
    elapsed = time.perf_counter() - t_start
    h = series[:, 0].cpu().numpy()
    times, s = [t0], 0
    while s < steps:
        s = min(s + save_every - (s % save_every), steps)
        times.append(t0 + s * dt)
    for i in range(1, len(times)):
        stepno = step0 + int(round((times[i] - t0) / dt))
        if physics == "mhd":
            print(f"Save time step: {stepno}, time: {times[i]:.6f}, E_k: {h[i, 0]:.8e}, "
                  f"E_m: {h[i, 3]:.8e}, H_c: {h[i, 4]:.8e}, enstrophy: {h[i, 1]:.8e}", file=out)
        else:
            print(f"Save time step: {stepno}, time: {times[i]:.6f}, enstrophy: {h[i, 1]:.8e}",
                  file=out)
    print(f"CUDA device: {torch.cuda.get_device_name()}", file=out)
    print(f"Reynolds number: Re = {2 * math.pi / nu if nu > 0 else float('inf'):.1f}", file=out)
    print(f"Simulated time: {total_time:.3f} ({steps} steps) in {elapsed:.3f} s", file=out)
    print(f"Energy trace: {h[0, 0]:.6f} -> {h[-1, 0]:.6f}", file=out)
    print(f"Max divergence: {h[:, 6].max():.3e}", file=out)
    if spectrum:
        e = plan.energy_spectrum(state).cpu().numpy()[0]
        print("E(k): " + json.dumps([float(x) for x in np.atleast_2d(e)[0]]), file=out)
    if plots:
        from .plots import save_plots
        r = save_plots(plan, state, times, series.cpu().numpy(), kind=physics, directory=plot_dir)
        lo, hi = min(x[0] for x in r["slice_ranges"]), max(x[1] for x in r["slice_ranges"])
        print(f"Saved: {r['slice']} (values {lo:.4e} .. {hi:.4e})", file=out)
        print(f"Saved: {r['diagnostics']}", file=out)
    if save:
        plan.save(save, state, step=step0 + steps, time=t0 + steps * dt, nu=nu, eta=eta, dt=dt,
                  series=series.cpu().numpy(), series_keys=np.array(DIAG_KEYS), times=np.array(times))
        print(f"Saved: {save}", file=out)
    return series


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m jax_tg_project_gb300",
                                 description="3D Taylor-Green vortex on one GB300 (sm_103a)")
    sub = ap.add_subparsers(dest="cmd", required=True)

    def common(p, n=128, dt=0.005, total=1.0, save_every=0.05):
        p.add_argument("--n", type=int, default=n)
        p.add_argument("--dt", type=float, default=dt)
        p.add_argument("--total-time", type=float, default=total)
        p.add_argument("--save-every-time", type=float, default=save_every)
        p.add_argument("--no-plots", action="store_true")
        p.add_argument("--plot-dir", default=".")
        p.add_argument("--precision", choices=("f32", "f64"), default="f32")
        p.add_argument("--save", default=None)
        p.add_argument("--resume", default=None)
        p.add_argument("--spectrum", action="store_true")

    ph = sub.add_parser("hydro", help="hydrodynamic Taylor-Green run")
    common(ph)
    ph.add_argument("--reynolds", type=float, default=1000.0)
    ph.add_argument("--nu", type=float, default=None, help="viscosity (overrides --reynolds)")
    pm = sub.add_parser("mhd", help="resistive MHD Taylor-Green run")
    common(pm)
    pm.add_argument("--reynolds", type=float, default=1000.0)
    pm.add_argument("--magnetic-reynolds", type=float, default=1000.0)
    pm.add_argument("--magnetic-amplitude", type=float, default=0.5)
    pm.add_argument("--lorentz-sign", type=float, default=1.0,
                    help="-1 reproduces the reference code's sign of j x b")
    pn = sub.add_parser("native", help="positional form: N dt Re total_time save_time")
    pn.add_argument("N", type=int, nargs="?", default=128)
    pn.add_argument("dt", type=float, nargs="?", default=0.005)
    pn.add_argument("Re", type=float, nargs="?", default=1000.0)
    pn.add_argument("total", type=float, nargs="?", default=1.0)
    pn.add_argument("save", type=float, nargs="?", default=0.05)
    a = ap.parse_args(argv)
    from .config import TaylorGreenConfig, TaylorGreenMhdConfig
    if a.cmd == "native":
        cfg = TaylorGreenConfig(a.N, a.dt, a.Re, a.total, a.save)
        return _run("hydro", cfg.n, cfg.dt, cfg.viscosity, 0.0, cfg.total_time, cfg.save_every_time,
                    "f32", None, None, False, 0.0, 1.0)
    if a.cmd == "hydro":
        cfg = TaylorGreenConfig(a.n, a.dt, a.reynolds, a.total_time, a.save_every_time)
        nu = cfg.viscosity if a.nu is None else a.nu
        return _run("hydro", cfg.n, cfg.dt, nu, 0.0, cfg.total_time, cfg.save_every_time,
                    a.precision, a.save, a.resume, a.spectrum, 0.0, 1.0, plots=not a.no_plots,
                    plot_dir=a.plot_dir)
    cfg = TaylorGreenMhdConfig(n=a.n, dt=a.dt, reynolds=a.reynolds,
                               magnetic_reynolds=a.magnetic_reynolds,
                               magnetic_amplitude=a.magnetic_amplitude, total_time=a.total_time,
                               save_every_time=a.save_every_time)
    return _run("mhd", cfg.n, cfg.dt, cfg.viscosity, cfg.resistivity, cfg.total_time,
                cfg.save_every_time, a.precision, a.save, a.resume, a.spectrum,
                cfg.magnetic_amplitude, a.lorentz_sign, plots=not a.no_plots, plot_dir=a.plot_dir)


if __name__ == "__main__":
    main()
