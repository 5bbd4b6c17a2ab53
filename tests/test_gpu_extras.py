"""CLI, state save / resume and the energy spectrum."""
import io
import contextlib

import numpy as np
import pytest

from conftest import from_state, rel_l2

pytestmark = pytest.mark.gpu


def test_energy_spectrum_sums_to_energy():
    import jax_tg_project_gb300 as tg
    p = tg.Plan(32, batch=2)
    s = p.initial_condition("taylor_green", seed=4, pert_amp=0.05, k0=4.0)
    e = p.energy_spectrum(s).cpu().numpy()
    d = p.diagnostics(s, nu=0.0).cpu().numpy()
    np.testing.assert_allclose(e.sum(axis=1), d[:, 0], rtol=1e-12)
    tgs = p.initial_condition("taylor_green")
    e0 = p.energy_spectrum(tgs).cpu().numpy()[0]
    assert e0[2] == pytest.approx(0.125, rel=1e-7) and abs(e0.sum() - e0[2]) < 1e-12  # |k| = sqrt(3)
    pm = tg.Plan(16, physics="mhd")
    sm = pm.initial_condition("mhd_equal_energy")
    em = pm.energy_spectrum(sm).cpu().numpy()[0]
    assert em[0].sum() == pytest.approx(0.125, rel=1e-7) and em[1].sum() == pytest.approx(0.125, rel=1e-7)


def test_save_and_resume_continue_a_run(tmp_path):
    import jax_tg_project_gb300 as tg
    p = tg.Plan(32)
    a = p.initial_condition("taylor_green", seed=1, pert_amp=0.02, k0=3.0)
    b = a.clone()
    p.step(a, dt=2e-3, nu=0.005, nsteps=10)
    p.step(b, dt=2e-3, nu=0.005, nsteps=4)
    path = str(tmp_path / "state.npz")
    p.save(path, b, step=4, time=8e-3)
    c, meta = p.load(path)
    assert int(meta["step"]) == 4
    p.step(c, dt=2e-3, nu=0.005, nsteps=6)
    assert rel_l2(from_state(p, c), from_state(p, a)) < 1e-12
    with pytest.raises(ValueError):
        tg.Plan(16).load(path)


def test_cli_hydro_and_resume(tmp_path):
    from jax_tg_project_gb300 import cli
    path = str(tmp_path / "run.npz")
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        cli.main(["hydro", "--n", "16", "--dt", "0.005", "--reynolds", "100", "--total-time", "0.02",
                  "--save-every-time", "0.01", "--save", path, "--spectrum", "--no-plots"])
    out = buf.getvalue()
    assert "Save time step: 2," in out and "Save time step: 4," in out and "E(k):" in out
    buf2 = io.StringIO()
    with contextlib.redirect_stdout(buf2):
        s2 = cli.main(["hydro", "--n", "16", "--dt", "0.005", "--reynolds", "100", "--total-time", "0.02",
                       "--save-every-time", "0.01", "--resume", path, "--plot-dir", str(tmp_path)])
    assert "Save time step: 6," in buf2.getvalue()
    from jax_tg_project_gb300.plots import read_png
    for f in ("taylor_green_cuda_slice.png", "taylor_green_cuda_diagnostics.png"):
        img = read_png(str(tmp_path / f))
        assert img.ndim == 3 and (img != 255).any()
    buf3 = io.StringIO()
    with contextlib.redirect_stdout(buf3):
        s3 = cli.main(["hydro", "--n", "16", "--dt", "0.005", "--reynolds", "100", "--total-time", "0.04",
                       "--save-every-time", "0.01", "--no-plots"])
    assert abs(float(s2[-1, 0, 0]) - float(s3[-1, 0, 0])) < 1e-12
    buf4 = io.StringIO()
    with contextlib.redirect_stdout(buf4):
        cli.main(["mhd", "--n", "8", "--dt", "0.005", "--reynolds", "100", "--magnetic-reynolds", "100",
                  "--total-time", "0.02", "--save-every-time", "0.01", "--plot-dir", str(tmp_path)])
    assert "E_m:" in buf4.getvalue() and "taylor_green_mhd_slice.png" in buf4.getvalue()
    assert read_png(str(tmp_path / "taylor_green_mhd_slice.png")).shape[0] > \
        read_png(str(tmp_path / "taylor_green_cuda_slice.png")).shape[0]  # two panel rows (u, B)
    buf5 = io.StringIO()
    with contextlib.redirect_stdout(buf5):
        cli.main(["native", "16", "0.005", "100", "0.01", "0.005"])
    assert "Save time step: 2," in buf5.getvalue()


def test_run_simulation_plots(tmp_path):
    """make_plots writes the reference's PNG files; the JAX-form slice is the y = N/2 plane."""
    import numpy as np

    from jax_tg_project_gb300 import taylor_green
    from jax_tg_project_gb300.plots import read_png
    u, e = taylor_green.run_simulation(N=16, dt=0.005, nu=0.01, total_time=0.02, save_every_time=0.01,
                                       verbose=False, make_plots=True, plot_dir=str(tmp_path))
    img = read_png(str(tmp_path / "taylor_green_slice.png"))
    d = read_png(str(tmp_path / "taylor_green_diagnostics.png"))
    assert img.shape[2] == 3 and d.shape[0] == 2 * 320  # energy and enstrophy panels
    # w = 0 for Taylor-Green at t = 0 stays ~0: its panel is a single colour
    assert np.isfinite(u.cpu().numpy()).all() and e[-1] < e[0]
