"""CPU oracle for the Taylor-Green pseudo-spectral time step.

TEST INFRASTRUCTURE ONLY.  This package is a plain NumPy FP64 restatement of the
reference solvers (``jax/taylor_green_jax.py`` for hydro and the CuPy
``cuda/taylor_green_mhd`` package for MHD).  It is imported by ``tests/``,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference`` legs
of ``bench.py``, as the reference values of parity tests and as the timed CPU
baseline.  The product path
(``jax_tg_project_gb300``) never imports it and has no CPU fallback.

Pinning: the restatement is checked against outputs of the reference's own
Python code, run in this container with NumPy standing in for ``jax.numpy`` and
``cupy`` (neither is installed).  The fixtures and the script that generated
them live in ``tests/golden/``.
"""
from . import tg_numpy, mhd_numpy, perturb  # noqa: F401
