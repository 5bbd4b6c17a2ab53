"""Host-side plan object over the C ABI (include/tgdns.h).

PyTorch provides device memory and the current CUDA stream only; all arithmetic
runs in the hand-written kernels of libtgdns.so.  States are complex tensors of
shape (batch, F, M, M, Hz) holding the dealiased half spectrum (see tgdns.h);
physical fields are real tensors of shape (batch, F, n, n, n).
"""
from __future__ import annotations

import ctypes

import torch

from . import _abi
from ._abi import check

_PHYS = {"hydro": _abi.TG_PHYS_HYDRO, "mhd": _abi.TG_PHYS_MHD}
_PREC = {"f32": _abi.TG_PREC_F32, "f64": _abi.TG_PREC_F64}
_IC = {"taylor_green": _abi.TG_IC_TAYLOR_GREEN, "mhd_reference": _abi.TG_IC_MHD_REFERENCE,
       "mhd_equal_energy": _abi.TG_IC_MHD_EQUAL_ENERGY, "zero": _abi.TG_IC_ZERO}

DIAG_KEYS = ("kinetic_energy", "enstrophy", "dissipation", "magnetic_energy", "cross_helicity",
             "total_energy", "divergence_u_max", "divergence_b_max")


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


class Plan:
    """A batch of ``batch`` independent runs on an ``n``^3 grid."""

    def __init__(self, n, batch=1, physics="hydro", precision="f32", explicit_viscosity=False,
                 lorentz_sign=1.0, cutoff=0, device=None, autotune=False):
        """``autotune``: time the register-resident and shared-memory pass variants, then the
        y-pass configurations, on this shape and batch when the plan is created and keep the
        fastest (``variant``, ``y_config``; TG_AUTOTUNE_CACHE names a file that keeps the
        choices across processes)."""
        if not torch.cuda.is_available():
            raise RuntimeError("jax_tg_project_gb300 needs a CUDA device (no CPU path exists)")
        self.lib = _abi.load()
        self.device = torch.device(device or "cuda")
        self.n = int(n)
        self.batch = int(batch)
        self.physics = physics
        self.precision = precision
        self.F = 6 if physics == "mhd" else 3
        flags = 0
        if explicit_viscosity:
            flags |= _abi.TG_FLAG_EXPLICIT_VISC
        if lorentz_sign < 0:
            flags |= _abi.TG_FLAG_LORENTZ_REF
        if autotune:
            flags |= _abi.TG_FLAG_AUTOTUNE
        self.lorentz_sign = -1.0 if lorentz_sign < 0 else 1.0
        desc = _abi.TgDesc(self.n, self.batch, _PHYS[physics], _PREC[precision], flags, int(cutoff))
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            check(self.lib.tg_plan_create(ctypes.byref(h), ctypes.byref(desc)))
        self._h = h
        dims = (ctypes.c_int * 7)()
        self.lib.tg_state_layout(self._h, dims)
        self.state_shape = tuple(dims[i] for i in range(5))
        self.K = dims[5]
        self.M = dims[2]
        self.Hz = dims[4]
        self.real_dtype = torch.float64 if precision == "f64" else torch.float32
        self.complex_dtype = torch.complex128 if precision == "f64" else torch.complex64

    # ------------------------------------------------------------------ plumbing
    def close(self):
        if getattr(self, "_h", None):
            self.lib.tg_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001 - interpreter shutdown
            pass

    def _sync_stream(self):
        s = torch.cuda.current_stream(self.device).cuda_stream
        check(self.lib.tg_set_stream(self._h, ctypes.c_void_p(s)))

    @property
    def scratch_bytes(self):
        return int(self.lib.tg_plan_scratch_bytes(self._h))

    @property
    def state_bytes(self):
        """Bytes of one state tensor (state_shape, complex)."""
        n = 1
        for d in self.state_shape:
            n *= d
        return n * (8 if self.precision == "f32" else 16)

    @property
    def variant(self):
        """Pass variant in use: bit 0 = shared-memory z passes, bit 1 = shared-memory x passes,
        bit 2 = the x stage with its state stashed in shared memory (64 ... 256)."""
        return int(self.lib.tg_pass_variant(self._h))

    @property
    def y_config(self):
        """(configuration in use, configurations built) of the y pass: radix plan and kz
        columns per CTA, chosen by ``autotune`` (0 = the default)."""
        count = ctypes.c_int(0)
        cur = int(self.lib.tg_y_config(self._h, ctypes.byref(count)))
        return cur, int(count.value)

    @property
    def last_launch_count(self):
        return int(self.lib.tg_last_launch_count(self._h))

    def _check_state(self, s):
        if not (isinstance(s, torch.Tensor) and s.is_cuda and s.dtype == self.complex_dtype
                and tuple(s.shape) == self.state_shape and s.is_contiguous()):
            raise ValueError(f"state must be a contiguous {self.complex_dtype} CUDA tensor of shape "
                             f"{self.state_shape}")
        return s

    def _check_phys(self, u):
        shape = (self.batch, self.F, self.n, self.n, self.n)
        if not (isinstance(u, torch.Tensor) and u.is_cuda and u.dtype == self.real_dtype
                and tuple(u.shape) == shape and u.is_contiguous()):
            raise ValueError(f"physical field must be a contiguous {self.real_dtype} CUDA tensor "
                             f"of shape {shape}")
        return u

    def new_state(self):
        return torch.zeros(self.state_shape, dtype=self.complex_dtype, device=self.device)

    def new_physical(self):
        return torch.zeros((self.batch, self.F, self.n, self.n, self.n), dtype=self.real_dtype,
                           device=self.device)

    # ------------------------------------------------------------------ operations
    def set_run_params(self, nu=None, eta=None, dt=None):
        def arr(v):
            if v is None:
                return None, 0
            vals = [float(x) for x in (v if hasattr(v, "__len__") else [v])]
            return (ctypes.c_double * len(vals))(*vals), len(vals)

        a, na = arr(nu)
        b, nb = arr(eta)
        c, nc = arr(dt)
        counts = {x for x in (na, nb, nc) if x}
        if len(counts) > 1:
            raise ValueError("nu, eta and dt must have the same length")
        count = counts.pop() if counts else 1
        self._sync_stream()
        check(self.lib.tg_set_run_params(self._h, a, b, c, count))

    def initial_condition(self, kind="taylor_green", seed=0, pert_amp=0.0, k0=4.0, b_amp=0.5,
                          out=None):
        s = self._check_state(out) if out is not None else self.new_state()
        self._sync_stream()
        check(self.lib.tg_initial_condition(self._h, _IC[kind], int(seed) & (2 ** 64 - 1),
                                            float(pert_amp), float(k0), float(b_amp), _ptr(s)))
        return s

    def forward(self, phys, out=None):
        self._check_phys(phys)
        s = self._check_state(out) if out is not None else self.new_state()
        self._sync_stream()
        check(self.lib.tg_forward(self._h, _ptr(phys), _ptr(s)))
        return s

    def inverse(self, state, out=None):
        self._check_state(state)
        u = self._check_phys(out) if out is not None else self.new_physical()
        self._sync_stream()
        check(self.lib.tg_inverse(self._h, _ptr(state), _ptr(u)))
        return u

    def rhs(self, state, nu=-1.0, eta=-1.0, out=None):
        self._check_state(state)
        r = self._check_state(out) if out is not None else self.new_state()
        self._sync_stream()
        check(self.lib.tg_rhs(self._h, _ptr(state), float(nu), float(eta), _ptr(r)))
        return r

    def step(self, state, dt=-1.0, nu=-1.0, eta=-1.0, nsteps=1):
        self._check_state(state)
        self._sync_stream()
        check(self.lib.tg_step(self._h, _ptr(state), float(dt), float(nu), float(eta), int(nsteps)))
        return state

    def run(self, state, dt=-1.0, nu=-1.0, eta=-1.0, nsteps=1, save_every=1):
        self._check_state(state)
        # (save_every < 1 is rejected by tg_run with TG_E_INVALID)
        nrec = 1 + (nsteps // save_every + (1 if nsteps % save_every else 0) if save_every >= 1 else 0)
        series = torch.zeros((nrec, self.batch, _abi.TG_DIAG_WIDTH), dtype=torch.float64,
                             device=self.device)
        self._sync_stream()
        check(self.lib.tg_run(self._h, _ptr(state), float(dt), float(nu), float(eta), int(nsteps),
                              int(save_every), _ptr(series)))
        return series

    def diagnostics(self, state, nu=-1.0, eta=-1.0):
        self._check_state(state)
        out = torch.zeros((self.batch, _abi.TG_DIAG_WIDTH), dtype=torch.float64, device=self.device)
        self._sync_stream()
        check(self.lib.tg_diagnostics(self._h, _ptr(state), float(nu), float(eta), _ptr(out)))
        return out

    def profile_passes(self, state, dt=-1.0, nu=-1.0, eta=-1.0, nsteps=1):
        """Mean CUDA-event duration (ms) and count of each pass kind over nsteps eager steps."""
        self._check_state(state)
        ms = (ctypes.c_double * _abi.TG_PROF_SLOTS)()
        cnt = (ctypes.c_int64 * _abi.TG_PROF_SLOTS)()
        self._sync_stream()
        check(self.lib.tg_profile_passes(self._h, _ptr(state), float(dt), float(nu), float(eta),
                                         int(nsteps), ms, cnt))
        return {name: (ms[i], int(cnt[i])) for i, name in enumerate(_abi.PASS_NAMES) if cnt[i]}

    def derived(self, state, which="vorticity"):
        """Physical curl (vorticity [, current]) or divergence field(s) of a state."""
        self._check_state(state)
        sel = _abi.TG_DERIVED_VORTICITY if which == "vorticity" else _abi.TG_DERIVED_DIVERGENCE
        nf = self.F if sel == _abi.TG_DERIVED_VORTICITY else self.F // 3
        out = torch.empty((self.batch, nf, self.n, self.n, self.n), dtype=self.real_dtype,
                          device=self.device)
        self._sync_stream()
        check(self.lib.tg_derived(self._h, _ptr(state), sel, _ptr(out)))
        return out

    def to_full(self, state):
        """State -> full complex fftn layout (batch, F, n, n, n), unnormalised."""
        self._check_state(state)
        out = torch.empty((self.batch, self.F, self.n, self.n, self.n), dtype=self.complex_dtype,
                          device=self.device)
        self._sync_stream()
        check(self.lib.tg_to_full_spectrum(self._h, _ptr(state), _ptr(out)))
        return out

    def from_full(self, full, out=None):
        shape = (self.batch, self.F, self.n, self.n, self.n)
        if not (isinstance(full, torch.Tensor) and full.is_cuda and full.dtype == self.complex_dtype
                and tuple(full.shape) == shape and full.is_contiguous()):
            raise ValueError(f"full spectrum must be a contiguous {self.complex_dtype} CUDA tensor "
                             f"of shape {shape}")
        s = self._check_state(out) if out is not None else self.new_state()
        self._sync_stream()
        check(self.lib.tg_from_full_spectrum(self._h, _ptr(full), _ptr(s)))
        return s

    def physical_energy(self, phys):
        """0.5 <|u|^2> [, 0.5 <|b|^2>] of physical fields, FP64, shape (batch, F/3)."""
        self._check_phys(phys)
        out = torch.zeros((self.batch, self.F // 3), dtype=torch.float64, device=self.device)
        self._sync_stream()
        check(self.lib.tg_physical_energy(self._h, _ptr(phys), _ptr(out)))
        return out

    def adjoint(self, state0, dt, nu, nsteps, checkpoint_every=0):
        """(loss, grad_state, grad_nu) of loss = final enstrophy after nsteps steps.

        checkpoint_every: > 0 checkpoints every that many steps and recomputes each
        segment (recording its stage tape in pinned host memory where the plan has the tape
        kernels); 0 every ceil(sqrt(nsteps)) steps; "tape" (or -1) records every step's
        stage data in pinned host memory in one forward sweep and recomputes nothing.
        """
        if checkpoint_every == "tape":
            checkpoint_every = _abi.TG_ADJ_HOST_TAPE
        self._check_state(state0)
        grad = self.new_state()
        out = torch.zeros(2, dtype=torch.float64, device=self.device)  # grad_nu, loss
        self._sync_stream()
        check(self.lib.tg_adjoint(self._h, _ptr(state0), float(dt), float(nu), int(nsteps),
                                  int(checkpoint_every), _ptr(grad), ctypes.c_void_p(out.data_ptr()),
                                  ctypes.c_void_p(out.data_ptr() + 8)))
        return out[1], grad, out[0]

    def adjoint_profile(self):
        """Device time (ms) of the phases of the last stage-tape ``adjoint`` call: the forward
        run with the loss, the tape recording sweeps of the segments, the backward sweeps."""
        ms = (ctypes.c_double * 3)()
        check(self.lib.tg_adjoint_profile(self._h, ms))
        return {"forward": ms[0], "record": ms[1], "backward": ms[2]}

    def release_tape(self):
        """Free the pinned host memory a ``checkpoint_every="tape"`` adjoint keeps for later calls."""
        check(self.lib.tg_release_host_tape(self._h))

    def energy_spectrum(self, state):
        """E(k) per run: (batch, bins) hydro or (batch, 2, bins) MHD (kinetic, magnetic)."""
        self._check_state(state)
        nb = int(self.lib.tg_spectrum_bins(self._h))
        shape = (self.batch, nb) if self.F == 3 else (self.batch, 2, nb)
        out = torch.zeros(shape, dtype=torch.float64, device=self.device)
        self._sync_stream()
        check(self.lib.tg_energy_spectrum(self._h, _ptr(state), _ptr(out)))
        return out

    def save(self, path, state, **meta):
        """Write the state (compact coefficients, padding dropped) and metadata to an .npz file."""
        import numpy as np
        self._check_state(state)
        np.savez_compressed(path, coefficients=state[..., : self.K + 1].cpu().numpy(), n=self.n,
                            physics=self.physics, precision=self.precision, K=self.K,
                            **{k: np.asarray(v) for k, v in meta.items()})

    def load(self, path):
        """Read a state written by ``save`` (same n, physics and cutoff); returns (state, meta)."""
        import numpy as np
        d = np.load(path, allow_pickle=False)
        if int(d["n"]) != self.n or str(d["physics"]) != self.physics or int(d["K"]) != self.K:
            raise ValueError(f"{path}: saved for n={int(d['n'])}, physics={d['physics']}, "
                             f"K={int(d['K'])}; this plan is n={self.n}, physics={self.physics}")
        c = d["coefficients"]
        if c.shape[0] != self.batch:
            raise ValueError(f"{path}: {c.shape[0]} runs saved, plan has batch {self.batch}")
        s = self.new_state()
        s[..., : self.K + 1] = torch.from_numpy(c).to(self.complex_dtype).to(self.device)
        meta = {k: d[k] for k in d.files if k not in ("coefficients", "n", "physics", "precision", "K")}
        return s, meta

    def absmax(self, state, which="velocity"):
        self._check_state(state)
        sel = _abi.TG_ABSMAX_VELOCITY if which == "velocity" else _abi.TG_ABSMAX_DIVERGENCE
        nf = self.F if sel == _abi.TG_ABSMAX_VELOCITY else self.F // 3
        out = torch.zeros((self.batch, nf), dtype=torch.float64, device=self.device)
        self._sync_stream()
        check(self.lib.tg_field_absmax(self._h, _ptr(state), sel, _ptr(out)))
        return out
