"""Plan cache and tensor plumbing shared by the reference-shaped APIs."""
from __future__ import annotations

import numpy as np
import torch

from .plan import Plan

_DEFAULTS = {"precision": "f32", "scheme": "lawson"}
_CACHE: dict = {}


def set_default_precision(precision: str) -> None:
    """'f32' (default, the GB300 fast path) or 'f64' (the FP64 check mode)."""
    if precision not in ("f32", "f64"):
        raise ValueError("precision must be 'f32' or 'f64'")
    _DEFAULTS["precision"] = precision


def set_default_scheme(scheme: str) -> None:
    """'lawson' (integrating-factor RK4, default) or 'explicit' (the reference's RK4)."""
    if scheme not in ("lawson", "explicit"):
        raise ValueError("scheme must be 'lawson' or 'explicit'")
    _DEFAULTS["scheme"] = scheme


def default_precision(precision=None):
    return precision or _DEFAULTS["precision"]


def get_plan(n, physics="hydro", precision=None, scheme=None, lorentz_sign=1.0):
    precision = default_precision(precision)
    scheme = scheme or _DEFAULTS["scheme"]
    key = (int(n), physics, precision, scheme, float(np.sign(lorentz_sign) or 1.0),
           torch.cuda.current_device())
    p = _CACHE.get(key)
    if p is None:
        p = Plan(n, physics=physics, precision=precision, explicit_viscosity=(scheme == "explicit"),
                 lorentz_sign=lorentz_sign)
        _CACHE[key] = p
    return p


def clear_plans() -> None:
    for p in _CACHE.values():
        p.close()
    _CACHE.clear()


def as_physical(u, plan, components):
    """Any array-like (C, N, N, N) -> contiguous (1, C, N, N, N) CUDA tensor of the plan dtype."""
    t = u if isinstance(u, torch.Tensor) else torch.as_tensor(np.asarray(u))
    if t.dim() != 4 or t.shape[0] != components or any(s != plan.n for s in t.shape[1:]):
        raise ValueError(f"expected a field of shape ({components}, {plan.n}, {plan.n}, {plan.n}), "
                         f"got {tuple(t.shape)}")
    return t.to(device=plan.device, dtype=plan.real_dtype).contiguous().unsqueeze(0)


def as_full_spectrum(f, plan, components):
    t = f if isinstance(f, torch.Tensor) else torch.as_tensor(np.asarray(f))
    if t.dim() != 4 or t.shape[0] != components or any(s != plan.n for s in t.shape[1:]):
        raise ValueError(f"expected a spectrum of shape ({components}, {plan.n}, {plan.n}, {plan.n}), "
                         f"got {tuple(t.shape)}")
    return t.to(device=plan.device, dtype=plan.complex_dtype).contiguous().unsqueeze(0)


def grid_size(*arrays):
    """N from the first array-like argument with a 3-D trailing shape."""
    for a in arrays:
        shape = getattr(a, "shape", None)
        if shape is not None and len(shape) >= 3:
            return int(shape[-1])
    raise ValueError("cannot infer the grid size")
