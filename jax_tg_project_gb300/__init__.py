"""GB300-native pseudo-spectral Taylor-Green DNS (hydro and MHD).

Hand-written sm_103a CUDA kernels (``csrc/``) behind a C ABI
(``include/tgdns.h``), bound with ctypes.  ``Plan`` is the low-level handle;
``taylor_green`` mirrors the reference JAX solver's function API and ``mhd``
the reference CuPy MHD shim.
"""
from .plan import DIAG_KEYS, Plan  # noqa: F401

__version__ = "0.1.0"
