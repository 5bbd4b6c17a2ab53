"""Seeded divergence-free random perturbation (oracle copy, test-only).

The reference has no random initial condition; the perturbed workloads need one
that the GPU path and this oracle both produce from a seed.  The GPU kernel
(``csrc/tg_init.cu``) and this module implement the same definition:

* for every kept half-spectrum mode (|kx|,|ky| <= K, 0 <= kz <= K, K the
  2/3 cutoff) and component c, two uniforms come from SplitMix64 (Steele,
  Lea & Flood 2014; Vigna's constants) of the counter
  ``((c*N + ix)*N + iy)*(N//2+1) + kz`` (ix, iy the FFT-ordered indices),
  doubled plus 0/1, mixed with ``splitmix64(seed)``;
* Box-Muller turns them into the real and imaginary parts of a unit complex
  Gaussian g_c(k);
* the mode is v(k) = |k| exp(-|k|^2/k0^2) * P(k) g(k)  (P = Leray projector),
  so the shell spectrum is E(k) ~ k^4 exp(-2 k^2 / k0^2); v(0) = 0;
* on the kz = 0 plane the half with (ky < 0) or (ky == 0 and kx < 0) is
  replaced by the conjugate of its mirror so that the field is real;
* the field is scaled so that its per-component rms sqrt(<|u|^2>/3) equals
  ``amp``.

Coefficients are Fourier coefficients (u(x) = sum_k v(k) e^{i k x}).
"""
from __future__ import annotations

import numpy as np

from .tg_numpy import dealias_cutoff

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)
_G = np.uint64(0x9E3779B97F4A7C15)
_C1 = np.uint64(0xBF58476D1CE4E5B9)
_C2 = np.uint64(0x94D049BB133111EB)


def splitmix64(x):
    """SplitMix64 output function of counter(s) ``x`` (uint64, wrapping)."""
    with np.errstate(over="ignore"):
        z = np.asarray(x, dtype=np.uint64) + _G
        z = (z ^ (z >> np.uint64(30))) * _C1
        z = (z ^ (z >> np.uint64(27))) * _C2
        return z ^ (z >> np.uint64(31))


def _uniform(h):
    """53-bit uniform in (0, 1]."""
    return ((h >> np.uint64(11)).astype(np.float64) + 1.0) * (2.0 ** -53)


def gaussian_pairs(seed, counters):
    """Box-Muller standard normals (real, imag) for each counter."""
    key = splitmix64(np.uint64(seed))
    c2 = np.asarray(counters, dtype=np.uint64) * np.uint64(2)
    u1 = _uniform(splitmix64(key ^ c2))
    u2 = _uniform(splitmix64(key ^ (c2 + np.uint64(1))))
    r = np.sqrt(-2.0 * np.log(u1))
    t = 2.0 * np.pi * u2
    return r * np.cos(t), r * np.sin(t)


def perturbation_compact(N, seed, amp=1e-3, k0=4.0):
    """Compact coefficients (3, 2K+1, 2K+1, K+1) of the perturbation."""
    K = dealias_cutoff(N)
    H = N // 2 + 1
    sig = np.concatenate([np.arange(0, K + 1), np.arange(-K, 0)]).astype(np.int64)
    ix = np.where(sig < 0, sig + N, sig)  # FFT-ordered index of each kept mode
    kz = np.arange(0, K + 1, dtype=np.int64)
    IX, IY, IZ = np.meshgrid(ix, ix, kz, indexing="ij")
    KX, KY, KZ = np.meshgrid(sig.astype(np.float64), sig.astype(np.float64),
                             kz.astype(np.float64), indexing="ij")
    g = []
    for c in range(3):
        cnt = ((np.uint64(c) * np.uint64(N) + IX.astype(np.uint64)) * np.uint64(N)
               + IY.astype(np.uint64)) * np.uint64(H) + IZ.astype(np.uint64)
        re, im = gaussian_pairs(seed, cnt)
        g.append(re + 1j * im)
    g = np.stack(g)
    k2 = KX * KX + KY * KY + KZ * KZ
    k2s = np.where(k2 == 0.0, 1.0, k2)
    kd = KX * g[0] + KY * g[1] + KZ * g[2]
    g = g - np.stack([KX * kd / k2s, KY * kd / k2s, KZ * kd / k2s])
    kk = np.sqrt(k2)
    v = g * (kk * np.exp(-k2 / (k0 * k0)))[None]
    v[:, 0, 0, 0] = 0.0
    # Hermitian completion of the kz = 0 plane: index of -k on a compact axis
    neg = np.where(np.arange(2 * K + 1) == 0, 0,
                   (2 * K + 1) - np.arange(2 * K + 1))
    plane = v[:, :, :, 0]
    mirror = np.conj(plane[:, neg][:, :, neg])
    s = sig
    lower = (s[None, :] < 0) | ((s[None, :] == 0) & (s[:, None] < 0))
    plane = np.where(lower[None], mirror, plane)
    v[:, :, :, 0] = plane
    w = np.where(np.arange(K + 1) == 0, 1.0, 2.0)[None, None, None, :]
    msq = float(np.sum(w * np.abs(v) ** 2))  # <|u|^2>
    if msq > 0.0:
        v *= amp / np.sqrt(msq / 3.0)
    return v
