"""Write tg_consts.cuh: cos/sin(2*pi*m/96) for m = 0..95, correctly rounded.

Every radix used by the in-register DFT codelets (2, 3, 4, 6, 8, 12, 16, 24, 32,
48, 96) divides 96, so W_R^m = W_96^(m*96/R).  Values are computed with mpmath at
50 digits and rounded once to IEEE double; exact 0, +-1/2 and +-1 come out exact.
Run: python jax_tg_project_gb300/csrc/gen_consts.py
"""
import os

import mpmath

mpmath.mp.dps = 50
HERE = os.path.dirname(os.path.abspath(__file__))


def main():
    cos_v, sin_v = [], []
    for m in range(96):
        a = 2 * mpmath.pi * m / 96
        cos_v.append(float(mpmath.cos(a)))
        sin_v.append(float(mpmath.sin(a)))
    for arr in (cos_v, sin_v):
        for i, v in enumerate(arr):
            if abs(v) < 1e-30:
                arr[i] = 0.0
    body = ["// Generated by gen_consts.py -- do not edit.",
            "// cos/sin(2*pi*m/96), m = 0..95, correctly rounded to double.",
            "#pragma once", "namespace tg {",
            "__host__ __device__ constexpr double kCos96(int m) {",
            "  constexpr double t[96] = {"]
    body += ["    " + ", ".join(repr(v) for v in cos_v[i:i + 4]) + "," for i in range(0, 96, 4)]
    body += ["  };", "  return t[m];", "}",
             "__host__ __device__ constexpr double kSin96(int m) {",
             "  constexpr double t[96] = {"]
    body += ["    " + ", ".join(repr(v) for v in sin_v[i:i + 4]) + "," for i in range(0, 96, 4)]
    body += ["  };", "  return t[m];", "}", "}  // namespace tg", ""]
    with open(os.path.join(HERE, "tg_consts.cuh"), "w") as f:
        f.write("\n".join(body))


if __name__ == "__main__":
    main()
