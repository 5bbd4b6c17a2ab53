"""Build libtgdns.so (the sm_103a kernels and the C ABI) in-tree with nvcc.

``tg_inst.cu`` is compiled once per (real type, grid size) with -DTG_REAL and
-DTG_N, in parallel, plus ``tg_api.cu``; the objects are linked into
``jax_tg_project_gb300/lib/libtgdns.so``.  A content hash of the sources and
flags skips up-to-date builds.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(os.path.dirname(PKG), "include")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIBDIR, "libtgdns.so")

SIZES_F32 = (8, 12, 16, 24, 32, 48, 64, 96, 128, 256, 512)
SIZES_F64 = (8, 16, 32, 64, 96, 128, 256)
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", CSRC, "-I", INCLUDE]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found (set NVCC or put CUDA's bin/ on PATH)")


def _sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC)
                  if f.endswith((".cu", ".cuh", ".h"))) + [os.path.join(INCLUDE, "tgdns.h")]


def _digest(extra=()):
    h = hashlib.sha256()
    for p in _sources():
        with open(p, "rb") as f:
            h.update(p.encode() + f.read())
    h.update(repr((ARCH, FLAGS, SIZES_F32, SIZES_F64, tuple(extra))).encode())
    return h.hexdigest()


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(force: bool = False, verbose: bool = False, jobs: int | None = None) -> str:
    """Compile (if needed) and return the path of libtgdns.so."""
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    stamp = os.path.join(BUILD, "stamp")
    digest = _digest()
    if not force and os.path.exists(LIB) and os.path.exists(stamp):
        with open(stamp) as f:
            if f.read().strip() == digest:
                return LIB
    nvcc = _nvcc()
    units = [(os.path.join(CSRC, "tg_api.cu"), os.path.join(BUILD, "tg_api.o"), []),
             (os.path.join(CSRC, "tg_noalloc.cu"), os.path.join(BUILD, "tg_noalloc.o"), [])]
    for real, sizes in (("float", SIZES_F32), ("double", SIZES_F64)):
        for n in sizes:
            units.append((os.path.join(CSRC, "tg_inst.cu"),
                          os.path.join(BUILD, f"tg_inst_{real}_{n}.o"),
                          [f"-DTG_REAL={real}", f"-DTG_N={n}"]))
    jobs = jobs or max(1, min(len(units), os.cpu_count() or 1))
    logs = []

    def compile_one(u):
        src, obj, defs = u
        return _run([nvcc, *ARCH, *FLAGS, *defs, "-c", src, "-o", obj])

    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        for out in ex.map(compile_one, units):
            logs.append(out)
    tmp = LIB + ".tmp"
    _run([nvcc, *ARCH, "-shared", "-o", tmp, *[u[1] for u in units], "-lcudart"])
    os.replace(tmp, LIB)
    with open(stamp, "w") as f:
        f.write(digest)
    if verbose:
        print("".join(logs))
    return LIB


if __name__ == "__main__":
    import time

    t0 = time.time()
    print(build(force=True), f"{time.time() - t0:.1f} s")
