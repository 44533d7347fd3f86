"""Build libsymeig.so in-tree with nvcc for sm_103a (GB300).

Each translation unit compiles in its own nvcc process (in parallel), then nvcc links the
shared library with the CUDA runtime linked statically.  No cmake, no torch extension
machinery: the library is a plain C ABI that Julia (ccall) or Python (ctypes) loads.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT = PKG / "_build"
LIB = OUT / "libsymeig.so"
SOURCES = ["apply.cu", "chase.cu", "api.cu", "peak.cu", "noalloc.cu", "batched.cu", "adjoint.cu", "sytrd.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "-Xcompiler", "-Wall", "-Xcompiler", "-Wextra", "-Xcompiler", "-Wno-unused-parameter",
              "-Xptxas", "-warn-spills", "--expt-relaxed-constexpr",
              "-I", str(ROOT / "include"), "-I", str(CSRC)]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(exe).exists():
        raise RuntimeError("nvcc not found: libsymeig.so cannot be built")
    return exe


def _stale() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    deps = [CSRC / s for s in SOURCES] + list(CSRC.glob("*.cuh")) + [ROOT / "include" / "symeig.h"]
    return any(p.stat().st_mtime > t for p in deps if p.exists())


def build(force: bool = False, verbose: bool = False, extra_flags: list[str] | None = None) -> Path:
    if not force and not _stale():
        return LIB
    OUT.mkdir(exist_ok=True)
    exe = nvcc()
    flags = NVCC_FLAGS + (extra_flags or [])

    def compile_one(src: str):
        obj = OUT / (Path(src).stem + ".o")
        cmd = [exe, *ARCH, *flags, "-c", str(CSRC / src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        return src, obj, r

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(compile_one, SOURCES))
    for src, _, r in results:
        if verbose or r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}")
    tmp = OUT / "libsymeig.so.tmp"
    cmd = [exe, *ARCH, "-shared", "-o", str(tmp), *[str(o) for _, o, _ in results]]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError("nvcc link of libsymeig.so failed")
    os.replace(tmp, LIB)
    return LIB


# The checked build: the translation units that hold the wave tile (the single-matrix and the
# batched apply) recompiled with -DSYMEIG_DEVICE_CHECKS, linked with the default build's other
# objects into _build/libsymeig_checked.so.  A debugging aid: every global access of a wave
# tile is checked against its pass's extent and a failed check is reported as SYMEIG_ERR_DEVICE.
CHECKED_SOURCES = ["apply.cu", "batched.cu"]
CHECKED_LIB = OUT / "libsymeig_checked.so"


def build_checked(force: bool = False, verbose: bool = False) -> Path:
    build()
    if not force and CHECKED_LIB.exists() and CHECKED_LIB.stat().st_mtime >= LIB.stat().st_mtime:
        return CHECKED_LIB
    exe = nvcc()
    cdir = OUT / "checked"
    cdir.mkdir(exist_ok=True)
    flags = NVCC_FLAGS + ["-DSYMEIG_DEVICE_CHECKS"]

    def compile_one(src: str):
        obj = cdir / (Path(src).stem + ".o")
        r = subprocess.run([exe, *ARCH, *flags, "-c", str(CSRC / src), "-o", str(obj)], capture_output=True, text=True)
        return src, obj, r

    with ThreadPoolExecutor(max_workers=len(CHECKED_SOURCES)) as ex:
        results = list(ex.map(compile_one, CHECKED_SOURCES))
    for src, _, r in results:
        if verbose or r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src} (checked build)")
    objs = [str(o) for _, o, _ in results] + [str(OUT / (Path(s).stem + ".o")) for s in SOURCES if s not in CHECKED_SOURCES]
    tmp = OUT / "libsymeig_checked.so.tmp"
    r = subprocess.run([exe, *ARCH, "-shared", "-o", str(tmp), *objs], capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError("nvcc link of libsymeig_checked.so failed")
    os.replace(tmp, CHECKED_LIB)
    return CHECKED_LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
