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


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
