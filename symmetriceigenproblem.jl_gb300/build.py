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


def _link(exe: str, objs: list[str], lib: Path):
    tmp = lib.with_name(lib.name + ".tmp")
    r = subprocess.run([exe, *ARCH, "-shared", "-o", str(tmp), *objs], capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError(f"nvcc link of {lib.name} failed")
    os.replace(tmp, lib)


def build(force: bool = False, verbose: bool = False, extra_flags: list[str] | None = None) -> Path:
    """Build libsymeig.so and its checked variant (libsymeig_checked.so, build_checked) in one
    pool of parallel nvcc processes."""
    if not force and not _stale():
        return LIB
    OUT.mkdir(exist_ok=True)
    (OUT / "checked").mkdir(exist_ok=True)
    exe = nvcc()
    flags = NVCC_FLAGS + (extra_flags or [])
    jobs = [(src, OUT / (Path(src).stem + ".o"), flags) for src in SOURCES]
    jobs += [(src, OUT / "checked" / (Path(src).stem + ".o"), flags + ["-DSYMEIG_DEVICE_CHECKS"])
             for src in CHECKED_SOURCES]

    def compile_one(job):
        src, obj, fl = job
        r = subprocess.run([exe, *ARCH, *fl, "-c", str(CSRC / src), "-o", str(obj)], capture_output=True, text=True)
        return src, obj, r

    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        results = list(ex.map(compile_one, jobs))
    for src, _, r in results:
        if verbose or r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}")
    _link(exe, [str(OUT / (Path(s).stem + ".o")) for s in SOURCES], LIB)
    _link(exe, _checked_objects(), CHECKED_LIB)
    return LIB


# The checked build: the translation units that hold the wave tile (the single-matrix and the
# batched apply) compiled with -DSYMEIG_DEVICE_CHECKS and linked with the default build's other
# objects into _build/libsymeig_checked.so.  A debugging aid: every global access of a wave
# tile is checked against its pass's extent and a failed check is reported as SYMEIG_ERR_DEVICE.
CHECKED_SOURCES = ["apply.cu", "batched.cu"]
CHECKED_LIB = OUT / "libsymeig_checked.so"


def _checked_objects() -> list[str]:
    return ([str(OUT / "checked" / (Path(s).stem + ".o")) for s in CHECKED_SOURCES] +
            [str(OUT / (Path(s).stem + ".o")) for s in SOURCES if s not in CHECKED_SOURCES])


def build_checked(force: bool = False, verbose: bool = False) -> Path:
    """libsymeig_checked.so (built by build(); rebuilt here if it is missing or older)."""
    build(force=force, verbose=verbose)
    if CHECKED_LIB.exists() and CHECKED_LIB.stat().st_mtime >= LIB.stat().st_mtime:
        return CHECKED_LIB
    return build(force=True, verbose=verbose) and CHECKED_LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
