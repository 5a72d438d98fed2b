"""Build the engine library ``librusterize_gb300.so`` for sm_103a.

Every translation unit is compiled by ``nvcc`` in parallel, then linked into
one shared library with a plain C ABI (``include/rusterize_gb300.h``).  The
library lands in ``rusterize_gb300/_lib/`` (in-tree, git-ignored).

Usage: ``python -m rusterize_gb300._build [--force]``.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT_DIR = PKG / "_lib"
OBJ_DIR = OUT_DIR / "obj"
LIB_NAME = "librusterize_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-pthread",
              "-Xcompiler", "-ffp-contract=off",
              "--expt-relaxed-constexpr", "-I", str(ROOT / "include")]


def lib_path() -> Path:
    return OUT_DIR / LIB_NAME


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the GB300 engine must be compiled with the CUDA toolkit")
    return cand


def _sources() -> list[Path]:
    srcs = sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))
    return srcs


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def needs_build() -> bool:
    """True when the library is missing, or older than its sources and a
    CUDA toolkit is available to rebuild it."""
    lib = lib_path()
    if not lib.exists():
        return True
    deps = _sources() + list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + [ROOT / "include" / "rusterize_gb300.h"]
    if not _stale(lib, deps):
        return False
    return bool(shutil.which("nvcc") or Path("/usr/local/cuda/bin/nvcc").exists())


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile (if needed) and return the path of the shared library."""
    nvcc = _nvcc()
    OBJ_DIR.mkdir(parents=True, exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + [ROOT / "include" / "rusterize_gb300.h"]
    srcs = _sources()
    jobs = []
    for src in srcs:
        obj = OBJ_DIR / (src.name + ".o")
        if force or _stale(obj, [src, *headers]):
            cmd = [nvcc, *ARCH, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)]
            if src.suffix == ".cpp":
                cmd = [nvcc, *NVCC_FLAGS, "-x", "c++", "-c", str(src), "-o", str(obj)]
            jobs.append((src, obj, cmd))
    if jobs:
        workers = max(1, min(len(jobs), os.cpu_count() or 4))
        with cf.ThreadPoolExecutor(max_workers=workers) as ex:
            futs = {ex.submit(subprocess.run, cmd, capture_output=True, text=True): (src, obj) for src, obj, cmd in jobs}
            errors = []
            for fut in cf.as_completed(futs):
                src, obj = futs[fut]
                res = fut.result()
                if verbose and (res.stdout or res.stderr):
                    print(res.stdout + res.stderr, file=sys.stderr)
                if res.returncode != 0:
                    errors.append(f"--- {src.name}\n{res.stdout}{res.stderr}")
            if errors:
                raise RuntimeError("nvcc failed:\n" + "\n".join(errors))
    objs = [OBJ_DIR / (s.name + ".o") for s in srcs]
    lib = lib_path()
    if force or jobs or _stale(lib, objs):
        cmd = [nvcc, *ARCH, "-shared", "-o", str(lib), *map(str, objs), "-lcudart", "-Xlinker", "-lpthread"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError("link failed:\n" + res.stdout + res.stderr)
    return lib


if __name__ == "__main__":
    p = build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(p)
