"""Build recipe for the in-tree shared libraries.

  namics_gb300/lib/libnamics_gb300.so   the product: CUDA kernels for sm_103a
                                        plus the C++ host layer, C ABI in
                                        include/namics_gb300.h
  oracle/liborc.so                      the CPU oracle (test infrastructure)
  oracle/_ref/namics                    the unmodified reference program,
                                        built only where its sources exist

Each translation unit compiles in its own process (in parallel); there is one
-gencode target, so a full build takes well under a minute.
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
LIBDIR = PKG / "lib"
OBJDIR = PKG / "lib" / "obj"
ORACLE = ROOT / "oracle"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
              "--expt-relaxed-constexpr"]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-Wall", "-Wno-unused-function"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _cuda_home() -> Path:
    return Path(_nvcc()).resolve().parent.parent


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_product(verbose: bool = False) -> Path:
    OBJDIR.mkdir(parents=True, exist_ok=True)
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [ROOT / "include" / "namics_gb300.h"]
    jobs = []
    objs = []
    nvcc = _nvcc()
    for src in sorted(CSRC.glob("*.cu")):
        obj = OBJDIR / (src.stem + ".cu.o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            jobs.append([nvcc, *ARCH, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)])
    for src in sorted(CSRC.glob("*.cpp")):
        obj = OBJDIR / (src.stem + ".cpp.o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            jobs.append(["g++", *CXX_FLAGS, f"-I{_cuda_home() / 'include'}", "-c", str(src), "-o", str(obj)])
    with cf.ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        for cmd in jobs:
            if verbose:
                print(" ".join(cmd), flush=True)
        list(ex.map(_run, jobs))
    lib = LIBDIR / "libnamics_gb300.so"
    if jobs or not lib.exists():
        _run([nvcc, *ARCH, "-shared", "-o", str(lib), *map(str, objs), "-lcudart"])
    return lib


def build_oracle(verbose: bool = False) -> Path:
    src = ORACLE / "scf_oracle.c"
    lib = ORACLE / "liborc.so"
    if _stale(lib, [src, ORACLE / "scf_oracle.h", ROOT / "include" / "namics_gb300.h"]):
        # no fast-math: the oracle keeps IEEE semantics
        _run(["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-o", str(lib), str(src), "-lm"])
    return lib


def build_reference(ref: str | None = None) -> Path | None:
    """Compile the unmodified reference program into oracle/_ref, only where
    its sources are present.  The sources' location is `ref`, else the
    environment variable NAMICS_REFERENCE, else the recipe's own default
    (oracle/Makefile.ref, REF)."""
    ref = ref or os.environ.get("NAMICS_REFERENCE")
    mk = ["make", "-s", "-f", str(ORACLE / "Makefile.ref")] + ([f"REF={ref}"] if ref else [])
    if subprocess.run(mk + ["have-sources"], capture_output=True).returncode != 0:
        return None
    _run(mk + ["-j", str(os.cpu_count() or 4)])
    return ORACLE / "_ref" / "namics"


def build(verbose: bool = False) -> None:
    build_product(verbose)
    build_oracle(verbose)
    build_reference()


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
