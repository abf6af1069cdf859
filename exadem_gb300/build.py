"""In-tree build of the native library ``libexadem_gb300.so`` (sm_103a only).

Every ``csrc/*.cu`` translation unit is compiled by nvcc in parallel, the host
``csrc/*.cpp`` units by g++, and all are linked into one shared library next
to this file.  The seeded input generator (``gen/``) is a separate host
library, ``libdem_workloads.so``.  FP64 contraction is disabled (``--fmad=false``) so the contact
law keeps the reference's operation order bit for bit.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libexadem_gb300.so"
GEN = PKG / "gen"
WORKLOADS_LIB = PKG / "libdem_workloads.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr"]
CXX_FLAGS = ["-O2", "-fPIC", "-std=c++17", "-ffp-contract=off"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build exadem_gb300")


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False, extra_nvcc: list[str] | None = None) -> Path:
    """Compile (if stale) and return the path of the shared library."""
    nvcc = _nvcc()
    BUILD.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + list((PKG.parent / "include").glob("*.h"))
    jobs = []
    objs = []
    for src in sources():
        obj = BUILD / (src.stem + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            if src.suffix == ".cu":
                cmd = [nvcc, *ARCH, *NVCC_FLAGS, *(extra_nvcc or []), "-c", str(src), "-o", str(obj)]
            else:
                cmd = ["g++", *CXX_FLAGS, "-c", str(src), "-o", str(obj)]
            jobs.append(cmd)
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for cmd, fut in [(c, ex.submit(_run, c)) for c in jobs]:
                if verbose:
                    print(" ".join(cmd), file=sys.stderr)
                fut.result()
    if force or jobs or _stale(LIB, objs):
        _run([nvcc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs)])
    build_workloads(force)
    return LIB


def build_workloads(force: bool = False) -> Path:
    """The seeded input generator (gen/*.cpp, include/dem_workloads.h) as a host library of its own."""
    srcs = sorted(GEN.glob("*.cpp"))
    deps = srcs + list((PKG.parent / "include").glob("*.h"))
    if force or _stale(WORKLOADS_LIB, deps):
        _run(["g++", *CXX_FLAGS, "-shared", "-o", str(WORKLOADS_LIB), *map(str, srcs)])
    return WORKLOADS_LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
