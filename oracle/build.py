"""Build recipe of the CPU oracle (test infrastructure only).

Produces ``oracle/libdem_oracle.so`` from ``oracle/dem_oracle.cpp`` with g++,
OpenMP and no FP contraction (``-ffp-contract=off``; GCC contracts to FMA by
default on aarch64), so its arithmetic is plain IEEE double in source order.
exaDEM's own hot-path headers are compiled separately, against stand-ins for
its missing dependencies, by ``oracle/ref_build.py`` (``oracle/_ref``); the tests
compare the two libraries function by function.
"""
from __future__ import annotations

import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIB = HERE / "libdem_oracle.so"
SRC = HERE / "dem_oracle.cpp"


def build(force: bool = False) -> Path:
    deps = [SRC, HERE.parent / "include" / "dem_hotpath.h"]
    if force or not LIB.exists() or any(d.stat().st_mtime > LIB.stat().st_mtime for d in deps):
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
               "-o", str(LIB), str(SRC)]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"oracle build failed:\n{res.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(force=True))
