"""Build recipe of ``oracle/_ref/libexadem_ref.so`` (test infrastructure only).

Compiles ``oracle/ref_harness.cpp``, which includes exaDEM's own headers from
the exaDEM source tree where they lie (never copied), against the stand-in
headers of ``oracle/ref_shim/`` (onika, exaNBody, MPI, yaml-cpp and tinyexpr
are not available).  Flags match the oracle's: ``-O2 -ffp-contract=off``, no
fast-math, so both sides compute plain IEEE double arithmetic in source order.

The library checks the oracle (``tests/test_oracle_vs_ref.py``) and generates
the committed golden vectors (``tests/golden/make_ref_vectors.py``).  It is
built only where the exaDEM sources are present; elsewhere ``build()`` returns
None and those tests use the committed vectors.
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
LIB = OUT / "libexadem_ref.so"
SRC = HERE / "ref_harness.cpp"
SHIM = HERE / "ref_shim"
# exaDEM source tree (read only); EXADEM_SRC overrides the default location.
EXADEM = Path(os.environ.get("EXADEM_SRC", "/root/reference"))
INCLUDE_DIRS = [
    "include",
    "src/shape/include",
    "src/forcefield/include",
    "src/numericalscheme/include",
    "src/interaction/include",
    "src/driver/include",
]


def available() -> bool:
    return (EXADEM / "src/forcefield/include/exaDEM/forcefield/contact_force.hpp").exists()


def build(force: bool = False) -> Path | None:
    if not available():
        return None
    OUT.mkdir(exist_ok=True)
    deps = [SRC, *SHIM.rglob("*.h"), *SHIM.rglob("*.hpp")]
    if force or not LIB.exists() or any(d.stat().st_mtime > LIB.stat().st_mtime for d in deps):
        # the stand-ins come first so they shadow exaDEM's yaml-bound contact_parameters.hpp
        cmd = ["g++", "-O2", "-std=c++20", "-fPIC", "-shared", "-ffp-contract=off", "-w", "-I", str(SHIM)]
        for d in INCLUDE_DIRS:
            cmd += ["-I", str(EXADEM / d)]
        cmd += ["-o", str(LIB), str(SRC)]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"reference harness build failed:\n{res.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(force=True))
