"""The onika plugin shims (exadem_gb300/onika_plugin/) compile (CPU).

They are built inside an exaDEM build, whose onika and exaNBody are not
available here; tests/onika_mock/ stands in for onika's operator API and an
exaNBody grid, oracle/ref_shim/ for onika's math, and exaDEM's own driver
headers are read in place.  g++ -fsyntax-only then instantiates every operator
class of gb300_operators.cpp on the mock grid.
"""
import subprocess
from pathlib import Path

import pytest

from oracle import ref_build

ROOT = Path(__file__).resolve().parents[1]


@pytest.mark.skipif(not ref_build.available(), reason="exaDEM sources not present")
def test_shims_compile():
    inc = [ROOT / "tests" / "onika_mock", ROOT / "oracle" / "ref_shim", ROOT / "include"]
    inc += [ref_build.EXADEM / d for d in ref_build.INCLUDE_DIRS]
    cmd = ["g++", "-std=c++20", "-fsyntax-only", "-w"] + [f"-I{p}" for p in inc]
    cmd.append(str(ROOT / "exadem_gb300" / "onika_plugin" / "gb300_operators.cpp"))
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
