"""The integer-pipe binary64 multiply (exadem_gb300/csrc/emu64.cuh) returns the
IEEE product bit for bit: on the host against the host's multiply (CPU), and
on the GPU against the hardware multiply, with its throughput next to the FP64
pipe's."""
import ctypes as C
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_emu_dmul_host_bit_exact(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = tmp_path / "emu64_check"
    subprocess.run([gxx, "-O2", "-ffp-contract=off", "-I", str(ROOT / "exadem_gb300" / "csrc"),
                    str(ROOT / "tests" / "emu64_check.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe), "4000000", "11"], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout
    assert out.stdout.strip().endswith("mismatches 0")


@pytest.mark.gpu
def test_emu_dmul_gpu_bit_exact(native_lib):
    bad = C.c_uint64(0)
    assert native_lib.dem_selftest_emu_mul(200_000_000, 2024, C.byref(bad)) == 0
    assert bad.value == 0


def _probe_lib():
    """tests/probe_mul_rates.cu, a measurement probe kept out of the library, built on demand."""
    import subprocess
    from pathlib import Path

    from exadem_gb300 import build as B

    here = Path(__file__).resolve().parent
    out = here / "_build" / "libdem_probe.so"
    src = here / "probe_mul_rates.cu"
    if not out.exists() or out.stat().st_mtime < src.stat().st_mtime:
        out.parent.mkdir(exist_ok=True)
        subprocess.run([B._nvcc(), *B.ARCH, "-O3", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC", "-shared",
                        "-o", str(out), str(src)], check=True)
    lib = C.CDLL(str(out))
    lib.dem_probe_mul_rates.argtypes = [C.c_int, C.POINTER(C.c_double)]
    return lib


@pytest.mark.gpu
def test_mul_rates_probe(native_lib):
    g = (C.c_double * 5)()
    assert _probe_lib().dem_probe_mul_rates(4096, g) == 0
    print("multiply rates, G/s: fp64 %.0f  integer %.0f  both 4:4 %.0f  4:2 %.0f  2:4 %.0f" % tuple(g))
    assert all(x > 0 for x in g)


@pytest.mark.gpu
def test_rolling_clip_shortcut_bit_exact(native_lib):
    bad, fast = C.c_uint64(0), C.c_uint64(0)
    assert native_lib.dem_selftest_rolling_clip(50_000_000, 77, C.byref(bad), C.byref(fast)) == 0
    assert bad.value == 0
    assert fast.value > 1_000_000  # both the shortcut and the formula are exercised
