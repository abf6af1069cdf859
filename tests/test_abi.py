"""CPU tests of the boundary: the library builds, loads and exports every
symbol declared in include/*.h (no compute call, no GPU needed)."""
import ctypes
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def declared_functions(headers=None):
    names = set()
    for h in (headers or (ROOT / "include").glob("*.h")):
        txt = h.read_text()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        for m in re.finditer(r"^\s*(?:int|const char\s*\*)\s+(dem_\w+)\s*\(", txt, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_headers_declare_functions():
    names = declared_functions()
    assert "dem_ctx_create" in names and "dem_step" in names and len(names) >= 20


PRODUCT_HEADERS = [ROOT / "include" / h for h in ("dem_hotpath.h", "dem_selftest.h", "dem_learned.h")]
WORKLOAD_HEADERS = [ROOT / "include" / "dem_workloads.h"]


def test_headers_are_all_accounted_for():
    assert set((ROOT / "include").glob("*.h")) == set(PRODUCT_HEADERS) | set(WORKLOAD_HEADERS)


def test_python_binding_declares_every_symbol():
    from exadem_gb300 import _abi as A

    assert set(A.EXPORTED) == set(declared_functions(PRODUCT_HEADERS))
    assert set(A.WORKLOADS_EXPORTED) == set(declared_functions(WORKLOAD_HEADERS))


def test_library_exports_every_declared_symbol(native_lib):
    lib = ctypes.CDLL(str(ROOT / "exadem_gb300" / "libexadem_gb300.so"))
    missing = [n for n in declared_functions(PRODUCT_HEADERS) if not hasattr(lib, n)]
    assert not missing, missing


def test_generator_library_is_separate(native_lib):
    """The seeded input generator is its own host library: the product library
    does not carry it, so a process that only generates inputs (the CPU
    reference leg of the benchmark) never maps the product library."""
    gen = ctypes.CDLL(str(ROOT / "exadem_gb300" / "libdem_workloads.so"))
    assert all(hasattr(gen, n) for n in declared_functions(WORKLOAD_HEADERS))
    lib = ctypes.CDLL(str(ROOT / "exadem_gb300" / "libexadem_gb300.so"))
    assert not hasattr(lib, "dem_generate_rsa_spheres")


def test_create_without_gpu_fails_cleanly(native_lib):
    import torch

    if torch.cuda.is_available():
        return
    from exadem_gb300 import System, make_params, DemError

    try:
        System(make_params((0, 0, 0), (1, 1, 1)))
    except DemError as e:
        assert e.code == 8  # DEM_ERR_NO_DEVICE: no silent CPU fallback
    else:
        raise AssertionError("context creation without a GPU must fail")


def test_params_validation_messages(native_lib):
    from exadem_gb300 import _abi as A

    assert A.ERRORS[4] == "DEM_ERR_UNSUPPORTED"
