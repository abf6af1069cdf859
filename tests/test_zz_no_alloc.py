"""GPU test of dem_simulation_state_noalloc, the state reduction for callers
that may not allocate device memory (their memory belongs to another
allocator, or they must not trigger cudaMalloc's implicit synchronisation).

It is called through the C ABI on particle arrays the test already holds on
the device, twice in a row on different data (the shared scratch array keeps
the previous call's contents), and compared with dem_simulation_state of a
context holding the same particles, within the energy tolerance of the parity
tests.  This file sorts last so that a run stopping at the first failure has
already run every other test."""
import ctypes as C

import numpy as np
import pytest

from tests.helpers import ENERGY_RTOL, assert_close_rel

pytestmark = pytest.mark.gpu

FIELDS = ["vx", "vy", "vz", "vrotx", "vroty", "vrotz", "mass"]


def _noalloc_state(lib, particles, torch):
    n = len(particles["mass"])
    dev = {k: torch.from_numpy(np.ascontiguousarray(particles[k])).cuda() for k in FIELDS}
    out = torch.full((7,), float("nan"), dtype=torch.float64, device="cuda")
    from exadem_gb300 import _abi as A

    st = A.Particles()
    st.n = n
    for k in FIELDS:
        setattr(st, k, C.cast(C.c_void_p(dev[k].data_ptr()), A.PD))
    torch.cuda.synchronize()
    rc = lib.dem_simulation_state_noalloc(C.byref(st), C.cast(C.c_void_p(out.data_ptr()), A.PD), None)
    assert rc == 0, rc
    torch.cuda.synchronize()
    o = out.cpu().numpy()
    return {"kinetic_energy": o[0:3], "rotation_energy": o[3:6], "mass": o[6]}


def test_state_noalloc_matches_context_reduction(native_lib):
    torch = pytest.importorskip("torch")
    from exadem_gb300 import workloads as W

    w = W.spheres_box(n=6000, box=25.0, seed=21)
    s = w.build()
    s.first_iteration()
    for steps in (20, 15):  # two calls in a row, on different particle states
        s.step(steps)
        ref = s.simulation_state()
        got = _noalloc_state(native_lib, s.particles(sort_by_id=False), torch)
        assert_close_rel(got["kinetic_energy"], ref["kinetic_energy"], ENERGY_RTOL, "kinetic_energy")
        assert_close_rel(got["rotation_energy"], ref["rotation_energy"], ENERGY_RTOL, "rotation_energy")
        assert_close_rel(np.array([got["mass"]]), np.array([ref["mass"]]), ENERGY_RTOL, "mass")


def test_state_noalloc_rejects_oversize(native_lib):
    from exadem_gb300 import _abi as A

    st = A.Particles()
    st.n = 16777216 + 1
    dummy = (C.c_double * 8)()
    for k in FIELDS:
        setattr(st, k, C.cast(dummy, A.PD))
    assert native_lib.dem_simulation_state_noalloc(C.byref(st), C.cast(dummy, A.PD), None) == 1  # INVALID_ARG
