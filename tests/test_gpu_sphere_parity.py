"""GPU parity of the sphere hot path against the CPU oracle (seeded inputs).

Contract: interaction list bit-exact after every rebuild; forces and torques
within 1e-12 relative after one force pass; kinetic energy and packing-fraction
profile within 1e-9 relative after 100 steps.  The GPU keeps the oracle's FP64
operation order, so most values are expected to be bit-identical.
"""
import numpy as np
import pytest

from exadem_gb300 import workloads as W
from tests.helpers import (ENERGY_RTOL, assert_close_rel, assert_forces, assert_same_list, assert_state,
                           bit_equal_fraction, pair)

pytestmark = pytest.mark.gpu


def _first(w):
    g, o = pair(w)
    g.first_iteration()
    o.first_iteration()
    return g, o


def test_box_first_iteration_list_and_forces(native_lib):
    w = W.spheres_box(n=3000, box=20.0, seed=11)
    g, o = _first(w)
    assert_same_list(g.interactions(), o.interactions())
    pg, po = g.particles(), o.particles()
    assert_forces(pg, po)
    assert bit_equal_fraction(pg, po, ["fx", "fy", "fz", "momx", "momy", "momz"]) == 1.0


def test_box_one_step(native_lib):
    w = W.spheres_box(n=3000, box=20.0, seed=12)
    g, o = _first(w)
    g.step(1)
    o.step(1)
    assert_state(g.particles(), o.particles(), 1e-12)
    assert_same_list(g.interactions(), o.interactions())


@pytest.mark.parametrize("seed", [1, 2])
def test_config1_100_steps(native_lib, seed):
    """Config 1 at full size (10,000 spheres, 30^3 walled box), 100 steps."""
    w = W.spheres_box(seed=seed)
    g, o = _first(w)
    g.step(100)
    o.step(100)
    sg, so = g.simulation_state(), o.simulation_state()
    assert_close_rel(sg["kinetic_energy"], so["kinetic_energy"], ENERGY_RTOL, "kinetic_energy")
    assert_close_rel(sg["rotation_energy"], so["rotation_energy"], ENERGY_RTOL, "rotation_energy")
    assert g.rebuild_count() == o.rebuild_count()
    assert_same_list(g.interactions(), o.interactions())
    zlo, zhi = 0.0, 30.0
    assert_close_rel(g.packing_profile(50, zlo, zhi), o.packing_profile(50, zlo, zhi), ENERGY_RTOL, "profile")
    assert_state(g.particles(), o.particles(), 1e-9)


def test_periodic_cohesive_floor(native_lib):
    """Config 2 physics on a small periodic patch: ghost pairs kept from both owners."""
    w = W.spheres_floor(n=6000, side=24.0, phi=0.3)
    g, o = _first(w)
    lg = g.interactions()
    assert_same_list(lg, o.interactions())
    assert_forces(g.particles(), o.particles())
    g.step(60)
    o.step(60)
    assert_same_list(g.interactions(), o.interactions())
    assert_state(g.particles(), o.particles(), 1e-9)
    np.testing.assert_allclose(g.interactions()["friction"], o.interactions()["friction"], rtol=1e-9, atol=1e-14)


def test_drum(native_lib):
    w = W.spheres_drum(n=4000)
    g, o = _first(w)
    assert_same_list(g.interactions(), o.interactions())
    g.step(80)
    o.step(80)
    assert_same_list(g.interactions(), o.interactions())
    assert_state(g.particles(), o.particles(), 1e-9)


def test_fp32_screen_is_exact(native_lib):
    """The FP32 separation screen must not change a single bit."""
    w = W.spheres_floor(n=6000, side=24.0, phi=0.3)
    w2 = W.spheres_floor(n=6000, side=24.0, phi=0.3, fp32_contact_screen=1)
    a, b = w.build(), w2.build()
    for s in (a, b):
        s.first_iteration()
        s.step(40)
    pa, pb = a.particles(), b.particles()
    assert bit_equal_fraction(pa, pb) == 1.0


def test_empty_and_single(native_lib):
    from exadem_gb300 import System, make_params

    p = make_params((0, 0, 0), (10, 10, 10))
    s = System(p)
    s.set_particles({"rx": np.zeros(0), "ry": np.zeros(0), "rz": np.zeros(0), "radius": np.zeros(0)})
    s.first_iteration()
    s.step(3)
    assert s.interaction_count() == 0
    s.set_particles({"rx": np.array([5.0]), "ry": np.array([5.0]), "rz": np.array([5.0]),
                     "radius": np.array([0.5]), "mass": np.array([2.0])})
    s.first_iteration()
    s.step(2)
    st = s.simulation_state()
    assert st["n_particles"] == 1 and s.interaction_count() == 0


def test_particles_outside_domain(native_lib):
    """Non-periodic particles outside the bounds are clamped into border cells, list unchanged."""
    w = W.spheres_box(n=1500, box=20.0, seed=5)
    w.particles["rz"][:50] += 25.0  # above the box
    g, o = _first(w)
    assert_same_list(g.interactions(), o.interactions())
    assert_forces(g.particles(), o.particles())


def test_exact_division_selftest(native_lib):
    """Reciprocal-based division (Markstein's step) equals a / b bit for bit."""
    import ctypes as C

    bad, fast = C.c_uint64(), C.c_uint64()
    assert native_lib.dem_selftest_division(40_000_000, 12345, C.byref(bad), C.byref(fast)) == 0
    assert fast.value > 25_000_000
    assert bad.value == 0


@pytest.mark.parametrize("flags", [dict(fused_step=1), dict(fused_step=1, fp32_contact_screen=1)])
def test_fused_step_bit_exact_with_plain(native_lib, flags):
    w1 = W.spheres_floor(n=6000, side=24.0, phi=0.3)
    w2 = W.spheres_floor(n=6000, side=24.0, phi=0.3, **flags)
    a, b = w1.build(), w2.build()
    for s in (a, b):
        s.first_iteration()
        s.step(80)
    pa, pb = a.particles(), b.particles()
    assert bit_equal_fraction(pa, pb) == 1.0
    la, lb = a.interactions(), b.interactions()
    assert_same_list(la, lb)
    np.testing.assert_array_equal(la["friction"], lb["friction"])
    np.testing.assert_array_equal(la["moment"], lb["moment"])
    assert a.simulation_state()["n_active_interactions"] == b.simulation_state()["n_active_interactions"]


@pytest.mark.parametrize("make", [lambda: W.spheres_box(n=4000, box=22.0, seed=9, fused_step=1, fp32_contact_screen=1),
                                  lambda: W.spheres_drum(n=4000, fused_step=1, fp32_contact_screen=1)])
def test_fused_step_matches_oracle(native_lib, make):
    w = make()
    g, o = pair(w)
    for s in (g, o):
        s.first_iteration()
        s.step(100)
    assert g.rebuild_count() == o.rebuild_count()
    assert_same_list(g.interactions(), o.interactions())
    assert_state(g.particles(), o.particles(), 1e-12)


@pytest.mark.parametrize("make", [
    lambda **f: W.spheres_floor(n=8000, side=26.0, phi=0.3, **f),
    lambda **f: W.spheres_box(n=3000, box=20.0, seed=4, **f),
    lambda **f: W.spheres_drum(n=3000, **f)])
def test_fp32_broad_phase_same_list(native_lib, make):
    """The FP32 cell-relative broad phase keeps exactly the FP64 candidate set, rebuild after rebuild."""
    a = make().build()
    b = make(fp32_broad_phase=1, fused_step=1, fp32_contact_screen=1).build()
    for s in (a, b):
        s.first_iteration()
    assert_same_list(a.interactions(), b.interactions())
    for _ in range(4):
        for s in (a, b):
            s.step(25)
            s.update_particle_neighbors()  # force a rebuild
        assert_same_list(a.interactions(), b.interactions())
    assert bit_equal_fraction(a.particles(), b.particles()) == 1.0
