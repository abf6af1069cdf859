"""GPU parity at the benchmarked sizes (GPU, against the oracle).

The benchmark times 2,000,000 cohesive spheres on a floor (config 2) and
200,000 polyhedra (config 3).  These tests run the same workloads, on the same
fused / FP32-screened / graph-replayed path as the benchmark, at full size:

- from the seeded initial state: the interaction list bit-exact after
  first_iteration and after a forced rebuild, forces and torques within 1e-12
  relative after the first force pass, the whole particle state within 1e-12
  after one step, kinetic and rotation energy and the packing-fraction profile
  within 1e-9 after 100 steps (and the list again);
- from the state the benchmark times: the GPU runs the benchmark's pre-roll,
  the particle state it reaches is loaded into a fresh GPU context and into the
  oracle, and both continue with the same checks.
"""
import copy

import numpy as np
import pytest

from exadem_gb300 import workloads as W
from tests.helpers import (ENERGY_RTOL, FORCE_RTOL, assert_close_rel, assert_forces, assert_same_list, assert_state)

pytestmark = pytest.mark.gpu

FAST = dict(fp32_contact_screen=1, fused_step=1, fp32_broad_phase=1)
SPHERE_PREROLL = 3000   # the benchmark's pre-roll for the spheres (bench.PREROLL)
POLY_PREROLL = 2000     # config 3's run length


def _from_state(w, state):
    """The workload with its particles replaced by a host state (ids, shapes and drivers kept)."""
    w2 = copy.copy(w)
    w2.particles = {k: np.ascontiguousarray(state[k]) for k in w.particles}
    return w2


def _check_window(g, o, zhi, steps=100):
    """first_iteration, a step, a forced rebuild, then `steps` steps, on both."""
    from oracle.oracle import oracle_system  # noqa: F401  (the oracle is the checker)

    g.first_iteration()
    o.first_iteration()
    assert_same_list(g.interactions(), o.interactions())
    assert_forces(g.particles(), o.particles(), FORCE_RTOL)
    g.step(1)
    o.step(1)
    assert_state(g.particles(), o.particles(), FORCE_RTOL)
    g.update_particle_neighbors()
    o.update_particle_neighbors()
    assert_same_list(g.interactions(), o.interactions())
    r0g, r0o = g.rebuild_count(), o.rebuild_count()
    g.step(steps)
    o.step(steps)
    assert g.rebuild_count() - r0g == o.rebuild_count() - r0o
    sg, so = g.simulation_state(), o.simulation_state()
    assert_close_rel(sg["kinetic_energy"], so["kinetic_energy"], ENERGY_RTOL, "kinetic_energy")
    assert_close_rel(sg["rotation_energy"], so["rotation_energy"], ENERGY_RTOL, "rotation_energy")
    assert_close_rel(g.packing_profile(50, 0.0, zhi), o.packing_profile(50, 0.0, zhi), ENERGY_RTOL, "profile")
    lg, lo = g.interactions(), o.interactions()
    assert_same_list(lg, lo)
    np.testing.assert_allclose(lg["friction"], lo["friction"], rtol=1e-9, atol=1e-14)
    return sg


def test_spheres_2m_initial_state(native_lib):
    from oracle.oracle import oracle_system

    w = W.spheres_floor(graph_step=1, **FAST)
    assert w.n == 2_000_000
    g, o = w.build(), w.build(oracle_system)
    _check_window(g, o, float(w.info["height"]) + 1.0)
    g.close()
    o.close()


def test_spheres_2m_benchmarked_state(native_lib):
    """The pre-rolled bed the benchmark times: a rebuild every few steps, about
    four listed pairs per sphere."""
    from oracle.oracle import oracle_system

    w = W.spheres_floor(graph_step=1, **FAST)
    s = w.build()
    s.first_iteration()
    s.step(SPHERE_PREROLL)
    state = s.particles(sort_by_id=True)
    s.close()
    w2 = _from_state(w, state)
    g, o = w2.build(), w2.build(oracle_system)
    r0 = g.rebuild_count()
    sg = _check_window(g, o, float(np.max(state["rz"])) + 1.0)
    assert g.rebuild_count() - r0 >= 3, "the benchmarked window triggers rebuilds"
    assert sg["n_interactions"] > 2 * w.n
    g.close()
    o.close()


def test_polyhedra_200k_initial_state(native_lib):
    from oracle.oracle import oracle_system

    w = W.polyhedra_floor(**FAST)
    assert w.n == 200_000
    g, o = w.build(), w.build(oracle_system)
    _check_window(g, o, float(w.info["height"]) + 4.0)
    g.close()
    o.close()


def test_polyhedra_200k_after_config_run(native_lib):
    """The state config 3's 2000-step run ends in, continued on both sides."""
    from oracle.oracle import oracle_system

    w = W.polyhedra_floor(**FAST)
    s = w.build()
    s.first_iteration()
    s.step(POLY_PREROLL)
    state = s.particles(sort_by_id=True)
    s.close()
    w2 = _from_state(w, state)
    g, o = w2.build(), w2.build(oracle_system)
    _check_window(g, o, float(np.max(state["rz"])) + 4.0)
    g.close()
    o.close()
