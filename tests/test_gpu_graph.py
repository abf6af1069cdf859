"""The fused step replayed as one CUDA graph (graph_step): same bits as the
fused step launched from the host, through rebuilds, batched systems and an
interaction-buffer overflow (rolled back and run again with more capacity)."""
import pytest

from exadem_gb300 import workloads as W
from tests.helpers import assert_same_list, bit_equal_fraction

pytestmark = pytest.mark.gpu

FUSED = dict(fused_step=1, fp32_contact_screen=1, fp32_broad_phase=1)


def _run(w, steps, capacity=None):
    s = w.build()
    s.first_iteration()
    if capacity is not None:
        s.set_graph_capacity(capacity)
    for _ in range(4):
        s.step(steps // 4)
    return s


def test_graph_step_equals_host_step_spheres(native_lib):
    a = _run(W.spheres_floor(n=8000, side=26.0, **FUSED), 600)
    b = _run(W.spheres_floor(n=8000, side=26.0, graph_step=1, **FUSED), 600)
    assert a.rebuild_count() == b.rebuild_count() and a.rebuild_count() > 1
    assert_same_list(a.interactions(), b.interactions())
    assert bit_equal_fraction(a.particles(), b.particles()) == 1.0
    assert a.simulation_state()["n_interactions"] == b.simulation_state()["n_interactions"]


def test_graph_step_overflow_rolls_back(native_lib):
    # the capacity starts at the first list's size + 1: the first rebuild that
    # finds one more pair overflows
    a = _run(W.spheres_drum(n=4000, seed=3, **FUSED), 600)
    b = _run(W.spheres_drum(n=4000, seed=3, graph_step=1, **FUSED), 600, capacity=64)
    assert a.rebuild_count() == b.rebuild_count() and a.rebuild_count() > 1
    assert b.interaction_count() > a.simulation_state()["n_particles"] // 4
    assert_same_list(a.interactions(), b.interactions())
    assert bit_equal_fraction(a.particles(), b.particles()) == 1.0


def test_graph_step_batched_drums(native_lib):
    a = W.drums_batch(nsys=6, nmin=300, nmax=3000, seed=12, **FUSED).build()
    b = W.drums_batch(nsys=6, nmin=300, nmax=3000, seed=12, graph_step=1, **FUSED).build()
    for s in (a, b):
        s.first_iteration()
        s.step(500)
    assert_same_list(a.interactions(), b.interactions())
    assert bit_equal_fraction(a.particles(), b.particles()) == 1.0
    assert a.rebuild_count() == b.rebuild_count() and a.rebuild_count() > 1
