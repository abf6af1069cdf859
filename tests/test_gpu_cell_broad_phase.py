"""The warp-per-cell sphere broad phase (dem_set_sphere_cell_broad_phase(1):
staged 27-cell neighbourhoods, ballot-compacted candidates, drivers per
particle) builds the same interaction lists as the thread-per-owner kernels,
bit for bit, through rebuilds: periodic ghosts kept from both owners, the
smallest periodic grid, neighbourhoods too large to stage (the per-owner walk),
drivers, mesh items, batched systems whose own trigger did not fire, and the
captured graph step; and it matches the oracle."""
import numpy as np
import pytest

from exadem_gb300 import workloads as W
from tests.helpers import assert_same_list, assert_state, bit_equal_fraction, pair

pytestmark = pytest.mark.gpu

FAST = dict(fused_step=1, fp32_contact_screen=1, fp32_broad_phase=1)


def _both(make, steps, chunks=4):
    """(thread-per-owner system, warp-per-cell system) after first_iteration and `steps` steps."""
    a, b = make().build(), make().build()
    b.set_sphere_cell_broad_phase(1)
    for s in (a, b):
        s.first_iteration()
    assert_same_list(a.interactions(), b.interactions())
    for _ in range(chunks):
        for s in (a, b):
            s.step(steps // chunks)
        assert_same_list(a.interactions(), b.interactions())
    assert a.rebuild_count() == b.rebuild_count()
    assert bit_equal_fraction(a.particles(), b.particles()) == 1.0
    return a, b


def test_periodic_floor_against_oracle(native_lib):
    w = W.spheres_floor(n=6000, side=24.0, phi=0.3, fp32_broad_phase=1)
    g, o = pair(w)
    g.set_sphere_cell_broad_phase(1)
    g.first_iteration()
    o.first_iteration()
    assert_same_list(g.interactions(), o.interactions())
    g.step(60)
    o.step(60)
    assert g.rebuild_count() == o.rebuild_count()
    assert_same_list(g.interactions(), o.interactions())
    assert_state(g.particles(), o.particles(), 1e-9)


def test_periodic_floor_fused(native_lib):
    a, _ = _both(lambda: W.spheres_floor(n=8000, side=26.0, **FAST), 400)
    assert a.rebuild_count() > 1


def test_three_cell_periodic_grid(native_lib):
    """The smallest periodic grid (three cells a side): every stencil wraps."""
    a, _ = _both(lambda: W.spheres_floor(n=60, side=3.8, phi=0.3, seed=4, **FAST), 200)
    assert a.interaction_count() > 0


def test_unstaged_neighbourhoods(native_lib):
    """One sphere of radius 1 sets the cell size; the small spheres (radius 0.1)
    put hundreds in a neighbourhood, beyond the staging capacity: the per-owner
    walk of the same kernel."""
    def make():
        w = W.spheres_floor(n=6000, side=14.0, rmin=0.1, rmax=0.12, phi=0.3, seed=8, **FAST)
        p = w.particles
        p["radius"][0] = 1.0
        p["rz"][0] = float(p["rz"].max()) + 3.0
        return w

    a, _ = _both(make, 200)
    assert a.interaction_count() > 0


def test_drum_drivers(native_lib):
    _both(lambda: W.spheres_drum(n=4000, seed=3, **FAST), 400)


def test_mesh_items(native_lib):
    _both(lambda: W.spheres_mesh_terrain(n=3000, **FAST), 300)


def test_batched_drums(native_lib):
    def run(on):
        b = W.drums_batch(nsys=5, nmin=400, nmax=2500, seed=9, **FAST)
        rng = np.random.default_rng(9)
        for m in b.members:
            m.particles["vy"] = rng.uniform(-2.0, 2.0, m.n)
        s = b.build()
        s.set_sphere_cell_broad_phase(on)
        s.first_iteration()
        s.step(600)
        return s

    a, b = run(0), run(1)
    assert a.rebuild_count() == b.rebuild_count() and a.rebuild_count() > 0
    assert_same_list(a.interactions(), b.interactions())
    assert bit_equal_fraction(a.particles(), b.particles()) == 1.0


def test_graph_step(native_lib):
    a = W.spheres_floor(n=8000, side=26.0, **FAST).build()
    b = W.spheres_floor(n=8000, side=26.0, graph_step=1, **FAST).build()
    b.set_sphere_cell_broad_phase(1)
    for s in (a, b):
        s.first_iteration()
        for _ in range(4):
            s.step(150)
    assert a.rebuild_count() == b.rebuild_count() and a.rebuild_count() > 1
    assert_same_list(a.interactions(), b.interactions())
    assert bit_equal_fraction(a.particles(), b.particles()) == 1.0
