"""Batched systems (dem_set_systems): each system of a batch evolves exactly as
the same system alone, checked against the oracle running each drum on its
own; a batch of one equals the unbatched context."""
import numpy as np
import pytest

from exadem_gb300 import _abi as A
from exadem_gb300 import workloads as W
from tests.helpers import ENERGY_RTOL, assert_close_rel, assert_same_list, assert_state, bit_equal_fraction

pytestmark = pytest.mark.gpu


def _split_list(lst: dict, lo: int, hi: int) -> dict:
    m = (lst["owner_id"] >= lo) & (lst["owner_id"] < hi)
    return {k: v[m] for k, v in lst.items()}


def _split_particles(p: dict, lo: int, hi: int) -> dict:
    m = (p["id"] >= lo) & (p["id"] < hi)
    return {k: v[m] for k, v in p.items()}


@pytest.mark.parametrize("flags", [{}, dict(fused_step=1, fp32_contact_screen=1, fp32_broad_phase=1)])
def test_batched_drums_match_each_drum_alone(native_lib, flags):
    from oracle.oracle import oracle_system

    b = W.drums_batch(nsys=5, nmin=400, nmax=2500, seed=9, **flags)
    g = b.build()
    g.first_iteration()
    g.step(150)
    lg, pg = g.interactions(), g.particles(sort_by_id=True)
    states = g.system_states()
    assert g.rebuild_count() > 0
    first = 0
    for k, m in enumerate(b.members):
        o = m.build(oracle_system)
        o.first_iteration()
        o.step(150)
        lo, hi = first, first + m.n
        assert_same_list(_split_list(lg, lo, hi), o.interactions())
        np.testing.assert_array_equal(_split_list(lg, lo, hi)["friction"], o.interactions()["friction"])
        pk, po = _split_particles(pg, lo, hi), o.particles(sort_by_id=True)
        assert_state(pk, po, 1e-12)
        assert bit_equal_fraction(pk, po) == 1.0
        so = o.simulation_state()
        assert states[k]["n_particles"] == m.n
        assert_close_rel(states[k]["kinetic_energy"], so["kinetic_energy"], ENERGY_RTOL, "ke")
        assert_close_rel(np.array([states[k]["mass"]]), np.array([so["mass"]]), ENERGY_RTOL, "mass")
        assert states[k]["n_interactions"] == so["n_interactions"]
        first = hi


def test_batch_of_one_equals_unbatched(native_lib):
    w = W.spheres_drum(n=3000, seed=17, fused_step=1, fp32_contact_screen=1, fp32_broad_phase=1)
    a = w.build()
    b = W.BatchWorkload("one", w.params, [w]).build()
    for s in (a, b):
        s.first_iteration()
        s.step(100)
    assert_same_list(a.interactions(), b.interactions())
    assert bit_equal_fraction(a.particles(sort_by_id=True), b.particles(sort_by_id=True)) == 1.0
    assert a.rebuild_count() == b.rebuild_count()


def test_systems_validation(native_lib):
    b = W.drums_batch(nsys=3, nmin=300, nmax=600, seed=4)
    s = b.build()
    good = b.systems()
    bad = [dict(d) for d in good]
    bad[1]["first"] += 1  # gap
    with pytest.raises(A.DemError):
        s.set_systems(bad)
    bad = [dict(d) for d in good]
    bad[2]["driver_first"] = 7  # unregistered driver
    with pytest.raises(A.DemError):
        s.set_systems(bad)
    with pytest.raises(A.DemError):
        s.set_systems(good[:2])  # does not cover all particles
    s.set_systems(good)
    assert s.system_count() == 3
    with pytest.raises(A.DemError):
        s.set_shapes([W.shape_cube(1.0, 0.01)])  # polyhedra are single-system
