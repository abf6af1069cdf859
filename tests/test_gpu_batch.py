"""Batched systems (dem_set_systems): each system of a batch evolves exactly as
the same system alone (every particle bit, its interaction list and history),
checked against the oracle running each drum on its own; a batch of one
equals the unbatched context."""
import numpy as np
import pytest

from exadem_gb300 import _abi as A
from exadem_gb300 import workloads as W
from tests.helpers import ENERGY_RTOL, assert_close_rel, assert_same_list, assert_state, bit_equal_fraction

pytestmark = pytest.mark.gpu

STEPS = 600


def _split_list(lst: dict, lo: int, hi: int) -> dict:
    m = (lst["owner_id"] >= lo) & (lst["owner_id"] < hi)
    return {k: v[m] for k, v in lst.items()}


def _touching(lst: dict) -> dict:
    f = np.asarray(lst["friction"]).reshape(-1, 3)
    m = np.asarray(lst["moment"]).reshape(-1, 3)
    keep = np.any(f != 0, axis=1) | np.any(m != 0, axis=1)
    return {k: v[keep] for k, v in lst.items()}


def _split_particles(p: dict, lo: int, hi: int) -> dict:
    m = (p["id"] >= lo) & (p["id"] < hi)
    return {k: v[m] for k, v in p.items()}


@pytest.mark.parametrize("flags", [{}, dict(fused_step=1, fp32_contact_screen=1, fp32_broad_phase=1)])
def test_batched_drums_match_each_drum_alone(native_lib, flags):
    from oracle.oracle import oracle_system

    b = W.drums_batch(nsys=5, nmin=400, nmax=2500, seed=9, **flags)
    # axial velocities: each drum triggers rebuilds on its own steps and particles
    # cross the periodic ends, so shared rebuilds must not wrap or re-base other drums
    rng = np.random.default_rng(9)
    for m in b.members:
        m.particles["vy"] = rng.uniform(-2.0, 2.0, m.n)
    g = b.build()
    g.first_iteration()
    g.step(STEPS)
    lg, pg = g.interactions(), g.particles(sort_by_id=True)
    states = g.system_states()
    assert g.rebuild_count() > 0
    first = 0
    for k, m in enumerate(b.members):
        o = m.build(oracle_system)
        o.first_iteration()
        o.step(STEPS)
        assert o.rebuild_count() > 3
        lo, hi = first, first + m.n
        # a shared rebuild keeps the slots and the list of a drum whose own trigger
        # did not fire: its whole list is the one it has alone
        lk, lo_ = _split_list(lg, lo, hi), o.interactions()
        assert_same_list(lk, lo_)
        np.testing.assert_array_equal(lk["friction"], lo_["friction"])
        np.testing.assert_array_equal(lk["moment"], lo_["moment"])
        assert len(_touching(lk)["owner_id"]) > 0
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
    from exadem_gb300 import make_params

    p = b.params
    coh = make_params(list(p.bounds_lo), list(p.bounds_hi), list(p.periodic), rcut_inc=p.rcut_inc, dt=p.dt,
                      law=A.LAW_HOOKE_COHESIVE, config=dict(fc=10.0, dncut=0.01))
    with pytest.raises(A.DemError):
        s.set_params(coh)  # cohesion would rebuild systems off their own schedule
    with pytest.raises(A.DemError):
        s.set_shapes([W.shape_cube(1.0, 0.01)])  # polyhedra are single-system
