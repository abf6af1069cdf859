"""Multi-material contact parameters (dem_set_multimat; multimat_parameters.hpp,
the contact_multimat_* operators): the parameters of a pair come from a table
indexed by the particles' group field, those of a particle and a driver from a
group x driver table.  GPU plain and fused paths against the oracle, bit for
bit, for spheres (Hooke, cohesive) and polyhedra, and the table checks."""
import numpy as np
import pytest

from exadem_gb300 import _abi as A
from exadem_gb300 import workloads as W
from exadem_gb300.system import contact_params
from oracle.oracle import oracle_system
from tests.helpers import assert_same_list, bit_equal_fraction

pytestmark = pytest.mark.gpu


def _tables(ng, nd, cohesive=False, seed=0):
    rng = np.random.default_rng(seed)
    pairs = [[None] * ng for _ in range(ng)]
    for a in range(ng):
        for b in range(a, ng):
            kw = dict(kn=float(rng.uniform(5e3, 2e4)), kt=float(rng.uniform(4e3, 1e4)), kr=0.0,
                      mu=float(rng.uniform(0.2, 0.6)), damp_rate=float(rng.uniform(0.5, 0.95)))
            if cohesive:
                kw.update(dncut=float(rng.uniform(0.005, 0.02)), fc=float(rng.uniform(5.0, 15.0)))
            pairs[a][b] = pairs[b][a] = contact_params(**kw)
    drivers = [[contact_params(kn=float(rng.uniform(5e3, 2e4)), kt=8e3, mu=float(rng.uniform(0.2, 0.6)),
                               damp_rate=0.9, **(dict(dncut=0.01, fc=10.0) if cohesive else {}))
                for _ in range(nd)] for _ in range(ng)]
    return pairs, drivers


def _run_pair(w, pairs, drivers, steps):
    out = []
    for factory in (None, oracle_system):
        s = w.build(factory)
        s.set_multimat(pairs, drivers)
        s.first_iteration()
        s.step(steps)
        out.append(s)
    return out


@pytest.mark.parametrize("fused", [0, 1])
def test_multimat_drum_matches_oracle(native_lib, fused):
    flags = dict(fused_step=fused, fp32_contact_screen=fused, fp32_broad_phase=fused)
    w = W.spheres_drum(n=3000, seed=81, **flags)
    w.particles["group"] = np.random.default_rng(81).integers(0, 3, w.n).astype(np.uint32)
    pairs, drivers = _tables(3, 1, seed=81)
    g, o = _run_pair(w, pairs, drivers, 200)
    assert_same_list(g.interactions(), o.interactions())
    assert bit_equal_fraction(g.particles(sort_by_id=True), o.particles(sort_by_id=True)) == 1.0


def test_multimat_cohesive_floor_matches_oracle(native_lib):
    w = W.spheres_floor(n=4000, side=14.0, seed=82, fused_step=1, fp32_contact_screen=1, fp32_broad_phase=1)
    w.particles["group"] = np.random.default_rng(82).integers(0, 2, w.n).astype(np.uint32)
    pairs, drivers = _tables(2, 1, cohesive=True, seed=82)
    g, o = _run_pair(w, pairs, drivers, 200)
    assert_same_list(g.interactions(), o.interactions())
    assert bit_equal_fraction(g.particles(sort_by_id=True), o.particles(sort_by_id=True)) == 1.0


def test_multimat_polyhedra_matches_oracle(native_lib):
    w = W.polyhedra_lattice(nx=6, ny=6, nz=4, seed=83, fused_step=1, fp32_broad_phase=1, fp32_contact_screen=1)
    w.particles["group"] = np.random.default_rng(83).integers(0, 2, w.n).astype(np.uint32)
    pairs, drivers = _tables(2, len(w.surfaces) + len(w.cylinders), seed=83)
    g, o = _run_pair(w, pairs, drivers, 60)
    assert_same_list(g.interactions(), o.interactions())
    assert bit_equal_fraction(g.particles(sort_by_id=True), o.particles(sort_by_id=True)) == 1.0


def test_uniform_table_equals_single_set(native_lib):
    w = W.spheres_drum(n=2000, seed=84, fused_step=1, fp32_contact_screen=1, fp32_broad_phase=1)
    w.particles["group"] = np.random.default_rng(84).integers(0, 2, w.n).astype(np.uint32)
    a, b = w.build(), w.build()
    cp, cpd = w.params.config, w.params.config_driver
    b.set_multimat([[cp, cp], [cp, cp]], [[cpd], [cpd]])
    for s in (a, b):
        s.first_iteration()
        s.step(150)
    assert bit_equal_fraction(a.particles(sort_by_id=True), b.particles(sort_by_id=True)) == 1.0


def test_multimat_checks(native_lib):
    w = W.spheres_drum(n=500, seed=85)
    w.particles["group"] = np.random.default_rng(85).integers(0, 2, w.n).astype(np.uint32)
    s = w.build()
    pairs, drivers = _tables(2, 1, seed=85)
    asym = [[pairs[0][0], pairs[0][1]], [contact_params(kn=1.0), pairs[1][1]]]
    with pytest.raises(A.DemError):
        s.set_multimat(asym, drivers)  # not symmetric
    with pytest.raises(A.DemError):
        s.set_multimat([[pairs[0][0]]], [[drivers[0][0]]])  # group 1 has no row
    with pytest.raises(A.DemError):
        s.set_multimat(pairs, [[drivers[0][0], drivers[0][0]]] * 2)  # two drivers, one registered
    s.set_multimat(pairs, drivers)
    s.set_multimat([], [])  # back to the single sets
