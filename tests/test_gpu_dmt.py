"""Hooke + DMT adhesion (contact_force.hpp:70-76,115-127): in contact and for
gamma > 0 the force gains -2 pi reff gamma n, reff = compute_effective_radius of
the radii (spheres), of the Minkowski radii (polyhedra), or the particle's own
radius against a driver.  GPU plain and fused paths against the oracle, bit for
bit, and the parameter checks."""
import numpy as np
import pytest

from exadem_gb300 import _abi as A
from exadem_gb300 import workloads as W
from tests.helpers import assert_same_list, assert_state, bit_equal_fraction, pair

pytestmark = pytest.mark.gpu


def _dmt(w, gamma):
    w.params.law = A.LAW_HOOKE_DMT
    w.params.config.gamma = gamma
    w.params.config_driver.gamma = gamma
    return w


@pytest.mark.parametrize("fused", [0, 1])
def test_dmt_drum_matches_oracle(native_lib, fused):
    flags = dict(fused_step=fused, fp32_contact_screen=fused, fp32_broad_phase=fused)
    w = _dmt(W.spheres_drum(n=3000, seed=71, **flags), 60.0)
    g, o = pair(w)
    for s in (g, o):
        s.first_iteration()
        s.step(200)
    assert_same_list(g.interactions(), o.interactions())
    pg, po = g.particles(sort_by_id=True), o.particles(sort_by_id=True)
    assert_state(pg, po, 1e-12)
    assert bit_equal_fraction(pg, po) == 1.0


def test_dmt_changes_the_forces(native_lib):
    """Sanity: the adhesion acts (the same drum without it ends elsewhere)."""
    flags = dict(fused_step=1, fp32_contact_screen=1, fp32_broad_phase=1)
    a = _dmt(W.spheres_drum(n=2000, seed=72, **flags), 60.0).build()
    b = W.spheres_drum(n=2000, seed=72, **flags).build()
    for s in (a, b):
        s.first_iteration()
        s.step(150)
    pa, pb = a.particles(sort_by_id=True), b.particles(sort_by_id=True)
    assert np.abs(pa["vz"] - pb["vz"]).max() > 0


def test_dmt_polyhedra_matches_oracle(native_lib):
    w = _dmt(W.polyhedra_lattice(nx=6, ny=6, nz=4, seed=73, fused_step=1, fp32_broad_phase=1,
                                 fp32_contact_screen=1), 0.5)
    g, o = pair(w)
    for s in (g, o):
        s.first_iteration()
        s.step(60)
    assert_same_list(g.interactions(), o.interactions())
    pg, po = g.particles(sort_by_id=True), o.particles(sort_by_id=True)
    assert bit_equal_fraction(pg, po) == 1.0


def test_dmt_parameter_checks(native_lib):
    w = _dmt(W.spheres_box(n=200), 1.0)
    w.build()  # accepted
    w.params.config.dncut = 0.01  # dncut belongs to the cohesive law only
    with pytest.raises(A.DemError):
        w.build()
