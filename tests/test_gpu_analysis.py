"""Contact state and stress tensor (stress_tensor.cu, contact_state.hpp):
GPU against the oracle bit for bit (state per interaction, stress per particle
and in total), for the plain and fused sphere paths, the cohesive law and
polyhedra (state in the contact law's frame, swapped pairs included); the
analysis mode leaves the trajectory's bits unchanged."""
import numpy as np
import pytest

from exadem_gb300 import _abi as A
from exadem_gb300 import workloads as W
from tests.helpers import assert_same_list, bit_equal_fraction, pair

pytestmark = pytest.mark.gpu


def _bits(x):
    return np.ascontiguousarray(x).view(np.uint64)


def _by_id(sys_, stress):
    ids = sys_.particles(sort_by_id=False)["id"]
    return stress[np.argsort(ids)]


@pytest.mark.parametrize("case", ["drum_fused", "drum_plain", "cohesive_floor", "poly_fused", "poly_plain"])
def test_contact_state_and_stress_match_oracle(native_lib, case):
    steps = 150
    if case == "cohesive_floor":
        w = W.spheres_floor(n=4000, side=14.0, seed=91, fused_step=1, fp32_contact_screen=1, fp32_broad_phase=1)
    elif case.startswith("poly"):
        fused = int(case == "poly_fused")
        w = W.polyhedra_lattice(nx=6, ny=6, nz=4, seed=93, fused_step=fused, fp32_broad_phase=fused,
                                fp32_contact_screen=fused)
        steps = 80
    else:
        fused = int(case == "drum_fused")
        w = W.spheres_drum(n=3000, seed=91, fused_step=fused, fp32_contact_screen=fused, fp32_broad_phase=fused)
    g, o = pair(w)
    for s in (g, o):
        s.set_analysis(True)
        s.first_iteration()
        s.step(steps)
    lg = g.interactions()
    assert_same_list(lg, o.interactions())
    cg, co = g.contact_state(), o.contact_state()
    assert np.sum(cg["dn"] < 0) > 0
    if case.startswith("poly"):
        assert np.sum(lg["swap"].astype(bool) & (cg["dn"] < 0)) > 0
    for k in ("dn", "cp", "fn", "ft"):
        assert np.array_equal(_bits(cg[k]), _bits(co[k])), k
    sg, tg = g.stress_tensor()
    so, to = o.stress_tensor()
    assert np.array_equal(_bits(_by_id(g, sg)), _bits(_by_id(o, so)))
    assert np.array_equal(_bits(tg), _bits(to))
    assert np.abs(tg).max() > 0


def test_analysis_keeps_the_trajectory(native_lib):
    w = W.spheres_drum(n=2500, seed=92, fused_step=1, fp32_contact_screen=1, fp32_broad_phase=1)
    a, b = w.build(), w.build()
    b.set_analysis(True)
    for s in (a, b):
        s.first_iteration()
        s.step(200)
    assert bit_equal_fraction(a.particles(sort_by_id=True), b.particles(sort_by_id=True)) == 1.0


def test_analysis_keeps_the_polyhedron_trajectory(native_lib):
    w = W.polyhedra_lattice(nx=6, ny=6, nz=4, seed=94, fused_step=1, fp32_broad_phase=1, fp32_contact_screen=1)
    a, b = w.build(), w.build()
    b.set_analysis(True)
    for s in (a, b):
        s.first_iteration()
        s.step(80)
    assert bit_equal_fraction(a.particles(sort_by_id=True), b.particles(sort_by_id=True)) == 1.0


def test_analysis_refusals(native_lib):
    s = W.spheres_box(n=300).build()
    s.first_iteration()
    with pytest.raises(A.DemError):
        s.stress_tensor()  # analysis off
    with pytest.raises(A.DemError):
        s.contact_state()
