"""GPU parity of fragmentation (inner bonds) against the CPU oracle.

Blocks of face-to-face cubes bonded by stick_polyhedra fall on a floor and
break in part.  The bonds made on the device's vertices, the bond list with its
state after every stretch of steps, the interaction list (with the history of
the broken bonds carried as vertex-vertex friction), the broken interface
count and every particle field must have the same bits as the oracle's, on the
plain and the fused step, for the three rupture modes.
"""
import numpy as np
import pytest

from exadem_gb300 import workloads as W
from tests.helpers import assert_same_list, pair

pytestmark = pytest.mark.gpu

FAST = dict(fused_step=1, fp32_broad_phase=1, fp32_contact_screen=1)
FIELDS = ["rx", "ry", "rz", "vx", "vy", "vz", "fx", "fy", "fz", "vrotx", "vroty", "vrotz", "arotx", "aroty",
          "arotz", "momx", "momy", "momz", "qw", "qx", "qy", "qz"]


def same_bits(a, b):
    return np.array_equal(np.ascontiguousarray(a).view(np.uint8), np.ascontiguousarray(b).view(np.uint8))


def assert_same_bonds(g, o):
    bg, bo = g.bonds(), o.bonds()
    assert len(bg["id_i"]) == len(bo["id_i"])
    for k in bg:
        assert same_bits(bg[k], bo[k]), k
    sg, so = g.bond_state(), o.bond_state()  # the analysis state of the last bond pass
    for k in sg:
        assert same_bits(sg[k], so[k]), k


def assert_same_particles(g, o):
    pg, po = g.particles(sort_by_id=True), o.particles(sort_by_id=True)
    for k in FIELDS:
        assert same_bits(pg[k], po[k]), k


@pytest.mark.parametrize("flags", [{}, FAST], ids=["plain", "fused"])
def test_stick_same_bonds(native_lib, flags):
    w = W.fragment_blocks(nblocks=4, nx=3, ny=2, nz=2, tilt=0.5, seed=3, **flags)
    g, o = pair(w)
    assert g.bond_count() == o.bond_count() > 0
    assert_same_bonds(g, o)


@pytest.mark.parametrize("bond", [
    dict(kn=1e4, kt=8e3, damp_rate=0.87, g=0.05),
    dict(kn=1e4, kt=8e3, damp_rate=0.87, gn=0.04, gt=0.02),
    dict(kn=1e4, kt=8e3, damp_rate=0.87, g=0.01, sigma=2.0),
], ids=["mixed", "separate", "stress"])
@pytest.mark.parametrize("flags", [{}, FAST], ids=["plain", "fused"])
def test_impact_breaks_like_oracle(native_lib, bond, flags):
    w = W.fragment_blocks(nblocks=2, bond=bond, **flags)
    g, o = pair(w)
    for s in (g, o):
        s.first_iteration()
    for _ in range(8):
        for s in (g, o):
            s.step(50)
        assert g.broken_interface_count() == o.broken_interface_count()
        assert g.rebuild_count() == o.rebuild_count()
        assert_same_bonds(g, o)
        lg, lo = g.interactions(), o.interactions()
        assert_same_list(lg, lo)
        assert same_bits(lg["friction"], lo["friction"]) and same_bits(lg["moment"], lo["moment"])
        assert_same_particles(g, o)
    assert 0 < o.broken_interface_count()


def test_many_blocks_fused(native_lib):
    """16 blocks of 4 x 4 x 4 cubes (1024 particles, 2304 interfaces), 300 steps."""
    w = W.fragment_blocks(nblocks=16, nx=4, ny=4, nz=4, seed=9, **FAST)
    g, o = pair(w)
    for s in (g, o):
        s.first_iteration()
        s.step(300)
    assert g.broken_interface_count() == o.broken_interface_count() > 0
    assert o.bond_count() > 0
    assert_same_bonds(g, o)
    assert_same_list(g.interactions(), o.interactions())
    assert_same_particles(g, o)


def test_operators_like_oracle(native_lib):
    """inner_bond_polyhedron and apply_interface_fracture_criterion called on
    their own, as the onika shims do: after the impact the criteria are lowered
    (dem_set_bonds), the list rebuilt, the bond pass run and the criterion
    applied."""
    w = W.fragment_blocks(nblocks=2, bond=dict(kn=1e4, kt=8e3, damp_rate=0.87, g=10.0))
    g, o = pair(w)
    for s in (g, o):
        s.first_iteration()
        s.step(250)
        b = s.bonds()
        b["crit1"][:] = 1e-30
        s.set_bonds(b)
        s.update_particle_neighbors()
        s.inner_bond_polyhedron()
    assert_same_particles(g, o)
    assert g.apply_interface_fracture_criterion() == o.apply_interface_fracture_criterion() > 0
    assert_same_bonds(g, o)


def test_gpu_bonds_resume_on_oracle(native_lib):
    """A GPU run saved before the impact (particles, contacts, bonds) continues
    on the oracle with the bits of the GPU's own continuation."""
    from oracle.oracle import oracle_system

    w = W.fragment_blocks(nblocks=2, **FAST)
    g = w.build()
    g.first_iteration()
    g.step(40)
    saved = (g.particles(sort_by_id=True), g.interactions(), g.bonds())
    o = W.fragment_blocks(nblocks=2, **FAST).build(oracle_system)
    o.set_particles(saved[0])
    o.set_interactions(saved[1])
    o.set_bonds(saved[2])
    o.update_particle_neighbors()
    g.step(300)
    o.step(300)
    assert g.broken_interface_count() == o.broken_interface_count() > 0
    assert_same_bonds(g, o)
    assert_same_particles(g, o)
