"""Fragmentation on the oracle (CPU): stick_polyhedra, the inner bond law, the
interface fracture criterion, broken bonds and the contact list around bonds.

Known answers built by hand: two unit cubes face to face, pulled, sheared or
left at rest, and the breakage of each rupture mode at the step after the one
whose energies pass the criterion (the criterion reads the previous force pass,
config_fragmentation.msp evaluate_particle_displ).  force_law_core and the face
areas are pinned against exaDEM itself in tests/test_oracle_vs_ref.py and
tests/test_oracle_golden.py.
"""
from __future__ import annotations

import numpy as np
import pytest

from exadem_gb300 import _abi as A
from exadem_gb300 import workloads as W
from oracle.oracle import oracle_system

G = 0.05


def pair(bond=None, vx=(0.0, 0.0), vy=(0.0, 0.0), swap_ids=False, walls=False, threshold=1e-4, cluster=(0, 0)):
    """Two unit cubes bonded face to face along x at rest, no gravity."""
    w = W.fragment_blocks(nblocks=1, nx=2, ny=1, nz=1, tilt=0.0, vz=0.0, gap=0.5, threshold=threshold,
                          bond=bond or dict(kn=1e4, kt=8e3, damp_rate=0.0, g=G))
    w.params.gravity[2] = 0.0
    w.particles["vx"][:] = vx
    w.particles["vy"][:] = vy
    w.bonds["cluster"] = np.asarray(cluster, dtype=np.float64)
    if swap_ids:
        w.particles["id"] = np.ascontiguousarray(w.particles["id"][::-1])
    if walls:
        x0 = float(w.particles["rx"].min()) - 0.5 - 0.02  # a wall 0.01 from the left cube's face
        w.surfaces.append(dict(offset=x0, normal=(1.0, 0.0, 0.0)))
    return w


def test_stick_two_cubes():
    w = pair()
    s = w.build(oracle_system)
    b = s.bonds()
    assert s.bond_count() == 4
    assert np.all(b["id_i"] == 0) and np.all(b["id_j"] == 1)
    # cube vertices 1, 2, 5, 6 (x = +1/2) bonded to 0, 3, 4, 7 (x = -1/2) of the right cube
    assert b["sub_i"].tolist() == [1, 2, 5, 6] and b["sub_j"].tolist() == [0, 3, 4, 7]
    assert np.all(b["weight"] == 0.25)
    assert np.all(np.abs(b["dn0"]) < 1e-12)
    assert np.all(b["mode"] == A.RUPTURE_ENERGY_MIXED) and np.all(b["crit1"] == 2 * 1.0 * G)
    assert np.all(b["unbroken"] == 1) and not b["friction"].any() and not b["tds"].any()
    s.first_iteration()
    assert s.interaction_count() == 0  # no contact between bonded cubes


@pytest.mark.parametrize("bond,c1,c2", [
    (dict(kn=1e4, kt=8e3, damp_rate=0.5, g=0.3), 0.6, 0.0),
    (dict(kn=1e4, kt=8e3, damp_rate=0.5, gn=0.3, gt=0.7), 0.6, 1.4),
    (dict(kn=1e4, kt=8e3, damp_rate=0.5, g=0.3, sigma=5.0), 0.6, 5.0),
])
def test_stick_criterion_modes(bond, c1, c2):
    s = pair(bond).build(oracle_system)
    b = s.bonds()
    mode = {"sigma": 2, "gn": 1}.get(next((k for k in ("sigma", "gn") if k in bond), ""), 0)
    assert np.all(b["mode"] == mode)
    assert np.allclose(b["crit1"], c1, rtol=0, atol=1e-15) and np.allclose(b["crit2"], c2, rtol=0, atol=1e-15)


def test_stick_needs_cluster_and_threshold():
    assert pair(cluster=(0, 1)).build(oracle_system).bond_count() == 0
    assert pair(threshold=-1e-3).build(oracle_system).bond_count() == 0
    w = pair()
    w.particles["rx"][1] += 1e-3  # faces 1e-3 apart: dn 1e-3 above the threshold
    assert w.build(oracle_system).bond_count() == 0


def test_bonded_pair_at_rest_stays():
    s = pair().build(oracle_system)
    s.first_iteration()
    p0 = s.particles()
    s.step(200)
    p = s.particles()
    assert s.bond_count() == 4 and s.broken_interface_count() == 0
    assert np.abs(p["rx"] - p0["rx"]).max() < 1e-12


def _energies(s):
    b = s.bonds()
    en = et = 0.0
    for x, y in zip(b["en"], b["et"]):  # summed in bond order, as the criterion does
        en += x
        et += y
    return en, et


@pytest.mark.parametrize("mode", ["mixed", "separate_n", "separate_t"])
def test_energy_criterion_breaks_at_the_next_step(mode):
    """The interface breaks at the first step whose previous force pass has the
    energies past the criterion, and not before."""
    if mode == "mixed":
        bond, vx, vy = dict(kn=1e4, kt=8e3, damp_rate=0.0, g=0.02), (-0.2, 0.2), (0.0, 0.0)
        crit = lambda en, et: en + et > 2 * 0.02
    elif mode == "separate_n":
        bond, vx, vy = dict(kn=1e4, kt=8e3, damp_rate=0.0, gn=0.02, gt=1e3), (-0.2, 0.2), (0.0, 0.0)
        crit = lambda en, et: en > 0.04 or et > 2e3
    else:
        bond, vx, vy = dict(kn=1e4, kt=8e3, damp_rate=0.0, gn=1e3, gt=0.002), (0.0, 0.0), (-0.2, 0.2)
        crit = lambda en, et: en > 2e3 or et > 0.004
    s = pair(bond, vx=vx, vy=vy).build(oracle_system)
    s.first_iteration()
    passed_at = None
    for k in range(3000):
        before = _energies(s)
        s.step(1)
        if s.broken_interface_count():
            assert crit(*before), (k, before)
            assert passed_at == k - 1 or passed_at is None and k == 0
            break
        assert not crit(*before), (k, before)
        if crit(*_energies(s)) and passed_at is None:
            passed_at = k
    else:
        pytest.fail("no break")
    assert s.bond_count() == 0 and s.broken_interface_count() == 1


def test_stress_criterion_needs_both():
    """StressEnergySeparateMode: En past 2 area g is not enough while the mean
    normal force stays below area sigma."""
    base = dict(kn=1e4, kt=8e3, damp_rate=0.0, g=0.01)
    weak = pair(dict(base, sigma=1e-3), vx=(-0.2, 0.2)).build(oracle_system)
    strong = pair(dict(base, sigma=1e9), vx=(-0.2, 0.2)).build(oracle_system)
    for s in (weak, strong):
        s.first_iteration()
        s.step(600)
    assert weak.broken_interface_count() == 1 and weak.bond_count() == 0
    assert strong.broken_interface_count() == 0 and strong.bond_count() == 4
    en, _ = _energies(strong)
    assert en > 2 * 0.01  # the energy alone is past the criterion


def test_broken_pair_gets_contacts():
    """After the break the cubes are an ordinary pair: contacts are listed when
    they come back together."""
    s = pair(dict(kn=1e4, kt=8e3, damp_rate=0.0, g=1e-4), vx=(0.05, -0.05)).build(oracle_system)
    s.first_iteration()
    s.step(400)
    assert s.broken_interface_count() == 1
    lst = s.interactions()
    assert len(lst["owner_id"]) > 0 and np.all(lst["owner_id"] == 0) and np.all(lst["partner_id"] == 1)


def test_bonded_owner_skips_driver_with_partner_index():
    """As exaDEM's ignore list: the owner of a bond to the particle of id k lists
    no interaction with driver k (driver 1 here, the wall next to the cube)."""
    w = pair(walls=True)  # driver 0: floor far below; driver 1: the wall next to the left cube
    w.surfaces[0] = dict(offset=-50.0, normal=(0.0, 0.0, 1.0))
    s = w.build(oracle_system)
    s.first_iteration()
    lst = s.interactions()
    assert not np.any(lst["type"] == A.ITYPE_VERTEX_SURFACE)  # the left cube is id 0, owner of the bond to id 1
    w2 = pair(walls=True, swap_ids=True)  # the left cube is id 1 now: not the owner
    w2.surfaces[0] = dict(offset=-50.0, normal=(0.0, 0.0, 1.0))
    s2 = w2.build(oracle_system)
    s2.first_iteration()
    l2 = s2.interactions()
    wall = (l2["type"] == A.ITYPE_VERTEX_SURFACE) & (l2["partner_id"] == 1)
    assert wall.sum() == 4 and np.all(l2["owner_id"][wall] == 1)


def test_last_single_bond_interface_joins_the_one_before():
    """update_interfaces never compares the last bond with the previous one: a
    one-bond interface at the end of the list breaks with the interface before."""
    w = W.fragment_blocks(nblocks=2, nx=2, ny=1, nz=1, tilt=0.0, vz=0.0, gap=0.5,
                          bond=dict(kn=1e4, kt=8e3, damp_rate=0.0, g=0.02))
    w.params.gravity[2] = 0.0
    w.particles["vx"][:] = (-0.2, 0.2, 0.0, 0.0)  # pull the first pair apart, leave the second at rest
    s = w.build(oracle_system)
    b = s.bonds()
    assert s.bond_count() == 8
    keep = np.r_[np.arange(4), 4]
    s.set_bonds({k: (v[keep] if v.ndim == 1 else v[keep]) for k, v in b.items()})
    assert s.bond_count() == 5
    s.first_iteration()
    for _ in range(3000):
        s.step(1)
        if s.broken_interface_count():
            break
    assert s.broken_interface_count() == 1
    assert s.bond_count() == 0  # the single bond of the second pair went with the first interface


def test_bond_restart_continues_bitwise():
    """Particles, contact history and bonds saved before the impact and restored
    in a new system continue with the same bits as the original run."""
    w = W.fragment_blocks(nblocks=2)
    a = w.build(oracle_system)
    a.first_iteration()
    a.step(40)
    saved = (a.particles(sort_by_id=True), a.interactions(), a.bonds())
    b = W.fragment_blocks(nblocks=2).build(oracle_system)
    b.set_particles(saved[0])
    b.set_interactions(saved[1])
    b.set_bonds(saved[2])
    b.update_particle_neighbors()
    a.step(300)
    b.step(300)
    assert a.broken_interface_count() > 0 and b.broken_interface_count() == a.broken_interface_count()
    pa, pb = a.particles(sort_by_id=True), b.particles(sort_by_id=True)
    for k in pa:
        assert np.array_equal(np.asarray(pa[k]).view(np.uint8), np.asarray(pb[k]).view(np.uint8)), k
    ba, bb = a.bonds(), b.bonds()
    for k in ba:
        assert np.array_equal(np.asarray(ba[k]).view(np.uint8), np.asarray(bb[k]).view(np.uint8)), k
