"""Polyhedra against mesh drivers in the oracle (nbh_polyhedron_driver.hpp:61-192,
polyhedron/contact.hpp:305-432), pinned by known answers on one cube (side 1,
Minkowski radius ra) at rest with gravity off:

* on a flat two-triangle mesh, the four bottom vertices touch its face
  (type 9) and the cube gets the force it gets on the equivalent wall;
* a mesh spike (one vertical triangle) whose tip is below the middle of the
  bottom face (type 12), below the middle of a bottom edge (type 11), or
  diagonally beside a bottom corner (type 7): the overlap is the analytic
  distance minus the two Minkowski radii and the force on the cube points
  away from the tip (types 11 and 12 apply the law with the mesh as particle
  i; the cube takes the opposite force).
Tolerances: 1e-12 relative for overlaps, 1e-9 for forces."""
import math

import numpy as np
import pytest

from exadem_gb300 import _abi as A
from exadem_gb300 import stl
from exadem_gb300 import workloads as W
from oracle.oracle import oracle_system

RA, MR = 0.01, 0.02


def _cube_system(z, mesh=None, surface=None, x=0.0, y=0.0):
    shapes = [W.shape_cube(1.0, RA)]
    arr = W.empty_particles(1)
    arr["rx"][:], arr["ry"][:], arr["rz"][:] = x, y, z
    arr["qw"][:] = 1.0
    arr["type"][:] = 0
    arr["id"][:] = 0
    arr["radius"][:] = shapes[0]["max_rcut"]
    arr["mass"][:] = shapes[0]["volume"]
    for ax in ("inertiax", "inertiay", "inertiaz"):
        arr[ax][:] = shapes[0]["volume"] * shapes[0]["i_over_m"]
    arr["homothety"][:] = 1.0
    cfg = dict(kn=1e4, kt=8e3, kr=0.0, mu=0.5, damp_rate=0.0)
    p = W.make_params((-5, -5, -5), (5, 5, 5), (0, 0, 0), rcut_inc=0.05, dt=1e-4, gravity=(0, 0, 0), config=cfg,
                      config_driver=cfg)
    s = oracle_system(p)
    s.set_shapes(shapes)
    s.set_particles(arr)
    if mesh is not None:
        s.register_mesh(**mesh)
    if surface is not None:
        s.register_surface(**surface)
    s.set_analysis(True)
    s.first_iteration()
    return s


def _mesh(tri):
    shp = stl.build_shape(list(np.asarray(tri, dtype=np.float64)))
    return dict(vertices=shp["vertices"], edges=shp["edges"], faces=shp["faces"], minkowski=MR)


def _touching(s):
    it, cs = s.interactions(), s.contact_state()
    t = cs["dn"] < 0
    return it["type"][t], cs["dn"][t]


def test_cube_on_flat_mesh_equals_wall():
    d = 0.003
    # the mesh triangle (-4,-4)-(4,-4)-(4,4) holds the whole cube footprint at x = 1.5, y = -1.5
    flat = _mesh([[[-4, -4, 0], [4, -4, 0], [4, 4, 0]], [[-4, -4, 0], [4, 4, 0], [-4, 4, 0]]])
    z = 0.5 + RA + MR - d
    a = _cube_system(z, mesh=flat, x=1.5, y=-1.5)
    types, dn = _touching(a)
    assert sorted(types.tolist()) == [9, 9, 9, 9]
    assert np.allclose(dn, -d, rtol=1e-9)
    b = _cube_system(z - MR, surface=dict(offset=0.0, normal=(0.0, 0.0, 1.0)), x=1.5, y=-1.5)
    fa, fb = a.particles()["fz"][0], b.particles()["fz"][0]
    assert fa > 0 and math.isclose(fa, fb, rel_tol=1e-9)
    assert math.isclose(fa, 4 * 1e4 * d, rel_tol=1e-9)


def _spike(tip):
    tx, ty, tz = tip
    return _mesh([[[tx - 0.1, ty, tz - 0.6], [tx + 0.1, ty, tz - 0.6], [tx, ty, tz]]])


@pytest.mark.parametrize("case", ["face", "edge", "corner"])
def test_spike_tip_against_the_cube(case):
    d = 0.004
    R = RA + MR
    zc = 1.0  # cube centre; bottom face at z = 0.5
    if case == "face":
        tip = (0.1, -0.2, 0.5 - R + d)
        want_type, dist = 12, R - d
    elif case == "edge":
        # below the bottom edge y = -0.5, x in (-0.5, 0.5), at distance R - d from it
        e = (R - d) / math.sqrt(2.0)
        tip = (0.2, -0.5 - e, 0.5 - e)
        want_type, dist = 11, R - d
    else:
        e = (R - d) / math.sqrt(3.0)
        tip = (-0.5 - e, -0.5 - e, 0.5 - e)
        want_type, dist = 7, R - d
    s = _cube_system(zc, mesh=_spike(tip))
    types, dn = _touching(s)
    assert want_type in types.tolist(), types
    k = types.tolist().index(want_type)
    assert math.isclose(dn[k], dist - R, rel_tol=1e-9, abs_tol=1e-12)
    p = s.particles()
    f = np.array([p["fx"][0], p["fy"][0], p["fz"][0]])
    c = np.array([0.0, 0.0, zc])
    away = c - np.array(tip)
    assert np.dot(f, away) > 0  # pushed away from the tip
    if len(types) == 1:
        assert math.isclose(np.linalg.norm(f), 1e4 * d, rel_tol=1e-9)


@pytest.mark.parametrize("homothety,skin", [(1.0, 0.05), (1.9, 0.05), (0.6, 0.6)])
def test_prefilter_keeps_every_candidate(oracle_lib, homothety, skin):
    """The oracle's reach prefilter of polyhedron-mesh candidates removes only
    features no filter keeps: the lists equal those of testing every feature, for
    random poses, large homothety and a large skin, on a terrain plus warped quads."""
    from oracle.oracle import oracle_system
    from tests.helpers import assert_same_list

    w = W.polyhedra_mesh_terrain(nx=4, ny=4, nz=2, amp=0.5, waves=3, m=8, skin=skin, seed=23)
    w.particles["homothety"] = np.full(w.n, homothety)
    w.particles["radius"] = w.particles["radius"] * homothety
    # a ring of warped quads near the lattice (non-planar faces)
    quads, verts = [], []
    for k in range(6):
        x0 = 1.0 + 1.3 * k
        base = len(verts)
        verts += [[x0, 1.0, 2.0], [x0 + 1.2, 1.0, 2.0], [x0 + 1.2, 2.2, 2.0 + 0.5 * (k % 3)], [x0, 2.2, 2.0]]
        quads.append([base, base + 1, base + 2, base + 3])
    edges = [[q[i], q[(i + 1) % 4]] for q in quads for i in range(4)]
    w.meshes.append(dict(vertices=np.asarray(verts, dtype=np.float64), edges=np.asarray(edges, dtype=np.int32),
                         faces=quads, minkowski=0.02))
    lists = []
    for brute in (1, 0):
        oracle_lib.oracle_set_mesh_brute_force(brute)
        try:
            s = w.build(oracle_system)
            s.first_iteration()
            out = [s.interactions()]
            s.step(150)
            s.update_particle_neighbors()
            out.append(s.interactions())
            s.close()
        finally:
            oracle_lib.oracle_set_mesh_brute_force(0)
        lists.append(out)
    assert sum(int((a["type"] >= 7).sum()) for a in lists[0]) > 0
    for a, b in zip(*lists):
        assert_same_list(a, b)
