"""Mesh drivers on the CPU: the STL reader and shape conversion
(stl_mesh_reader.hpp:25-132, stl_mesh_to_driver.hpp:26-121), and the oracle's
sphere-mesh contacts (nbh_sphere.hpp:25-86, contact_sphere.hpp:300-396) pinned
by known answers: a sphere on a flat mesh face gets the force of a sphere on
the equivalent wall (1e-12 relative), and a sphere over a mesh vertex or edge
gets the overlap of the analytic distance."""
import math

import numpy as np
import pytest

from exadem_gb300 import stl
from exadem_gb300 import workloads as W
from exadem_gb300.system import contact_params
from oracle.oracle import oracle_system


def test_binary_stl_round_trip(tmp_path):
    tri = W.terrain_triangles(8.0, 4, 0.5, 1, 0.0)
    path = str(tmp_path / "t.stl")
    stl.write_stl_binary(path, tri)
    faces = stl.read_stl(path, True)
    assert len(faces) == len(tri)
    assert np.array_equal(np.asarray(faces), tri.astype(np.float32).astype(np.float64))
    shp = stl.build_shape(faces)
    assert len(shp["vertices"]) == 25  # a 5 x 5 grid
    v = [tuple(x) for x in shp["vertices"]]
    assert v == sorted(set(v))  # sorted, unique
    assert len(shp["edges"]) == 3 * len(tri)  # each face's edges, shared ones twice
    for f, t in zip(shp["faces"], faces):
        assert np.array_equal(shp["vertices"][f], t)


def test_ascii_stl(tmp_path):
    path = tmp_path / "a.stl"
    path.write_text("solid s\n facet normal 0 0 1\n  outer loop\n   vertex 0 0 0\n   vertex 1 0 0\n"
                    "   vertex 0 1 0\n  endloop\n endfacet\n facet normal 0 0 1\n  outer loop\n"
                    "   vertex 1 0 0\n   vertex 1 1 0\n   vertex 0 1 0\n  endloop\n endfacet\nendsolid s\n")
    shp = stl.build_shape(stl.read_stl(str(path), False))
    assert shp["vertices"].tolist() == [[0, 0, 0], [0, 1, 0], [1, 0, 0], [1, 1, 0]]
    assert shp["faces"] == [[0, 2, 1], [2, 3, 1]]
    assert shp["edges"].tolist() == [[0, 2], [2, 1], [1, 0], [2, 3], [3, 1], [1, 2]]


def test_consecutive_edge_duplicates_only():
    # std::unique without a sort: a degenerate face repeats its edge consecutively
    a = np.zeros(3)
    faces = [np.array([a, a, a]), np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0.0]])]
    shp = stl.build_shape(faces)
    assert shp["edges"].tolist() == [[0, 0], [0, 2], [2, 1], [1, 0]]


def test_rescale_keeps_topology():
    shp = stl.build_shape(list(W.terrain_triangles(4.0, 2, 0.3, 1, 0.0)))
    big = stl.rescale(shp, 100.0)
    assert np.array_equal(big["vertices"], 100.0 * shp["vertices"])
    assert big["faces"] == shp["faces"] and np.array_equal(big["edges"], shp["edges"])


def _one_sphere(z, x=0.0, y=0.0, r=0.5, mesh=None, surface=None, vz=0.0):
    from exadem_gb300 import _abi as A

    cfg = dict(kn=1e4, kt=8e3, kr=0.0, mu=0.4, damp_rate=0.0)
    p = W.make_params((-10, -10, -10), (10, 10, 10), (0, 0, 0), rcut_inc=0.1, dt=1e-4, gravity=(0, 0, 0),
                      config=cfg, config_driver=cfg)
    parts = {f: np.zeros(1) for f in A.PARTICLE_FIELDS}
    parts.update(rx=np.array([x]), ry=np.array([y]), rz=np.array([z]), radius=np.array([r]),
                 vz=np.array([vz]), mass=np.array([1.0]), qw=np.array([1.0]),
                 inertia=np.full(1, 0.4 * r * r), homothety=np.ones(1))
    parts["id"] = np.zeros(1, np.uint64)
    parts["type"] = np.zeros(1, np.uint32)
    parts["group"] = np.zeros(1, np.uint32)
    s = oracle_system(p)
    s.set_particles(parts)
    if mesh:
        s.register_mesh(**mesh)
    if surface:
        s.register_surface(**surface)
    s.set_analysis(True)
    s.first_iteration()
    return s


def _plane_mesh(z, mr):
    tri = np.array([[[-5, -5, 0], [5, -5, 0], [5, 5, 0]], [[-5, -5, 0], [5, 5, 0], [-5, 5, 0]]], dtype=np.float64)
    shp = stl.build_shape(list(tri))
    return dict(vertices=shp["vertices"], edges=shp["edges"], faces=shp["faces"], minkowski=mr, center=(0, 0, z))


@pytest.mark.parametrize("x,y", [(1.3, -2.1), (-0.7, 3.9)])
def test_face_contact_equals_wall(x, y):
    mr, d = 0.05, 0.004
    z = 0.5 + mr - d  # overlap d with the plane z = 0 thickened by mr
    a = _one_sphere(z, x, y, mesh=_plane_mesh(0.0, mr))
    b = _one_sphere(z - mr, x, y, surface=dict(offset=0.0, normal=(0.0, 0.0, 1.0)))
    la, sa = a.interactions(), a.contact_state()
    touch = sa["dn"] < 0
    assert list(la["type"][touch]) == [9]  # one face; vertices and edges are out of reach
    sb = b.contact_state()
    assert sb["dn"][0] < 0
    assert math.isclose(sa["dn"][touch][0], -d, rel_tol=1e-9)
    assert math.isclose(sa["dn"][touch][0], sb["dn"][0], rel_tol=1e-9)
    fa, fb = a.particles()["fz"][0], b.particles()["fz"][0]
    assert fa > 0 and math.isclose(fa, fb, rel_tol=1e-9)
    assert math.isclose(fa, 1e4 * d, rel_tol=1e-9)


@pytest.mark.parametrize("kind", ["vertex", "edge"])
def test_vertex_and_edge_overlaps(kind):
    mr = 0.05
    tri = np.array([[[0, 0, 0], [4, 0, 0], [0, 4, 0]]], dtype=np.float64)
    shp = stl.build_shape(list(tri))
    mesh = dict(vertices=shp["vertices"], edges=shp["edges"], faces=shp["faces"], minkowski=mr)
    # beside the corner (0, 0, 0) below the plane, or beside the edge y = 0
    pos = (-0.3, -0.2, -0.4) if kind == "vertex" else (1.7, -0.3, -0.35)
    dist = math.sqrt(pos[0] ** 2 + pos[1] ** 2 + pos[2] ** 2) if kind == "vertex" else math.hypot(pos[1], pos[2])
    s = _one_sphere(pos[2], pos[0], pos[1], mesh=mesh)
    it, cs = s.interactions(), s.contact_state()
    touch = cs["dn"] < 0
    want = 7 if kind == "vertex" else 8
    assert want in set(it["type"][touch].tolist())
    k = int(np.flatnonzero(touch & (it["type"] == want))[0])
    assert math.isclose(cs["dn"][k], dist - (0.5 + mr), rel_tol=1e-12)


def test_mesh_candidates_cover_the_touching_features():
    w = W.spheres_mesh_terrain(n=800, seed=12)
    s = w.build(oracle_system)
    s.set_analysis(True)
    s.first_iteration()
    s.step(300)
    it, cs = s.interactions(), s.contact_state()
    mesh_items = (it["type"] >= 7) & (it["type"] <= 9)
    assert mesh_items.sum() > 0
    assert ((cs["dn"] < 0) & mesh_items).sum() > 0
    assert np.all(it["partner_id"][mesh_items] == 4)  # the driver after the four walls


def test_stl_file_to_simulation(tmp_path):
    """register_stl_mesh from a file: the STL read, converted and rescaled
    (float32 vertices, scale 2) gives the same run as the same arrays given
    directly."""
    tri = W.terrain_triangles(8.0, 8, 0.4, 1, 0.0)
    path = str(tmp_path / "terrain.stl")
    stl.write_stl_binary(path, tri)
    shp = stl.load_stl_mesh(path, True, scale=2.0)
    direct = stl.rescale(stl.build_shape(list(tri.astype(np.float32).astype(np.float64))), 2.0)
    assert np.array_equal(shp["vertices"], direct["vertices"])
    runs = []
    for sh in (shp, direct):
        w = W.spheres_mesh_terrain(n=400, side=16.0, seed=61)
        w.meshes = [dict(w.meshes[0], vertices=sh["vertices"], edges=sh["edges"], faces=sh["faces"])]
        s = w.build(oracle_system)
        s.first_iteration()
        s.step(300)
        runs.append((s.interactions(), s.particles(sort_by_id=True)))
    (la, pa), (lb, pb) = runs
    assert np.sum((la["type"] >= 7) & (la["type"] <= 9)) > 0
    for k in la:
        assert np.array_equal(la[k], lb[k]), k
    for k in ("rx", "ry", "rz", "vx", "vy", "vz"):
        assert np.array_equal(pa[k], pb[k]), k
