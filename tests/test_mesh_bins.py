"""The mesh feature bins (exadem_gb300/csrc/mesh_bins.hpp, built on the host and
used by the GPU neighbour passes) list, in the bin of every sphere centre,
every mesh feature that passes its Verlet filter for that sphere.  The oracle
enumerates the candidates brute force over all features
(nbh_sphere.hpp:25-86); each of its sphere-mesh interactions must be listed
in the sphere's bin."""
import ctypes as C
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from exadem_gb300 import workloads as W
from oracle.oracle import oracle_system

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def mb(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    so = tmp_path_factory.mktemp("mb") / "libmb.so"
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", "-shared", "-fPIC", "-I",
                    str(ROOT / "exadem_gb300" / "csrc"), str(ROOT / "tests" / "mesh_bins_capi.cpp"), "-o", str(so)],
                   check=True)
    lib = C.CDLL(str(so))
    PD, PI = C.POINTER(C.c_double), C.POINTER(C.c_int)
    lib.mb_build.restype = C.c_void_p
    lib.mb_build.argtypes = [C.c_int, PD, PD, PD, C.c_int, PI, C.c_int, PI, PI, C.c_double, C.c_double, C.c_double,
                             PI]
    lib.mb_items.restype = C.c_int
    lib.mb_items.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_double, C.POINTER(C.c_uint32), C.c_int]
    lib.mb_free.argtypes = [C.c_void_p]
    return lib


def _world(mesh):
    """center + quat * v (shape::get_vertex with homothety 1)."""
    v = np.asarray(mesh["vertices"], dtype=np.float64)
    w, x, y, z = mesh.get("quat", (1.0, 0.0, 0.0, 0.0))
    u = np.array([x, y, z])
    uv = np.cross(u, v)
    uuv = np.cross(u, uv)
    return np.asarray(mesh.get("center", (0.0, 0.0, 0.0))) + v + uv * (2.0 * w) + uuv * 2.0


def _bins(mb, mesh, rad, skin):
    wv = _world(mesh)
    x, y, z = (np.ascontiguousarray(wv[:, k]) for k in range(3))
    e = np.ascontiguousarray(np.asarray(mesh["edges"], dtype=np.int32).reshape(-1))
    faces = mesh["faces"]
    fo = np.zeros(len(faces) + 1, dtype=np.int32)
    fo[1:] = np.cumsum([len(f) for f in faces])
    fv = np.ascontiguousarray(np.concatenate([np.asarray(f, dtype=np.int32) for f in faces]))
    PD, PI = C.POINTER(C.c_double), C.POINTER(C.c_int)
    st = C.c_int(-1)
    h = mb.mb_build(len(wv), x.ctypes.data_as(PD), y.ctypes.data_as(PD), z.ctypes.data_as(PD), len(e) // 2,
                    e.ctypes.data_as(PI), len(faces), fo.ctypes.data_as(PI), fv.ctypes.data_as(PI),
                    float(mesh["minkowski"]), rad, skin, C.byref(st))
    assert st.value == 0
    return h


@pytest.mark.parametrize("case", ["terrain", "mixer"])
def test_bins_hold_every_candidate(mb, case):
    if case == "terrain":
        w = W.spheres_mesh_terrain(n=1500, seed=41)
        steps = 400
    else:
        w = W.spheres_mixer(n=3000)
        steps = 400
    s = w.build(oracle_system)
    s.first_iteration()
    s.step(steps)
    p = s.particles(sort_by_id=True)
    row = {int(i): k for k, i in enumerate(p["id"])}
    it = s.interactions()
    sel = np.flatnonzero((it["type"] >= 7) & (it["type"] <= 9))
    assert len(sel) > 0
    mesh_driver = len(w.surfaces) + len(w.cylinders)  # the mesh is registered after them
    h = _bins(mb, w.meshes[0], float(np.max(w.particles["radius"])), float(w.params.rcut_inc))
    buf = (C.c_uint32 * 4096)()
    try:
        for k in sel:
            assert int(it["partner_id"][k]) == mesh_driver
            q = row[int(it["owner_id"][k])]
            n = mb.mb_items(h, p["rx"][q], p["ry"][q], p["rz"][q], buf, 4096)
            assert 0 <= n <= 4096
            want = ((int(it["type"][k]) - 7) << 30) | int(it["partner_sub"][k])
            assert want in set(buf[:n]), (int(it["type"][k]), int(it["partner_sub"][k]))
    finally:
        mb.mb_free(h)


def test_nonplanar_face_in_bins(mb, oracle_lib):
    """A non-planar quad: every point the reference's face filter keeps (it projects on
    the plane of the first, second and last vertex) is in a bin listing the face."""
    from oracle import units as U

    h_warp = 0.6
    mesh = {"vertices": [[0, 0, 0], [2, 0, 0], [2, 2, h_warp], [0, 2, 0]], "edges": [[0, 1], [1, 2], [2, 3], [3, 0]],
            "faces": [[0, 1, 2, 3]], "minkowski": 0.02}
    rad, skin = 0.3, 0.1
    hb = _bins(mb, mesh, rad, skin)
    rng = np.random.default_rng(5)
    pts = rng.uniform([-0.5, -0.5, -0.6], [2.5, 2.5, 1.2], (40000, 3))
    rows = np.zeros((len(pts), 6 + 12))
    rows[:, 0] = skin
    rows[:, 1:4] = pts
    rows[:, 4] = rad
    rows[:, 5] = 1.0
    rows[:, 6:] = np.asarray(mesh["vertices"], dtype=np.float64).reshape(-1)
    shape = {"vertices": np.asarray(mesh["vertices"], dtype=np.float64), "faces": mesh["faces"],
             "radius": mesh["minkowski"]}
    keep = U.run_vertex_face_oracle(oracle_lib, shape, 0, rows)[:, 0] > 0
    assert keep.sum() > 1000
    buf = (C.c_uint32 * 4096)()
    face_item = (2 << 30) | 0
    try:
        for x, y, z in pts[keep]:
            n = mb.mb_items(hb, x, y, z, buf, 4096)
            assert face_item in set(buf[:n]), (x, y, z)
    finally:
        mb.mb_free(hb)
