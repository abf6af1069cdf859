"""The oracle against exaDEM's own functions, bit for bit (CPU).

exaDEM's headers are compiled on the host, unchanged, by oracle/ref_build.py
(oracle/ref_harness.cpp, with the stand-ins of oracle/ref_shim/ for onika,
exaNBody, MPI, yaml-cpp and tinyexpr).  Each test draws seeded cases that mix
random values with the edge cases the functions branch on and requires every
output double of the oracle to have the same bits as exaDEM's.  Skipped where
the exaDEM sources are not present (tests/test_oracle_golden.py then checks the
oracle against vectors generated here).
"""
from __future__ import annotations

import ctypes as C
import glob
import os

import numpy as np
import pytest

from oracle import build as oracle_build
from oracle import ref_build
from oracle import units as U

pytestmark = pytest.mark.skipif(not ref_build.available(), reason="exaDEM sources not present")

N = 200_000


@pytest.fixture(scope="module")
def libs():
    return C.CDLL(str(ref_build.build())), C.CDLL(str(oracle_build.build()))


def same_bits(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Per row: every double has identical bits."""
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    return (a.view(np.uint64) == b.view(np.uint64)).all(axis=1)


def check(name, rows, ref_out, orc_out):
    ok = same_bits(ref_out, orc_out)
    if not ok.all():
        i = int(np.nonzero(~ok)[0][0])
        pytest.fail(f"{name}: {int((~ok).sum())} of {len(ok)} cases differ; first input {rows[i].tolist()}\n"
                    f"exaDEM {ref_out[i].tolist()}\noracle {orc_out[i].tolist()}")


@pytest.mark.parametrize("law", [0, 1, 2], ids=["hooke", "cohesive", "dmt"])
def test_contact_force_core(libs, law):
    """contact_force_core<Hooke, None|Cohesive|DMT> and compute_moments: spin exactly zero
    (the mur = 0 clip keeps the moment), dn at 0 and at the cohesion distance, zero history."""
    ref, orc = libs
    x = U.cases("contact_force_core", N, 100 + law)
    check("contact_force_core", x, U.run(ref, "ref", "contact_force_core", x, law),
          U.run(orc, "oracle", "contact_force_core", x, law))


@pytest.mark.parametrize("name", [n for n in U.LAYOUT if n != "contact_force_core"])
def test_unit(libs, name):
    ref, orc = libs
    x = U.cases(name, N, 7)
    check(name, x, U.run(ref, "ref", name, x), U.run(orc, "oracle", name, x))


def test_filters_reach_both_outcomes(libs):
    """The drawn cases exercise both results of every filter and detection."""
    ref, _ = libs
    for name, col in [("filter_vv", 0), ("filter_ve", 0), ("filter_ee", 0), ("detect_vv", 0), ("detect_ve", 0),
                      ("detect_ee", 0), ("obb_intersect", 0), ("surface", 0), ("surface", 1), ("cylinder", 0),
                      ("cylinder", 1)]:
        out = U.run(ref, "ref", name, U.cases(name, 20_000, 3))
        frac = out[:, col].mean()
        assert 0.02 < frac < 0.98, (name, col, frac)


def test_pair_order(libs):
    """InteractionPair::operator< and == on keys with many ties."""
    ref, orc = libs
    k = U.pair_keys(N, 5)
    a, b = U.run_pair_order(ref, "ref", k), U.run_pair_order(orc, "oracle", k)
    assert np.array_equal(a, b)
    assert 0.1 < a[:, 1].mean() < 0.5


def _exadem_shape_files():
    return sorted(glob.glob(os.path.join(str(ref_build.EXADEM), "**", "*.shp"), recursive=True))


def test_shp_reader_and_shape_obb(libs):
    """exadem_gb300.shp reads every shape file of the exaDEM tree as read_shp does, and
    workloads.build_obb gives the shape OBB of build_obb_from_shape, bit for bit."""
    from exadem_gb300 import shp

    ref, orc_lib = libs
    files = _exadem_shape_files()
    assert len(files) >= 10
    nshapes = 0
    for f in files:
        R, M = U.read_shps_ref(ref, f), shp.read_shps(f)
        assert len(R) == len(M), f
        for r, m in zip(R, M):
            nshapes += 1
            assert r["name"] == m["name"], f
            assert r["faces"] == m["faces"], f
            assert np.array_equal(r["edges"], m["edges"]), f
            for k in ("vertices", "radius", "volume", "i_over_m"):
                assert same_bits(np.atleast_2d(r[k]), np.atleast_2d(m[k])).all(), (f, k)
            for k in ("center", "e1", "e2", "e3", "extent"):
                assert same_bits(np.atleast_2d(r["obb"][k]), np.atleast_2d(m["obb"][k])).all(), (f, "obb", k)
            # the quantities set_fields takes from the shape (radius, mass and inertia of a polyhedron)
            ref.ref_shape_derived.argtypes = [C.c_int, C.c_double, C.POINTER(C.c_double)]
            for h in (1.0, 0.8, 1.3):
                d = np.zeros(5)
                ref.ref_shape_derived(r["index"], h, d.ctypes.data_as(C.POINTER(C.c_double)))
                iom = m["i_over_m"]
                mine = np.array([m["max_rcut"], h * h * h * m["volume"], h * h * iom[0], h * h * iom[1], h * h * iom[2]])
                assert same_bits(d[None], mine[None]).all(), (f, h)
            # the face areas (compute_face_areas; the criterion area of stick_polyhedra)
            if all(len(fc) >= 3 for fc in m["faces"]):
                assert same_bits(U.face_areas_ref(ref, r["index"], len(m["faces"])),
                                 U.face_areas_oracle(orc_lib, m)).all(), f
    assert nshapes >= 40


@pytest.mark.parametrize("length,mink", [(1.0, 0.01), (0.98, 0.01), (0.25, 1e-4), (2.5, 0.2)])
def test_add_cube_shape(libs, length, mink):
    """workloads.exadem_cube against exaDEM's create_cube (add_cube): vertices,
    edges, faces, volume, inertia over mass and shape OBB, bit for bit."""
    from exadem_gb300 import workloads as W

    ref, orc_lib = libs
    idx = C.c_int()
    ref.ref_create_cube.argtypes = [C.c_double, C.c_double, C.POINTER(C.c_int)]
    assert ref.ref_create_cube(length, mink, C.byref(idx)) == 0
    r, m = U._ref_shape(ref, idx.value), W.exadem_cube("cube", length, mink)
    assert r["faces"] == m["faces"] and np.array_equal(r["edges"], np.asarray(m["edges"]))
    for k in ("vertices", "radius", "volume", "i_over_m"):
        assert same_bits(np.atleast_2d(r[k]), np.atleast_2d(np.asarray(m[k], dtype=np.float64))).all(), k
    for k in ("center", "e1", "e2", "e3", "extent"):
        assert same_bits(np.atleast_2d(r["obb"][k]), np.atleast_2d(np.asarray(m["obb"][k]))).all(), ("obb", k)
    assert same_bits(U.face_areas_ref(ref, idx.value, 6), U.face_areas_oracle(orc_lib, m)).all()


def _shape_files(tmp_path):
    from exadem_gb300 import shp, workloads as W

    out = []
    for s in (W.shape_cube(), W.shape_tetrahedron(), W.shape_octahedron()):
        p = tmp_path / f"{s['name']}.shp"
        p.write_text(shp.format_shp(s))
        out.append(str(p))
    return out + [f for f in _exadem_shape_files() if os.path.getsize(f) < 20_000]


def test_vertex_face(libs, tmp_path):
    """filter_vertex_face and detection_vertex_face_core on every face of the bench
    shapes and of exaDEM's example shapes: points inside, on edges, at vertices, above
    and below the face plane, homothety 0.8-1.2."""
    from exadem_gb300 import shp

    ref, orc = libs
    hits = total = 0
    for f in _shape_files(tmp_path):
        for R, M in zip(U.read_shps_ref(ref, f), shp.read_shps(f)):
            for face in range(len(M["faces"])):
                x = U.vertex_face_cases(M, face, 2000, 1000 + face)
                a = U.run_vertex_face_ref(ref, R["index"], face, len(M["vertices"]), x)
                b = U.run_vertex_face_oracle(orc, M, face, x)
                check(f"vertex_face {os.path.basename(f)}:{M['name']} face {face}", x, a, b)
                hits += int(a[:, 0].sum())
                total += len(x)
    assert total > 100_000 and 0.1 < hits / total < 0.9
