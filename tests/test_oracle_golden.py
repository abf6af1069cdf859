"""The oracle against exaDEM's outputs stored in tests/golden/ref_units.npz (CPU).

The vectors were produced by exaDEM's own functions (tests/golden/make_ref_vectors.py,
exaDEM's headers compiled on the host), so this pins the oracle wherever the
exaDEM sources are absent.  Every output double must match bit for bit.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np
import pytest

from oracle import build as oracle_build
from oracle import units as U

GOLDEN = Path(__file__).resolve().parent / "golden" / "ref_units.npz"


@pytest.fixture(scope="module")
def data():
    return np.load(GOLDEN)


@pytest.fixture(scope="module")
def orc():
    return C.CDLL(str(oracle_build.build()))


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.uint64)


def test_units_match_exadem(data, orc):
    checked = 0
    for name in U.LAYOUT:
        for law in ([0, 1, 2] if name == "contact_force_core" else [0]):
            x, want = data[f"{name}/{law}/in"], data[f"{name}/{law}/out"]
            got = U.run(orc, "oracle", name, x, law)
            assert np.array_equal(bits(got), bits(want)), f"{name} law {law}"
            checked += len(x)
    k = data["pair_order/in"]
    assert np.array_equal(U.run_pair_order(orc, "oracle", k), data["pair_order/out"])
    assert checked >= 2000


@pytest.mark.parametrize("name", ["Cube", "Tetrahedron", "Octahedron"])
def test_shapes_and_vertex_face_match_exadem(data, orc, name):
    """The .shp reader and the shape OBB against read_shp; the vertex-face filter and
    detection of the oracle against exaDEM's on every face."""
    from exadem_gb300 import shp

    tag = f"shape/{name}"
    s = shp.parse_shps(data[f"{tag}/text"].tobytes().decode())[0]
    assert np.array_equal(bits(s["vertices"]), bits(data[f"{tag}/vertices"]))
    obb = np.concatenate([np.asarray(s["obb"][k], dtype=np.float64) for k in ("center", "e1", "e2", "e3", "extent")])
    assert np.array_equal(bits(obb), bits(data[f"{tag}/obb"]))
    assert np.array_equal(bits(U.face_areas_oracle(orc, s)), bits(data[f"{tag}/face_areas"]))
    for face in range(len(s["faces"])):
        x = data[f"{tag}/vf{face}/in"]
        got = U.run_vertex_face_oracle(orc, s, face, x)
        assert np.array_equal(bits(got), bits(data[f"{tag}/vf{face}/out"])), face
