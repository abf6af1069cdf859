"""The .shp reader (exadem_gb300/shp.py) on written shapes and malformed files (CPU)."""
from __future__ import annotations

import numpy as np
import pytest

from exadem_gb300 import shp, workloads as W


@pytest.mark.parametrize("make", [W.shape_cube, W.shape_tetrahedron, W.shape_octahedron])
def test_round_trip(make):
    s = make()
    r = shp.parse_shps(shp.format_shp(s))[0]
    assert r["name"] == s["name"]
    np.testing.assert_array_equal(r["vertices"], s["vertices"])
    np.testing.assert_array_equal(r["edges"], s["edges"])
    assert r["faces"] == s["faces"] and r["radius"] == s["radius"] and r["volume"] == s["volume"]
    assert r["obb"] == s["obb"]


def test_several_shapes_and_ignored_keys():
    text = ("junk line\n<\nname A\nradius 0.1\npreCompDone y\nnv 1\n0 0 0\nne 0\nnf 0\n"
            "obb.extent 1 2 3\nposition 4 5 6\norientation 1 0 0 0\nvolume 2\nI/m 1 2 3\n>\n"
            "<\nname B\nradius 0.2\npreCompDone y\nnv 2\n0 0 0\n1 0 0 extra\nne 1\n0 1\nnf 0\nvolume 1\nI/m 1 1 1\n>\n")
    a, b = shp.parse_shps(text)
    assert a["name"] == "A" and a["i_over_m"] == (1.0, 2.0, 3.0) and a["volume"] == 2.0
    assert b["name"] == "B" and len(b["vertices"]) == 2 and b["edges"].tolist() == [[0, 1]]


@pytest.mark.parametrize("text,msg", [
    ("<\nname A\npreCompDone n\n>\n", "preCompDone"),
    ("<\nname A\nradius 0.1\npreCompDone y\nnv 1\n0 0 0\n", "end of file"),
    ("<\nname A\npreCompDone y\nnv 1\n0 0 0\nne 1\n0 3\n>\n", "missing vertex"),
    ("<\nname A\npreCompDone y\nnv 1\n0 0 x\n>\n", "bad value"),
    ("<\nname A\npreCompDone y\n>\n", "no vertices"),
])
def test_malformed(text, msg):
    with pytest.raises(ValueError, match=msg):
        shp.parse_shps(text)
