"""The .msp deck reader (exadem_gb300/msp.py) on exaDEM's own decks (CPU).

Every deck of the exaDEM tree parses; three example decks (a rotating drum of
spheres, a DMT polyhedron deposition on a wall, octahedra in an STL box) are
read unchanged, give the workloads committed under tests/golden/ (which the GPU
tests run), and step on the oracle.  Skipped where the exaDEM sources are absent,
except the fixture checks, which need no sources.
"""
from __future__ import annotations

import glob
import os
from pathlib import Path

import numpy as np
import pytest

from exadem_gb300 import msp
from exadem_gb300.workloads import load_workload

HERE = Path(__file__).resolve().parent
EXADEM = Path(os.environ.get("EXADEM_SRC", "/root/reference"))
needs_src = pytest.mark.skipif(not (EXADEM / "data" / "config").exists(), reason="exaDEM sources not present")
KEYS = ["rotating_drum_spheres", "polyhedra_spread_dmt", "polyhedra_stl_box"]


@needs_src
def test_every_exadem_deck_parses():
    files = glob.glob(str(EXADEM / "**" / "*.msp"), recursive=True)
    assert len(files) > 100
    for f in files:
        msp.parse_yaml(Path(f).read_text())


@needs_src
def test_drum_deck_resolves():
    d = msp.load_deck(EXADEM / "example/spheres/rotating-drum/rotating-drum-mini.msp", [EXADEM / "data/config"])
    assert d["global"]["dt"] == 1e-4 and d["global"]["rcut_inc"] == 0.4
    assert d["domain"]["periodic"] == [False, True, False]
    names = [next(iter(x)) if isinstance(x, dict) else x for x in d["compute_force"]]
    assert names == ["gravity_force", "contact_sphere"]  # +compute_force appended to the common deck's
    assert "simulation" in d and "compute_loop" in d     # main-config.msp read first


@needs_src
@pytest.mark.parametrize("key", KEYS)
def test_deck_gives_committed_workload(key):
    """Reading the deck now gives the fixture the GPU tests run."""
    import importlib.util

    spec = importlib.util.spec_from_file_location("mk", HERE / "golden" / "make_deck_fixtures.py")
    mk = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mk)
    a, b = mk.deck_workload(key), load_workload(HERE / "golden" / f"deck_{key}.npz")
    assert a.n == b.n and a.steps == b.steps
    for k in a.particles:
        assert np.array_equal(np.asarray(a.particles[k]), np.asarray(b.particles[k])), k
    assert bytes(a.params) == bytes(b.params)
    assert a.surfaces == b.surfaces and a.cylinders == b.cylinders
    assert len(a.meshes) == len(b.meshes)


def test_yaml_subset():
    doc = msp.parse_yaml("""
a: 1
b: 2.5 m   # a quantity with a unit
c: [1, [2, 3], {x: 1 s, y: true}]
d:
  - op1
  - op2: {k: v}
  - op3:
     p: 1
     q: [a,
         b]
e: |
  text line
f:
  g: null
+h: [9]
""")
    assert doc["a"] == 1 and doc["b"] == 2.5
    assert doc["c"] == [1, [2, 3], {"x": 1.0, "y": True}]
    assert doc["d"] == ["op1", {"op2": {"k": "v"}}, {"op3": {"p": 1, "q": ["a", "b"]}}]
    assert doc["e"].strip() == "text line" and doc["f"] == {"g": None} and doc["+h"] == [9]


@pytest.mark.parametrize("key", KEYS)
def test_fixture_steps_on_oracle(key):
    from oracle.oracle import oracle_system

    w = load_workload(HERE / "golden" / f"deck_{key}.npz")
    o = w.build(oracle_system)
    o.first_iteration()
    o.step(300)
    p = o.particles()
    assert all(np.isfinite(p[k]).all() for k in ("rx", "ry", "rz", "vx", "vy", "vz"))
    o.close()


@needs_src
@pytest.mark.parametrize("test,g", [("traction", 1e-2), ("shear", 5e-3)])
def test_fragmentation_verification_deck(tmp_path, test, g):
    """exaDEM's bonded-cube verification decks (traction and shear of two cubes
    made by add_cube, stuck by stick_polyhedra): the deck gives the cube of
    create_cube and, through inner_bond_params and apply_particle_sticking, four
    bonds with the criterion 2 A g of the 0.98 x 0.98 face.  The decks' imposed
    motion (pas_libere_pas_delivre, set_velocity in compute_force) is reported
    as ignored."""
    from oracle.oracle import oracle_system

    src = EXADEM / "example/polyhedra/fragmentation/verification_test" / test / f"{test}.msp"
    text = src.read_text().replace("GC", repr(g))  # the value its run script substitutes
    p = tmp_path / f"{test}.msp"
    p.write_text(text)
    w = msp.deck_workload(msp.load_deck(p, [EXADEM / "data/config"]), base_dir=src.parent)
    assert w.n == 2 and w.shapes[0]["name"] == "cube" and w.bonds is not None
    assert any("pas_libere_pas_delivre" in x for x in w.info["notes"])
    s = w.build(oracle_system)
    b = s.bonds()
    assert s.bond_count() == 4 and np.all(b["weight"] == 0.25)
    face = 0.98 * 0.98
    assert np.allclose(b["crit1"], 2 * face * g, rtol=1e-14, atol=0)
    # (the decks' domain is periodic in y, which the polyhedron path does not run)
