"""Generates tests/golden/deck_*.npz: the workloads exaDEM example decks describe,
as read by this project's deck reader (test fixture generator).

Each deck is read unchanged from the exaDEM source tree with
exadem_gb300.msp.load_deck (includes resolved against exaDEM's data/config)
and converted by deck_workload; the resulting particles, parameters, drivers,
shapes and meshes are saved with workloads.save_workload.  The GPU tests run
these fixtures (the exaDEM tree is not available where they run);
tests/test_decks.py re-reads the decks and checks they still give the same
workloads.

    python tests/golden/make_deck_fixtures.py
"""
from __future__ import annotations

import os
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

EXADEM = Path(os.environ.get("EXADEM_SRC", "/root/reference"))
DECKS = {
    "rotating_drum_spheres": "example/spheres/rotating-drum/rotating-drum-mini.msp",
    "polyhedra_spread_dmt": "example/polyhedra/rigid_surface/rigid_surface_spread_DMT.msp",
    "polyhedra_stl_box": "example/polyhedra/stl_mesh/stl_mesh_box_octahedron_mini.msp",
}
HERE = Path(__file__).resolve().parent


def deck_workload(key: str):
    from exadem_gb300 import msp

    path = EXADEM / DECKS[key]
    deck = msp.load_deck(path, [EXADEM / "data" / "config"])
    return msp.deck_workload(deck, base_dir=path.parent, seed=1)


def main() -> None:
    from exadem_gb300.workloads import save_workload

    if not (EXADEM / DECKS["rotating_drum_spheres"]).exists():
        raise SystemExit("exaDEM sources not found (set EXADEM_SRC)")
    for key in DECKS:
        w = deck_workload(key)
        out = HERE / f"deck_{key}.npz"
        save_workload(w, out)
        print(f"{out.name}: {w.n} particles, {out.stat().st_size} bytes")


if __name__ == "__main__":
    main()
