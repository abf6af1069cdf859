"""exaDEM example decks on the GPU against the oracle (GPU).

The workloads are those the deck reader gives for three unchanged exaDEM decks
(tests/golden/deck_*.npz, see tests/test_decks.py): a rotating drum of 250
spheres, 512 octahedra falling on a wall with the DMT law, 27 octahedra in an
STL box mesh.  Each runs through the C ABI on the plain and on the fused path
for several thousand steps, until contacts have formed, and must keep the
interaction list bit-exact and the state within 1e-9 of the oracle.
"""
from pathlib import Path

import numpy as np
import pytest

from exadem_gb300.workloads import load_workload
from tests.helpers import ENERGY_RTOL, assert_close_rel, assert_same_list, assert_state

pytestmark = pytest.mark.gpu
HERE = Path(__file__).resolve().parent
STEPS = {"rotating_drum_spheres": 14000, "polyhedra_spread_dmt": 12000, "polyhedra_stl_box": 8000}


@pytest.mark.parametrize("fast", [0, 1], ids=["plain", "fused"])
@pytest.mark.parametrize("key", list(STEPS))
def test_deck(native_lib, key, fast):
    from oracle.oracle import oracle_system

    w = load_workload(HERE / "golden" / f"deck_{key}.npz")
    w.params.fused_step = w.params.fp32_broad_phase = w.params.fp32_contact_screen = fast
    g, o = w.build(), w.build(oracle_system)
    g.first_iteration()
    o.first_iteration()
    done = 0
    for chunk in (STEPS[key] // 4,) * 4:
        g.step(chunk)
        o.step(chunk)
        done += chunk
        assert_same_list(g.interactions(), o.interactions())
        assert_state(g.particles(), o.particles(), ENERGY_RTOL)
    sg, so = g.simulation_state(), o.simulation_state()
    assert_close_rel(sg["kinetic_energy"], so["kinetic_energy"], ENERGY_RTOL, "kinetic_energy")
    assert g.rebuild_count() == o.rebuild_count()
    assert sg["n_active_interactions"] > 0, "the deck's particles reached contact"
    g.close()
    o.close()
