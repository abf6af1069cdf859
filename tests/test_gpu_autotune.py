"""dem_autotune changes launch shapes, the cell size and (where it cannot
change a bit) the skin: the tuned run equals the untuned one bit for bit."""
import numpy as np
import pytest

from exadem_gb300 import workloads as W
from tests.helpers import assert_same_list, bit_equal_fraction

pytestmark = pytest.mark.gpu

FUSED = dict(fused_step=1, fp32_contact_screen=1, fp32_broad_phase=1)


@pytest.mark.parametrize("make", [
    lambda: W.spheres_box(n=4000, box=22.0, seed=8, **FUSED),      # walls only: the skin may be tuned
    lambda: W.spheres_drum(n=4000, seed=8, **FUSED),                # periodic axis: skin kept (policy 1)
])
def test_autotuned_run_equals_untuned(native_lib, make):
    a, b = make().build(), make().build()
    for s in (a, b):
        s.first_iteration()
        s.step(20)
    r = b.autotune(steps_per_trial=3, skin_policy=1)
    assert r["trials"] >= 10 and r["ms_per_step"] <= r["ms_per_step_before"] * 1.0001
    for s in (a, b):
        s.step(300)
    assert bit_equal_fraction(a.particles(), b.particles()) == 1.0
    la, lb = a.interactions(), b.interactions()
    contact = lambda l: {k: v[np.any(l["friction"].reshape(-1, 3) != 0, axis=1)] for k, v in l.items()}
    assert_same_list(contact(la), contact(lb))  # the listed non-touching pairs may differ with the skin


def test_autotune_keeps_skin_with_cohesion(native_lib):
    w = W.spheres_floor(n=4000, side=20.0, **FUSED)
    s = w.build()
    s.first_iteration()
    r = s.autotune(steps_per_trial=2, skin_policy=2)
    assert r["rcut_inc"] == w.params.rcut_inc
