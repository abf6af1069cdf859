"""Contact parameters changed in the middle of a run (dem_set_params,
dem_set_multimat) on the fused sphere step, against the oracle: the list's
per-pair damping follows the new parameters, both for the pairs kept at the
next rebuild and for the list in place, and every bit matches."""
import numpy as np
import pytest

from exadem_gb300 import system as S
from exadem_gb300 import workloads as W
from tests.helpers import assert_same_list, bit_equal_fraction, pair

pytestmark = pytest.mark.gpu

FAST = dict(fused_step=1, fp32_contact_screen=1, fp32_broad_phase=1)


@pytest.mark.parametrize("graph", [0, 1])
def test_set_params_mid_run(native_lib, graph):
    w = W.spheres_drum(n=3000, seed=61, graph_step=graph, **FAST)
    g, o = pair(w)
    for s in (g, o):
        s.first_iteration()
        s.step(120)
    p = w.params
    p.config = S.contact_params(kn=2.5e4, kt=2e4, mu=0.35, damp_rate=0.6)
    p.config_driver = S.contact_params(kn=3e4, kt=2.4e4, mu=0.4, damp_rate=0.7)
    for s in (g, o):
        s.set_params(p)
        s.step(150)
    assert g.rebuild_count() == o.rebuild_count() and g.rebuild_count() > 2
    assert_same_list(g.interactions(), o.interactions())
    assert bit_equal_fraction(g.particles(sort_by_id=True), o.particles(sort_by_id=True)) == 1.0


def test_set_multimat_mid_run(native_lib):
    w = W.spheres_drum(n=3000, seed=62, **FAST)
    w.particles["group"] = np.random.default_rng(62).integers(0, 2, w.n).astype(np.uint32)
    g, o = pair(w)
    for s in (g, o):
        s.first_iteration()
        s.step(100)
    a = S.contact_params(kn=1.5e4, kt=1.2e4, mu=0.3, damp_rate=0.5)
    b = S.contact_params(kn=3e4, kt=2.4e4, mu=0.45, damp_rate=0.8)
    d = S.contact_params(kn=2e4, kt=1.6e4, mu=0.4, damp_rate=0.9)
    for s in (g, o):
        s.set_multimat([[a, b], [b, a]], [[d], [d]])
        s.step(150)
    assert g.rebuild_count() == o.rebuild_count() and g.rebuild_count() > 2
    assert_same_list(g.interactions(), o.interactions())
    assert bit_equal_fraction(g.particles(sort_by_id=True), o.particles(sort_by_id=True)) == 1.0
