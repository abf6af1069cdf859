"""Multiply placement of the fused integration kernels (dem_set_mul_mode): every
mode puts a different share of the FP64 multiplies on the integer pipe, and
every mode gives the same bits, on workloads where every particle spins and
collides: a rotating drum of spheres and a spinning polyhedron lattice."""
import numpy as np
import pytest

from exadem_gb300 import workloads as W
from tests.helpers import assert_same_list, assert_state, bit_equal_fraction, pair

pytestmark = pytest.mark.gpu


def _run(w, mode, steps):
    s = w.build()
    s.set_mul_mode(mode)
    assert s.mul_mode() == mode
    s.first_iteration()
    s.step(steps)
    return s


def test_mul_modes_same_bits_drum(native_lib):
    w = W.spheres_drum(n=4000, seed=31, fused_step=1, fp32_contact_screen=1, fp32_broad_phase=1)
    rng = np.random.default_rng(31)
    for k in ("vrotx", "vroty", "vrotz"):
        w.particles[k] = rng.uniform(-5.0, 5.0, w.n)
    runs = [_run(w, m, 300) for m in (0, 1, 2, 3, 4, 7)]
    ref = runs[0].particles(sort_by_id=True)
    assert np.abs(ref["vrotx"]).max() > 0
    for s in runs[1:]:
        assert bit_equal_fraction(s.particles(sort_by_id=True), ref) == 1.0
        assert_same_list(s.interactions(), runs[0].interactions())


def test_mul_modes_same_bits_spinning_polyhedra(native_lib):
    w = W.polyhedra_lattice(nx=6, ny=6, nz=4, seed=23, fused_step=1, fp32_broad_phase=1, fp32_contact_screen=1)
    rng = np.random.default_rng(23)
    for k in ("vrotx", "vroty", "vrotz"):
        w.particles[k] = rng.uniform(-30.0, 30.0, w.n)
    runs = [_run(w, m, 120) for m in range(4)]
    ref = runs[0].particles(sort_by_id=True)
    for s in runs[1:]:
        assert bit_equal_fraction(s.particles(sort_by_id=True), ref) == 1.0
        assert s.rebuild_count() == runs[0].rebuild_count()


@pytest.mark.parametrize("case", ["drum", "cohesive_floor"])
def test_mul_mode_integer_pipe_matches_oracle(native_lib, case):
    """Every placement on the integer pipe (mode 7: integration and contact law)
    against the oracle, for the plain Hooke law (a drum) and the cohesive one."""
    flags = dict(fused_step=1, fp32_contact_screen=1, fp32_broad_phase=1)
    if case == "drum":
        w = W.spheres_drum(n=3000, seed=41, **flags)
    else:
        w = W.spheres_floor(n=4000, side=14.0, seed=41, **flags)
    g, o = pair(w)
    g.set_mul_mode(7)
    for s in (g, o):
        s.first_iteration()
        s.step(200)
    assert_same_list(g.interactions(), o.interactions())
    assert_state(g.particles(sort_by_id=True), o.particles(sort_by_id=True), 1e-12)
    assert bit_equal_fraction(g.particles(sort_by_id=True), o.particles(sort_by_id=True)) == 1.0


def test_mul_mode_validation(native_lib):
    s = W.spheres_box(n=200).build()
    from exadem_gb300 import _abi as A

    with pytest.raises(A.DemError):
        s.set_mul_mode(8)


@pytest.mark.parametrize("share", [3, 8])
@pytest.mark.parametrize("case", ["drum", "cohesive_floor", "dmt_floor"])
def test_contact_int_share_matches_oracle(native_lib, case, share):
    """A share of the fused contact kernel's Hooke tiles (or all of them) with
    the law's multiplies and additions on the integer pipe: the same bits as
    the oracle, for the plain Hooke law (a drum), the cohesive law on a periodic
    floor and the DMT law."""
    from exadem_gb300 import _abi as A

    flags = dict(fused_step=1, fp32_contact_screen=1, fp32_broad_phase=1)
    if case == "drum":
        w = W.spheres_drum(n=3000, seed=43, **flags)
    elif case == "cohesive_floor":
        w = W.spheres_floor(n=4000, side=14.0, seed=43, **flags)
    else:
        w = W.spheres_floor(n=4000, side=14.0, seed=43, **flags)
        w.params.law = A.LAW_HOOKE_DMT
        for cfg in (w.params.config, w.params.config_driver):
            cfg.gamma, cfg.fc, cfg.dncut = 0.5, 0.0, 0.0
    g, o = pair(w)
    g.set_contact_int_share(share)
    for s in (g, o):
        s.first_iteration()
        s.step(200)
    assert g.simulation_state()["n_active_interactions"] > 0
    assert_same_list(g.interactions(), o.interactions())
    lg, lo = g.interactions(), o.interactions()
    assert np.array_equal(lg["friction"].view(np.uint64), lo["friction"].view(np.uint64))
    assert bit_equal_fraction(g.particles(sort_by_id=True), o.particles(sort_by_id=True)) == 1.0
    with pytest.raises(A.DemError):
        g.set_contact_int_share(9)
