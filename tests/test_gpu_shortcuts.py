"""Exact shortcuts of the fused integration, compared bit for bit (including
the sign of zeros) with the oracle, which runs the plain formulas:
- spin-free quaternion step (signed-zero derivative decided from the signs of
  Q) and the unit-norm normalisation, over every sign pattern of zero and
  nonzero quaternion components, with norm^2 equal to 1 and not;
- the idle rotation (no spin, no torque: arot = w = +0) next to rotating and
  touching particles;
- skipped all-zero contact records in the force gather."""
import copy
import itertools

import numpy as np
import pytest

from exadem_gb300 import workloads as W
from tests.helpers import assert_same_list, pair

pytestmark = pytest.mark.gpu

QFIELDS = ("qw", "qx", "qy", "qz")
STATE = ("rx", "ry", "rz", "vx", "vy", "vz", "vrotx", "vroty", "vrotz", "arotx", "aroty", "arotz", "qw", "qx",
         "qy", "qz", "momx", "momy", "momz", "fx", "fy", "fz")


def _bits_equal(a: dict, b: dict, fields=STATE) -> None:
    for f in fields:
        x, y = np.ascontiguousarray(a[f]).view(np.uint64), np.ascontiguousarray(b[f]).view(np.uint64)
        bad = np.nonzero(x != y)[0]
        assert bad.size == 0, f"{f}: {bad.size} values differ in their bits, first at {bad[:4]}"


def _quaternion_cases():
    vals = (0.0, -0.0, 0.5, -0.5, 1.0, -1.0)
    cases = [q for q in itertools.product(vals, repeat=4) if any(abs(c) > 0 for c in q)]
    return np.array(cases, dtype=np.float64)  # 1295 quaternions, many with norm^2 exactly 1


@pytest.mark.parametrize("mode", [0, 1, 3])
def test_spin_free_quaternions_bit_exact(native_lib, mode):
    q = _quaternion_cases()
    n = len(q)
    w = W.spheres_box(n=n, box=60.0, seed=3, fused_step=1, fp32_contact_screen=1, fp32_broad_phase=1)
    # spread on a lattice, far apart: no contacts, no torque, no spin
    side = int(np.ceil(n ** (1 / 3)))
    idx = np.arange(n)
    w.particles["rx"] = 2.0 + 3.0 * (idx % side)
    w.particles["ry"] = 2.0 + 3.0 * ((idx // side) % side)
    w.particles["rz"] = 20.0 + 3.0 * (idx // (side * side))
    for k, f in enumerate(QFIELDS):
        w.particles[f] = q[:, k].copy()
    for f in ("vrotx", "vroty", "vrotz"):
        w.particles[f] = np.zeros(n)
    g, o = pair(w)
    g.set_mul_mode(mode)
    for s in (g, o):
        s.first_iteration()
        s.step(6)
    pg, po = g.particles(sort_by_id=True), o.particles(sort_by_id=True)
    _bits_equal(pg, po)
    # the cases really hold signed zeros after the step
    assert np.any(np.signbit(pg["qx"]) & (pg["qx"] == 0))


@pytest.mark.parametrize("mode", [0, 1])
def test_signed_zero_velocities_bit_exact(native_lib, mode):
    """Zero-aware translation and velocity updates: velocity components drawn
    from {+0, -0, 0.3, -0.3}, gravity (-0, +0, -9.81), no contacts."""
    vals = np.array([0.0, -0.0, 0.3, -0.3])
    combos = np.array(list(itertools.product(range(4), repeat=3)))
    n = len(combos) * 4
    w = W.spheres_box(n=n, box=60.0, seed=4, fused_step=1, fp32_contact_screen=1, fp32_broad_phase=1)
    side = int(np.ceil(n ** (1 / 3)))
    idx = np.arange(n)
    w.particles["rx"] = 4.0 + 3.0 * (idx % side)
    w.particles["ry"] = 4.0 + 3.0 * ((idx // side) % side)
    w.particles["rz"] = 20.0 + 3.0 * (idx // (side * side))
    c = np.tile(combos, (4, 1))
    for k, f in enumerate(("vx", "vy", "vz")):
        w.particles[f] = vals[c[:, k]].copy()
    for f in ("vrotx", "vroty", "vrotz"):
        w.particles[f] = np.zeros(n)
    w.params.gravity[0] = -0.0
    w.params.gravity[1] = 0.0
    g, o = pair(w)
    g.set_mul_mode(mode)
    for s in (g, o):
        s.first_iteration()
        s.step(5)
    _bits_equal(g.particles(sort_by_id=True), o.particles(sort_by_id=True))


@pytest.mark.parametrize("mode", [0, 1])
def test_idle_and_rotating_mix_bit_exact(native_lib, mode):
    """A settling box: some particles touch (torque), some spin freely, the rest
    are idle; zero records of listed but separated pairs are skipped."""
    w = W.spheres_box(n=2000, box=16.0, seed=5, fused_step=1, fp32_contact_screen=1, fp32_broad_phase=1)
    rng = np.random.default_rng(5)
    spin = rng.random(w.n) < 0.2
    for f in ("vrotx", "vroty", "vrotz"):
        w.particles[f] = np.where(spin, rng.uniform(-3, 3, w.n), 0.0)
    g, o = pair(w)
    g.set_mul_mode(mode)
    for s in (g, o):
        s.first_iteration()
        s.step(150)
    pg, po = g.particles(sort_by_id=True), o.particles(sort_by_id=True)
    _bits_equal(pg, po)
    assert_same_list(g.interactions(), o.interactions())
    idle = np.ones(w.n, dtype=bool)
    for f in ("vrotx", "vroty", "vrotz", "momx", "momy", "momz"):
        idle &= pg[f].view(np.uint64) == 0
    assert 0 < idle.sum() < w.n


@pytest.mark.parametrize("graph", [0, 1])
def test_pair_damping_follows_parameter_change(native_lib, graph):
    """The per-pair damping cached in the list is refreshed when the contact
    parameters change without a rebuild (the oracle computes it per contact)."""
    w = W.spheres_drum(n=3000, seed=51, fused_step=1, fp32_contact_screen=1, fp32_broad_phase=1, graph_step=graph)
    g, o = pair(w)
    for s in (g, o):
        s.first_iteration()
        s.step(80)
    p2 = copy.deepcopy(w.params)
    p2.config.kn = 2.0e4
    p2.config.damp_rate = 0.5
    p2.config_driver.kn = 1.5e4
    for s in (g, o):
        s.set_params(p2)
        s.step(80)
    _bits_equal(g.particles(sort_by_id=True), o.particles(sort_by_id=True))
    assert_same_list(g.interactions(), o.interactions())


def test_live_flags_across_plain_and_fused_steps(native_lib):
    """Records written by the plain contact kernel (which does not keep the live
    flags) are read again by the fused step's gather: switching the path between
    steps keeps the oracle's bits."""
    w = W.spheres_floor(n=4000, side=14.0, seed=61, fused_step=1, fp32_contact_screen=1, fp32_broad_phase=1)
    g, o = pair(w)
    for s in (g, o):
        s.first_iteration()
        s.step(60)
    plain = copy.deepcopy(w.params)
    plain.fused_step = 0
    plain.fp32_contact_screen = 0
    g.set_params(plain)
    g.step(30)
    g.set_params(w.params)
    g.step(60)
    o.step(90)
    _bits_equal(g.particles(sort_by_id=True), o.particles(sort_by_id=True))
    assert_same_list(g.interactions(), o.interactions())
