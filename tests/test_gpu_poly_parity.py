"""GPU parity of the sphero-polyhedron path (VV, VE, VF, EE and vertex-wall
interactions) against the CPU oracle on seeded inputs: interaction list
(owner id, partner id, type, swap, subs) bit-exact after every rebuild, forces
within 1e-12, state after 100 steps within 1e-12 (the FP64 order is kept, so
values are expected to be identical)."""
import numpy as np
import pytest

from exadem_gb300 import workloads as W
from tests.helpers import assert_forces, assert_same_list, assert_state, bit_equal_fraction, pair

pytestmark = pytest.mark.gpu


def test_lattice_first_iteration(native_lib):
    w = W.polyhedra_lattice()
    g, o = pair(w)
    g.first_iteration()
    o.first_iteration()
    lg, lo = g.interactions(), o.interactions()
    assert_same_list(lg, lo)
    assert set(np.unique(lg["type"])) >= {1, 2, 3}
    assert lg["swap"].sum() > 0
    pg, po = g.particles(), o.particles()
    assert_forces(pg, po)
    assert bit_equal_fraction(pg, po, ["fx", "fy", "fz", "momx", "momy", "momz"]) == 1.0


@pytest.mark.parametrize("flags", [{}, dict(fused_step=1, fp32_broad_phase=1, fp32_contact_screen=1)])
def test_lattice_100_steps(native_lib, flags):
    w = W.polyhedra_lattice(seed=11, **flags)
    g, o = pair(w)
    for s in (g, o):
        s.first_iteration()
        s.step(100)
    assert g.rebuild_count() == o.rebuild_count()
    lg, lo = g.interactions(), o.interactions()
    assert_same_list(lg, lo)
    np.testing.assert_array_equal(lg["friction"], lo["friction"])
    assert_state(g.particles(), o.particles(), 1e-12)
    assert g.simulation_state()["n_active_interactions"] == o.simulation_state()["n_active_interactions"]


def test_spinning_lattice_rebuild_steps(native_lib):
    """Fast rotation (vertex speeds ~25 m/s, max_displ reached every ~10 steps):
    the FP32-decided vertex_displ_over of the fused step rebuilds on the same
    steps as the oracle, and the state stays on the oracle's."""
    w = W.polyhedra_lattice(nx=8, ny=8, nz=4, seed=21, fused_step=1, fp32_broad_phase=1, fp32_contact_screen=1)
    rng = np.random.default_rng(21)
    n = w.n
    for k in ("vrotx", "vroty", "vrotz"):
        w.particles[k] = rng.uniform(-30.0, 30.0, n)
    g, o = pair(w)
    for s in (g, o):
        s.first_iteration()
    for _ in range(6):
        for s in (g, o):
            s.step(10)
        assert g.rebuild_count() == o.rebuild_count()
        assert_same_list(g.interactions(), o.interactions())
    assert g.rebuild_count() >= 4
    assert_state(g.particles(), o.particles(), 1e-12)


def test_floor_deposition(native_lib):
    """Config 3 physics on a small column: polyhedra falling onto a floor between walls."""
    w = W.polyhedra_floor(n=2400, side=12.0)
    g, o = pair(w)
    for s in (g, o):
        s.first_iteration()
        s.step(300)
    assert_same_list(g.interactions(), o.interactions())
    assert_state(g.particles(), o.particles(), 1e-12)


def test_forced_rebuilds_keep_history(native_lib):
    w = W.polyhedra_lattice(nx=10, ny=10, nz=5, seed=3)
    g, o = pair(w)
    for s in (g, o):
        s.first_iteration()
    for _ in range(3):
        for s in (g, o):
            s.step(20)
            s.update_particle_neighbors()
        lg, lo = g.interactions(), o.interactions()
        assert_same_list(lg, lo)
        np.testing.assert_array_equal(lg["friction"], lo["friction"])
        np.testing.assert_array_equal(lg["moment"], lo["moment"])


@pytest.mark.parametrize("seed", [5, 6])
def test_fp32_prefilters_same_list(native_lib, seed):
    """FP32 rejection tests (vertex gates and feature bounding spheres) keep exactly the FP64 list."""
    a = W.polyhedra_lattice(nx=9, ny=9, nz=6, seed=seed).build()
    b = W.polyhedra_lattice(nx=9, ny=9, nz=6, seed=seed, fp32_broad_phase=1, fused_step=1).build()
    for s in (a, b):
        s.first_iteration()
    assert_same_list(a.interactions(), b.interactions())
    for _ in range(3):
        for s in (a, b):
            s.step(30)
            s.update_particle_neighbors()
        assert_same_list(a.interactions(), b.interactions())
    assert bit_equal_fraction(a.particles(), b.particles()) == 1.0


@pytest.mark.parametrize("distort", [False, True])
def test_fp32_broad_phase_same_list_large(native_lib, distort):
    """64k polyhedra: the FP32-decided, slab-gated enumeration writes the FP64 list.
    distort: homothety in [0.8, 1.2] and quaternions 2 % off unit norm (qrotate is
    then not a rotation), which the per-particle vertex slabs must still bound."""
    w = [W.polyhedra_lattice(nx=40, ny=40, nz=40, seed=11, **f) for f in ({}, dict(fp32_broad_phase=1))]
    if distort:
        rng = np.random.default_rng(3)
        h = rng.uniform(0.8, 1.2, 64000)
        for x in w:
            x.particles["homothety"] = h.copy()
            for k in ("qw", "qx", "qy", "qz"):
                x.particles[k] = x.particles[k] * 1.02
    a, b = (x.build() for x in w)
    for s in (a, b):
        s.update_particle_neighbors()
    la, lb = a.interactions(), b.interactions()
    assert len(la["type"]) > 100_000
    assert_same_list(la, lb)


def test_fp32_decisions_selftest(native_lib):
    """The FP32 decisions of the broad-phase tests agree with FP64 whenever they decide."""
    import ctypes as C

    counts = (C.c_uint64 * 24)()
    n = 24_000_000
    assert native_lib.dem_selftest_poly_decisions(n, 2024, counts) == 0
    names = ["gate", "vv", "ve", "vf", "ee", "displacement"]
    for k, name in enumerate(names):
        bad, undecided, dec_true, exact_true = counts[4 * k: 4 * k + 4]
        assert bad == 0, (name, bad)
        # every draw sits near a threshold (offsets log-uniform in [1e-10, 1e-1]
        # of the particle size), so a large share stays undecided by design
        assert undecided < 0.8 * (n // 6), (name, undecided)
        assert 0 < dec_true <= exact_true, name
