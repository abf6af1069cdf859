"""Checkpoint and restart (exadem_gb300/dump.py, dem_set_interactions) on the
oracle (CPU): a run stopped, written, read back into a new context and
continued ends in the same bits, history included, as the run that never
stopped."""
import numpy as np
import pytest

from exadem_gb300 import dump, workloads as W
from tests.helpers import FIELDS_STATE, assert_same_list


def _bits_equal(a, b, fields):
    for f in fields:
        assert np.array_equal(np.asarray(a[f]).view(np.uint64), np.asarray(b[f]).view(np.uint64)), f


def _with_history(lst):
    keep = (lst["friction"] != 0).any(axis=1) | (lst["moment"] != 0).any(axis=1)
    return {k: v[keep] for k, v in lst.items()}


def run_restart(w, factory, n1, n2, tmp_path):
    """factory: the oracle's system factory, or None for the native library."""
    a = w.build(factory)
    a.first_iteration()
    a.step(n1 + n2)
    b = w.build(factory)
    b.first_iteration()
    b.step(n1)
    path = tmp_path / "ck.npz"
    dump.write_dump_particle_interaction(b, path, timestep=n1)
    b.close()
    c = w.build(factory)
    info = dump.read_dump_particle_interaction(c, path)
    assert info["timestep"] == n1
    c.step(n2)
    pa, pc = a.particles(), c.particles()
    _bits_equal(pa, pc, FIELDS_STATE)
    # the restarted run rebuilds at other steps than the run that never stopped, so
    # the two lists may differ in listed pairs that do not touch (zero history);
    # the pairs that carry history must be the same, with the same bits
    la, lc = _with_history(a.interactions()), _with_history(c.interactions())
    assert len(la["owner_id"]) > 0, "the restart carried nonzero history"
    assert_same_list(la, lc)
    assert np.array_equal(la["friction"].view(np.uint64), lc["friction"].view(np.uint64))
    assert np.array_equal(la["moment"].view(np.uint64), lc["moment"].view(np.uint64))
    a.close()
    c.close()


def test_restart_spheres_oracle(tmp_path):
    from oracle.oracle import oracle_system

    run_restart(W.spheres_floor(n=6000, side=24.0, phi=0.3), oracle_system, 120, 80, tmp_path)


def test_restart_polyhedra_oracle(tmp_path):
    from oracle.oracle import oracle_system

    run_restart(W.polyhedra_lattice(nx=5, ny=5, nz=4, vmax=0.5), oracle_system, 150, 100, tmp_path)


def test_restart_fragmentation_oracle(tmp_path):
    """With bonds: the checkpoint (write_dump_particle_fragmentation) carries the
    bond list; stopped before the impact, the restarted run breaks the same
    interfaces with the same bits."""
    from oracle.oracle import oracle_system

    w = W.fragment_blocks(nblocks=2)
    run_restart(w, oracle_system, 40, 300, tmp_path)
    a = w.build(oracle_system)
    a.first_iteration()
    a.step(40)
    path = tmp_path / "frag.npz"
    dump.write_dump_particle_fragmentation(a, path, timestep=40)
    c = w.build(oracle_system)
    dump.read_dump_particle_fragmentation(c, path)
    a.step(300)
    c.step(300)
    assert a.broken_interface_count() > 0 and c.broken_interface_count() == a.broken_interface_count()
    ba, bc = a.bonds(), c.bonds()
    for k in ba:
        assert np.array_equal(np.asarray(ba[k]).view(np.uint8), np.asarray(bc[k]).view(np.uint8)), k


def test_restart_rejects_unknown_ids(tmp_path):
    from oracle.oracle import oracle_system

    w = W.spheres_box(n=500, box=10.0, seed=3)
    s = w.build(oracle_system)
    s.first_iteration()
    lst = s.interactions()
    lst["owner_id"] = lst["owner_id"] + 10_000
    if len(lst["owner_id"]):
        with pytest.raises(Exception):
            s.set_interactions(lst)
    s.close()
