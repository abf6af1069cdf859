"""Checkpoint and restart on the GPU (dem_set_interactions, exadem_gb300/dump.py):
a run stopped, written, read back into a new context and continued ends in
the same bits as the run that never stopped, on the plain, fused and graph
paths; a checkpoint written by the GPU resumes on the oracle with the same
result."""
import numpy as np
import pytest

from exadem_gb300 import dump, workloads as W
from tests.test_restart import _bits_equal, _with_history, run_restart
from tests.helpers import FIELDS_STATE, assert_same_list

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("flags", [{}, dict(fused_step=1, fp32_broad_phase=1, fp32_contact_screen=1),
                                   dict(fused_step=1, fp32_broad_phase=1, fp32_contact_screen=1, graph_step=1)],
                         ids=["plain", "fused", "graph"])
def test_restart_spheres(native_lib, tmp_path, flags):
    run_restart(W.spheres_floor(n=6000, side=24.0, phi=0.3, **flags), None, 120, 80, tmp_path)


@pytest.mark.parametrize("fused", [0, 1])
def test_restart_polyhedra(native_lib, tmp_path, fused):
    w = W.polyhedra_lattice(nx=5, ny=5, nz=4, vmax=0.5, fused_step=fused, fp32_broad_phase=fused,
                            fp32_contact_screen=fused)
    run_restart(w, None, 150, 100, tmp_path)


def test_gpu_checkpoint_resumes_on_oracle(native_lib, tmp_path):
    from oracle.oracle import oracle_system

    w = W.spheres_floor(n=6000, side=24.0, phi=0.3, fused_step=1, fp32_broad_phase=1, fp32_contact_screen=1)
    g = w.build()
    g.first_iteration()
    g.step(100)
    path = tmp_path / "gpu.npz"
    dump.write_dump_particle_interaction(g, path, timestep=100)
    g.step(60)
    o = w.build(oracle_system)
    dump.read_dump_particle_interaction(o, path)
    o.step(60)
    _bits_equal(g.particles(), o.particles(), FIELDS_STATE)
    lg, lo = _with_history(g.interactions()), _with_history(o.interactions())
    assert_same_list(lg, lo)
    assert np.array_equal(lg["friction"].view(np.uint64), lo["friction"].view(np.uint64))
    g.close()
    o.close()


@pytest.mark.parametrize("fused", [0, 1])
def test_restart_fragmentation(native_lib, tmp_path, fused):
    """Bonds saved before the impact and restored (read_dump_particle_fragmentation)
    break the same interfaces with the same bits as the run that never stopped."""
    flags = dict(fused_step=fused, fp32_broad_phase=fused, fp32_contact_screen=fused)
    run_restart(W.fragment_blocks(nblocks=2, **flags), None, 40, 300, tmp_path)
