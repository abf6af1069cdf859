"""Mesh drivers (register_stl_mesh) on the GPU against the oracle, bit for bit:
spheres (interaction types 7-9, nbh_sphere.hpp:25-86, contact_sphere.hpp:300-396)
and polyhedra (types 7-12, nbh_polyhedron_driver.hpp:61-192,
polyhedron/contact.hpp:305-432) landing on a triangulated terrain.  Compared:
the interaction list (owner / partner sub = the particle's / mesh's feature),
the particles and the contact state, on the plain and fused paths (graph
replay included), with the cohesive and DMT laws and with multi-material
tables; and the registration checks."""
import numpy as np
import pytest

from exadem_gb300 import _abi as A
from exadem_gb300 import workloads as W
from exadem_gb300.system import contact_params
from tests.helpers import assert_same_list, bit_equal_fraction, pair

pytestmark = pytest.mark.gpu


def _bits(x):
    return np.ascontiguousarray(x).view(np.uint64)


def _run(w, steps, analysis=False, setup=None):
    g, o = pair(w)
    for s in (g, o):
        if setup:
            setup(s)
        if analysis:
            s.set_analysis(True)
        s.first_iteration()
        s.step(steps)
    return g, o


def _mesh_types(lst, state=None):
    t = lst["type"]
    out = {k: int(np.sum(t == k)) for k in (7, 8, 9)}
    if state is not None:
        out.update({k + 10: int(np.sum((t == k) & (state["dn"] < 0))) for k in (7, 8, 9)})
    return out


@pytest.mark.parametrize("path", ["plain", "fused", "fused_graph"])
def test_mesh_terrain_matches_oracle(native_lib, path):
    flags = dict(fused_step=int(path != "plain"), fp32_contact_screen=int(path != "plain"),
                 fp32_broad_phase=int(path != "plain"), graph_step=int(path == "fused_graph"))
    w = W.spheres_mesh_terrain(n=3000, seed=21, **flags)
    g, o = _run(w, 400, analysis=(path == "plain"))
    lg = g.interactions()
    assert_same_list(lg, o.interactions())
    if path == "plain":
        cg, co = g.contact_state(), o.contact_state()
        for k in ("dn", "cp", "fn", "ft"):
            assert np.array_equal(_bits(cg[k]), _bits(co[k])), k
        seen = _mesh_types(lg, cg)
        assert seen[18] > 0 and seen[19] > 0, seen  # touching edges and faces
    assert bit_equal_fraction(g.particles(sort_by_id=True), o.particles(sort_by_id=True)) == 1.0


@pytest.mark.parametrize("law", [A.LAW_HOOKE_COHESIVE, A.LAW_HOOKE_DMT])
def test_mesh_laws_match_oracle(native_lib, law):
    w = W.spheres_mesh_terrain(n=2500, seed=22, fused_step=1, fp32_contact_screen=1, fp32_broad_phase=1)
    w.params.law = law
    for cp in (w.params.config, w.params.config_driver):
        if law == A.LAW_HOOKE_COHESIVE:
            cp.dncut, cp.fc = 0.01, 10.0
        else:
            cp.gamma = 5.0
    g, o = _run(w, 400)
    assert_same_list(g.interactions(), o.interactions())
    assert bit_equal_fraction(g.particles(sort_by_id=True), o.particles(sort_by_id=True)) == 1.0


def test_mesh_multimat_matches_oracle(native_lib):
    w = W.spheres_mesh_terrain(n=2500, seed=23, fused_step=1, fp32_contact_screen=1, fp32_broad_phase=1)
    w.particles["group"] = np.random.default_rng(23).integers(0, 2, w.n).astype(np.uint32)
    pairs = [[contact_params(kn=1e4, kt=8e3, mu=0.4, damp_rate=0.9), contact_params(kn=2e4, kt=9e3, mu=0.3,
                                                                                    damp_rate=0.8)],
             [None, contact_params(kn=1.5e4, kt=7e3, mu=0.5, damp_rate=0.7)]]
    pairs[1][0] = pairs[0][1]
    nd = len(w.surfaces) + len(w.meshes)
    drivers = [[contact_params(kn=1e4 * (1 + 0.2 * g + 0.1 * d), kt=8e3, mu=0.3 + 0.05 * d, damp_rate=0.9)
                for d in range(nd)] for g in range(2)]
    g, o = _run(w, 400, setup=lambda s: s.set_multimat(pairs, drivers))
    assert_same_list(g.interactions(), o.interactions())
    assert bit_equal_fraction(g.particles(sort_by_id=True), o.particles(sort_by_id=True)) == 1.0


def test_mesh_registration_checks(native_lib):
    w = W.spheres_mesh_terrain(n=300, seed=24)
    s = w.build()
    m = dict(w.meshes[0])
    bad_edge = dict(m, edges=np.array([[0, 10 ** 6]], dtype=np.int32))
    with pytest.raises(A.DemError):
        s.register_mesh(**bad_edge)
    with pytest.raises(A.DemError):
        s.register_mesh(**dict(m, faces=[[0, 1]]))  # a face needs 3 vertices
    with pytest.raises(A.DemError):
        s.register_mesh(**dict(m, minkowski=-1.0))


@pytest.mark.parametrize("path", ["plain", "fused"])
def test_poly_mesh_terrain_matches_oracle(native_lib, path):
    f = int(path == "fused")
    w = W.polyhedra_mesh_terrain(amp=0.5, waves=3, fused_step=f, fp32_broad_phase=f, fp32_contact_screen=f)
    g, o = _run(w, 600, analysis=(path == "plain"))
    lg = g.interactions()
    assert_same_list(lg, o.interactions())
    t = lg["type"]
    assert all(np.sum(t == k) > 0 for k in (8, 9, 10, 12)), {k: int(np.sum(t == k)) for k in range(13)}
    if path == "plain":
        cg, co = g.contact_state(), o.contact_state()
        for k in ("dn", "cp", "fn", "ft"):
            assert np.array_equal(_bits(cg[k]), _bits(co[k])), k
        assert np.sum((cg["dn"] < 0) & (t >= 7)) > 0
        sg, tg = g.stress_tensor()
        so, to = o.stress_tensor()
        assert np.array_equal(_bits(tg), _bits(to))
    assert bit_equal_fraction(g.particles(sort_by_id=True), o.particles(sort_by_id=True)) == 1.0
    assert g.simulation_state()["n_active_interactions"] == o.simulation_state()["n_active_interactions"]


@pytest.mark.parametrize("law", [A.LAW_HOOKE_COHESIVE, A.LAW_HOOKE_DMT])
def test_poly_mesh_laws_match_oracle(native_lib, law):
    w = W.polyhedra_mesh_terrain(amp=0.5, waves=3, seed=31, fused_step=1, fp32_broad_phase=1, fp32_contact_screen=1)
    w.params.law = law
    for cp in (w.params.config, w.params.config_driver):
        if law == A.LAW_HOOKE_COHESIVE:
            cp.dncut, cp.fc = 0.01, 5.0
        else:
            cp.gamma = 2.0
    g, o = _run(w, 600)
    assert_same_list(g.interactions(), o.interactions())
    assert bit_equal_fraction(g.particles(sort_by_id=True), o.particles(sort_by_id=True)) == 1.0
    assert g.simulation_state()["n_active_interactions"] == o.simulation_state()["n_active_interactions"]
