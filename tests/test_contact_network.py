"""Contact network (dump_contact_network, network.hpp:40-235) written from the
contact state, with the oracle on the CPU: the exact text of the reference's
VTK files for two touching spheres, periodic image pairs left out (the
reference's PartnerGhost filter), and polyhedron pairs keyed by the contact
law's particles (swapped pairs included)."""
import xml.etree.ElementTree as ET

import numpy as np

from exadem_gb300 import _abi as A
from exadem_gb300 import workloads as W
from exadem_gb300.analysis import contact_network, write_contact_network
from oracle.oracle import oracle_system


def _two_spheres():
    cfg = dict(kn=1e4, kt=8e3, kr=0.0, mu=0.4, damp_rate=0.0)
    p = W.make_params((-5, -5, -5), (5, 5, 5), (0, 0, 0), rcut_inc=0.1, dt=1e-4, gravity=(0, 0, 0), config=cfg,
                      config_driver=cfg)
    parts = {f: np.zeros(2) for f in A.PARTICLE_FIELDS}
    parts.update(rx=np.array([0.0, 0.999]), radius=np.full(2, 0.5), mass=np.ones(2), qw=np.ones(2),
                 inertiax=np.full(2, 0.1), inertiay=np.full(2, 0.1), inertiaz=np.full(2, 0.1), homothety=np.ones(2))
    parts["id"] = np.array([3, 7], dtype=np.uint64)
    parts["type"] = np.zeros(2, np.uint32)
    parts["group"] = np.zeros(2, np.uint32)
    s = oracle_system(p)
    s.set_particles(parts)
    s.set_analysis(True)
    s.first_iteration()
    return s


def test_two_spheres_exact_text(tmp_path):
    s = _two_spheres()
    net = contact_network(s)
    assert net["pairs"].tolist() == [[3, 7]] and net["n"].tolist() == [1]
    f = 1e4 * (1.0 - 0.999)  # kn * overlap, on sphere 3 along -x
    assert np.isclose(net["fn"][0][0], -f, rtol=1e-9) and np.all(net["ft"] == 0.0)
    path = write_contact_network(s, str(tmp_path / "network"))
    fx = "%g" % net["fn"][0][0]
    want = ('<?xml version="1.0"?>\n<VTKFile type="PolyData">\n  <PolyData>\n'
            '    <Piece NumberOfPoints="2" NumberOfLines="1">\n    <PointData>\n'
            '      <DataArray type="Int32" Name="N" NumberOfComponents="1" format="ascii">\n 1 1\n'
            '      </DataArray>\n      <DataArray type="Float64" Name="fn" NumberOfComponents="3" format="ascii">\n'
            f' {fx} 0 0 {fx} 0 0\n'
            '      </DataArray>\n      <DataArray type="Float64" Name="ft" NumberOfComponents="3" format="ascii">\n'
            ' 0 0 0 0 0 0\n'
            '      </DataArray>\n    </PointData>\n    <Points>\n'
            '      <DataArray type="Float64" Name=""  NumberOfComponents="3" format="ascii">\n'
            ' 0 0 0 0.999 0 0\n'
            '      </DataArray>\n    </Points>\n    <Lines>\n'
            '      <DataArray type="Int32" Name="connectivity" format="ascii">\n'
            ' 0 1      </DataArray>\n      <DataArray type="Int32" Name="offsets" format="ascii">\n 2\n'
            '      </DataArray>\n    </Lines>\n    </Piece>\n  </PolyData>\n</VTKFile>\n')
    assert open(path).read() == want
    idx = ET.parse(str(tmp_path / "network.pvtp")).getroot()
    assert [p.get("Source") for p in idx.iter("Piece")] == ["network/000000.vtp"]


def test_periodic_images_left_out(tmp_path):
    w = W.spheres_floor(n=3000, side=12.0, seed=51)
    s = w.build(oracle_system)
    s.set_analysis(True)
    s.first_iteration()
    s.step(300)
    net = contact_network(s)
    assert len(net["n"]) > 0
    d = np.linalg.norm(net["rj"] - net["ri"], axis=1)
    assert d.max() < 1.3 + w.params.rcut_inc + w.params.config.dncut  # no image partner
    # image pairs exist and are dropped; each is listed from both owners
    it, cs = s.interactions(), s.contact_state()
    f = cs["fn"].reshape(-1, 3) + cs["ft"].reshape(-1, 3)
    nz = (it["type"] == 0) & (np.linalg.norm(f, axis=1) != 0)
    dropped = int(nz.sum() - net["n"].sum())
    assert dropped > 0 and dropped % 2 == 0
    ET.parse(write_contact_network(s, str(tmp_path / "net")))  # well-formed XML


def test_polyhedra_keyed_by_law_particles():
    w = W.polyhedra_lattice(nx=4, ny=4, nz=3, seed=52)
    s = w.build(oracle_system)
    s.set_analysis(True)
    s.first_iteration()
    s.step(60)
    it, cs = s.interactions(), s.contact_state()
    f = cs["fn"].reshape(-1, 3) + cs["ft"].reshape(-1, 3)
    nz = (it["type"] <= 3) & (np.linalg.norm(f, axis=1) != 0)
    net = contact_network(s)
    assert net["n"].sum() == nz.sum() > 0  # no periodic axes: nothing is dropped
    law_i = np.where(it["swap"].astype(bool), it["partner_id"], it["owner_id"])[nz]
    law_j = np.where(it["swap"].astype(bool), it["owner_id"], it["partner_id"])[nz]
    assert set(map(tuple, net["pairs"].tolist())) == set(zip(law_i.tolist(), law_j.tolist()))
    assert np.any(it["swap"][nz])  # swapped pairs are exercised


def test_multimat_cohesive_range_beyond_the_skin():
    """A pair attracting within a group pair's dncut (0.3, beyond rcut_inc + the
    single set's dncut) stays in the network: the ghost test is the minimum
    image along the periodic axes, not a distance bound."""
    cfg = dict(kn=1e4, kt=8e3, kr=0.0, mu=0.4, damp_rate=0.0, fc=0.1, dncut=0.01)
    p = W.make_params((-10, -5, -5), (10, 5, 5), (1, 0, 0), rcut_inc=0.1, dt=1e-3, gravity=(0, 0, 0),
                      law=A.LAW_HOOKE_COHESIVE, config=cfg, config_driver=cfg)
    parts = {f: np.zeros(2) for f in A.PARTICLE_FIELDS}
    parts.update(rx=np.array([0.0, 1.09]), vx=np.array([-0.2, 0.2]), radius=np.full(2, 0.5), mass=np.ones(2),
                 qw=np.ones(2), inertiax=np.full(2, 0.1), inertiay=np.full(2, 0.1), inertiaz=np.full(2, 0.1),
                 homothety=np.ones(2))
    parts["id"] = np.array([3, 7], dtype=np.uint64)
    parts["type"] = np.zeros(2, np.uint32)
    parts["group"] = np.zeros(2, np.uint32)
    s = oracle_system(p)
    s.set_particles(parts)
    wide = W.contact_params(**{**cfg, "dncut": 0.3})
    s.set_multimat([[wide]], [[]])
    s.set_analysis(True)
    s.first_iteration()
    s.step(220)  # each sphere moves about 0.044 < skin/2: no rebuild, gap about 0.18
    assert s.rebuild_count() == 1
    q = s.particles(sort_by_id=True)
    gap = q["rx"][1] - q["rx"][0] - 1.0
    assert 0.1 + 0.01 < gap < 0.3
    net = contact_network(s)
    assert net["pairs"].tolist() == [[3, 7]] and net["n"].tolist() == [1]
    assert net["fn"][0][0] > 0.0  # cohesion pulls sphere 3 towards +x


def test_inner_bonds_in_network():
    """Inner bonds enter the network after the contacts, keyed by the bond's
    particles, with inner_bond_law's fn = f_i - friction and friction."""
    w = W.fragment_blocks(nblocks=1, nx=2, ny=1, nz=1, vz=0.0)
    w.particles["vx"] = np.array([-0.05, 0.05])  # stretch the face bonds
    s = w.build(oracle_system)
    s.set_analysis(True)
    s.first_iteration()
    s.step(5)
    bl, bs = s.bonds(), s.bond_state()
    assert len(bl["id_i"]) == 4  # the four vertex bonds of the shared face
    f = bs["fn"] + bs["ft"]
    assert np.all(np.linalg.norm(f, axis=1) > 0)
    net = contact_network(s)
    key = (int(bl["id_i"][0]), int(bl["id_j"][0]))
    k = net["pairs"].tolist().index(list(key))
    assert net["n"][k] == 4
    fn_sum, ft_sum = np.zeros(3), np.zeros(3)
    for q in range(4):  # the network's order: bond rows in sequence
        fn_sum, ft_sum = fn_sum + bs["fn"][q], ft_sum + bs["ft"][q]
    assert np.array_equal(net["fn"][k], fn_sum) and np.array_equal(net["ft"][k], ft_sum)
