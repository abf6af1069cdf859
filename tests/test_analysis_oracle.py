"""The oracle's stress tensor (stress_tensor.cu:40-75) against the formula
evaluated in numpy from its own contact state and interaction list: the pair's
particle i of the contact law (pi_: the owner unless the polyhedron pair is
swapped, interaction_pair.hpp:70-112) takes (fn + ft) (cp - r_i)^T, particle j
the opposite force about its own centre (pairs only, not drivers), and only
pairs with dn < 0 count.  Summation order differs from the oracle's, so the
comparison carries a tolerance (1e-12 of the largest entry)."""
import numpy as np
import pytest

from exadem_gb300 import workloads as W
from oracle.oracle import oracle_system

DRIVER_TYPES = 4  # interaction types >= 4 are particle-driver pairs


def _numpy_stress(s):
    p = s.particles(sort_by_id=True)
    row = {int(i): k for k, i in enumerate(p["id"])}
    r = np.stack([p["rx"], p["ry"], p["rz"]], axis=1)
    it = s.interactions()
    cs = s.contact_state()
    cp, fn, ft = (cs[k].reshape(-1, 3) for k in ("cp", "fn", "ft"))
    m = np.zeros((len(p["id"]), 3, 3))
    touching = 0
    for k in range(len(cs["dn"])):
        if not cs["dn"][k] < 0.0:
            continue
        touching += 1
        f = fn[k] + ft[k]
        o = row[int(it["owner_id"][k])]
        if it["type"][k] >= DRIVER_TYPES:
            m[o] += np.outer(f, cp[k] - r[o])
            continue
        q = row[int(it["partner_id"][k])]
        i, j = (q, o) if it["swap"][k] else (o, q)
        m[i] += np.outer(f, cp[k] - r[i])
        m[j] += np.outer(-f, cp[k] - r[j])
    return m.reshape(-1, 9), touching, int(np.sum(it["swap"].astype(bool) & (cs["dn"] < 0)))


def _oracle_stress_by_id(s):
    stress, total = s.stress_tensor()
    ids = s.particles(sort_by_id=False)["id"]
    return stress[np.argsort(ids, kind="stable")], total


@pytest.mark.parametrize("case", ["spheres_drum", "polyhedra"])
def test_oracle_stress_is_the_formula(case):
    if case == "spheres_drum":
        w = W.spheres_drum(n=600, seed=95)
        steps = 150
    else:
        w = W.polyhedra_lattice(nx=4, ny=4, nz=3, seed=96)
        steps = 60
    s = w.build(oracle_system)
    s.set_analysis(True)
    s.first_iteration()
    s.step(steps)
    want, touching, swapped = _numpy_stress(s)
    got, total = _oracle_stress_by_id(s)
    assert touching > 0
    if case == "polyhedra":
        assert swapped > 0  # the swap sign is exercised
    scale = np.abs(want).max()
    assert scale > 0
    assert np.abs(got - want).max() <= 1e-12 * scale
    assert np.abs(total - want.sum(axis=0)).max() <= 1e-12 * scale * len(want)
