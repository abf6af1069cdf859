"""Contact network (dump_contact_network, src/interaction/dump_contact_network.cpp
and src/interaction/include/exaDEM/network.hpp:40-235) from the contact state
the library keeps while analysis is on (System.set_analysis).

Per particle pair (the contact law's particles i = pi_, j = pj_) the network
holds the number of interactions with a non-zero force |fn + ft| and the
sums of their fn and ft: the particle-particle contacts (types 0-3), then the
inner bonds (dump_contact_network.cpp:69-88 adds both, in that order; a bond's
state is inner_bond_law's fn = f_i - friction and friction, read with
System.bond_state).  The reference skips interactions whose partner is a
ghost (filter_duplicates): here those are the periodic images, found as pairs
whose raw centre offset is longer than half the period along a periodic axis
(a periodic axis has at least three cells of the interaction reach, so a pair
in reach directly is never that far apart).  Its std::map orders pairs by grid
cell; here they come in (id_i, id_j) order.  The files are the reference's VTK PolyData text: one
`.vtp` per rank in `basename/`, indexed by `basename.pvtp`, values printed
like a C++ stream's default format (6 significant digits)."""
from __future__ import annotations

import os

import numpy as np


def contact_network(system) -> dict:
    """Pairs (id_i, id_j), counts n, summed fn and ft (law frame), positions."""
    it = system.interactions()
    cs = system.contact_state()
    p = system.particles(sort_by_id=True)
    row = {int(i): k for k, i in enumerate(p["id"])}
    r = np.stack([p["rx"], p["ry"], p["rz"]], 1)
    fn = cs["fn"].reshape(-1, 3)
    ft = cs["ft"].reshape(-1, 3)
    prm = system.params
    period = np.array([prm.bounds_hi[d] - prm.bounds_lo[d] for d in range(3)])
    periodic = np.array([bool(prm.periodic[d]) for d in range(3)])
    net = {}

    def add(i, j, fnk, ftk):
        f = fnk + ftk
        if not np.sqrt(f @ f) != 0.0:
            return
        d = r[row[j]] - r[row[i]]
        if np.any(periodic & (np.abs(d) > 0.5 * period)):
            return  # a periodic image partner: the reference's PartnerGhost
        e = net.setdefault((i, j), [0, np.zeros(3), np.zeros(3)])
        e[0] += 1
        e[1] = e[1] + fnk
        e[2] = e[2] + ftk

    for k in np.flatnonzero(it["type"] <= 3):
        a, b = int(it["owner_id"][k]), int(it["partner_id"][k])
        i, j = (b, a) if it["swap"][k] else (a, b)  # the law's particles pi_, pj_
        add(i, j, fn[k], ft[k])
    if system.bond_count():
        bl, bs = system.bonds(), system.bond_state()
        for k in range(len(bl["id_i"])):
            add(int(bl["id_i"][k]), int(bl["id_j"][k]), bs["fn"][k], bs["ft"][k])
    keys = sorted(net)
    return {"pairs": np.asarray(keys, dtype=np.uint64).reshape(-1, 2),
            "n": np.asarray([net[q][0] for q in keys], dtype=np.int64),
            "fn": np.asarray([net[q][1] for q in keys]).reshape(-1, 3),
            "ft": np.asarray([net[q][2] for q in keys]).reshape(-1, 3),
            "ri": np.asarray([r[row[q[0]]] for q in keys]).reshape(-1, 3),
            "rj": np.asarray([r[row[q[1]]] for q in keys]).reshape(-1, 3)}


def _g(x) -> str:
    return "%g" % float(x)


def write_contact_network(system, basename: str, rank: int = 0, nranks: int = 1) -> str:
    """Writes basename.pvtp (rank 0) and basename/%06d.vtp; returns the .vtp path."""
    net = contact_network(system)
    n = len(net["n"])
    os.makedirs(basename, exist_ok=True)
    if rank == 0:
        sub = os.path.basename(basename)
        with open(basename + ".pvtp", "w") as f:
            f.write('<?xml version="1.0"?>\n<VTKFile type="PPolyData"> \n   <PPolyData GhostLevel="0">\n'
                    '     <PPoints>\n       <PDataArray type="Float64" NumberOfComponents="3"/>\n'
                    '     </PPoints> \n     <PPointData>\n'
                    '       <PDataArray type="Int32" Name="N" NumberOfComponents="1"/>\n'
                    '       <PDataArray type="Float64" Name="fn" NumberOfComponents="3"/>\n'
                    '       <PDataArray type="Float64" Name="ft" NumberOfComponents="3"/>\n'
                    '     </PPointData>\n')
            for q in range(nranks):
                f.write('     <Piece Source="%s/%06d.vtp"/>\n' % (sub, q))
            f.write("   </PPolyData>\n</VTKFile>\n")
    pos = "".join(" " + " ".join(_g(v) for v in (*net["ri"][k], *net["rj"][k])) for k in range(n))
    cnt = "".join(" %d %d" % (net["n"][k], net["n"][k]) for k in range(n))
    fns = "".join(" " + " ".join(_g(v) for v in (*net["fn"][k], *net["fn"][k])) for k in range(n))
    fts = "".join(" " + " ".join(_g(v) for v in (*net["ft"][k], *net["ft"][k])) for k in range(n))
    path = os.path.join(basename, "%06d.vtp" % rank)
    with open(path, "w") as f:
        f.write('<?xml version="1.0"?>\n<VTKFile type="PolyData">\n  <PolyData>\n')
        f.write('    <Piece NumberOfPoints="%d" NumberOfLines="%d">\n    <PointData>\n' % (2 * n, n))
        f.write('      <DataArray type="Int32" Name="N" NumberOfComponents="1" format="ascii">\n')
        if n:
            f.write(cnt + "\n")
        f.write('      </DataArray>\n      <DataArray type="Float64" Name="fn" NumberOfComponents="3" format="ascii">\n')
        if n:
            f.write(fns + "\n")
        f.write('      </DataArray>\n      <DataArray type="Float64" Name="ft" NumberOfComponents="3" format="ascii">\n')
        if n:
            f.write(fts + "\n")
        f.write('      </DataArray>\n    </PointData>\n    <Points>\n'
                '      <DataArray type="Float64" Name=""  NumberOfComponents="3" format="ascii">\n')
        if n:
            f.write(pos + "\n")
        f.write('      </DataArray>\n    </Points>\n    <Lines>\n'
                '      <DataArray type="Int32" Name="connectivity" format="ascii">\n')
        f.write("".join(" %d" % q for q in range(2 * n)))
        f.write('      </DataArray>\n      <DataArray type="Int32" Name="offsets" format="ascii">\n')
        f.write("".join(" %d" % (2 * q) for q in range(1, n + 1)) + "\n")
        f.write("      </DataArray>\n    </Lines>\n    </Piece>\n  </PolyData>\n</VTKFile>\n")
    return path
