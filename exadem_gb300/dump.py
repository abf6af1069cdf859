"""Checkpoint and restart of a run: particles plus the interaction list with
its friction/moment history, and the inner bonds of a fragmentation run.

Named after exaDEM's dump operators write_dump_particle_interaction
(src/io/sim_dump_writer_interaction.cpp:43-45) and read_dump_particle_interaction
(src/io/sim_dump_reader_interaction.cpp:56-63), which write the particles and
the interactions (as extra data of the grid) to an exaNBody dump.  exaNBody's
dump layout is not part of exaDEM's sources, so the file here is this
library's own: one .npz with every particle field and the list in
InteractionPair order.  A run restarted from it continues with the same bits
as the run that wrote it (System setup -> read -> step).  With bonds
(write_dump_particle_fragmentation / read_dump_particle_fragmentation in
exaDEM's config_fragmentation.msp) the bond list and its state are saved too;
the record of the last bond pass (dn, fn) is not, as in exaDEM, so a restart
matches bit for bit when no interface breaks on its first step.
"""
from __future__ import annotations

import json

import numpy as np

FORMAT = "exadem_gb300 checkpoint 1"


def write_dump_particle_interaction(system, path, timestep: int = 0, **meta) -> None:
    """Writes the system's particles and interactions (with history) to `path`."""
    parts = system.particles(sort_by_id=True)
    inter = system.interactions()
    arrays = {f"p/{k}": v for k, v in parts.items()}
    arrays.update({f"i/{k}": v for k, v in inter.items()})
    nb = system.bond_count()
    if nb:
        arrays.update({f"b/{k}": v for k, v in system.bonds().items()})
    info = {"format": FORMAT, "timestep": int(timestep), "n": int(len(parts["id"])),
            "n_interactions": int(len(inter["owner_id"])), "n_bonds": int(nb), **meta}
    arrays["meta"] = np.frombuffer(json.dumps(info).encode(), dtype=np.uint8)
    np.savez(path, **arrays)


def read_dump(path) -> tuple[dict, dict, dict]:
    """(particles, interactions, meta) of a checkpoint; meta["bonds"] holds the
    bond list when the checkpoint has one."""
    z = np.load(path)
    info = json.loads(z["meta"].tobytes().decode())
    if info.get("format") != FORMAT:
        raise ValueError(f"{path}: not a checkpoint of this library ({info.get('format')!r})")
    parts = {k[2:]: np.ascontiguousarray(z[k]) for k in z.files if k.startswith("p/")}
    inter = {k[2:]: np.ascontiguousarray(z[k]) for k in z.files if k.startswith("i/")}
    bonds = {k[2:]: np.ascontiguousarray(z[k]) for k in z.files if k.startswith("b/")}
    if bonds:
        info["bonds"] = bonds
    return parts, inter, info


def read_dump_particle_interaction(system, path) -> dict:
    """Restores a checkpoint into a system whose parameters, drivers and shapes
    are set: the particles, the history, then the neighbour list.  Returns the
    checkpoint's metadata (timestep, counts)."""
    parts, inter, info = read_dump(path)
    system.set_particles(parts)
    system.set_interactions(inter)
    bonds = info.pop("bonds", None)
    if bonds is not None:
        system.set_bonds(bonds)
    system.update_particle_neighbors()
    return info


# exaDEM's operator names for the checkpoint of a fragmentation run
write_dump_particle_fragmentation = write_dump_particle_interaction
read_dump_particle_fragmentation = read_dump_particle_interaction
