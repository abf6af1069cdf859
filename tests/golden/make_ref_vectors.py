"""Generates tests/golden/ref_units.npz: inputs and exaDEM's outputs for the
oracle's unit entry points (test fixture generator).

Run where the exaDEM sources are present (oracle/ref_build.py compiles exaDEM's
own headers into oracle/_ref/libexadem_ref.so).  Each record holds seeded input
rows (oracle/units.py) and the rows exaDEM's functions return on them; the
vertex-face records also hold the shape, written by this project's .shp writer
from its own cube, tetrahedron and octahedron builders, together with exaDEM's
read_shp result for it (vertices, OBB, face areas).  tests/test_oracle_golden.py checks the oracle against
these outputs bit for bit wherever the sources are absent.

    python tests/golden/make_ref_vectors.py
"""
from __future__ import annotations

import ctypes as C
import os
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import ref_build  # noqa: E402
from oracle import units as U  # noqa: E402

OUT = Path(__file__).resolve().parent / "ref_units.npz"
ROWS = 128


def main() -> None:
    from exadem_gb300 import shp, workloads as W

    lib = ref_build.build()
    if lib is None:
        raise SystemExit("exaDEM sources not found (set EXADEM_SRC)")
    ref = C.CDLL(str(lib))
    rec = {}
    for name in U.LAYOUT:
        for law in ([0, 1, 2] if name == "contact_force_core" else [0]):
            x = U.cases(name, ROWS, 9000 + law)
            rec[f"{name}/{law}/in"] = x
            rec[f"{name}/{law}/out"] = U.run(ref, "ref", name, x, law)
    k = U.pair_keys(4 * ROWS, 9100)
    rec["pair_order/in"] = k
    rec["pair_order/out"] = U.run_pair_order(ref, "ref", k)
    with tempfile.TemporaryDirectory() as d:
        for s in (W.shape_cube(), W.shape_tetrahedron(), W.shape_octahedron()):
            text = shp.format_shp(s)
            p = os.path.join(d, "s.shp")
            Path(p).write_text(text)
            r = U.read_shps_ref(ref, p)[0]
            tag = f"shape/{s['name']}"
            rec[f"{tag}/text"] = np.frombuffer(text.encode(), dtype=np.uint8)
            rec[f"{tag}/vertices"] = r["vertices"]
            rec[f"{tag}/obb"] = np.concatenate([np.asarray(r["obb"][k_], dtype=np.float64)
                                                for k_ in ("center", "e1", "e2", "e3", "extent")])
            rec[f"{tag}/face_areas"] = U.face_areas_ref(ref, r["index"], len(s["faces"]))
            for face in range(len(s["faces"])):
                x = U.vertex_face_cases(s, face, ROWS // 4, 9200 + face)
                rec[f"{tag}/vf{face}/in"] = x
                rec[f"{tag}/vf{face}/out"] = U.run_vertex_face_ref(ref, r["index"], face, len(s["vertices"]), x)
    np.savez_compressed(OUT, **rec)
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes, {len(rec)} arrays)")


if __name__ == "__main__":
    main()
