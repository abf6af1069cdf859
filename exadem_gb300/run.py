"""Runs an exaDEM ``.msp`` deck on the GPU hot path.

    python -m exadem_gb300.run DECK.msp [--config-dir DIR] [--steps N] [--plain]

The deck is read with exadem_gb300.msp (includes resolved in the deck's folder,
then in --config-dir, e.g. exaDEM's data/config), then run for
``global.simulation_end_iteration`` steps (or --steps) from first_iteration.
Every ``global.simulation_log_frequency`` steps one line reports the step, the
physical time, the number of interactions, the kinetic and rotation energies
and the throughput in particle-steps/s, the quantities of exaDEM's
print_simulation_state (src/io/print_simulation_state.cpp:122-145).
"""
from __future__ import annotations

import argparse
import time
from pathlib import Path


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("deck")
    ap.add_argument("--config-dir", action="append", default=[], help="where the deck's includes are searched")
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--plain", action="store_true", help="plain FP64 operator kernels (no fused step)")
    ap.add_argument("--seed", type=int, default=1, help="seed of the random initial velocities / orientations")
    a = ap.parse_args(argv)

    from . import msp

    deck_path = Path(a.deck)
    deck = msp.load_deck(deck_path, a.config_dir)
    opt = 0 if a.plain else 1
    w = msp.deck_workload(deck, base_dir=deck_path.parent, seed=a.seed, fused_step=opt, fp32_broad_phase=opt,
                          fp32_contact_screen=opt)
    for note in w.info.get("notes", []):
        print(f"# note: {note}")
    glob = deck.get("global", {}) or {}
    steps = a.steps if a.steps is not None else w.steps
    every = int(glob.get("simulation_log_frequency", 1000) or 1000)
    every = max(1, every if every > 0 else steps)
    s = w.build()
    s.first_iteration()
    print(f"# {w.n} particles, {w.info['contact_operator']}, dt {w.params.dt}, {steps} steps")
    print(f"{'step':>9} {'time':>10} {'interactions':>12} {'kinetic_energy':>16} {'rotation_energy':>16} "
          f"{'particle-steps/s':>16}")
    done = 0
    while done < steps:
        k = min(every, steps - done)
        t0 = time.perf_counter()
        s.step(k)
        st = s.simulation_state()  # synchronises
        el = time.perf_counter() - t0
        done += k
        ke, re = float(sum(st["kinetic_energy"])), float(sum(st["rotation_energy"]))
        print(f"{done:>9} {done * w.params.dt:>10.4g} {st['n_interactions']:>12} {ke:>16.8e} {re:>16.8e} "
              f"{w.n * k / el:>16.4e}")
    s.close()
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
