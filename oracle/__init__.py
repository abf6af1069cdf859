"""CPU oracle of the exaDEM per-timestep hot path (test infrastructure only)."""
