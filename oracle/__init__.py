"""CPU oracle of the FluidGrid SPH hot path (test infrastructure only)."""
