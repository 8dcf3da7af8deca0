"""CPU oracle of the MPS time step (test infrastructure only)."""
