"""CPU oracle of the render hot path (test infrastructure only)."""
