"""CPU oracle of the reference SIFT path (test infrastructure only)."""
