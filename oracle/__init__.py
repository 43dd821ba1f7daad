"""CPU oracle for the 2D Euler split step (test infrastructure only)."""
