"""FP64 CPU oracle of the WCSPH right-hand side (test infrastructure only)."""
