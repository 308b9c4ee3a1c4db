"""CPU oracle of the path tracer - test infrastructure only (see oracle.h)."""
