"""CPU oracle and reference-build helpers (test infrastructure only)."""
