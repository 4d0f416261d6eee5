"""Recipe and sources of the reference-kernel CPU harness (test infrastructure)."""
