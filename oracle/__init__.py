"""CPU oracle of the tessellated-cluster build chain (test infrastructure only)."""
