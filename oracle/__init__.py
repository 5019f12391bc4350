"""CPU oracle of the Hybrid2D kinetic path -- test infrastructure only."""
