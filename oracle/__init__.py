"""CPU oracle of the Volumetric ReSTIR frame loop (test infrastructure only)."""
