"""TEST INFRASTRUCTURE ONLY: the CPU oracle of the HDoG path and the reference-kernel launcher."""
