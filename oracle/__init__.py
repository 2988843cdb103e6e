"""CPU oracle of the GPU scattering path and the harness that drives the
reference library with the same random streams.  Test infrastructure only."""
