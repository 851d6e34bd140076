"""Empirical phase structure function along x (theory/phase_screens/sf.py:4-8
of the reference): for each lag r = 1..N-1, the mean over x of
(phi[:, x] - phi[:, x + r])^2, per row.  The row mean of it for CUDA screens
is the engine's atm_structure_function kernel
(simulations.structure_function.calculate_structure_function)."""
from ...simulations.structure_function import calculate_sf  # noqa: F401
