"""Solver modules of the GB300 backend: NS (velocity) and VV (velocity-vorticity)."""
