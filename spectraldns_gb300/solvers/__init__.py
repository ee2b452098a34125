"""Solver modules of the GB300 backend (only NS)."""
