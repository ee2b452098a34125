"""Single-rank mpi4py stand-in (one process per GPU)."""
