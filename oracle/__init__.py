"""Test infrastructure only: the CPU oracle of the DFSPH step and the recipe
that builds the reference's own kernels for parity runs. Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg import this package."""
