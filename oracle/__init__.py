"""Test infrastructure only: the CPU oracle of the DFSPH step and the recipe
that builds the reference's own kernels for parity runs. Only tests/,
__graft_entry__.smoke() and bench.py's baseline legs (the CPU baseline, the
reference arm, and the timings of the reference's own kernels beside this
build's) import this package; the product never does."""
