"""Test infrastructure: the FP64 oracle (oracle.py), the reference compiled for
the CPU (refrun.py, build_ref.sh) and their build recipes.  Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg use this package."""
