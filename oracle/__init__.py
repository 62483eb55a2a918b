"""TEST INFRASTRUCTURE ONLY: the CPU oracle (restatement of the reference's
algorithms) and the recipe that builds the reference's own C++ programs.
Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it."""
