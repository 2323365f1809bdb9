"""CPU oracle for the LatticeModels.jl evolution path -- test infrastructure only.

Imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the checker;
the product library (lmgpu / liblmgpu.so) never uses it.
"""
