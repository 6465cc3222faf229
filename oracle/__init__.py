"""FP64 CPU oracle for the casa-imaging hot path: test infrastructure only.

Imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg.
The product library never imports this package.
"""
