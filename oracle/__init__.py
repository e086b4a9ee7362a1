"""CPU oracle of the solve path (test infrastructure only).

Used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the
checker of the GPU library; never imported by the product package.
"""
