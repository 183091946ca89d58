"""CPU oracle for the convection/diffusion hot path (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline and
reference legs import this package.  The product library never does.
"""
