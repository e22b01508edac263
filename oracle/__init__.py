"""CPU oracle for the stencil3d hot path (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py`` import this package.  The product (``stencil3d_gb300``) never
does.
"""
