"""CPU oracle for the SM/dark shower transport path.

TEST INFRASTRUCTURE.  This package restates PETITE's algorithm on the CPU
(float64, one particle at a time) so the CUDA engine can be checked against
it.  Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import it; the product (``petite_gb300``) never does and has
no CPU fallback.

Pinning: the restatement is checked against golden vectors produced by the
unmodified PETITE reference (``tests/golden/make_golden.py``).
"""
