"""CPU oracle for the FDTD hot path -- TEST INFRASTRUCTURE ONLY.

This package restates, in float64 NumPy (``fd1d``, ``fd2d``) and plain C
(``fdtd_oracle.c``, loaded through ``ccore``), the reference programs of
dsarvan/simulation that the GPU library replaces.  Every function cites the
reference file and line it follows.

It is the checker, never the product: only ``tests/``, ``__graft_entry__.smoke``
and the CPU-baseline legs of ``bench.py`` import it.  The product path
(``simulation_gb300``) never imports, links or calls anything in here and
fails loudly when its CUDA library is missing.

Parity pinning: ``refload`` imports the reference's own Python programs (with
stub ``matplotlib``/``numba`` modules) and ``tests/golden/make_golden.py``
runs them to produce the committed fixtures in ``tests/golden/``; the CPU test
suite checks this oracle against those fixtures.  ``Makefile`` also compiles the
reference's own C step functions into ``oracle/_ref`` (in a container that has
the reference checked out) so the C restatement can be compared with them.
"""
