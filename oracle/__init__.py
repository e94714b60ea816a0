"""CPU oracle for the axisymmetric (z, r) vorticity-streamfunction hot path.

TEST INFRASTRUCTURE ONLY. This package is the checker: a plain numpy (and C)
restatement of the PyAxisymFlow per-timestep kernels, each function citing the
reference file:line it follows. Only ``tests/``, ``__graft_entry__.smoke()``
and ``bench.py``'s CPU-baseline / ``--impl reference`` legs may import it.
The product package ``pyaxisymflow_gb300`` never imports, links or runs
anything from here; it fails loudly when its CUDA library is missing.

Parity pin: the restatement is checked against golden vectors produced by
running the reference's own Python kernels (``tests/golden/make_golden.py``)
and against the reference's two known-answer tests (Brinkman KAT, 3x3 pivoted
Gauss elimination). The pystencils ENO3 kernels cannot be run (pystencils is
not installed), so the ENO3 ghost-layer detail is restated from pystencils'
documented automatic ghost-layer rule and is pinned only by property tests.
"""
