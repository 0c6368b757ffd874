"""CPU oracle for the basis-function-expansion path — TEST INFRASTRUCTURE.

This package restates, in vectorised float64 NumPy, the exptool reference
algorithms the GPU path implements (spherical SL accumulation/evaluation, EOF
accumulation/evaluation, Fields forces and the leapfrog integrator).  Each
function cites the reference file:line it follows.  It is pinned against the
golden vectors in ``tests/golden`` that were produced by running the reference
itself.

Only the test suite, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU baseline
(and its ``--impl reference`` arm) may import it, and only as the checker or
the timed CPU baseline.  The product package ``exptool_gb300`` never imports
it and has no CPU fallback.
"""
