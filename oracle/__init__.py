"""CPU oracle for the qibo state-vector hot path.

TEST INFRASTRUCTURE ONLY.  The product path (``qibo_gb300``) never imports,
calls or executes anything in this package; only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py`` (its CPU-baseline leg and the
``--impl reference`` arm) use it, and only as the checker / the timed CPU
baseline.

``oracle.numpy_ref`` restates, function by function, the numpy algorithms of
qibo 0.3.5's ``NumpyBackend`` (``src/qibo/backends/abstract.py``,
``backends/numpy.py``, ``backends/npmatrices.py``, ``backends/einsum_utils.py``)
and cites the reference file:line each function follows.  It is pinned
against golden vectors produced by the reference itself
(``tests/golden/make_golden.py`` imports qibo from the reference tree and runs
it) and against the reference tests' own known-answer values; see
``tests/test_oracle.py``.
"""
