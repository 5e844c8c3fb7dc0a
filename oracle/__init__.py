"""CPU oracle for the smolyax evaluation path -- TEST INFRASTRUCTURE ONLY.

This package restates, in plain Python and numpy, the algorithms of the
reference implementation (JoWestermann/smolyax) that the GPU library replaces:

* ``oracle.indices``  -- anisotropic multi-index sets, Smolyak coefficients,
  cardinalities and the threshold bisection (``src/smolyax/indices.py``);
* ``oracle.nodes``    -- Leja and Gauss-Hermite nodes, barycentric weights and
  quadrature weights (``src/smolyax/nodes/*.py``, ``src/smolyax/barycentric.py``);
* ``oracle.interp``   -- block assembly of ``set_f`` and the evaluation,
  gradient and integral of the barycentric Smolyak interpolant
  (``src/smolyax/interpolation.py``, ``src/smolyax/barycentric.py``).

Every function cites the reference file and lines it follows.  The oracle is
pinned against golden vectors produced by running the reference itself
(``tests/golden/``) and against the reference's own known-answer pins
(cardinalities 98 / 1000 / 10003 of ``tests/test_indices_runtime.py``).

Only the test-suite, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this package, and only as the checker or the timed CPU
baseline.  The product package ``smolyax_gb300`` never imports it.
"""
