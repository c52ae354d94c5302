"""CPU oracle for the gate-application hot path.

TEST INFRASTRUCTURE ONLY. Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline legs of ``bench.py`` may import this package, and only as the
checker or as the timed CPU reference. The shipped package never imports it.

* ``oracle.ncon``  -- NCON contraction (the reference's ``ncon_torch``
  dependency, restated from the published convention).
* ``oracle.ref``   -- NumPy complex128 restatement of the reference's
  statevector / density-matrix / noise / expectation / trajectory algorithms,
  each function citing the reference file and lines it follows.
* ``oracle.refload`` -- imports the real reference package (only where its
  source tree is present) for fixture generation and cross-checks.

Parity pin: ``tests/golden/*.npz`` were produced by the real reference
(``tests/golden/make_golden.py``) and ``tests/test_oracle_golden.py`` checks
this restatement against them.
"""
