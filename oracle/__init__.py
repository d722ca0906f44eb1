"""CPU oracle for the TEMPO / PT-TEMPO / compute_dynamics hot path.

TEST INFRASTRUCTURE ONLY.  Nothing in the product package ``oqupy_gb300``
imports, calls or links anything under ``oracle/``.  The oracle is used
exclusively by ``tests/``, by ``__graft_entry__.smoke()`` as the checker and
by ``bench.py``'s CPU baseline / reference arm.

Contents
--------
``tempo_oracle``   plain-numpy restatement of OQuPy's TEMPO step, PT-TEMPO
                   build and process-tensor sweep (complex128), citing the
                   reference file:line for every stage.
``bath_oracle``    the reference's bath-correlation integrals (scipy quad)
                   and influence matrices, restated.
``tnshim/``        a from-scratch stand-in for the third-party
                   ``tensornetwork`` package so that the unmodified OQuPy
                   reference can run in the development container to produce
                   the golden fixtures under ``tests/golden/``.

Pinning: the restatement is checked against fixtures produced by running the
unmodified reference (``tests/golden/make_golden.py``) and against the
reference's own physics goldens (``tests/physics/tempo_spin_boson_test.py``
``:45-46``, ``tests/physics/tempo_qutrit_test.py:59-62``).
"""
