"""CPU oracle for the tyxonq_gb300 statevector path.

TEST INFRASTRUCTURE ONLY.  This package is a plain-NumPy restatement of the
reference's statevector algorithm (TyxonQ, tyxonq/libs/quantum_library/kernels
and tyxonq/devices/simulators/statevector/engine.py), each function citing
the reference lines it follows.  Only ``tests/``, ``__graft_entry__.smoke()``
and the ``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may use
it, and only as the checker or the timed CPU baseline.  The product package
``tyxonq_gb300`` never imports it.

Parity pin: the restatement is checked against golden vectors produced by the
reference itself (``tests/golden/make_golden.py`` imports TyxonQ from its
source tree and records states, probabilities, expectations, energies and
autograd gradients), and against the reference tests' known answers.
"""
