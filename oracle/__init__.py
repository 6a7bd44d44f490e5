"""CPU oracle — TEST INFRASTRUCTURE ONLY.

A complex128 NumPy restatement of the reference's parameterized-circuit
semantics (TensorCircuit 0.12.1), used to check the GPU engine.  Only
``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline /
reference leg import this package; the engine never routes through it.

Parity pins: the restatement is checked against the known-answer values in
the reference's own tests (``tests/golden/reference_kats.json``, each entry
citing the reference test file:line).  The reference itself cannot run here
(it needs the un-vendored third-party ``tensornetwork`` package, pinned as
``tensornetwork-ng`` / ``tensornetwork==0.4.6`` in the reference's
requirements), so parity at the configured circuit sizes is pinned by those
small-n known answers plus internal consistency checks (finite differences,
unitarity, sum rules), not by reference outputs at full size.
"""
