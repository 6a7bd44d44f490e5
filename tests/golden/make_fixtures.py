"""Generate the oracle fixtures under tests/golden/ (run from the repo root:
``python tests/golden/make_fixtures.py``).

* ``c1_hea_n10.npz`` -- the plain-statevector workload: n=10, complex
  amplitudes of the 4-layer hardware-efficient ansatz (rx on every qubit then
  rzz on the open chain) with 76 parameters ~U[0, 2pi) from seed 1, its
  energy under H = sum Z_i Z_{i+1} + sum X_i, and the exact adjoint gradient
  (complex128 oracle).
* ``sample_n12.npz`` -- a seeded n=12 complex64 state, 4096 seeded uniforms
  and the indices the declared integer-CDF rule draws (bit-exact target).
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import statevector as sv  # noqa: E402
from tensorcircuit_gb300 import templates  # noqa: E402


def c1() -> None:
    n, nl = 10, 4
    rng = np.random.default_rng(1)
    params = rng.uniform(0, 2 * np.pi, templates.hea_nparams(n, nl))
    layout = templates.hea_layout(n, nl)
    psi = sv.run_circuit(n, [(name, q, {"theta": params[k]}) for name, q, k in layout])
    terms = templates.tfim_terms(n, 1.0, 1.0)
    ops = [(name, q, {"theta": 0.0}) for name, q, _ in layout]
    val, grad = sv.value_and_grad_adjoint(n, ops, [k for _, _, k in layout], params, terms)
    np.savez(os.path.join(HERE, "c1_hea_n10.npz"), params=params, psi=psi, energy=val, grad=grad)


def sample12() -> None:
    rng = np.random.default_rng(7)
    n = 12
    psi = rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)
    psi = (psi / np.linalg.norm(psi)).astype(np.complex64)
    u = rng.uniform(size=4096).astype(np.float32)
    idx = sv.sample_declared(psi, u)
    np.savez(os.path.join(HERE, "sample_n12.npz"), psi=psi, u=u, idx=idx)


if __name__ == "__main__":
    c1()
    sample12()
    print("fixtures written to", HERE)
