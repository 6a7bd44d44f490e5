"""Density-matrix oracle (test infrastructure; only tests/ import it).

Restates in complex128 numpy what tensorcircuit/densitymatrix.py computes:
rho -> G rho G^dag for a gate (``_meta_apply`` gates acting on both the ket
and the bra legs, densitymatrix.py:134-138), rho -> sum_i K_i rho K_i^dag
for a channel (:179-202 and the superoperator form :332-366), tr(rho O) for
expectations, diag(rho) for probabilities, and the sequential measurement of
basecircuit.py:371-441 (pu = P(0 | earlier outcomes), outcome
sign(status - pu + eps)/2 + 1/2, eps = 0.31415926e-12).
"""

from typing import Any, Dict, List, Optional, Sequence, Tuple

import numpy as np

from . import statevector as sv

C = np.complex128


def apply_op(rho: np.ndarray, m: np.ndarray, qubits: Sequence[int], n: int) -> np.ndarray:
    """m rho m^dag with m on ``qubits``."""
    N = 1 << n
    # columns of rho are states: apply m to every column, then to every row
    r = np.stack([sv.apply_matrix(rho[:, j], m, qubits, n) for j in range(N)], axis=1)
    r = np.stack([sv.apply_matrix(r[i, :].conj(), m, qubits, n).conj() for i in range(N)], axis=0)
    return r


def apply_channel(rho: np.ndarray, kraus: Sequence[np.ndarray], qubits: Sequence[int], n: int) -> np.ndarray:
    return sum(apply_op(rho, np.asarray(k, dtype=C), qubits, n) for k in kraus)


def run_dm(n: int, ops: Sequence[Tuple[str, Sequence[int], Any]], rho0: Optional[np.ndarray] = None) -> np.ndarray:
    """Gate list with channel entries ("channel", qubits, [K_i]) next to
    ordinary (name, qubits, params) gates."""
    if rho0 is None:
        rho = np.zeros((1 << n, 1 << n), dtype=C)
        rho[0, 0] = 1.0
    else:
        rho = np.asarray(rho0, dtype=C).reshape(1 << n, 1 << n).copy()
    for name, q, p in ops:
        q = [int(i) for i in q]
        if name == "channel":
            rho = apply_channel(rho, p, q, n)
        else:
            rho = apply_op(rho, sv.gate_matrix(name, **p), q, n)
    return rho


def pauli_matrix(n: int, x: Sequence[int] = (), y: Sequence[int] = (), z: Sequence[int] = ()) -> np.ndarray:
    mats = [np.eye(2, dtype=C)] * n
    for lst, m in ((x, sv.X), (y, sv.Y), (z, sv.Z)):
        for q in lst:
            mats[int(q)] = m
    out = np.ones((1, 1), dtype=C)
    for m in mats:
        out = np.kron(out, m)
    return out


def expectation_ps(rho: np.ndarray, n: int, x: Sequence[int] = (), y: Sequence[int] = (),
                   z: Sequence[int] = ()) -> complex:
    return complex(np.trace(rho @ pauli_matrix(n, x, y, z)))


def measure_sequential(rho: np.ndarray, n: int, index: Sequence[int], status: Sequence[float]) -> Tuple[List[int], float]:
    p = np.real(np.diag(rho)).reshape([2] * n)
    bits: List[int] = []
    prob = 1.0
    for k, j in enumerate(index):
        sl = [slice(None)] * n
        for i, b in zip(index[:k], bits):
            sl[i] = b
        sub = p[tuple(sl)]
        # axes left in sub: the qubits not fixed yet, in order
        free = [q for q in range(n) if q not in index[:k]]
        ax = free.index(j)
        p0 = np.take(sub, 0, axis=ax).sum()
        pu = p0 / prob
        s = np.sign(status[k] - pu + 0.31415926e-12) / 2 + 0.5
        b = int(s > 0.5)
        bits.append(b)
        prob = prob * (pu if b == 0 else 1 - pu)
    return bits, prob
