"""Monte-Carlo trajectory noise oracle (test infrastructure; only tests/,
``__graft_entry__.smoke()`` and bench.py's CPU legs import it -- the engine
never does).

Restates, in complex128 numpy, independently of the engine package:

* the Kraus sets of the reference's channels (tensorcircuit/channels.py):
  depolarizing :56-102, isotropic depolarizing :104-138, general
  depolarizing :140-215, amplitude damping :217-268, reset :270-295, phase
  damping :297-326, thermal relaxation (the ``ByKraus`` branch) :328-398;
* the pick rule of ``unitary_kraus`` (tensorcircuit/circuit.py:513-560):
  without ``prob`` the probabilities are tr(K^dag K)/d and every operator is
  divided by sqrt(p); with cumulative sums c_i the pick for a uniform x is
  int(sum_{i<l-1} sign(x - c_i) / 2 + (l - 1) / 2), i.e. the number of c_i
  strictly below x plus half the number equal to x, truncated;
* ``general_kraus`` (circuit.py:635-694): p_i = <psi|K_i^dag K_i|psi>, the
  operators rescaled by 1/(sqrt(p_i) + 1e-10), then the unitary_kraus pick
  with those probabilities.
"""

from typing import Any, List, Optional, Sequence, Tuple

import numpy as np

from . import statevector as sv

C = np.complex128
I2 = np.eye(2, dtype=C)
PAULIS = [I2, sv.X, sv.Y, sv.Z]


# ------------------------------------------------------------------ channels
def depolarizing(px: float, py: float, pz: float) -> List[np.ndarray]:
    return [np.sqrt(1 - px - py - pz) * I2, np.sqrt(px) * sv.X, np.sqrt(py) * sv.Y, np.sqrt(pz) * sv.Z]


def general_depolarizing(p: Any, num_qubits: int = 1) -> List[np.ndarray]:
    m = 4 ** num_qubits - 1
    probs = [1 - m * p] + m * [p] if isinstance(p, float) else [1 - sum(p)] + list(p)
    mats = list(PAULIS)
    for _ in range(num_qubits - 1):
        mats = [np.kron(a, b) for a in PAULIS for b in mats]
    return [np.sqrt(q) * m_ for q, m_ in zip(probs, mats)]


def amplitude_damping(gamma: float, p: float) -> List[np.ndarray]:
    return [np.sqrt(p) * np.array([[1, 0], [0, np.sqrt(1 - gamma)]], dtype=C),
            np.sqrt(p) * np.array([[0, np.sqrt(gamma)], [0, 0]], dtype=C),
            np.sqrt(1 - p) * np.array([[np.sqrt(1 - gamma), 0], [0, 1]], dtype=C),
            np.sqrt(1 - p) * np.array([[0, 0], [np.sqrt(gamma), 0]], dtype=C)]


def reset() -> List[np.ndarray]:
    return [np.array([[1, 0], [0, 0]], dtype=C), np.array([[0, 1], [0, 0]], dtype=C)]


def phase_damping(gamma: float) -> List[np.ndarray]:
    return [np.array([[1, 0], [0, np.sqrt(1 - gamma)]], dtype=C), np.array([[0, 0], [0, np.sqrt(gamma)]], dtype=C)]


def thermal_relaxation_bykraus(t1: float, t2: float, time: float, pop1: float = 0.0) -> List[np.ndarray]:
    p_reset = 1 - np.exp(-time / t1)
    p0, p1 = 1 - pop1, pop1
    p_z = (1 - p_reset) * (1 - np.exp(-time * (1 / t2 - 1 / t1))) / 2
    probs = [1 - p_z - p_reset * p0 - p_reset * p1, p_z, p_reset * p0, p_reset * p0, p_reset * p1, p_reset * p1]
    mats = [I2, sv.Z, np.array([[1, 0], [0, 0]], dtype=C), np.array([[0, 1], [0, 0]], dtype=C),
            np.array([[0, 0], [1, 0]], dtype=C), np.array([[0, 0], [0, 1]], dtype=C)]
    return [np.sqrt(q) * m for q, m in zip(probs, mats)]


def identity_defect(kraus: Sequence[np.ndarray]) -> float:
    """max |sum K^dag K - I| (channels.py:490-516 asserts it below 1e-5)."""
    d = kraus[0].shape[0]
    acc = sum(k.conj().T @ k for k in kraus)
    return float(np.max(np.abs(acc - np.eye(d))))


# --------------------------------------------------------------------- picks
def pick(x: float, prob: Sequence[float], dtype: Any = np.float32) -> int:
    """unitary_kraus's step function in the given float type."""
    x = dtype(x)
    cum = np.cumsum(np.asarray(prob, dtype=dtype)).astype(dtype)
    l = len(prob)
    if l == 1:
        return 0
    s = float(np.sum(np.sign(x - cum[: l - 1])))
    return int(s / 2.0 + (l - 1) / 2.0)


def unitary_kraus(psi: np.ndarray, n: int, kraus: Sequence[np.ndarray], qubits: Sequence[int],
                  x: float, prob: Optional[Sequence[float]] = None) -> Tuple[np.ndarray, int]:
    ks = [np.asarray(k, dtype=C) for k in kraus]
    if prob is None:
        prob = [float(np.real(np.trace(k.conj().T @ k)) / k.shape[0]) for k in ks]
        ks = [k / np.sqrt(p) for k, p in zip(ks, prob)]
    r = pick(x, prob)
    return sv.apply_matrix(psi, ks[r], list(qubits), n), r


def kraus_probs(psi: np.ndarray, n: int, kraus: Sequence[np.ndarray], qubits: Sequence[int]) -> np.ndarray:
    return np.array([np.vdot(v, v).real for v in
                     (sv.apply_matrix(psi, np.asarray(k, dtype=C), list(qubits), n) for k in kraus)])


def general_kraus(psi: np.ndarray, n: int, kraus: Sequence[np.ndarray], qubits: Sequence[int],
                  x: float) -> Tuple[np.ndarray, int, np.ndarray]:
    p = kraus_probs(psi, n, kraus, qubits)
    ks = [np.asarray(k, dtype=C) / (np.sqrt(w) + 1e-10) for k, w in zip(kraus, p)]
    r = pick(x, p)
    return sv.apply_matrix(psi, ks[r], list(qubits), n), r, p


def run_noisy(n: int, ops: Sequence[Tuple[str, Sequence[int], Any]],
              psi0: Optional[np.ndarray] = None) -> Tuple[np.ndarray, List[int]]:
    """Gate list with noise entries: ("unitary_kraus", qubits, dict(kraus=,
    status=, prob=)) and ("general_kraus", qubits, dict(kraus=, status=)) next
    to ordinary (name, qubits, params) gates.  Returns the final state and the
    picks in order."""
    if psi0 is None:
        psi = np.zeros(1 << n, dtype=C)
        psi[0] = 1.0
    else:
        psi = np.asarray(psi0, dtype=C).reshape(-1).copy()
    picks = []
    for name, q, p in ops:
        if name == "unitary_kraus":
            psi, r = unitary_kraus(psi, n, p["kraus"], q, p["status"], p.get("prob"))
            picks.append(r)
        elif name == "general_kraus":
            psi, r, _ = general_kraus(psi, n, p["kraus"], q, p["status"])
            picks.append(r)
        else:
            psi = sv.apply_matrix(psi, sv.gate_matrix(name, **p), [int(i) % n for i in q], n)
    return psi, picks
