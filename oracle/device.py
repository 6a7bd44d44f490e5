"""Complex128 statevector oracle written with torch ops (test infrastructure,
see oracle/__init__.py).

The same restatement as ``oracle/statevector.py`` -- gate matrices from
``statevector.gate_matrix``, big-endian layout with gate leg i on qubit
index[i] (tensorcircuit/basecircuit.py:120-245, tests/test_circuit.py:21-44),
one contraction per gate in circuit order (the reference's per-gate
tensordot, tensorcircuit/cons.py:605-623), Pauli-string expectations
(tensorcircuit/abstractcircuit.py:1208-1288) and the state-level adjoint
value+gradient -- but on torch tensors, so that the checker runs on whatever
device holds the engine's result.  This is what makes complex128 checks
possible at the configured sizes: a 28-qubit complex128 state is 4 GiB and
a numpy sweep of 270 gates over it takes far too long for a test.

Pinned against ``oracle/statevector.py`` on the CPU (tests/test_oracle_kats.py).
"""

from typing import Any, Dict, Optional, Sequence, Tuple

import numpy as np
import torch

from . import statevector as sv

C128 = torch.complex128

_PAULI = {
    "x": np.array([[0, 1], [1, 0]], dtype=np.complex128),
    "y": np.array([[0, -1j], [1j, 0]], dtype=np.complex128),
    "z": np.array([[1, 0], [0, -1]], dtype=np.complex128),
}


def _as_matrix(m: Any, device: torch.device) -> torch.Tensor:
    if isinstance(m, torch.Tensor):
        return m.to(device=device, dtype=C128)
    return torch.as_tensor(np.asarray(m, dtype=np.complex128), device=device)


def apply_matrix(psi: torch.Tensor, m: Any, qubits: Sequence[int], n: int) -> torch.Tensor:
    """psi (2^n complex128, any device) -> M applied on `qubits` (first
    listed qubit = most significant bit of the gate's sub-index).

    The state is viewed with one dimension per gate qubit and one per run of
    other qubits between them (at most 2k+1 dimensions), the gate's input
    legs are contracted with those dimensions and its output legs moved back
    to the same positions."""
    k = len(qubits)
    qs = [int(q) % n for q in qubits]
    shape = []
    pos = {}
    prev = 0
    for q in sorted(qs):
        shape.append(1 << (q - prev))
        pos[q] = len(shape)
        shape.append(2)
        prev = q + 1
    shape.append(1 << (n - prev))
    t = psi.reshape(shape)
    g = _as_matrix(m, psi.device).reshape([2] * (2 * k))
    dims = [pos[q] for q in qs]
    t = torch.tensordot(g, t, dims=(list(range(k, 2 * k)), dims))
    t = torch.movedim(t, list(range(k)), dims)
    return t.reshape(-1)


def zero_state(n: int, device: Any) -> torch.Tensor:
    psi = torch.zeros(1 << n, dtype=C128, device=device)
    psi[0] = 1.0
    return psi


def run_circuit(n: int, ops: Sequence[Tuple[str, Sequence[int], Dict[str, Any]]], device: Any,
                psi0: Optional[torch.Tensor] = None) -> torch.Tensor:
    """Apply (name, qubits, params) gates in order to |0..0> (or psi0)."""
    psi = zero_state(n, device) if psi0 is None else psi0.to(device=device, dtype=C128).reshape(-1).clone()
    for name, qubits, params in ops:
        psi = apply_matrix(psi, sv.gate_matrix(name, **params), qubits, n)
    return psi


def pauli_apply(psi: torch.Tensor, n: int, x: Sequence[int] = (), y: Sequence[int] = (),
                z: Sequence[int] = ()) -> torch.Tensor:
    out = psi
    for lst, key in ((x, "x"), (y, "y"), (z, "z")):
        for q in lst:
            out = apply_matrix(out, _PAULI[key], [q], n)
    return out


def expectation_ps(psi: torch.Tensor, n: int, x: Sequence[int] = (), y: Sequence[int] = (),
                   z: Sequence[int] = ()) -> complex:
    seen = [int(q) % n for q in list(x) + list(y) + list(z)]
    if len(set(seen)) != len(seen):
        raise ValueError("Cannot measure two operators in one index")
    return complex(torch.vdot(psi, pauli_apply(psi, n, x, y, z)).item())


def energy(psi: torch.Tensor, n: int, terms: Sequence[Tuple[float, Dict[str, Sequence[int]]]]) -> float:
    return float(sum(c * expectation_ps(psi, n, **t).real for c, t in terms))


def hamiltonian_apply(psi: torch.Tensor, n: int,
                      terms: Sequence[Tuple[float, Dict[str, Sequence[int]]]]) -> torch.Tensor:
    out = torch.zeros_like(psi)
    for c, t in terms:
        out += c * pauli_apply(psi, n, **t)
    return out


def value_and_grad_adjoint(n: int, ops: Sequence[Tuple[str, Sequence[int], Dict[str, Any]]],
                           pidx: Sequence[Optional[int]], params: np.ndarray,
                           terms: Sequence[Tuple[float, Dict[str, Sequence[int]]]],
                           device: Any) -> Tuple[float, np.ndarray]:
    """Complex128 adjoint value+gradient of E(params) = <H>, the algorithm of
    ``statevector.value_and_grad_adjoint`` (dG/dtheta by a central
    difference of the gate matrix, exact to ~1e-10 for these trigonometric
    gates) on torch tensors."""
    params = np.asarray(params, dtype=np.float64)
    pops = sv._param_ops(ops, pidx, params)
    psi = run_circuit(n, pops, device)
    val = energy(psi, n, terms)
    lam = hamiltonian_apply(psi, n, terms)
    g = np.zeros_like(params)
    h = 1e-6
    for (name, q, p), k in zip(reversed(pops), reversed(list(pidx))):
        m = sv.gate_matrix(name, **p)
        psi = apply_matrix(psi, m.conj().T, q, n)
        if k is not None:
            pp = dict(p)
            pp["theta"] = p["theta"] + h
            mp = sv.gate_matrix(name, **pp)
            pp["theta"] = p["theta"] - h
            mm = sv.gate_matrix(name, **pp)
            dm = (mp - mm) / (2 * h)
            g[k] += 2.0 * torch.vdot(lam, apply_matrix(psi, dm, q, n)).real.item()
        lam = apply_matrix(lam, m.conj().T, q, n)
    return val, g
