"""Reference-algorithm restatement for the CPU baseline (test / bench
infrastructure only, see oracle/__init__.py).

LABELLED RESTATEMENT, NOT TENSORCIRCUIT: the reference cannot be imported
here (its third-party ``tensornetwork`` dependency is absent), so its CPU path
for ``backend.vvag`` on the pytorch backend is restated in torch on the host:
gates are built with the reference's formulas (tensorcircuit/gates.py:579-594
rx, :825-865 rzz = exp1 with half angle), contracted one ``tensordot`` per gate
in circuit order (the ``plain`` contractor semantics, tensorcircuit/cons.py:
334-370), the energy is a sum of per-term Pauli sandwiches on the cached
state (basecircuit.py:267-319), and value+gradient is
``torch.vmap(torch.func.grad_and_value(f))`` with taped reverse-mode AD
(tensorcircuit/backends/pytorch_backend.py:533-544, 605-617, 673-709).
"""

from typing import Any, Dict, List, Sequence, Tuple

import numpy as np
import torch

C64 = torch.complex64


def _rx(theta: torch.Tensor) -> torch.Tensor:
    c = torch.cos(theta / 2).to(C64)
    s = torch.sin(theta / 2).to(C64)
    i2 = torch.eye(2, dtype=C64, device=theta.device)
    x = torch.tensor([[0, 1], [1, 0]], dtype=C64, device=theta.device)
    return c * i2 - 1j * s * x


def _rzz(theta: torch.Tensor) -> torch.Tensor:
    c = torch.cos(theta / 2).to(C64)
    s = torch.sin(theta / 2).to(C64)
    zz = torch.diag(torch.tensor([1, -1, -1, 1], dtype=C64, device=theta.device))
    return (c * torch.eye(4, dtype=C64, device=theta.device) - 1j * s * zz).reshape(2, 2, 2, 2)


_PAULI = {
    "x": torch.tensor([[0, 1], [1, 0]], dtype=C64),
    "y": torch.tensor([[0, -1j], [1j, 0]], dtype=C64),
    "z": torch.tensor([[1, 0], [0, -1]], dtype=C64),
}


def _apply(psi: torch.Tensor, g: torch.Tensor, qubits: Sequence[int]) -> torch.Tensor:
    k = len(qubits)
    out = torch.tensordot(g, psi, dims=(list(range(k, 2 * k)), list(qubits)))
    return torch.movedim(out, list(range(k)), list(qubits))


def hea_energy_fn(n: int, layout: Sequence[Tuple[str, Tuple[int, ...], int]],
                  terms: Sequence[Tuple[float, Dict[str, List[int]]]], device: str = "cpu") -> Any:
    psi0 = torch.zeros([2] * n, dtype=C64, device=device)
    psi0.view(-1)[0] = 1.0
    paulis = {k: v.to(device) for k, v in _PAULI.items()}

    def f(params: torch.Tensor) -> torch.Tensor:
        psi = psi0
        for name, q, k in layout:
            g = _rx(params[k]) if name == "rx" else _rzz(params[k])
            psi = _apply(psi, g, q)
        e = torch.zeros((), dtype=torch.float32, device=device)
        for coef, t in terms:
            phi = psi
            for kind, qs in t.items():
                for qq in qs:
                    phi = _apply(phi, paulis[kind], (qq,))
            e = e + coef * torch.real(torch.sum(torch.conj(psi) * phi))
        return e

    return f


def vvag_hea(n: int, layout: Sequence[Tuple[str, Tuple[int, ...], int]],
             terms: Sequence[Tuple[float, Dict[str, List[int]]]], params: np.ndarray,
             threads: int, device: str = "cpu") -> Tuple[np.ndarray, np.ndarray]:
    """``device="cuda"`` runs the same taped-AD restatement on the GPU (the
    reference's pytorch backend placed on the GPU)."""
    torch.set_num_threads(threads)
    f = hea_energy_fn(n, layout, terms, device)
    vg = torch.func.vmap(torch.func.grad_and_value(f))
    g, v = vg(torch.as_tensor(params, dtype=torch.float32, device=device))
    return v.cpu().numpy(), g.cpu().numpy()


def run_gate_list(n: int, gl: Sequence[Tuple[str, Tuple[int, ...], Dict[str, Any]]], threads: int) -> torch.Tensor:
    """Forward-only: constant-matrix gates (``any``/unitary, e.g. the Haar
    brick wall) contracted one ``tensordot`` per gate in circuit order, the
    reference's per-gate contraction on a complex64 state."""
    torch.set_num_threads(threads)
    psi = torch.zeros([2] * n, dtype=C64)
    psi.view(-1)[0] = 1.0
    for name, q, p in gl:
        if name not in ("any", "unitary"):
            raise NotImplementedError(name)
        k = len(q)
        g = torch.as_tensor(np.asarray(p["unitary"], dtype=np.complex64)).reshape([2] * (2 * k))
        psi = _apply(psi, g, q)
    return psi.reshape(-1)


def run_gate_list_numpy(n: int, gl: Sequence[Tuple[str, Tuple[int, ...], Dict[str, Any]]]) -> np.ndarray:
    """The same forward contraction on numpy arrays: one ``numpy.tensordot``
    per gate in circuit order on a complex64 state, as the reference's numpy
    backend runs it (tensorcircuit/backends/numpy_backend.py:12-16 builds on
    tensornetwork's NumPy backend, whose tensordot is ``numpy.tensordot``;
    the plain contractor's order, tensorcircuit/cons.py:334-370)."""
    psi = np.zeros([2] * n, dtype=np.complex64)
    psi.reshape(-1)[0] = 1.0
    for name, q, p in gl:
        if name not in ("any", "unitary"):
            raise NotImplementedError(name)
        k = len(q)
        g = np.asarray(p["unitary"], dtype=np.complex64).reshape([2] * (2 * k))
        out = np.tensordot(g, psi, axes=(list(range(k, 2 * k)), list(q)))
        psi = np.moveaxis(out, list(range(k)), list(q))
    return np.ascontiguousarray(psi).reshape(-1)


def _exp1_zz(theta: torch.Tensor) -> torch.Tensor:
    """exp1(ZZ, theta) = cos(theta) I - i sin(theta) ZZ (tensorcircuit/gates.py:825-846, half=False)."""
    c = torch.cos(theta).to(C64)
    s = torch.sin(theta).to(C64)
    zz = torch.diag(torch.tensor([1, -1, -1, 1], dtype=C64))
    return (c * torch.eye(4, dtype=C64) - 1j * s * zz).reshape(2, 2, 2, 2)


def qaoa_value_and_grad(n: int, edges: Sequence[Tuple[int, int]], p: int, params: np.ndarray,
                        threads: int) -> Tuple[float, np.ndarray]:
    """MaxCut QAOA energy sum_(ij) (1 - <Z_i Z_j>)/2 and its gradient for one
    circuit, per-gate tensordot in circuit order with taped reverse-mode AD
    (the reference's ``K.value_and_grad`` on the pytorch backend,
    tensorcircuit/backends/pytorch_backend.py:533-544; circuit from
    tensorcircuit/templates/blocks.py:84-110)."""
    torch.set_num_threads(threads)
    h = torch.tensor([[1, 1], [1, -1]], dtype=C64) / np.sqrt(2)
    z = _PAULI["z"]

    def f(prm: torch.Tensor) -> torch.Tensor:
        psi = torch.zeros([2] * n, dtype=C64)
        psi.view(-1)[0] = 1.0
        for i in range(n):
            psi = _apply(psi, h, (i,))
        for layer in range(p):
            g = _exp1_zz(prm[layer])
            for a, b in edges:
                psi = _apply(psi, g, (a, b))
            r = _rx(prm[p + layer])
            for i in range(n):
                psi = _apply(psi, r, (i,))
        e = torch.zeros((), dtype=torch.float32)
        for a, b in edges:
            phi = _apply(_apply(psi, z, (a,)), z, (b,))
            e = e + 0.5 * (1.0 - torch.real(torch.sum(torch.conj(psi) * phi)))
        return e

    g, v = torch.func.grad_and_value(f)(torch.as_tensor(params, dtype=torch.float32))
    return float(v), g.numpy()


def _pick_sign_rule(x: float, cum: Sequence[float]) -> int:
    """int(sum_{i<l-1} sign(x - c_i) / 2 + (l - 1) / 2)
    (tensorcircuit/circuit.py:541-556)."""
    l = len(cum)
    s = sum(float(np.sign(np.float32(x) - np.float32(c))) for c in cum[: l - 1])
    return int(s / 2.0 + (l - 1) / 2.0)


def mcnoise_value_and_grad(n: int, nlayer: int, gamma: float, params: np.ndarray, status: np.ndarray,
                           threads: int) -> Tuple[float, np.ndarray]:
    """One Monte-Carlo trajectory of the phase-damping circuit of
    examples/mcnoise_boost_v2.py:20-37 (H on all; per layer cnot(i, i+1)
    then phase damping on i and i+1 through general_kraus, then rx on every
    qubit; <Z_{n/2}>), value and gradient by taped AD.  general_kraus as
    tensorcircuit/circuit.py:635-694: p_k = ||K_k psi||^2 by contraction, the
    sign-rule pick, K_r psi / (sqrt(p_r) + 1e-10)."""
    torch.set_num_threads(threads)
    h = torch.tensor([[1, 1], [1, -1]], dtype=C64) / np.sqrt(2)
    cnot = torch.tensor([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0]], dtype=C64).reshape(2, 2, 2, 2)
    k0 = torch.tensor([[1, 0], [0, np.sqrt(1 - gamma)]], dtype=C64)
    k1 = torch.tensor([[0, 0], [0, np.sqrt(gamma)]], dtype=C64)
    z = _PAULI["z"]

    def f(prm: torch.Tensor) -> torch.Tensor:
        psi = torch.zeros([2] * n, dtype=C64)
        psi.view(-1)[0] = 1.0
        for i in range(n):
            psi = _apply(psi, h, (i,))
        s = 0
        for j in range(nlayer):
            for i in range(n - 1):
                psi = _apply(psi, cnot, (i, i + 1))
                for q in (i, i + 1):
                    v = [_apply(psi, k0, (q,)), _apply(psi, k1, (q,))]
                    p = [torch.real(torch.sum(torch.conj(t) * t)) for t in v]
                    cum = np.cumsum([float(t.detach()) for t in p], dtype=np.float32)
                    r = _pick_sign_rule(float(status[s]), cum)
                    psi = v[r] / (torch.sqrt(p[r]) + 1e-10).to(C64)
                    s += 1
            for i in range(n):
                psi = _apply(psi, _rx(prm[j, i]), (i,))
        phi = _apply(psi, z, (n // 2,))
        return torch.real(torch.sum(torch.conj(psi) * phi))

    g, v = torch.func.grad_and_value(f)(torch.as_tensor(params, dtype=torch.float32))
    return float(v), g.numpy()


def dm_value_and_grad(n: int, nlayers: int, p: float, params: np.ndarray, threads: int) -> Tuple[float, np.ndarray]:
    """Noisy HEA on a density matrix, the reference's DMCircuit2 algorithm
    (tensorcircuit/densitymatrix.py:331-366): rho as a [2]*2n tensor, each
    gate contracted on the row legs and its conjugate on the column legs, the
    depolarizing channel (channels.py:56-102) as the superoperator
    sum_i K_i (x) conj(K_i) contracted on (row, column) legs; per layer rx on
    every qubit, rzz on the open chain, depolarizing(p, p, p) on every qubit;
    energy sum <Z_i Z_i+1> + sum <X_i> = tr(rho H); taped AD."""
    torch.set_num_threads(threads)
    x = _PAULI["x"]
    z = _PAULI["z"]
    ks = [np.sqrt(1 - 3 * p) * np.eye(2), np.sqrt(p) * np.array([[0, 1], [1, 0]]),
          np.sqrt(p) * np.array([[0, -1j], [1j, 0]]), np.sqrt(p) * np.array([[1, 0], [0, -1]])]
    sup = torch.tensor(sum(np.kron(k, np.conj(k)) for k in ks), dtype=C64).reshape(2, 2, 2, 2)

    def both(rho: torch.Tensor, g: torch.Tensor, q: Sequence[int]) -> torch.Tensor:
        rho = _apply(rho, g, q)
        return _apply(rho, torch.conj(g), [i + n for i in q])

    def f(prm: torch.Tensor) -> torch.Tensor:
        rho = torch.zeros([2] * (2 * n), dtype=C64)
        rho.view(-1)[0] = 1.0
        k = 0
        for _ in range(nlayers):
            for i in range(n):
                rho = both(rho, _rx(prm[k]), (i,))
                k += 1
            for i in range(n - 1):
                rho = both(rho, _rzz(prm[k]), (i, i + 1))
                k += 1
            for i in range(n):
                rho = _apply(rho, sup, (i, i + n))
        m = rho.reshape(1 << n, 1 << n)
        e = torch.zeros((), dtype=torch.float32)
        for i in range(n - 1):
            op = _apply(_apply(rho, z, (i,)), z, (i + 1,)).reshape(1 << n, 1 << n)
            e = e + torch.real(torch.trace(op))
        for i in range(n):
            e = e + torch.real(torch.trace(_apply(rho, x, (i,)).reshape(1 << n, 1 << n)))
        del m
        return e

    g, v = torch.func.grad_and_value(f)(torch.as_tensor(params, dtype=torch.float32))
    return float(v), g.numpy()
