"""Circuit templates and the synthetic workloads the engine is measured on.

Restates the reference's workload builders: ``QAOA_block``
(tensorcircuit/templates/blocks.py:84-110: ``exp1(zz, theta=gamma*w)`` on
every edge then ``rx(theta=beta)`` on every node), ``spin_glass_measurements``
(templates/measurements.py:290-335) and the MaxCut cost
(applications/graphdata.py:292-306).  Random regular graphs are drawn by a
seeded configuration model here (no networkx dependency); they follow the
same distribution family as ``networkx.random_regular_graph`` but are not the
same instances.

Workload generators return plain gate lists ``(name, qubits, params)`` so the
engine's Circuit and the CPU oracle build the same circuits.
"""

from typing import Any, Dict, List, Optional, Sequence, Tuple

import numpy as np
import torch

from . import gates as G

GateList = List[Tuple[str, Tuple[int, ...], Dict[str, Any]]]


# ------------------------------------------------------------------ ansatz
def hea_layout(n: int, nlayers: int) -> List[Tuple[str, Tuple[int, ...], int]]:
    """Hardware-efficient ansatz: per layer rx(theta) on every qubit, then
    rzz(phi) on the open chain (i, i+1).  Returns (name, qubits, param index);
    a layer uses 2n-1 parameters, e.g. n=10, 4 layers -> 76 and n=20,
    8 layers -> 312."""
    out = []
    per = 2 * n - 1
    for layer in range(nlayers):
        for i in range(n):
            out.append(("rx", (i,), layer * per + i))
        for i in range(n - 1):
            out.append(("rzz", (i, i + 1), layer * per + n + i))
    return out


def hea_nparams(n: int, nlayers: int) -> int:
    return nlayers * (2 * n - 1)


def apply_hea(c: Any, n: int, nlayers: int, params: Any) -> Any:
    # one unbind instead of a select per gate: under autograd its backward
    # is a single stack, where per-gate selects each scatter into a zero
    # tensor of all parameters
    ps = params.unbind(-1) if isinstance(params, torch.Tensor) and params.dim() == 1 else params
    for name, q, k in hea_layout(n, nlayers):
        getattr(c, name)(*q, theta=ps[k])
    return c


def hea_gate_list(n: int, nlayers: int, params: np.ndarray) -> GateList:
    return [(name, q, {"theta": float(params[k])}) for name, q, k in hea_layout(n, nlayers)]


def tfim_terms(n: int, jzz: float = 1.0, hx: float = 1.0) -> List[Tuple[float, Dict[str, List[int]]]]:
    """Open-chain TFIM as Pauli terms: sum jzz Z_i Z_{i+1} + sum hx X_i."""
    terms = [(jzz, {"z": [i, i + 1]}) for i in range(n - 1)]
    terms += [(hx, {"x": [i]}) for i in range(n)]
    return terms


def tfim_terms_random(J: Sequence[float], h: Sequence[float]) -> List[Tuple[float, Dict[str, List[int]]]]:
    """H = -sum J_i Z_i Z_{i+1} - sum h_i X_i (open chain)."""
    n = len(h)
    terms = [(-float(J[i]), {"z": [i, i + 1]}) for i in range(n - 1)]
    terms += [(-float(h[i]), {"x": [i]}) for i in range(n)]
    return terms


def energy(c: Any, terms: Sequence[Tuple[float, Dict[str, List[int]]]]) -> Any:
    """sum_t coef_t <P_t>, one expectation_ps call per term (the reference's
    VQE pattern, benchmarks/scripts/vqe_tc.py:75-81)."""
    import torch

    e = 0.0
    for coef, t in terms:
        e = e + coef * torch.real(c.expectation_ps(**t))
    return e


# -------------------------------------------------------------- brick wall
def haar_unitary(d: int, rng: np.random.Generator) -> np.ndarray:
    """Haar-random unitary: QR of a complex Gaussian with R's diagonal phases
    moved into Q."""
    z = (rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d))) / np.sqrt(2)
    q, r = np.linalg.qr(z)
    ph = np.diag(r) / np.abs(np.diag(r))
    return q * ph[None, :]


def brickwall_gate_list(n: int, depth: int, seed: int) -> GateList:
    """Depth-``depth`` brick wall of Haar 4x4 gates on alternating even/odd
    pairs (i, i+1); n=28, depth 20 gives 270 gates."""
    rng = np.random.default_rng(seed)
    out: GateList = []
    for layer in range(depth):
        for i in range(layer % 2, n - 1, 2):
            out.append(("any", (i, i + 1), {"unitary": haar_unitary(4, rng).astype(np.complex64)}))
    return out


def apply_gate_list(c: Any, gl: GateList) -> Any:
    for name, q, p in gl:
        getattr(c, name)(*q, **p)
    return c


# --------------------------------------------------------------------- QAOA
def random_regular_graph(d: int, n: int, rng: np.random.Generator) -> List[Tuple[int, int]]:
    """Uniform-ish random d-regular simple graph by the configuration model
    with restarts; needs n*d even (3-regular graphs need even n)."""
    if (n * d) % 2:
        raise ValueError("n * d must be even")
    for _ in range(10000):
        stubs = np.repeat(np.arange(n), d)
        rng.shuffle(stubs)
        pairs = stubs.reshape(-1, 2)
        a, b = np.minimum(pairs[:, 0], pairs[:, 1]), np.maximum(pairs[:, 0], pairs[:, 1])
        if np.any(a == b):
            continue
        key = a * n + b
        if len(np.unique(key)) != len(key):
            continue
        order = np.argsort(key)
        return [(int(a[i]), int(b[i])) for i in order]
    raise RuntimeError("could not draw a simple regular graph")


def qaoa_gate_list(n: int, edges: Sequence[Tuple[int, int]], gammas: Sequence[float],
                   betas: Sequence[float]) -> GateList:
    out: GateList = [("h", (i,), {}) for i in range(n)]
    for g, b in zip(gammas, betas):
        for e1, e2 in edges:
            out.append(("exp1", (e1, e2), {"unitary": G._zz_matrix, "theta": float(g)}))
        for i in range(n):
            out.append(("rx", (i,), {"theta": float(b)}))
    return out


def QAOA_block(c: Any, edges: Sequence[Tuple[int, int]], paramzz: Any, paramx: Any,
               nodes: Optional[Sequence[int]] = None) -> Any:
    """One QAOA layer with the reference's conventions (blocks.py:84-110)."""
    for e1, e2 in edges:
        c.exp1(e1, e2, unitary=G._zz_matrix, theta=paramzz)
    for i in (nodes if nodes is not None else range(c._nqubits)):
        c.rx(i, theta=paramx)
    return c


def maxcut_terms(edges: Sequence[Tuple[int, int]]) -> Tuple[float, List[Tuple[float, Dict[str, List[int]]]]]:
    """MaxCut energy sum_(ij) (1 - Z_i Z_j)/2 as (constant, terms)."""
    return 0.5 * len(edges), [(-0.5, {"z": [a, b]}) for a, b in edges]


def spin_glass_measurements(c: Any, edges: Sequence[Tuple[int, int, float]],
                            node_weights: Optional[Dict[int, float]] = None) -> Any:
    import torch

    loss = 0.0
    for e1, e2, w in edges:
        loss = loss + w * c.expectation_ps(z=[e1, e2])
    for v, w in (node_weights or {}).items():
        loss = loss + w * c.expectation_ps(z=[v])
    return torch.real(loss)


def qaoa_uneven_workload(count: int = 512, seed: int = 5, nmin: int = 12, nmax: int = 24,
                         pmax: int = 6) -> Tuple[List[Any], List[np.ndarray]]:
    """The uneven QAOA MaxCut batch: ``count`` circuits with n ~ U{nmin,
    nmin+2, ..., nmax} (3-regular graphs need even n), a random 3-regular
    graph each, depth p ~ U{1..pmax}, gamma, beta ~ U[0, pi) (float32).
    Returns (specs for tensorcircuit_gb300.batch.UnevenBatch, parameter
    vectors [gammas, betas])."""
    from .batch import qaoa_spec

    rng = np.random.default_rng(seed)
    specs, params = [], []
    for _ in range(count):
        n = int(rng.choice(np.arange(nmin, nmax + 1, 2)))
        p = int(rng.integers(1, pmax + 1))
        edges = random_regular_graph(3, n, np.random.default_rng(int(rng.integers(1 << 31))))
        specs.append(qaoa_spec(n, edges, p))
        params.append(rng.uniform(0, np.pi, 2 * p).astype(np.float32))
    return specs, params
