"""CPU oracle for the warm-start network (test infrastructure only, see
oracle/__init__.py): float64 NumPy forward and backward of the dense GELU
network with the engine's bfloat16 rounding of hidden activations, the
periodic angle loss, Adam, and a dense exact-diagonalisation check of the
free-fermion ground energy.  The reference has no counterpart (its VQE
examples start from random angles); the formulas are the standard ones:
GELU in its tanh form, Adam with bias correction (Kingma & Ba, 2015)."""

from typing import List, Sequence, Tuple

import numpy as np

K0, K1 = np.sqrt(2.0 / np.pi), 0.044715


def bf16_round(x: np.ndarray) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest, ties to even), back as float64."""
    b = np.asarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    lsb = (b >> 16) & 1
    r = ((b + 0x7FFF + lsb) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def gelu(x: np.ndarray) -> np.ndarray:
    return 0.5 * x * (1.0 + np.tanh(K0 * (x + K1 * x ** 3)))


def gelu_grad(x: np.ndarray) -> np.ndarray:
    t = np.tanh(K0 * (x + K1 * x ** 3))
    return 0.5 * (1.0 + t) + 0.5 * x * (1.0 - t * t) * K0 * (1.0 + 3.0 * K1 * x * x)


def forward(x: np.ndarray, Ws: Sequence[np.ndarray], bs: Sequence[np.ndarray]) -> Tuple[np.ndarray, List]:
    h = np.asarray(x, dtype=np.float64)
    cache = []
    for i, (W, b) in enumerate(zip(Ws, bs)):
        z = h @ np.asarray(W, np.float64).T + np.asarray(b, np.float64)
        last = i == len(Ws) - 1
        cache.append((h, z))
        h = z if last else bf16_round(gelu(z))
    return h, cache


def periodic_loss(pred: np.ndarray, target: np.ndarray) -> Tuple[float, np.ndarray]:
    d = pred - target
    return float(np.mean(1.0 - np.cos(d))), np.sin(d) / d.size


def backward(dpred: np.ndarray, Ws: Sequence[np.ndarray], cache: List) -> Tuple[List[np.ndarray], List[np.ndarray]]:
    dW: List[np.ndarray] = [None] * len(Ws)  # type: ignore
    db: List[np.ndarray] = [None] * len(Ws)  # type: ignore
    dy = dpred
    for i in reversed(range(len(Ws))):
        h, z = cache[i]
        dz = dy if i == len(Ws) - 1 else dy * gelu_grad(z)
        dW[i] = dz.T @ h
        db[i] = dz.sum(0)
        dy = dz @ np.asarray(Ws[i], np.float64)
    return dW, db


def adam(p: np.ndarray, g: np.ndarray, m: np.ndarray, v: np.ndarray, step: int, lr: float,
         b1: float = 0.9, b2: float = 0.999, eps: float = 1e-8) -> None:
    m[:] = b1 * m + (1 - b1) * g
    v[:] = b2 * v + (1 - b2) * g * g
    p -= lr * (m / (1 - b1 ** step)) / (np.sqrt(v / (1 - b2 ** step)) + eps)


def tfim_dense_e0(J: Sequence[float], h: Sequence[float]) -> float:
    """Ground energy of H = -sum J_i Z_i Z_{i+1} - sum h_i X_i by dense
    diagonalisation (small n only)."""
    n = len(h)
    X = np.array([[0, 1], [1, 0]], dtype=np.float64)
    Z = np.diag([1.0, -1.0])

    def op(ms):
        out = np.ones((1, 1))
        for q in range(n):
            out = np.kron(out, ms.get(q, np.eye(2)))
        return out

    H = np.zeros((1 << n, 1 << n))
    for i in range(n - 1):
        H -= J[i] * op({i: Z, i + 1: Z})
    for i in range(n):
        H -= h[i] * op({i: X})
    return float(np.linalg.eigvalsh(H)[0])
