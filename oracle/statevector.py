"""Complex128 statevector oracle (test infrastructure, see oracle/__init__.py).

Restates, independently of the engine package:

* gate matrices: tensorcircuit/gates.py:26-127 (constants), :463-865
  (phase, u, r, rx/ry/rz, iswap, cr, any, exp, exp1, rzz/rxx/ryy), :294-331
  (controlled / ocontrolled), :949-982 (registration of sd/td/ox/...);
* big-endian layout, gate leg i on qubit index[i]: tensorcircuit/
  basecircuit.py:120-245 and tests/test_circuit.py:21-44;
* expectation_ps / expectation: tensorcircuit/abstractcircuit.py:1208-1288,
  basecircuit.py:267-319 (duplicate index -> ValueError);
* probability = |psi|^2: basecircuit.py:510-523;
* sampling: abstract_backend.py:1124-1157 (p/sum, cumsum, cdf[-1]*(1-u),
  left searchsorted) in two arithmetics: ``sample_reference_fp32`` (the
  reference's literal float32 path) and ``sample_declared`` (the engine's
  declared integer CDF, bit-exact target);
* vvag contract: abstract_backend.py:1706-1756 (values [B], grads [B, ...],
  non-vectorised argnums summed over the batch).
"""

from typing import Any, Dict, List, Optional, Sequence, Tuple

import numpy as np

C = np.complex128

I2 = np.eye(2, dtype=C)
X = np.array([[0, 1], [1, 0]], dtype=C)
Y = np.array([[0, -1j], [1j, 0]], dtype=C)
Z = np.array([[1, 0], [0, -1]], dtype=C)
H = np.array([[1, 1], [1, -1]], dtype=C) / np.sqrt(2)
S = np.array([[1, 0], [0, 1j]], dtype=C)
T = np.array([[1, 0], [0, np.exp(1j * np.pi / 4)]], dtype=C)
WROOT = np.array([[1, -(1 + 1j) / np.sqrt(2)], [(1 - 1j) / np.sqrt(2), 1]], dtype=C) / np.sqrt(2)


def _ctrl(u: np.ndarray) -> np.ndarray:
    d = u.shape[0]
    out = np.zeros((2 * d, 2 * d), dtype=C)
    out[:d, :d] = np.eye(d)
    out[d:, d:] = u
    return out


def _octrl(u: np.ndarray) -> np.ndarray:
    d = u.shape[0]
    out = np.zeros((2 * d, 2 * d), dtype=C)
    out[:d, :d] = u
    out[d:, d:] = np.eye(d)
    return out


def _perm(n: int, a: int, b: int) -> np.ndarray:
    m = np.eye(n, dtype=C)
    m[[a, b]] = m[[b, a]]
    return m


CONST: Dict[str, np.ndarray] = {
    "i": I2, "x": X, "y": Y, "z": Z, "h": H, "s": S, "t": T, "wroot": WROOT,
    "sd": S.conj().T, "td": T.conj().T,
    "cnot": _ctrl(X), "cz": _ctrl(Z), "cy": _ctrl(Y), "swap": _perm(4, 1, 2),
    "ox": _octrl(X), "oy": _octrl(Y), "oz": _octrl(Z),
    "toffoli": _perm(8, 6, 7), "fredkin": _perm(8, 5, 6),
}
ALIASES = {"cx": "cnot", "cswap": "fredkin", "ccnot": "toffoli", "ccx": "toffoli", "unitary": "any",
           "sdg": "sd", "tdg": "td"}


def rot(p: np.ndarray, theta: float) -> np.ndarray:
    """cos(theta/2) I - i sin(theta/2) P."""
    d = p.shape[0]
    return np.cos(theta / 2) * np.eye(d, dtype=C) - 1j * np.sin(theta / 2) * p


def exp1(u: np.ndarray, theta: float, half: bool = False) -> np.ndarray:
    t = theta / 2 if half else theta
    return np.cos(t) * np.eye(u.shape[0], dtype=C) - 1j * np.sin(t) * u


def r_mat(theta: float, alpha: float, phi: float) -> np.ndarray:
    return (np.cos(theta) * I2 - 1j * np.cos(phi) * np.sin(alpha) * np.sin(theta) * X
            - 1j * np.sin(phi) * np.sin(alpha) * np.sin(theta) * Y - 1j * np.sin(theta) * np.cos(alpha) * Z)


def u_mat(theta: float, phi: float, lbd: float) -> np.ndarray:
    c, s = np.cos(theta / 2), np.sin(theta / 2)
    return np.array([[c, -np.exp(1j * lbd) * s], [np.exp(1j * phi) * s, np.exp(1j * (phi + lbd)) * c]], dtype=C)


def phase_mat(theta: float) -> np.ndarray:
    return np.array([[1, 0], [0, np.exp(1j * theta)]], dtype=C)


def iswap_mat(theta: float = 1.0) -> np.ndarray:
    c, s = np.cos(np.pi * theta / 2), np.sin(np.pi * theta / 2)
    return np.array([[1, 0, 0, 0], [0, c, 1j * s, 0], [0, 1j * s, c, 0], [0, 0, 0, 1]], dtype=C)


def expm_herm(u: np.ndarray, theta: float) -> np.ndarray:
    w, v = np.linalg.eigh((u + u.conj().T) / 2) if np.allclose(u, u.conj().T) else (None, None)
    if w is not None:
        return (v * np.exp(-1j * theta * w)) @ v.conj().T
    import scipy.linalg

    return scipy.linalg.expm(-1j * theta * u)


def _f(v: Any) -> Any:
    a = np.asarray(v)
    return complex(a) if np.iscomplexobj(a) else float(a)


def gate_matrix(name: str, **p: Any) -> np.ndarray:
    """Matrix M[out, in] of a named gate, first qubit = most significant."""
    name = ALIASES.get(name, name)
    if name in CONST:
        return CONST[name]
    th = _f(p.get("theta", 0.0))
    if name == "rx":
        return rot(X, th)
    if name == "ry":
        return rot(Y, th)
    if name == "rz":
        return rot(Z, th)
    if name == "rxx":
        return exp1(np.kron(X, X), th, True)
    if name == "ryy":
        return exp1(np.kron(Y, Y), th, True)
    if name == "rzz":
        return exp1(np.kron(Z, Z), th, True)
    if name == "phase":
        return phase_mat(th)
    if name == "r":
        return r_mat(th, _f(p.get("alpha", 0.0)), _f(p.get("phi", 0.0)))
    if name == "u":
        return u_mat(th, _f(p.get("phi", 0.0)), _f(p.get("lbd", 0.0)))
    if name == "iswap":
        return iswap_mat(_f(p.get("theta", 1.0)))
    if name in ("crx", "cry", "crz"):
        return _ctrl(gate_matrix(name[1:], theta=th))
    if name in ("orx", "ory", "orz"):
        return _octrl(gate_matrix(name[1:], theta=th))
    if name == "cphase":
        return _ctrl(phase_mat(th))
    if name == "cr":
        return _ctrl(r_mat(th, _f(p.get("alpha", 0.0)), _f(p.get("phi", 0.0))))
    if name == "cu":
        return _ctrl(u_mat(th, _f(p.get("phi", 0.0)), _f(p.get("lbd", 0.0))))
    if name in ("any", "exp1", "exp"):
        u = np.asarray(p["unitary"], dtype=C)
        d = int(round(np.sqrt(u.size)))
        u = u.reshape(d, d)
        if name == "any":
            return u
        if name == "exp1":
            return exp1(u, th, bool(p.get("half", False)))
        return expm_herm(u, th)
    raise KeyError(name)


def apply_matrix(psi: np.ndarray, m: np.ndarray, qubits: Sequence[int], n: int) -> np.ndarray:
    k = len(qubits)
    t = psi.reshape([2] * n)
    g = m.reshape([2] * (2 * k))
    t = np.tensordot(g, t, axes=(list(range(k, 2 * k)), list(qubits)))
    # tensordot puts the k output legs first: move them back to their qubits
    t = np.moveaxis(t, list(range(k)), list(qubits))
    return t.reshape(-1)


def run_circuit(n: int, ops: Sequence[Tuple[str, Sequence[int], Dict[str, Any]]],
                psi0: Optional[np.ndarray] = None) -> np.ndarray:
    """Apply (name, qubits, params) gates in order to |0..0> (or psi0)."""
    if psi0 is None:
        psi = np.zeros(1 << n, dtype=C)
        psi[0] = 1.0
    else:
        psi = np.asarray(psi0, dtype=C).reshape(-1).copy()
    for name, qubits, params in ops:
        q = [int(i) % n for i in qubits]
        if len(set(q)) != len(q):
            raise AssertionError("duplicate qubit")
        psi = apply_matrix(psi, gate_matrix(name, **params), q, n)
    return psi


def pauli_apply(psi: np.ndarray, n: int, x: Sequence[int] = (), y: Sequence[int] = (),
                z: Sequence[int] = ()) -> np.ndarray:
    out = psi
    for lst, m in ((x, X), (y, Y), (z, Z)):
        for q in lst:
            out = apply_matrix(out, m, [int(q) % n], n)
    return out


def expectation_ps(psi: np.ndarray, n: int, x: Sequence[int] = (), y: Sequence[int] = (),
                   z: Sequence[int] = ()) -> complex:
    seen = [int(q) % n for q in list(x) + list(y) + list(z)]
    if len(set(seen)) != len(seen):
        raise ValueError("Cannot measure two operators in one index")
    return complex(np.vdot(psi, pauli_apply(psi, n, x, y, z)))


def probability(psi: np.ndarray) -> np.ndarray:
    return np.abs(psi) ** 2


# ---------------------------------------------------------------- sampling
def qweight(x: np.ndarray) -> np.ndarray:
    """floor(x^2 * 2^60) from the exact fp32 bits of x (declared CDF weight)."""
    bits = np.asarray(x, dtype=np.float32).view(np.uint32) & np.uint32(0x7FFFFFFF)
    e = (bits >> np.uint32(23)).astype(np.int64)
    m = ((bits & np.uint32(0x7FFFFF)) | np.uint32(0x800000)).astype(np.uint64)
    m2 = m * m
    s = 2 * e - 240
    out = np.zeros(bits.shape, dtype=np.uint64)
    pos = (s >= 0) & (e > 0)
    neg = (s < 0) & (e > 0) & (s > -64)
    out[pos] = m2[pos] << np.minimum(s[pos], 15).astype(np.uint64)
    out[neg] = m2[neg] >> (-s[neg]).astype(np.uint64)
    return out


def declared_cdf(psi64: np.ndarray) -> np.ndarray:
    """Inclusive uint64 prefix sum of w(re) + w(im) over a complex64 state."""
    a = np.asarray(psi64, dtype=np.complex64)
    q = qweight(a.real) + qweight(a.imag)
    return np.cumsum(q, dtype=np.uint64)


def sample_declared(psi64: np.ndarray, u: np.ndarray) -> np.ndarray:
    """Engine's declared arithmetic: t = floor((1 - u) * total) in double,
    first index with cdf >= t, clamped to len - 1."""
    cdf = declared_cdf(psi64)
    total = cdf[-1]
    w = 1.0 - np.asarray(u, dtype=np.float32).astype(np.float64)
    t = np.floor(w * np.float64(total))
    t = np.where(t <= 0, 0, t).astype(np.uint64)
    idx = np.searchsorted(cdf, t, side="left")
    return np.minimum(idx, cdf.shape[0] - 1).astype(np.int64)


def sample_reference_fp32(p: np.ndarray, u: np.ndarray) -> np.ndarray:
    """The reference's literal float32 arithmetic (sequential cumsum)."""
    p = np.asarray(p, dtype=np.float32)
    p = p / np.sum(p, dtype=np.float32)
    cdf = np.cumsum(p, dtype=np.float32)
    r = cdf[-1] * (np.float32(1.0) - np.asarray(u, dtype=np.float32))
    return np.minimum(np.searchsorted(cdf, r, side="left"), p.shape[0] - 1)


def sample_int2bin(sample: np.ndarray, n: int) -> np.ndarray:
    return (np.asarray(sample)[..., None] >> np.arange(n - 1, -1, -1)) % 2


# ---------------------------------------------------------------- gradients
def energy(psi: np.ndarray, n: int, terms: Sequence[Tuple[float, Dict[str, Sequence[int]]]]) -> float:
    return float(sum(c * expectation_ps(psi, n, **t).real for c, t in terms))


def hamiltonian_apply(psi: np.ndarray, n: int, terms: Sequence[Tuple[float, Dict[str, Sequence[int]]]]) -> np.ndarray:
    out = np.zeros_like(psi)
    for c, t in terms:
        out += c * pauli_apply(psi, n, **t)
    return out


def _param_ops(ops: Sequence[Tuple[str, Sequence[int], Dict[str, Any]]], pidx: Sequence[Optional[int]],
               params: np.ndarray) -> List[Tuple[str, Sequence[int], Dict[str, Any]]]:
    out = []
    for (name, q, p), k in zip(ops, pidx):
        if k is not None:
            p = dict(p)
            p["theta"] = float(params[k])
        out.append((name, q, p))
    return out


def value_and_grad_adjoint(n: int, ops: Sequence[Tuple[str, Sequence[int], Dict[str, Any]]],
                           pidx: Sequence[Optional[int]], params: np.ndarray,
                           terms: Sequence[Tuple[float, Dict[str, Sequence[int]]]]) -> Tuple[float, np.ndarray]:
    """Exact complex128 adjoint value+gradient of E(params) = <H> for
    rotation gates whose ``theta`` is params[pidx[i]]: dG/dtheta via a
    central difference of the 2x2/4x4 matrix (exact to ~1e-10 for these
    trigonometric gates), state-level adjoint sweep."""
    params = np.asarray(params, dtype=np.float64)
    pops = _param_ops(ops, pidx, params)
    psi = run_circuit(n, pops)
    val = energy(psi, n, terms)
    lam = hamiltonian_apply(psi, n, terms)
    g = np.zeros_like(params)
    h = 1e-6
    for (name, q, p), k in zip(reversed(pops), reversed(list(pidx))):
        qq = [int(i) % n for i in q]
        m = gate_matrix(name, **p)
        psi = apply_matrix(psi, m.conj().T, qq, n)
        if k is not None:
            pp = dict(p)
            pp["theta"] = p["theta"] + h
            mp = gate_matrix(name, **pp)
            pp["theta"] = p["theta"] - h
            mm = gate_matrix(name, **pp)
            dm = (mp - mm) / (2 * h)
            g[k] += 2.0 * np.real(np.vdot(lam, apply_matrix(psi, dm, qq, n)))
        lam = apply_matrix(lam, m.conj().T, qq, n)
    return val, g


def grad_fd(n: int, ops: Sequence[Tuple[str, Sequence[int], Dict[str, Any]]], pidx: Sequence[Optional[int]],
            params: np.ndarray, terms: Sequence[Tuple[float, Dict[str, Sequence[int]]]],
            eps: float = 1e-3, which: Optional[Sequence[int]] = None) -> np.ndarray:
    """Central finite differences (complex128), optionally for a subset."""
    params = np.asarray(params, dtype=np.float64)
    which = range(params.size) if which is None else which
    g = np.zeros_like(params)
    for k in which:
        pp = params.copy()
        pp[k] += eps
        ep = energy(run_circuit(n, _param_ops(ops, pidx, pp)), n, terms)
        pp[k] -= 2 * eps
        em = energy(run_circuit(n, _param_ops(ops, pidx, pp)), n, terms)
        g[k] = (ep - em) / (2 * eps)
    return g
