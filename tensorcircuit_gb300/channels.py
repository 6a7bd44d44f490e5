"""Quantum channels as Kraus lists, for Monte-Carlo trajectory noise.

Mirrors the reference's tensorcircuit/channels.py: every ``<name>channel``
function returns a :class:`KrausList` of :class:`Gate` objects, and
:class:`~tensorcircuit_gb300.Circuit` registers a ``<name>`` method for each
(circuit.py:727-764 of the reference): ``depolarizing`` and
``generaldepolarizing`` apply their operators through ``unitary_kraus``
(state-independent pick), the others through ``general_kraus``
(probabilities <psi|K^dag K|psi> from the current state).

Arguments may be Python numbers (the operators are numpy constants; the
engine keys its plans on their content) or torch tensors (the operators are
torch tensors and gradients flow to the channel parameters).
"""

import sys
from typing import Any, Dict, List, Optional, Sequence, Union

import numpy as np
import torch

from .gates import Gate

C64 = torch.complex64

_I = np.eye(2, dtype=np.complex128)
_X = np.array([[0, 1], [1, 0]], dtype=np.complex128)
_Y = np.array([[0, -1j], [1j, 0]], dtype=np.complex128)
_Z = np.array([[1, 0], [0, -1]], dtype=np.complex128)
_E00 = np.array([[1, 0], [0, 0]], dtype=np.complex128)
_E01 = np.array([[0, 1], [0, 0]], dtype=np.complex128)
_E10 = np.array([[0, 0], [1, 0]], dtype=np.complex128)
_E11 = np.array([[0, 0], [0, 1]], dtype=np.complex128)


class KrausList(list):  # type: ignore[type-arg]
    """A list of Kraus operators with the channel's name and whether the
    operators are multiples of unitaries (channels.py:25-30)."""

    def __init__(self, iterable: Any, name: str, is_unitary: bool) -> None:
        super().__init__(iterable)
        self.name = name
        self.is_unitary = is_unitary


def _is_t(*a: Any) -> bool:
    return any(isinstance(v, torch.Tensor) for v in a)


def _sqrt(a: Any) -> Any:
    """sqrt of a real probability, complex-typed (channels.py:32-46)."""
    if isinstance(a, torch.Tensor):
        return torch.sqrt(a.to(torch.float32)).to(C64)
    return complex(np.sqrt(float(a)))


_DEV: Dict[Any, torch.Tensor] = {}


def _dc(m: np.ndarray, dev: torch.device) -> torch.Tensor:
    """Device copy of a constant matrix, made once (a pageable host-to-device
    copy per call would wait for the stream)."""
    key = (id(m), str(dev))
    t = _DEV.get(key)
    if t is None:
        t = torch.as_tensor(m, dtype=C64, device=dev)
        _DEV[key] = t
    return t


def _scale(s: Any, m: np.ndarray) -> Any:
    if isinstance(s, torch.Tensor):
        return s * _dc(m, s.device)
    return s * m


def _gates(mats: Sequence[Any], k: int) -> List[Gate]:
    out = []
    for m in mats:
        shape = [2] * (2 * k)
        out.append(Gate(m.reshape(shape) if isinstance(m, torch.Tensor) else np.asarray(m).reshape(shape)))
    return out


def depolarizingchannel(px: Any, py: Any, pz: Any) -> KrausList:
    """sqrt(1-px-py-pz) I, sqrt(px) X, sqrt(py) Y, sqrt(pz) Z."""
    mats = [_scale(_sqrt(1 - px - py - pz), _I), _scale(_sqrt(px), _X), _scale(_sqrt(py), _Y),
            _scale(_sqrt(pz), _Z)]
    return KrausList(_gates(mats, 1), name="depolarizing", is_unitary=True)


def generaldepolarizingchannel(p: Union[float, Sequence[float]], num_qubits: int = 1) -> KrausList:
    """(1 - sum p) rho + sum_j p_j P_j rho P_j over the 4^k - 1 non-identity
    Pauli strings (channels.py:140-215); ``p`` a float gives every string
    the same weight.  Strings are ordered with the first qubit's Pauli as the
    outermost (slowest) index."""
    m = 4 ** num_qubits - 1
    if isinstance(p, float):
        probs = [1 - m * p] + m * [p]
    elif isinstance(p, (list, tuple)):
        if len(p) != m:
            raise ValueError("Invalid probability input %s" % (p,))
        probs = [1 - sum(p)] + list(p)
    else:
        raise ValueError("p should be float or list")
    if not np.all(np.array([float(q) for q in probs]) >= 0):
        raise ValueError("Invalid probability input %s" % (p,))
    paulis = [_I, _X, _Y, _Z]
    strings = list(paulis)
    for _ in range(num_qubits - 1):
        strings = [np.kron(a, b) for a in paulis for b in strings]
    mats = [_scale(_sqrt(q), s) for q, s in zip(probs, strings)]
    return KrausList(_gates(mats, num_qubits), name="depolarizing", is_unitary=True)


def isotropicdepolarizingchannel(p: float, num_qubits: int = 1) -> KrausList:
    """(1 - p) rho + p/(4^k - 1) sum_j P_j rho P_j (channels.py:104-138)."""
    return generaldepolarizingchannel(p / (4 ** num_qubits - 1), num_qubits)


def amplitudedampingchannel(gamma: Any, p: Any) -> KrausList:
    """Generalised amplitude damping (channels.py:217-268); p = 1 is plain
    amplitude damping."""
    sg, s1g = _sqrt(gamma), _sqrt(1 - gamma)
    sp, s1p = _sqrt(p), _sqrt(1 - p)
    if _is_t(gamma, p):
        dev = next(v.device for v in (gamma, p) if isinstance(v, torch.Tensor))
        t = lambda a: _dc(a, dev)  # noqa: E731
        m0 = sp * (t(_E00) + s1g * t(_E11))
        m1 = sp * (sg * t(_E01))
        m2 = s1p * (s1g * t(_E00) + t(_E11))
        m3 = s1p * (sg * t(_E10))
    else:
        m0 = sp * (_E00 + s1g * _E11)
        m1 = sp * (sg * _E01)
        m2 = s1p * (s1g * _E00 + _E11)
        m3 = s1p * (sg * _E10)
    return KrausList(_gates([m0, m1, m2, m3], 1), name="amplitude_damping", is_unitary=False)


def resetchannel() -> KrausList:
    """|0><0| and |0><1|: every trajectory ends in |0> (channels.py:270-295)."""
    return KrausList(_gates([_E00, _E01], 1), name="reset", is_unitary=False)


def phasedampingchannel(gamma: Any) -> KrausList:
    """diag(1, sqrt(1-gamma)) and diag(0, sqrt(gamma)) (channels.py:297-326)."""
    if isinstance(gamma, torch.Tensor):
        t = lambda a: _dc(a, gamma.device)  # noqa: E731
        m0 = t(_E00) + _sqrt(1 - gamma) * t(_E11)
        m1 = _sqrt(gamma) * t(_E11)
    else:
        m0 = _E00 + _sqrt(1 - gamma) * _E11
        m1 = _sqrt(gamma) * _E11
    return KrausList(_gates([m0, m1], 1), name="phase_damping", is_unitary=False)


def thermalrelaxationchannel(t1: float, t2: float, time: float, method: str = "ByChoi",
                             excitedstatepopulation: float = 0.0) -> KrausList:
    """T1/T2 relaxation over ``time`` (channels.py:328-463).

    ``ByKraus`` (valid for t2 <= t1, where the dephasing rate is at least
    the relaxation rate): identity, Z and the four reset operators with
    their probabilities; ``ByChoi``: the Kraus
    operators of the channel's Choi matrix (largest 4 eigenvectors, 3 when
    the excited population is 0 or 1); ``AUTO`` picks ByKraus when
    t1 > t2."""
    t1, t2, time = float(t1), float(t2), float(time)
    rate1, rate2 = 1.0 / t1, 1.0 / t2
    p_reset = 1 - np.exp(-time * rate1)
    exp_t2 = np.exp(-time * rate2)
    p0, p1 = 1 - excitedstatepopulation, excitedstatepopulation
    if method == "ByKraus" or (method == "AUTO" and t1 > t2):
        p_z = (1 - p_reset) * (1 - np.exp(-time * (rate2 - rate1))) / 2
        pr0, pr1 = p_reset * p0, p_reset * p1
        probs = [1 - p_z - pr0 - pr1, p_z, pr0, pr0, pr1, pr1]
        mats = [_I, _Z, _E00, _E01, _E10, _E11]
        return KrausList(_gates([_sqrt(q) * m for q, m in zip(probs, mats)], 1), name="thermal_relaxation",
                         is_unitary=False)
    if method == "ByChoi" or (method == "AUTO" and t2 >= t1):
        choi = np.zeros((4, 4), dtype=np.complex128)
        choi[0, 0] = 1 - p1 * p_reset
        choi[0, 3] = choi[3, 0] = exp_t2
        choi[1, 1] = p1 * p_reset
        choi[2, 2] = p0 * p_reset
        choi[3, 3] = 1 - p0 * p_reset
        nmax = 3 if (abs(excitedstatepopulation) < 1e-3 or abs(excitedstatepopulation - 1.0) < 1e-3) else 4
        ks = choi_to_kraus(choi, truncation_rules={"max_singular_values": nmax})
        return KrausList(_gates(ks, 1), name="thermal_relaxation", is_unitary=False)
    raise ValueError("No valid method is provided")


def choi_to_kraus(choi: Any, truncation_rules: Optional[Dict[str, Any]] = None) -> List[np.ndarray]:
    """Kraus operators sqrt(g_k) V_k from the eigenpairs (g_k, vec(V_k)) of a
    Choi matrix, largest first, with the column-major vectorisation of the
    reference (channels.py:657-737)."""
    c = np.asarray(choi, dtype=np.complex128)
    din = int(round(np.sqrt(c.shape[0])))
    dout = int(round(np.sqrt(c.shape[1])))
    if din * din != c.shape[0] or dout * dout != c.shape[1]:
        raise ValueError("The input must be a square number.")
    e, v = np.linalg.eigh(c)
    e = e.real
    v = v.T
    rules = truncation_rules or {}
    out = []
    nmax = rules.get("max_singular_values")
    if nmax is not None:
        for i in range(int(nmax)):
            out.append(np.sqrt(complex(e[-(i + 1)])) * v[-(i + 1)].reshape(dout, din).T)
    else:
        atol = rules.get("max_truncattion_err", 1e-5)
        for i in range(c.shape[0]):
            if e[-(i + 1)] > atol:
                out.append(np.sqrt(complex(e[-(i + 1)])) * v[-(i + 1)].reshape(dout, din).T)
    if not out:
        out.append(np.zeros((dout, din), dtype=np.complex128))
    return out


def kraus_identity_check(kraus: Sequence[Any]) -> None:
    """Assert sum_k K_k^dag K_k = I within 1e-5 (channels.py:490-516)."""
    ms = [_matrix(k) for k in kraus]
    acc = sum(m.conj().T @ m for m in ms)
    np.testing.assert_allclose(acc, np.eye(ms[0].shape[0]), atol=1e-5)


single_qubit_kraus_identity_check = kraus_identity_check


def _matrix(k: Any) -> np.ndarray:
    t = k.tensor if isinstance(k, Gate) else k
    if isinstance(t, torch.Tensor):
        t = t.detach().cpu().numpy()
    a = np.asarray(t, dtype=np.complex128)
    d = int(round(np.sqrt(a.size)))
    return a.reshape(d, d)


def _collect_channels() -> List[str]:
    mod = sys.modules[__name__]
    return sorted(name[:-7] for name in dir(mod) if name.endswith("channel") and not name.startswith("_"))


channels = _collect_channels()
UNITARY_CHANNELS = ("depolarizing", "generaldepolarizing")
