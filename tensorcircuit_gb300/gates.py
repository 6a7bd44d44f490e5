"""Gate library: the reference's gate names, matrices and parameter conventions.

Conventions restated from ``tensorcircuit/gates.py``:

* constant matrices ``_x_matrix`` ... (tensorcircuit/gates.py:26-127);
* ``rx/ry/rz(theta) = cos(theta/2) I - i sin(theta/2) P`` (gates.py:579-636);
* ``exp1(U, theta, half) = cos(t) I - i sin(t) U`` with ``t = theta/2`` when
  ``half`` (gates.py:825-865); ``rzz/rxx/ryy`` are ``exp1`` with ``half=True``;
* ``exp(U, theta) = expm(-i theta U)`` (gates.py:787-812);
* ``r``, ``u``, ``phase``, ``iswap``, ``cr`` (gates.py:463-770);
* ``controlled`` puts U in the lower-right block, ``ocontrolled`` in the
  upper-left block, the control being the first listed qubit
  (gates.py:294-331); ``sd/td`` are adjoints of ``s/t``.

Every parameterized family has a vectorised torch builder: given the stacked
parameters of all G gates of that family in a circuit it returns their
matrices as one ``[G, E]`` complex64 tensor (E = 4^k dense entries, or 2^k
diagonal entries for diagonal gates).  Building the matrices with torch ops
keeps them differentiable: the engine's adjoint kernel returns the cotangent
of each matrix entry and torch maps it back to the parameters.
"""

from operator import mul
from typing import Any, Callable, Dict, List, Optional, Sequence, Tuple

import numpy as np
import torch

npdtype = np.complex64

zero_state = np.array([1.0, 0.0], dtype=npdtype)
one_state = np.array([0.0, 1.0], dtype=npdtype)
plus_state = 1.0 / np.sqrt(2) * (zero_state + one_state)
minus_state = 1.0 / np.sqrt(2) * (zero_state - one_state)

_h_matrix = 1 / np.sqrt(2) * np.array([[1.0, 1.0], [1.0, -1.0]])
_i_matrix = np.array([[1.0, 0.0], [0.0, 1.0]])
_x_matrix = np.array([[0.0, 1.0], [1.0, 0.0]])
_y_matrix = np.array([[0.0, -1j], [1j, 0.0]])
_z_matrix = np.array([[1.0, 0.0], [0.0, -1.0]])
_s_matrix = np.array([[1.0, 0.0], [0.0, 1j]])
_t_matrix = np.array([[1.0, 0.0], [0.0, np.exp(np.pi / 4 * 1j)]])
_wroot_matrix = (
    1 / np.sqrt(2) * np.array([[1, -1 / np.sqrt(2) * (1 + 1.0j)], [1 / np.sqrt(2) * (1 - 1.0j), 1]])
)
_ii_matrix = np.kron(_i_matrix, _i_matrix)
_xx_matrix = np.kron(_x_matrix, _x_matrix)
_yy_matrix = np.kron(_y_matrix, _y_matrix)
_zz_matrix = np.kron(_z_matrix, _z_matrix)
_ix_matrix = np.kron(_i_matrix, _x_matrix)
_iy_matrix = np.kron(_i_matrix, _y_matrix)
_iz_matrix = np.kron(_i_matrix, _z_matrix)
_xi_matrix = np.kron(_x_matrix, _i_matrix)
_yi_matrix = np.kron(_y_matrix, _i_matrix)
_zi_matrix = np.kron(_z_matrix, _i_matrix)
_xy_matrix = np.kron(_x_matrix, _y_matrix)
_xz_matrix = np.kron(_x_matrix, _z_matrix)
_yx_matrix = np.kron(_y_matrix, _x_matrix)
_yz_matrix = np.kron(_y_matrix, _z_matrix)
_zx_matrix = np.kron(_z_matrix, _x_matrix)
_zy_matrix = np.kron(_z_matrix, _y_matrix)
_cnot_matrix = np.array([[1.0, 0, 0, 0], [0, 1.0, 0, 0], [0, 0, 0, 1.0], [0, 0, 1.0, 0]])
_cz_matrix = np.diag([1.0, 1.0, 1.0, -1.0])
_cy_matrix = np.array([[1.0, 0, 0, 0], [0, 1.0, 0, 0], [0, 0, 0, -1.0j], [0, 0, 1.0j, 0]])
_swap_matrix = np.array([[1.0, 0, 0, 0], [0, 0, 1.0, 0], [0, 1.0, 0, 0], [0, 0, 0, 1.0]])
_toffoli_matrix = np.eye(8)
_toffoli_matrix[[6, 7]] = _toffoli_matrix[[7, 6]]
_fredkin_matrix = np.eye(8)
_fredkin_matrix[[5, 6]] = _fredkin_matrix[[6, 5]]


def _controlled_np(u: np.ndarray) -> np.ndarray:
    s = u.shape[0]
    out = np.zeros([2 * s, 2 * s], dtype=np.complex128)
    out[:s, :s] = np.eye(s)
    out[s:, s:] = u
    return out


def _ocontrolled_np(u: np.ndarray) -> np.ndarray:
    s = u.shape[0]
    out = np.zeros([2 * s, 2 * s], dtype=np.complex128)
    out[:s, :s] = u
    out[s:, s:] = np.eye(s)
    return out


def reshape2(m: Any) -> Any:
    """[2^k, 2^k] -> [2]*(2k), as the reference's ``backend.reshape2``."""
    k = int(round(np.log2(int(np.prod(m.shape))) / 1))
    return m.reshape([2] * k)


def reshapem(m: Any) -> Any:
    """Any [2]*(2k) or [2^k, 2^k] tensor -> [2^k, 2^k] (``backend.reshapem``)."""
    size = int(np.prod(m.shape))
    d = int(round(np.sqrt(size)))
    return m.reshape([d, d])


class Gate:
    """A gate tensor with a name, standing in for the reference's ``tn.Node``
    wrapper (tensorcircuit/gates.py:138-177): ``.tensor`` holds the matrix in
    the ``[2]*(2k)`` leg shape."""

    def __init__(self, tensor: Any, name: str = "__unnamed_node__") -> None:
        self.tensor = tensor
        self.name = name

    @property
    def shape(self) -> Tuple[int, ...]:
        return tuple(self.tensor.shape)

    def copy(self) -> "Gate":
        return Gate(self.tensor, self.name)

    def __repr__(self) -> str:
        return "Gate(name=%r, shape=%s)" % (self.name, self.shape)


class GateF:
    """Constant-gate factory: ``gates.x()`` -> ``Gate`` (gates.py:248-292)."""

    def __init__(self, m: np.ndarray, n: str) -> None:
        self.m = np.asarray(m, dtype=np.complex128)
        self.n = n

    def __call__(self, *args: Any, **kws: Any) -> Gate:
        return Gate(reshape2(self.m.astype(npdtype)), name=self.n)

    def matrix(self) -> np.ndarray:
        return self.m

    def adjoint(self) -> "GateF":
        return GateF(self.m.conj().T, self.n + "d")

    def controlled(self) -> "GateF":
        return GateF(_controlled_np(self.m), "c" + self.n)

    def ocontrolled(self) -> "GateF":
        return GateF(_ocontrolled_np(self.m), "o" + self.n)

    def __str__(self) -> str:
        return self.n

    __repr__ = __str__


CONSTANT_GATES: Dict[str, np.ndarray] = {}


def _register_constants() -> None:
    g = globals()
    for name in [
        "h", "i", "x", "y", "z", "s", "t", "wroot", "ii", "xx", "yy", "zz", "ix", "iy", "iz",
        "xi", "yi", "zi", "xy", "xz", "yx", "yz", "zx", "zy", "cnot", "cz", "cy", "swap",
        "toffoli", "fredkin",
    ]:
        m = g["_%s_matrix" % name]
        CONSTANT_GATES[name] = np.asarray(m, dtype=np.complex128)
        f = GateF(m, name)
        g[name] = f
        g[name + "gate"] = f
        g[name + "_gate"] = f
    for name in ["sd", "td"]:
        f = g[name[:-1]].adjoint()
        CONSTANT_GATES[name] = f.m
        g[name] = f
        g[name + "gate"] = f
    for name in ["ox", "oy", "oz"]:
        f = g[name[1:]].ocontrolled()
        CONSTANT_GATES[name] = f.m
        g[name] = f
        g[name + "gate"] = f


_register_constants()
pauli_gates = [i(), x(), y(), z()]  # type: ignore  # noqa: F821


def matrix_for_gate(gate: Any, tol: float = 1e-6) -> np.ndarray:
    t = gate.tensor if isinstance(gate, Gate) else gate
    if isinstance(t, torch.Tensor):
        t = t.detach().cpu().numpy()
    t = np.array(reshapem(np.asarray(t)), dtype=np.complex128)
    t.real[abs(t.real) < tol] = 0.0
    t.imag[abs(t.imag) < tol] = 0.0
    return t


# ----------------------------------------------------------------------------
# vectorised builders for parameterized families
# ----------------------------------------------------------------------------
C64 = torch.complex64


def _c(x: torch.Tensor) -> torch.Tensor:
    return x.to(torch.complex128)


def _hi(theta: torch.Tensor) -> torch.Tensor:
    """Parameters are evaluated in double precision and the finished matrix
    entries rounded to complex64 once: fp32 cos/sin leave each gate ~1e-7
    away from unitary, and the adjoint sweep (uncompute through G^H) would
    compound that over forward + backward."""
    return theta.to(torch.complex128) if theta.is_complex() else theta.to(torch.float64)


def _cs(theta: torch.Tensor, scale: float) -> Tuple[torch.Tensor, torch.Tensor]:
    t = _hi(theta) * scale
    return torch.cos(t), torch.sin(t)


J = 1j


def build_rx(theta: torch.Tensor) -> torch.Tensor:
    c, s = _cs(theta, 0.5)
    c, s = _c(c), _c(s)
    return torch.stack([c, -J * s, -J * s, c], -1)


def build_ry(theta: torch.Tensor) -> torch.Tensor:
    c, s = _cs(theta, 0.5)
    c, s = _c(c), _c(s)
    return torch.stack([c, -s, s, c], -1)


def build_rz(theta: torch.Tensor) -> torch.Tensor:  # diagonal
    c, s = _cs(theta, 0.5)
    c, s = _c(c), _c(s)
    return torch.stack([c - J * s, c + J * s], -1)


def build_phase(theta: torch.Tensor) -> torch.Tensor:  # diagonal
    e = torch.exp(J * _c(_hi(theta)))
    return torch.stack([torch.ones_like(e), e], -1)


def build_r(theta: torch.Tensor, alpha: torch.Tensor, phi: torch.Tensor) -> torch.Tensor:
    theta, alpha, phi = _hi(theta), _hi(alpha), _hi(phi)
    ct, st = _c(torch.cos(theta)), _c(torch.sin(theta))
    ca, sa = _c(torch.cos(alpha)), _c(torch.sin(alpha))
    cp, sp = _c(torch.cos(phi)), _c(torch.sin(phi))
    a = cp * sa * st
    b = sp * sa * st
    zc = st * ca
    return torch.stack([ct - J * zc, -J * a - b, -J * a + b, ct + J * zc], -1)


def build_u(theta: torch.Tensor, phi: torch.Tensor, lbd: torch.Tensor) -> torch.Tensor:
    c, s = _cs(theta, 0.5)
    c, s = _c(c), _c(s)
    ephi = torch.exp(J * _c(_hi(phi)))
    elbd = torch.exp(J * _c(_hi(lbd)))
    return torch.stack([c, -elbd * s, ephi * s, ephi * elbd * c], -1)


def build_iswap(theta: torch.Tensor) -> torch.Tensor:
    c, s = _cs(theta, np.pi / 2)
    c, s = _c(c), _c(s)
    one = torch.ones_like(c)
    zero = torch.zeros_like(c)
    return torch.stack(
        [one, zero, zero, zero, zero, c, J * s, zero, zero, J * s, c, zero, zero, zero, zero, one], -1
    )


def build_exp1_dense(theta: torch.Tensor, unitary: torch.Tensor, half: bool) -> torch.Tensor:
    """``cos(t) I - i sin(t) U``; unitary [G, d, d] or [d, d]."""
    t = _hi(theta) * 0.5 if half else _hi(theta)
    c, s = _c(torch.cos(t)), _c(torch.sin(t))
    u = _c(unitary)
    d = u.shape[-1]
    eye = torch.eye(d, dtype=torch.complex128, device=u.device)
    m = c[..., None, None] * eye - J * s[..., None, None] * u
    return m.reshape(m.shape[:-2] + (d * d,))


def build_exp1_diag(theta: torch.Tensor, udiag: torch.Tensor, half: bool) -> torch.Tensor:
    t = _hi(theta) * 0.5 if half else _hi(theta)
    c, s = _c(torch.cos(t)), _c(torch.sin(t))
    return c[..., None] - J * s[..., None] * _c(udiag)


def build_exp_dense(theta: torch.Tensor, unitary: torch.Tensor) -> torch.Tensor:
    u = _c(unitary)
    m = torch.linalg.matrix_exp(-J * _c(_hi(theta))[..., None, None] * u)
    d = u.shape[-1]
    return m.reshape(m.shape[:-2] + (d * d,))


def controlled_dense(m: torch.Tensor, d: int, ctrl_first_one: bool = True) -> torch.Tensor:
    """Embed U (entries [G, d*d]) as [[I, 0], [0, U]] (or [[U, 0], [0, I]])."""
    u = m.reshape(m.shape[:-1] + (d, d))
    eye = torch.eye(d, dtype=m.dtype, device=m.device).expand(u.shape)
    zero = torch.zeros_like(u)
    if ctrl_first_one:
        top = torch.cat([eye, zero], -1)
        bot = torch.cat([zero, u], -1)
    else:
        top = torch.cat([u, zero], -1)
        bot = torch.cat([zero, eye], -1)
    full = torch.cat([top, bot], -2)
    return full.reshape(full.shape[:-2] + (4 * d * d,))


def controlled_diag(dvals: torch.Tensor, ctrl_first_one: bool = True) -> torch.Tensor:
    ones = torch.ones_like(dvals)
    return torch.cat([ones, dvals] if ctrl_first_one else [dvals, ones], -1)


# family name -> (nq, diagonal, param names with defaults, builder)
class Family:
    def __init__(self, name: str, nq: int, diag: bool, params: Sequence[Tuple[str, float]],
                 build: Callable[..., torch.Tensor]) -> None:
        self.name = name
        self.nq = nq
        self.diag = diag
        self.params = list(params)
        self.build = build
        # Pauli rotations cos(phi) I - i sin(phi) P, phi = scale * theta:
        # the engine takes them as one entry exp(i phi) (see PROT_FAMILIES)
        self.pauli: Optional[str] = None
        self.scale = 1.0

    @property
    def entries(self) -> int:
        if self.pauli is not None:
            return 1
        return (1 << self.nq) if self.diag else (1 << (2 * self.nq))


PAULI_CODE = {"x": 1, "y": 2, "z": 3}


def build_prot(theta: torch.Tensor, scale: float) -> torch.Tensor:
    """exp(i phi), phi = scale * theta, as [G, 1]: the engine's encoding of
    cos(phi) I - i sin(phi) P (cos and sin evaluated in double precision)."""
    phi = _hi(theta) * scale
    return torch.exp(1j * _c(phi))[..., None]


_DEV_CONSTS: Dict[Tuple[str, str], torch.Tensor] = {}


def device_const(name: str, m: np.ndarray, device: torch.device) -> torch.Tensor:
    """A constant matrix on ``device``, copied from the host once; later
    uses (including under CUDA-graph capture, where a host-to-device copy is
    not allowed) reuse the device copy."""
    key = (name, str(device))
    t = _DEV_CONSTS.get(key)
    if t is None:
        t = torch.as_tensor(np.array(m, dtype=np.complex128), device=device)
        _DEV_CONSTS[key] = t
    return t


def _ctrl(f: Callable[..., torch.Tensor], base_nq: int, diag: bool, one: bool) -> Callable[..., torch.Tensor]:
    d = 1 << base_nq

    def b(*args: torch.Tensor) -> torch.Tensor:
        m = f(*args)
        return controlled_diag(m, one) if diag else controlled_dense(m, d, one)

    return b


FAMILIES: Dict[str, Family] = {
    "rx": Family("rx", 1, False, [("theta", 0.0)], build_rx),
    "ry": Family("ry", 1, False, [("theta", 0.0)], build_ry),
    "rz": Family("rz", 1, True, [("theta", 0.0)], build_rz),
    "phase": Family("phase", 1, True, [("theta", 0.0)], build_phase),
    "r": Family("r", 1, False, [("theta", 0.0), ("alpha", 0.0), ("phi", 0.0)], build_r),
    "u": Family("u", 1, False, [("theta", 0.0), ("phi", 0.0), ("lbd", 0.0)], build_u),
    "iswap": Family("iswap", 2, False, [("theta", 1.0)], build_iswap),
    "rxx": Family("rxx", 2, False, [("theta", 0.0)],
                  lambda t: build_exp1_dense(t, device_const("xx", _xx_matrix, t.device), True)),
    "ryy": Family("ryy", 2, False, [("theta", 0.0)],
                  lambda t: build_exp1_dense(t, device_const("yy", _yy_matrix, t.device), True)),
    "rzz": Family("rzz", 2, True, [("theta", 0.0)],
                  lambda t: build_exp1_diag(t, device_const("zzdiag", np.diag(_zz_matrix), t.device), True)),
    "crx": Family("crx", 2, False, [("theta", 0.0)], _ctrl(build_rx, 1, False, True)),
    "cry": Family("cry", 2, False, [("theta", 0.0)], _ctrl(build_ry, 1, False, True)),
    "crz": Family("crz", 2, True, [("theta", 0.0)], _ctrl(build_rz, 1, True, True)),
    "cphase": Family("cphase", 2, True, [("theta", 0.0)], _ctrl(build_phase, 1, True, True)),
    "cr": Family("cr", 2, False, [("theta", 0.0), ("alpha", 0.0), ("phi", 0.0)], _ctrl(build_r, 1, False, True)),
    "cu": Family("cu", 2, False, [("theta", 0.0), ("phi", 0.0), ("lbd", 0.0)], _ctrl(build_u, 1, False, True)),
    "orx": Family("orx", 2, False, [("theta", 0.0)], _ctrl(build_rx, 1, False, False)),
    "ory": Family("ory", 2, False, [("theta", 0.0)], _ctrl(build_ry, 1, False, False)),
    "orz": Family("orz", 2, True, [("theta", 0.0)], _ctrl(build_rz, 1, True, False)),
}

# Families that are Pauli rotations exp(-i theta/2 P) (tensorcircuit/gates.py:
# 579-636 rx/ry/rz, :825-865 rxx/ryy/rzz = exp1(PP, theta, half=True)).
for _name, _p in [("rx", "x"), ("ry", "y"), ("rz", "z"), ("rxx", "xx"), ("ryy", "yy"), ("rzz", "zz")]:
    FAMILIES[_name].pauli = _p
    FAMILIES[_name].scale = 0.5

# gate method names as in the reference (tensorcircuit/abstractcircuit.py:28-66)
sgates = ["i", "x", "y", "z", "h", "t", "s", "td", "sd", "wroot"] + \
    ["cnot", "cz", "swap", "cy", "ox", "oy", "oz"] + ["toffoli", "fredkin"]
vgates = ["r", "cr", "u", "cu", "rx", "ry", "rz", "phase", "rxx", "ryy", "rzz", "cphase", "crx",
          "cry", "crz", "orx", "ory", "orz", "iswap", "any", "exp", "exp1"]
mpogates = ["multicontrol", "mpo"]
gate_aliases = [["cnot", "cx"], ["fredkin", "cswap"], ["toffoli", "ccnot"], ["toffoli", "ccx"],
                ["any", "unitary"], ["sd", "sdg"], ["td", "tdg"]]


def is_diagonal(m: np.ndarray, tol: float = 0.0) -> bool:
    return bool(np.all(np.abs(m - np.diag(np.diag(m))) <= tol))


def _np_param(v: Any) -> Any:
    if isinstance(v, torch.Tensor):
        return v.detach().cpu().numpy()
    return np.asarray(v)


def _fam_np(name: str, **kws: Any) -> np.ndarray:
    fam = FAMILIES[name]
    args = [torch.as_tensor(_np_param(kws.get(p, d)), dtype=torch.float64) for p, d in fam.params]
    e = fam.build(*args).detach().numpy().astype(np.complex128)
    if fam.diag:
        return np.diag(e)
    d = 1 << fam.nq
    return e.reshape(d, d)


def _vgate_factory(name: str) -> Callable[..., Gate]:
    def f(**kws: Any) -> Gate:
        m = _fam_np(name, **kws)
        return Gate(reshape2(m.astype(npdtype)), name=name)

    return f


for _n in FAMILIES:
    globals()[_n] = _vgate_factory(_n)
    globals()[_n + "_gate"] = globals()[_n]
    globals()[_n + "gate"] = globals()[_n]


def any_gate(unitary: Any, name: str = "any") -> Gate:
    if isinstance(unitary, Gate):
        return unitary
    return Gate(reshape2(unitary), name=name)


def exponential_gate_unity(unitary: Any, theta: Any, half: bool = False, name: str = "none") -> Gate:
    u = np.asarray(_np_param(unitary.tensor if isinstance(unitary, Gate) else unitary), dtype=np.complex128)
    d = int(round(np.sqrt(u.size)))
    u = u.reshape(d, d)
    t = np.asarray(_np_param(theta), dtype=np.float64) * (0.5 if half else 1.0)
    return Gate(reshape2((np.cos(t) * np.eye(d) - 1j * np.sin(t) * u).astype(npdtype)), name="exp1-" + name)


def exponential_gate(unitary: Any, theta: Any, name: str = "none") -> Gate:
    import scipy.linalg

    u = np.asarray(_np_param(unitary.tensor if isinstance(unitary, Gate) else unitary), dtype=np.complex128)
    d = int(round(np.sqrt(u.size)))
    u = u.reshape(d, d)
    t = float(np.asarray(_np_param(theta)))
    return Gate(reshape2(scipy.linalg.expm(-1j * t * u).astype(npdtype)), name="exp-" + name)


any = any_gate  # noqa: A001
unitary = any_gate
exp1 = exp1_gate = exponential_gate_unity
exp = exp_gate = exponential_gate
