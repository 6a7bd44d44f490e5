"""``Circuit``: the reference's circuit API on top of the GB300 engine.

Gate methods are registered from the same name lists as the reference
(``sgates``, ``vgates``, ``mpogates``, ``gate_aliases``;
tensorcircuit/abstractcircuit.py:28-66, ``_meta_apply`` :218-326), take the
same keyword parameters and broadcast over index lists the same way
(``apply_list``, :149-165).  A gate call only RECORDS the gate
(tensorcircuit/basecircuit.py:120-245 queues a tensor-network node instead);
the state is computed by the engine when it is first needed and cached, like
the reference's ``state_tensor`` cache (basecircuit.py:249-265).
"""

import hashlib
from typing import Any, Dict, List, Optional, Sequence, Tuple, Union

import numpy as np
import torch

from . import _native as nat
from . import engine as eng
from . import channels as _channels
from . import gates
from .quantum import sample2all, sample_int2bin

Tensor = Any
C64 = torch.complex64

_PAULI_1Q = {
    0: np.eye(2, dtype=np.complex128),
    1: gates._x_matrix.astype(np.complex128),
    2: gates._y_matrix.astype(np.complex128),
    3: gates._z_matrix.astype(np.complex128),
}


def _is_complex(v: Any) -> bool:
    if isinstance(v, torch.Tensor):
        return v.is_complex()
    return bool(np.iscomplexobj(v))


def _is_seq(x: Any) -> bool:
    return isinstance(x, (list, tuple, range)) or (isinstance(x, np.ndarray) and x.ndim > 0)


def _to_np_matrix(m: Any) -> Optional[np.ndarray]:
    """numpy matrix for constant operands, None for torch tensors."""
    if isinstance(m, gates.Gate):
        m = m.tensor
    if isinstance(m, torch.Tensor):
        return None
    a = np.asarray(m, dtype=np.complex128)
    d = int(round(np.sqrt(a.size)))
    return a.reshape(d, d)


_PAULI_CACHE: Dict[bytes, Optional[Tuple[int, ...]]] = {}


def _pauli_decompose(m: np.ndarray) -> Optional[List[int]]:
    """If m is a tensor product of single-qubit Paulis, return their codes
    (memoised by the matrix bytes: circuits repeat the same few matrices)."""
    key = m.tobytes() + bytes([m.shape[0]])
    if key in _PAULI_CACHE:
        r = _PAULI_CACHE[key]
        return None if r is None else list(r)
    r = _pauli_decompose_uncached(m)
    if len(_PAULI_CACHE) < 4096:
        _PAULI_CACHE[key] = None if r is None else tuple(r)
    return r


def _pauli_decompose_uncached(m: np.ndarray) -> Optional[List[int]]:
    d = m.shape[0]
    k = int(round(np.log2(d)))
    if (1 << k) != d:
        return None
    codes: List[int] = []

    def rec(mat: np.ndarray, kk: int) -> bool:
        if kk == 0:
            return bool(np.allclose(mat, 1.0, atol=1e-12))
        h = mat.shape[0] // 2
        for c, p in _PAULI_1Q.items():
            # mat = p (x) rest  ->  rest = block / p_ij for a nonzero p entry
            i, j = (0, 0) if abs(p[0, 0]) > 0 else (0, 1)
            rest = mat[i * h:(i + 1) * h, j * h:(j + 1) * h] / p[i, j]
            if np.allclose(np.kron(p, rest), mat, atol=1e-10):
                codes.append(c)
                if rec(rest, kk - 1):
                    return True
                codes.pop()
        return False

    return codes if rec(m, k) else None


class _Op:
    """One recorded gate.

    kind: "const" (numpy matrix), "fam" (parameterized family), "prot"
    (Pauli rotation: data = (theta, scale, Pauli codes)), "any" (user torch
    matrix), "exp1"/"exp" (exponential of a given hermitian), "kraus" (one
    operator of a Kraus set picked per trajectory: data = (set key, operator
    stack [l, entries] on the device, pick index))."""

    __slots__ = ("kind", "name", "qubits", "data", "diag", "nq", "conj")

    def __init__(self, kind: str, name: str, qubits: Tuple[int, ...], data: Any, diag: bool, nq: int,
                 conj: bool = False) -> None:
        self.kind = kind
        self.name = name
        self.qubits = qubits
        self.data = data
        self.diag = diag
        self.nq = nq
        # the gate's matrix is the complex conjugate of the one its data
        # builds (the column-side twin of a density-matrix gate)
        self.conj = conj


class _PlanEntry:
    """Cached per-structure data: native plan + matrix-buffer layout."""

    def __init__(self, plan: eng.GatePlan, const_block: Optional[np.ndarray], groups: List[Any], nmat: int,
                 gates_c: Optional[List[Any]] = None) -> None:
        self.plan = plan
        # (kind, qubits, mat_off, grad_off[, Pauli codes]) per gate
        self.gates_c = gates_c or []
        # Pauli terms the last circuit of this structure asked for, in order
        self.last_terms: Optional[List[Tuple[int, int]]] = None
        self.const_np = const_block
        self.const_dev: Dict[int, torch.Tensor] = {}
        self.groups = groups  # (gkey, op indices, E)
        self.nmat = nmat

    def const_block(self, dev: torch.device) -> Optional[torch.Tensor]:
        if self.const_np is None:
            return None
        t = self.const_dev.get(dev.index)
        if t is None:
            t = torch.as_tensor(self.const_np, dtype=C64, device=dev)
            self.const_dev[dev.index] = t
        return t


_entries: Dict[Any, _PlanEntry] = {}


def _group_key(op: _Op) -> Any:
    k = _group_key_plain(op)
    return k + ("*",) if op.conj else k


def _group_key_plain(op: _Op) -> Any:
    if op.kind == "prot":
        return ("prot", op.data[1])
    if op.kind == "fam":
        return ("fam", op.name)
    if op.kind == "any":
        return ("any", op.nq, op.diag)
    if op.kind == "exp1":
        return ("exp1", op.nq, op.data[2], op.diag)
    if op.kind == "exp":
        return ("exp", op.nq)
    if op.kind == "kraus":
        return ("kraus", op.nq, op.diag, op.data[0])
    raise ValueError(op.kind)


def _struct_key(n: int, ops: Sequence[_Op]) -> Any:
    parts = []
    for op in ops:
        if op.kind == "const":
            parts.append(("c", op.name, op.qubits))
        elif op.kind == "prot":
            parts.append((_group_key(op), op.qubits, op.data[2]))
        else:
            parts.append((_group_key(op), op.qubits))
    return (n, tuple(parts))


def _build_entry(n_eng: int, ops: Sequence[_Op]) -> _PlanEntry:
    # constant block first, then one block per parameterized group
    const_mats: List[np.ndarray] = []
    const_off: Dict[int, int] = {}
    off = 0
    for i, op in enumerate(ops):
        if op.kind == "const":
            m = op.data
            e = np.diag(m) if op.diag else m.reshape(-1)
            const_off[i] = off
            const_mats.append(e.astype(np.complex64))
            off += e.size
    groups: Dict[Any, List[int]] = {}
    order: List[Any] = []
    for i, op in enumerate(ops):
        if op.kind != "const":
            k = _group_key(op)
            if k not in groups:
                groups[k] = []
                order.append(k)
            groups[k].append(i)
    mat_off: Dict[int, int] = dict(const_off)
    grad_off: Dict[int, int] = {}
    glist = []
    for k in order:
        idx = groups[k]
        op0 = ops[idx[0]]
        if op0.kind == "prot":
            E = 1
        else:
            E = (1 << op0.nq) if op0.diag else (1 << (2 * op0.nq))
        # constant Kraus sets take no gradient
        const_kraus = op0.kind == "kraus" and k[3][0] == "n"
        for j, i in enumerate(idx):
            mat_off[i] = off + j * E
            if (ops[i].nq <= 2 or ops[i].kind == "prot") and not const_kraus:
                grad_off[i] = off + j * E
        off += E * len(idx)
        glist.append((k, idx, E))
    gates_c = []
    for i, op in enumerate(ops):
        if op.kind == "prot":
            gates_c.append((nat.TCG_GATE_PAULI_ROT, op.qubits, mat_off[i], grad_off.get(i, -1), op.data[2]))
        else:
            kind = nat.TCG_GATE_DIAG if op.diag else nat.TCG_GATE_DENSE
            gates_c.append((kind, op.qubits, mat_off[i], grad_off.get(i, -1)))
    plan = eng.GatePlan(n_eng, gates_c, off)
    const_block = np.concatenate(const_mats) if const_mats else None
    return _PlanEntry(plan, const_block, glist, off, gates_c)


def _stack_scalars(vals: Sequence[Any], dev: torch.device) -> torch.Tensor:
    if all(not isinstance(v, torch.Tensor) for v in vals):
        arr = np.asarray([np.asarray(v) for v in vals])
        if np.iscomplexobj(arr):
            return torch.as_tensor(arr.astype(np.complex64), device=dev)
        return torch.as_tensor(arr.astype(np.float32), device=dev)
    if all(isinstance(v, torch.Tensor) for v in vals):
        v0 = vals[0]
        if all(v.dtype == v0.dtype and v.device == v0.device and v.dim() == 0 for v in vals) and \
                v0.dtype in (torch.float32, torch.float64, torch.complex64, torch.complex128):
            # one stack op; no per-parameter casts (each torch op costs tens of
            # microseconds under torch.func transforms)
            t = torch.stack(list(vals))
            return t if t.device == dev else t.to(dev)
    cplx = any(v.is_complex() if isinstance(v, torch.Tensor) else np.iscomplexobj(v) for v in vals)
    dt = torch.complex64 if cplx else torch.float32
    ts = []
    for v in vals:
        if isinstance(v, torch.Tensor):
            t = v.to(device=dev, dtype=dt)
        else:
            t = torch.as_tensor(np.asarray(v), device=dev).to(dt)
        ts.append(t.reshape(()))
    return torch.stack(ts)


def _stack_mats(vals: Sequence[Any], d: int, dev: torch.device) -> torch.Tensor:
    ts = []
    for v in vals:
        if isinstance(v, gates.Gate):
            v = v.tensor
        if not isinstance(v, torch.Tensor):
            v = torch.as_tensor(np.asarray(v, dtype=np.complex64))
        ts.append(v.to(device=dev, dtype=C64).reshape(d, d))
    return torch.stack(ts)


def _group_block(key: Any, ops: Sequence[_Op], idx: Sequence[int], dev: torch.device) -> torch.Tensor:
    if key[-1] == "*":
        # a physical conjugate (the engine reads the raw buffer, which a
        # lazily conjugated view would leave unconjugated), built from
        # real/imag so that vmap batches it
        b = _group_block(key[:-1], ops, idx, dev).to(C64)
        return torch.complex(b.real, -b.imag)
    kind = key[0]
    if kind == "prot":
        return gates.build_prot(_stack_scalars([ops[i].data[0] for i in idx], dev), key[1])
    if kind == "fam":
        fam = gates.FAMILIES[key[1]]
        args = []
        for p, (pname, _) in enumerate(fam.params):
            args.append(_stack_scalars([ops[i].data[p] for i in idx], dev))
        return fam.build(*args)
    if kind == "any":
        nq, diag = key[1], key[2]
        d = 1 << nq
        m = _stack_mats([ops[i].data for i in idx], d, dev)
        if diag:
            return torch.diagonal(m, dim1=-2, dim2=-1)
        return m.reshape(m.shape[:-2] + (d * d,))
    if kind == "exp1":
        nq, half, diag = key[1], key[2], key[3]
        d = 1 << nq
        theta = _stack_scalars([ops[i].data[0] for i in idx], dev)
        u = _stack_mats([ops[i].data[1] for i in idx], d, dev)
        if diag:
            return gates.build_exp1_diag(theta, torch.diagonal(u, dim1=-2, dim2=-1), half)
        return gates.build_exp1_dense(theta, u, half)
    if kind == "exp":
        d = 1 << key[1]
        theta = _stack_scalars([ops[i].data[0] for i in idx], dev)
        u = _stack_mats([ops[i].data[1] for i in idx], d, dev)
        return gates.build_exp_dense(theta, u)
    if kind == "kraus":
        rs = torch.stack([ops[i].data[2] for i in idx], -1).long()
        if key[3][0] == "n":
            # one shared constant set: a single gather for the whole group
            return ops[idx[0]].data[1][rs]
        return torch.stack([ops[i].data[1][r] for i, r in zip(idx, rs.unbind(-1))], -2)
    raise ValueError(kind)


# ----------------------------------------------------------------------------
# Monte-Carlo trajectory noise (tensorcircuit/circuit.py:354-764)
# ----------------------------------------------------------------------------
_PAULI_NP = [np.eye(2), np.array([[0, 1], [1, 0]]), np.array([[0, -1j], [1j, 0]]), np.diag([1.0, -1.0])]
_KRAUS_DEV: Dict[Any, torch.Tensor] = {}


def _kraus_mats(kraus: Sequence[Any], d: int) -> Tuple[List[Any], bool]:
    """Kraus operators as d x d numpy (complex128) or torch (complex64)
    matrices; the flag says whether any is a torch tensor."""
    out: List[Any] = []
    is_t = False
    for k in kraus:
        t = k.tensor if isinstance(k, gates.Gate) else k
        if isinstance(t, torch.Tensor):
            is_t = True
            out.append(t.to(C64).reshape(d, d))
        else:
            a = np.asarray(t, dtype=np.complex128)
            if a.size != d * d:
                raise ValueError("Kraus operator of size %d does not act on %d qubits" % (a.size, d.bit_length() - 1))
            out.append(a.reshape(d, d))
    if not out:
        raise ValueError("empty Kraus list")
    return out, is_t


def _kraus_device_set(mats: Sequence[np.ndarray], extra: np.ndarray, diag: bool,
                      dev: torch.device) -> Tuple[Any, torch.Tensor]:
    """Content key and cached device stack [l, entries] of a constant set."""
    stack = np.stack([np.diag(m) if diag else m.reshape(-1) for m in mats]).astype(np.complex64)
    h = hashlib.sha1(stack.tobytes())
    h.update(np.ascontiguousarray(extra).tobytes())
    key = ("n", stack.shape, h.hexdigest())
    t = _KRAUS_DEV.get((key, dev.index))
    if t is None:
        t = torch.as_tensor(stack, device=dev)
        _KRAUS_DEV[(key, dev.index)] = t
    return key, t


_UK_PREP: Dict[Any, Any] = {}


def _unitary_kraus_prep(mats: Sequence[np.ndarray], prob: Optional[Sequence[float]], d: int,
                        dev: torch.device) -> Tuple[Any, torch.Tensor, torch.Tensor, bool]:
    """For a constant set: (set key, device operator stack, device
    cumulative probabilities, diagonal flag), memoised by content.  Without
    ``prob`` the probabilities are tr(K^dag K)/d in float32 and each operator
    is divided by sqrt(p) (a zero-probability operator stays zero)."""
    pb = b"" if prob is None else np.asarray(prob, dtype=np.float32).tobytes()
    fp = (d, dev.index, pb, prob is None, b"".join(np.ascontiguousarray(m).tobytes() for m in mats))
    r = _UK_PREP.get(fp)
    if r is None:
        if len(_UK_PREP) > 4096:
            _UK_PREP.clear()
        if prob is None:
            m64 = [m.astype(np.complex64) for m in mats]
            p = np.array([np.real(np.trace(m.conj().T @ m)) / d for m in m64], dtype=np.float32)
            mats = [m / np.sqrt(float(q)) if q > 0 else np.zeros_like(m) for m, q in zip(mats, p)]
        else:
            p = np.asarray(prob, dtype=np.float32).reshape(-1)
        if len(p) != len(mats):
            raise ValueError("prob has %d entries for %d Kraus operators" % (len(p), len(mats)))
        cum_np = np.cumsum(p, dtype=np.float32)
        diag = all(gates.is_diagonal(m) for m in mats)
        key, kdev = _kraus_device_set(mats, cum_np, diag, dev)
        r = (key, kdev, torch.as_tensor(cum_np, device=dev), diag)
        _UK_PREP[fp] = r
    return r


def _uniform(status: Any, dev: torch.device) -> torch.Tensor:
    """The trajectory's uniform draw as fp32 on the device: ``status`` (its
    real part), or a fresh draw when it is None."""
    if status is None:
        return torch.rand((), device=dev)
    if isinstance(status, torch.Tensor):
        x = torch.real(status) if status.is_complex() else status
        x = x.to(device=dev, dtype=torch.float32)
        if x.dim() > 0 and x.numel() == 1:
            x = x.reshape(())
        return x
    return torch.full((), float(np.real(np.asarray(status).reshape(-1)[0])), dtype=torch.float32, device=dev)


def _pick(status: Any, cum: torch.Tensor, dev: torch.device) -> torch.Tensor:
    """The Kraus pick of tensorcircuit/circuit.py:541-556: for a uniform x
    and cumulative probabilities c, int(sum_{i<l-1} sign(x - c_i) / 2 +
    (l - 1) / 2) -- the number of c_i below x plus half the number equal to
    x, truncated.  ``cum`` may carry batch dimensions."""
    x = _uniform(status, dev)
    l = cum.shape[-1]
    if l == 1:
        return torch.zeros_like(x, dtype=torch.int32)
    s = torch.sign(x.unsqueeze(-1) - cum[..., : l - 1]).sum(-1)
    return (s * 0.5 + (l - 1) * 0.5).to(torch.int32)


_STRINGS: Dict[int, List[Tuple[Tuple[int, ...], np.ndarray]]] = {}


def _pauli_strings(k: int) -> List[Tuple[Tuple[int, ...], np.ndarray]]:
    """All 4^k Pauli strings on k gate legs (codes per leg, matrix), the
    first leg outermost."""
    out = _STRINGS.get(k)
    if out is None:
        out = [((), np.ones((1, 1)))]
        for _ in range(k):
            out = [(c + (j,), np.kron(m, _PAULI_NP[j])) for c, m in out for j in range(4)]
        _STRINGS[k] = out
    return out


# Device-side constants are made once and reused: a host-to-device copy from
# pageable memory would wait for the stream (and cannot be captured into a
# CUDA graph).
_DEV_CONST: Dict[Any, torch.Tensor] = {}


def _dev_const(m: np.ndarray, dev: torch.device) -> torch.Tensor:
    key = (m.tobytes(), m.shape, dev.index)
    t = _DEV_CONST.get(key)
    if t is None:
        if len(_DEV_CONST) > 4096:
            _DEV_CONST.clear()
        t = torch.as_tensor(np.asarray(m, dtype=np.complex64), device=dev)
        _DEV_CONST[key] = t
    return t


def _pauli_stack(k: int, dev: torch.device) -> torch.Tensor:
    return _dev_const(np.stack([s for _, s in _pauli_strings(k)]), dev)


_ARANGE: Dict[Any, torch.Tensor] = {}


def _arange(l: int, dev: torch.device) -> torch.Tensor:
    t = _ARANGE.get((l, dev.index))
    if t is None:
        t = torch.arange(l, device=dev)
        _ARANGE[(l, dev.index)] = t
    return t


_KRAUS_PREP: Dict[Any, Any] = {}


def _kraus_prep(mats: Sequence[np.ndarray], k: int, dev: torch.device) -> Tuple[Any, torch.Tensor, torch.Tensor, bool]:
    """For a constant Kraus set: (set key, device operator stack, device
    matrix coef[i, s] = tr(K_i^dag K_i P_s) / 2^k of the Pauli expansion,
    diagonal flag), memoised by content."""
    fp = (k, dev.index, b"".join(np.ascontiguousarray(m).tobytes() for m in mats))
    r = _KRAUS_PREP.get(fp)
    if r is None:
        if len(_KRAUS_PREP) > 4096:
            _KRAUS_PREP.clear()
        d = 1 << k
        coef = np.array([[np.real(np.trace(m.conj().T @ m @ s)) / d for _, s in _pauli_strings(k)] for m in mats])
        diag = all(gates.is_diagonal(m) for m in mats)
        key, kdev = _kraus_device_set(mats, np.zeros(0), diag, dev)
        r = (key, kdev, torch.as_tensor(coef.astype(np.float32), device=dev), diag)
        _KRAUS_PREP[fp] = r
    return r


_SPECS: Dict[Any, Tuple[Tuple[int, int], ...]] = {}


def _kraus_spec(idx: Tuple[int, ...], n_eng: int) -> Tuple[Tuple[int, int], ...]:
    """The 4^k Pauli strings on qubits idx as (xmask, zmask) terms."""
    spec = _SPECS.get((idx, n_eng))
    if spec is None:
        out = []
        for codes, _ in _pauli_strings(len(idx)):
            xs = [q for q, c in zip(idx, codes) if c == 1]
            ys = [q for q, c in zip(idx, codes) if c == 2]
            zs = [q for q, c in zip(idx, codes) if c == 3]
            out.append(eng.pauli_masks(n_eng, xs, ys, zs))
        spec = tuple(out)
        _SPECS[(idx, n_eng)] = spec
    return spec


def _apply_local(psi: torch.Tensor, m: torch.Tensor, idx: Sequence[int], n: int) -> torch.Tensor:
    """psi -> (m on qubits idx) psi for a per-trajectory, differentiable
    operator ``m`` [..., d, d]; used only for Kraus operators given as
    tensors that need gradients (the engine's adjoint sweep assumes the
    operators it un-applies are unitary)."""
    k = len(idx)
    lead = psi.shape[:-1]
    nl = len(lead)
    if m.dim() > 2:
        m = m.expand(lead + m.shape[-2:])
    t = psi.reshape(lead + (2,) * n)
    g = m.reshape(m.shape[:-2] + (2,) * (2 * k))
    # contract the gate's input legs with the state's legs idx
    letters = "abcdefghijklmnopqrstuvwxyzABCDEFGHIJKLMNOPQRSTUVWXYZ"
    sl = letters[:nl]
    st = list(letters[nl:nl + n])
    outl = list(st)
    gin = [st[q] for q in idx]
    gout = list(letters[nl + n:nl + n + k])
    for j, q in enumerate(idx):
        outl[q] = gout[j]
    gl = (sl if m.dim() > 2 else "") + "".join(gout) + "".join(gin)
    r = torch.einsum("%s,%s->%s" % (gl, sl + "".join(st), sl + "".join(outl)), g, t)
    return r.reshape(lead + (1 << n,))


class Circuit:
    """Statevector circuit with the reference's ``tc.Circuit`` surface."""

    sgates = gates.sgates
    vgates = gates.vgates
    mpogates = gates.mpogates
    gate_aliases = gate_aliases = gates.gate_aliases
    is_dm = False
    is_mps = False

    def __init__(self, nqubits: int, inputs: Optional[Tensor] = None, mps_inputs: Optional[Any] = None,
                 split: Optional[Dict[str, Any]] = None) -> None:
        if mps_inputs is not None:
            raise NotImplementedError("mps_inputs is not supported by the statevector engine")
        if nqubits < 1:
            raise ValueError("a circuit needs at least one qubit")
        self._nqubits = nqubits
        # qubits of the vector the engine evolves (2n for a density matrix)
        self._nvec = nqubits
        self.inputs = inputs
        self.mps_inputs = None
        self.split = split
        self.circuit_param = {"nqubits": nqubits, "inputs": inputs, "mps_inputs": None, "split": split}
        self._qir: List[Dict[str, Any]] = []
        self._extra_qir: List[Dict[str, Any]] = []
        self._ops: List[_Op] = []
        self._cache: Optional[Tuple[Any, ...]] = None
        # Pauli terms requested from this circuit's state, in order; the next
        # circuit with the same structure uses the list as its prediction
        self._req_terms: List[Tuple[int, int]] = []
        self._pred_terms: Optional[List[Tuple[int, int]]] = None
        self._term_batch: Optional[Tuple[torch.Tensor, ...]] = None
        # general Kraus channels need the state in the middle of the circuit:
        # the gates before one become a finished segment whose (rescaled)
        # output state is the input of the gates after it
        self._seg_input: Optional[torch.Tensor] = None
        self._seg_ops = 0

    # ------------------------------------------------------------------ gates
    def _norm_index(self, index: Sequence[int]) -> Tuple[int, ...]:
        n = self._nqubits
        idx = tuple(int(i) if int(i) >= 0 else n + int(i) for i in index)
        for i in idx:
            if not 0 <= i < n:
                raise ValueError("qubit index %d out of range for %d qubits" % (i, n))
        assert len(idx) == len(set(idx)), "a gate cannot act twice on one qubit"
        return idx

    def _record(self, op: _Op, ir: Dict[str, Any]) -> None:
        self._qir.append(ir)
        self._ops.append(op)
        self._cache = None
        self._req_terms = []
        self._pred_terms = None
        self._term_batch = None

    def _apply_const(self, name: str, index: Sequence[int], ir_extra: Optional[Dict[str, Any]] = None) -> None:
        idx = self._norm_index(index)
        m = gates.CONSTANT_GATES[name]
        k = int(round(np.log2(m.shape[0])))
        if k != len(idx):
            raise ValueError("gate %s acts on %d qubits, got %d indices" % (name, k, len(idx)))
        ir = {"gatef": getattr(gates, name), "index": tuple(index), "name": name, "split": None, "mpo": False}
        if ir_extra:
            ir.update(ir_extra)
        if name == "i":  # identity: recorded, nothing to apply
            self._qir.append(ir)
            return
        self._record(_Op("const", name, idx, m, gates.is_diagonal(m), k), ir)

    def _apply_var(self, name: str, index: Sequence[int], vars: Dict[str, Any]) -> None:
        localname = vars.pop("name", name)
        split = vars.pop("split", None)
        idx = self._norm_index(index)
        ir = {"gatef": name, "index": tuple(index), "target": list(index), "name": localname, "split": split,
              "mpo": False, "parameters": dict(vars)}
        if name in gates.FAMILIES:
            fam = gates.FAMILIES[name]
            if len(idx) != fam.nq:
                raise ValueError("gate %s acts on %d qubits, got %d indices" % (name, fam.nq, len(idx)))
            data = tuple(vars.get(p, d) for p, d in fam.params)
            if fam.pauli is not None and not _is_complex(data[0]):
                codes = tuple(gates.PAULI_CODE[c] for c in fam.pauli)
                self._record(_Op("prot", name, idx, (data[0], fam.scale, codes), False, fam.nq), ir)
            else:
                self._record(_Op("fam", name, idx, data, fam.diag, fam.nq), ir)
            return
        if name == "any":
            u = vars.get("unitary")
            if u is None:
                raise ValueError("any/unitary gate needs unitary=")
            self._apply_matrix(u, idx, ir, localname)
            return
        if name in ("exp1", "exp"):
            u = vars.get("unitary", vars.get("hermitian", vars.get("hamiltonian")))
            theta = vars.get("theta")
            if u is None or theta is None:
                raise ValueError("%s gate needs unitary= and theta=" % name)
            half = bool(vars.get("half", False))
            un = _to_np_matrix(u)
            d = 1 << len(idx)
            if un is not None and un.shape[0] != d:
                raise ValueError("unitary size does not match %d qubits" % len(idx))
            if name == "exp1":
                codes = _pauli_decompose(un) if un is not None else None
                if codes is not None and any(c != 0 for c in codes) and \
                        sum(c in (1, 2) for c in codes) <= 4 and not _is_complex(theta):
                    # exp1 of a Pauli string: the engine's Pauli-rotation kind
                    # (identity factors dropped)
                    pq = tuple(q for q, c in zip(idx, codes) if c != 0)
                    pc = tuple(c for c in codes if c != 0)
                    self._record(_Op("prot", name, pq, (theta, 0.5 if half else 1.0, pc), False, len(pq)), ir)
                    return
                diag = un is not None and gates.is_diagonal(un)
                self._record(_Op("exp1", name, idx, (theta, u if un is None else un, half), diag, len(idx)), ir)
            else:
                self._record(_Op("exp", name, idx, (theta, u if un is None else un), False, len(idx)), ir)
            return
        raise NotImplementedError("gate %s" % name)

    def _apply_matrix(self, u: Any, idx: Tuple[int, ...], ir: Dict[str, Any], name: str) -> None:
        un = _to_np_matrix(u)
        k = len(idx)
        if k > nat.MAX_GATE_QUBITS:
            raise NotImplementedError("gates on more than %d qubits" % nat.MAX_GATE_QUBITS)
        if un is not None:
            if un.shape[0] != (1 << k):
                raise ValueError("matrix of size %d does not act on %d qubits" % (un.shape[0], k))
            key = "m:" + hashlib.sha1(un.astype(np.complex128).tobytes()).hexdigest()
            gates.CONSTANT_GATES.setdefault(key, un)
            self._record(_Op("const", key, idx, un, gates.is_diagonal(un), k), ir)
        else:
            t = u.tensor if isinstance(u, gates.Gate) else u
            if int(np.prod(t.shape[-2 * k:] if t.dim() >= 2 * k else t.shape)) != (1 << (2 * k)):
                raise ValueError("matrix does not act on %d qubits" % k)
            self._record(_Op("any", "any", idx, t, False, k), ir)

    def apply_general_gate(self, gate: Any, *index: int, name: Optional[str] = None,
                           split: Optional[Dict[str, Any]] = None, mpo: bool = False,
                           ir_dict: Optional[Dict[str, Any]] = None) -> None:
        if mpo:
            raise NotImplementedError("MPO gates are not supported by the statevector engine")
        idx = self._norm_index(index)
        ir = {"gate": gate, "index": index, "name": name or "", "split": split, "mpo": mpo}
        if ir_dict is not None:
            ir_dict.update(ir)
            ir = ir_dict
        self._apply_matrix(gate, idx, ir, name or "any")

    apply = apply_general_gate

    def multicontrol(self, *index: int, ctrl: Union[int, Sequence[int]] = 1, unitary: Any = None,
                     **kws: Any) -> None:
        """Controlled unitary: U on the trailing qubits when the leading
        qubits equal ``ctrl`` (tensorcircuit/gates.py:871-940)."""
        if isinstance(ctrl, int):
            ctrl = [ctrl]
        ctrl = [int(c) for c in ctrl]
        u = _to_np_matrix(unitary)
        if u is None:
            raise NotImplementedError("multicontrol with a traced unitary")
        nc = len(ctrl)
        du = u.shape[0]
        full = np.eye((1 << nc) * du, dtype=np.complex128)
        cidx = 0
        for c in ctrl:
            cidx = cidx * 2 + c
        full[cidx * du:(cidx + 1) * du, cidx * du:(cidx + 1) * du] = u
        idx = self._norm_index(index)
        ir = {"gatef": "multicontrol", "index": tuple(index), "name": "multicontrol", "split": None, "mpo": True,
              "parameters": {"ctrl": ctrl, "unitary": unitary}}
        self._apply_matrix(full, idx, ir, "multicontrol")

    def mpo(self, *index: int, **kws: Any) -> None:
        raise NotImplementedError("MPO gates are not supported by the statevector engine")

    # ------------------------------------------------------------------ noise
    def unitary_kraus(self, kraus: Sequence[Any], *index: int, prob: Optional[Sequence[float]] = None,
                      status: Optional[Any] = None, name: Optional[str] = None) -> Tensor:
        """Apply one operator of ``kraus``, picked by ``status`` (a uniform
        in [0, 1); drawn when None) against the cumulative ``prob``
        (tensorcircuit/circuit.py:473-560).  Without ``prob`` the
        probabilities are tr(K^dag K)/d and each operator is divided by
        sqrt(p).  Returns the pick as an int32 tensor.

        The operator becomes one gate of the engine's plan whose matrix is
        gathered per trajectory from the set, so a ``vmap`` over statuses
        runs every trajectory in the same batched sweep.  A zero-probability
        operator is stored as zero instead of 0/0."""
        idx = self._norm_index(index)
        d = 1 << len(idx)
        mats, is_t = _kraus_mats(kraus, d)
        dev = eng.device()
        if not is_t and (prob is None or not any(isinstance(p, torch.Tensor) for p in
                                                 (prob if _is_seq(prob) else [prob]))):
            key, kdev, cum, diag = _unitary_kraus_prep(mats, prob, d, dev)
        else:
            kt = torch.stack([m.to(dev) if isinstance(m, torch.Tensor) else _dev_const(m, dev) for m in mats])
            if prob is None:
                p = torch.real(torch.einsum("kij,kij->k", kt.conj(), kt)) / d
                pos = p > 0
                inv = torch.where(pos, torch.rsqrt(torch.where(pos, p, torch.ones_like(p))), torch.zeros_like(p))
                kt = kt * inv.to(C64).reshape(-1, 1, 1)
            else:
                p = torch.stack([q.to(device=dev, dtype=torch.float32) if isinstance(q, torch.Tensor)
                                 else torch.full((), float(q), dtype=torch.float32, device=dev) for q in prob])
            cum = torch.cumsum(p.to(torch.float32), -1)
            diag = False
            key, kdev = ("t", len(mats), d), kt.reshape(len(mats), d * d)
        r = _pick(status, cum, dev)
        ir = {"gatef": "unitary_kraus", "index": tuple(index), "name": name or "unitary_kraus", "split": None,
              "mpo": False, "parameters": {"prob": prob, "status": status}}
        self._record(_Op("kraus", "kraus", idx, (key, kdev, r), diag, len(idx)), ir)
        return r

    unitary_kraus2 = unitary_kraus

    def general_kraus(self, kraus: Sequence[Any], *index: int, status: Optional[Any] = None,
                      with_prob: bool = False, name: Optional[str] = None) -> Any:
        """Monte-Carlo trajectory step of a general channel
        (tensorcircuit/circuit.py:635-724): p_i = <psi|K_i^dag K_i|psi>,
        the pick of ``unitary_kraus`` with those probabilities, and the
        state continues as K_r psi / (sqrt(p_r) + 1e-10).

        The p_i come from ONE measurement pass over the current state: K_i^dag
        K_i expanded in the 4^k Pauli strings of its qubits, all measured by
        the engine's Pauli kernel (differentiable through the adjoint sweep).
        The gates so far become a finished segment; its rescaled output is
        the next segment's input and K_r that segment's first gate (for
        constant operators; operators given as tensors are applied to the
        state directly, so that their gradients are exact).  Returns the
        pick (and, with ``with_prob``, the list of p_i)."""
        idx = self._norm_index(index)
        k = len(idx)
        d = 1 << k
        mats, is_t = _kraus_mats(kraus, d)
        dev = eng.device()
        strings = _pauli_strings(k)
        if is_t:
            kt = torch.stack([m if isinstance(m, torch.Tensor) else _dev_const(m, dev) for m in mats]).to(dev)
            mm = torch.einsum("kji,kjl->kil", kt.conj(), kt)
            coef = torch.real(torch.einsum("kil,sli->ks", mm, _pauli_stack(k, dev))) / d
        else:
            key, kdev, coef, diag = _kraus_prep(mats, k, dev)
        psi, psi_eng, anchor, run, n_eng = self._engine_state()
        spec = _kraus_spec(idx, n_eng)
        evc = eng.ExpectFn.apply(psi_eng, anchor, spec, run)
        if is_t or with_prob:
            # p itself is wanted (or depends on the operators' gradients):
            # the same steps as torch operations
            ev = torch.real(evc)
            p = ev @ coef.t()
            r = _pick(status, torch.cumsum(p, -1), dev)
            pr = torch.sum(torch.where(r.unsqueeze(-1) == _arange(len(mats), dev), p, 0.0), -1)
            scale = (1.0 / (torch.sqrt(pr) + 1e-10)).to(C64)
        else:
            # constant operators: probabilities, pick and rescale in one kernel
            r, scale, p = eng.KrausPickFn.apply(evc, coef, _uniform(status, dev))
        ir = {"gatef": "general_kraus", "index": tuple(index), "name": name or "general_kraus", "split": None,
              "mpo": False, "parameters": {"status": status}}
        self._seg_ops += len(self._ops)
        self._ops = []
        if is_t:
            kr = kt[r.long()]
            self._seg_input = _apply_local(psi, kr, idx, self._nqubits) * scale.unsqueeze(-1)
            self._qir.append(ir)
            self._cache = None
            self._req_terms = []
            self._pred_terms = None
            self._term_batch = None
        else:
            self._seg_input = psi * scale.unsqueeze(-1)
            self._record(_Op("kraus", "kraus", idx, (key, kdev, r), diag, k), ir)
        if with_prob:
            return r, list(p.unbind(-1))
        return r

    apply_general_kraus = general_kraus

    def depolarizing2(self, index: int, *, px: float, py: float, pz: float,
                      status: Optional[Any] = None) -> float:
        """X, Y, Z or I on ``index`` with probabilities px, py, pz, rest
        (tensorcircuit/circuit.py:354-386)."""
        self.unitary_kraus([gates.CONSTANT_GATES["x"], gates.CONSTANT_GATES["y"], gates.CONSTANT_GATES["z"],
                            gates.CONSTANT_GATES["i"]], index, prob=[px, py, pz, 1 - px - py - pz],
                           status=status)
        return 0.0

    def depolarizing_reference(self, index: int, *, px: float, py: float, pz: float,
                               status: Optional[Any] = None) -> Tensor:
        """As :meth:`depolarizing2`, returning the pick [0: X, 1: Y, 2: Z,
        3: I] (tensorcircuit/circuit.py:389-445)."""
        return self.unitary_kraus([gates.CONSTANT_GATES["x"], gates.CONSTANT_GATES["y"],
                                   gates.CONSTANT_GATES["z"], gates.CONSTANT_GATES["i"]], index,
                                  prob=[px, py, pz, 1 - px - py - pz], status=status)

    def _apply_nonunitary(self, m: Any, idx: Tuple[int, ...], ir: Dict[str, Any]) -> None:
        """Apply a non-unitary operator (projector, superoperator).

        The adjoint sweep un-applies a segment's gates with G^dag to rebuild
        the state each gradient needs; that is exact for unitary gates and
        wrong for this one, while the cotangent it passes on (m^dag mu) is
        exact either way.  So a constant non-unitary operator may sit in a
        segment only ahead of every gate that takes a gradient: it joins the
        current segment while that holds only constant gates, and otherwise
        starts a new one, whose input is the current output state.  Tensors
        that need gradients are applied to the materialised state by a
        torch contraction."""
        if not isinstance(m, torch.Tensor) and all(op.kind == "const" for op in self._ops):
            m = np.asarray(m, dtype=np.complex128)
            key = "m:" + hashlib.sha1(m.tobytes()).hexdigest()
            Circuit._record(self, _Op("const", key, idx, m, gates.is_diagonal(m), len(idx)), ir)
            return
        psi = self._engine_state()[0]
        self._seg_ops += len(self._ops)
        self._ops = []
        if isinstance(m, torch.Tensor):
            self._seg_input = _apply_local(psi, m.to(device=psi.device, dtype=C64), idx, self._nvec)
            self._qir.append(ir)
            self._cache = None
            self._req_terms = []
            self._pred_terms = None
            self._term_batch = None
            return
        m = np.asarray(m, dtype=np.complex128)
        self._seg_input = psi
        key = "m:" + hashlib.sha1(m.tobytes()).hexdigest()
        Circuit._record(self, _Op("const", key, idx, m, gates.is_diagonal(m), len(idx)), ir)

    def mid_measurement(self, index: int, keep: int = 0) -> Tensor:
        """Post-select qubit ``index`` on |keep> (unnormalised), returning
        ``keep`` as an int32 tensor (tensorcircuit/circuit.py:302-348)."""
        idx = self._norm_index([index])
        proj = np.diag([1.0, 0.0]) if keep < 0.5 else np.diag([0.0, 1.0])
        ir = {"gatef": "mid_measurement", "index": (index,), "name": "mid_measurement", "split": None,
              "mpo": False, "parameters": {"keep": keep}}
        self._apply_nonunitary(proj, idx, ir)
        return torch.full((), int(keep >= 0.5), dtype=torch.int32, device=eng.device())

    mid_measure = mid_measurement
    post_select = mid_measurement
    post_selection = mid_measurement

    def cond_measurement(self, index: int, status: Optional[Any] = None) -> Tensor:
        """Z measurement of qubit ``index`` that collapses the trajectory:
        ``general_kraus`` with the two projectors (basecircuit.py:824-853).
        Returns the outcome."""
        return self.general_kraus([np.diag([1.0, 0.0]), np.diag([0.0, 1.0])], index, status=status,
                                  name="measure")

    cond_measure = cond_measurement

    def select_gate(self, which: Any, kraus: Sequence[Any], *index: int) -> None:
        """Apply ``kraus[which]`` for an int tensor ``which``
        (abstractcircuit.py:1076-1095): one engine gate whose matrix row is
        gathered per batch element."""
        idx = self._norm_index(index)
        d = 1 << len(idx)
        mats, is_t = _kraus_mats(kraus, d)
        dev = eng.device()
        if is_t:
            kt = torch.stack([m.to(dev) if isinstance(m, torch.Tensor) else _dev_const(m, dev) for m in mats])
            key, kdev, diag = ("t", len(mats), d), kt.reshape(len(mats), d * d), False
        else:
            diag = all(gates.is_diagonal(m) for m in mats)
            key, kdev = _kraus_device_set(mats, np.zeros(0), diag, dev)
        if isinstance(which, torch.Tensor):
            r = which.to(device=dev, dtype=torch.int32)
        else:
            r = torch.full((), int(which), dtype=torch.int32, device=dev)
        ir = {"gatef": "select_gate", "index": tuple(index), "name": "select_gate", "split": None, "mpo": False,
              "parameters": {"which": which}}
        self._record(_Op("kraus", "kraus", idx, (key, kdev, r), diag, len(idx)), ir)

    conditional_gate = select_gate

    def _probability_vector(self) -> Tensor:
        psi = self.wavefunction()
        return torch.real(psi * torch.conj(psi))

    def measure_jit(self, *index: int, with_prob: bool = False, status: Optional[Any] = None) -> Tuple[Tensor, Any]:
        """Sequential Z measurement of ``index`` (basecircuit.py:371-441):
        for the k-th qubit, pu = P(0 | earlier outcomes), outcome
        int(sign(status[k] - pu + eps)/2 + 1/2) with eps = 0.31415926e-12,
        and p multiplied by pu or 1 - pu.  The marginals come from one
        probability vector summed over the unmeasured qubits."""
        n = self._nqubits
        idx = [int(i) if int(i) >= 0 else n + int(i) for i in index]
        p = self._probability_vector()
        dev = p.device
        lead = p.shape[:-1]
        t = p.reshape(lead + (2,) * n)
        nl = len(lead)
        rest = [nl + q for q in range(n) if q not in idx]
        if rest:
            t = t.sum(dim=rest)
        # order the measured qubits as requested
        order = sorted(range(len(idx)), key=lambda j: idx[j])
        perm = list(range(nl)) + [nl + order.index(j) for j in range(len(idx))]
        t = t.permute(perm)
        if status is None:
            u = torch.rand(lead + (len(idx),), device=dev)
        else:
            u = status if isinstance(status, torch.Tensor) else torch.as_tensor(np.asarray(status, dtype=np.float32))
            u = torch.real(u).to(device=dev, dtype=torch.float32)
        prob = torch.ones(lead, dtype=torch.float32, device=dev)
        bits = []
        cur = t
        for k in range(len(idx)):
            marg = cur.sum(dim=tuple(range(nl + 1, cur.dim()))) if cur.dim() > nl + 1 else cur
            pu = marg[..., 0] / prob
            s = torch.sign(u[..., k] - pu + 0.31415926e-12) / 2 + 0.5
            bits.append(s)
            prob = prob * (pu * (1 - 2 * s) + s)
            # condition on the outcome: keep the slice of the drawn bit
            one = (s > 0.5).reshape(lead + (1,) * (cur.dim() - nl - 1))
            cur = torch.where(one, cur.select(nl, 1), cur.select(nl, 0))
        sample = torch.stack(bits, -1)
        if with_prob:
            return sample, prob
        return sample, -1.0

    measure = measure_jit

    def perfect_sampling(self, status: Optional[Any] = None) -> Tuple[Tensor, Tensor]:
        """All qubits by ``measure_jit`` (basecircuit.py:359-369)."""
        return self.measure_jit(*range(self._nqubits), with_prob=True, status=status)

    @staticmethod
    def apply_general_kraus_delayed(krausf: Any, is_unitary: bool = False) -> Any:
        """Circuit method for a channel constructor
        (tensorcircuit/circuit.py:727-745)."""

        def apply(self: "Circuit", *index: int, status: Optional[Any] = None, name: Optional[str] = None,
                  **vars: Any) -> None:
            kraus = krausf(**vars)
            if is_unitary:
                self.unitary_kraus(kraus, *index, status=status, name=name)
            else:
                self.general_kraus(kraus, *index, status=status, name=name)

        return apply

    # ------------------------------------------------------------------ state
    def _engine_state(self) -> Tuple[torch.Tensor, torch.Tensor, torch.Tensor, eng.Run, int]:
        if self._cache is not None:
            return self._cache  # type: ignore
        dev = eng.device()
        n = self._nvec
        n_eng = max(n, nat.MIN_QUBITS)
        pad = n_eng - n
        key = _struct_key(n_eng, self._ops)
        entry = _entries.get(key)
        if entry is None:
            entry = _build_entry(n_eng, self._ops)
            _entries[key] = entry
        blocks = []
        cb = entry.const_block(dev)
        if cb is not None:
            blocks.append(cb)
        for gkey, idx, E in entry.groups:
            b = _group_block(gkey, self._ops, idx, dev).to(C64)
            blocks.append(b.reshape(b.shape[:-2] + (b.shape[-2] * b.shape[-1],)))
        if blocks:
            if len(blocks) > 1 and len({tuple(b.shape[:-1]) for b in blocks}) > 1:
                # some groups carry batch dimensions (per-trajectory Kraus
                # picks, batched parameters): broadcast the others to them
                lead = torch.broadcast_shapes(*[b.shape[:-1] for b in blocks])
                blocks = [b.expand(lead + b.shape[-1:]) for b in blocks]
            mats = blocks[0] if len(blocks) == 1 else torch.cat(blocks, -1)
        else:
            mats = torch.zeros(1, dtype=C64, device=dev)
        # input state
        N = 1 << n
        inp = self._seg_input if self._seg_input is not None else self.inputs
        if inp is None:
            psi0 = _basis0(n_eng, dev)
        else:
            if isinstance(inp, gates.Gate):
                inp = inp.tensor
            if not isinstance(inp, torch.Tensor):
                inp = torch.as_tensor(np.asarray(inp, dtype=np.complex64))
            inp = inp.to(device=dev, dtype=C64)
            if inp.shape[-1] != N:
                inp = inp.reshape(-1)  # the [2] * n leg form
            if inp.shape[-1] != N:
                raise ValueError("inputs has %d amplitudes, %d qubits need %d" % (inp.shape[-1], n, N))
            if pad:
                inp = torch.cat([inp.unsqueeze(-1), torch.zeros(inp.shape + ((1 << pad) - 1,), dtype=C64,
                                                                device=dev)], -1).reshape(inp.shape[:-1] + (1 << n_eng,))
            psi0 = inp
        run = eng.Run(entry.plan, n_eng)
        psi_eng, anchor = eng.StateFn.apply(mats, psi0, run)
        self._req_terms = []
        self._term_batch = None
        self._pred_terms = entry.last_terms
        entry.last_terms = self._req_terms
        psi = psi_eng if pad == 0 else psi_eng.reshape(psi_eng.shape[:-1] + (N, 1 << pad))[..., 0]
        self._cache = (psi, psi_eng, anchor, run, n_eng)
        return self._cache  # type: ignore

    def wavefunction(self, form: str = "default") -> Tensor:
        psi = self._engine_state()[0]
        if form == "default":
            return psi
        if form == "ket":
            return psi.reshape(psi.shape[:-1] + (-1, 1))
        if form == "bra":
            return psi.reshape(psi.shape[:-1] + (1, -1))
        raise ValueError("unknown form %s" % form)

    state = wavefunction

    def get_state_as_quvector(self) -> Any:
        raise NotImplementedError("QuVector views are tensor-network objects; use wavefunction()")

    quvector = get_state_as_quvector

    def matrix(self) -> Tensor:
        """The circuit unitary, from running the plan on all 2^n basis states
        as one batch."""
        if self._seg_input is not None:
            raise ValueError("a circuit with general Kraus channels has no unitary")
        n = self._nqubits
        dev = eng.device()
        c = Circuit(n, inputs=torch.eye(1 << n, dtype=C64, device=dev))
        c._ops = list(self._ops)
        c._qir = list(self._qir)
        return c.wavefunction().transpose(-1, -2)

    # ------------------------------------------------------------ observables
    def _pauli_term(self, x: Sequence[int], y: Sequence[int], z: Sequence[int], n_eng: int) -> Tuple[int, int]:
        n = self._nqubits
        occupied = set()
        norm = []
        for lst in (x, y, z):
            out = []
            for q in lst:
                q = int(q)
                q = q if q >= 0 else n + q
                if not 0 <= q < n:
                    raise ValueError("qubit index out of range")
                if q in occupied:
                    raise ValueError("Cannot measure two operators in one index")
                occupied.add(q)
                out.append(q)
            norm.append(out)
        return eng.pauli_masks(n_eng, *norm)

    def expectation_ps(self, x: Optional[Sequence[int]] = None, y: Optional[Sequence[int]] = None,
                       z: Optional[Sequence[int]] = None, ps: Optional[Sequence[int]] = None, reuse: bool = True,
                       noise_conf: Optional[Any] = None, nmc: int = 1000, status: Optional[Tensor] = None,
                       **kws: Any) -> Tensor:
        """Pauli-string expectation (tensorcircuit/abstractcircuit.py:1208-1288).

        ``ps`` codes 0/1/2/3 = I/X/Y/Z override x/y/z.  Returns a complex64
        tensor, like the reference."""
        if noise_conf is not None:
            raise NotImplementedError("noisy expectations are outside the statevector engine")
        if ps is not None:
            from .quantum import ps2xyz

            d = ps2xyz(list(ps))
            x, y, z = d.get("x", None), d.get("y", None), d.get("z", None)
        _, psi_eng, anchor, run, n_eng = self._engine_state()
        term = self._pauli_term(x or [], y or [], z or [], n_eng)
        return self._expect_pauli(term)

    def _expect_pauli(self, term: Tuple[int, int]) -> Tensor:
        """<P> for one Pauli term (masks over the engine's index bits).

        VQE-style code asks a circuit for the same list of terms every step
        (one ``expectation_ps`` per Hamiltonian term, as in the reference's
        benchmarks/scripts/vqe_tc.py:75-81).  The first request evaluates every
        term the previous circuit of this structure asked for in ONE
        measurement plan (a few reads of the state instead of one read per
        term); a request returns a slice of that batch only when it is exactly
        the predicted term at that position, otherwise it is evaluated on its
        own."""
        _, psi_eng, anchor, run, n_eng = self._engine_state()
        i = len(self._req_terms)
        self._req_terms.append(term)
        pred = self._pred_terms
        if pred is not None and len(pred) > 1 and i < len(pred) and pred[i] == term:
            if self._term_batch is None:
                # unbound once: the backward of all the slices is one stack
                self._term_batch = eng.ExpectFn.apply(psi_eng, anchor, tuple(pred), run).unbind(-1)
            return self._term_batch[i]
        return eng.ExpectFn.apply(psi_eng, anchor, (term,), run)[..., 0]

    def expectation_ps_batch(self, terms: Sequence[Dict[str, Sequence[int]]]) -> Tensor:
        """Many Pauli strings in one call (one engine measurement plan).

        ``terms`` is a list of ``{"x": [...], "y": [...], "z": [...]}``; the
        result has one complex entry per term in the last dimension."""
        _, psi_eng, anchor, run, n_eng = self._engine_state()
        spec = tuple(self._pauli_term(t.get("x", []), t.get("y", []), t.get("z", []), n_eng) for t in terms)
        return eng.ExpectFn.apply(psi_eng, anchor, spec, run)

    def expectation(self, *ops: Any, reuse: bool = True, enable_lightcone: bool = False,
                    noise_conf: Optional[Any] = None, nmc: int = 1000, status: Optional[Tensor] = None,
                    **kws: Any) -> Tensor:
        """<psi| (x)_k O_k |psi> for ``(operator, [indices])`` pairs
        (tensorcircuit/circuit.py:914-981).  Pauli products take the
        measurement kernel; other operators are applied to a copy of the
        state by a forward sweep and contracted."""
        if noise_conf is not None:
            raise NotImplementedError("noisy expectations are outside the statevector engine")
        n = self._nqubits
        occupied = set()
        xs: List[int] = []
        ys: List[int] = []
        zs: List[int] = []
        general: List[Tuple[Any, Tuple[int, ...]]] = []
        for op, index in ops:
            if isinstance(index, (int, np.integer)):
                index = [int(index)]
            idx = tuple(int(i) if int(i) >= 0 else n + int(i) for i in index)
            for q in idx:
                if q in occupied:
                    raise ValueError("Cannot measure two operators in one index")
                occupied.add(q)
            m = _to_np_matrix(op)
            codes = _pauli_decompose(m) if m is not None and m.shape[0] == (1 << len(idx)) else None
            if codes is not None:
                for c, q in zip(codes, idx):
                    if c == 1:
                        xs.append(q)
                    elif c == 2:
                        ys.append(q)
                    elif c == 3:
                        zs.append(q)
            else:
                general.append((op, idx))
        psi, psi_eng, anchor, run, n_eng = self._engine_state()
        if not general:
            return self._expect_pauli(eng.pauli_masks(n_eng, xs, ys, zs))
        # general operators: phi = O psi through a forward sweep on a copy
        c = Circuit(n, inputs=psi)
        for op, idx in general:
            c._apply_matrix(op, idx, {"gate": op, "index": idx, "name": "op"}, "op")
        for q in xs:
            c._apply_const("x", [q])
        for q in ys:
            c._apply_const("y", [q])
        for q in zs:
            c._apply_const("z", [q])
        phi = c.wavefunction()
        return torch.sum(torch.conj(psi) * phi, -1)

    def probability(self) -> Tensor:
        """|psi|^2 over the computational basis (basecircuit.py:510-523), by
        the engine's probability kernel (computed as re^2 + im^2; the
        reference squares abs(psi), which can differ in the last bit),
        differentiable through its autograd Function."""
        return eng.ProbabilityFn.apply(self.wavefunction())

    def amplitude(self, l: Union[str, Tensor]) -> Tensor:
        """<l|psi> for a bitstring (basecircuit.py:447-508)."""
        psi = self.wavefunction()
        n = self._nqubits
        if isinstance(l, str):
            if len(l) != n:
                raise ValueError("bitstring length %d != %d qubits" % (len(l), n))
            return psi[..., int(l, 2)]
        lt = l if isinstance(l, torch.Tensor) else torch.as_tensor(np.asarray(l))
        lt = lt.to(device=psi.device, dtype=C64)
        t = psi.reshape(psi.shape[:-1] + (2,) * n)
        for i in range(n):
            vec = torch.stack([1 - lt[..., i], lt[..., i]], -1)
            t = torch.sum(t * vec.reshape(vec.shape[:-1] + (2,) + (1,) * (n - 1 - i)), dim=-(n - i))
        return t

    def sample(self, batch: Optional[int] = None, allow_state: bool = False,
               readout_error: Optional[Sequence[Any]] = None, format: Optional[str] = None,
               random_generator: Optional[Any] = None, status: Optional[Tensor] = None, **kws: Any) -> Any:
        """Samples of the final state (basecircuit.py:525-616).

        With ``status`` (uniforms in [0, 1)) the draw follows the reference's
        inverse-CDF rule bit-exactly under the engine's declared integer CDF
        (see ``include/tcgb300.h``).  Without it, uniforms come from torch's
        generator (``random_generator`` may be a ``torch.Generator``).
        ``allow_state=False`` selects the reference's per-qubit perfect
        sampling there; the samples here come from the same distribution
        through the state's CDF."""
        if "format_" in kws:
            format = kws.pop("format_")
        if readout_error is not None:
            raise NotImplementedError("readout error is outside the statevector engine")
        nb = 1 if batch is None else int(batch)
        psi, psi_eng, anchor, run, n_eng = self._engine_state()
        dev = psi_eng.device
        if status is None:
            gen = random_generator if isinstance(random_generator, torch.Generator) else None
            if gen is not None and gen.device.type != "cuda":
                u = torch.rand(nb, generator=gen).to(dev)
            else:
                u = torch.rand(nb, generator=gen, device=dev)
        else:
            u = status if isinstance(status, torch.Tensor) else torch.as_tensor(np.asarray(status))
            u = u.to(device=dev, dtype=torch.float32)
            if u.shape[-1] < nb:
                raise ValueError("status has %d draws, batch needs %d" % (u.shape[-1], nb))
            u = u[..., :nb]
        ch = eng.SampleFn.apply(psi_eng, u, n_eng, nb)
        pad = n_eng - self._nqubits
        if pad:
            ch = torch.bitwise_right_shift(ch, pad)
        n = self._nqubits
        if format is None:
            confg = sample_int2bin(ch, n)
            p = torch.abs(psi.detach()) ** 2
            prob = torch.gather(p, -1, ch)
            r = list(zip(confg, prob))
            if batch is None:
                return r[0]
            return r
        return sample2all(sample=ch, n=n, format=format, jittable=True)

    def sample_expectation_ps(self, x: Optional[Sequence[int]] = None, y: Optional[Sequence[int]] = None,
                              z: Optional[Sequence[int]] = None, shots: Optional[int] = None,
                              random_generator: Optional[Any] = None, status: Optional[Tensor] = None,
                              readout_error: Optional[Sequence[Any]] = None, noise_conf: Optional[Any] = None,
                              nmc: int = 1000, statusc: Optional[Tensor] = None, **kws: Any) -> Tensor:
        """Pauli expectation from measurement shots (basecircuit.py:618-756):
        rotate X sites by H and Y sites by rx(pi/2), then average the parity
        of the measured bits.  ``shots=None`` gives the exact value."""
        if noise_conf is not None or readout_error is not None:
            raise NotImplementedError("noisy sampling is outside the statevector engine")
        x, y, z = list(x or []), list(y or []), list(z or [])
        if shots is None:
            return torch.real(self.expectation_ps(x=x, y=y, z=z))
        c = self._measurement_copy()
        for i in x:
            c.H(i)
        for i in y:
            c.rx(i, theta=np.pi / 2)
        s = c.sample(batch=shots, allow_state=True, status=status, random_generator=random_generator,
                     format="sample_bin")
        sites = [q if q >= 0 else self._nqubits + q for q in x + y + z]
        if not sites:
            return torch.ones(s.shape[:-2], dtype=torch.float32, device=s.device)
        par = torch.sum(s[..., sites], -1) % 2
        return torch.mean((1 - 2 * par).to(torch.float32), -1)

    sexpps = sample_expectation_ps

    def _measurement_copy(self) -> "Circuit":
        """A fresh circuit starting from this one's output state."""
        return Circuit(self._nqubits, inputs=self.wavefunction())

    # ---------------------------------------------------------------- misc
    def to_qir(self) -> List[Dict[str, Any]]:
        return self._qir

    # Entries that are trajectory draws or projections rather than gates;
    # rebuilding a circuit from its qir (from_qir, inverse, to_circuit)
    # leaves them out, as the reference's qir holds gates only.
    _NON_GATE_QIR = ("unitary_kraus", "general_kraus", "mid_measurement", "select_gate")

    @staticmethod
    def _qir_name(d: Dict[str, Any]) -> str:
        g = d.get("gatef")
        if isinstance(g, str):
            return g
        if g is not None and hasattr(g, "n"):
            return g.n
        return d.get("name") or "any"

    @classmethod
    def from_qir(cls, qir: List[Dict[str, Any]], circuit_params: Optional[Dict[str, Any]] = None) -> "Circuit":
        """Rebuild a circuit from its gate records (abstractcircuit.py:
        366-425); ``nqubits`` defaults to one more than the largest index."""
        params = dict(circuit_params or {})
        if "nqubits" not in params:
            params["nqubits"] = 1 + max((max(d["index"]) for d in qir if d.get("index")), default=0)
        c = cls(**params)
        return cls._apply_qir(c, qir)

    @staticmethod
    def _apply_qir(c: "Circuit", qir: List[Dict[str, Any]]) -> "Circuit":
        for d in qir:
            name = Circuit._qir_name(d)
            if name in Circuit._NON_GATE_QIR:
                continue
            idx = tuple(d["index"])
            if "gatef" not in d or d.get("gatef") is None:
                c.apply_general_gate(d["gate"], *idx, name=d.get("name"))
            elif "parameters" in d:
                getattr(c, name)(*idx, **dict(d["parameters"]))
            else:
                getattr(c, name)(*idx)
        return c

    def append_from_qir(self, qir: List[Dict[str, Any]]) -> None:
        self._apply_qir(self, qir)

    def prepend(self, c: "Circuit") -> "Circuit":
        """``c``'s gates, then this circuit's (abstractcircuit.py:1133-1146)."""
        newc = type(self).from_qir(c.to_qir() + self.to_qir(), dict(self.circuit_param))
        self.__dict__.update(newc.__dict__)
        return self

    def append(self, c: "Circuit", indices: Optional[List[int]] = None) -> "Circuit":
        """This circuit's gates, then ``c``'s, with ``c``'s qubit i placed on
        ``indices[i]`` (abstractcircuit.py:1148-1183)."""
        qir = c.to_qir()
        if indices is not None:
            qir = [dict(d, index=tuple(indices[i] for i in d["index"])) for d in qir]
        self._apply_qir(self, qir)
        return self

    def inverse(self, circuit_params: Optional[Dict[str, Any]] = None) -> "Circuit":
        """The adjoint circuit: gates in reverse order, each inverted
        (abstractcircuit.py:428-507): self-inverse constant gates repeat,
        sd/td become s/t and s/t/wroot their adjoints, rotations negate
        theta (iswap's default angle is 1), u/cu map (phi, lbd) to
        (pi - lbd, pi - phi), ``any`` takes the conjugate transpose."""
        params = dict(circuit_params or {})
        params.setdefault("nqubits", self._nqubits)
        c = type(self)(**params)
        self_inverse = [g for g in gates.sgates if g not in ("wroot", "sd", "td", "s", "t")]
        for d in reversed(self._qir):
            name = self._qir_name(d)
            if name in self._NON_GATE_QIR:
                continue
            idx = tuple(d["index"])
            if d.get("gatef") is None:
                # a general gate recorded by its matrix
                m = d["gate"].tensor if isinstance(d.get("gate"), gates.Gate) else d.get("gate")
                if isinstance(m, torch.Tensor):
                    dd = int(round(m.numel() ** 0.5))
                    m = torch.conj(m.reshape(dd, dd)).transpose(0, 1)
                else:
                    m = _to_np_matrix(m).conj().T
                c.apply_general_gate(m, *idx, name=d.get("name"))
                continue
            if "parameters" not in d:
                if name in self_inverse:
                    getattr(c, name)(*idx)
                elif name in ("sd", "td"):
                    getattr(c, name[:-1])(*idx)
                else:
                    c.apply_general_gate(_to_np_matrix(gates.CONSTANT_GATES[name]).conj().T, *idx, name=name)
                continue
            p = dict(d["parameters"])
            if name in ("u", "cu"):
                phi, lbd = p.get("phi", 0.0), p.get("lbd", 0.0)
                p["lbd"], p["phi"] = -phi + np.pi, -lbd + np.pi
            elif name == "any":
                u = p["unitary"]
                u = u.tensor if isinstance(u, gates.Gate) else u
                if isinstance(u, torch.Tensor):
                    dd = int(round(u.numel() ** 0.5))
                    p["unitary"] = torch.conj(u.reshape(dd, dd)).transpose(0, 1)
                else:
                    p["unitary"] = _to_np_matrix(u).conj().T
            elif name == "multicontrol":
                u = _to_np_matrix(p["unitary"])
                p["unitary"] = u.conj().T
            else:
                p["theta"] = -p.get("theta", 1.0 if name == "iswap" else 0.0)
            getattr(c, name)(*idx, **p)
        return c

    def __len__(self) -> int:
        return self._seg_ops + len(self._ops)

    @staticmethod
    def standardize_gate(name: str) -> str:
        """The canonical name of a gate alias (cx -> cnot, ccx -> toffoli)."""
        name = name.lower()
        for group in gates.gate_aliases:
            if name in group:
                return group[0]
        return name

    def gate_count(self, gate_list: Optional[Union[str, Sequence[str]]] = None) -> int:
        """Number of recorded gates, or of those whose canonical name is in
        ``gate_list`` (abstractcircuit.py:623-653)."""
        if gate_list is None:
            return len(self._qir)
        if isinstance(gate_list, str):
            gate_list = [gate_list]
        names = {self.standardize_gate(g) for g in gate_list}
        return sum(1 for d in self._qir if self._qir_name(d) in names)

    def gate_count_by_condition(self, cond_func: Any) -> int:
        return sum(1 for d in self._qir if cond_func(d))

    def gate_summary(self) -> Dict[str, int]:
        summary: Dict[str, int] = {}
        for d in self._qir:
            summary[d["name"]] = summary.get(d["name"], 0) + 1
        return summary

    # --------------------------------------------------------------- text I/O
    def to_json(self, file: Optional[str] = None, simplified: bool = False) -> str:
        """The gate records as JSON (tensorcircuit/translation.py:616-673)."""
        from . import translation

        s = translation.dumps(self.to_qir(), simplified=simplified)
        if file is not None:
            with open(file, "w") as fh:
                fh.write(s)
        return s

    @classmethod
    def from_json(cls, jsonstr: Any, circuit_params: Optional[Dict[str, Any]] = None) -> "Circuit":
        import json

        from . import translation

        data = json.loads(jsonstr) if isinstance(jsonstr, str) else jsonstr
        return cls.from_qir(translation.json2qir(data), circuit_params)

    @classmethod
    def from_json_file(cls, file: str, circuit_params: Optional[Dict[str, Any]] = None) -> "Circuit":
        with open(file) as fh:
            return cls.from_json(fh.read(), circuit_params)

    def to_openqasm(self, **kws: Any) -> str:
        """OpenQASM 2 text with the qelib1 gates (the reference goes through
        qiskit, abstractcircuit.py:793-802); other 1-qubit gates become u3
        (global phase dropped), other multi-qubit gates raise."""
        from . import translation

        return translation.qir2qasm(self.to_qir(), self._nqubits)

    @classmethod
    def from_openqasm(cls, qasmstr: str, circuit_params: Optional[Dict[str, Any]] = None,
                      keep_measure_order: bool = False) -> "Circuit":
        from . import translation

        return translation.qasm2circuit(qasmstr, cls, circuit_params)

    @classmethod
    def from_openqasm_file(cls, file: str, circuit_params: Optional[Dict[str, Any]] = None,
                           keep_measure_order: bool = False) -> "Circuit":
        with open(file) as fh:
            return cls.from_openqasm(fh.read(), circuit_params)

    @classmethod
    def from_qsim_file(cls, file: str, circuit_params: Optional[Dict[str, Any]] = None) -> "Circuit":
        """A qsim circuit file: the qubit count on the first line, then one
        gate per line."""
        from . import translation

        with open(file) as fh:
            lines = fh.readlines()
        params = dict(circuit_params or {})
        params.setdefault("nqubits", int(lines[0]))
        return translation.apply_qsim(cls(**params), lines[1:])

    def engine_stats(self) -> Dict[str, int]:
        """Pass/stage counts of the plan the engine uses for this circuit."""
        _, _, _, run, n_eng = self._engine_state()
        return {"nqubits": n_eng, "gates": run.plan.ngates, "passes": run.plan.npasses,
                "stages": run.plan.nstages, "tile_bits": run.plan.tile_bits}


_basis_cache: Dict[Tuple[int, int], torch.Tensor] = {}


def _basis0(n: int, dev: torch.device) -> torch.Tensor:
    key = (n, dev.index)
    t = _basis_cache.get(key)
    if t is None:
        t = torch.zeros(1 << n, dtype=C64, device=dev)
        t[0] = 1.0
        _basis_cache[key] = t
    return t


# ----------------------------------------------------------------------------
# gate-method registration (tensorcircuit/abstractcircuit.py:218-326)
# ----------------------------------------------------------------------------
def _make_sgate(name: str) -> Any:
    def apply(self: Circuit, *index: Any, split: Optional[Dict[str, Any]] = None, name_: Optional[str] = None,
              **kws: Any) -> None:
        if index and _is_seq(index[0]):
            for ind in zip(*index):
                self._apply_const(name, ind)
            return
        self._apply_const(name, index)

    apply.__name__ = name
    apply.__doc__ = "Apply the constant **%s** gate (tensorcircuit/gates.py)." % name.upper()
    return apply


def _make_vgate(name: str) -> Any:
    def apply(self: Circuit, *index: Any, **vars: Any) -> None:
        if index and _is_seq(index[0]):
            for i, ind in enumerate(zip(*index)):
                nvars = {}
                for k, v in vars.items():
                    try:
                        nvars[k] = v[i]
                    except Exception:  # scalars broadcast to every index
                        nvars[k] = v
                self._apply_var(name, ind, nvars)
            return
        self._apply_var(name, index, dict(vars))

    apply.__name__ = name
    apply.__doc__ = "Apply the parameterized **%s** gate (tensorcircuit/gates.py)." % name.upper()
    return apply


for _g in gates.sgates:
    setattr(Circuit, _g, _make_sgate(_g))
    setattr(Circuit, _g.upper(), _make_sgate(_g))
for _g in gates.vgates:
    setattr(Circuit, _g, _make_vgate(_g))
    setattr(Circuit, _g.upper(), _make_vgate(_g))
setattr(Circuit, "MULTICONTROL", Circuit.multicontrol)
setattr(Circuit, "MPO", Circuit.mpo)
for _a in gates.gate_aliases:
    for _alias in _a[1:]:
        setattr(Circuit, _alias, getattr(Circuit, _a[0]))
        setattr(Circuit, _alias.upper(), getattr(Circuit, _a[0].upper()))

# channel methods (tensorcircuit/circuit.py:747-764): depolarizing and
# generaldepolarizing through unitary_kraus, the others through general_kraus
for _c in _channels.channels:
    setattr(Circuit, _c, Circuit.apply_general_kraus_delayed(getattr(_channels, _c + "channel"),
                                                             is_unitary=_c in _channels.UNITARY_CHANNELS))
