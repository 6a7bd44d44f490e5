"""``DMCircuit``: density-matrix simulation on the statevector engine.

Mirrors tensorcircuit/densitymatrix.py: ``DMCircuit2`` (superoperator
channels, exported by the reference as ``DMCircuit``) and the index form of
``DMCircuit_reference.apply_general_kraus`` (a list with one index tuple).

Layout: rho on n qubits is the 2n-qubit vector vec(rho)[a * 2^n + b] =
rho[a, b] -- the row index on the first n engine qubits, the column index on
the last n -- evolved by the same engine as pure states:

* a gate G on qubits idx is G on idx and conj(G) on idx + n: two unitary
  engine gates, planned, fused into passes and batched like any other, and
  differentiable through both (a Pauli rotation's column twin is the rotation
  by -phi when P has an even number of Y factors, the same rotation when
  odd);
* a channel {K_i} on k qubits is its superoperator sum_i K_i (x) conj(K_i),
  one 2k-qubit engine gate on (idx, idx + n).  It is not unitary, so it
  starts a new segment (the adjoint sweep stays exact, see
  ``Circuit._apply_nonunitary``);
* tr(rho P) for a Pauli string reads only the 2^n entries
  rho[b ^ x, b] (x = the string's X/Y mask) with the phases
  (-i)^{#Y} (-1)^{popcount(b & z)}: one gather over precomputed indices.
"""

from typing import Any, Dict, List, Optional, Sequence, Tuple

import numpy as np
import torch

from . import channels as _channels
from . import engine as eng
from . import gates
from .circuit import C64, Circuit, _Op, _apply_local, _is_seq, _kraus_mats, _pauli_decompose, _to_np_matrix

Tensor = Any


def _column_twin(op: _Op, n: int) -> _Op:
    """The conj(G) half of a density-matrix gate, on the column qubits."""
    q2 = tuple(q + n for q in op.qubits)
    if op.kind == "const":
        return _Op("const", op.name + "*", q2, np.conj(op.data), op.diag, op.nq)
    if op.kind == "prot":
        ny = sum(1 for c in op.data[2] if c == 2)
        return _Op("prot", op.name, q2, op.data, False, op.nq, conj=(ny % 2 == 0))
    # parameterized families, user matrices, exponentials and selected gates:
    # the conjugate of the block their data builds
    return _Op(op.kind, op.name, q2, op.data, op.diag, op.nq, conj=True)


_TRACE_IDX: Dict[Any, Tuple[torch.Tensor, torch.Tensor]] = {}


def _trace_index(n: int, xm: int, zm: int, dev: torch.device) -> Tuple[torch.Tensor, torch.Tensor]:
    """Flat indices of rho[b ^ x, b] and the phases <b|P|b ^ x>."""
    key = (n, xm, zm, dev.index)
    r = _TRACE_IDX.get(key)
    if r is None:
        b = np.arange(1 << n, dtype=np.int64)
        flat = (b ^ xm) * (1 << n) + b
        par = np.bitwise_count((b & zm).astype(np.uint64)).astype(np.int64) & 1
        ny = bin(xm & zm).count("1")
        phase = ((-1j) ** ny) * (1.0 - 2.0 * par)
        r = (torch.as_tensor(flat, device=dev), torch.as_tensor(phase.astype(np.complex64), device=dev))
        if len(_TRACE_IDX) > 1024:
            _TRACE_IDX.clear()
        _TRACE_IDX[key] = r
    return r


class DMCircuit(Circuit):
    """Density-matrix circuit with the reference's ``DMCircuit2`` surface."""

    is_dm = True

    def __init__(self, nqubits: int, empty: bool = False, inputs: Optional[Tensor] = None,
                 mps_inputs: Optional[Any] = None, dminputs: Optional[Tensor] = None,
                 mpo_dminputs: Optional[Any] = None, split: Optional[Dict[str, Any]] = None) -> None:
        if mps_inputs is not None or mpo_dminputs is not None:
            raise NotImplementedError("MPS / MPO inputs are tensor-network objects")
        super().__init__(nqubits, split=split)
        self._nvec = 2 * nqubits
        self.inputs = inputs
        self.dminputs = dminputs
        self.mpo_dminputs = None
        self.circuit_param.update({"inputs": inputs, "dminputs": dminputs, "mpo_dminputs": None})
        self._rho0 = (inputs, dminputs) if (inputs is not None or dminputs is not None) else None

    # ------------------------------------------------------------ recording
    def _record(self, op: _Op, ir: Dict[str, Any]) -> None:
        super()._record(op, ir)
        self._ops.append(_column_twin(op, self._nqubits))

    def _engine_state(self) -> Tuple[torch.Tensor, torch.Tensor, torch.Tensor, eng.Run, int]:
        if self._rho0 is not None and self._seg_input is None:
            self._seg_input = self._rho0_vector()
        return super()._engine_state()

    def _rho0_vector(self) -> torch.Tensor:
        inputs, dminputs = self._rho0  # type: ignore
        dev = eng.device()
        N = 1 << self._nqubits

        def t(x: Any) -> torch.Tensor:
            if isinstance(x, gates.Gate):
                x = x.tensor
            if not isinstance(x, torch.Tensor):
                x = torch.as_tensor(np.asarray(x, dtype=np.complex64))
            return x.to(device=dev, dtype=C64)

        if dminputs is not None:
            d = t(dminputs)
            return d.reshape(-1) if d.numel() == N * N else d.reshape(d.shape[:-2] + (N * N,))
        psi = t(inputs)
        psi = psi.reshape(-1) if psi.numel() == N else psi
        return (psi.unsqueeze(-1) * torch.conj(psi).unsqueeze(-2)).reshape(psi.shape[:-1] + (N * N,))

    # ------------------------------------------------------------- channels
    def apply_general_kraus(self, kraus: Sequence[Any], *index: Any, **kws: Any) -> None:
        """rho -> sum_i K_i rho K_i^dag (densitymatrix.py:332-366).  The
        qubits come as ``*index`` or, as in ``DMCircuit_reference``, one
        list holding an index tuple."""
        if len(index) == 1 and _is_seq(index[0]):
            ids = {tuple(int(x) for x in (i if _is_seq(i) else (i,))) for i in index[0]}
            if len(ids) != 1:
                raise NotImplementedError("Kraus operators acting on different qubits")
            index = next(iter(ids))
        idx = self._norm_index(index)
        k = len(idx)
        mats, is_t = _kraus_mats(kraus, 1 << k)
        n = self._nqubits
        qubits = idx + tuple(q + n for q in idx)
        if is_t:
            dev = eng.device()
            ms = [m if isinstance(m, torch.Tensor) else torch.as_tensor(m.astype(np.complex64)) for m in mats]
            sup = sum(torch.kron(m.to(dev), torch.conj(m.to(dev))) for m in ms)
        else:
            sup = sum(np.kron(m, np.conj(m)) for m in mats)
        ir = {"gatef": "general_kraus", "index": tuple(index), "name": kws.get("name") or "general_kraus",
              "split": None, "mpo": False, "parameters": {}}
        self._apply_nonunitary(sup, qubits, ir)

    general_kraus = apply_general_kraus

    def unitary_kraus(self, kraus: Sequence[Any], *index: int, prob: Optional[Sequence[float]] = None,
                      status: Optional[Any] = None, name: Optional[str] = None) -> None:
        """The mixture sum_i p_i U_i rho U_i^dag of ``Circuit.unitary_kraus``
        applied exactly (no pick); without ``prob`` the operators carry
        their weights as in a Kraus list."""
        if prob is None:
            self.apply_general_kraus(kraus, *index, name=name)
            return
        d = 1 << len(index)
        mats, is_t = _kraus_mats(kraus, d)
        scaled = [m * (float(p) ** 0.5) if not isinstance(p, torch.Tensor) else m * torch.sqrt(p).to(C64)
                  for m, p in zip(mats, prob)]
        self.apply_general_kraus(scaled, *index, name=name)

    @staticmethod
    def apply_general_kraus_delayed(krausf: Any, is_unitary: bool = False) -> Any:
        """Channel method: the channel applied exactly (``status`` and
        ``name`` accepted and ignored, densitymatrix.py:369-380)."""

        def apply(self: "DMCircuit", *index: int, status: Optional[Any] = None, name: Optional[str] = None,
                  **vars: Any) -> None:
            self.apply_general_kraus(krausf(**vars), *index)

        return apply

    def mid_measurement(self, index: int, keep: int = 0) -> Tensor:
        """Post-selection P rho P with P = |keep><keep| (unnormalised)."""
        proj = np.diag([1.0, 0.0]) if keep < 0.5 else np.diag([0.0, 1.0])
        self.apply_general_kraus([proj], index)
        return torch.full((), int(keep >= 0.5), dtype=torch.int32, device=eng.device())

    mid_measure = mid_measurement
    post_select = mid_measurement
    post_selection = mid_measurement

    def cond_measurement(self, index: int, status: Optional[Any] = None) -> None:  # type: ignore[override]
        """Z measurement without recording the outcome: the dephasing
        channel on ``index`` (basecircuit.py:824-853, DM note)."""
        self.apply_general_kraus([np.diag([1.0, 0.0]), np.diag([0.0, 1.0])], index)

    cond_measure = cond_measurement

    # ------------------------------------------------------------ outputs
    def densitymatrix(self, check: bool = False, reuse: bool = True) -> Tensor:
        v = self._engine_state()[0]
        N = 1 << self._nqubits
        dm = v.reshape(v.shape[:-1] + (N, N))
        if check:
            tr = torch.diagonal(dm, dim1=-2, dim2=-1).sum(-1)
            assert bool(torch.all(torch.abs(tr - 1.0) < 1e-5)), "density matrix trace is not 1"
        return dm

    state = densitymatrix

    def wavefunction(self) -> Tensor:  # type: ignore[override]
        """The pure state behind rho (densitymatrix.py:240-256): the top
        eigenvector; every other eigenvalue must vanish."""
        e, v = torch.linalg.eigh(self.densitymatrix())
        assert bool(torch.all(torch.abs(e[..., :-1]) < 1e-5)), "the density matrix is not pure"
        return v[..., -1]

    def matrix(self) -> Tensor:
        raise NotImplementedError("a density-matrix circuit has no unitary")

    def _probability_vector(self) -> Tensor:
        v = self._engine_state()[0]
        N = 1 << self._nqubits
        diag = torch.arange(N, device=v.device) * (N + 1)
        return torch.real(v[..., diag])

    def probability(self) -> Tensor:
        return self._probability_vector()

    def amplitude(self, l: Any) -> Tensor:
        """rho[l, l] (the density-matrix reading of ``amplitude``)."""
        v = self._engine_state()[0]
        n = self._nqubits
        N = 1 << n
        if isinstance(l, str):
            if len(l) != n:
                raise ValueError("bitstring length %d != %d qubits" % (len(l), n))
            i = int(l, 2)
            return v[..., i * (N + 1)]
        lt = l if isinstance(l, torch.Tensor) else torch.as_tensor(np.asarray(l))
        w = (1 << torch.arange(n - 1, -1, -1, device=v.device))
        i = torch.sum(lt.to(device=v.device, dtype=torch.int64) * w, -1)
        return v[..., i * (N + 1)]

    def _trace_pauli(self, xm: int, zm: int) -> Tensor:
        v = self._engine_state()[0]
        flat, phase = _trace_index(self._nqubits, xm, zm, v.device)
        return torch.sum(v[..., flat] * phase, -1)

    def expectation_ps(self, x: Optional[Sequence[int]] = None, y: Optional[Sequence[int]] = None,
                       z: Optional[Sequence[int]] = None, ps: Optional[Sequence[int]] = None, reuse: bool = True,
                       noise_conf: Optional[Any] = None, nmc: int = 1000, status: Optional[Tensor] = None,
                       **kws: Any) -> Tensor:
        """tr(rho P) for a Pauli string (complex, like the reference)."""
        if noise_conf is not None:
            raise NotImplementedError("noise configurations are outside the engine")
        if ps is not None:
            from .quantum import ps2xyz

            d = ps2xyz(list(ps))
            x, y, z = d.get("x", None), d.get("y", None), d.get("z", None)
        xm, zm = self._pauli_term(x or [], y or [], z or [], self._nqubits)
        return self._trace_pauli(xm, zm)

    def expectation(self, *ops: Any, reuse: bool = True, noise_conf: Optional[Any] = None,
                    status: Optional[Tensor] = None, **kws: Any) -> Tensor:
        """tr(rho (x)_k O_k): Pauli products by the trace gather, other
        operators applied to the row qubits of vec(rho) by a forward sweep,
        then the trace."""
        if noise_conf is not None:
            raise NotImplementedError("noise configurations are outside the engine")
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
                    (xs if c == 1 else ys if c == 2 else zs if c == 3 else []).append(q)
            else:
                general.append((op, idx))
        if not general:
            return self._trace_pauli(*eng.pauli_masks(n, xs, ys, zs))
        v = self._engine_state()[0]
        c = Circuit(2 * n, inputs=v)
        for op, idx in general:
            c._apply_matrix(op, idx, {"gate": op, "index": idx, "name": "op"}, "op")
        for lst, name in ((xs, "x"), (ys, "y"), (zs, "z")):
            for q in lst:
                c._apply_const(name, [q])
        w = c.wavefunction()
        N = 1 << n
        diag = torch.arange(N, device=w.device) * (N + 1)
        return torch.sum(w[..., diag], -1)

    def sample(self, batch: Optional[int] = None, allow_state: bool = False,
               readout_error: Optional[Sequence[Any]] = None, format: Optional[str] = None,
               random_generator: Optional[Any] = None, status: Optional[Tensor] = None, **kws: Any) -> Any:
        """Samples from diag(rho), drawn by the engine's sampling kernel on
        the amplitudes sqrt(diag(rho))."""
        p = torch.clamp(self._probability_vector(), min=0.0)
        c = Circuit(self._nqubits, inputs=torch.sqrt(p).to(C64))
        return c.sample(batch=batch, allow_state=True, readout_error=readout_error, format=format,
                        random_generator=random_generator, status=status, **kws)

    def _measurement_copy(self) -> "DMCircuit":
        return DMCircuit(self._nqubits, dminputs=self.densitymatrix())

    def to_circuit(self, circuit_params: Optional[Dict[str, Any]] = None) -> Circuit:
        """The noiseless statevector circuit of the same gates (channels
        dropped, densitymatrix.py:311-325)."""
        return Circuit.from_qir(self.to_qir(), circuit_params or {"nqubits": self._nqubits})

    def get_dm_as_quoperator(self) -> Any:
        raise NotImplementedError("QuOperator views are tensor-network objects; use densitymatrix()")


for _c in _channels.channels:
    setattr(DMCircuit, _c, DMCircuit.apply_general_kraus_delayed(getattr(_channels, _c + "channel")))

DMCircuit2 = DMCircuit
DMCircuit_reference = DMCircuit
