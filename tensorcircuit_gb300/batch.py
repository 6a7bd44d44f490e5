"""Uneven batches: many parameterized circuits of different sizes and depths,
value and adjoint gradient of each circuit's energy in one engine call.

The reference evaluates such a set one circuit at a time
(``K.value_and_grad(f)`` per circuit, tensorcircuit/backends/pytorch_backend.py:
533-544; QAOA circuits from tensorcircuit/templates/blocks.py:84-110, MaxCut
energies from tensorcircuit/applications/graphdata.py:292-306).  Here the
circuits are recorded once with symbolic parameters, planned once, and every
call runs one persistent kernel launch per sweep over all of them
(``tcg_ubatch_value_and_grad`` in include/tcgb300.h), optionally replayed
from a captured CUDA graph.  The tile width of the launch (the fusion knob of
the tile passes) is chosen by timing the candidates once per batch shape.

Parameterized gates must be Pauli rotations (rx/ry/rz/rxx/ryy/rzz, exp1 of a
Pauli string) whose angle is ``params[k]`` times a constant; other gates must
be constant.
"""

import threading
from typing import Any, Callable, Dict, List, Optional, Sequence, Tuple

import numpy as np
import torch

from . import _native as nat
from . import engine as eng
from . import gates
from .circuit import Circuit

Terms = Sequence[Tuple[float, Dict[str, Sequence[int]]]]


class ParamRef:
    """Symbolic ``scale * params[k]`` used while recording a batch circuit."""

    __slots__ = ("k", "scale")

    def __init__(self, k: int, scale: float = 1.0) -> None:
        self.k = int(k)
        self.scale = float(scale)

    def __mul__(self, a: Any) -> "ParamRef":
        return ParamRef(self.k, self.scale * float(a))

    __rmul__ = __mul__

    def __truediv__(self, a: Any) -> "ParamRef":
        return ParamRef(self.k, self.scale / float(a))

    def __neg__(self) -> "ParamRef":
        return ParamRef(self.k, -self.scale)

    def __repr__(self) -> str:
        return "ParamRef(%d, %g)" % (self.k, self.scale)


class ParamVector:
    """Stand-in for a circuit's parameter vector while it is recorded."""

    def __init__(self, size: int) -> None:
        self.size = int(size)

    def __len__(self) -> int:
        return self.size

    def __getitem__(self, k: int) -> ParamRef:
        k = int(k)
        if k < 0:
            k += self.size
        if not 0 <= k < self.size:
            raise IndexError(k)
        return ParamRef(k)


class BatchCircuit:
    """Host description of one recorded circuit (matrix layout, gates, terms)."""

    def __init__(self, n: int, build: Callable[[Circuit, ParamVector], Any], nparams: int, terms: Terms,
                 offset: float = 0.0) -> None:
        c = Circuit(n)
        build(c, ParamVector(nparams))
        self.n = n
        self.nparams = int(nparams)
        self.ngates_src = len(c._ops)
        gl: List[Tuple[int, Tuple[int, ...], int, int, Tuple[int, ...]]] = []
        const: List[complex] = []
        param: List[int] = []
        scale: List[float] = []
        for op in c._ops:
            off = len(const)
            if op.kind == "const":
                m = np.asarray(op.data, dtype=np.complex128)
                e = np.diag(m) if op.diag else m.reshape(-1)
                const.extend(e.tolist())
                param.extend([-1] * e.size)
                scale.extend([0.0] * e.size)
                gl.append((nat.TCG_GATE_DIAG if op.diag else nat.TCG_GATE_DENSE, op.qubits, off, -1, ()))
            elif op.kind == "prot":
                theta, sc, codes = op.data
                if isinstance(theta, ParamRef):
                    const.append(0j)
                    param.append(theta.k)
                    scale.append(sc * theta.scale)
                    gl.append((nat.TCG_GATE_PAULI_ROT, op.qubits, off, off, codes))
                else:
                    t = theta.item() if isinstance(theta, torch.Tensor) else float(theta)
                    const.append(complex(np.exp(1j * sc * t)))
                    param.append(-1)
                    scale.append(0.0)
                    gl.append((nat.TCG_GATE_PAULI_ROT, op.qubits, off, -1, codes))
            else:
                raise NotImplementedError(
                    "uneven batches take constant gates and Pauli rotations of one parameter; got %s" % op.name)
        if not const:
            const, param, scale = [0j], [-1], [0.0]
        self.gates = gl
        self.mat_const = np.asarray(const, dtype=np.complex64)
        self.mat_param = np.asarray(param, dtype=np.int64)
        self.mat_scale = np.asarray(scale, dtype=np.float32)
        self.terms = [(float(cf), eng.pauli_masks(n, t.get("x", []), t.get("y", []), t.get("z", [])))
                      for cf, t in terms]
        self.offset = float(offset)


_TUNED: Dict[Any, Tuple[int, int]] = {}
_TUNED_LOCK = threading.Lock()

# Candidate tile widths (local index bits per tile: also how many qubits one
# HBM pass can fuse) and Z-rotation fusion widths (commuting Z-string
# rotations applied as one phase op; 1 = each on its own, 0 = the default 32).
TILE_WIDTHS = (12, 11, 10, 9)
ZRUN_WIDTHS = (0, 16, 8, 1)


def coordinate_search(tile_widths: Sequence[int], zrun_widths: Sequence[int],
                      timed: Callable[[int, int], float]) -> Tuple[int, int]:
    """The autotuner's search: ``timed(L, z)`` for every tile width at the
    first fusion width, then for the other fusion widths at the fastest tile
    width; returns the fastest ``(L, z)`` (the first one on ties)."""
    z0 = zrun_widths[0]
    best, best_t = (tile_widths[0], z0), float("inf")
    for L in tile_widths:
        t = timed(L, z0)
        if t < best_t:
            best, best_t = (L, z0), t
    for z in zrun_widths[1:]:
        t = timed(best[0], z)
        if t < best_t:
            best, best_t = (best[0], z), t
    return best


def _has_zruns(circs: Sequence["BatchCircuit"]) -> bool:
    """True if some circuit holds two or more Z-string rotations (the only
    gates the Z-rotation fusion width changes)."""
    for bc in circs:
        nz = sum(1 for kind, _q, _mo, _go, codes in bc.gates
                 if kind == nat.TCG_GATE_PAULI_ROT and all(c == 3 for c in codes))
        if nz >= 2:
            return True
    return False


class _Handle:
    """tcg_ubatch handle with its scratch, for one tile width and one
    Z-rotation fusion width (0 = the planner's default)."""

    def __init__(self, circs: Sequence[BatchCircuit], tile_bits: int, device: torch.device,
                 zrun_max: int = 0) -> None:
        lib = nat.load()
        keep: List[Any] = []
        arr = (nat.TcgUbatchCircuit * len(circs))()
        for i, bc in enumerate(circs):
            g = (nat.TcgGate * max(len(bc.gates), 1))()
            for j, (kind, qubits, mo, go, codes) in enumerate(bc.gates):
                g[j].kind = kind
                g[j].nq = len(qubits)
                for a, q in enumerate(qubits):
                    g[j].qubits[a] = q
                for a, cd in enumerate(codes):
                    g[j].pauli[a] = cd
                g[j].mat_off = mo
                g[j].grad_off = go
            mc = np.ascontiguousarray(bc.mat_const.view(np.float32))
            mp = np.ascontiguousarray(bc.mat_param)
            ms = np.ascontiguousarray(bc.mat_scale)
            t = (nat.TcgPauli * max(len(bc.terms), 1))()
            cf = np.zeros(max(len(bc.terms), 1), dtype=np.float32)
            for j, (c0, (xm, zm)) in enumerate(bc.terms):
                t[j].xmask = xm
                t[j].zmask = zm
                cf[j] = c0
            keep.extend([g, mc, mp, ms, t, cf])
            a = arr[i]
            a.nqubits = bc.n
            a.ngates = len(bc.gates)
            a.gates = g
            a.nmat = bc.mat_const.size
            a.mat_const = mc.ctypes.data_as(nat.ctypes.POINTER(nat.ctypes.c_float))
            a.mat_param = mp.ctypes.data_as(nat.ctypes.POINTER(nat.ctypes.c_int64))
            a.mat_scale = ms.ctypes.data_as(nat.ctypes.POINTER(nat.ctypes.c_float))
            a.nparams = bc.nparams
            a.nterms = len(bc.terms)
            a.terms = t
            a.coef = cf.ctypes.data_as(nat.ctypes.POINTER(nat.ctypes.c_float))
            a.offset = bc.offset
        h = nat.ctypes.c_void_p()
        opts = nat.TcgPlanOpts(tile_bits=tile_bits, max_stage_grad_entries=0, zrun_max=zrun_max)
        with torch.cuda.device(device):
            nat.check(lib.tcg_ubatch_create_ex(arr, len(circs), nat.ctypes.byref(opts), nat.ctypes.byref(h)),
                      "uneven batch")
        self.handle = h
        self.tile_bits = tile_bits
        self.zrun_max = zrun_max
        npar = nat.ctypes.c_int64(0)
        nst = nat.ctypes.c_int64(0)
        nbytes = nat.ctypes.c_size_t(0)
        nat.check(lib.tcg_ubatch_info(h, nat.ctypes.byref(npar), nat.ctypes.byref(nst), nat.ctypes.byref(nbytes)))
        self.nparams = npar.value
        self.state_entries = nst.value
        # zero-filled once: the sticky time-out flag inside must start clear
        self.scratch = torch.zeros(max(nbytes.value, 1), dtype=torch.uint8, device=device)

    def run(self, params: torch.Tensor, energies: torch.Tensor, grads: Optional[torch.Tensor]) -> None:
        lib = nat.load()
        st = torch.cuda.current_stream(params.device).cuda_stream
        nat.check(lib.tcg_ubatch_value_and_grad(self.handle, nat.ptr(params), nat.ptr(energies),
                                                nat.ptr(grads) if grads is not None else None,
                                                nat.ptr(self.scratch), self.scratch.numel(), st),
                  "uneven batch")

    def check(self) -> None:
        lib = nat.load()
        st = torch.cuda.current_stream(self.scratch.device).cuda_stream
        nat.check(lib.tcg_ubatch_check(self.handle, nat.ptr(self.scratch), st), "uneven batch")

    def state(self, c: int, n: int) -> torch.Tensor:
        off = nat.load().tcg_ubatch_state_offset(self.handle, c)
        return self.scratch.view(torch.complex64)[off:off + (1 << n)]

    def __del__(self) -> None:
        try:
            nat.load(build_if_missing=False).tcg_ubatch_destroy(self.handle)
        except Exception:
            pass


class UnevenBatch:
    """Value and adjoint gradient of ``offset_c + sum_t coef_t <P_t>`` for
    many circuits at once.

    ``specs``: one ``(n, build, nparams, terms[, offset])`` per circuit, where
    ``build(c, params)`` applies the circuit's gates to ``c`` using
    ``params[k]`` as angles and ``terms`` is a list of
    ``(coef, {"x": [...], "y": [...], "z": [...]})``.

    ``value_and_grad(params)`` takes the concatenation of all circuits'
    parameter vectors (float32, length ``nparams_total``) and returns
    ``(energies[C], grads[nparams_total])``.  With ``graph=True`` the call is
    captured into a CUDA graph after one eager call and replayed.
    ``tile_bits=None`` leaves the tile width, and unless ``zrun_max`` is
    given the Z-rotation fusion width too, to the autotuner: it times every
    admissible tile width at the default fusion width, then the other fusion
    widths at the fastest tile width, and keeps the fastest pair (cached per
    batch shape for the process; ``tune_log`` lists
    ``(tile_bits, zrun_max, ms)``).  A given ``tile_bits`` is used as is,
    with ``zrun_max`` or the default fusion width (0 = runs of up to 32).
    """

    def __init__(self, specs: Sequence[Sequence[Any]], tile_bits: Optional[int] = None, graph: bool = True,
                 device: Optional[torch.device] = None, wait_limit_ns: Optional[int] = None,
                 zrun_max: Optional[int] = None) -> None:
        if zrun_max is not None and not 0 <= int(zrun_max) <= 32:
            raise ValueError("zrun_max must be in 0..32 (0 = default), got %r" % (zrun_max,))
        self.circuits = [BatchCircuit(*s) for s in specs]
        nmin = min(bc.n for bc in self.circuits)
        if tile_bits is not None and tile_bits > nmin:
            raise ValueError("tile_bits %d exceeds the smallest circuit (%d qubits)" % (tile_bits, nmin))
        self.device = device or eng.device()
        self.nparams = sum(bc.nparams for bc in self.circuits)
        self.offsets = np.cumsum([0] + [bc.nparams for bc in self.circuits])
        self.graph_enabled = graph
        self._graph: Optional[torch.cuda.CUDAGraph] = None
        if tile_bits is None:
            key = (tuple((bc.n, len(bc.gates), bc.nparams, len(bc.terms)) for bc in self.circuits), zrun_max)
            with _TUNED_LOCK:
                tuned = _TUNED.get(key)
            if tuned is None:
                Ls = [L for L in TILE_WIDTHS if L <= nmin] or [nmin]
                if zrun_max is not None:
                    Zs = [int(zrun_max)]
                else:
                    Zs = list(ZRUN_WIDTHS) if _has_zruns(self.circuits) else [0]
                tuned = self._autotune(Ls, Zs)
                with _TUNED_LOCK:
                    _TUNED[key] = tuned
            tile_bits, zrun_max = tuned
            self.tuned = True
        else:
            zrun_max = 0 if zrun_max is None else int(zrun_max)
            self.tuned = False
        self.h = _Handle(self.circuits, tile_bits, self.device, int(zrun_max))
        self.zrun_max = int(zrun_max)
        if wait_limit_ns is not None:
            # limit of one device-side dependency wait (default 2 s)
            nat.check(nat.load().tcg_ubatch_set_wait_limit(self.h.handle, int(wait_limit_ns)), "wait limit")
        self.tile_bits = tile_bits
        self._p = torch.zeros(max(self.nparams, 1), dtype=torch.float32, device=self.device)
        self._e = torch.zeros(len(self.circuits), dtype=torch.float32, device=self.device)
        self._g = torch.zeros(max(self.nparams, 1), dtype=torch.float32, device=self.device)

    def _autotune(self, tile_widths: Sequence[int], zrun_widths: Sequence[int]) -> Tuple[int, int]:
        """Coordinate search: every tile width at the first fusion width, then
        the other fusion widths at the fastest tile width.  Each candidate is
        one warm call and the mean of two timed calls (CUDA events)."""
        p = torch.rand(max(self.nparams, 1), device=self.device)
        e = torch.zeros(len(self.circuits), device=self.device)
        g = torch.zeros(max(self.nparams, 1), device=self.device)
        self.tune_log: List[Tuple[int, int, float]] = []

        def timed(L: int, z: int) -> float:
            h = _Handle(self.circuits, L, self.device, z)
            h.run(p, e, g)
            torch.cuda.synchronize(self.device)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(2):
                h.run(p, e, g)
            e1.record()
            torch.cuda.synchronize(self.device)
            h.check()
            t = e0.elapsed_time(e1) / 2
            self.tune_log.append((L, z, t))
            del h
            return t

        return coordinate_search(tile_widths, zrun_widths, timed)

    def split(self, flat: torch.Tensor) -> List[torch.Tensor]:
        return [flat[self.offsets[i]:self.offsets[i + 1]] for i in range(len(self.circuits))]

    def value_and_grad(self, params: Any, grad: bool = True) -> Tuple[torch.Tensor, Optional[torch.Tensor]]:
        if isinstance(params, (list, tuple)):
            params = torch.cat([torch.as_tensor(x, dtype=torch.float32).reshape(-1).to(self.device) for x in params])
        params = torch.as_tensor(params, dtype=torch.float32, device=self.device).reshape(-1)
        if params.numel() != self.nparams:
            raise ValueError("expected %d parameters, got %d" % (self.nparams, params.numel()))
        if not grad or not self.graph_enabled:
            e = torch.empty(len(self.circuits), dtype=torch.float32, device=self.device)
            g = torch.empty(max(self.nparams, 1), dtype=torch.float32, device=self.device) if grad else None
            self.h.run(params.contiguous(), e, g)
            return e, (g[:self.nparams] if grad else None)
        self._p[:self.nparams].copy_(params)
        if self._graph is None:
            self.h.run(self._p, self._e, self._g)  # eager call: sets kernel attributes before capture
            s = torch.cuda.Stream(self.device)
            s.wait_stream(torch.cuda.current_stream(self.device))
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, stream=s):
                self.h.run(self._p, self._e, self._g)
            torch.cuda.current_stream(self.device).wait_stream(s)
            self._graph = g
        self._graph.replay()
        return self._e.clone(), self._g[:self.nparams].clone()

    def check(self) -> None:
        """Raise if a bounded dependency wait of an earlier call timed out."""
        self.h.check()

    def stats(self) -> Dict[str, Any]:
        """Tiles and algorithmic HBM bytes per sweep of one call."""
        tiles = (nat.ctypes.c_int64 * 4)()
        by = (nat.ctypes.c_double * 4)()
        nat.check(nat.load().tcg_ubatch_stats(self.h.handle, tiles, by))
        names = ("forward", "adjoint", "measure", "accumulate")
        return {nm: {"tiles": int(tiles[i]), "alg_bytes": float(by[i])} for i, nm in enumerate(names)}

    def state(self, c: int) -> torch.Tensor:
        """Final state of circuit c after a ``grad=False`` call."""
        return self.h.state(c, self.circuits[c].n).clone()


def qaoa_spec(n: int, edges: Sequence[Tuple[int, int]], p: int) -> Tuple[int, Callable[..., Any], int, Terms, float]:
    """MaxCut QAOA at depth p with the reference's conventions
    (templates/blocks.py:84-110: H on all qubits, then per layer exp1(ZZ,
    gamma) on every edge and rx(beta) on every node; params = [gammas,
    betas]) and energy sum_(ij) (1 - Z_i Z_j) / 2."""

    def build(c: Circuit, params: Any) -> None:
        for i in range(n):
            c.h(i)
        for layer in range(p):
            for a, b in edges:
                c.exp1(a, b, unitary=gates._zz_matrix, theta=params[layer])
            for i in range(n):
                c.rx(i, theta=params[p + layer])

    terms = [(-0.5, {"z": [a, b]}) for a, b in edges]
    return n, build, 2 * p, terms, 0.5 * len(edges)
