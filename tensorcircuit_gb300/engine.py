"""Bridge between the Circuit API and the native engine.

* :class:`GatePlan` wraps a native ``tcg_plan`` for one circuit *structure*
  (gate kinds and qubits); plans are cached, so a VQE loop that rebuilds the
  same circuit every step plans once.
* :class:`StateFn` runs the forward sweep (``tcg_forward``) and is
  differentiable: its backward is the adjoint sweep (``tcg_backward``), which
  returns the cotangent of every gate-matrix entry and of the input state.
* :class:`ExpectFn` evaluates Pauli strings (``tcg_expect_pauli``).  Its
  backward does not materialise ``P psi``; it records ``(P, g)`` in the
  circuit's :class:`Run` and passes a zero to the state's ``anchor`` output, so
  the state node's backward -- which autograd runs once, after every
  expectation node -- seeds the adjoint sweep with
  ``mu = grad_psi + sum_t 2 Re(g_t) P_t psi`` in one fused kernel
  (``tcg_pauli_accumulate``).  This is the adjoint method: O(1) extra states
  instead of the taped tensordots the reference's torch AD keeps
  (tensorcircuit/backends/pytorch_backend.py:533-544, 673-709).

All four Functions carry ``vmap`` rules, so ``torch.func.vmap`` /
``torch.func.grad_and_value`` -- what the reference's pytorch backend uses for
``vvag`` -- batch whole circuits into single kernel launches.
"""

import threading
from collections import OrderedDict
from typing import Any, Dict, List, Optional, Sequence, Tuple

import numpy as np
import torch

from . import _native as nat

C64 = torch.complex64


def device() -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError(
            "tensorcircuit_gb300 runs on a CUDA GPU only (no CPU fallback); "
            "torch.cuda.is_available() is False"
        )
    return torch.device("cuda", torch.cuda.current_device())


def _stream() -> int:
    return int(torch.cuda.current_stream().cuda_stream)


# ----------------------------------------------------------------------------
# native plans
# ----------------------------------------------------------------------------
class GatePlan:
    """A native gate plan plus its matrix-buffer layout."""

    def __init__(self, n: int, gates: Sequence[Tuple[Any, ...]], nmat: int) -> None:
        """gates: (kind, qubits, mat_off, grad_off[, pauli codes]) tuples."""
        lib = nat.load()
        arr = (nat.TcgGate * max(len(gates), 1))()
        for i, g in enumerate(gates):
            kind, qubits, mat_off, grad_off = g[:4]
            arr[i].kind = kind
            arr[i].nq = len(qubits)
            for j, q in enumerate(qubits):
                arr[i].qubits[j] = q
            if len(g) > 4:
                for j, c in enumerate(g[4]):
                    arr[i].pauli[j] = c
            arr[i].mat_off = mat_off
            arr[i].grad_off = grad_off
        h = nat.ctypes.c_void_p()
        nat.check(lib.tcg_plan_create(n, arr, len(gates), None, nat.ctypes.byref(h)), "plan")
        self.handle = h
        self.n = n
        self.ngates = len(gates)
        self.nmat = nmat
        st = nat.TcgPlanStats()
        nat.check(lib.tcg_plan_get_stats(h, nat.ctypes.byref(st)))
        self.npasses = st.npasses
        self.nstages = st.nstages
        self.tile_bits = st.tile_bits
        # matrix-buffer entries of Pauli rotations: the engine writes dL/dphi
        # there, which the autograd glue turns into the e^{i phi} cotangent
        self.prot_offs = [g[3] for g in gates if g[0] == nat.TCG_GATE_PAULI_ROT and g[3] >= 0]
        self._prot_mask: Dict[Any, torch.Tensor] = {}

    def tensor_passes(self) -> int:
        """Forward passes that run as fused blocks on the tensor cores under
        the current policy (``TCG_TC`` / ``tcg_set_tensor_policy``)."""
        return int(nat.load().tcg_plan_tensor_passes(self.handle))

    def check(self, stream: Optional[int] = None) -> None:
        """Synchronise and raise if a bounded device-side wait of a
        tensor-core pass ran out of time (its results are then invalid)."""
        st = torch.cuda.current_stream().cuda_stream if stream is None else stream
        nat.check(nat.load().tcg_plan_check(self.handle, st), "tensor-core pass")

    def prot_mask(self, device: torch.device) -> Optional[torch.Tensor]:
        if not self.prot_offs:
            return None
        m = self._prot_mask.get(device)
        if m is None:
            h = torch.zeros(self.nmat, dtype=torch.bool)
            h[self.prot_offs] = True
            m = h.to(device)
            self._prot_mask[device] = m
        return m

    def __del__(self) -> None:
        try:
            nat.load(build_if_missing=False).tcg_plan_destroy(self.handle)
        except Exception:  # interpreter shutdown
            pass


class TermPlan:
    """A native measurement plan for a tuple of Pauli strings."""

    def __init__(self, n: int, terms: Sequence[Tuple[int, int]]) -> None:
        lib = nat.load()
        arr = (nat.TcgPauli * max(len(terms), 1))()
        for i, (x, z) in enumerate(terms):
            arr[i].xmask = x
            arr[i].zmask = z
        h = nat.ctypes.c_void_p()
        nat.check(lib.tcg_mplan_create(n, arr, len(terms), nat.ctypes.byref(h)), "measurement plan")
        self.handle = h
        self.n = n
        self.nterms = len(terms)
        self.npasses = lib.tcg_mplan_passes(h)

    def __del__(self) -> None:
        try:
            nat.load(build_if_missing=False).tcg_mplan_destroy(self.handle)
        except Exception:
            pass


class _LRU:
    def __init__(self, cap: int) -> None:
        self.cap = cap
        self.d: "OrderedDict[Any, Any]" = OrderedDict()
        self.lock = threading.Lock()

    def get(self, key: Any, make: Any) -> Any:
        with self.lock:
            v = self.d.get(key)
            if v is not None:
                self.d.move_to_end(key)
                return v
        v = make()
        with self.lock:
            self.d[key] = v
            while len(self.d) > self.cap:
                self.d.popitem(last=False)
        return v


_gate_plans = _LRU(256)
_term_plans = _LRU(1024)


def gate_plan(key: Any, n: int, gates: Sequence[Tuple[int, Tuple[int, ...], int, int]], nmat: int) -> GatePlan:
    return _gate_plans.get(key, lambda: GatePlan(n, gates, nmat))


def term_plan(n: int, terms: Tuple[Tuple[int, int], ...]) -> TermPlan:
    return _term_plans.get((n, terms), lambda: TermPlan(n, terms))


def pauli_masks(n: int, x: Sequence[int], y: Sequence[int], z: Sequence[int]) -> Tuple[int, int]:
    """Qubit lists -> (xmask, zmask) over amplitude-index bits (qubit q is bit n-1-q)."""
    xm = zm = 0
    for q in x:
        xm |= 1 << (n - 1 - q)
    for q in y:
        xm |= 1 << (n - 1 - q)
        zm |= 1 << (n - 1 - q)
    for q in z:
        zm |= 1 << (n - 1 - q)
    return xm, zm


# ----------------------------------------------------------------------------
# run context: one per evaluated circuit
# ----------------------------------------------------------------------------
class Run:
    """Per-circuit context shared by the state node and its observables."""

    def __init__(self, plan: GatePlan, n: int) -> None:
        self.plan = plan
        self.n = n
        self.records: List[Tuple[Tuple[Tuple[int, int], ...], torch.Tensor]] = []

    def record(self, terms: Tuple[Tuple[int, int], ...], g: torch.Tensor) -> None:
        self.records.append((terms, g))

    def take(self) -> List[Tuple[Tuple[Tuple[int, int], ...], torch.Tensor]]:
        r, self.records = self.records, []
        return r


def _lead(*shapes: Tuple[int, ...]) -> Tuple[int, ...]:
    return tuple(torch.broadcast_shapes(*shapes))


def _flat(t: torch.Tensor, lead: Tuple[int, ...], tail: int) -> torch.Tensor:
    # conjugate / negative views (autograd produces them, e.g. the backward
    # of conj) become physical here, before a raw pointer is taken
    return t.resolve_conj().resolve_neg().expand(lead + (tail,)).reshape(-1, tail)


def _input_rows(psi0: torch.Tensor, lead: Tuple[int, ...], tail: int) -> Tuple[torch.Tensor, int]:
    """Input states as (rows, row stride in complex entries): one row with
    stride 0 when every circuit starts from the same state, else one row per
    circuit."""
    x = psi0.resolve_conj().resolve_neg()
    if x.dtype != C64:
        x = x.to(C64)
    if x.numel() == tail:
        return x.reshape(tail).contiguous(), 0
    return _flat(x, lead, tail).contiguous(), tail


def _bd(x: Optional[torch.Tensor], d: Optional[int]) -> Optional[torch.Tensor]:
    if x is None or d is None:
        return x
    return x.movedim(d, 0)


# ----------------------------------------------------------------------------
# autograd Functions
# ----------------------------------------------------------------------------
class StateFn(torch.autograd.Function):
    """(gate matrices, input state) -> (output state, anchor)."""

    @staticmethod
    def forward(mats: torch.Tensor, psi0: torch.Tensor, run: Run) -> Tuple[torch.Tensor, torch.Tensor]:
        lib = nat.load()
        N = 1 << run.n
        M = mats.shape[-1]
        lead = _lead(mats.shape[:-1], psi0.shape[:-1])
        B = int(np.prod(lead)) if lead else 1
        m = _flat(mats, lead, M).contiguous()
        if run.plan.ngates > 0 and B > 0:
            # the first pass reads the input rows where they are (one shared
            # row for a broadcast input such as |0...0>): no copy of the input
            # into the output buffer first
            src, stride = _input_rows(psi0, lead, N)
            psi = torch.empty((B, N), dtype=C64, device=src.device)
            nat.check(lib.tcg_forward_from(run.plan.handle, nat.ptr(src), stride, nat.ptr(psi), B, nat.ptr(m), M,
                                           _stream()), "forward")
        else:
            psi = _flat(psi0, lead, N).contiguous().clone()
        anchor = torch.zeros(lead, dtype=torch.float32, device=psi.device)
        return psi.reshape(lead + (N,)), anchor

    @staticmethod
    def setup_context(ctx: Any, inputs: Tuple[Any, ...], output: Tuple[Any, ...]) -> None:
        mats, psi0, run = inputs
        psi, _ = output
        ctx.save_for_backward(mats, psi)
        ctx.run = run
        ctx.mats_shape = mats.shape
        ctx.psi0_shape = psi0.shape
        ctx.set_materialize_grads(False)

    @staticmethod
    def backward(ctx: Any, gpsi: Optional[torch.Tensor], ganchor: Optional[torch.Tensor]) -> Tuple[Any, ...]:
        mats, psi = ctx.saved_tensors
        recs = ctx.run.take()
        terms: List[Tuple[int, int]] = []
        gs: List[torch.Tensor] = []
        for t, g in recs:
            terms.extend(t)
            gs.append(g)
        gcoef = torch.cat(gs, -1) if gs else None
        spec = tuple(terms)
        gm, gp0 = AdjointFn.apply(mats, psi, gpsi, gcoef, ctx.run, spec)
        gm = gm.sum_to_size(ctx.mats_shape) if gm.shape != ctx.mats_shape else gm
        pm = ctx.run.plan.prot_mask(gm.device)
        if pm is not None:
            # Pauli rotation entries hold z = e^{i phi} and the sweep returned
            # g = dL/dphi; the cotangent with Re(conj(c) dz/dphi) = g is c = i z g
            gm = torch.where(pm, 1j * mats * gm.real, gm)
        gp0 = gp0.sum_to_size(ctx.psi0_shape) if gp0.shape != ctx.psi0_shape else gp0
        return gm, gp0, None

    @staticmethod
    def vmap(info: Any, in_dims: Tuple[Any, ...], mats: torch.Tensor, psi0: torch.Tensor, run: Run) -> Any:
        md, pd, _ = in_dims
        mats = mats.movedim(md, 0) if md is not None else mats.unsqueeze(0)
        psi0 = psi0.movedim(pd, 0) if pd is not None else psi0.unsqueeze(0)
        out = StateFn.apply(mats, psi0, run)
        return out, (0, 0)


class AdjointFn(torch.autograd.Function):
    """Adjoint sweep: (mats, psi_out, grad_psi, expectation cotangents) ->
    (grad_mats, grad_psi_in)."""

    @staticmethod
    def forward(mats: torch.Tensor, psi: torch.Tensor, gpsi: Optional[torch.Tensor],
                gcoef: Optional[torch.Tensor], run: Run, spec: Tuple[Tuple[int, int], ...]) -> Tuple[torch.Tensor, torch.Tensor]:
        lib = nat.load()
        N = 1 << run.n
        M = mats.shape[-1]
        shapes = [mats.shape[:-1], psi.shape[:-1]]
        if gpsi is not None:
            shapes.append(gpsi.shape[:-1])
        if gcoef is not None:
            shapes.append(gcoef.shape[:-1])
        lead = _lead(*shapes)
        # the output states are only read (by the accumulation and the first
        # adjoint pass, which writes the working copy psi_w): no clone
        psi_out = _flat(psi, lead, N).contiguous()
        B = psi_out.shape[0]
        st = _stream()
        accumulate = gcoef is not None and len(spec) > 0
        if gpsi is not None:
            mu = _flat(gpsi.to(C64), lead, N).contiguous().clone()
        elif accumulate:
            mu = torch.empty_like(psi_out)  # the accumulation writes every entry
        else:
            mu = torch.zeros_like(psi_out)
        if accumulate:
            tp = term_plan(run.n, spec)
            coef = _flat((2.0 * gcoef.real).to(torch.float32), lead, len(spec)).contiguous()
            flags = 0 if gpsi is not None else nat.TCG_ACC_OVERWRITE
            nat.check(lib.tcg_pauli_accumulate_ex(tp.handle, nat.ptr(psi_out), nat.ptr(mu), B, nat.ptr(coef),
                                                  len(spec), flags, st), "pauli accumulate")
        m = _flat(mats, lead, M).contiguous()
        grads = torch.zeros_like(m)
        if run.plan.ngates > 0 and B > 0:
            nbytes = int(lib.tcg_backward_scratch_bytes(run.plan.handle, B))
            scratch = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=psi_out.device)
            psi_w = torch.empty_like(psi_out)
            nat.check(lib.tcg_backward_from(run.plan.handle, nat.ptr(psi_out), nat.ptr(psi_w), nat.ptr(mu), B,
                                            nat.ptr(m), M, nat.ptr(grads), M, nat.ptr(scratch), nbytes, st),
                      "backward")
        return grads.reshape(lead + (M,)), mu.reshape(lead + (N,))

    @staticmethod
    def setup_context(ctx: Any, inputs: Tuple[Any, ...], output: Any) -> None:
        pass

    @staticmethod
    def backward(ctx: Any, *grads: Any) -> Any:
        raise NotImplementedError("second derivatives through the adjoint sweep are not supported")

    @staticmethod
    def vmap(info: Any, in_dims: Tuple[Any, ...], mats: torch.Tensor, psi: torch.Tensor,
             gpsi: Optional[torch.Tensor], gcoef: Optional[torch.Tensor], run: Run, spec: Any) -> Any:
        md, pd, gd, cd, _, _ = in_dims

        def mv(x: Optional[torch.Tensor], d: Optional[int]) -> Optional[torch.Tensor]:
            if x is None:
                return None
            return x.movedim(d, 0) if d is not None else x.unsqueeze(0)

        out = AdjointFn.apply(mv(mats, md), mv(psi, pd), mv(gpsi, gd), mv(gcoef, cd), run, spec)
        return out, (0, 0)


class ExpectFn(torch.autograd.Function):
    """(state, anchor) -> <psi|P_t|psi> for the Pauli strings in ``spec``."""

    @staticmethod
    def forward(psi: torch.Tensor, anchor: torch.Tensor, spec: Tuple[Tuple[int, int], ...], run: Run) -> torch.Tensor:
        lib = nat.load()
        N = 1 << run.n
        lead = _lead(psi.shape[:-1], anchor.shape)
        p = _flat(psi, lead, N).contiguous()
        B = p.shape[0]
        T = len(spec)
        tp = term_plan(run.n, spec)
        out = torch.empty((B, T, 2), dtype=torch.float64, device=p.device)
        nbytes = int(lib.tcg_expect_scratch_bytes(tp.handle, B))
        scratch = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=p.device)
        nat.check(lib.tcg_expect_pauli(tp.handle, nat.ptr(p), B, nat.ptr(out), nat.ptr(scratch), nbytes,
                                       _stream()), "expectation")
        val = torch.view_as_complex(out).to(C64)
        return val.reshape(lead + (T,))

    @staticmethod
    def setup_context(ctx: Any, inputs: Tuple[Any, ...], output: Any) -> None:
        psi, anchor, spec, run = inputs
        ctx.spec = spec
        ctx.run = run
        ctx.anchor_shape = anchor.shape

    @staticmethod
    def backward(ctx: Any, g: torch.Tensor) -> Any:
        ctx.run.record(ctx.spec, g)
        z = torch.zeros(g.shape[:-1], dtype=torch.float32, device=g.device)
        z = z.sum_to_size(ctx.anchor_shape) if z.shape != ctx.anchor_shape else z
        return None, z, None, None

    @staticmethod
    def vmap(info: Any, in_dims: Tuple[Any, ...], psi: torch.Tensor, anchor: torch.Tensor, spec: Any, run: Run) -> Any:
        pd, ad, _, _ = in_dims
        psi = psi.movedim(pd, 0) if pd is not None else psi.unsqueeze(0)
        anchor = anchor.movedim(ad, 0) if ad is not None else anchor.unsqueeze(0)
        return ExpectFn.apply(psi, anchor, spec, run), 0


class KrausPickFn(torch.autograd.Function):
    """Monte-Carlo branch choice of a general channel (``tcg_kraus_pick``):
    (Pauli expectations ev [..., S] complex64, constant expansion coef
    [K, S] fp32, uniforms x) -> (pick int32 [...], rescale 1 / (sqrt(p_pick)
    + 1e-10) complex64 [...], p fp32 [..., K]).  Only the rescale carries a
    gradient (to Re ev); the pick and p are constants of the trajectory."""

    @staticmethod
    def forward(ev: torch.Tensor, coef: torch.Tensor, x: torch.Tensor) -> Tuple[torch.Tensor, torch.Tensor,
                                                                                  torch.Tensor]:
        lib = nat.load()
        S = ev.shape[-1]
        K = coef.shape[0]
        lead = tuple(torch.broadcast_shapes(ev.shape[:-1], x.shape))
        e = ev.detach().expand(lead + (S,)).resolve_conj().resolve_neg().contiguous()
        xd = x.detach().to(torch.float32)
        if xd.numel() == 1:
            xf, xs = xd.reshape(1).contiguous(), 0
        else:
            xf, xs = xd.expand(lead).contiguous(), 1
        cf = coef.detach().to(torch.float32).contiguous()
        B = e.numel() // S
        pick = torch.empty(lead, dtype=torch.int32, device=ev.device)
        scale = torch.empty(lead, dtype=C64, device=ev.device)
        p = torch.empty(lead + (K,), dtype=torch.float32, device=ev.device)
        nat.check(lib.tcg_kraus_pick(nat.ptr(e), S, nat.ptr(cf), K, nat.ptr(xf), xs, B, nat.ptr(pick),
                                     nat.ptr(scale), nat.ptr(p), _stream()), "kraus pick")
        return pick, scale, p

    @staticmethod
    def setup_context(ctx: Any, inputs: Tuple[Any, ...], output: Any) -> None:
        ev, coef, _ = inputs
        pick, _, p = output
        ctx.mark_non_differentiable(pick, p)
        ctx.save_for_backward(pick, p)
        ctx.coef = coef.detach().to(torch.float32).contiguous()
        ctx.ev_shape = ev.shape

    @staticmethod
    def backward(ctx: Any, g_pick: Any, g_scale: Any, g_p: Any) -> Any:
        if g_scale is None:
            return None, None, None
        pick, p = ctx.saved_tensors
        gev = KrausPickBwdFn.apply(g_scale, pick, p, ctx.coef)
        if gev.shape != ctx.ev_shape:
            gev = gev.sum_to_size(ctx.ev_shape)
        return gev, None, None

    @staticmethod
    def vmap(info: Any, in_dims: Tuple[Any, ...], ev: torch.Tensor, coef: torch.Tensor, x: torch.Tensor) -> Any:
        ed, cd, xd = in_dims
        if cd is not None:
            raise NotImplementedError("KrausPickFn: batched Kraus expansions")
        if ed is None and xd is None:
            return KrausPickFn.apply(ev, coef, x), (None, None, None)
        ev = ev.movedim(ed, 0) if ed is not None else ev.unsqueeze(0)
        x = x.movedim(xd, 0) if xd is not None else x.unsqueeze(0)
        return KrausPickFn.apply(ev, coef, x), (0, 0, 0)


class KrausPickBwdFn(torch.autograd.Function):
    """Backward of :class:`KrausPickFn` (``tcg_kraus_pick_backward``):
    (rescale cotangent [...], pick [...], p [..., K], coef [K, S]) -> the
    cotangent of ev [..., S].  A Function of its own so that, like the
    adjoint sweep, it runs on plain tensors under ``vmap``."""

    @staticmethod
    def forward(gscale: torch.Tensor, pick: torch.Tensor, p: torch.Tensor, coef: torch.Tensor) -> torch.Tensor:
        lib = nat.load()
        K, S = coef.shape
        lead = tuple(torch.broadcast_shapes(gscale.shape, pick.shape, p.shape[:-1]))
        gs = gscale.detach().to(C64).expand(lead).resolve_conj().resolve_neg().contiguous()
        pk = pick.expand(lead).contiguous()
        pp = p.expand(lead + (K,)).contiguous()
        cf = coef.detach().to(torch.float32).contiguous()
        gev = torch.empty(lead + (S,), dtype=C64, device=gs.device)
        nat.check(lib.tcg_kraus_pick_backward(nat.ptr(gs), nat.ptr(pk), nat.ptr(pp), K, nat.ptr(cf), S, gs.numel(),
                                              nat.ptr(gev), _stream()), "kraus pick backward")
        return gev

    @staticmethod
    def setup_context(ctx: Any, inputs: Tuple[Any, ...], output: Any) -> None:
        pass

    @staticmethod
    def backward(ctx: Any, *grads: Any) -> Any:
        raise NotImplementedError("second derivatives through the Kraus pick are not supported")

    @staticmethod
    def vmap(info: Any, in_dims: Tuple[Any, ...], gscale: torch.Tensor, pick: torch.Tensor, p: torch.Tensor,
             coef: torch.Tensor) -> Any:
        gd, kd, pd, cd = in_dims
        if cd is not None:
            raise NotImplementedError("KrausPickBwdFn: batched Kraus expansions")
        if gd is None and kd is None and pd is None:
            return KrausPickBwdFn.apply(gscale, pick, p, coef), None

        def mv(x: torch.Tensor, d: Optional[int]) -> torch.Tensor:
            return x.movedim(d, 0) if d is not None else x.unsqueeze(0)

        return KrausPickBwdFn.apply(mv(gscale, gd), mv(pick, kd), mv(p, pd), coef), 0


class SampleFn(torch.autograd.Function):
    """Inverse-CDF sampling with given uniforms (``tcg_sample``); int64 out."""

    @staticmethod
    def forward(psi: torch.Tensor, u: torch.Tensor, n: int, nshots: int) -> torch.Tensor:
        lib = nat.load()
        N = 1 << n
        lead = _lead(psi.shape[:-1], u.shape[:-1])
        p = _flat(psi.detach(), lead, N).contiguous()
        B = p.shape[0]
        uu = u.detach().to(torch.float32)
        if uu.dim() == 1 and len(lead) > 0:
            uf = uu.contiguous()
            ustride = 0
        else:
            uf = _flat(uu, lead, nshots).contiguous()
            ustride = nshots
        out = torch.empty((B, nshots), dtype=torch.int64, device=p.device)
        nbytes = int(lib.tcg_sample_scratch_bytes(n, B))
        scratch = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=p.device)
        nat.check(lib.tcg_sample(nat.ptr(p), n, B, nat.ptr(uf), ustride, nshots, nat.ptr(out), nat.ptr(scratch),
                                 nbytes, _stream()), "sample")
        return out.reshape(lead + (nshots,))

    @staticmethod
    def setup_context(ctx: Any, inputs: Any, output: Any) -> None:
        ctx.mark_non_differentiable(output)

    @staticmethod
    def backward(ctx: Any, g: Any) -> Any:
        return None, None, None, None

    @staticmethod
    def vmap(info: Any, in_dims: Tuple[Any, ...], psi: torch.Tensor, u: torch.Tensor, n: int, nshots: int) -> Any:
        pd, ud, _, _ = in_dims
        psi = psi.movedim(pd, 0) if pd is not None else psi.unsqueeze(0)
        if ud is not None:
            u = u.movedim(ud, 0)
        return SampleFn.apply(psi, u, n, nshots), 0


class ProbabilityFn(torch.autograd.Function):
    """p = |psi|^2 by the engine's probability kernel (re^2 + im^2 in fp32);
    backward dL/dpsi = 2 g psi in torch's complex convention.  The vmap rule
    runs the kernel once over the whole batch."""

    @staticmethod
    def forward(psi: torch.Tensor) -> torch.Tensor:  # type: ignore[override]
        return probability_native(psi)

    @staticmethod
    def setup_context(ctx: Any, inputs: Tuple[Any, ...], output: Any) -> None:
        ctx.save_for_backward(inputs[0])

    @staticmethod
    def backward(ctx: Any, g: torch.Tensor) -> torch.Tensor:  # type: ignore[override]
        (psi,) = ctx.saved_tensors
        return 2.0 * g * psi

    @staticmethod
    def vmap(info: Any, in_dims: Tuple[Any, ...], psi: torch.Tensor) -> Tuple[torch.Tensor, Any]:
        d = in_dims[0]
        if d is None:
            return ProbabilityFn.apply(psi), None
        return ProbabilityFn.apply(psi.movedim(d, 0)), 0


def probability_native(psi: torch.Tensor) -> torch.Tensor:
    """|psi|^2 through the engine kernel (no autograd).  The state must be a
    CUDA tensor: the engine has no CPU path."""
    if not psi.is_cuda:
        raise RuntimeError("probability: the state must be a CUDA tensor (the engine has no CPU path)")
    lib = nat.load()
    p = torch.empty(psi.shape, dtype=torch.float32, device=psi.device)
    src = psi.detach().resolve_conj().resolve_neg().contiguous()
    nat.check(lib.tcg_probability(nat.ptr(src), src.numel(), nat.ptr(p), _stream()), "probability")
    return p
