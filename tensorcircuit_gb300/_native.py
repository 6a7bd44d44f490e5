"""ctypes binding of the engine's C ABI (``include/tcgb300.h``).

The library is loaded from the package's ``lib/`` folder.  There is no CPU
fallback: when the library or a CUDA device is missing, every entry point
raises, so a silent non-native path can never stand in for the kernels.
"""

import ctypes
import os
import threading
from typing import Any, Optional

from . import _build

TCG_OK = 0
TCG_ERR_INVALID_ARG = 1
TCG_ERR_DUP_QUBIT = 2
TCG_ERR_UNSUPPORTED = 3
TCG_ERR_CUDA = 4
TCG_ERR_SCRATCH = 5
TCG_ERR_OOM = 6
TCG_ERR_TOO_LARGE = 7
TCG_ERR_TIMEOUT = 8
TCG_ACC_OVERWRITE = 1

TCG_GATE_DENSE = 0
TCG_GATE_DIAG = 1
TCG_GATE_PAULI_ROT = 2
MAX_GATE_QUBITS = 6
MIN_QUBITS = 6


class TcgGate(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int32),
        ("nq", ctypes.c_int32),
        ("qubits", ctypes.c_int32 * MAX_GATE_QUBITS),
        ("pauli", ctypes.c_int32 * MAX_GATE_QUBITS),
        ("mat_off", ctypes.c_int64),
        ("grad_off", ctypes.c_int64),
    ]


class TcgPlanOpts(ctypes.Structure):
    _fields_ = [("tile_bits", ctypes.c_int32), ("max_stage_grad_entries", ctypes.c_int32), ("zrun_max", ctypes.c_int32)]


class TcgPlanStats(ctypes.Structure):
    _fields_ = [
        ("nqubits", ctypes.c_int32),
        ("ngates", ctypes.c_int32),
        ("npasses", ctypes.c_int32),
        ("nstages", ctypes.c_int32),
        ("tile_bits", ctypes.c_int32),
        ("grad_entries", ctypes.c_int64),
    ]


class TcgPauli(ctypes.Structure):
    _fields_ = [("xmask", ctypes.c_uint64), ("zmask", ctypes.c_uint64)]


class TcgUbatchCircuit(ctypes.Structure):
    _fields_ = [
        ("nqubits", ctypes.c_int32),
        ("ngates", ctypes.c_int32),
        ("gates", ctypes.POINTER(TcgGate)),
        ("nmat", ctypes.c_int64),
        ("mat_const", ctypes.POINTER(ctypes.c_float)),
        ("mat_param", ctypes.POINTER(ctypes.c_int64)),
        ("mat_scale", ctypes.POINTER(ctypes.c_float)),
        ("nparams", ctypes.c_int32),
        ("nterms", ctypes.c_int32),
        ("terms", ctypes.POINTER(TcgPauli)),
        ("coef", ctypes.POINTER(ctypes.c_float)),
        ("offset", ctypes.c_double),
    ]


# (name, restype, argtypes) for every exported symbol
_P = ctypes.c_void_p
_I32 = ctypes.c_int32
_I64 = ctypes.c_int64
_SZ = ctypes.c_size_t
SIGNATURES = [
    ("tcg_abi_version", _I32, []),
    ("tcg_status_string", ctypes.c_char_p, [_I32]),
    ("tcg_plan_create", ctypes.c_int, [_I32, ctypes.POINTER(TcgGate), _I32, ctypes.POINTER(TcgPlanOpts), ctypes.POINTER(_P)]),
    ("tcg_plan_destroy", ctypes.c_int, [_P]),
    ("tcg_plan_get_stats", ctypes.c_int, [_P, ctypes.POINTER(TcgPlanStats)]),
    ("tcg_plan_tensor_passes", ctypes.c_int, [_P]),
    ("tcg_set_tensor_policy", _I32, [_I32]),
    ("tcg_plan_check", ctypes.c_int, [_P, _P]),
    ("tcg_debug_tc_mma", ctypes.c_int, [_P, _P, _P, _I32, _I32, _P, _P]),
    ("tcg_debug_tc_program", ctypes.c_int, [_P, ctypes.POINTER(_P), ctypes.POINTER(_I64), ctypes.POINTER(_I64)]),
    ("tcg_forward", ctypes.c_int, [_P, _P, _I64, _P, _I64, _P]),
    ("tcg_forward_from", ctypes.c_int, [_P, _P, _I64, _P, _I64, _P, _I64, _P]),
    ("tcg_backward_scratch_bytes", _SZ, [_P, _I64]),
    ("tcg_backward", ctypes.c_int, [_P, _P, _P, _I64, _P, _I64, _P, _I64, _P, _SZ, _P]),
    ("tcg_backward_from", ctypes.c_int, [_P, _P, _P, _P, _I64, _P, _I64, _P, _I64, _P, _SZ, _P]),
    ("tcg_mplan_create", ctypes.c_int, [_I32, ctypes.POINTER(TcgPauli), _I32, ctypes.POINTER(_P)]),
    ("tcg_mplan_destroy", ctypes.c_int, [_P]),
    ("tcg_mplan_passes", ctypes.c_int, [_P]),
    ("tcg_expect_scratch_bytes", _SZ, [_P, _I64]),
    ("tcg_expect_pauli", ctypes.c_int, [_P, _P, _I64, _P, _P, _SZ, _P]),
    ("tcg_pauli_accumulate", ctypes.c_int, [_P, _P, _P, _I64, _P, _I64, _P]),
    ("tcg_pauli_accumulate_ex", ctypes.c_int, [_P, _P, _P, _I64, _P, _I64, ctypes.c_int32, _P]),
    ("tcg_expect_pauli_noalloc", ctypes.c_int, [_P, _I32, _I64, ctypes.POINTER(TcgPauli), _I32, _P, _P]),
    ("tcg_sample_scratch_bytes", _SZ, [_I32, _I64]),
    ("tcg_sample", ctypes.c_int, [_P, _I32, _I64, _P, _I64, _I64, _P, _P, _SZ, _P]),
    ("tcg_kraus_pick", ctypes.c_int, [_P, _I32, _P, _I32, _P, _I64, _I64, _P, _P, _P, _P]),
    ("tcg_kraus_pick_backward", ctypes.c_int, [_P, _P, _P, _I32, _P, _I32, _I64, _P, _P]),
    ("tcg_probability", ctypes.c_int, [_P, _I64, _P, _P]),
    ("tcg_inner_scratch_bytes", _SZ, [_I64, _I64]),
    ("tcg_inner", ctypes.c_int, [_P, _P, _I64, _I64, _P, _P, _SZ, _P]),
    ("tcg_ubatch_create", ctypes.c_int, [ctypes.POINTER(TcgUbatchCircuit), _I32, _I32, ctypes.POINTER(_P)]),
    ("tcg_ubatch_create_ex", ctypes.c_int,
     [ctypes.POINTER(TcgUbatchCircuit), _I32, ctypes.POINTER(TcgPlanOpts), ctypes.POINTER(_P)]),
    ("tcg_ubatch_destroy", ctypes.c_int, [_P]),
    ("tcg_ubatch_info", ctypes.c_int, [_P, ctypes.POINTER(_I64), ctypes.POINTER(_I64), ctypes.POINTER(_SZ)]),
    ("tcg_ubatch_state_offset", _I64, [_P, _I32]),
    ("tcg_ubatch_value_and_grad", ctypes.c_int, [_P, _P, _P, _P, _P, _SZ, _P]),
    ("tcg_ubatch_stats", ctypes.c_int, [_P, ctypes.POINTER(_I64), ctypes.POINTER(ctypes.c_double)]),
    ("tcg_ubatch_check", ctypes.c_int, [_P, _P, _P]),
    ("tcg_ubatch_set_wait_limit", ctypes.c_int, [_P, ctypes.c_uint64]),
    ("tcg_debug_ubatch_set_need", ctypes.c_int, [_P, _I32, _I32, ctypes.c_uint32]),
    ("tcg_mlp_linear_forward", ctypes.c_int, [_P, _I32, _P, _P, _I64, _I32, _I32, _I32, _P, _P, _I32, _P]),
    ("tcg_mlp_linear_backward", ctypes.c_int,
     [_P, _P, _I32, _P, _I32, _P, _I64, _I32, _I32, _P, _P, _P, _P, _P]),
    ("tcg_periodic_loss", ctypes.c_int, [_P, _P, _I64, _P, _P, _I32, _P]),
    ("tcg_adam_update", ctypes.c_int, [_P, _P, _P, _P, _I64, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                       ctypes.c_float, _I32, _P]),
    ("tcg_launch_count", _I64, []),
    ("tcg_debug_jit", ctypes.c_int, [_P, _I32, _I32, ctypes.POINTER(_I32), ctypes.c_char_p, _I64, _I32]),
    ("tcg_debug_program", ctypes.c_int, [_P, _I32, ctypes.POINTER(_P), ctypes.POINTER(_I64), ctypes.POINTER(_I64)]),
]


# Mirrors of the device-program records (tensorcircuit_gb300/csrc/engine.h),
# read by the CPU replay in the tests.
class DevPass(ctypes.Structure):
    _fields_ = [("L", ctypes.c_int32), ("nnonlocal", ctypes.c_int32), ("lbits", ctypes.c_int32 * 13),
                ("nlbits", ctypes.c_int32 * 32), ("stage_begin", ctypes.c_int32), ("stage_end", ctypes.c_int32),
                ("runs_off", ctypes.c_int32), ("pad", ctypes.c_int32)]


class DevStage(ctypes.Structure):
    _fields_ = [("R", ctypes.c_int32), ("smem_stage", ctypes.c_int32), ("lanes_low", ctypes.c_int32),
                ("nthread_bits", ctypes.c_int32), ("reg_tile", ctypes.c_int32 * 6),
                ("thr_tile", ctypes.c_int32 * 16), ("op_begin", ctypes.c_int32), ("op_end", ctypes.c_int32),
                ("nslots", ctypes.c_int32), ("slot_out_begin", ctypes.c_int32), ("slot_out_end", ctypes.c_int32)]


class DevOp(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("k", ctypes.c_int32), ("p", ctypes.c_int32 * 6),
                ("xreg", ctypes.c_int32), ("nY", ctypes.c_int32), ("zmask", ctypes.c_uint32),
                ("slot", ctypes.c_int32), ("mat_off", ctypes.c_int64), ("grad_off", ctypes.c_int64)]


class ZEnt(ctypes.Structure):
    _fields_ = [("zmask", ctypes.c_uint32), ("zreg", ctypes.c_int32), ("slot", ctypes.c_int32),
                ("pad", ctypes.c_int32), ("mat_off", ctypes.c_int64), ("grad_off", ctypes.c_int64)]


class SlotOut(ctypes.Structure):
    _fields_ = [("slot", ctypes.c_int32), ("pad", ctypes.c_int32), ("out_off", ctypes.c_int64)]


def jit_info(handle: Any, which: int, mode: int, what: int = 0, cap: int = 1 << 22) -> "tuple[int, str]":
    """(state, text) of a plan direction's specialised kernels: state 0 not
    built, 1 built, -1 failed; text = compile log (what=0) or generated
    source (what=1)."""
    lib = load()
    st = ctypes.c_int32(0)
    buf = ctypes.create_string_buffer(cap)
    check(lib.tcg_debug_jit(handle, which, mode, ctypes.byref(st), buf, cap, what), "debug_jit")
    return st.value, buf.value.decode(errors="replace")


def debug_program(handle: Any, which: int) -> dict:
    """Copy of a plan's device program as lists of ctypes records."""
    lib = load()
    arrs = (ctypes.c_void_p * 6)()
    cnts = (ctypes.c_int64 * 6)()
    szs = (ctypes.c_int64 * 6)()
    check(lib.tcg_debug_program(handle, which, arrs, cnts, szs), "debug_program")
    out = {}
    for i, (name, typ) in enumerate([("passes", DevPass), ("stages", DevStage), ("ops", DevOp),
                                     ("slot_out", SlotOut), ("runs", ctypes.c_uint32), ("zents", ZEnt)]):
        if ctypes.sizeof(typ) != szs[i]:
            raise EngineError("record size mismatch for %s: %d vs %d" % (name, ctypes.sizeof(typ), szs[i]))
        if cnts[i] == 0:
            out[name] = []
            continue
        arr = (typ * cnts[i]).from_address(arrs[i])
        out[name] = [arr[j] for j in range(cnts[i])] if typ is not ctypes.c_uint32 else list(arr)
    return out

class TcPassDesc(ctypes.Structure):
    _fields_ = [("pass_", ctypes.c_int32), ("block_begin", ctypes.c_int32), ("block_end", ctypes.c_int32),
                ("ldpair", ctypes.c_int32), ("ldaddr", ctypes.c_uint32 * 12)]


class TcBlock(ctypes.Structure):
    _fields_ = [("bbits", ctypes.c_int32 * 6), ("cbits", ctypes.c_int32 * 6), ("gate_begin", ctypes.c_int32),
                ("gate_end", ctypes.c_int32), ("slot", ctypes.c_int32), ("pairbit", ctypes.c_int32),
                ("raddr", ctypes.c_uint32 * 64), ("caddr", ctypes.c_uint32 * 64)]


class TcGate(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("k", ctypes.c_int32), ("pos", ctypes.c_int32 * 6),
                ("xmask", ctypes.c_int32), ("zmask", ctypes.c_int32), ("nY", ctypes.c_int32),
                ("pad", ctypes.c_int32), ("mat_off", ctypes.c_int64)]


def debug_tc_program(handle: Any) -> dict:
    """Copy of a plan's fused-block (tensor-core) program: pass descriptors,
    blocks, source gates and the cost model's per-pass preference."""
    lib = load()
    arrs = (ctypes.c_void_p * 4)()
    cnts = (ctypes.c_int64 * 4)()
    szs = (ctypes.c_int64 * 4)()
    check(lib.tcg_debug_tc_program(handle, arrs, cnts, szs), "debug_tc_program")
    out = {}
    for i, (name, typ) in enumerate([("passes", TcPassDesc), ("blocks", TcBlock), ("gates", TcGate),
                                     ("prefer", ctypes.c_int32)]):
        if ctypes.sizeof(typ) != szs[i]:
            raise EngineError("record size mismatch for %s: %d vs %d" % (name, ctypes.sizeof(typ), szs[i]))
        if cnts[i] == 0:
            out[name] = []
            continue
        arr = (typ * cnts[i]).from_address(arrs[i])
        out[name] = [arr[j] for j in range(cnts[i])] if typ is not ctypes.c_int32 else list(arr)
    return out


_lib: Optional[ctypes.CDLL] = None
_lock = threading.Lock()


class EngineError(RuntimeError):
    """A status code other than TCG_OK from the native engine."""


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load (building first if needed) the engine library."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.lib_path()
        if build_if_missing:
            path = _build.build()
        if not os.path.exists(path):
            raise EngineError("engine library %s is missing; run tensorcircuit_gb300._build.build()" % path)
        lib = ctypes.CDLL(path)
        for name, res, args in SIGNATURES:
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def check(status: int, what: str = "") -> None:
    """Map a status code to the exception type the reference raises."""
    if status == TCG_OK:
        return
    msg = load().tcg_status_string(status).decode()
    if what:
        msg = "%s: %s" % (what, msg)
    if status == TCG_ERR_DUP_QUBIT:
        raise AssertionError(msg)
    if status in (TCG_ERR_INVALID_ARG, TCG_ERR_TOO_LARGE):
        raise ValueError(msg)
    if status == TCG_ERR_UNSUPPORTED:
        raise NotImplementedError(msg)
    raise EngineError(msg)


def ptr(t: Any) -> int:
    """Device address of a tensor handed to a kernel entry point."""
    # a host address must never reach a kernel
    if not t.is_cuda:
        raise ValueError("a host tensor reached a device entry point of the engine; move it to the GPU first")
    # a lazily conjugated / negated view shares the raw buffer of its base:
    # the kernels would read the unconjugated values
    if t.is_conj() or t.is_neg():
        raise ValueError("a conjugate or negative view reached the engine; resolve it first")
    return int(t.data_ptr())


def stream_ptr(device: Any = None) -> int:
    import torch

    return int(torch.cuda.current_stream(device).cuda_stream)
