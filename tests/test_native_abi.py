"""CPU: the C-ABI library builds, loads and exports every symbol that
include/tcgb300.h declares; host-only entry points behave."""

import ctypes
import os
import re

import pytest

from tensorcircuit_gb300 import _native as nat

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    with open(os.path.join(ROOT, "include", "tcgb300.h")) as fh:
        src = fh.read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(tcg_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    lib = nat.load()
    names = declared_functions()
    assert len(names) >= 20
    for name in names:
        assert hasattr(lib, name), name
    assert nat.TCG_ACC_OVERWRITE == 1
    bound = {n for n, _, _ in nat.SIGNATURES}
    assert set(names) == bound, set(names) ^ bound


def test_status_strings_and_version():
    lib = nat.load()
    assert lib.tcg_abi_version() == 3
    assert lib.tcg_status_string(0) == b"ok"
    assert b"twice" in lib.tcg_status_string(2)


def test_host_side_errors_without_gpu():
    lib = nat.load()
    h = ctypes.c_void_p()
    assert lib.tcg_plan_create(3, None, 0, None, ctypes.byref(h)) == nat.TCG_ERR_INVALID_ARG
    assert lib.tcg_forward(None, None, 1, None, 0, None) == nat.TCG_ERR_INVALID_ARG
    assert lib.tcg_sample(None, 10, 1, None, 0, 1, None, None, 0, None) == nat.TCG_ERR_INVALID_ARG
    assert lib.tcg_sample_scratch_bytes(10, 2) >= 2 * 8 * 1024
    # Kraus pick: bad sizes are refused, an empty batch is a no-op, and a
    # non-empty batch without buffers is refused -- all before any launch
    assert lib.tcg_kraus_pick(None, 4, None, 2, None, 0, -1, None, None, None, None) == nat.TCG_ERR_INVALID_ARG
    assert lib.tcg_kraus_pick(None, 0, None, 2, None, 0, 1, None, None, None, None) == nat.TCG_ERR_INVALID_ARG
    assert lib.tcg_kraus_pick(None, 4, None, 2, None, -1, 1, None, None, None, None) == nat.TCG_ERR_INVALID_ARG
    assert lib.tcg_kraus_pick(None, 4, None, 2, None, 0, 0, None, None, None, None) == nat.TCG_OK
    assert lib.tcg_kraus_pick(None, 4, None, 2, None, 0, 3, None, None, None, None) == nat.TCG_ERR_INVALID_ARG
    assert lib.tcg_kraus_pick_backward(None, None, None, 0, None, 4, 1, None, None) == nat.TCG_ERR_INVALID_ARG
    assert lib.tcg_kraus_pick_backward(None, None, None, 2, None, 4, 0, None, None) == nat.TCG_OK
    assert lib.tcg_kraus_pick_backward(None, None, None, 2, None, 4, 5, None, None) == nat.TCG_ERR_INVALID_ARG
    # sweeps whose first pass reads elsewhere: argument checks come first
    from tensorcircuit_gb300 import engine as eng

    plan = eng.GatePlan(6, [(nat.TCG_GATE_DENSE, (0,), 0, -1)], 4)
    fake = ctypes.c_void_p(0x1000)
    other = ctypes.c_void_p(0x2000)
    assert lib.tcg_forward_from(None, fake, 0, other, 1, fake, 4, None) == nat.TCG_ERR_INVALID_ARG
    assert lib.tcg_forward_from(plan.handle, None, 0, other, 1, fake, 4, None) == nat.TCG_ERR_INVALID_ARG
    assert lib.tcg_forward_from(plan.handle, fake, -1, other, 1, fake, 4, None) == nat.TCG_ERR_INVALID_ARG
    # in place needs the state's own stride (2^6 here)
    assert lib.tcg_forward_from(plan.handle, fake, 0, fake, 1, fake, 4, None) == nat.TCG_ERR_INVALID_ARG
    assert lib.tcg_forward_from(plan.handle, fake, 0, other, 0, fake, 4, None) == nat.TCG_OK
    assert lib.tcg_backward_from(plan.handle, None, other, other, 1, fake, 4, None, 0, None, 0,
                                 None) == nat.TCG_ERR_INVALID_ARG
    assert lib.tcg_pauli_accumulate_ex(None, fake, other, 1, fake, 1, 0, None) == nat.TCG_ERR_INVALID_ARG
    # planner options: a negative Z-rotation fusion width is refused; the
    # uneven batch's option entry point checks its options before any work
    g = (nat.TcgGate * 1)()
    g[0].kind, g[0].nq, g[0].mat_off, g[0].grad_off = nat.TCG_GATE_DENSE, 1, 0, -1
    bad = nat.TcgPlanOpts(tile_bits=0, max_stage_grad_entries=0, zrun_max=-1)
    assert lib.tcg_plan_create(6, g, 1, ctypes.byref(bad), ctypes.byref(h)) == nat.TCG_ERR_INVALID_ARG
    ok = nat.TcgPlanOpts(tile_bits=0, max_stage_grad_entries=0, zrun_max=1)
    assert lib.tcg_plan_create(6, g, 1, ctypes.byref(ok), ctypes.byref(h)) == nat.TCG_OK
    assert lib.tcg_plan_destroy(h) == nat.TCG_OK
    uc = (nat.TcgUbatchCircuit * 1)()
    ub = ctypes.c_void_p()
    assert lib.tcg_ubatch_create_ex(uc, 1, None, ctypes.byref(ub)) == nat.TCG_ERR_INVALID_ARG
    assert lib.tcg_ubatch_create_ex(uc, 1, ctypes.byref(bad), ctypes.byref(ub)) == nat.TCG_ERR_INVALID_ARG
    assert lib.tcg_ubatch_create_ex(None, 1, ctypes.byref(ok), ctypes.byref(ub)) == nat.TCG_ERR_INVALID_ARG
    # the probability kernel takes device states only: a host tensor is refused
    # before anything reaches the library
    import torch

    with pytest.raises(RuntimeError, match="CUDA tensor"):
        eng.probability_native(torch.zeros(8, dtype=torch.complex64))
    # and no host tensor's address is handed to a kernel entry point
    with pytest.raises(ValueError, match="host tensor"):
        nat.ptr(torch.zeros(4))
    assert lib.tcg_launch_count() == 0
