"""CPU: the plan specialiser's generated kernels compile for sm_103a (with
the same preamble NVRTC uses), for every op kind and all four modes, and fit
the register budget without spilling -- with nvcc (for the register report)
and with NVRTC itself, the compiler the engine runs (it accepts a narrower
language: no compiler builtins such as __builtin_popcount).  Skipped when
nvcc is absent."""

import ctypes
import os
import re
import shutil
import subprocess
import tempfile

import numpy as np
import pytest

from tensorcircuit_gb300 import _native as nat
from tensorcircuit_gb300 import circuit as cmod
from tensorcircuit_gb300 import engine as eng
from tensorcircuit_gb300 import templates
from tests.test_plan_replay import random_gate_list

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PREAMBLE = os.path.join(ROOT, "tensorcircuit_gb300", "csrc", "jit_device.cuh")

nvcc = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else None)
pytestmark = pytest.mark.skipif(nvcc is None, reason="nvcc not available")


def compile_source(src):
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "k.cu")
        with open(path, "w") as fh:
            fh.write(open(PREAMBLE).read() + "\n" + src)
        r = subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "-cubin",
                            "-Xptxas", "-v", path, "-o", os.path.join(d, "k.cubin")],
                           capture_output=True, text=True)
        return r.returncode, r.stdout + r.stderr


def _nvrtc():
    for name in ("libnvrtc.so.13", "libnvrtc.so", "/usr/local/cuda/lib64/libnvrtc.so.13"):
        try:
            return ctypes.CDLL(name)
        except OSError:
            continue
    return None


def compile_nvrtc(src):
    """Compile as the engine does (csrc/jit.cpp: same options, same name)."""
    lib = _nvrtc()
    if lib is None:
        pytest.skip("NVRTC not available")
    full = (open(PREAMBLE).read() + "\n" + src).encode()
    prog = ctypes.c_void_p()
    assert lib.nvrtcCreateProgram(ctypes.byref(prog), full, b"tcg_pass.cu", 0, None, None) == 0
    opts = [b"--gpu-architecture=sm_103a", b"--std=c++17", b"-lineinfo", b"--ptxas-options=-v"]
    arr = (ctypes.c_char_p * len(opts))(*opts)
    rc = lib.nvrtcCompileProgram(prog, len(opts), arr)
    size = ctypes.c_size_t(0)
    lib.nvrtcGetProgramLogSize(prog, ctypes.byref(size))
    buf = ctypes.create_string_buffer(max(size.value, 1))
    lib.nvrtcGetProgramLog(prog, buf)
    lib.nvrtcDestroyProgram(ctypes.byref(prog))
    return rc, buf.value.decode(errors="replace")


def check_compiles(handle, which, mode):
    st, src = nat.jit_info(handle, which, mode, what=1)
    assert "tcgk" in src and "_0(" in src
    rc, log = compile_source(src)
    assert rc == 0, log[-3000:]
    rc, nlog = compile_nvrtc(src)
    assert rc == 0, nlog[-3000:]
    spills = [int(x) for x in re.findall(r"(\d+) bytes spill stores", log)]
    regs = [int(x) for x in re.findall(r"Used (\d+) registers", log)]
    return regs, spills


def test_hea_forward_and_adjoint_kernels_compile():
    n, nl = 20, 8
    c = templates.apply_hea(cmod.Circuit(n), n, nl, np.zeros(templates.hea_nparams(n, nl)))
    e = cmod._build_entry(n, c._ops)
    regs_f, sp_f = check_compiles(e.plan.handle, 0, 0)
    regs_b, sp_b = check_compiles(e.plan.handle, 1, 1)
    print("forward registers", regs_f, "adjoint registers", regs_b, "spills", sp_f, sp_b)
    # forward passes (Z-rotation runs included) run three CTAs per SM (<= 80
    # registers), the adjoint two (<= 128); either may spill a few words
    assert max(sp_f + [0]) <= 64 and max(sp_b + [0]) <= 64
    assert max(regs_f) <= 80 and max(regs_b) <= 128, (regs_f, regs_b)


def test_brickwall_forward_kernels_fit_three_ctas():
    """Dense 2-qubit passes (no Z runs) run three CTAs per SM: <= 80
    registers with at most a few spilled words."""
    n = 24
    gl = templates.brickwall_gate_list(n, 8, 3)
    c = templates.apply_gate_list(cmod.Circuit(n), gl)
    e = cmod._build_entry(n, c._ops)
    regs, spills = check_compiles(e.plan.handle, 0, 0)
    assert max(regs) <= 80 and max(spills + [0]) <= 64, (regs, spills)


def test_random_circuit_kernels_compile():
    rng = np.random.default_rng(5)
    gl = random_gate_list(14, 60, rng)
    c = templates.apply_gate_list(cmod.Circuit(14), gl)
    e = cmod._build_entry(14, c._ops)
    check_compiles(e.plan.handle, 0, 0)
    check_compiles(e.plan.handle, 1, 1)


def test_measure_kernels_compile():
    n = 16
    terms = [eng.pauli_masks(n, [i], [], []) for i in range(n)]
    terms += [eng.pauli_masks(n, [], [], [i, i + 1]) for i in range(n - 1)]
    terms += [eng.pauli_masks(n, [], [i, i + 1], [i + 2]) for i in range(n - 2)]
    tp = eng.TermPlan(n, tuple(terms))
    check_compiles(tp.handle, 2, 2)
    check_compiles(tp.handle, 2, 3)
