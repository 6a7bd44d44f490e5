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


# ---- shared-memory barrier discipline of the generated kernels -------------
_BUF = r"(smp|smq|smu)"


def _stage_cases(kernel_src):
    """The stage-entry code of one kernel in execution order (the stage loop
    runs its cases 0, 1, ...), followed by the code after the loop."""
    i = kernel_src.index("switch (s) {")
    j = kernel_src.index("default: break;", i)
    cases = re.split(r"\n    case \d+: \{", kernel_src[i:j])[1:]
    tail = kernel_src[kernel_src.rindex("\n  }\n") :]
    return cases + [tail]


def _check_barriers(kernel_src):
    """A tile buffer is never written while another thread may still be
    reading it: after a read, the next write to the same buffer comes after
    a __syncthreads()."""
    pending = set()
    for block in _stage_cases(kernel_src):
        for line in block.split("\n"):
            if "__syncthreads" in line:
                pending.clear()
            if "denseK_smem" in line:
                buf = re.search(r"denseK_smem<\d+>\(" + _BUF, line).group(1)
                assert buf not in pending, line
                pending.add(buf)
                continue
            for m in re.finditer(_BUF + r"\[[^\]]*\]\s*=(?!=)", line):
                assert m.group(1) not in pending, (m.group(1), line)
            for m in re.finditer(r"=\s*" + _BUF + r"\[|, c = " + _BUF + r"\[", line):
                pending.add(m.group(1) or m.group(2))


def _kernels(handle, which, mode):
    st, src = nat.jit_info(handle, which, mode, what=1)
    return re.split(r'extern "C"', src)[1:]


def test_tile_buffers_wait_for_readers():
    """Kernels that hold psi only alternate two tile buffers so a layout
    change needs one barrier; every write into a buffer must still follow a
    barrier after the last read of that buffer (forward with register and
    shared-memory stages, adjoint, measurement)."""
    n, nl = 20, 8
    c = templates.apply_hea(cmod.Circuit(n), n, nl, np.zeros(templates.hea_nparams(n, nl)))
    e = cmod._build_entry(n, c._ops)
    rng = np.random.default_rng(5)
    gl = random_gate_list(14, 60, rng)
    cr = templates.apply_gate_list(cmod.Circuit(14), gl)
    er = cmod._build_entry(14, cr._ops)
    terms = [eng.pauli_masks(16, [i], [], []) for i in range(16)]
    terms += [eng.pauli_masks(16, [], [], [i, i + 1]) for i in range(15)]
    tp = eng.TermPlan(16, tuple(terms))
    checked = 0
    for handle, which, mode in ((e.plan.handle, 0, 0), (e.plan.handle, 1, 1), (er.plan.handle, 0, 0),
                                (er.plan.handle, 1, 1), (tp.handle, 2, 2), (tp.handle, 2, 3)):
        for k in _kernels(handle, which, mode):
            _check_barriers(k)
            checked += 1
    assert checked >= 10
    # the forward kernels do use the second buffer
    assert any("smq[" in k for k in _kernels(e.plan.handle, 0, 0))


def test_long_rotation_pass_compiles():
    """A pass with more rotations than the CTA's shear table holds (a deep
    ansatz on few qubits: every gate in one pass) still generates code that
    compiles: rotations past the table compute their own parameters.  (Such
    a pass's operand tables exceed the constant bank, so the engine keeps
    the generic kernels for it; the source is still well formed.)"""
    n, nl = 8, 140  # 1120 rx rotations (and 140 Z-rotation runs) in one pass
    c = templates.apply_hea(cmod.Circuit(n), n, nl, np.zeros(templates.hea_nparams(n, nl)))
    e = cmod._build_entry(n, c._ops)
    assert e.plan.npasses == 1
    st, src = nat.jit_info(e.plan.handle, 0, 0, what=1)
    # table rotations read shk[]; the ones past it compute their parameters
    assert "shk[op.g0]" in src and "pneg ^= shear_params" in src
    rc, log = compile_source(src)
    assert rc == 0, log[-3000:]
