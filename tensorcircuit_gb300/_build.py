"""Build recipe for the engine's shared library (``libtcgb300.so``).

Every CUDA translation unit is compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``) in parallel, then linked into
one C-ABI shared library that the Python layer loads with ctypes.  The
library is written in-tree (``tensorcircuit_gb300/lib/``) so the process that
uses it loads it from the repository.
"""

import concurrent.futures
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
OBJDIR = os.path.join(HERE, "lib", "obj")
LIBNAME = "libtcgb300.so"
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

SOURCES = ["pass.cu", "pass_inst.cu", "misc.cu", "api.cu", "plan.cpp", "jit.cpp", "noalloc.cu", "batch.cu", "mlp.cu",
           "tcpass.cu"]
HEADERS = ["engine.h", "kernels.h", "plan.h", "jit.h", "jit_device.cuh", "pass.cuh"]

# pass_inst.cu is compiled once per kernel family of pass.cuh (mode x body:
# 0 pass_kernel, 1 batch_kernel full body, 2 batch_kernel light body), so the
# twelve large kernel bodies compile in parallel.
_PASS_FAMILIES = [(mode, kind) for mode in range(4) for kind in range(3)]


def _units():
    """(source, object name, extra nvcc flags) for every object of the library."""
    out = []
    for src in SOURCES:
        stem = os.path.splitext(src)[0]
        if src == "pass_inst.cu":
            for mode, kind in _PASS_FAMILIES:
                out.append((src, "%s_m%d_k%d.o" % (stem, mode, kind),
                            ["-DTCG_PASS_MODE=%d" % mode, "-DTCG_PASS_KIND=%d" % kind]))
        else:
            out.append((src, stem + ".o", []))
    return out


def _write_jit_include() -> None:
    """Embed jit_device.cuh in the library as a string literal
    (lib/obj/jit_device.inc), the preamble NVRTC compiles with every
    generated pass kernel."""
    with open(os.path.join(CSRC, "jit_device.cuh")) as fh:
        text = fh.read()
    if ")TCGJIT" in text:
        raise RuntimeError("jit_device.cuh must not contain the raw-string delimiter")
    out = os.path.join(OBJDIR, "jit_device.inc")
    body = 'R"TCGJIT(' + text + ')TCGJIT"\n'
    if not os.path.exists(out) or open(out).read() != body:
        with open(out, "w") as fh:
            fh.write(body)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the engine needs the CUDA toolkit to build")


def lib_path() -> str:
    return os.path.join(LIBDIR, LIBNAME)


def _digest() -> str:
    h = hashlib.sha256()
    for f in SOURCES + HEADERS:
        with open(os.path.join(CSRC, f), "rb") as fh:
            h.update(f.encode())
            h.update(fh.read())
    with open(os.path.join(INCLUDE, "tcgb300.h"), "rb") as fh:
        h.update(fh.read())
    h.update(" ".join(ARCH).encode())
    return h.hexdigest()[:16]


def _compile(unit, nvcc: str, verbose: bool) -> str:
    src, objname, flags = unit
    obj = os.path.join(OBJDIR, objname)
    cmd = [nvcc, *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", *flags,
           "-I", INCLUDE, "-I", OBJDIR, "-c", os.path.join(CSRC, src), "-o", obj]
    if src.endswith(".cpp"):
        cmd[1:1] = ["-x", "cu"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    if verbose and (r.stdout or r.stderr):
        print(r.stdout, r.stderr, file=sys.stderr)
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile (if sources changed) and return the path of the library."""
    os.makedirs(OBJDIR, exist_ok=True)
    stamp = os.path.join(LIBDIR, "build.stamp")
    dig = _digest()
    if not force and os.path.exists(lib_path()) and os.path.exists(stamp):
        with open(stamp) as fh:
            if fh.read().strip() == dig:
                return lib_path()
    nvcc = nvcc_path()
    _write_jit_include()
    units = _units()
    # the slowest units first, so a machine with fewer cores than units
    # starts them early
    order = sorted(range(len(units)), key=lambda i: units[i][0] != "pass_inst.cu")
    workers = min(len(units), max(2, os.cpu_count() or 2))
    with concurrent.futures.ThreadPoolExecutor(max_workers=workers) as ex:
        done = dict(zip(order, ex.map(lambda i: _compile(units[i], nvcc, verbose), order)))
    objs = [done[i] for i in range(len(units))]
    tmp = lib_path() + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, lib_path())
    with open(stamp, "w") as fh:
        fh.write(dig)
    return lib_path()


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
