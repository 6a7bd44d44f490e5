"""Circuit records to and from text: the reference's JSON form
(tensorcircuit/translation.py:587-702), qsim files
(abstractcircuit.py ``from_qsim_file`` / ``_apply_qsim``) and OpenQASM 2.

JSON entries are ``{"name", "qubits"}`` plus, unless ``simplified``, the
gate matrix as ``[real, imag]`` nested lists, the U-gate angles of 1-qubit
gates, the parameters (each as ``[real]`` or ``[real, imag]`` lists) and the
``mpo`` flag; ``simplified`` keeps the parameters and, for the gates whose
name alone does not define them (any, unitary, mpo, exp, exp1, r, cr), the
U angles or the matrix.  Host-side only: nothing here touches the device.
"""

import json
from typing import Any, Dict, List, Sequence, Tuple

import numpy as np
import torch

from . import gates


def tensor_to_json(a: Any) -> List[Any]:
    if isinstance(a, (float, int, complex, list, tuple)):
        a = np.array(a)
    if isinstance(a, gates.Gate):
        a = a.tensor
    if isinstance(a, torch.Tensor):
        a = a.detach().cpu().numpy()
    a = np.asarray(a)
    if np.iscomplexobj(a):
        return [np.real(a).tolist(), np.imag(a).tolist()]
    return [a.tolist()]


def json_to_tensor(a: Sequence[Any]) -> np.ndarray:
    ar = np.array(a[0])
    if len(a) == 1:
        return ar
    if len(a) != 2:
        raise ValueError("a JSON tensor is [real] or [real, imag]")
    return ar + 1.0j * np.array(a[1])


def get_u_parameter(m: np.ndarray) -> Tuple[float, float, float]:
    """(theta, phi, lbd) of the U gate equal to the 1-qubit unitary m up to
    a global phase (gates.py:485-506): scale m into SU(2), then theta =
    2 acos|U11|, lbd + phi = 2 arg U11, lbd - phi = -2 arg U10."""
    m = np.asarray(m, dtype=np.complex128).reshape(2, 2)
    u = m * np.linalg.det(m) ** (-0.5)
    theta = 2 * np.arccos(min(1.0, abs(u[1, 1])))
    s = 2 * np.angle(u[1, 1])
    d = -2 * np.angle(u[1, 0])
    return float(theta), float((s - d) / 2), float((s + d) / 2)


def _multicontrol_matrix(unitary: Any, ctrl: Sequence[int]) -> np.ndarray:
    u = np.asarray(unitary.tensor if isinstance(unitary, gates.Gate) else unitary, dtype=np.complex128)
    du = int(round(np.sqrt(u.size)))
    u = u.reshape(du, du)
    nc = len(ctrl)
    full = np.eye((1 << nc) * du, dtype=np.complex128)
    cidx = 0
    for c in ctrl:
        cidx = cidx * 2 + int(c)
    full[cidx * du:(cidx + 1) * du, cidx * du:(cidx + 1) * du] = u
    return full


def qir_matrix(d: Dict[str, Any]) -> np.ndarray:
    """The square matrix of one gate record."""
    k = len(d["index"])
    dim = 1 << k
    g = d.get("gatef")
    if g is None:
        m = d["gate"]
    elif not isinstance(g, str):
        m = gates.CONSTANT_GATES[g.n]
    elif g == "multicontrol":
        p = d["parameters"]
        ctrl = p.get("ctrl", 1)
        m = _multicontrol_matrix(p["unitary"], [ctrl] if isinstance(ctrl, int) else list(ctrl))
    else:
        m = getattr(gates, g)(**d.get("parameters", {}))
    if isinstance(m, gates.Gate):
        m = m.tensor
    if isinstance(m, torch.Tensor):
        m = m.detach().cpu().numpy()
    return np.asarray(m, dtype=np.complex128).reshape(dim, dim)


_UNSUPPORTED = ["any", "unitary", "mpo", "exp", "exp1", "r", "cr"]


def qir2json(qir: List[Dict[str, Any]], simplified: bool = False) -> List[Dict[str, Any]]:
    from .circuit import Circuit

    out = []
    for r in qir:
        name = Circuit._qir_name(r)
        if name in Circuit._NON_GATE_QIR:
            continue
        nm = qir_matrix(r)
        nmr, nmi = tensor_to_json(nm.astype(np.complex128))
        uparams = list(get_u_parameter(nm)) if nm.shape == (2, 2) else []
        if r.get("gatef") is None:
            # a gate recorded by its matrix alone travels as ``any``
            name = "any"
            params = {"unitary": [nmr, nmi]}
        else:
            params = {k: tensor_to_json(v) for k, v in r.get("parameters", {}).items()}
        item: Dict[str, Any] = {"name": name, "qubits": [int(q) for q in r["index"]]}
        if not simplified:
            item.update({"matrix": [nmr, nmi], "uparams": uparams, "parameters": params, "mpo": r.get("mpo", False)})
        else:
            if name in _UNSUPPORTED and uparams:
                item["uparams"] = uparams
            elif name in _UNSUPPORTED:
                item["matrix"] = [nmr, nmi]
            if params:
                item["parameters"] = params
            if r.get("mpo"):
                item["mpo"] = r["mpo"]
        out.append(item)
    return out


def json2qir(tcqasm: List[Dict[str, Any]]) -> List[Dict[str, Any]]:
    qir = []
    for d in tcqasm:
        param = {k: json_to_tensor(v) for k, v in d.get("parameters", {}).items()}
        if d["name"] == "multicontrol" and "ctrl" in param:
            param["ctrl"] = [int(c) for c in np.atleast_1d(param["ctrl"])]
        if "matrix" in d:
            gatem = json_to_tensor(d["matrix"])
        elif d["name"] in gates.CONSTANT_GATES:
            gatem = gates.CONSTANT_GATES[d["name"]]
        else:
            gatem = None
        entry = {"gate": gatem, "index": tuple(d["qubits"]), "mpo": d.get("mpo", False), "split": {},
                 "name": d["name"]}
        if d["name"] in gates.CONSTANT_GATES and not param:
            entry["gatef"] = getattr(gates, d["name"], None) or gates.GateF(gates.CONSTANT_GATES[d["name"]], d["name"])
        else:
            entry["gatef"] = d["name"]
            entry["parameters"] = param
        qir.append(entry)
    return qir


def apply_qsim(c: Any, lines: Sequence[str]) -> Any:
    """qsim gate lines (time, name, qubits..., params...) onto ``c``; the
    name table follows the reference's (fs/fsim = iswap(-theta) then
    cphase(-phi), x_1_2 = rx(pi/2), hz_1_2 = wroot, ...)."""

    def conv(x: str) -> Any:
        for f in (int, float):
            try:
                return f(x)
            except ValueError:
                pass
        return x.lower()

    one = {"h": "H", "x": "X", "y": "Y", "z": "Z", "hz_1_2": "WROOT"}
    two = {"cnot": "CNOT", "cx": "CX", "cy": "CY", "cz": "CZ", "is": "ISWAP", "iswap": "ISWAP"}
    half = {"x_1_2": "RX", "y_1_2": "RY", "z_1_2": "RZ"}
    for line in lines:
        if not line.strip():
            continue
        g = tuple(conv(x) for x in line.strip().split(" "))
        nm = g[1]
        if nm in one:
            getattr(c, one[nm])(g[2])
        elif nm in two:
            getattr(c, two[nm])(g[2], g[3])
        elif nm == "s":
            c.PHASE(g[2], theta=np.pi / 2)
        elif nm == "t":
            c.PHASE(g[2], theta=np.pi / 4)
        elif nm in half:
            getattr(c, half[nm])(g[2], theta=np.pi / 2)
        elif nm == "w_1_2":
            c.U(g[2], theta=np.pi / 2, phi=-np.pi / 4, lbd=np.pi / 4)
        elif nm in ("rx", "ry", "rz"):
            getattr(c, nm.upper())(g[2], theta=g[3])
        elif nm in ("fs", "fsim"):
            i, j, theta, phi = g[2:]
            c.ISWAP(i, j, theta=-theta)
            c.CPHASE(i, j, theta=-phi)
        else:
            raise NotImplementedError("qsim gate %s" % nm)
    return c


def dumps(qir: List[Dict[str, Any]], simplified: bool = False) -> str:
    return json.dumps(qir2json(qir, simplified=simplified))


# ----------------------------------------------------------------- OpenQASM 2
# The reference writes and reads OpenQASM through qiskit (abstractcircuit.py:
# 793-840), which this image does not have; the same gate vocabulary of
# qelib1.inc is written and parsed here directly.
_QASM_FIXED = {"i": "id", "x": "x", "y": "y", "z": "z", "h": "h", "s": "s", "t": "t", "sd": "sdg", "td": "tdg",
               "cnot": "cx", "cz": "cz", "cy": "cy", "swap": "swap", "toffoli": "ccx", "fredkin": "cswap"}
_QASM_ROT = {"rx": "rx", "ry": "ry", "rz": "rz", "crx": "crx", "cry": "cry", "crz": "crz", "rxx": "rxx",
             "ryy": "ryy", "rzz": "rzz", "phase": "u1", "cphase": "cu1"}


def _num(v: Any) -> float:
    if isinstance(v, torch.Tensor):
        v = v.detach().cpu()
    return float(np.real(np.asarray(v)))


def qir2qasm(qir: List[Dict[str, Any]], n: int) -> str:
    from .circuit import Circuit

    lines = ["OPENQASM 2.0;", 'include "qelib1.inc";', "qreg q[%d];" % n]
    for d in qir:
        name = Circuit._qir_name(d)
        if name in Circuit._NON_GATE_QIR:
            continue
        qs = ",".join("q[%d]" % int(q) for q in d["index"])
        p = d.get("parameters", {}) if d.get("gatef") is not None else {}
        if d.get("gatef") is not None and name in _QASM_FIXED and not p:
            lines.append("%s %s;" % (_QASM_FIXED[name], qs))
        elif name in _QASM_ROT:
            lines.append("%s(%.17g) %s;" % (_QASM_ROT[name], _num(p.get("theta", 0.0)), qs))
        elif name == "u":
            lines.append("u3(%.17g,%.17g,%.17g) %s;" % (_num(p.get("theta", 0.0)), _num(p.get("phi", 0.0)),
                                                        _num(p.get("lbd", 0.0)), qs))
        elif len(d["index"]) == 1:
            # any other 1-qubit gate: its U angles (the global phase is dropped)
            th, ph, lb = get_u_parameter(qir_matrix(d))
            lines.append("u3(%.17g,%.17g,%.17g) %s;" % (th, ph, lb, qs))
        else:
            raise NotImplementedError("gate %s has no OpenQASM 2 form here" % name)
    return "\n".join(lines) + "\n"


def _qasm_expr(s: str) -> float:
    """Arithmetic of numbers and pi (+ - * / ^, parentheses, unary minus)."""
    import ast

    tree = ast.parse(s.strip().replace("^", "**"), mode="eval")

    def ev(node: Any) -> float:
        if isinstance(node, ast.Expression):
            return ev(node.body)
        if isinstance(node, ast.Constant) and isinstance(node.value, (int, float)):
            return float(node.value)
        if isinstance(node, ast.Name) and node.id == "pi":
            return float(np.pi)
        if isinstance(node, ast.UnaryOp) and isinstance(node.op, (ast.USub, ast.UAdd)):
            v = ev(node.operand)
            return -v if isinstance(node.op, ast.USub) else v
        if isinstance(node, ast.BinOp) and isinstance(node.op, (ast.Add, ast.Sub, ast.Mult, ast.Div, ast.Pow)):
            a, b = ev(node.left), ev(node.right)
            return {ast.Add: a + b, ast.Sub: a - b, ast.Mult: a * b,
                    ast.Div: a / b if isinstance(node.op, ast.Div) else 0.0,
                    ast.Pow: a ** b if isinstance(node.op, ast.Pow) else 0.0}[type(node.op)]
        raise ValueError("unsupported OpenQASM expression: %s" % s)

    return ev(tree)


def qasm2circuit(text: str, cls: Any, circuit_params: Any = None) -> Any:
    """Parse OpenQASM 2 (qelib1 gates, one or more qregs; measure, barrier
    and creg lines are skipped) onto a new circuit of class ``cls``."""
    import re

    body = re.sub(r"//[^\n]*", "", text)
    stmts = [s.strip() for s in body.split(";") if s.strip()]
    regs: Dict[str, int] = {}
    total = 0
    gates_: List[Tuple[str, List[float], List[int]]] = []
    inv_fixed = {v: k for k, v in _QASM_FIXED.items()}
    inv_rot = {v: k for k, v in _QASM_ROT.items()}
    for s in stmts:
        if s.startswith("OPENQASM") or s.startswith("include") or s.startswith("creg") or \
                s.startswith("barrier") or s.startswith("measure"):
            continue
        m = re.match(r"qreg\s+(\w+)\s*\[\s*(\d+)\s*\]$", s)
        if m:
            regs[m.group(1)] = total
            total += int(m.group(2))
            continue
        m = re.match(r"(\w+)\s*(\(([^)]*)\))?\s+(.+)$", s, re.S)
        if not m:
            raise ValueError("cannot parse OpenQASM statement: %s" % s)
        params = [_qasm_expr(x) for x in m.group(3).split(",")] if m.group(3) else []
        qs = []
        for a in m.group(4).split(","):
            mm = re.match(r"\s*(\w+)\s*\[\s*(\d+)\s*\]\s*$", a)
            if not mm:
                raise ValueError("cannot parse OpenQASM operand: %s" % a)
            qs.append(regs[mm.group(1)] + int(mm.group(2)))
        gates_.append((m.group(1).lower(), params, qs))
    cp = dict(circuit_params or {})
    cp.setdefault("nqubits", total)
    c = cls(**cp)
    for name, params, qs in gates_:
        if name in inv_fixed:
            getattr(c, inv_fixed[name])(*qs)
        elif name in ("cu1", "cp"):
            c.cphase(*qs, theta=params[0])
        elif name in ("u1", "p"):
            c.phase(*qs, theta=params[0])
        elif name in inv_rot:
            getattr(c, inv_rot[name])(*qs, theta=params[0])
        elif name in ("u3", "u"):
            c.u(*qs, theta=params[0], phi=params[1], lbd=params[2])
        elif name == "u2":
            c.u(*qs, theta=np.pi / 2, phi=params[0], lbd=params[1])
        elif name == "sx":
            c.rx(*qs, theta=np.pi / 2)
        else:
            raise NotImplementedError("OpenQASM gate %s" % name)
    return c
