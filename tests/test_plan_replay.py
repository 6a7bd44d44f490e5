"""CPU: replay the engine's device programs (planner output) and check them
against the complex128 oracle -- forward states, adjoint cotangents and
Pauli measurements -- plus the index invariants every kernel launch relies
on.  No GPU needed: plans are built by the native library on the host."""

import numpy as np
import pytest
import torch

from oracle import statevector as sv
from tests.plan_emulator import Replay
from tensorcircuit_gb300 import _native as nat
from tensorcircuit_gb300 import circuit as cmod
from tensorcircuit_gb300 import engine as eng
from tensorcircuit_gb300 import templates

ONE_Q = ["x", "y", "z", "h", "s", "t", "sd", "td", "wroot"]
ONE_Q_P = ["rx", "ry", "rz", "phase"]
TWO_Q = ["cnot", "cz", "swap", "cy", "ox", "oy", "oz"]
TWO_Q_P = ["rxx", "ryy", "rzz", "crx", "cry", "crz", "cphase", "orx", "ory", "orz", "iswap"]


def random_gate_list(n, ngates, rng, allow3=True):
    gl = []
    for _ in range(ngates):
        r = rng.random()
        if r < 0.25:
            gl.append((str(rng.choice(ONE_Q)), (int(rng.integers(n)),), {}))
        elif r < 0.5:
            gl.append((str(rng.choice(ONE_Q_P)), (int(rng.integers(n)),), {"theta": float(rng.uniform(0, 6.3))}))
        elif r < 0.65:
            q = rng.choice(n, 2, replace=False)
            gl.append((str(rng.choice(TWO_Q)), (int(q[0]), int(q[1])), {}))
        elif r < 0.85:
            q = rng.choice(n, 2, replace=False)
            gl.append((str(rng.choice(TWO_Q_P)), (int(q[0]), int(q[1])), {"theta": float(rng.uniform(0, 6.3))}))
        elif r < 0.95 or not allow3:
            q = rng.choice(n, 2, replace=False)
            u = templates.haar_unitary(4, rng)
            gl.append(("any", (int(q[0]), int(q[1])), {"unitary": u}))
        else:
            q = rng.choice(n, 3, replace=False)
            gl.append((str(rng.choice(["toffoli", "fredkin"])), tuple(int(x) for x in q), {}))
    return gl


def build_host(n, gl):
    """Record a gate list on a Circuit and build plan + matrices on the CPU."""
    c = cmod.Circuit(n)
    templates.apply_gate_list(c, gl)
    n_eng = max(n, nat.MIN_QUBITS)
    entry = cmod._build_entry(n_eng, c._ops)
    blocks = []
    if entry.const_np is not None:
        blocks.append(torch.as_tensor(entry.const_np))
    for gkey, idx, E in entry.groups:
        b = cmod._group_block(gkey, c._ops, idx, torch.device("cpu")).to(torch.complex64)
        blocks.append(b.reshape(-1))
    mats = torch.cat(blocks).numpy() if blocks else np.zeros(1, np.complex64)
    return c, entry, mats, n_eng


def oracle_cotangents(n, gl, mu_out):
    """Reference cotangent of every gate matrix entry, d Re<mu|psi_out>."""
    psis = [sv.run_circuit(n, [])]
    for g in gl:
        psis.append(sv.run_circuit(n, [g], psis[-1]))
    out = [None] * len(gl)
    mu = mu_out.astype(np.complex128)
    for i in reversed(range(len(gl))):
        name, q, p = gl[i]
        q = [int(x) % n for x in q]
        m = sv.gate_matrix(name, **p)
        k = len(q)
        # M_ab = sum_rest mu[a, rest] conj(psi_in[b, rest])
        rest = [a for a in range(n) if a not in q]
        mt = np.transpose(mu.reshape([2] * n), q + rest).reshape(1 << k, -1)
        pt = np.transpose(psis[i].reshape([2] * n), q + rest).reshape(1 << k, -1)
        out[i] = mt @ pt.conj().T
        mu = sv.apply_matrix(mu, m.conj().T, q, n)
    return out, mu


@pytest.mark.parametrize("n,ngates,seed", [(6, 40, 0), (7, 60, 1), (9, 80, 2), (13, 60, 3), (14, 70, 4),
                                           (15, 50, 5)])
def test_forward_program_replay_matches_oracle(n, ngates, seed):
    rng = np.random.default_rng(seed)
    gl = random_gate_list(n, ngates, rng)
    c, entry, mats, n_eng = build_host(n, gl)
    assert n_eng == n
    prog = nat.debug_program(entry.plan.handle, 0)
    psi0 = np.zeros(1 << n, np.complex128)
    psi0[0] = 1
    got = Replay(prog, n).forward(psi0, mats)
    want = sv.run_circuit(n, gl)
    np.testing.assert_allclose(got, want, atol=2e-5)


@pytest.mark.parametrize("n,ngates,seed", [(6, 30, 10), (8, 50, 11), (13, 40, 12), (14, 40, 13)])
def test_backward_program_replay_matches_oracle(n, ngates, seed):
    rng = np.random.default_rng(seed)
    gl = random_gate_list(n, ngates, rng, allow3=True)
    c, entry, mats, n_eng = build_host(n, gl)
    psi_out = sv.run_circuit(n, gl)
    mu_out = rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)
    prog = nat.debug_program(entry.plan.handle, 1)
    nout = max(1, mats.size)
    psi_in, mu_in, grads = Replay(prog, n).backward(psi_out, mu_out, mats, nout)
    want_cot, want_mu = oracle_cotangents(n, gl, mu_out)
    e0 = np.zeros(1 << n)
    e0[0] = 1
    np.testing.assert_allclose(psi_in, e0, atol=2e-5)
    np.testing.assert_allclose(mu_in, want_mu, atol=1e-4)
    # compare the cotangents of gates that carry a gradient slot (the random
    # lists never contain the identity, so engine ops and list entries align)
    assert len(entry.gates_c) == len(gl)
    nprot = 0
    for gi, g in enumerate(entry.gates_c):
        kind, qubits, mat_off, grad_off = g[:4]
        if grad_off < 0:
            continue
        cot = want_cot[gi]
        if kind == nat.TCG_GATE_PAULI_ROT:
            # the engine returns dL/dphi for G = cos(phi) I - i sin(phi) P
            nprot += 1
            z = complex(mats[mat_off])
            pm = np.ones((1, 1), np.complex128)
            for code in g[4]:
                pm = np.kron(pm, sv.gate_matrix("ixyz"[code]))
            dg = -z.imag * np.eye(pm.shape[0]) - 1j * z.real * pm
            want = np.sum(np.conj(cot) * dg).real
            np.testing.assert_allclose(grads[grad_off].real, want, atol=1e-3, rtol=1e-4)
            assert grads[grad_off].imag == 0
            continue
        want = np.diag(cot) if kind == nat.TCG_GATE_DIAG else cot.reshape(-1)
        got = grads[grad_off:grad_off + want.size]
        np.testing.assert_allclose(got, want, atol=1e-3, rtol=1e-4)
    assert nprot > 0


@pytest.mark.parametrize("n,seed", [(6, 0), (10, 1), (14, 2)])
def test_measure_program_replay_matches_oracle(n, seed):
    rng = np.random.default_rng(seed)
    psi = rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)
    psi /= np.linalg.norm(psi)
    terms = []
    specs = []
    for _ in range(30):
        k = int(rng.integers(0, 4))
        q = rng.choice(n, min(n, 1 + k + int(rng.integers(0, 3))), replace=False)
        kinds = rng.integers(1, 4, size=len(q))
        x = [int(a) for a, b in zip(q, kinds) if b == 1]
        y = [int(a) for a, b in zip(q, kinds) if b == 2]
        z = [int(a) for a, b in zip(q, kinds) if b == 3]
        specs.append(dict(x=x, y=y, z=z))
        terms.append(eng.pauli_masks(n, x, y, z))
    tp = eng.TermPlan(n, tuple(terms))
    prog = nat.debug_program(tp.handle, 2)
    got = Replay(prog, n).measure(psi, len(terms))
    direct = set()
    for t, (xm, zm) in enumerate(terms):
        if bin(xm).count("1") > 2:
            direct.add(t)
    for t, s in enumerate(specs):
        if t in direct:
            assert got[t] == 0  # handled by the plain kernel, not the program
            continue
        np.testing.assert_allclose(got[t], sv.expectation_ps(psi, n, **s), atol=1e-10)


def test_plan_errors_map_to_reference_exceptions():
    with pytest.raises(AssertionError):
        eng.GatePlan(6, [(nat.TCG_GATE_DENSE, (1, 1), 0, -1)], 16)
    with pytest.raises(ValueError):
        eng.GatePlan(6, [(nat.TCG_GATE_DENSE, (7,), 0, -1)], 4)
    with pytest.raises(NotImplementedError):
        eng.GatePlan(6, [(nat.TCG_GATE_DENSE, (0, 1, 2), 0, 0)], 64)


def test_hea_plan_pass_counts():
    """The n=20 hardware-efficient ansatz fits in a few HBM passes."""
    n, nl = 20, 8
    c = cmod.Circuit(n)
    templates.apply_hea(c, n, nl, np.zeros(templates.hea_nparams(n, nl)))
    entry = cmod._build_entry(n, c._ops)
    assert entry.plan.npasses <= 8
    assert entry.plan.ngates == 312


def test_pauli_rotation_exp1_forms_replay():
    """exp1 on Pauli strings (identity factors, Y factors, half angles) is
    recorded as the Pauli-rotation kind; the replayed forward program and
    its adjoint cotangents match the oracle."""
    X, Y, Z, I2 = (np.array(m, dtype=np.complex128) for m in
                   ([[0, 1], [1, 0]], [[0, -1j], [1j, 0]], [[1, 0], [0, -1]], np.eye(2)))
    gl = [("h", (0,), {}), ("h", (5,), {}),
          ("exp1", (1, 5, 6), {"unitary": np.kron(np.kron(X, I2), Y), "theta": 0.7}),
          ("exp1", (0, 3), {"unitary": np.kron(Y, Y), "theta": 1.3, "half": True}),
          ("exp1", (2, 4, 7), {"unitary": np.kron(np.kron(Z, X), Z), "theta": -0.4}),
          ("exp1", (6, 7, 2, 0), {"unitary": np.kron(np.kron(X, Y), np.kron(X, Y)), "theta": 2.1}),
          ("rzz", (0, 7), {"theta": 0.9}), ("ry", (3,), {"theta": 0.2})]
    n = 8
    c, entry, mats, n_eng = build_host(n, gl)
    kinds = [g[0] for g in entry.gates_c]
    assert kinds.count(nat.TCG_GATE_PAULI_ROT) == 6
    # the first exp1 drops its identity factor
    assert tuple(entry.gates_c[2][1]) == (1, 6)
    prog = nat.debug_program(entry.plan.handle, 0)
    psi0 = np.zeros(1 << n, np.complex128)
    psi0[0] = 1
    np.testing.assert_allclose(Replay(prog, n).forward(psi0, mats), sv.run_circuit(n, gl), atol=2e-6)


@pytest.mark.parametrize("n,nl", [(8, 2), (10, 3)])
def test_zrun_hea_replay_forward_backward(n, nl):
    """The HEA's rzz layers become runs of commuting Z rotations (one
    phase per amplitude); replayed forward states and adjoint cotangents
    match the oracle."""
    rng = np.random.default_rng(n)
    params = rng.uniform(0, 2 * np.pi, templates.hea_nparams(n, nl))
    gl = templates.hea_gate_list(n, nl, params)
    c, entry, mats, n_eng = build_host(n, gl)
    for which in (0, 1):
        prog = nat.debug_program(entry.plan.handle, which)
        kinds = [op.kind for op in prog["ops"]]
        assert 7 in kinds and len(prog["zents"]) >= n - 1
    prog = nat.debug_program(entry.plan.handle, 0)
    psi0 = np.zeros(1 << n, np.complex128)
    psi0[0] = 1
    np.testing.assert_allclose(Replay(prog, n).forward(psi0, mats), sv.run_circuit(n, gl), atol=2e-6)
    psi_out = sv.run_circuit(n, gl)
    mu_out = rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)
    prog_b = nat.debug_program(entry.plan.handle, 1)
    psi_in, mu_in, grads = Replay(prog_b, n).backward(psi_out, mu_out, mats, max(1, mats.size))
    want_cot, want_mu = oracle_cotangents(n, gl, mu_out)
    np.testing.assert_allclose(mu_in, want_mu, atol=1e-4)
    for gi, g in enumerate(entry.gates_c):
        kind, qubits, mat_off, grad_off = g[:4]
        z = complex(mats[mat_off])
        pm = np.ones((1, 1), np.complex128)
        for code in g[4]:
            pm = np.kron(pm, sv.gate_matrix("ixyz"[code]))
        dg = -z.imag * np.eye(pm.shape[0]) - 1j * z.real * pm
        want = np.sum(np.conj(want_cot[gi]) * dg).real
        np.testing.assert_allclose(grads[grad_off].real, want, atol=1e-3, rtol=1e-4)


def _plan_with_opts(n, gates, opts):
    """A plan of the recorded engine gates, built with explicit planner options."""
    lib = nat.load()
    arr = (nat.TcgGate * max(len(gates), 1))()
    for i, g in enumerate(gates):
        kind, qubits, mat_off, grad_off = g[:4]
        arr[i].kind, arr[i].nq, arr[i].mat_off, arr[i].grad_off = kind, len(qubits), mat_off, grad_off
        for j, q in enumerate(qubits):
            arr[i].qubits[j] = q
        if len(g) > 4:
            for j, code in enumerate(g[4]):
                arr[i].pauli[j] = code
    h = nat.ctypes.c_void_p()
    nat.check(lib.tcg_plan_create(n, arr, len(gates), nat.ctypes.byref(opts), nat.ctypes.byref(h)), "plan")
    return h


@pytest.mark.parametrize("zrun_max", [1, 2, 3, 32])
def test_zrun_fusion_width_replay(zrun_max):
    """The Z-rotation fusion width (``tcg_plan_opts.zrun_max``, one of the
    uneven batch's autotuned knobs) only regroups commuting Z rotations: no
    run is longer than the width (none at all for 1), and the replayed
    forward states and adjoint cotangents still match the oracle."""
    n, nl = 10, 3
    rng = np.random.default_rng(40 + zrun_max)
    params = rng.uniform(0, 2 * np.pi, templates.hea_nparams(n, nl))
    gl = templates.hea_gate_list(n, nl, params)
    c, entry, mats, n_eng = build_host(n, gl)
    h = _plan_with_opts(n, entry.gates_c, nat.TcgPlanOpts(tile_bits=0, max_stage_grad_entries=0, zrun_max=zrun_max))
    try:
        for which in (0, 1):
            prog = nat.debug_program(h, which)
            runs = [op.k for op in prog["ops"] if op.kind == 7]
            if zrun_max == 1:
                assert runs == []
            else:
                assert runs and max(runs) <= zrun_max
                assert sum(runs) == len(prog["zents"])
        psi0 = np.zeros(1 << n, np.complex128)
        psi0[0] = 1
        np.testing.assert_allclose(Replay(nat.debug_program(h, 0), n).forward(psi0, mats), sv.run_circuit(n, gl),
                                   atol=2e-6)
        psi_out = sv.run_circuit(n, gl)
        mu_out = rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)
        psi_in, mu_in, grads = Replay(nat.debug_program(h, 1), n).backward(psi_out, mu_out, mats, max(1, mats.size))
        want_cot, want_mu = oracle_cotangents(n, gl, mu_out)
        np.testing.assert_allclose(mu_in, want_mu, atol=1e-4)
        for gi, g in enumerate(entry.gates_c):
            kind, qubits, mat_off, grad_off = g[:4]
            z = complex(mats[mat_off])
            pm = np.ones((1, 1), np.complex128)
            for code in g[4]:
                pm = np.kron(pm, sv.gate_matrix("ixyz"[code]))
            dg = -z.imag * np.eye(pm.shape[0]) - 1j * z.real * pm
            want = np.sum(np.conj(want_cot[gi]) * dg).real
            np.testing.assert_allclose(grads[grad_off].real, want, atol=1e-3, rtol=1e-4)
    finally:
        nat.load().tcg_plan_destroy(h)


def test_zterm_measure_program_replay():
    """Z-string terms (the TFIM's ZZ couplings) are measured as one Walsh-
    Hadamard op per run; the replayed measurement matches the oracle."""
    n = 12
    rng = np.random.default_rng(8)
    psi = rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)
    psi /= np.linalg.norm(psi)
    specs = [dict(z=[i, i + 1]) for i in range(n - 1)] + [dict(x=[i]) for i in range(n)] + \
        [dict(z=[0, 5, 11]), dict(y=[2, 3]), dict(z=[7])]
    terms = [eng.pauli_masks(n, s.get("x", []), s.get("y", []), s.get("z", [])) for s in specs]
    tp = eng.TermPlan(n, tuple(terms))
    prog = nat.debug_program(tp.handle, 2)
    assert any(op.kind == 7 for op in prog["ops"])
    got = Replay(prog, n).measure(psi, len(terms))
    for t, s in enumerate(specs):
        np.testing.assert_allclose(got[t], sv.expectation_ps(psi, n, **s), atol=1e-10)


def _kat_cases():
    from tests.golden import reference_kats as K

    return K.KATS + K.GATE_KATS


@pytest.mark.parametrize("case", _kat_cases(), ids=[c["id"] for c in _kat_cases()])
def test_engine_program_replay_matches_known_answers(case):
    """The reference's known answers through the engine's own gate records,
    planner and device program (replayed on the CPU)."""
    inputs = case.get("inputs")
    if inputs is not None:
        a = np.asarray(inputs, np.complex128).reshape(-1)
        n = int(round(np.log2(a.size)))
    else:
        a = None
        n = case["n"]
    c, entry, mats, n_eng = build_host(n, case["ops"])
    pad = n_eng - n
    psi0 = np.zeros(1 << n_eng, np.complex128)
    if a is None:
        psi0[0] = 1
    else:
        psi0[np.arange(a.size) << pad] = a  # padded qubits are the low index bits
    out = Replay(nat.debug_program(entry.plan.handle, 0), n_eng).forward(psi0, mats)
    psi = out[np.arange(1 << n) << pad]
    q = case["query"]
    if q[0] == "amp":
        got = psi[q[1]].real
    elif q[0] == "amp_complex":
        got = psi[q[1]]
    elif q[0] == "bitstring":
        got = psi[int(q[1], 2)].real
    elif q[0] == "state":
        got = psi
    elif q[0] == "state4x4":
        got = psi.reshape(4, 4)
    elif q[0] == "prob":
        got = np.abs(psi) ** 2
    elif q[0] == "ps":
        kw = dict(q[1])
        if "ps" in kw:
            ps = kw.pop("ps")
            kw = {k: [i for i, code in enumerate(ps) if code == v] for k, v in (("x", 1), ("y", 2), ("z", 3))}
        got = sv.expectation_ps(psi, n, **kw).real
    else:
        kw = {"x": [], "y": [], "z": []}
        for name, idx in q[1]:
            kw[name].extend(idx)
        got = sv.expectation_ps(psi, n, **kw).real
    np.testing.assert_allclose(got, case["expect"], atol=max(case["atol"], 2e-6))
