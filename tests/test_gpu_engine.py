"""GPU parity: the engine (through the Circuit API / C ABI) against the
complex128 oracle, the reference's known answers and the committed fixtures.

Tolerances: complex64 state vs complex128 oracle within atol 2e-5 (amplitudes
of normalised states) / rtol 1e-5 on energies and gradients where the
magnitudes allow; sampling is bit-exact under the declared integer CDF."""

import os

import numpy as np
import pytest
import torch

from oracle import statevector as sv
from tests.golden import reference_kats as K

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def _circ(tc, case):
    inputs = case.get("inputs")
    n = case["n"]
    if inputs is not None:
        inp = np.asarray(inputs, dtype=np.complex64).reshape(-1)
        ntot = int(round(np.log2(inp.size)))
        c = tc.Circuit(ntot, inputs=inp)
    else:
        c = tc.Circuit(n)
    from tensorcircuit_gb300 import templates

    templates.apply_gate_list(c, case["ops"])
    return c


@pytest.mark.parametrize("case", K.KATS, ids=[c["id"] for c in K.KATS])
def test_engine_reference_kats(tc, case):
    c = _circ(tc, case)
    q = case["query"]
    if q[0] == "amp":
        got = c.wavefunction()[q[1]].real
    elif q[0] == "bitstring":
        got = c.amplitude(q[1]).real
    elif q[0] == "state":
        got = c.state()
    elif q[0] == "state4x4":
        got = c.state().reshape(4, 4)
    elif q[0] == "prob":
        got = c.probability()
    elif q[0] == "ps":
        got = tc.backend.real(c.expectation_ps(**q[1]))
    elif q[0] == "expect_ops":
        got = tc.backend.real(c.expectation(*[(getattr(tc.gates, name)(), idx) for name, idx in q[1]]))
    got = got.detach().cpu().numpy() if isinstance(got, torch.Tensor) else got
    np.testing.assert_allclose(got, case["expect"], atol=max(case["atol"], 1e-6))


def test_engine_matrix_list_operand(tc):
    c = tc.Circuit(2)
    c.x(1)
    c.crx(1, 0, theta=0.3)
    r = c.expectation([tc.gates._z_matrix, 0])
    np.testing.assert_allclose(r.real.item(), 0.95533645, atol=1e-5)


def test_engine_rxx_equivalence(tc):
    from tensorcircuit_gb300 import templates

    e = K.RXX_EQUIV
    a = templates.apply_gate_list(tc.Circuit(e["n"]), e["ops_a"]).state()
    b = templates.apply_gate_list(tc.Circuit(e["n"]), e["ops_b"]).state()
    np.testing.assert_allclose(a.cpu().numpy(), b.cpu().numpy(), atol=e["atol"])


def test_engine_errors(tc):
    c = tc.Circuit(3)
    with pytest.raises(AssertionError):
        c.cnot(1, 1)
    c.h(0)
    with pytest.raises(ValueError):
        c.expectation_ps(x=[0], z=[0])


@pytest.mark.parametrize("n,ngates,seed", [(6, 60, 0), (9, 120, 1), (12, 200, 2), (13, 150, 3),
                                           (14, 150, 4), (16, 120, 5), (18, 80, 6)])
def test_engine_random_circuits(tc, n, ngates, seed):
    from tests.test_plan_replay import random_gate_list
    from tensorcircuit_gb300 import templates

    rng = np.random.default_rng(seed)
    gl = random_gate_list(n, ngates, rng)
    c = templates.apply_gate_list(tc.Circuit(n), gl)
    got = c.state().cpu().numpy()
    want = sv.run_circuit(n, gl)
    np.testing.assert_allclose(got, want, atol=2e-5)


def test_engine_small_n_padding(tc):
    from tests.test_plan_replay import random_gate_list
    from tensorcircuit_gb300 import templates

    for n in range(1, 6):
        rng = np.random.default_rng(100 + n)
        gl = random_gate_list(n, 25, rng, allow3=n >= 3) if n >= 2 else [("h", (0,), {}), ("rx", (0,), {"theta": 0.4})]
        c = templates.apply_gate_list(tc.Circuit(n), gl)
        np.testing.assert_allclose(c.state().cpu().numpy(), sv.run_circuit(n, gl), atol=2e-5)


def test_c1_plain_statevector_fixture(tc):
    """n=10 HEA, 4 layers, 76 params (seed 1): amplitudes and energy."""
    from tensorcircuit_gb300 import templates

    fx = np.load(os.path.join(HERE, "golden", "c1_hea_n10.npz"))
    n, nl = 10, 4
    c = templates.apply_hea(tc.Circuit(n), n, nl, torch.tensor(fx["params"], dtype=torch.float32))
    psi = c.state().cpu().numpy()
    np.testing.assert_allclose(psi, fx["psi"], atol=2e-6)
    e = templates.energy(c, templates.tfim_terms(n, 1.0, 1.0)).item()
    assert abs(e - float(fx["energy"])) <= 1e-5 * max(1.0, abs(float(fx["energy"])))


def test_c1_gradient_classic_backward(tc):
    from tensorcircuit_gb300 import templates

    fx = np.load(os.path.join(HERE, "golden", "c1_hea_n10.npz"))
    n, nl = 10, 4
    p = torch.tensor(fx["params"], dtype=torch.float32, device="cuda", requires_grad=True)
    c = templates.apply_hea(tc.Circuit(n), n, nl, p)
    e = templates.energy(c, templates.tfim_terms(n, 1.0, 1.0))
    e.backward()
    g = p.grad.cpu().numpy()
    np.testing.assert_allclose(g, fx["grad"], atol=2e-5 * np.max(np.abs(fx["grad"])) + 1e-6)


def _hea_vvag(tc, n, nl, batch, seed, hz=-1.0, hx=-1.0):
    from tensorcircuit_gb300 import templates

    K_ = tc.set_backend("pytorch")
    terms = templates.tfim_terms(n, hz, hx)

    def f(p):
        c = templates.apply_hea(tc.Circuit(n), n, nl, p)
        return templates.energy(c, terms)

    rng = np.random.default_rng(seed)
    params = rng.uniform(0, 2 * np.pi, (batch, templates.hea_nparams(n, nl)))
    v, g = K_.vvag(f, argnums=0, vectorized_argnums=0)(torch.tensor(params, dtype=torch.float32, device="cuda"))
    return params, v.detach().cpu().numpy(), g.detach().cpu().numpy(), terms


def test_vvag_matches_oracle_adjoint(tc):
    from tensorcircuit_gb300 import templates

    n, nl, B = 10, 3, 6
    params, v, g, terms = _hea_vvag(tc, n, nl, B, seed=11)
    layout = templates.hea_layout(n, nl)
    ops = [(name, q, {"theta": 0.0}) for name, q, _ in layout]
    pidx = [k for _, _, k in layout]
    for b in range(B):
        p32 = params[b].astype(np.float32).astype(np.float64)
        ve, ge = sv.value_and_grad_adjoint(n, ops, pidx, p32, terms)
        assert abs(v[b] - ve) <= 1e-5 * max(1.0, abs(ve))
        np.testing.assert_allclose(g[b], ge, atol=1e-5 * max(1.0, np.max(np.abs(ge))))


def test_vvag_c2_shape_vs_finite_differences(tc):
    """The batched value+gradient workload at full size (n=20, 8 layers, 312
    params, batch 64): one row against the oracle's adjoint gradient and a
    few parameters against complex128 central differences (eps=1e-3)."""
    from tensorcircuit_gb300 import templates

    n, nl, B = 20, 8, 64
    params, v, g, terms = _hea_vvag(tc, n, nl, B, seed=2)
    assert v.shape == (B,) and g.shape == (B, 312)
    layout = templates.hea_layout(n, nl)
    ops = [(name, q, {"theta": 0.0}) for name, q, _ in layout]
    pidx = [k for _, _, k in layout]
    p32 = params[5].astype(np.float32).astype(np.float64)
    ve, ge = sv.value_and_grad_adjoint(n, ops, pidx, p32, terms)
    assert abs(v[5] - ve) <= 1e-5 * max(1.0, abs(ve))
    np.testing.assert_allclose(g[5], ge, atol=1e-5 * max(1.0, np.max(np.abs(ge))))
    which = [0, 77, 311]
    gfd = sv.grad_fd(n, ops, pidx, p32, terms, eps=1e-3, which=which)
    # central differences carry O(eps^2) truncation error
    np.testing.assert_allclose(g[5][which], gfd[which], atol=2e-4)


def test_vvag_reference_selfconsistency(tc):
    """tests/test_backends.py:426-476: vvag rows equal value_and_grad, and
    the non-vectorised argnum's gradient is the batch sum."""
    K_ = tc.set_backend("pytorch")
    n, nlayers, batch = K.VVAG["n"], K.VVAG["nlayers"], K.VVAG["batch"]

    def vqe_energy(inputs, param):
        c = tc.Circuit(n, inputs=inputs)
        paramc = K_.cast(param, "complex64")
        for i in range(n):
            c.H(i)
        for j in range(nlayers):
            for i in range(n - 1):
                c.ryy(i, i + 1, theta=paramc[2 * j, i])
            for i in range(n):
                c.rx(i, theta=paramc[2 * j + 1, i])
        e = 0.0
        for i in range(n):
            e += c.expectation((tc.gates.x(), [i]))
        for i in range(n - 1):
            e += c.expectation((tc.gates.z(), [i]), (tc.gates.z(), [(i + 1) % n]))
        return K_.real(e)

    inp = (torch.ones([2 ** n], device="cuda") / 2 ** (n / 2)).to(torch.complex64)
    param = torch.ones([2 * nlayers, n], device="cuda")
    v0, (g00, g01) = K_.value_and_grad(vqe_energy, argnums=(0, 1))(inp, param)
    inps = (torch.ones([batch, 2 ** n], device="cuda") / 2 ** (n / 2)).to(torch.complex64)
    v1, (g10, g11) = K_.vvag(vqe_energy, argnums=(0, 1))(inps, param)
    np.testing.assert_allclose(v1[0].item(), v0.item(), atol=K.VVAG["atol"])
    np.testing.assert_allclose(g10[0].cpu().numpy(), g00.cpu().numpy(), atol=K.VVAG["atol"])
    np.testing.assert_allclose((g11 / batch).cpu().numpy(), g01.cpu().numpy(), atol=K.VVAG["atol"])


@pytest.mark.parametrize("n", [8, 14, 20])
def test_expectations_many_terms(tc, n):
    rng = np.random.default_rng(n)
    from tests.test_plan_replay import random_gate_list
    from tensorcircuit_gb300 import templates

    gl = random_gate_list(n, 60, rng)
    c = templates.apply_gate_list(tc.Circuit(n), gl)
    psi = sv.run_circuit(n, gl)
    specs = []
    for _ in range(25):
        q = rng.choice(n, int(rng.integers(1, min(n, 6))), replace=False)
        kinds = rng.integers(1, 4, size=len(q))
        specs.append({"x": [int(a) for a, b in zip(q, kinds) if b == 1],
                      "y": [int(a) for a, b in zip(q, kinds) if b == 2],
                      "z": [int(a) for a, b in zip(q, kinds) if b == 3]})
    batch = c.expectation_ps_batch(specs).cpu().numpy()
    for t, s in enumerate(specs):
        want = sv.expectation_ps(psi, n, **s)
        one = c.expectation_ps(**s).item()
        np.testing.assert_allclose(one, want, atol=2e-5)
        np.testing.assert_allclose(batch[t], want, atol=2e-5)


def test_sampling_bit_exact_fixture(tc):
    fx = np.load(os.path.join(HERE, "golden", "sample_n12.npz"))
    c = tc.Circuit(12, inputs=fx["psi"])
    got = c.sample(batch=4096, allow_state=True, status=torch.tensor(fx["u"]), format="sample_int")
    np.testing.assert_array_equal(got.cpu().numpy(), fx["idx"])


@pytest.mark.parametrize("n", [6, 13, 20])
def test_sampling_bit_exact_vs_oracle(tc, n):
    rng = np.random.default_rng(50 + n)
    psi = rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)
    psi = (psi / np.linalg.norm(psi)).astype(np.complex64)
    psi[rng.integers(0, 1 << n, size=8)] = 0  # zero-probability entries
    psi = (psi / np.linalg.norm(psi)).astype(np.complex64)
    u = rng.uniform(size=50000).astype(np.float32)
    u[:3] = [0.0, np.float32(1.0) - np.float32(2 ** -24), 0.5]
    c = tc.Circuit(n, inputs=psi)
    got = c.sample(batch=u.size, allow_state=True, status=torch.tensor(u), format="sample_int")
    np.testing.assert_array_equal(got.cpu().numpy(), sv.sample_declared(psi, u))


def test_sample_formats(tc):
    c = tc.Circuit(3)
    c.H(0)
    c.cnot(0, 1)
    u = torch.rand(8)
    for fmt in [None, "sample_int", "sample_bin", "count_vector", "count_tuple", "count_dict_bin",
                "count_dict_int"]:
        r = c.sample(batch=8, allow_state=True, status=u, format=fmt)
        if fmt == "sample_bin":
            assert tuple(r.shape) == (8, 3)
        if fmt == "count_vector":
            assert int(r.sum()) == 8
    single = c.sample(allow_state=True)
    assert len(single) == 2


def test_sample_expectation_ps(tc):
    from tensorcircuit_gb300 import templates

    e = K.SEXPPS_CIRCUIT
    c = templates.apply_gate_list(tc.Circuit(e["n"]), e["ops"])
    exact = c.expectation_ps(**e["term"]).real.item()
    analytic = c.sample_expectation_ps(**e["term"]).item()
    assert abs(exact - analytic) < 1e-5
    shots = c.sample_expectation_ps(**e["term"], shots=e["shots"]).item()
    assert abs(shots - exact) < e["shot_tol"]
    psi = sv.run_circuit(e["n"], e["ops"])
    assert abs(exact - sv.expectation_ps(psi, e["n"], **e["term"]).real) < 1e-5


def test_large_state_properties(tc):
    """n=26 brick wall (512 MiB state): norm preserved, <Z0 Z25> and <X13> in
    range, and forward then inverse circuit returns |0>."""
    from tensorcircuit_gb300 import templates

    n = 26
    gl = templates.brickwall_gate_list(n, 6, 3)
    c = templates.apply_gate_list(tc.Circuit(n), gl)
    psi = c.state()
    assert abs(torch.linalg.norm(psi).item() - 1.0) < 1e-4
    inv = [(name, q, {"unitary": np.asarray(p["unitary"]).conj().T}) for name, q, p in reversed(gl)]
    c2 = templates.apply_gate_list(tc.Circuit(n, inputs=psi), inv)
    back = c2.state()
    assert abs(back[0].item() - 1.0) < 1e-4
    zz = c.expectation_ps(z=[0, n - 1]).real.item()
    assert -1.0001 <= zz <= 1.0001


def test_backend_jit_graph_replay_matches_eager(tc):
    """K.jit(K.vvag(f)) captures a CUDA graph after its warm-up calls; every
    replay must use the new inputs and agree with the eager call."""
    from tensorcircuit_gb300 import templates

    K_ = tc.set_backend("pytorch")
    n, nl, B = 11, 2, 6
    terms = templates.tfim_terms(n, -1.0, -1.0)

    def f(p):
        c = templates.apply_hea(tc.Circuit(n), n, nl, p)
        return templates.energy(c, terms)

    eager = K_.vvag(f)
    jitted = K_.jit(K_.vvag(f))
    rng = np.random.default_rng(9)
    for it in range(7):
        p = torch.tensor(rng.uniform(0, 2 * np.pi, (B, templates.hea_nparams(n, nl))), dtype=torch.float32,
                         device="cuda")
        v1, g1 = jitted(p)
        v0, g0 = eager(p)
        np.testing.assert_allclose(v1.cpu().numpy(), v0.cpu().numpy(), atol=1e-6)
        np.testing.assert_allclose(g1.cpu().numpy(), g0.cpu().numpy(), atol=1e-5)
    ent = list(jitted.cache.values())[0]
    assert ent["graph"] is not None and not ent["failed"]


def test_expectation_batching_follows_requests(tc):
    """Repeated circuits of one structure batch their expectation_ps calls;
    a request that differs from the predicted sequence is still exact."""
    from tensorcircuit_gb300 import templates

    n = 8
    gl = templates.hea_gate_list(n, 2, np.linspace(0.1, 2.0, templates.hea_nparams(n, 2)))
    psi = sv.run_circuit(n, gl)
    seqs = [[{"z": [0, 1]}, {"x": [3]}, {"y": [2], "z": [5]}],
            [{"z": [0, 1]}, {"x": [3]}, {"y": [2], "z": [5]}],
            [{"z": [0, 1]}, {"x": [4]}, {"y": [2], "z": [5]}, {"x": [7]}]]
    for seq in seqs:
        c = templates.apply_gate_list(tc.Circuit(n), gl)
        for s in seq:
            np.testing.assert_allclose(c.expectation_ps(**s).item(), sv.expectation_ps(psi, n, **s), atol=2e-5)


def test_pauli_rotation_forms_state_and_gradient(tc):
    """exp1 on Pauli strings (identity factors dropped, Y factors, half
    angles, far-apart qubits) and the rotation families run as the engine's
    Pauli-rotation kind; states and adjoint gradients match the oracle."""
    X, Y, Z, I2 = (np.array(m, dtype=np.complex128) for m in
                   ([[0, 1], [1, 0]], [[0, -1j], [1j, 0]], [[1, 0], [0, -1]], np.eye(2)))
    n = 9
    spec = [
        ("rx", (0,), {}), ("ry", (8,), {}), ("rz", (4,), {}),
        ("rxx", (1, 7), {}), ("ryy", (2, 3), {}), ("rzz", (0, 8), {}),
        ("exp1", (1, 5, 6), {"unitary": np.kron(np.kron(X, I2), Y), "half": False}),
        ("exp1", (0, 3), {"unitary": np.kron(Y, Y), "half": True}),
        ("exp1", (2, 4, 8), {"unitary": np.kron(np.kron(Z, X), Z)}),
        ("h", (3,), None), ("cnot", (3, 6), None),
        ("exp1", (6, 7, 2, 0), {"unitary": np.kron(np.kron(X, Y), np.kron(X, Y))}),
    ]
    rng = np.random.default_rng(41)
    thetas = rng.uniform(0, 2 * np.pi, len(spec))
    terms = [(0.7, {"x": [0], "z": [5]}), (-1.1, {"y": [3, 8]}), (0.4, {"z": [2]})]

    def build(c, th):
        for i, (name, q, kw) in enumerate(spec):
            if kw is None:
                getattr(c, name)(*q)
            else:
                getattr(c, name)(*q, theta=th[i], **kw)
        return c

    from tensorcircuit_gb300 import templates

    c = build(tc.Circuit(n), torch.tensor(thetas, dtype=torch.float32, device="cuda"))
    assert any(op.kind == "prot" for op in c._ops)
    ops = []
    for i, (name, q, kw) in enumerate(spec):
        ops.append((name, q, {} if kw is None else dict(kw, theta=float(np.float32(thetas[i])))))
    want = sv.run_circuit(n, ops)
    np.testing.assert_allclose(c.state().cpu().numpy(), want, atol=2e-5)

    K = tc.set_backend("pytorch")

    def f(th):
        return templates.energy(build(tc.Circuit(n), th), terms)

    v, g = K.value_and_grad(f)(torch.tensor(thetas, dtype=torch.float32, device="cuda"))
    pidx = [i if kw is not None else None for i, (_, _, kw) in enumerate(spec)]
    ops0 = [(name, q, {} if kw is None else dict(kw, theta=0.0)) for name, q, kw in spec]
    ve, ge = sv.value_and_grad_adjoint(n, ops0, pidx, thetas.astype(np.float32).astype(np.float64), terms)
    assert abs(v.item() - ve) < 1e-5
    np.testing.assert_allclose(g.cpu().numpy(), ge, atol=2e-5)
