"""GPU: the specialised (NVRTC-compiled) pass kernels agree with the oracle
and with the generic kernels -- forward states, adjoint cotangents, Pauli
expectations and cotangent seeding."""

import numpy as np
import pytest
import torch

from oracle import statevector as sv
from tests.test_plan_replay import random_gate_list

pytestmark = pytest.mark.gpu


@pytest.fixture
def jit_on(monkeypatch):
    monkeypatch.setenv("TCG_JIT", "1")
    yield


@pytest.fixture
def jit_off(monkeypatch):
    monkeypatch.setenv("TCG_JIT", "0")
    yield


def _state(tc, n, gl):
    from tensorcircuit_gb300 import templates

    c = templates.apply_gate_list(tc.Circuit(n), gl)
    return c, c.state()


@pytest.mark.parametrize("n,ngates,seed", [(7, 50, 20), (13, 120, 21), (16, 100, 22)])
def test_jit_forward_matches_oracle(tc, jit_on, n, ngates, seed):
    from tensorcircuit_gb300 import _native as nat

    rng = np.random.default_rng(seed)
    gl = random_gate_list(n, ngates, rng)
    c, psi = _state(tc, n, gl)
    np.testing.assert_allclose(psi.cpu().numpy(), sv.run_circuit(n, gl), atol=2e-5)
    run = c._engine_state()[3]
    state, log = nat.jit_info(run.plan.handle, 0, 0)
    assert state == 1, log[-2000:]


def test_jit_gradients_match_generic_and_oracle(tc, monkeypatch):
    from tensorcircuit_gb300 import templates

    K = tc.set_backend("pytorch")
    n, nl, B = 12, 3, 5
    terms = templates.tfim_terms(n, -1.0, -0.7)

    def f(p):
        c = templates.apply_hea(tc.Circuit(n), n, nl, p)
        return templates.energy(c, terms)

    rng = np.random.default_rng(31)
    params = torch.tensor(rng.uniform(0, 2 * np.pi, (B, templates.hea_nparams(n, nl))), dtype=torch.float32,
                          device="cuda")
    monkeypatch.setenv("TCG_JIT", "0")
    v0, g0 = K.vvag(f)(params)
    monkeypatch.setenv("TCG_JIT", "1")
    v1, g1 = K.vvag(f)(params)
    np.testing.assert_allclose(v1.cpu().numpy(), v0.cpu().numpy(), atol=1e-6)
    np.testing.assert_allclose(g1.cpu().numpy(), g0.cpu().numpy(), atol=1e-5)
    layout = templates.hea_layout(n, nl)
    ops = [(name, q, {"theta": 0.0}) for name, q, _ in layout]
    ve, ge = sv.value_and_grad_adjoint(n, ops, [k for _, _, k in layout], params[2].cpu().double().numpy(), terms)
    np.testing.assert_allclose(g1[2].cpu().numpy(), ge, atol=2e-5)


def test_jit_dense_gate_gradients(tc, jit_on):
    """Cotangents of dense 2-qubit (and 1-qubit) matrices through the
    specialised adjoint kernel against torch autograd on the oracle-like
    reconstruction: d<psi|Z0|psi>/dU for Haar gates."""
    from tensorcircuit_gb300 import templates

    n = 9
    rng = np.random.default_rng(40)
    gl = templates.brickwall_gate_list(n, 4, 41)
    us = [torch.tensor(p["unitary"], dtype=torch.complex64, device="cuda", requires_grad=True) for _, _, p in gl]
    c = tc.Circuit(n)
    for (name, q, p), u in zip(gl, us):
        c.any(*q, unitary=u)
    e = torch.real(c.expectation_ps(z=[0], x=[n - 1]))
    e.backward()
    # reference: complex128 torch contraction of the same circuit
    psi = torch.zeros([2] * n, dtype=torch.complex128)
    psi.view(-1)[0] = 1
    us64 = [u.detach().cpu().to(torch.complex128).requires_grad_(True) for u in us]
    for (name, q, p), u in zip(gl, us64):
        g = u.reshape(2, 2, 2, 2)
        psi = torch.movedim(torch.tensordot(g, psi, dims=([2, 3], list(q))), [0, 1], list(q))
    zx = psi.clone()
    zx = torch.movedim(torch.tensordot(torch.tensor([[1, 0], [0, -1]], dtype=torch.complex128), zx, dims=([1], [0])), 0, 0)
    zx = torch.movedim(torch.tensordot(torch.tensor([[0, 1], [1, 0]], dtype=torch.complex128), zx, dims=([1], [n - 1])), 0, n - 1)
    er = torch.real(torch.sum(torch.conj(psi) * zx))
    er.backward()
    assert abs(e.item() - er.item()) < 1e-5
    for u, u64 in zip(us, us64):
        np.testing.assert_allclose(u.grad.cpu().numpy(), u64.grad.numpy(), atol=2e-5)


@pytest.mark.parametrize("n", [10, 17])
def test_jit_expectations(tc, jit_on, n):
    rng = np.random.default_rng(n + 100)
    gl = random_gate_list(n, 40, rng)
    c, _ = _state(tc, n, gl)
    psi = sv.run_circuit(n, gl)
    specs = [{"x": [i]} for i in range(n)] + [{"z": [i, i + 1]} for i in range(n - 1)] + \
            [{"y": [0, n - 1], "z": [1]}, {"x": [2], "y": [3]}]
    got = c.expectation_ps_batch(specs).cpu().numpy()
    for t, s in enumerate(specs):
        np.testing.assert_allclose(got[t], sv.expectation_ps(psi, n, **s), atol=2e-5)


def test_jit_refuses_oversized_tables_and_generic_kernels_run(tc, jit_on):
    """One pass holding 1120 rx rotations and 140 Z-rotation runs (a deep
    ansatz on 8 qubits): its operand tables exceed the constant bank, so the
    specialiser reports the failure and the generic kernels compute the
    state, which matches the oracle."""
    from tensorcircuit_gb300 import _native as nat
    from tensorcircuit_gb300 import templates

    n, nl = 8, 140
    params = np.random.default_rng(12).uniform(0, 2 * np.pi, templates.hea_nparams(n, nl))
    c = templates.apply_hea(tc.Circuit(n), n, nl, params)
    psi = c.state()
    run = c._engine_state()[3]
    assert run.plan.npasses == 1
    state, log = nat.jit_info(run.plan.handle, 0, 0)
    assert state == -1 and "constant bank" in log, (state, log[-500:])
    want = sv.run_circuit(n, templates.hea_gate_list(n, nl, params))
    np.testing.assert_allclose(psi.cpu().numpy(), want, atol=5e-5)
