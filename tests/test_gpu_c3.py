"""GPU: the large single circuit -- a Haar brick wall of depth 20 (seeded
QR-of-Gaussian 4x4 gates on alternating even/odd pairs), <Z0 Z_{n-1}>,
<X13> and 2^20 samples from seeded uniforms.

n=20: state, expectations and samples against the complex128 oracle.
n=28 (2 GiB state, 270 gates): size-independent properties -- norm, the
inverse circuit returning |0>, the engine's expectations against the same
quantities formed with plain torch ops from the engine's state, and the 2^20
samples bit-exact against the oracle's declared-CDF sampler run on that state.
"""

import numpy as np
import pytest
import torch

from oracle import statevector as sv

pytestmark = pytest.mark.gpu

SHOTS = 1 << 20


def _uniforms():
    return np.random.default_rng(4).random(SHOTS, dtype=np.float32)


def _x_expect_torch(psi, n, q):
    """<X_q> = sum_x conj(psi[x]) psi[x ^ bit(q)], big-endian qubit order."""
    t = psi.reshape(1 << q, 2, -1)
    a = t[:, 0, :].to(torch.complex128)
    b = t[:, 1, :].to(torch.complex128)
    return torch.sum(torch.conj(a) * b).real.item() * 2.0


def _zz_first_last_torch(psi, n):
    """<Z_0 Z_{n-1}> from |psi|^2 in float64 (qubit 0 = most significant bit)."""
    p = (psi.real.double() ** 2 + psi.imag.double() ** 2).reshape(2, -1, 2)
    s = torch.tensor([1.0, -1.0], dtype=torch.float64, device=psi.device)
    return torch.sum(p * s.reshape(2, 1, 1) * s.reshape(1, 1, 2)).item()


def test_brickwall_n20_vs_oracle(tc):
    from tensorcircuit_gb300 import templates

    n = 20
    gl = templates.brickwall_gate_list(n, 20, 3)
    assert len(gl) == 190
    c = templates.apply_gate_list(tc.Circuit(n), gl)
    psi = c.state()
    want = sv.run_circuit(n, gl)
    np.testing.assert_allclose(psi.cpu().numpy(), want, atol=2e-5)
    zz = c.expectation_ps(z=[0, n - 1]).real.item()
    x13 = c.expectation_ps(x=[13]).real.item()
    assert abs(zz - sv.expectation_ps(want, n, z=[0, n - 1]).real) < 1e-5
    assert abs(x13 - sv.expectation_ps(want, n, x=[13]).real) < 1e-5
    u = _uniforms()
    s = c.sample(batch=SHOTS, allow_state=True, status=torch.from_numpy(u), format="sample_int")
    ref = sv.sample_declared(psi.cpu().numpy(), u)
    np.testing.assert_array_equal(s.cpu().numpy(), ref)


def test_brickwall_n28_depth20(tc):
    from tensorcircuit_gb300 import templates

    n = 28
    gl = templates.brickwall_gate_list(n, 20, 3)
    assert len(gl) == 270
    c = templates.apply_gate_list(tc.Circuit(n), gl)
    psi = c.state()
    assert psi.shape == (1 << n,)
    norm = torch.linalg.vector_norm(psi).item()
    assert abs(norm - 1.0) < 1e-4
    zz = c.expectation_ps(z=[0, n - 1]).real.item()
    x13 = c.expectation_ps(x=[13]).real.item()
    assert abs(zz - _zz_first_last_torch(psi, n)) < 1e-5
    assert abs(x13 - _x_expect_torch(psi, n, 13)) < 1e-5
    u = _uniforms()
    s = c.sample(batch=SHOTS, allow_state=True, status=torch.from_numpy(u), format="sample_int")
    s = s.cpu().numpy()
    host = psi.cpu().numpy()
    del c
    ref = sv.sample_declared(host, u)
    np.testing.assert_array_equal(s, ref)
    del host, ref
    # forward then inverse returns |0...0>
    inv = [(name, q, {"unitary": np.asarray(p["unitary"]).conj().T}) for name, q, p in reversed(gl)]
    back = templates.apply_gate_list(tc.Circuit(n, inputs=psi), inv).state()
    assert abs(back[0].item() - 1.0) < 1e-4
    assert torch.linalg.vector_norm(back[1:]).item() < 1e-3
