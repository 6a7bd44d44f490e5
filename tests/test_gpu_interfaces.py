"""GPU: torch_interface and TorchLayer (tensorcircuit/interfaces/torch.py,
tensorcircuit/torchnn.py) on the engine: values and gradients against the
oracle and the reference docstrings' usage."""

import numpy as np
import pytest
import torch

from oracle import statevector as sv

pytestmark = pytest.mark.gpu


def test_torch_interface_docstring_example(tc):
    K = tc.set_backend("pytorch")

    def f(params):
        c = tc.Circuit(1)
        c.rx(0, theta=params[0])
        c.ry(0, theta=params[1])
        return K.real(c.expectation([tc.gates.z(), [0]]))

    f_torch = tc.interfaces.torch_interface(f, jit=True)
    a = torch.ones([2], requires_grad=True)
    b = f_torch(a)
    (b ** 2).backward()
    # <Z> = cos(a0) cos(a1) for ry(a1) rx(a0)|0>
    want = np.cos(1.0) ** 2
    assert abs(b.item() - want) < 1e-6
    g = 2 * want * np.array([-np.sin(1.0) * np.cos(1.0), -np.cos(1.0) * np.sin(1.0)])
    np.testing.assert_allclose(a.grad.numpy(), g, atol=1e-5)
    with torch.no_grad():  # graph-replayed path
        for _ in range(5):
            assert abs(f_torch(torch.ones([2])).item() - want) < 1e-6


def test_torch_layer_forward_backward(tc):
    K = tc.set_backend("pytorch")
    n, nlayers, batch = 6, 2, 3

    def qpred(x, weights):
        c = tc.Circuit(n)
        for i in range(n):
            c.rx(i, theta=x[i])
        for j in range(nlayers):
            for i in range(n - 1):
                c.cnot(i, i + 1)
            for i in range(n):
                c.rx(i, theta=weights[2 * j, i])
                c.ry(i, theta=weights[2 * j + 1, i])
        return K.real(K.stack([c.expectation_ps(x=[i]) for i in range(n)]))

    torch.manual_seed(0)
    ql = tc.torchnn.QuantumNet(qpred, weights_shape=[2 * nlayers, n])
    x = torch.rand(batch, n)
    y = ql(x)
    assert y.shape == (batch, n)
    w = ql.q_weights[0].detach().numpy().astype(np.float64)
    for b in range(batch):
        ops = [("rx", (i,), {"theta": float(x[b, i])}) for i in range(n)]
        for j in range(nlayers):
            ops += [("cnot", (i, i + 1), {}) for i in range(n - 1)]
            for i in range(n):
                ops += [("rx", (i,), {"theta": w[2 * j, i]}), ("ry", (i,), {"theta": w[2 * j + 1, i]})]
        psi = sv.run_circuit(n, ops)
        want = [sv.expectation_ps(psi, n, x=[i]).real for i in range(n)]
        np.testing.assert_allclose(y[b].detach().cpu().numpy(), want, atol=2e-5)
    y.sum().backward()
    g = ql.q_weights[0].grad
    assert g is not None and g.shape == (2 * nlayers, n) and torch.isfinite(g).all()
    # central differences on two weights
    for (j, i) in [(0, 1), (3, 4)]:
        eps = 1e-3
        with torch.no_grad():
            ql.q_weights[0][j, i] += eps
            yp = ql(x).sum().item()
            ql.q_weights[0][j, i] -= 2 * eps
            ym = ql(x).sum().item()
            ql.q_weights[0][j, i] += eps
        assert abs((yp - ym) / (2 * eps) - g[j, i].item()) < 2e-3
