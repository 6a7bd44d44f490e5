"""GPU: the engine at n=30 (an 8 GiB state, 16 GiB with the adjoint's
cotangent) checked through size-independent, closed-form properties -- the
oracle cannot hold these states.

rx(theta_i) on every qubit gives a product state with <Z_i> = cos theta_i,
<Y_i> = -sin theta_i, <Z_i Z_j> = cos theta_i cos theta_j; a CNOT ladder and
its inverse, or the rx layer and its inverse, return to known states;
per-qubit sample frequencies follow (1 - cos theta_i) / 2; and
d sum_i <Z_i> / d theta_i = -sin theta_i through the adjoint sweep."""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

N = 30


def _thetas():
    return np.random.default_rng(30).uniform(0.2, 2.9, N)


def test_n30_product_state_and_inverse(tc):
    th = _thetas()
    c = tc.Circuit(N)
    for i in range(N):
        c.rx(i, theta=float(th[i]))
    for i in (0, 7, 29):
        np.testing.assert_allclose(float(torch.real(c.expectation_ps(z=[i]))), np.cos(th[i]), atol=2e-5)
        np.testing.assert_allclose(float(torch.real(c.expectation_ps(y=[i]))), -np.sin(th[i]), atol=2e-5)
    np.testing.assert_allclose(float(torch.real(c.expectation_ps(z=[3, 28]))), np.cos(th[3]) * np.cos(th[28]),
                               atol=2e-5)
    # an entangling ladder and its inverse leave the product state unchanged
    for i in range(N - 1):
        c.cnot(i, i + 1)
    for i in reversed(range(N - 1)):
        c.cnot(i, i + 1)
    np.testing.assert_allclose(float(torch.real(c.expectation_ps(z=[12]))), np.cos(th[12]), atol=2e-5)
    # and the inverse rotations return to |0...0>
    for i in range(N):
        c.rx(i, theta=float(-th[i]))
    np.testing.assert_allclose(abs(complex(c.amplitude("0" * N))), 1.0, atol=1e-4)


def test_n30_sampling_marginals(tc):
    th = _thetas()
    c = tc.Circuit(N)
    for i in range(N):
        c.rx(i, theta=float(th[i]))
    shots = 1 << 15
    s = c.sample(batch=shots, allow_state=True, format="sample_bin",
                 random_generator=torch.Generator(device="cuda").manual_seed(1))
    freq = s.to(torch.float64).mean(0).cpu().numpy()
    p1 = (1 - np.cos(th)) / 2
    sigma = np.sqrt(p1 * (1 - p1) / shots)
    assert np.all(np.abs(freq - p1) < 6 * sigma + 1e-9)


def test_n30_adjoint_gradient(tc):
    K_ = tc.set_backend("pytorch")
    th = _thetas()

    def f(t):
        c = tc.Circuit(N)
        for i in range(N):
            c.rx(i, theta=t[i])
        e = 0.0
        for i in range(0, N, 5):
            e = e + torch.real(c.expectation_ps(z=[i]))
        return e

    v, g = K_.value_and_grad(f)(torch.as_tensor(th, dtype=torch.float32, device="cuda"))
    want = np.zeros(N)
    want[0::5] = -np.sin(th[0::5])
    np.testing.assert_allclose(float(v), np.sum(np.cos(th[0::5])), atol=1e-4)
    np.testing.assert_allclose(g.cpu().numpy(), want, atol=1e-4)
