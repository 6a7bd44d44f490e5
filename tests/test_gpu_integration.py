"""GPU: the reference-side binding shown in INTEGRATION.md (section 3), run
as written on a mock of the reference's qir (dicts whose "gate" has a
``.tensor``, as tensornetwork nodes do), and the probability kernel behind
``Circuit.probability`` with its gradient."""

import os
import re
import types

import numpy as np
import pytest
import torch

from oracle import device as dv
from oracle import statevector as sv

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _snippet_module():
    from tensorcircuit_gb300 import _build

    with open(os.path.join(ROOT, "INTEGRATION.md")) as fh:
        text = fh.read()
    sec = text[text.index("## 3."):]
    code = re.search(r"```python\n(.*?)```", sec, re.S).group(1)
    assert 'ctypes.CDLL("libtcgb300.so")' in code
    code = code.replace('ctypes.CDLL("libtcgb300.so")', "ctypes.CDLL(%r)" % _build.lib_path())
    mod = types.ModuleType("gb300_engine_snippet")
    exec(compile(code, "INTEGRATION.md#3", "exec"), mod.__dict__)
    return mod


def _mock_qir(gl):
    qir = []
    for name, q, p in gl:
        m = sv.gate_matrix(name, **p)
        node = types.SimpleNamespace(tensor=torch.tensor(m.reshape([2] * (2 * len(q)))))
        qir.append({"gate": node, "index": list(q), "name": name})
    return qir


@pytest.mark.parametrize("n", [8, 14])
def test_integration_snippet_wavefunction_from_qir(tc, n):
    from tests.test_plan_replay import random_gate_list

    mod = _snippet_module()
    gl = random_gate_list(n, 80, np.random.default_rng(n))
    psi = mod.wavefunction_from_qir(n, _mock_qir(gl))
    want = dv.run_circuit(n, gl, "cuda")
    assert torch.linalg.vector_norm(psi.to(torch.complex128) - want).item() < 1e-5


def test_probability_kernel_and_gradient(tc):
    """Circuit.probability runs the engine kernel (re^2 + im^2) and is
    differentiable: d/dtheta of sum_a w_a p_a matches central differences of
    the complex128 oracle."""
    from tensorcircuit_gb300 import _native as nat

    n = 10
    w = torch.linspace(-1.0, 1.0, 1 << n, device="cuda")
    gl0 = [("h", (i,), {}) for i in range(n)] + [("cnot", (i, i + 1), {}) for i in range(n - 1)]

    def build(theta):
        c = tc.Circuit(n)
        for name, q, p in gl0:
            getattr(c, name)(*q, **p)
        c.rx(3, theta=theta)
        c.ry(7, theta=0.7 * theta)
        return c

    theta = torch.tensor(0.37, device="cuda", requires_grad=True)
    l0 = nat.load().tcg_launch_count()
    p = build(theta).probability()
    assert nat.load().tcg_launch_count() > l0
    gl = gl0 + [("rx", (3,), {"theta": 0.37}), ("ry", (7,), {"theta": 0.7 * 0.37})]
    want = np.abs(sv.run_circuit(n, gl)) ** 2
    np.testing.assert_allclose(p.detach().cpu().numpy(), want, atol=2e-6)
    (p * w).sum().backward()

    def f(t):
        g = gl0 + [("rx", (3,), {"theta": t}), ("ry", (7,), {"theta": 0.7 * t})]
        return float(np.sum((np.abs(sv.run_circuit(n, g)) ** 2) * w.cpu().numpy().astype(np.float64)))

    fd = (f(0.37 + 1e-4) - f(0.37 - 1e-4)) / 2e-4
    assert abs(theta.grad.item() - fd) < 2e-4, (theta.grad.item(), fd)
