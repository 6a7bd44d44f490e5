"""GPU: circuits rebuilt from records (JSON, inverse, append/prepend) and the
measurement API (post-selection, collapsing measurement, select_gate,
sequential perfect sampling) on pure states, against the oracle and the
reference's known answers."""

import numpy as np
import pytest
import torch

from oracle import densitymatrix as dmo
from oracle import statevector as sv

pytestmark = pytest.mark.gpu


def _np(t):
    return t.detach().cpu().numpy() if isinstance(t, torch.Tensor) else np.asarray(t)


def test_json_round_trip_state(tc):
    """tests/test_circuit.py:1449-1462: from_json(to_json(c)) has c's state."""
    from tests.test_records_host import _json_circuit

    c = _json_circuit(tc)
    for simplified in (False, True):
        c2 = tc.Circuit.from_json(c.to_json(simplified=simplified))
        np.testing.assert_allclose(_np(c.state()), _np(c2.state()), atol=1e-5)


def test_inverse_undoes_the_circuit(tc):
    rng = np.random.default_rng(12)
    n = 5
    c = tc.Circuit(n)
    for _ in range(30):
        k = rng.integers(5)
        a, b = (int(x) for x in rng.choice(n, 2, replace=False))
        if k == 0:
            getattr(c, str(rng.choice(["h", "s", "t", "sd", "td", "x", "y", "wroot"])))(a)
        elif k == 1:
            getattr(c, str(rng.choice(["rx", "ry", "rz", "phase"])))(a, theta=float(rng.uniform(-3, 3)))
        elif k == 2:
            getattr(c, str(rng.choice(["rxx", "rzz", "crx", "cphase", "iswap"])))(a, b, theta=float(rng.uniform(-3, 3)))
        elif k == 3:
            c.u(a, theta=float(rng.uniform(-3, 3)), phi=float(rng.uniform(-3, 3)), lbd=float(rng.uniform(-3, 3)))
        else:
            c.any(a, b, unitary=np.linalg.qr(rng.standard_normal((4, 4)) + 1j * rng.standard_normal((4, 4)))[0])
    psi = c.state()
    ci = c.inverse()
    back = tc.Circuit(n, inputs=psi)
    back.append(ci)
    want = np.zeros(1 << n)
    want[0] = 1.0
    np.testing.assert_allclose(np.abs(_np(back.state())), want, atol=2e-5)


def test_prepend_append_state(tc):
    """tests/test_dmcircuit.py:459-471 on pure states."""
    a = tc.Circuit(2)
    a.H(0)
    b = tc.Circuit(2)
    b.cnot(0, 1)
    b3 = b.append(a).prepend(a)
    want = sv.run_circuit(2, [("h", (0,), {}), ("cnot", (0, 1), {}), ("h", (0,), {})])
    np.testing.assert_allclose(_np(b3.state()), want, atol=1e-6)
    s = b3.state()
    np.testing.assert_allclose(_np(s[0]), _np(s[1]), atol=1e-5)
    c = tc.Circuit(3)
    c.x(2)
    c.append(a, indices=[2, 0])  # a's qubit 0 -> qubit 2
    np.testing.assert_allclose(_np(c.state()), sv.run_circuit(3, [("x", (2,), {}), ("h", (2,), {})]), atol=1e-6)


def test_post_selection_and_measurement(tc):
    n = 3
    c = tc.Circuit(n)
    c.h(0)
    c.cnot(0, 1)
    c.rx(2, theta=0.7)
    r = c.mid_measurement(1, keep=1)
    assert int(r) == 1
    want = sv.run_circuit(n, [("h", (0,), {}), ("cnot", (0, 1), {}), ("rx", (2,), {"theta": 0.7})])
    proj = sv.apply_matrix(want, np.diag([0.0, 1.0]), [1], n)
    np.testing.assert_allclose(_np(c.state()), proj, atol=1e-6)  # unnormalised, like the reference

    # a collapsing measurement: the Bell pair ends in |00> or |11>
    for status, bit in ((0.2, 0), (0.8, 1)):
        c = tc.Circuit(2)
        c.h(0)
        c.cnot(0, 1)
        r = c.cond_measure(0, status=status)
        assert int(r) == bit
        z = float(torch.real(c.expectation_ps(z=[1])))
        np.testing.assert_allclose(z, 1.0 - 2 * bit, atol=1e-5)
        # select_gate: undo the outcome on qubit 1
        c.select_gate(r, [tc.gates.i(), tc.gates.x()], 1)
        np.testing.assert_allclose(float(torch.real(c.expectation_ps(z=[1]))), 1.0, atol=1e-5)


def test_perfect_sampling_pure(tc):
    rng = np.random.default_rng(3)
    n = 4
    th = rng.uniform(-2, 2, n)
    ops = [("ry", (q,), {"theta": th[q]}) for q in range(n)] + [("cnot", (0, 1), {}), ("cnot", (2, 3), {})]
    c = tc.Circuit(n)
    for name, q, p in ops:
        getattr(c, name)(*q, **p)
    psi = sv.run_circuit(n, ops)
    rho = np.outer(psi, psi.conj())
    for _ in range(5):
        status = rng.random(n)
        s, p = c.perfect_sampling(status)
        bits, pw = dmo.measure_sequential(rho, n, list(range(n)), status)
        assert [int(x) for x in _np(s)] == bits
        np.testing.assert_allclose(float(p), pw, atol=1e-5)
        sub = [2, 0]
        s2, p2 = c.measure(*sub, with_prob=True, status=status[:2])
        bits2, pw2 = dmo.measure_sequential(rho, n, sub, status[:2])
        assert [int(x) for x in _np(s2)] == bits2
        np.testing.assert_allclose(float(p2), pw2, atol=1e-5)
