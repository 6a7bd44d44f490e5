"""CPU: the density-matrix oracle pinned to the reference's known answers
(tests/test_dmcircuit.py), and the host logic of ``DMCircuit`` (column-twin
recording, the trace gather's indices and phases) and of the qir tools
(from_qir, inverse, append, prepend) checked without a GPU."""

import numpy as np
import torch

from oracle import densitymatrix as dmo
from oracle import noise as nz
from oracle import statevector as sv
from tests.golden import reference_kats as K

DM = K.DM


def test_oracle_gate_kat():
    rho = dmo.run_dm(3, [("h", (0,), {}), ("rx", (1,), {"theta": np.pi})])
    np.testing.assert_allclose(dmo.expectation_ps(rho, 3, z=[0]).real, DM["gate"]["z0"], atol=DM["gate"]["atol"])
    np.testing.assert_allclose(dmo.expectation_ps(rho, 3, z=[1]).real, DM["gate"]["z1"], atol=DM["gate"]["atol"])


def test_oracle_state_inputs_kat():
    c = DM["state_inputs"]
    w = np.zeros(8)
    w[1] = 1.0
    rho = dmo.run_dm(3, [("cnot", (2, 1), {})], np.outer(w, w.conj()))
    for q, want in zip((1, 2, 0), c["w1_z"]):
        np.testing.assert_allclose(dmo.expectation_ps(rho, 3, z=[q]).real, want, atol=1e-12)
    rho = dmo.run_dm(2, [("y", (0,), {})], np.outer(c["w2"], c["w2"].conj()))
    np.testing.assert_allclose(rho, c["answer"], atol=1e-12)


def test_oracle_dm_inputs_kat():
    c = DM["dm_inputs"]
    rho = dmo.apply_channel(c["rho0"], [c["b1"], c["b2"]], [1], 2)
    np.testing.assert_allclose(rho, c["rho1"], atol=c["atol"])
    rho = dmo.run_dm(2, [("y", (1,), {})], rho)
    np.testing.assert_allclose(rho, c["rho2"], atol=c["atol"])


def test_oracle_depolarizing_kat():
    rho = dmo.run_dm(2, [("h", (0,), {}), ("channel", (1,), nz.depolarizing(0.1, 0.1, 0.1))])
    np.testing.assert_allclose(rho, DM["depolarizing"]["ans"], atol=DM["depolarizing"]["atol"])


def _noise_param(p):
    rho = dmo.run_dm(2, [("x", (1,), {}), ("channel", (1,), nz.depolarizing(p, p, p))])
    return dmo.expectation_ps(rho, 2, z=[1]).real


def _ad_channel(p, theta):
    rho = dmo.run_dm(3, [("rx", (1,), {"theta": theta}), ("channel", (1,), nz.depolarizing(p, 0.2 * p, p)),
                         ("h", (0,), {})])
    return dmo.expectation_ps(rho, 3, z=[1]).real


def _mult_kraus(theta):
    c = DM["mult_qubit_kraus"]
    rho = dmo.run_dm(3, [("h", (0,), {}), ("rx", (1,), {"theta": theta}),
                         ("channel", (0, 1), [c["xx"], c["yz"]]), ("h", (1,), {})])
    return np.sum(rho).real


def test_oracle_gradient_kats():
    c = DM["noise_param_ad"]
    eps = 1e-5
    np.testing.assert_allclose(_noise_param(c["p"]), c["value"], atol=c["atol"])
    np.testing.assert_allclose((_noise_param(c["p"] + eps) - _noise_param(c["p"] - eps)) / (2 * eps), c["grad"],
                               atol=c["atol"])
    c = DM["ad_channel"]
    np.testing.assert_allclose(_ad_channel(c["p"], c["theta"]), c["value"], atol=c["atol"])
    g = (_ad_channel(c["p"] + eps, c["theta"]) - _ad_channel(c["p"] - eps, c["theta"])) / (2 * eps)
    np.testing.assert_allclose(g, c["grad"], atol=c["atol"])
    c = DM["mult_qubit_kraus"]
    g = (_mult_kraus(c["theta"] + eps) - _mult_kraus(c["theta"] - eps)) / (2 * eps)
    np.testing.assert_allclose(g, c["grad"], atol=c["atol"])


def test_oracle_misc_kats():
    rho = dmo.run_dm(2, [("h", (0,), {}), ("channel", (1,), [np.sqrt(0.5) * np.eye(2), np.sqrt(0.5) * sv.X])],
                     0.25 * np.eye(4))
    np.testing.assert_allclose(dmo.expectation_ps(rho, 2, z=[0]).real, DM["inputs_pipeline"]["value"], atol=1e-12)
    rho = dmo.run_dm(3, [("h", (1,), {}), ("channel", (0,), nz.depolarizing(0.05, 0.02, 0.02)),
                         ("toffoli", (1, 0, 2), {})])
    np.testing.assert_allclose(dmo.expectation_ps(rho, 3, z=[2]).real, DM["multicontrol"]["value"], atol=1e-6)
    rho = dmo.run_dm(2, [("x", (0,), {}), ("channel", (0,), nz.depolarizing(0.1, 0.1, 0.1)), ("cnot", (0, 1), {})])
    np.testing.assert_allclose(dmo.expectation_ps(rho, 2, z=[1]).real, DM["to_circuit"]["dm"], atol=1e-12)
    ops = [("h", (i,), {}) for i in range(3)] + [("channel", (i,), nz.amplitude_damping(0.1, 1.0)) for i in range(3)]
    rho = dmo.run_dm(3, ops)
    bits, p = dmo.measure_sequential(rho, 3, [0, 1, 2], DM["perfect_sampling"]["status"])
    assert bits == DM["perfect_sampling"]["bits"]
    np.testing.assert_allclose(p, DM["perfect_sampling"]["p"], atol=DM["perfect_sampling"]["atol"])
    rho = dmo.run_dm(2, [("h", (0,), {}), ("cnot", (0, 1), {})])
    np.testing.assert_allclose(rho[3, 3].real, DM["amplitude"]["before"], atol=1e-12)
    rho = dmo.apply_channel(rho, nz.depolarizing(0.2, 0.0, 0.0), [1], 2)
    np.testing.assert_allclose(rho[3, 3].real, DM["amplitude"]["after"], atol=1e-12)


def test_trace_gather_matches_oracle():
    from tensorcircuit_gb300 import engine as eng
    from tensorcircuit_gb300.densitymatrix import _trace_index

    n = 4
    rng = np.random.default_rng(3)
    a = rng.standard_normal((16, 16)) + 1j * rng.standard_normal((16, 16))
    rho = a @ a.conj().T
    rho /= np.trace(rho)
    v = torch.as_tensor(rho.reshape(-1))
    for kw in (dict(z=[0]), dict(x=[1]), dict(y=[2]), dict(x=[0], y=[1], z=[3]), dict(y=[0, 3]), dict(y=[1, 2], x=[3])):
        xm, zm = eng.pauli_masks(n, kw.get("x", []), kw.get("y", []), kw.get("z", []))
        flat, phase = _trace_index(n, xm, zm, torch.device("cpu"))
        got = complex(torch.sum(v[flat] * phase.to(torch.complex128)))
        np.testing.assert_allclose(got, dmo.expectation_ps(rho, n, **kw), atol=1e-12)


def test_column_twin_recording():
    import tensorcircuit_gb300 as tc

    c = tc.DMCircuit(3)
    c.H(0)
    c.rx(1, theta=0.3)
    c.ry(2, theta=0.4)
    c.rzz(0, 2, theta=0.5)
    c.cnot(0, 1)
    ops = c._ops
    assert len(ops) == 10
    pairs = list(zip(ops[0::2], ops[1::2]))
    for a, b in pairs:
        assert b.qubits == tuple(q + 3 for q in a.qubits)
    assert pairs[0][1].name == "h*"
    assert pairs[1][1].conj is True      # rx: X has no Y factor -> rotation by -phi
    assert pairs[2][1].conj is False     # ry is real: the same rotation
    assert pairs[3][1].conj is True      # rzz
    assert len(c.to_qir()) == 5


def test_qir_tools():
    import tensorcircuit_gb300 as tc

    c = tc.Circuit(3)
    c.H(0)
    c.rx(1, theta=0.5)
    c.s(2)
    c.cnot(0, 1)
    c.rzz(0, 2, theta=-1.0)
    c.iswap(1, 2)
    ci = c.inverse()
    names = [tc.Circuit._qir_name(d) for d in ci.to_qir()]
    # s is applied as its adjoint matrix under its own name, as the reference does
    assert names == ["iswap", "rzz", "cnot", "s", "rx", "h"]
    q = ci.to_qir()
    assert q[0]["parameters"]["theta"] == -1.0 and q[1]["parameters"]["theta"] == 1.0
    assert q[3].get("gatef") is None
    np.testing.assert_allclose(q[3]["gate"], np.diag([1, -1j]), atol=1e-12)
    c2 = tc.Circuit.from_qir(c.to_qir())
    assert c2._nqubits == 3 and [tc.Circuit._qir_name(d) for d in c2.to_qir()] == \
        [tc.Circuit._qir_name(d) for d in c.to_qir()]
    # tests/test_dmcircuit.py:459-471: prepend / append order
    a = tc.Circuit(2)
    a.H(0)
    b = tc.Circuit(2)
    b.cnot(0, 1)
    b2 = b.append(a)
    b3 = b2.prepend(a)
    assert [d["name"] for d in b3.to_qir()] == ["h", "cnot", "h"]
    assert c.gate_count(["rx", "rzz"]) == 2 and c.gate_count("h") == 1
