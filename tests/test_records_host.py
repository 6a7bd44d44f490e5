"""CPU: circuit records -- gate counting (reference known answer), the JSON
form (round trip of names, qubits, parameters and matrices), qsim text, and
the U-angle decomposition -- checked without a GPU."""

import json

import numpy as np

from oracle import statevector as sv
from tests.golden import reference_kats as K


def test_gate_count_kat():
    import tensorcircuit_gb300 as tc

    c = tc.Circuit(3)
    c.x(0)
    c.h(0)
    c.rx(1, theta=-0.2)
    c.h(2)
    c.multicontrol(0, 1, 2, ctrl=[0, 1], unitary=tc.gates._x_matrix)
    c.toffoli(0, 2, 1)
    c.ccnot(1, 2, 0)
    c.ccx(1, 2, 0)
    k = K.GATE_COUNT
    assert c.gate_count() == k["total"]
    assert c.gate_count("h") == k["h"]
    assert c.gate_count(["ccnot"]) == k["ccnot"]
    assert c.gate_count(["rx", "multicontrol"]) == k["rx_multicontrol"]
    assert c.gate_count_by_condition(lambda qir: qir["index"] == (0,)) == k["on_q0"]
    assert c.gate_summary()["h"] == 2


def _json_circuit(tc):
    # tests/test_circuit.py:1449-1462's circuit
    c = tc.Circuit(3)
    c.h(0)
    c.CNOT(1, 2)
    c.rxx(0, 2, theta=0.3)
    c.crx(0, 1, theta=-0.8)
    c.r(1, theta=1.0, alpha=0.2)
    c.toffoli(0, 2, 1)
    c.ccnot(0, 1, 2)
    c.multicontrol(1, 2, 0, ctrl=[0, 1], unitary=tc.gates._x_matrix)
    c.any(0, unitary=sv.gate_matrix("u", theta=0.4, phi=0.1, lbd=-0.3))
    return c


def test_json_round_trip():
    import tensorcircuit_gb300 as tc
    from tensorcircuit_gb300 import translation as tr

    c = _json_circuit(tc)
    for simplified in (False, True):
        s = c.to_json(simplified=simplified)
        data = json.loads(s)
        assert [d["name"] for d in data] == ["h", "cnot", "rxx", "crx", "r", "toffoli", "toffoli", "multicontrol",
                                             "any"]
        c2 = tc.Circuit.from_json(s)
        assert c2._nqubits == 3
        for a, b in zip(c.to_qir(), c2.to_qir()):
            assert tuple(a["index"]) == tuple(b["index"])
            np.testing.assert_allclose(tr.qir_matrix(a), tr.qir_matrix(b), atol=1e-12)
    full = json.loads(c.to_json())
    np.testing.assert_allclose(tr.json_to_tensor(full[2]["matrix"]), sv.gate_matrix("rxx", theta=0.3), atol=1e-6)


def test_u_parameters_rebuild_the_gate():
    from tensorcircuit_gb300 import translation as tr

    rng = np.random.default_rng(4)
    for _ in range(20):
        th, ph, lb = rng.uniform(-3, 3, 3)
        m = sv.gate_matrix("u", theta=th, phi=ph, lbd=lb) * np.exp(1j * rng.uniform(-3, 3))
        t2, p2, l2 = tr.get_u_parameter(m)
        m2 = sv.gate_matrix("u", theta=t2, phi=p2, lbd=l2)
        # equal up to a global phase
        ph = np.vdot(m2.reshape(-1), m.reshape(-1))
        np.testing.assert_allclose(abs(ph), 2.0, atol=1e-9)


def test_qsim_text(tmp_path):
    import tensorcircuit_gb300 as tc

    f = tmp_path / "c.qsim"
    f.write_text("3\n0 h 0\n0 x_1_2 1\n1 cz 0 1\n2 rz 2 0.25\n3 fs 1 2 0.3 0.2\n4 t 0\n")
    c = tc.Circuit.from_qsim_file(str(f))
    assert c._nqubits == 3
    names = [tc.Circuit._qir_name(d) for d in c.to_qir()]
    assert names == ["h", "rx", "cz", "rz", "iswap", "cphase", "phase"]
    assert c.to_qir()[4]["parameters"]["theta"] == -0.3


def test_openqasm_round_trip():
    import tensorcircuit_gb300 as tc
    from tensorcircuit_gb300 import translation as tr

    c = tc.Circuit(4)
    c.h(0)
    c.sd(1)
    c.cnot(0, 2)
    c.rx(1, theta=0.25)
    c.rzz(2, 3, theta=-0.5)
    c.cphase(0, 3, theta=0.75)
    c.u(2, theta=0.1, phi=0.2, lbd=0.3)
    c.toffoli(0, 1, 3)
    c.wroot(1)
    text = c.to_openqasm()
    assert text.startswith("OPENQASM 2.0;") and "qreg q[4];" in text
    assert "sdg q[1];" in text and "cx q[0],q[2];" in text and "ccx q[0],q[1],q[3];" in text
    c2 = tc.Circuit.from_openqasm(text)
    names = [tc.Circuit._qir_name(d) for d in c2.to_qir()]
    assert names == ["h", "sd", "cnot", "rx", "rzz", "cphase", "u", "toffoli", "u"]
    # every gate matches up to the global phase u3 drops
    for a, b in zip(c.to_qir(), c2.to_qir()):
        ma, mb = tr.qir_matrix(a), tr.qir_matrix(b)
        ph = np.vdot(mb.reshape(-1), ma.reshape(-1)) / ma.shape[0]
        np.testing.assert_allclose(abs(ph), 1.0, atol=1e-9)
        np.testing.assert_allclose(ma, ph * mb, atol=1e-9)


def test_openqasm_parsing_forms():
    import tensorcircuit_gb300 as tc

    text = """OPENQASM 2.0;
include "qelib1.inc";
qreg a[2];
qreg b[1];
creg c[3];
// comment
u2(0, pi) a[0];
cu1(pi/4) a[1],b[0];
rx(-pi/2 + 0.5*2) b[0];
barrier a[0],a[1];
measure a[0] -> c[0];
"""
    c = tc.Circuit.from_openqasm(text)
    assert c._nqubits == 3
    q = c.to_qir()
    assert [d["index"] for d in q] == [(0,), (1, 2), (2,)]
    np.testing.assert_allclose(q[1]["parameters"]["theta"], np.pi / 4)
    np.testing.assert_allclose(q[2]["parameters"]["theta"], -np.pi / 2 + 1.0)
