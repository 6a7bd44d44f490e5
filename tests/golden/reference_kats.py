"""Known-answer cases transcribed from the reference's own test-suite.

Each case gives the circuit (gate list in the oracle's ``(name, qubits,
params)`` form, plus optional ``inputs``), the queried quantity and the value
the reference's test asserts, with the reference file:line it comes from.
The values are copied from the assertions in those test files (read as
text; the reference cannot be imported in this environment).  Both the CPU
oracle (tests/test_oracle_kats.py) and the GPU engine
(tests/test_gpu_engine.py, test_engine_reference_kats) are checked
against them.
"""

import numpy as np

S2 = 1 / np.sqrt(2)

KATS = [
    # tests/test_circuit.py:21-44 -- gate leg order / big-endian layout
    dict(id="unitary01_amp2", src="tests/test_circuit.py:23-28", n=2,
         ops=[("any", (0, 1), {"unitary": np.arange(16).reshape(4, 4)})],
         query=("amp", 2), expect=8.0, atol=0.0),
    dict(id="unitary10_amp2", src="tests/test_circuit.py:29-36", n=2,
         ops=[("any", (1, 0), {"unitary": np.arange(16).reshape(4, 4)})],
         query=("amp", 2), expect=4.0, atol=0.0),
    dict(id="unitary0_amp2", src="tests/test_circuit.py:37-42", n=2,
         ops=[("any", (0,), {"unitary": np.arange(4).reshape(2, 2)})],
         query=("amp", 2), expect=2.0, atol=0.0),
    # tests/test_circuit.py:47-53 -- amplitude
    dict(id="x_amp10", src="tests/test_circuit.py:49-51", n=2, ops=[("x", (0,), {})],
         query=("bitstring", "10"), expect=1.0, atol=1e-7),
    dict(id="x_cnot_amp11", src="tests/test_circuit.py:49-53", n=2,
         ops=[("x", (0,), {}), ("cnot", (0, 1), {})],
         query=("bitstring", "11"), expect=1.0, atol=1e-7),
    # tests/test_circuit.py:64-68 -- iswap on identity inputs (2n-leg inputs)
    dict(id="iswap_eye", src="tests/test_circuit.py:64-68", n=2, inputs=np.eye(4).reshape(-1),
         ops=[("iswap", (0, 1), {})], query=("state4x4",),
         expect=np.array([[1, 0, 0, 0], [0, 0, 1j, 0], [0, 1j, 0, 0], [0, 0, 0, 1]]), atol=1e-5),
    # tests/test_circuit.py:71-77 -- controlled rotation
    dict(id="crx_z0", src="tests/test_circuit.py:71-77", n=2,
         ops=[("x", (1,), {}), ("crx", (1, 0), {"theta": 0.3})],
         query=("expect_ops", [("z", [0])]), expect=0.95533645, atol=1e-5),
    # tests/test_circuit.py:80-84 -- adjoint gate
    dict(id="x_sd_state", src="tests/test_circuit.py:80-84", n=1,
         ops=[("x", (0,), {}), ("sd", (0,), {})], query=("state",),
         expect=np.array([0.0, -1.0j]), atol=1e-6),
    # tests/test_circuit.py:405-413 -- X (x) Y on identity inputs
    dict(id="xy_eye", src="tests/test_circuit.py:405-413", n=2, inputs=np.eye(4).reshape(-1),
         ops=[("x", (0,), {}), ("y", (1,), {})], query=("state4x4",),
         expect=np.kron(np.array([[0, 1], [1, 0]]), np.array([[0, -1j], [1j, 0]])), atol=1e-4),
    # tests/test_circuit.py:416-429 -- expectation_ps forms
    dict(id="ps_zz", src="tests/test_circuit.py:418-421", n=2, ops=[("x", (0,), {})],
         query=("ps", dict(z=[0, 1])), expect=-1.0, atol=1e-5),
    dict(id="ps_xz", src="tests/test_circuit.py:423-426", n=2, ops=[("h", (0,), {})],
         query=("ps", dict(z=[1], x=[0])), expect=1.0, atol=1e-5),
    dict(id="ps_codes", src="tests/test_circuit.py:427-428", n=2, ops=[("h", (0,), {})],
         query=("ps", dict(ps=[1, 3])), expect=1.0, atol=1e-5),
    dict(id="ps_overrides", src="tests/test_circuit.py:429", n=2, ops=[("h", (0,), {})],
         query=("ps", dict(z=[1, 2], ps=[1, 3])), expect=1.0, atol=1e-5),
    # tests/test_circuit.py:432-440 -- probability
    dict(id="hh_prob", src="tests/test_circuit.py:432-440", n=2,
         ops=[("h", (0,), {}), ("h", (1,), {})], query=("prob",),
         expect=np.array([1, 1, 1, 1]) / 4, atol=1e-5),
    # tests/test_circuit.py:1278-1281 -- Y sign
    dict(id="y_sign", src="tests/test_circuit.py:1278-1281", n=1, inputs=S2 * np.array([-1, 1.0j]),
         ops=[], query=("ps", dict(y=[0])), expect=-1.0, atol=1e-5),
    # tests/test_circuit.py:1373-1381 -- negative indices
    dict(id="minus_x0", src="tests/test_circuit.py:1373-1377", n=3,
         ops=[("h", (-2,), {}), ("h", (0,), {})], query=("ps", dict(x=[0])), expect=1.0, atol=1e-5),
    dict(id="minus_x1", src="tests/test_circuit.py:1378", n=3,
         ops=[("h", (-2,), {}), ("h", (0,), {})], query=("ps", dict(x=[1])), expect=1.0, atol=1e-5),
    dict(id="minus_xm1", src="tests/test_circuit.py:1379", n=3,
         ops=[("h", (-2,), {}), ("h", (0,), {})], query=("ps", dict(x=[-1])), expect=0.0, atol=1e-5),
    dict(id="minus_zm2", src="tests/test_circuit.py:1380", n=3,
         ops=[("h", (-2,), {}), ("h", (0,), {})], query=("ps", dict(z=[-2])), expect=0.0, atol=1e-5),
    # tests/test_circuit.py:1384-1390 -- Y expectation on a given input
    dict(id="sexpps_y", src="tests/test_circuit.py:1385-1390", n=1, inputs=S2 * np.array([1.0, 1.0j]),
         ops=[], query=("ps", dict(y=[0])), expect=1.0, atol=1e-5),
    # abstractcircuit.py docstring of expectation_ps (:1221-1225)
    dict(id="doc_xh", src="tensorcircuit/abstractcircuit.py:1221-1225", n=2,
         ops=[("x", (0,), {}), ("h", (1,), {})], query=("ps", dict(x=[1], z=[0])), expect=-1.0, atol=1e-5),
    # tests/test_circuit.py:240-245 -- <Z0> after H
    dict(id="h_z0", src="tests/test_circuit.py:240-245", n=2, ops=[("h", (0,), {})],
         query=("expect_ops", [("z", [0])]), expect=0.0, atol=1e-7),
    # tests/test_circuit.py:319-323 -- one-qubit state
    dict(id="single_h_state", src="tests/test_circuit.py:319-323", n=1, ops=[("h", (0,), {})],
         query=("state",), expect=np.array([1, 1]) * S2, atol=1e-4),
    # tests/test_circuit.py:371-390 -- X on given input states
    dict(id="inputs_11_x_z0", src="tests/test_circuit.py:372-375", n=2, inputs=np.array([0.0, 0.0, 0.0, 1.0]),
         ops=[("x", (0,), {})], query=("expect_ops", [("z", [0])]), expect=1.0, atol=0.0),
    dict(id="inputs_10_x_z0", src="tests/test_circuit.py:376-379", n=2, inputs=np.array([0.0, 0.0, 1.0, 0.0]),
         ops=[("x", (0,), {})], query=("expect_ops", [("z", [0])]), expect=1.0, atol=0.0),
    dict(id="inputs_00_x_z0", src="tests/test_circuit.py:380-383", n=2, inputs=np.array([1.0, 0.0, 0.0, 0.0]),
         ops=[("x", (0,), {})], query=("expect_ops", [("z", [0])]), expect=-1.0, atol=0.0),
    dict(id="inputs_plus_x_z0", src="tests/test_circuit.py:384-390", n=2, inputs=np.array([S2, 0.0, S2, 0.0]),
         ops=[("x", (0,), {})], query=("expect_ops", [("z", [0])]), expect=0.0, atol=1e-4),
    # tests/test_circuit.py:584-589 -- state after x(1), cnot(0, 1)
    dict(id="x1_cnot_state", src="tests/test_circuit.py:587-589", n=2,
         ops=[("x", (1,), {}), ("cnot", (0, 1), {})], query=("state",),
         expect=np.array([0, 1.0, 0, 0]), atol=1e-5),
    # tests/test_circuit.py:707-727 -- a circuit rebuilt from its qir and the
    # same qir appended once more: <Z1> of the doubled gate list
    dict(id="toqir_append_z1", src="tests/test_circuit.py:707-727", n=3,
         ops=[("h", (0,), {}), ("rx", (1,), {"theta": 0.7}),
              ("exp1", (0, 1), {"unitary": np.diag([1.0, -1.0, -1.0, 1.0]), "theta": -0.2})] * 2,
         query=("expect_ops", [("z", [1])]), expect=0.202728, atol=1e-5),
    # tests/test_templates.py:17-26 -- any_measurements (codes 1 = X, 3 = Z, 0 = I) after H on both
    dict(id="anymeas_xx", src="tests/test_templates.py:17-23", n=2, ops=[("h", (0,), {}), ("h", (1,), {})],
         query=("ps", dict(x=[0, 1])), expect=1.0, atol=1e-5),
    dict(id="anymeas_z0", src="tests/test_templates.py:24-26", n=2, ops=[("h", (0,), {}), ("h", (1,), {})],
         query=("ps", dict(z=[0])), expect=0.0, atol=1e-5),
    # tests/test_templates.py:30-39 -- local measurements in bases Z, Z, X
    dict(id="localmeas_z0", src="tests/test_templates.py:30-39", n=3,
         ops=[("x", (0,), {}), ("cnot", (0, 1), {}), ("h", (-1,), {})],
         query=("ps", dict(z=[0])), expect=-1.0, atol=1e-5),
    dict(id="localmeas_z1", src="tests/test_templates.py:30-39", n=3,
         ops=[("x", (0,), {}), ("cnot", (0, 1), {}), ("h", (-1,), {})],
         query=("ps", dict(z=[1])), expect=-1.0, atol=1e-5),
    dict(id="localmeas_x2", src="tests/test_templates.py:30-39", n=3,
         ops=[("x", (0,), {}), ("cnot", (0, 1), {}), ("h", (-1,), {})],
         query=("ps", dict(x=[2])), expect=1.0, atol=1e-5),
]

# Gate conventions from the reference's gate tests (tests/test_gates.py).
# Checked on the oracle and, through the engine's planner and the CPU replay
# of its device programs, on the engine's own program (tests/
# test_oracle_kats.py, tests/test_plan_replay.py).
_WROOT = np.array([[1, -np.sqrt(1j)], [np.sqrt(-1j), 1]]) * S2  # tensorcircuit/gates.py:39-43
_OCX = np.eye(8, dtype=np.complex128)  # ocontrolled(cx) on (1, 0, 2): CX on (0, 2) when qubit 1 is 0
_OCX[:4, :4] = np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0]])
GATE_KATS = [
    dict(id="phase_h", src="tests/test_gates.py:18-22", n=1,
         ops=[("h", (0,), {}), ("phase", (0,), {"theta": np.pi / 2})],
         query=("amp_complex", 1), expect=0.7071j, atol=1e-4),
    dict(id="cu_block", src="tests/test_gates.py:25-31", n=2, inputs=np.eye(4).reshape(-1),
         ops=[("cu", (0, 1), {"theta": np.pi / 2, "phi": -np.pi / 4, "lbd": np.pi / 4})],
         query=("state4x4",),
         expect=np.block([[np.eye(2), np.zeros((2, 2))], [np.zeros((2, 2)), _WROOT]]), atol=1e-5),
    dict(id="fsim", src="tests/test_gates.py:61-77", n=2, inputs=np.eye(4).reshape(-1),
         ops=[("iswap", (0, 1), {"theta": -0.2}), ("cphase", (0, 1), {"theta": -0.3})],
         query=("state4x4",),
         expect=np.array([[1.0, 0, 0, 0], [0, 0.95105654, -0.309017j, 0], [0, -0.309017j, 0.95105654, 0],
                          [0, 0, 0, 0.9553365 - 0.29552022j]]), atol=1e-5),
    dict(id="exp_zz", src="tests/test_gates.py:80-90", n=2,
         ops=[("exp", (0, 1), {"unitary": np.diag([1.0, -1.0, -1.0, 1.0]), "theta": np.pi / 2})],
         query=("amp_complex", 0), expect=-1j, atol=1e-6),
    dict(id="any_eye_z0", src="tests/test_gates.py:93-96", n=2, ops=[("any", (0,), {"unitary": np.eye(2)})],
         query=("expect_ops", [("z", [0])]), expect=1.0, atol=1e-7),
    dict(id="ocx_z2", src="tests/test_gates.py:111-124", n=3,
         ops=[("x", (0,), {}), ("any", (1, 0, 2), {"unitary": _OCX})],
         query=("expect_ops", [("z", [2])]), expect=-1.0, atol=1e-5),
]

# tests/test_circuit.py:1392-1406 -- a 4-qubit circuit whose sampled and
# exact Pauli expectations must agree (exact within 1e-5, 81920 shots
# within 0.01); the value itself is not asserted by the reference.
SEXPPS_CIRCUIT = dict(
    src="tests/test_circuit.py:1392-1406", n=4,
    ops=[("h", (0,), {}), ("cnot", (0, 1), {}), ("rx", (1,), {"theta": 0.3}), ("rz", (2,), {"theta": -1.2}),
         ("ccnot", (2, 3, 1), {}), ("rzz", (0, 3), {"theta": 0.5}), ("ry", (3,), {"theta": 2.2}),
         ("s", (1,), {}), ("td", (2,), {})],
    term=dict(x=[1], y=[0], z=[2, 3]), shots=81920, shot_tol=0.01,
)

# tests/test_gates.py:147-156 -- rxx/ryy/rzz equal exp1 with half angle
RXX_EQUIV = dict(
    src="tests/test_gates.py:147-156", n=3,
    ops_a=[("rxx", (0, 1), {"theta": 1.0}), ("ryy", (0, 2), {"theta": 0.5}), ("rzz", (0, 1), {"theta": -0.5})],
    ops_b=[("exp1", (0, 1), {"theta": 0.5, "unitary": np.kron([[0, 1], [1, 0]], [[0, 1], [1, 0]])}),
           ("exp1", (0, 2), {"theta": 0.25, "unitary": np.kron([[0, -1j], [1j, 0]], [[0, -1j], [1j, 0]])}),
           ("exp1", (0, 1), {"theta": -0.25, "unitary": np.diag([1, -1, -1, 1])})],
    atol=1e-5,
)

# tests/test_backends.py:283-291 -- probability_sample histogram
PROB_SAMPLE = dict(src="tests/test_backends.py:283-291",
                   p=np.array([0.05] * 8 + [0.2, 0.4], dtype=np.float32), shots=10000, atol=200)

# tests/test_backends.py:426-476 -- vvag self-consistency (torch backend)
VVAG = dict(src="tests/test_backends.py:426-476", n=4, nlayers=3, batch=8, atol=1e-4)

# tests/test_quantum.py:495-502 -- ps2xyz / xyz2ps
PS_XYZ = dict(src="tests/test_quantum.py:495-502",
              xyz={"x": [1], "z": [2]}, ps=[0, 1, 3], ps6=[0, 1, 3, 0, 0, 0])

# tests/test_circuit.py:1595-1640 -- general_kraus on |++>: operators
# sqrt(.5)|0><0|, sqrt(.5)|1><1|, sqrt(.5) I have probabilities .25/.25/.5;
# status .3 picks 1 (qubit 0 -> |1>), status .8 picks 2 (identity)
GENERAL_KRAUS = dict(
    src="tests/test_circuit.py:1595-1640", n=2, pre=[("h", (0,), {}), ("h", (1,), {})],
    kraus=[np.sqrt(0.5) * np.array([[1.0, 0], [0, 0]]), np.sqrt(0.5) * np.array([[0, 0], [0, 1.0]]),
           np.sqrt(0.5) * np.eye(2)],
    status=[0.3, 0.8], picks=[1, 2], z=[-1.0, 0.0], probs=[0.25, 0.25, 0.5], atol=1e-5,
)

# tests/test_circuit.py:1439-1446 -- the registered reset channel on |+>
# with status .8 leaves amplitude 1 on |00>
RESET = dict(src="tests/test_circuit.py:1439-1446", n=2, pre=[("h", (0,), {})], status=0.8, amp0=1.0,
             atol=1e-9)

# tests/test_channels.py:24-45 -- Kraus completeness of the channel
# constructors, and isotropic(0.3, 2) == general(0.02, 2)
CHANNEL_IDENTITY = dict(src="tests/test_channels.py:24-45",
                        cases=[("depolarizing", (0.1, 0.15, 0.2)), ("amplitudedamping", (0.25, 0.3)),
                               ("phasedamping", (0.6,)), ("reset", ()), ("generaldepolarizing", (0.1, 1)),
                               ("generaldepolarizing", ([0.1, 0.1, 0.1], 1)), ("generaldepolarizing", (0.02, 2))],
                        iso=((0.02 * 15, 2), (0.02, 2)), atol=1e-5)

# tests/test_circuit.py:119-238 -- depolarizing trajectories keep the state
# normalised (n=5: H on all, cnot ring, one noise op per qubit, then cz ring
# or X on all); the reference asserts norm 1 within 1e-4
DEPOLARIZING_NORM = dict(src="tests/test_circuit.py:119-238", n=5, probs=[0.2, 0.2, 0.2, 0.4], p=0.2, atol=1e-4)

# tests/test_dmcircuit.py -- density-matrix known answers
_RHO0 = np.array([[0, 0, 0, 0], [0, 0.5, 0, -0.5j], [0, 0, 0, 0], [0, 0.5j, 0, 0.5]])
_B1 = np.array([[0, 1.0j], [0, 0]])
_B2 = np.array([[0, 0], [1.0j, 0]])
_IB1, _IB2 = np.kron(np.eye(2), _B1), np.kron(np.eye(2), _B2)
_RHO1 = _IB1 @ _RHO0 @ _IB1.conj().T + _IB2 @ _RHO0 @ _IB2.conj().T
_IY = np.kron(np.eye(2), np.array([[0, -1.0j], [1.0j, 0]]))
DM = dict(
    gate=dict(src="tests/test_dmcircuit.py:19-24", n=3, z0=0.0, z1=-1.0, atol=1e-4),
    state_inputs=dict(src="tests/test_dmcircuit.py:27-50", w1_z=(-1.0, -1.0, 1.0),
                      w2=np.array([1, 0, 0, 1.0j]) / np.sqrt(2),
                      answer=np.array([[0, 0, 0, 0], [0, 0.5, -0.5j, 0], [0, 0.5j, 0.5, 0], [0, 0, 0, 0]])),
    dm_inputs=dict(src="tests/test_dmcircuit.py:53-71", rho0=_RHO0, b1=_B1, b2=_B2, rho1=_RHO1,
                   rho2=_IY @ _RHO1 @ _IY.conj().T, atol=1e-4),
    depolarizing=dict(src="tests/test_dmcircuit.py:108-128",
                      ans=np.array([[0.4, 0, 0.4, 0], [0, 0.1, 0, 0.1], [0.4, 0, 0.4, 0], [0, 0.1, 0, 0.1]]),
                      atol=1e-5),
    mult_qubit_kraus=dict(src="tests/test_dmcircuit.py:131-175",
                          xx=np.array([[0, 0, 0, 1], [0, 0, 1, 0], [0, 1, 0, 0], [1, 0, 0, 0]]) / np.sqrt(2),
                          yz=np.array([[0, 0, -1.0j, 0], [0, 0, 0, 1.0j], [1.0j, 0, 0, 0], [0, -1.0j, 0, 0]])
                          / np.sqrt(2), theta=0.2, grad=0.199, atol=1e-2),
    noise_param_ad=dict(src="tests/test_dmcircuit.py:178-198", p=0.1, value=-0.6, grad=4.0, atol=1e-2),
    ad_channel=dict(src="tests/test_dmcircuit.py:201-214", p=0.1, theta=0.1, value=0.7562, grad=-2.388,
                    atol=1e-4),
    inputs_pipeline=dict(src="tests/test_dmcircuit.py:217-226", value=0.0, atol=1e-5),
    multicontrol=dict(src="tests/test_dmcircuit.py:247-254", value=0.93, atol=1e-6),
    to_circuit=dict(src="tests/test_dmcircuit.py:257-268", dm=-0.6, pure=-1.0, atol=1e-5),
    perfect_sampling=dict(src="tests/test_dmcircuit.py:289-303", status=[0.9, 0.5, 0.7], bits=[1, 0, 1],
                          p=0.111375, atol=1e-5),
    amplitude=dict(src="tests/test_dmcircuit.py:392-399", before=0.5, after=0.4, atol=1e-5),
    cond_measure=dict(src="tests/test_dmcircuit.py:450-456", before=1.0, after=0.0, atol=1e-5),
    sexpps=dict(src="tests/test_dmcircuit.py:474-502", y=1.0, atol=1e-5, shot_tol=0.015),
)

# tests/test_circuit.py:1465-1479 -- gate counting with aliases
GATE_COUNT = dict(src="tests/test_circuit.py:1465-1479", total=8, h=2, ccnot=3, rx_multicontrol=2, on_q0=2)
