"""GPU parity of ``DMCircuit``: vec(rho) evolved by the engine (gates as G on
the row qubits and conj(G) on the column qubits, channels as superoperator
gates starting new segments) against the complex128 density-matrix oracle
and the reference's known answers (tests/test_dmcircuit.py).

Tolerances: density-matrix entries atol 2e-5; expectations 1e-5;
gradients against complex128 central differences within 2e-4."""

import numpy as np
import pytest
import torch

from oracle import densitymatrix as dmo
from oracle import noise as nz
from oracle import statevector as sv
from tests.golden import reference_kats as K

pytestmark = pytest.mark.gpu
DM = K.DM


def _np(t):
    return t.detach().cpu().numpy() if isinstance(t, torch.Tensor) else np.asarray(t)


def _re(t):
    return float(torch.real(t)) if isinstance(t, torch.Tensor) else float(np.real(t))


def test_dm_gate_and_inputs_kats(tc):
    c = tc.DMCircuit(3)
    c.H(0)
    c.rx(1, theta=np.pi)
    np.testing.assert_allclose(_re(c.expectation((tc.gates.z(), [0]))), DM["gate"]["z0"], atol=1e-4)
    np.testing.assert_allclose(_re(c.expectation((tc.gates.z(), [1]))), DM["gate"]["z1"], atol=1e-4)
    w = np.zeros(8)
    w[1] = 1.0
    c = tc.DMCircuit(3, inputs=w)
    c.cnot(2, 1)
    for q, want in zip((1, 2, 0), DM["state_inputs"]["w1_z"]):
        np.testing.assert_allclose(_re(c.expectation((tc.gates.z(), [q]))), want, atol=1e-6)
    c = tc.DMCircuit(2, inputs=DM["state_inputs"]["w2"])
    c.Y(0)
    np.testing.assert_allclose(_np(c.densitymatrix()), DM["state_inputs"]["answer"], atol=2e-6)


def test_dm_kraus_kats(tc):
    k = DM["dm_inputs"]
    for form in ("list", "args"):
        c = tc.DMCircuit(nqubits=2, dminputs=k["rho0"])
        ks = [tc.gates.Gate(k["b1"]), tc.gates.Gate(k["b2"])]
        if form == "list":
            c.apply_general_kraus(ks, [(1,)])
        else:
            c.apply_general_kraus(ks, 1)
        np.testing.assert_allclose(_np(c.densitymatrix()), k["rho1"], atol=k["atol"])
        c.y(1)
        np.testing.assert_allclose(_np(c.densitymatrix()), k["rho2"], atol=k["atol"])
    for api in ("v1", "v2"):
        c = tc.DMCircuit(2)
        c.H(0)
        if api == "v1":
            c.apply_general_kraus(tc.channels.depolarizingchannel(0.1, 0.1, 0.1), [(1,)])
        else:
            c.depolarizing(1, px=0.1, py=0.1, pz=0.1)
        np.testing.assert_allclose(_np(c.densitymatrix(check=True)), DM["depolarizing"]["ans"], atol=1e-5)


def test_dm_gradient_kats(tc):
    dev = torch.device("cuda")
    K_ = tc.set_backend("pytorch")
    c0 = DM["mult_qubit_kraus"]

    def forward2(theta):
        c = tc.DMCircuit(3)
        c.H(0)
        c.rx(1, theta=theta)
        c.apply_general_kraus([tc.gates.Gate(c0["xx"]), tc.gates.Gate(c0["yz"])], 0, 1)
        c.H(1)
        return torch.real(torch.sum(c.densitymatrix()))

    _, g = K_.value_and_grad(forward2)(torch.tensor(c0["theta"], device=dev))
    np.testing.assert_allclose(float(g), c0["grad"], atol=c0["atol"])

    c1 = DM["noise_param_ad"]

    def forward(p):
        c = tc.DMCircuit(2)
        c.X(1)
        c.depolarizing(1, px=p, py=p, pz=p)
        return torch.real(c.expectation((tc.gates.z(), [1])))

    v, g = K_.value_and_grad(forward)(torch.tensor(c1["p"], device=dev))
    np.testing.assert_allclose(float(v), c1["value"], atol=c1["atol"])
    np.testing.assert_allclose(float(g), c1["grad"], atol=c1["atol"])

    c2 = DM["ad_channel"]
    p = torch.tensor(c2["p"], device=dev, requires_grad=True)
    c = tc.DMCircuit(3)
    c.rx(1, theta=c2["theta"])
    c.apply_general_kraus(tc.channels.depolarizingchannel(p, 0.2 * p, p), [(1,)])
    c.H(0)
    loss = torch.real(c.expectation((tc.gates.z(), [1])))
    loss.backward()
    np.testing.assert_allclose(float(loss.detach()), c2["value"], atol=c2["atol"])
    np.testing.assert_allclose(float(p.grad), c2["grad"], atol=1e-3)


def test_dm_misc_kats(tc):
    c = tc.DMCircuit(2, dminputs=0.25 * np.eye(4))
    c.H(0)
    c.general_kraus([np.sqrt(0.5) * tc.gates._i_matrix, np.sqrt(0.5) * tc.gates._x_matrix], 1)
    np.testing.assert_allclose(_re(c.expectation_ps(z=[0])), DM["inputs_pipeline"]["value"], atol=1e-5)

    c = tc.DMCircuit(3)
    c.H(1)
    c.depolarizing(0, px=0.05, py=0.02, pz=0.02)
    c.multicontrol(1, 0, 2, ctrl=[1, 1], unitary=tc.gates.x())
    np.testing.assert_allclose(_re(c.expectation_ps(z=[2])), DM["multicontrol"]["value"], atol=1e-5)

    c = tc.DMCircuit(2)
    c.X(0)
    c.depolarizing(0, px=0.1, py=0.1, pz=0.1)
    c.cnot(0, 1)
    np.testing.assert_allclose(_re(c.expectation_ps(z=[1])), DM["to_circuit"]["dm"], atol=1e-5)
    np.testing.assert_allclose(_re(c.to_circuit().expectation_ps(z=[1])), DM["to_circuit"]["pure"], atol=1e-5)

    c = tc.DMCircuit(3)
    for i in range(3):
        c.H(i)
    for i in range(3):
        c.amplitudedamping(i, p=1.0, gamma=0.1)
    s, p = c.perfect_sampling(np.array(DM["perfect_sampling"]["status"]))
    np.testing.assert_allclose(_np(s), DM["perfect_sampling"]["bits"])
    np.testing.assert_allclose(float(p), DM["perfect_sampling"]["p"], atol=DM["perfect_sampling"]["atol"])

    c = tc.DMCircuit(2)
    c.H(0)
    c.cnot(0, 1)
    np.testing.assert_allclose(_re(c.amplitude("11")), DM["amplitude"]["before"], atol=1e-5)
    c.depolarizing(1, px=0.2, py=0, pz=0)
    np.testing.assert_allclose(_re(c.amplitude("11")), DM["amplitude"]["after"], atol=1e-5)
    np.testing.assert_allclose(_re(c.amplitude(torch.tensor([1, 0]))), 0.1, atol=1e-5)

    c = tc.DMCircuit(2)
    c.H(0)
    np.testing.assert_allclose(_re(c.expectation_ps(x=[0])), DM["cond_measure"]["before"], atol=1e-5)
    c.cond_measure(0)
    np.testing.assert_allclose(_re(c.expectation_ps(x=[0])), DM["cond_measure"]["after"], atol=1e-5)

    c = tc.DMCircuit(1, inputs=1 / np.sqrt(2) * np.array([1.0, 1.0j]))
    np.testing.assert_allclose(_re(c.sample_expectation_ps(y=[0])), DM["sexpps"]["y"], atol=1e-5)
    np.testing.assert_allclose(_re(c.expectation_ps(y=[0])), DM["sexpps"]["y"], atol=1e-5)


def test_dm_sexpps_shots_and_inverse(tc):
    """tests/test_dmcircuit.py:271-287 and :474-502."""
    c = tc.DMCircuit(4)
    c.H(0)
    c.H(1)
    c.X(2)
    c.Y(3)
    c.cnot(0, 1)
    c.depolarizing(1, px=0.05, py=0.05, pz=0.1)
    c.rx(1, theta=0.3)
    c.ccnot(2, 3, 1)
    c.depolarizing(0, px=0.05, py=0.0, pz=0.1)
    c.rzz(0, 3, theta=0.5)
    c.ry(3, theta=2.2)
    c.amplitudedamping(2, gamma=0.1, p=0.95)
    c.s(1)
    c.td(2)
    c.cswap(3, 0, 1)
    y = _re(c.sample_expectation_ps(x=[1], y=[0], z=[2, 3]))
    ye = _re(c.expectation_ps(x=[1], y=[0], z=[2, 3]))
    np.testing.assert_allclose(ye, y, atol=1e-5)
    y2 = _re(c.sample_expectation_ps(x=[1], y=[0], z=[2, 3], shots=81920))
    assert abs(y2 - y) < DM["sexpps"]["shot_tol"]

    c = tc.DMCircuit2(3)
    c.h(0)
    c.rx(1, theta=0.5)
    c.amplitudedamping(1, gamma=0.1, p=0.9)
    c.amplitudedamping(2, gamma=0.1, p=0.9)
    c.rzz(0, 2, theta=-1.0)
    r = _re(c.inverse().expectation_ps(z=[2]))
    c2 = tc.DMCircuit2(3)
    c2.rzz(0, 2, theta=1.0)
    c2.rx(1, theta=-0.5)
    c2.h(0)
    np.testing.assert_allclose(r, _re(c2.expectation_ps(z=[2])), atol=1e-5)


# random density-matrix circuits against the oracle
def _random_dm_program(n, depth, rng):
    names1 = ["h", "x", "y", "z", "s", "t", "sd", "td", "wroot"]
    prog = []
    for _ in range(depth):
        kind = rng.integers(6) if n > 1 else int(rng.choice([0, 1, 4]))
        if kind == 0:
            prog.append((str(rng.choice(names1)), (int(rng.integers(n)),), {}))
        elif kind == 1:
            prog.append((str(rng.choice(["rx", "ry", "rz", "phase"])), (int(rng.integers(n)),),
                         {"theta": float(rng.uniform(-3, 3))}))
        elif kind == 2:
            a, b = rng.choice(n, 2, replace=False)
            prog.append((str(rng.choice(["rxx", "ryy", "rzz", "crx", "cry", "cphase"])), (int(a), int(b)),
                         {"theta": float(rng.uniform(-3, 3))}))
        elif kind == 3:
            a, b = rng.choice(n, 2, replace=False)
            prog.append((str(rng.choice(["cnot", "cz", "swap", "iswap"])), (int(a), int(b)), {}))
        elif kind == 4:
            q = int(rng.integers(n))
            ch = int(rng.integers(4))
            ks = [nz.depolarizing(0.05, 0.1, 0.02), nz.amplitude_damping(0.3, 0.8), nz.phase_damping(0.25),
                  nz.reset()][ch]
            prog.append(("channel", (q,), ks))
        else:
            a, b = rng.choice(n, 2, replace=False)
            prog.append(("channel", (int(a), int(b)), nz.general_depolarizing(0.02, 2)))
    return prog


def _build(tc, n, prog):
    c = tc.DMCircuit(n)
    for name, q, p in prog:
        if name == "channel":
            c.apply_general_kraus([tc.gates.Gate(k) for k in p], *q)
        else:
            getattr(c, name)(*q, **p)
    return c


@pytest.mark.parametrize("n,seed", [(1, 1), (3, 2), (5, 3), (7, 4)])
def test_dm_random_circuits_match_oracle(tc, n, seed):
    rng = np.random.default_rng(seed)
    prog = _random_dm_program(n, 24, rng)
    c = _build(tc, n, prog)
    want = dmo.run_dm(n, prog)
    np.testing.assert_allclose(_np(c.densitymatrix()), want, atol=2e-5)
    for q in range(n):
        np.testing.assert_allclose(_re(c.expectation_ps(x=[q])), dmo.expectation_ps(want, n, x=[q]).real, atol=1e-5)
    np.testing.assert_allclose(_np(c.probability()), np.real(np.diag(want)), atol=2e-5)


def test_dm_parameter_gradient_vs_finite_differences(tc):
    """d tr(rho H) / d theta through gates on both sides of rho and several
    channel segments, against complex128 central differences."""
    n = 4
    rng = np.random.default_rng(9)
    th = rng.uniform(-2, 2, 10)
    terms = [(1.0, dict(z=[0, 1])), (0.5, dict(x=[2])), (-0.7, dict(y=[1, 3])), (0.3, dict(z=[3]))]

    def prog(t):
        return [("rx", (0,), {"theta": t[0]}), ("ry", (1,), {"theta": t[1]}), ("rzz", (0, 1), {"theta": t[2]}),
                ("channel", (1,), nz.amplitude_damping(0.2, 0.9)), ("crx", (1, 2), {"theta": t[3]}),
                ("rxx", (2, 3), {"theta": t[4]}), ("channel", (2,), nz.depolarizing(0.05, 0.05, 0.1)),
                ("ryy", (0, 3), {"theta": t[5]}), ("phase", (3,), {"theta": t[6]}),
                ("channel", (0, 3), nz.general_depolarizing(0.03, 2)), ("rz", (2,), {"theta": t[7]}),
                ("u", (1,), {"theta": t[8], "phi": 0.3, "lbd": t[9]})]

    def oracle(t):
        rho = dmo.run_dm(n, prog(t))
        return sum(cf * dmo.expectation_ps(rho, n, **kw).real for cf, kw in terms)

    dev = torch.device("cuda")
    tt = torch.tensor(th, dtype=torch.float32, device=dev, requires_grad=True)
    c = _build(tc, n, prog(tt.unbind(0)))
    e = sum(cf * torch.real(c.expectation_ps(**kw)) for cf, kw in terms)
    e.backward()
    g = _np(tt.grad)
    th32 = th.astype(np.float32).astype(np.float64)
    np.testing.assert_allclose(float(e.detach()), oracle(th32), atol=1e-5)
    eps = 1e-4
    for k in range(10):
        tp, tm = th32.copy(), th32.copy()
        tp[k] += eps
        tm[k] -= eps
        np.testing.assert_allclose(g[k], (oracle(tp) - oracle(tm)) / (2 * eps), atol=2e-4)


def test_dm_vmap_batch(tc):
    """A vmap over parameters batches whole density-matrix circuits,
    channel segments included."""
    K_ = tc.set_backend("pytorch")
    n = 3
    dev = torch.device("cuda")

    def f(t):
        c = tc.DMCircuit(n)
        for q in range(n):
            c.rx(q, theta=t[q])
        c.amplitudedamping(1, gamma=0.3, p=1.0)
        c.cnot(0, 2)
        c.depolarizing(2, px=0.1, py=0.0, pz=0.05)
        return torch.real(c.expectation_ps(z=[2]))

    ts = torch.as_tensor(np.random.default_rng(5).uniform(-2, 2, (6, n)).astype(np.float32), device=dev)
    v, g = K_.vvag(f, argnums=0, vectorized_argnums=0)(ts)
    for b in range(6):
        vb, gb = K_.value_and_grad(f)(ts[b])
        np.testing.assert_allclose(_np(v)[b], float(vb), atol=1e-6)
        np.testing.assert_allclose(_np(g)[b], _np(gb), atol=1e-5)
        t = _np(ts[b]).astype(np.float64)
        rho = dmo.run_dm(n, [("rx", (q,), {"theta": t[q]}) for q in range(n)] +
                         [("channel", (1,), nz.amplitude_damping(0.3, 1.0)), ("cnot", (0, 2), {}),
                          ("channel", (2,), nz.depolarizing(0.1, 0.0, 0.05))])
        np.testing.assert_allclose(_np(v)[b], dmo.expectation_ps(rho, n, z=[2]).real, atol=1e-5)
