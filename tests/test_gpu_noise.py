"""GPU parity of Monte-Carlo trajectory noise: unitary_kraus / general_kraus
and the registered channel methods through the engine, against the
complex128 oracle (oracle/noise.py) and the reference's known answers.

Tolerances: states within atol 2e-5; energies within 1e-5 relative;
gradients against complex128 central differences (eps 1e-3) within 2e-4
(the differences' own truncation error); picks exact."""

import numpy as np
import pytest
import torch

from oracle import noise as nz
from oracle import statevector as sv
from tests.golden import reference_kats as K

pytestmark = pytest.mark.gpu


def _np(t):
    return t.detach().cpu().numpy() if isinstance(t, torch.Tensor) else np.asarray(t)


def test_general_kraus_kat(tc):
    c0 = K.GENERAL_KRAUS
    c = tc.Circuit(c0["n"])
    c.h([0, 1])
    rs = [c.general_kraus(c0["kraus"], q, status=x, with_prob=True) for q, x in enumerate(c0["status"])]
    assert [int(r) for r, _ in rs] == c0["picks"]
    for _, p in rs:
        np.testing.assert_allclose([float(v) for v in p], c0["probs"], atol=c0["atol"])
    for q, z in enumerate(c0["z"]):
        np.testing.assert_allclose(float(torch.real(c.expectation_ps(z=[q]))), z, atol=c0["atol"])
    np.testing.assert_allclose(float(torch.linalg.norm(c.state())), 1.0, atol=c0["atol"])


def test_reset_kat(tc):
    c0 = K.RESET
    c = tc.Circuit(c0["n"])
    c.H(0)
    c.reset(0, status=c0["status"])
    np.testing.assert_allclose(abs(complex(c.state()[0])), c0["amp0"], atol=1e-6)


def _ring_prefix(n):
    return [("h", (i,), {}) for i in range(n)] + [("cnot", (i, (i + 1) % n), {}) for i in range(n)]


@pytest.mark.parametrize("form", ["prob_list", "channel", "method", "method2"])
def test_depolarizing_forms_match_oracle(tc, form):
    """tests/test_circuit.py:119-238's four depolarizing spellings, with
    fixed statuses: the state equals the oracle's trajectory, norm 1."""
    c0 = K.DEPOLARIZING_NORM
    n = c0["n"]
    rng = np.random.default_rng(7)
    xs = rng.random(n, dtype=np.float32)
    c = tc.Circuit(n)
    ops = _ring_prefix(n)
    for name, q, p in ops:
        getattr(c, name)(*q, **p)
    pauli = [tc.gates._x_matrix, tc.gates._y_matrix, tc.gates._z_matrix, tc.gates._i_matrix]
    for i in range(n):
        if form == "prob_list":
            c.unitary_kraus(pauli, i, prob=c0["probs"], status=float(xs[i]))
            ops.append(("unitary_kraus", (i,), dict(kraus=[sv.X, sv.Y, sv.Z, np.eye(2)], prob=c0["probs"],
                                                    status=float(xs[i]))))
        elif form == "channel":
            c.unitary_kraus(tc.channels.depolarizingchannel(0.2, 0.2, 0.2), i, status=float(xs[i]))
            ops.append(("unitary_kraus", (i,), dict(kraus=nz.depolarizing(0.2, 0.2, 0.2), status=float(xs[i]))))
        elif form == "method":
            c.depolarizing(i, px=0.2, py=0.2, pz=0.2, status=float(xs[i]))
            ops.append(("unitary_kraus", (i,), dict(kraus=nz.depolarizing(0.2, 0.2, 0.2), status=float(xs[i]))))
        else:
            c.depolarizing2(i, px=0.2, py=0.2, pz=0.2, status=float(xs[i]))
            ops.append(("unitary_kraus", (i,), dict(kraus=[sv.X, sv.Y, sv.Z, np.eye(2)], prob=[0.2, 0.2, 0.2, 0.4],
                                                    status=float(xs[i]))))
    for i in range(n):
        c.X(i)
        ops.append(("x", (i,), {}))
    want, _ = nz.run_noisy(n, ops)
    got = _np(c.state())
    np.testing.assert_allclose(np.linalg.norm(got), 1.0, atol=c0["atol"])
    np.testing.assert_allclose(got, want, atol=2e-5)


# a layered noisy ansatz: rx / rzz layers with unitary and general channels
N6 = 6


def _program(nl=2):
    prog = []
    k = 0
    s = 0
    for _ in range(nl):
        for q in range(N6):
            prog.append(("g", "rx", (q,), k))
            k += 1
        for q in range(N6 - 1):
            prog.append(("g", "rzz", (q, q + 1), k))
            k += 1
        prog.append(("n", "dep", (0,), (0.05, 0.1, 0.15), s))
        prog.append(("n", "ad", (1,), (0.3, 0.9), s + 1))
        prog.append(("n", "pd", (3,), (0.4,), s + 2))
        prog.append(("n", "gdep2", (4, 5), (0.03,), s + 3))
        prog.append(("n", "uk", (2,), ([0.1, 0.2, 0.3, 0.4],), s + 4))
        s += 5
    return prog, k, s


TERMS6 = [(-1.0, {"z": [i, i + 1]}) for i in range(N6 - 1)] + [(-0.7, {"x": [i]}) for i in range(N6)]


def _engine_energy(tc, params, status, prog):
    from tensorcircuit_gb300 import templates

    c = tc.Circuit(N6)
    for e in prog:
        if e[0] == "g":
            getattr(c, e[1])(*e[2], theta=params[e[3]])
            continue
        _, kind, q, a, si = e
        x = status[si]
        if kind == "dep":
            c.depolarizing(*q, px=a[0], py=a[1], pz=a[2], status=x)
        elif kind == "ad":
            c.amplitudedamping(*q, gamma=a[0], p=a[1], status=x)
        elif kind == "pd":
            c.phasedamping(*q, gamma=a[0], status=x)
        elif kind == "gdep2":
            c.generaldepolarizing(*q, p=a[0], num_qubits=2, status=x)
        else:
            c.unitary_kraus([tc.gates._x_matrix, tc.gates._y_matrix, tc.gates._z_matrix, tc.gates._i_matrix],
                            *q, prob=a[0], status=x)
    return torch.real(templates.energy(c, TERMS6))


def _oracle_ops(params, status, prog):
    ops = []
    for e in prog:
        if e[0] == "g":
            ops.append((e[1], e[2], {"theta": float(params[e[3]])}))
            continue
        _, kind, q, a, si = e
        x = float(status[si])
        if kind == "dep":
            ops.append(("unitary_kraus", q, dict(kraus=nz.depolarizing(*a), status=x)))
        elif kind == "ad":
            ops.append(("general_kraus", q, dict(kraus=nz.amplitude_damping(*a), status=x)))
        elif kind == "pd":
            ops.append(("general_kraus", q, dict(kraus=nz.phase_damping(*a), status=x)))
        elif kind == "gdep2":
            ops.append(("unitary_kraus", q, dict(kraus=nz.general_depolarizing(a[0], 2), status=x)))
        else:
            ops.append(("unitary_kraus", q, dict(kraus=[sv.X, sv.Y, sv.Z, np.eye(2)], prob=a[0], status=x)))
    return ops


def _oracle_energy(params, status, prog):
    psi, picks = nz.run_noisy(N6, _oracle_ops(params, status, prog))
    return sv.energy(psi, N6, TERMS6).real, picks


def test_noisy_trajectories_vmap(tc):
    """A batch of trajectories (one status vector each) under vmap: one
    batched engine sweep per segment; every trajectory's energy equals the
    oracle's."""
    K_ = tc.set_backend("pytorch")
    prog, P, S = _program()
    rng = np.random.default_rng(21)
    params = rng.uniform(0, 2 * np.pi, P).astype(np.float32)
    B = 24
    status = rng.random((B, S), dtype=np.float32)
    dev = torch.device("cuda")
    pt = torch.as_tensor(params, device=dev)

    def f(st):
        return _engine_energy(tc, pt, st, prog)

    got = _np(K_.vmap(f, vectorized_argnums=0)(torch.as_tensor(status, device=dev)))
    for b in range(B):
        e, _ = _oracle_energy(params.astype(np.float64), status[b], prog)
        assert abs(got[b] - e) <= 1e-5 * max(1.0, abs(e)), (b, got[b], e)


def test_noisy_status_tensor_batch(tc):
    """Statuses given as [B] tensors (no vmap) batch the trajectories the
    same way."""
    prog, P, S = _program(1)
    rng = np.random.default_rng(22)
    params = rng.uniform(0, 2 * np.pi, P).astype(np.float32)
    B = 8
    status = rng.random((B, S), dtype=np.float32)
    dev = torch.device("cuda")
    st = torch.as_tensor(status, device=dev)
    got = _np(_engine_energy(tc, torch.as_tensor(params, device=dev), [st[:, j] for j in range(S)], prog))
    assert got.shape == (B,)
    for b in range(B):
        e, _ = _oracle_energy(params.astype(np.float64), status[b], prog)
        assert abs(got[b] - e) <= 1e-5 * max(1.0, abs(e))


def test_noisy_gradient_vs_finite_differences(tc):
    """Energy gradient through unitary and general channels (segments,
    probability-dependent rescaling) against complex128 central differences
    with the picks held fixed."""
    prog, P, S = _program()
    rng = np.random.default_rng(23)
    params = rng.uniform(0, 2 * np.pi, P).astype(np.float32)
    status = rng.random(S, dtype=np.float32)
    dev = torch.device("cuda")
    pt = torch.as_tensor(params, device=dev).requires_grad_(True)
    e = _engine_energy(tc, pt, [float(x) for x in status], prog)
    e.backward()
    g = _np(pt.grad)
    p64 = params.astype(np.float64)
    e0, picks0 = _oracle_energy(p64, status, prog)
    assert abs(float(e.detach()) - e0) <= 1e-5 * max(1.0, abs(e0))
    eps = 1e-3
    for k in range(0, P, 3):
        pp, pm = p64.copy(), p64.copy()
        pp[k] += eps
        pm[k] -= eps
        ep, kp = _oracle_energy(pp, status, prog)
        em, km = _oracle_energy(pm, status, prog)
        if kp != picks0 or km != picks0:
            continue  # a pick flips inside the stencil
        np.testing.assert_allclose(g[k], (ep - em) / (2 * eps), atol=2e-4)


def test_noisy_vvag_rows(tc):
    """vvag over (params, statuses): each row equals a single
    value_and_grad of that trajectory."""
    K_ = tc.set_backend("pytorch")
    prog, P, S = _program(1)
    rng = np.random.default_rng(24)
    B = 6
    dev = torch.device("cuda")
    params = torch.as_tensor(rng.uniform(0, 2 * np.pi, (B, P)).astype(np.float32), device=dev)
    status = torch.as_tensor(rng.random((B, S), dtype=np.float32), device=dev)

    def f(p, st):
        return _engine_energy(tc, p, st, prog)

    v, g = K_.vvag(f, argnums=0, vectorized_argnums=(0, 1))(params, status)
    for b in (0, 3, 5):
        vb, gb = K_.value_and_grad(f)(params[b], status[b])
        np.testing.assert_allclose(_np(v)[b], _np(vb), rtol=1e-5, atol=1e-6)
        np.testing.assert_allclose(_np(g)[b], _np(gb), rtol=1e-4, atol=1e-5)


def test_differentiable_channel_parameter(tc):
    """Kraus operators given as tensors (a damping rate that needs a
    gradient) are applied exactly; d energy / d gamma matches central
    differences."""
    from tensorcircuit_gb300 import templates

    n = 4
    rng = np.random.default_rng(25)
    th = rng.uniform(0, 2 * np.pi, n)
    xs = [0.35, 0.8]
    dev = torch.device("cuda")
    terms = [(1.0, {"z": [0, 1]}), (0.5, {"x": [2]}), (0.8, {"z": [1]})]

    def engine(gamma):
        c = tc.Circuit(n)
        for q in range(n):
            c.rx(q, theta=float(th[q]))
        c.cnot(0, 1)
        c.amplitudedamping(1, gamma=gamma, p=torch.tensor(1.0, device=dev), status=xs[0])
        c.cnot(1, 2)
        c.amplitudedamping(2, gamma=gamma, p=torch.tensor(1.0, device=dev), status=xs[1])
        return torch.real(templates.energy(c, terms))

    def oracle(gamma):
        ops = [("rx", (q,), {"theta": th[q]}) for q in range(n)] + [("cnot", (0, 1), {})]
        ops += [("general_kraus", (1,), dict(kraus=nz.amplitude_damping(gamma, 1.0), status=xs[0])),
                ("cnot", (1, 2), {}),
                ("general_kraus", (2,), dict(kraus=nz.amplitude_damping(gamma, 1.0), status=xs[1]))]
        psi, picks = nz.run_noisy(n, ops)
        return sv.energy(psi, n, terms).real, picks

    g0 = 0.3
    gt = torch.tensor(g0, device=dev, requires_grad=True)
    e = engine(gt)
    e.backward()
    e0, pk = oracle(g0)
    assert abs(float(e.detach()) - e0) <= 1e-5
    eps = 1e-4
    ep, kp = oracle(g0 + eps)
    em, km = oracle(g0 - eps)
    assert kp == pk == km
    np.testing.assert_allclose(float(gt.grad), (ep - em) / (2 * eps), atol=2e-4)


def test_zero_probability_operator_is_finite(tc):
    c = tc.Circuit(3)
    c.h(0)
    c.cnot(0, 1)
    # probabilities (0.9, 0.1, 0, 0): status 0.95 picks X
    c.depolarizing(1, px=0.1, py=0.0, pz=0.0, status=0.95)
    c.depolarizing(2, px=0.0, py=0.0, pz=0.0, status=0.5)
    s = _np(c.state())
    assert np.all(np.isfinite(s))
    want, _ = nz.run_noisy(3, [("h", (0,), {}), ("cnot", (0, 1), {}),
                               ("unitary_kraus", (1,), dict(kraus=[sv.X], prob=[1.0], status=0.0))])
    np.testing.assert_allclose(s, want, atol=2e-5)


def test_noisy_vvag_graph_replay_matches_eager(tc):
    """K.jit(K.vvag(f)) over trajectories replays one CUDA graph (every
    segment, pick and rescaling on the device, no host round trip); the
    replay equals the eager evaluation for new statuses and parameters."""
    K_ = tc.set_backend("pytorch")
    prog, P, S = _program(1)
    rng = np.random.default_rng(26)
    B = 16
    dev = torch.device("cuda")

    def f(p, st):
        return _engine_energy(tc, p, st, prog)

    eager = K_.vvag(f, argnums=0, vectorized_argnums=1)
    jf = K_.jit(K_.vvag(f, argnums=0, vectorized_argnums=1))
    for it in range(6):
        p = torch.as_tensor(rng.uniform(0, 2 * np.pi, P).astype(np.float32), device=dev)
        st = torch.as_tensor(rng.random((B, S), dtype=np.float32), device=dev)
        v1, g1 = jf(p, st)
        v0, g0 = eager(p, st)
        np.testing.assert_allclose(_np(v1), _np(v0), rtol=1e-5, atol=1e-6)
        np.testing.assert_allclose(_np(g1), _np(g0), rtol=1e-4, atol=1e-5)
    assert jf.capture_errors() == []
    assert any(e["graph"] is not None for e in jf.cache.values())


def _pick_torch(ev, coef, x):
    """The general-channel branch step as fp32 torch operations (the steps of
    tensorcircuit/circuit.py:541-556 and :682-687)."""
    p = torch.real(ev) @ coef.t()
    cum = torch.cumsum(p, -1)
    l = cum.shape[-1]
    if l == 1:
        r = torch.zeros(p.shape[:-1], dtype=torch.int32, device=p.device)
    else:
        s = torch.sign(x.unsqueeze(-1) - cum[..., : l - 1]).sum(-1)
        r = (s * 0.5 + (l - 1) * 0.5).to(torch.int32)
    pr = torch.gather(p, -1, r.long().unsqueeze(-1)).squeeze(-1)
    return r, (1.0 / (torch.sqrt(pr) + 1e-10)).to(torch.complex64), p


@pytest.mark.parametrize("nk,ns", [(1, 4), (2, 4), (4, 16)])
def test_kraus_pick_kernel_matches_torch_steps(tc, nk, ns):
    """tcg_kraus_pick against the same steps in torch: picks exact (ties
    x == c_i included: dyadic inputs make every sum exact), rescale and p
    within 1e-6 relative, the gradient to Re(ev) within 1e-5, and the vmap
    rule equal to the unbatched call."""
    from tensorcircuit_gb300 import engine as eng

    rng = np.random.default_rng(40 + nk)
    dev = torch.device("cuda")
    B = 257
    ev_np = rng.integers(1, 9, (B, ns)) / 8.0 + 1j * rng.standard_normal((B, ns))
    coef_np = rng.integers(1, 5, (nk, ns)) / (16.0 * ns)
    ev = torch.as_tensor(ev_np.astype(np.complex64), device=dev)
    coef = torch.as_tensor(coef_np.astype(np.float32), device=dev)
    cum = np.cumsum(np.real(ev_np) @ coef_np.T, -1)
    x_np = rng.random(B) * cum[:, -1]
    x_np[:40] = cum[:40, max(nk - 3, 0)]   # ties with a running sum
    x = torch.as_tensor(x_np.astype(np.float32), device=dev)
    w = torch.as_tensor(rng.standard_normal(B).astype(np.float32), device=dev)

    e1 = ev.clone().requires_grad_(True)
    r1, s1, p1 = eng.KrausPickFn.apply(e1, coef, x)
    (g1,) = torch.autograd.grad((torch.real(s1) * w).sum(), e1)
    e0 = ev.clone().requires_grad_(True)
    r0, s0, p0 = _pick_torch(e0, coef, x)
    (g0,) = torch.autograd.grad((torch.real(s0) * w).sum(), e0)

    assert torch.equal(r1, r0)
    if nk > 1:
        assert len(set(_np(r1).tolist())) > 1
    np.testing.assert_allclose(_np(p1), _np(p0), rtol=1e-6)
    np.testing.assert_allclose(_np(s1), _np(s0), rtol=1e-6)
    np.testing.assert_allclose(_np(g1), _np(g0), rtol=1e-5, atol=1e-6)
    assert float(torch.abs(torch.imag(g1)).max()) == 0.0

    rv, sv_, pv = torch.func.vmap(lambda e, xx: eng.KrausPickFn.apply(e, coef, xx))(ev, x)
    assert torch.equal(rv, r1)
    np.testing.assert_allclose(_np(sv_), _np(s1), rtol=0)
    # one shared draw for every row (x_stride 0)
    rs, _, _ = eng.KrausPickFn.apply(ev, coef, x[7])
    r7, _, _ = _pick_torch(ev, coef, x[7].expand(B))
    assert torch.equal(rs, r7)
