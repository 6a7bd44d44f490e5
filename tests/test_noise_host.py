"""CPU: Monte-Carlo trajectory noise -- the oracle pinned to the reference's
known answers, and the package's host logic (channel constructors, the
Kraus pick rule, the local-operator contraction) against the oracle."""

import numpy as np
import pytest
import torch

from oracle import noise as nz
from oracle import statevector as sv
from tests.golden import reference_kats as K
from tensorcircuit_gb300 import channels as ch
from tensorcircuit_gb300.circuit import _apply_local, _pauli_strings, _pick


def test_oracle_general_kraus_kat():
    c = K.GENERAL_KRAUS
    psi = sv.run_circuit(c["n"], c["pre"])
    picks, probs = [], []
    for q, x in enumerate(c["status"]):
        psi, r, p = nz.general_kraus(psi, c["n"], c["kraus"], [q], x)
        picks.append(r)
        probs.append(p)
    assert picks == c["picks"]
    for q, z in enumerate(c["z"]):
        np.testing.assert_allclose(sv.expectation_ps(psi, c["n"], z=[q]).real, z, atol=c["atol"])
    for p in probs:
        np.testing.assert_allclose(p, c["probs"], atol=c["atol"])
    np.testing.assert_allclose(np.linalg.norm(psi), 1.0, atol=c["atol"])


def test_oracle_reset_kat():
    c = K.RESET
    psi = sv.run_circuit(c["n"], c["pre"])
    psi, r, _ = nz.general_kraus(psi, c["n"], nz.reset(), [0], c["status"])
    np.testing.assert_allclose(abs(psi[0]), c["amp0"], atol=c["atol"])


@pytest.mark.parametrize("name,args", K.CHANNEL_IDENTITY["cases"])
def test_channel_completeness(name, args):
    ks = getattr(ch, name + "channel")(*args)
    ch.kraus_identity_check(ks)
    oracle_f = {"depolarizing": nz.depolarizing, "amplitudedamping": nz.amplitude_damping,
                "phasedamping": nz.phase_damping, "reset": nz.reset,
                "generaldepolarizing": nz.general_depolarizing}[name]
    want = oracle_f(*args)
    assert len(want) == len(ks)
    for a, b in zip(ks, want):
        np.testing.assert_allclose(np.asarray(a.tensor).reshape(b.shape), b, atol=1e-12)
    assert nz.identity_defect(want) < K.CHANNEL_IDENTITY["atol"]


def test_isotropic_equals_general():
    a_args, b_args = K.CHANNEL_IDENTITY["iso"]
    for a, b in zip(ch.isotropicdepolarizingchannel(*a_args), ch.generaldepolarizingchannel(*b_args)):
        np.testing.assert_allclose(np.asarray(a.tensor), np.asarray(b.tensor), atol=1e-12)


def test_thermal_relaxation_both_methods():
    kb = ch.thermalrelaxationchannel(300, 200, 100, "ByKraus", 0.1)
    ch.kraus_identity_check(kb)
    for a, b in zip(kb, nz.thermal_relaxation_bykraus(300, 200, 100, 0.1)):
        np.testing.assert_allclose(np.asarray(a.tensor).reshape(2, 2), b, atol=1e-12)
    kc = ch.thermalrelaxationchannel(100, 200, 100, "ByChoi", 0.1)
    assert len(kc) == 4
    ch.kraus_identity_check(kc)
    assert len(ch.thermalrelaxationchannel(100, 200, 100, "AUTO", 0.0)) == 3
    # the two constructions describe the same channel when both apply
    rho = np.array([[0.3, 0.2 - 0.1j], [0.2 + 0.1j, 0.7]])
    ka = [np.asarray(k.tensor).reshape(2, 2) for k in ch.thermalrelaxationchannel(300, 200, 100, "ByKraus", 0.1)]
    kc = [np.asarray(k.tensor).reshape(2, 2) for k in ch.thermalrelaxationchannel(300, 200, 100, "ByChoi", 0.1)]
    ra = sum(k @ rho @ k.conj().T for k in ka)
    rc = sum(k @ rho @ k.conj().T for k in kc)
    np.testing.assert_allclose(ra, rc, atol=1e-12)


def test_pick_rule_matches_oracle():
    rng = np.random.default_rng(3)
    for l in (1, 2, 3, 4, 6):
        prob = rng.dirichlet(np.ones(l)).astype(np.float32)
        cum = torch.as_tensor(np.cumsum(prob, dtype=np.float32))
        xs = np.concatenate([rng.random(64, dtype=np.float32), np.cumsum(prob, dtype=np.float32)[:-1]])
        for x in xs:
            got = int(_pick(torch.tensor(float(x)), cum, torch.device("cpu")))
            assert got == nz.pick(float(x), prob), (l, x)


def test_pick_ties_follow_the_sign_rule():
    cpu = torch.device("cpu")
    # x on a single boundary: half of one equality truncates away
    assert int(_pick(0.5, torch.tensor([0.5, 1.0]), cpu)) == 0 == nz.pick(0.5, [0.5, 0.5])
    # two equal boundaries (a zero-probability operator): the rule lands on it
    assert int(_pick(0.5, torch.tensor([0.5, 0.5, 1.0]), cpu)) == 1 == nz.pick(0.5, [0.5, 0.0, 0.5])
    # batched statuses
    r = _pick(torch.tensor([0.1, 0.6, 0.95]), torch.tensor([0.25, 0.5, 1.0]), cpu)
    assert r.tolist() == [0, 2, 2]


@pytest.mark.parametrize("qubits", [(0,), (3,), (4, 1), (2, 3)])
def test_apply_local_matches_oracle(qubits):
    n = 5
    rng = np.random.default_rng(11)
    k = len(qubits)
    d = 1 << k
    psi = rng.standard_normal((3, 1 << n)) + 1j * rng.standard_normal((3, 1 << n))
    m = rng.standard_normal((3, d, d)) + 1j * rng.standard_normal((3, d, d))
    got = _apply_local(torch.as_tensor(psi), torch.as_tensor(m), qubits, n).numpy()
    for b in range(3):
        np.testing.assert_allclose(got[b], sv.apply_matrix(psi[b], m[b], list(qubits), n), atol=1e-10)
    got1 = _apply_local(torch.as_tensor(psi[0]), torch.as_tensor(m[0]), qubits, n).numpy()
    np.testing.assert_allclose(got1, sv.apply_matrix(psi[0], m[0], list(qubits), n), atol=1e-10)


def test_pauli_expansion_of_kraus_products():
    """p_i = sum_s coef[i, s] <P_s>: the expansion general_kraus measures."""
    rng = np.random.default_rng(5)
    n = 4
    psi = rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)
    psi /= np.linalg.norm(psi)
    for qubits, kraus in (((1,), nz.amplitude_damping(0.3, 0.8)), ((2, 0), nz.general_depolarizing(0.05, 2))):
        kk = len(qubits)
        strings = _pauli_strings(kk)
        ev = []
        for codes, _ in strings:
            kw = {"x": [], "y": [], "z": []}
            for q, c in zip(qubits, codes):
                if c:
                    kw["xyz"[c - 1]].append(q)
            ev.append(sv.expectation_ps(psi, n, **kw).real)
        d = 1 << kk
        coef = np.array([[np.real(np.trace(m.conj().T @ m @ s)) / d for _, s in strings] for m in kraus])
        np.testing.assert_allclose(coef @ np.array(ev), nz.kraus_probs(psi, n, kraus, qubits), atol=1e-12)


class _FakePickLib:
    """Stands in for the library's two Kraus-pick entry points on CPU
    tensors (the pointer helper is patched to pass tensors through), so the
    autograd and vmap wiring around them can run without a GPU."""

    def tcg_kraus_pick(self, e, S, cf, K_, xf, xs, B, pick, scale, p, st):
        ev = e.reshape(B, S)
        x = xf.reshape(-1).expand(B) if xs == 0 else xf.reshape(-1)
        pp = torch.real(ev) @ cf.t()
        r = _pick(x, torch.cumsum(pp, -1), torch.device("cpu"))
        pr = torch.gather(pp, -1, r.long().unsqueeze(-1)).squeeze(-1)
        pick.view(-1).copy_(r)
        p.view(-1).copy_(pp.reshape(-1))
        scale.view(-1).copy_((1.0 / (torch.sqrt(pr) + 1e-10)).to(torch.complex64))
        return 0

    def tcg_kraus_pick_backward(self, gs, pk, pp, K_, cf, S, B, gev, st):
        r = pk.reshape(-1).long()
        pr = pp.reshape(B, K_).gather(-1, r.unsqueeze(-1)).squeeze(-1)
        den = torch.sqrt(pr) + 1e-10
        gp = -gs.reshape(-1).real / (den * den) / (2 * torch.sqrt(pr))
        gev.view(B, S).copy_((gp.unsqueeze(-1) * cf[r]).to(torch.complex64))
        return 0


def test_kraus_pick_functions_under_vmap_and_grad(monkeypatch):
    """KrausPickFn / KrausPickBwdFn wiring: values and gradients of
    vmap(grad_and_value(f)) through the Functions equal those of the same
    steps written as torch operations -- batched and shared draws, batched
    and unbatched expectations, two chained channels -- and every tensor
    handed to the library has storage (no functorch wrapper reaches it)."""
    from tensorcircuit_gb300 import _native as nat
    from tensorcircuit_gb300 import engine as eng

    monkeypatch.setattr(nat, "load", lambda: _FakePickLib())
    monkeypatch.setattr(nat, "ptr", lambda t: (t.data_ptr(), t)[1])
    monkeypatch.setattr(nat, "check", lambda rc, name: None)
    monkeypatch.setattr(eng, "_stream", lambda: 0)
    g = torch.Generator().manual_seed(3)
    K_, S, B = 4, 16, 6
    coef = torch.rand(K_, S, generator=g) * 0.1 + 0.01
    W = torch.randn(S, S, generator=g) * 0.1
    theta = torch.randn(S, generator=g)
    a = torch.randn(B, S, generator=g)
    xb = torch.rand(B, generator=g) * 3

    def evf(t, shift):
        re = torch.sigmoid(t @ W + shift)
        return torch.complex(re, torch.zeros_like(re))

    def step_torch(ev, x):
        p = torch.real(ev) @ coef.t()
        r = _pick(x, torch.cumsum(p, -1), torch.device("cpu"))
        pr = torch.sum(torch.where(r.unsqueeze(-1) == torch.arange(K_), p, 0.0), -1)
        return (1.0 / (torch.sqrt(pr) + 1e-10)).to(torch.complex64)

    def step_fn(ev, x):
        return eng.KrausPickFn.apply(ev, coef, x)[1]

    def chained(step):
        def f(t, shift, x):
            s = step(evf(t, shift), x)
            s2 = step(evf(t * torch.real(s), 0.0), x * 0.5)
            return torch.real(s2) + 0.3 * torch.real(s)
        return f

    def shared(step):
        return lambda t, shift: torch.real(step(evf(t, shift), torch.tensor(1.3)))

    def unbatched_ev(step):
        return lambda t, x: torch.real(step(evf(t, 0.0), x))

    cases = [(chained, (None, 0, 0), (theta, a, xb)), (shared, (None, 0), (theta, a)),
             (unbatched_ev, (None, 0), (theta, xb))]
    for make, dims, args in cases:
        vg = [torch.func.vmap(torch.func.grad_and_value(make(s)), in_dims=dims)(*args) for s in (step_fn, step_torch)]
        torch.testing.assert_close(vg[0][1], vg[1][1], rtol=1e-6, atol=0)
        torch.testing.assert_close(vg[0][0], vg[1][0], rtol=1e-5, atol=1e-7)
    g1 = torch.func.grad(unbatched_ev(step_fn))(theta, xb[0])
    g0 = torch.func.grad(unbatched_ev(step_torch))(theta, xb[0])
    torch.testing.assert_close(g1, g0, rtol=1e-5, atol=1e-7)
