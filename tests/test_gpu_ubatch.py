"""GPU: uneven batches (many circuits of different sizes and depths, one
persistent launch per sweep) against the complex128 oracle and against the
engine's own per-circuit path."""

import numpy as np
import pytest
import torch

from oracle import statevector as sv

pytestmark = pytest.mark.gpu


def _qaoa_oracle(n, edges, p, params):
    from tensorcircuit_gb300 import templates

    gl = templates.qaoa_gate_list(n, edges, [0.0] * p, [0.0] * p)
    pidx = [None] * n
    for layer in range(p):
        pidx += [layer] * len(edges) + [p + layer] * n
    terms = [(-0.5, {"z": [a, b]}) for a, b in edges]
    v, g = sv.value_and_grad_adjoint(n, gl, pidx, np.asarray(params, np.float64), terms)
    return v + 0.5 * len(edges), g


def _mixed_spec():
    """A non-QAOA circuit: every rotation family, exp1 Pauli strings, a
    constant Haar gate and an energy with X and Y terms."""
    from tensorcircuit_gb300 import templates

    X = np.array([[0, 1], [1, 0]], np.complex128)
    Y = np.array([[0, -1j], [1j, 0]], np.complex128)
    u = templates.haar_unitary(4, np.random.default_rng(9))
    n = 9
    ops = [("h", (0,), None), ("rx", (1,), 0), ("ry", (2,), 1), ("rz", (0,), 2), ("rxx", (3, 8), 3),
           ("ryy", (4, 5), 4), ("rzz", (0, 7), 5), ("any", (2, 6), None), ("cnot", (1, 4), None),
           ("exp1", (6, 3), 6), ("rx", (8,), 1)]
    kw = {"any": {"unitary": u}, "exp1": {"unitary": np.kron(X, Y)}}

    def build(c, params):
        for name, q, k in ops:
            extra = kw.get(name, {})
            if k is None:
                getattr(c, name)(*q, **extra)
            else:
                getattr(c, name)(*q, theta=params[k], **extra)

    terms = [(0.8, {"x": [2], "z": [0]}), (-0.3, {"y": [5, 8]}), (1.1, {"z": [6]})]

    def oracle(params):
        gl = [(name, q, dict(kw.get(name, {}), **({} if k is None else {"theta": 0.0}))) for name, q, k in ops]
        pidx = [k for _, _, k in ops]
        v, g = sv.value_and_grad_adjoint(n, gl, pidx, np.asarray(params, np.float64), terms)
        return v + 0.25, g

    return (n, build, 7, terms, 0.25), oracle


def test_uneven_batch_matches_oracle(tc):
    from tensorcircuit_gb300 import batch, templates

    rng = np.random.default_rng(17)
    specs, oracles = [], []
    for n, p in [(8, 2), (10, 1), (12, 3), (8, 4), (14, 2)]:
        edges = templates.random_regular_graph(3, n, rng)
        specs.append(batch.qaoa_spec(n, edges, p))
        oracles.append(lambda prm, n=n, e=edges, p=p: _qaoa_oracle(n, e, p, prm))
    s, o = _mixed_spec()
    specs.append(s)
    oracles.append(o)
    ub = batch.UnevenBatch(specs, graph=False)
    params = [rng.uniform(0, np.pi, sp[2]).astype(np.float32) for sp in specs]
    e, g = ub.value_and_grad(params)
    ub.check()
    gs = ub.split(g)
    for i, (prm, orc) in enumerate(zip(params, oracles)):
        ve, ge = orc(prm.astype(np.float64))
        assert abs(e[i].item() - ve) <= 1e-5 * max(1.0, abs(ve)), (i, e[i].item(), ve)
        np.testing.assert_allclose(gs[i].cpu().numpy(), ge, atol=2e-5 * max(1.0, np.abs(ge).max()))
    # value-only call leaves the final states readable
    e2, _ = ub.value_and_grad(params, grad=False)
    np.testing.assert_array_equal(e2.cpu().numpy(), e.cpu().numpy())
    st = ub.state(0).cpu().numpy()
    assert abs(np.linalg.norm(st) - 1.0) < 1e-5


def test_uneven_batch_tile_widths_agree(tc):
    from tensorcircuit_gb300 import batch, templates

    rng = np.random.default_rng(5)
    specs = []
    for n in (12, 13, 16, 12, 18):
        specs.append(batch.qaoa_spec(n + (n % 2), templates.random_regular_graph(3, n + (n % 2), rng),
                                     int(rng.integers(1, 5))))
    params = torch.tensor(np.concatenate([rng.uniform(0, np.pi, sp[2]) for sp in specs]), dtype=torch.float32)
    out = {}
    for L in (12, 10, 8):
        ub = batch.UnevenBatch(specs, tile_bits=L, graph=False)
        out[L] = ub.value_and_grad(params)
        ub.check()
    for L in (10, 8):
        np.testing.assert_allclose(out[L][0].cpu().numpy(), out[12][0].cpu().numpy(), atol=2e-5)
        np.testing.assert_allclose(out[L][1].cpu().numpy(), out[12][1].cpu().numpy(), atol=5e-5)


def test_uneven_batch_fusion_widths_match_oracle(tc):
    """Z-rotation fusion widths 1 (every rzz on its own), 3 and the default
    (runs of up to 32) give the oracle's energies and gradients, and the
    autotuner searches both knobs and keeps its fastest candidate."""
    from tensorcircuit_gb300 import batch, templates

    rng = np.random.default_rng(23)
    specs, oracles = [], []
    for n, p in [(8, 2), (12, 3), (10, 1)]:
        edges = templates.random_regular_graph(3, n, rng)
        specs.append(batch.qaoa_spec(n, edges, p))
        oracles.append(lambda prm, n=n, e=edges, p=p: _qaoa_oracle(n, e, p, prm))
    params = [rng.uniform(0, np.pi, sp[2]).astype(np.float32) for sp in specs]
    for z in (1, 3, 0):
        ub = batch.UnevenBatch(specs, tile_bits=8, zrun_max=z, graph=False)
        assert ub.zrun_max == z and not ub.tuned
        e, g = ub.value_and_grad(params)
        ub.check()
        gs = ub.split(g)
        for i, (prm, orc) in enumerate(zip(params, oracles)):
            ve, ge = orc(prm.astype(np.float64))
            assert abs(e[i].item() - ve) <= 1e-5 * max(1.0, abs(ve)), (z, i, e[i].item(), ve)
            np.testing.assert_allclose(gs[i].cpu().numpy(), ge, atol=2e-5 * max(1.0, np.abs(ge).max()))
    batch._TUNED.clear()
    ub = batch.UnevenBatch(specs, graph=False)
    assert ub.tuned
    assert {z for _, z, _ in ub.tune_log} == set(batch.ZRUN_WIDTHS)
    assert {L for L, _, _ in ub.tune_log} == {8}  # the smallest circuit bounds the tile width
    fastest = min(ub.tune_log, key=lambda x: x[2])
    assert (ub.tile_bits, ub.zrun_max) == fastest[:2]


def test_uneven_batch_c4_graph_replay_vs_per_circuit_engine(tc):
    """512 QAOA MaxCut circuits, n ~ U{12, 14, ..., 24}, random 3-regular
    graphs, p ~ U{1..6}, gamma, beta ~ U[0, pi): the captured-graph batch
    agrees with the eager batch and, on a sample of circuits, with the
    engine's per-circuit Circuit + value_and_grad path."""
    from tensorcircuit_gb300 import batch, templates

    specs, params = templates.qaoa_uneven_workload(512, seed=5)
    ub = batch.UnevenBatch(specs, graph=True)
    flat = torch.tensor(np.concatenate(params), dtype=torch.float32, device="cuda")
    e_eager, g_eager = batch.UnevenBatch(specs, tile_bits=ub.tile_bits, zrun_max=ub.zrun_max,
                                         graph=False).value_and_grad(flat)
    e1, g1 = ub.value_and_grad(flat)
    e2, g2 = ub.value_and_grad(flat)
    ub.check()
    assert torch.equal(e1, e2) and torch.equal(g1, g2)
    assert torch.equal(e1, e_eager) and torch.equal(g1, g_eager)
    K = tc.set_backend("pytorch")
    gs = ub.split(g1)
    rng = np.random.default_rng(0)
    for i in rng.choice(len(specs), 6, replace=False):
        n, build, npar, terms, offset = specs[i]

        def f(p, n=n, build=build, terms=terms, offset=offset):
            c = tc.Circuit(n)
            build(c, p)
            return templates.energy(c, terms) + offset

        v, g = K.value_and_grad(f)(torch.tensor(params[i], dtype=torch.float32, device="cuda"))
        assert abs(v.item() - e1[i].item()) <= 1e-5 * max(1.0, abs(v.item()))
        np.testing.assert_allclose(gs[i].cpu().numpy(), g.cpu().numpy(), atol=1e-4)


def test_uneven_batch_small_circuits_and_errors(tc):
    """Circuits down to 6 qubits with the smallest tile width, a circuit
    with no parameters, and the error mapping of invalid batches."""
    from tensorcircuit_gb300 import batch, templates

    def fixed(c, params):
        c.h(0)
        c.cnot(0, 3)
        c.rzz(1, 5, theta=0.4)

    rng = np.random.default_rng(3)
    specs = [batch.qaoa_spec(6, templates.random_regular_graph(3, 6, rng), 2),
             (6, fixed, 0, [(1.0, {"z": [0, 3]}), (0.5, {"x": [1]})], 0.0),
             batch.qaoa_spec(8, templates.random_regular_graph(3, 8, rng), 1)]
    ub = batch.UnevenBatch(specs, tile_bits=6, graph=False)
    params = [rng.uniform(0, np.pi, s[2]).astype(np.float32) for s in specs]
    e, g = ub.value_and_grad(params)
    ub.check()
    want0, g0 = _qaoa_oracle(6, [tuple(t["z"]) for _, t in specs[0][3]], 2, params[0].astype(np.float64))
    assert abs(e[0].item() - want0) < 1e-5
    np.testing.assert_allclose(ub.split(g)[0].cpu().numpy(), g0, atol=2e-5)
    psi = sv.run_circuit(6, [("h", (0,), {}), ("cnot", (0, 3), {}), ("rzz", (1, 5), {"theta": 0.4})])
    want1 = (sv.expectation_ps(psi, 6, z=[0, 3]) + 0.5 * sv.expectation_ps(psi, 6, x=[1])).real
    assert abs(e[1].item() - want1) < 1e-5
    with pytest.raises(ValueError):
        batch.UnevenBatch(specs, tile_bits=7, graph=False)  # wider than the 6-qubit circuits
    with pytest.raises(ValueError):
        ub.value_and_grad(np.zeros(3, np.float32))  # wrong parameter count


def test_uneven_batch_wait_limit_runs_out_and_is_reported(tc):
    """The persistent kernel's bounded dependency wait, made to run out
    without faulting anything: a dependency count no sweep reaches is written
    into the first segment's descriptor from the host and the wait limit is
    50 ms (a legitimate wait of a first, cold call can exceed 1 ms).  The
    launch must finish, tcg_ubatch_check must report
    TCG_ERR_TIMEOUT once (the flag then clears), and with the count restored
    the batch computes correct values again."""
    from tensorcircuit_gb300 import _native as nat
    from tensorcircuit_gb300 import batch, templates

    lib = nat.load()
    rng = np.random.default_rng(23)
    specs = [batch.qaoa_spec(n, templates.random_regular_graph(3, n, rng), 2) for n in (8, 10, 12)]
    ub = batch.UnevenBatch(specs, tile_bits=6, graph=False, wait_limit_ns=50_000_000)
    params = torch.tensor(np.concatenate([rng.uniform(0, np.pi, sp[2]) for sp in specs]), dtype=torch.float32)
    e0, g0 = ub.value_and_grad(params)
    ub.check()
    nat.check(lib.tcg_debug_ubatch_set_need(ub.h.handle, 0, 0, 0xFFFFFFF0), "inject")
    ub.value_and_grad(params)
    torch.cuda.synchronize()
    with pytest.raises(RuntimeError, match="ran out of time"):
        ub.check()
    ub.check()  # the flag was cleared by the check that reported it
    nat.check(lib.tcg_debug_ubatch_set_need(ub.h.handle, 0, 0, 0), "restore")
    e1, g1 = ub.value_and_grad(params)
    ub.check()
    assert torch.equal(e1, e0) and torch.equal(g1, g0)
