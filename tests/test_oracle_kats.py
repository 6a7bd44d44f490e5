"""CPU: pin the complex128 oracle to the reference's known-answer tests."""

import numpy as np
import pytest

from oracle import statevector as sv
from tests.golden import reference_kats as K


def _oracle_state(case):
    n = case["n"]
    inputs = case.get("inputs")
    if inputs is not None:
        inp = np.asarray(inputs, dtype=np.complex128).reshape(-1)
        ntot = int(round(np.log2(inp.size)))
        return sv.run_circuit(ntot, case["ops"], inp), ntot
    return sv.run_circuit(n, case["ops"]), n


def _query(case, psi, ntot):
    q = case["query"]
    n = case["n"]
    if q[0] == "amp":
        return psi[q[1]].real
    if q[0] == "bitstring":
        return psi[int(q[1], 2)].real
    if q[0] == "amp_complex":
        return psi[q[1]]
    if q[0] == "state":
        return psi
    if q[0] == "state4x4":
        return psi.reshape(4, 4)
    if q[0] == "prob":
        return sv.probability(psi)
    if q[0] == "ps":
        kw = dict(q[1])
        if "ps" in kw:
            ps = kw.pop("ps")
            kw = {"x": [i for i, c in enumerate(ps) if c == 1], "y": [i for i, c in enumerate(ps) if c == 2],
                  "z": [i for i, c in enumerate(ps) if c == 3]}
        return sv.expectation_ps(psi, ntot, **kw).real
    if q[0] == "expect_ops":
        kw = {"x": [], "y": [], "z": []}
        for name, idx in q[1]:
            kw[name].extend(idx)
        return sv.expectation_ps(psi, ntot, **kw).real
    raise KeyError(q[0])


@pytest.mark.parametrize("case", K.KATS, ids=[c["id"] for c in K.KATS])
def test_oracle_matches_reference_kat(case):
    psi, ntot = _oracle_state(case)
    got = _query(case, psi, ntot)
    np.testing.assert_allclose(got, case["expect"], atol=max(case["atol"], 1e-12))


@pytest.mark.parametrize("case", K.GATE_KATS, ids=[c["id"] for c in K.GATE_KATS])
def test_oracle_matches_reference_gate_kat(case):
    psi, ntot = _oracle_state(case)
    got = _query(case, psi, ntot)
    np.testing.assert_allclose(got, case["expect"], atol=max(case["atol"], 1e-12))


def test_oracle_rxx_equivalence():
    c = K.RXX_EQUIV
    a = sv.run_circuit(c["n"], c["ops_a"])
    b = sv.run_circuit(c["n"], c["ops_b"])
    np.testing.assert_allclose(a, b, atol=1e-12)


def test_oracle_duplicate_measurement_raises():
    psi = sv.run_circuit(2, [("h", (0,), {})])
    with pytest.raises(ValueError):
        sv.expectation_ps(psi, 2, x=[0], z=[0])


def test_oracle_sample_histogram():
    c = K.PROB_SAMPLE
    rng = np.random.default_rng(0)
    u = rng.uniform(size=c["shots"]).astype(np.float32)
    r = sv.sample_reference_fp32(c["p"], u)
    _, cnt = np.unique(r, return_counts=True)
    np.testing.assert_allclose(cnt - c["p"] * c["shots"], 0, atol=c["atol"])
    # the declared integer-CDF arithmetic draws from the same distribution
    amps = np.sqrt(c["p"]).astype(np.complex64)
    r2 = sv.sample_declared(amps, u)
    _, cnt2 = np.unique(r2, return_counts=True)
    np.testing.assert_allclose(cnt2 - c["p"] * c["shots"], 0, atol=c["atol"])


def test_declared_cdf_matches_fp64_when_exactly_representable():
    # amplitudes whose squares are dyadic: the integer CDF equals the exact one
    amps = np.array([0.5, 0.5, 0.5, 0.5], dtype=np.complex64)
    cdf = sv.declared_cdf(amps)
    np.testing.assert_array_equal(cdf, np.array([1, 2, 3, 4], dtype=np.uint64) << np.uint64(58))
    u = np.array([0.0, 0.2499, 0.25, 0.5, 0.74, 0.99], dtype=np.float32)
    ref = sv.sample_reference_fp32(np.abs(amps) ** 2, u)
    np.testing.assert_array_equal(sv.sample_declared(amps, u), ref)


def test_declared_sampling_agrees_with_fp32_reference_at_small_n():
    rng = np.random.default_rng(3)
    n = 8
    psi = (rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n))
    psi = (psi / np.linalg.norm(psi)).astype(np.complex64)
    u = rng.uniform(size=4096).astype(np.float32)
    a = sv.sample_declared(psi, u)
    b = sv.sample_reference_fp32(np.abs(psi) ** 2, u)
    # fp32 cumsum rounding moves a draw only when u falls within ~1e-7 of a
    # CDF step; at n=8 that is rare
    assert np.mean(a != b) < 0.01


def test_oracle_adjoint_gradient_matches_finite_differences():
    from tensorcircuit_gb300 import templates

    n, nl = 5, 2
    rng = np.random.default_rng(1)
    P = templates.hea_nparams(n, nl)
    params = rng.uniform(0, 2 * np.pi, P)
    layout = templates.hea_layout(n, nl)
    ops = [(name, q, {"theta": 0.0}) for name, q, k in layout]
    pidx = [k for _, _, k in layout]
    terms = templates.tfim_terms(n, -1.0, -1.0)
    v, g = sv.value_and_grad_adjoint(n, ops, pidx, params, terms)
    gfd = sv.grad_fd(n, ops, pidx, params, terms, eps=1e-4)
    np.testing.assert_allclose(g, gfd, atol=1e-7)
    psi = sv.run_circuit(n, [(name, q, {"theta": params[k]}) for name, q, k in layout])
    assert abs(v - sv.energy(psi, n, terms)) < 1e-12


def test_ps_xyz_roundtrip():
    from tensorcircuit_gb300 import quantum

    c = K.PS_XYZ
    assert quantum.xyz2ps(c["xyz"]) == c["ps"]
    assert quantum.xyz2ps(c["xyz"], 6) == c["ps6"]
    d = dict(c["xyz"])
    d.update({"y": []})
    assert quantum.ps2xyz(c["ps"]) == d
    assert quantum.ps2xyz(c["ps"] + [0]) == d


@pytest.mark.parametrize("case", K.KATS, ids=[c["id"] for c in K.KATS])
def test_device_oracle_matches_reference_kat(case):
    """The torch restatement (oracle/device.py, run here on the CPU) gives the
    same states as the numpy oracle on every known-answer case."""
    import torch

    from oracle import device as dv

    n = case["n"]
    inputs = case.get("inputs")
    if inputs is not None:
        inp = np.asarray(inputs, dtype=np.complex128).reshape(-1)
        ntot = int(round(np.log2(inp.size)))
        got = dv.run_circuit(ntot, case["ops"], "cpu", torch.from_numpy(inp))
    else:
        got = dv.run_circuit(n, case["ops"], "cpu")
    want, _ = _oracle_state(case)
    np.testing.assert_allclose(got.numpy(), want, atol=1e-12)


def test_device_oracle_random_circuits_and_adjoint():
    """Random circuits with every gate width (1..3 qubits, unordered qubit
    lists), Pauli expectations and the adjoint gradient: torch restatement vs
    numpy oracle."""
    import torch

    from oracle import device as dv
    from tests.test_plan_replay import random_gate_list

    rng = np.random.default_rng(5)
    for n in (3, 7, 10):
        gl = random_gate_list(n, 40, rng)
        want = sv.run_circuit(n, gl)
        got = dv.run_circuit(n, gl, "cpu")
        np.testing.assert_allclose(got.numpy(), want, atol=1e-12)
        for kw in ({"x": [0], "z": [n - 1]}, {"y": [1, 2]}, {"z": [0, n - 1]}):
            assert abs(dv.expectation_ps(got, n, **kw) - sv.expectation_ps(want, n, **kw)) < 1e-12
    n = 6
    ops = [("rx", (i,), {"theta": 0.0}) for i in range(n)] + [("rzz", (i, i + 1), {"theta": 0.0}) for i in range(n - 1)]
    pidx = list(range(len(ops)))
    params = rng.uniform(0, 2 * np.pi, len(ops))
    terms = [(-1.0, {"z": [i, i + 1]}) for i in range(n - 1)] + [(-0.7, {"x": [i]}) for i in range(n)]
    v0, g0 = sv.value_and_grad_adjoint(n, ops, pidx, params, terms)
    v1, g1 = dv.value_and_grad_adjoint(n, ops, pidx, params, terms, "cpu")
    assert abs(v0 - v1) < 1e-12
    np.testing.assert_allclose(g1, g0, atol=1e-9)


def test_cpu_baseline_restatements_match_oracle():
    """The timed CPU baselines compute what the oracle computes: the per-gate
    tensordot restatements (torch and numpy forms) of a Haar brick wall, and
    the taped-AD value+gradient of the HEA energy."""
    import torch

    from oracle import reference_algo as ra
    from tensorcircuit_gb300 import templates

    threads0 = torch.get_num_threads()  # the restatements set torch's thread count
    n = 9
    gl = templates.brickwall_gate_list(n, 6, 11)
    want = sv.run_circuit(n, gl)
    np.testing.assert_allclose(ra.run_gate_list_numpy(n, gl), want, atol=2e-6)
    np.testing.assert_allclose(ra.run_gate_list(n, gl, 2).numpy(), want, atol=2e-6)
    nl = 2
    layout = templates.hea_layout(n, nl)
    terms = templates.tfim_terms(n, -1.0, -1.0)
    params = np.random.default_rng(5).uniform(0, 2 * np.pi, (2, templates.hea_nparams(n, nl))).astype(np.float32)
    v, g = ra.vvag_hea(n, layout, terms, params, 2)
    ops = [(name, q, {"theta": 0.0}) for name, q, _ in layout]
    pidx = [k for _, _, k in layout]
    for b in range(2):
        ve, ge = sv.value_and_grad_adjoint(n, ops, pidx, params[b].astype(np.float64), terms)
        assert abs(v[b] - ve) < 1e-4
        np.testing.assert_allclose(g[b], ge, atol=1e-4)
    torch.set_num_threads(threads0)
