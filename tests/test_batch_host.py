"""CPU: recording of uneven-batch circuits (symbolic parameters, matrix
layout, parameter map) -- everything the batch does before the GPU."""

import numpy as np
import pytest

from tensorcircuit_gb300 import _native as nat
from tensorcircuit_gb300 import batch, templates


def test_param_refs_scale_and_index():
    pv = batch.ParamVector(4)
    r = -0.5 * pv[3] / 2
    assert (r.k, r.scale) == (3, -0.25)
    assert pv[-1].k == 3
    with pytest.raises(IndexError):
        pv[4]


def test_qaoa_spec_layout():
    rng = np.random.default_rng(1)
    n, p = 12, 3
    edges = templates.random_regular_graph(3, n, rng)
    spec = batch.qaoa_spec(n, edges, p)
    assert spec[2] == 2 * p and spec[4] == 0.5 * len(edges)
    bc = batch.BatchCircuit(*spec)
    assert len(bc.gates) == n + p * (len(edges) + n)
    # H gates are constant dense matrices
    for kind, q, mo, go, codes in bc.gates[:n]:
        assert kind == nat.TCG_GATE_DENSE and go == -1
        np.testing.assert_allclose(bc.mat_const[mo:mo + 4], np.array([1, 1, 1, -1]) / np.sqrt(2), atol=1e-7)
    rot = bc.gates[n:]
    for layer in range(p):
        blk = rot[layer * (len(edges) + n):(layer + 1) * (len(edges) + n)]
        for kind, q, mo, go, codes in blk[:len(edges)]:
            assert kind == nat.TCG_GATE_PAULI_ROT and codes == (3, 3) and go == mo
            assert bc.mat_param[mo] == layer and bc.mat_scale[mo] == 1.0   # exp1(ZZ, gamma)
        for kind, q, mo, go, codes in blk[len(edges):]:
            assert codes == (1,) and bc.mat_param[mo] == p + layer and bc.mat_scale[mo] == 0.5  # rx(beta)
    assert len(bc.terms) == len(edges)
    for (cf, (xm, zm)), (a, b) in zip(bc.terms, edges):
        assert cf == -0.5 and xm == 0 and zm == (1 << (n - 1 - a)) | (1 << (n - 1 - b))


def test_batch_rejects_non_rotation_parameters():
    def build(c, params):
        c.cphase(0, 1, theta=params[0])

    with pytest.raises(NotImplementedError):
        batch.BatchCircuit(8, build, 1, [])


def test_constant_rotation_angles_become_constants():
    def build(c, params):
        c.rx(0, theta=0.3)
        c.rzz(1, 2, theta=params[0])

    bc = batch.BatchCircuit(8, build, 1, [(1.0, {"z": [0]})])
    k0, q0, mo0, go0, c0 = bc.gates[0]
    assert go0 == -1 and bc.mat_param[mo0] == -1
    np.testing.assert_allclose(bc.mat_const[mo0], np.exp(0.15j), atol=1e-7)
    assert bc.mat_param[bc.gates[1][2]] == 0 and bc.mat_scale[bc.gates[1][2]] == 0.5


def test_uneven_workload_shape():
    specs, params = templates.qaoa_uneven_workload(64, seed=5)
    ns = [s[0] for s in specs]
    assert all(n % 2 == 0 and 12 <= n <= 24 for n in ns)
    assert all(1 <= s[2] // 2 <= 6 and len(p) == s[2] for s, p in zip(specs, params))
    assert all(0 <= x < np.pi for p in params for x in p)


def test_autotune_coordinate_search():
    """Every tile width at the first fusion width, then the other fusion
    widths at the fastest tile width; the fastest pair wins, ties keep the
    first candidate."""
    cost = {(12, 0): 5.0, (11, 0): 4.0, (10, 0): 6.0, (11, 16): 3.5, (11, 8): 3.9, (11, 1): 9.0}
    calls = []

    def timed(L, z):
        calls.append((L, z))
        return cost[(L, z)]

    assert batch.coordinate_search([12, 11, 10], [0, 16, 8, 1], timed) == (11, 16)
    assert calls == [(12, 0), (11, 0), (10, 0), (11, 16), (11, 8), (11, 1)]
    # a single fusion width tunes the tile width only
    calls.clear()
    assert batch.coordinate_search([12, 11, 10], [0], timed) == (11, 0)
    assert calls == [(12, 0), (11, 0), (10, 0)]
    # ties keep the earlier candidate
    assert batch.coordinate_search([9, 8], [0, 4], lambda L, z: 1.0) == (9, 0)


def test_fusion_width_tuned_only_with_z_runs():
    """The Z-rotation fusion width changes only circuits with two or more
    Z-string rotations; batches without them tune the tile width alone."""
    rng = np.random.default_rng(3)
    qaoa = batch.BatchCircuit(*batch.qaoa_spec(8, templates.random_regular_graph(3, 8, rng), 1))
    assert batch._has_zruns([qaoa])

    def build(c, params):
        c.rx(0, theta=params[0])
        c.rzz(1, 2, theta=params[1])
        c.ry(3, theta=params[0])

    single = batch.BatchCircuit(8, build, 2, [(1.0, {"z": [0]})])
    assert not batch._has_zruns([single])
    assert batch.ZRUN_WIDTHS[0] == 0 and 1 in batch.ZRUN_WIDTHS
    # argument checks come before any device work
    spec = batch.qaoa_spec(8, templates.random_regular_graph(3, 8, rng), 1)
    with pytest.raises(ValueError):
        batch.UnevenBatch([spec], tile_bits=8, zrun_max=33)
    with pytest.raises(ValueError):
        batch.UnevenBatch([spec], tile_bits=9)  # wider than the 8-qubit circuit
