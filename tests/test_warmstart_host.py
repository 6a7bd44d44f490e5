"""CPU: the warm-start study's exact ground energy and input features."""

import numpy as np

from oracle import mlp as om
from tensorcircuit_gb300 import warmstart as ws


def test_free_fermion_energy_matches_dense_diagonalisation():
    for n, seed in [(4, 0), (6, 1), (8, 2)]:
        J, h = ws.tfim_instances(3, seed, n=n)
        e0 = ws.free_fermion_e0(J, h)
        for i in range(3):
            assert abs(e0[i] - om.tfim_dense_e0(J[i], h[i])) < 1e-10


def test_instances_and_features():
    J, h = ws.tfim_instances(1000, 6)
    assert J.shape == (1000, 15) and h.shape == (1000, 16)
    assert 0.5 <= J.min() and J.max() <= 1.5 and 0.2 <= h.min() and h.max() <= 2.0
    f = ws.features(J, h).numpy()
    assert f.shape == (1000, 31)
    assert np.all(np.abs(f.mean(0)) < 0.15) and np.all(np.abs(f.std(0) - 1) < 0.15)
    assert ws.n_params() == 186


def test_bf16_rounding_oracle():
    x = np.array([1.0, 1.00390625, 1.005859375, -3.14159265, 1e-30], dtype=np.float32)
    r = om.bf16_round(x)
    assert r[0] == 1.0 and r[1] == 1.0   # tie to even
    assert r[2] == 1.0078125
    assert abs(r[3] + 3.140625) < 1e-12
