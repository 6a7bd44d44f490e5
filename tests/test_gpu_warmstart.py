"""GPU: the warm-start network's kernels against the float64 CPU oracle, and
a small end-to-end study showing what the trained network gains over random
starting angles."""

import numpy as np
import pytest
import torch

from oracle import mlp as om

pytestmark = pytest.mark.gpu


def test_mlp_forward_backward_match_oracle(tc):
    from tensorcircuit_gb300 import warmstart as ws

    net = ws.WarmStartMLP(seed=3)
    rng = np.random.default_rng(0)
    B = 300  # not a multiple of the 64-row tile
    x = rng.standard_normal((B, 31)).astype(np.float32)
    target = rng.uniform(-np.pi, np.pi, (B, 186)).astype(np.float32)
    Ws = [W.cpu().numpy() for W in net.W]
    bs = [b.cpu().numpy() for b in net.b]
    pred_o, cache = om.forward(x, Ws, bs)
    pred = net(torch.from_numpy(x)).cpu().numpy()
    # float32 accumulation vs float64 with the same bfloat16 activations
    np.testing.assert_allclose(pred, pred_o, atol=5e-3, rtol=2e-2)
    loss_o, dpred_o = om.periodic_loss(pred_o, target.astype(np.float64))
    dW_o, db_o = om.backward(dpred_o, Ws, cache)
    loss, grads = net.gradients(torch.from_numpy(x), torch.from_numpy(target))
    assert abs(loss - loss_o) < 1e-4 * max(1.0, abs(loss_o))
    for g, go in zip(grads, dW_o + db_o):
        go = np.asarray(go)
        err = np.abs(g.cpu().numpy() - go).max() / max(np.abs(go).max(), 1e-12)
        assert err < 2e-2, err


def test_adam_kernel_matches_oracle(tc):
    from tensorcircuit_gb300 import _native as nat

    rng = np.random.default_rng(1)
    n = 1000
    p = rng.standard_normal(n)
    m = np.zeros(n)
    v = np.zeros(n)
    pd = torch.tensor(p, dtype=torch.float32, device="cuda")
    md = torch.zeros(n, device="cuda")
    vd = torch.zeros(n, device="cuda")
    lib = nat.load()
    for step in range(1, 6):
        g = rng.standard_normal(n)
        gd = torch.tensor(g, dtype=torch.float32, device="cuda")
        nat.check(lib.tcg_adam_update(nat.ptr(pd), nat.ptr(gd), nat.ptr(md), nat.ptr(vd), n, 0.02, 0.9, 0.999,
                                      1e-8, step, torch.cuda.current_stream().cuda_stream))
        om.adam(p, g, m, v, step, 0.02)
    np.testing.assert_allclose(pd.cpu().numpy(), p, atol=1e-5)


def test_warm_start_study_small(tc):
    """256 training chains, 32 held-out: the network's angles start closer to
    the ground energy and reach the random start's final error in fewer
    Adam steps."""
    from tensorcircuit_gb300 import warmstart as ws

    r = ws.study(n_train=256, n_test=32, steps=60, gen_steps=120, epochs=150)
    print(r)
    assert r["fit_loss_first_last"][1] < r["fit_loss_first_last"][0]
    assert r["rel_err_median_warm"]["0"] < r["rel_err_median_random"]["0"]
    assert r["steps_to_target_median_warm"] < r["steps_to_target_median_random"]
