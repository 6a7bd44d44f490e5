"""GPU: the tensor-core passes (fused 6-qubit blocks as complex GEMMs on
tcgen05, fp16 hi/lo operands, fp32 accumulation).

* the MMA probe through the C ABI against a float32 matmul of the same fp16
  operands (layout, descriptors, tensor-memory readback in isolation);
* brick walls and random circuits with every pass that qualifies forced onto
  the tensor cores, against the complex128 oracle and the register path;
* batches of unnormalised input states (the per-tile power-of-two scaling);
* the bounded-wait flag stays clear.
"""

import numpy as np
import pytest
import torch

from oracle import device as dv
from oracle import statevector as sv

pytestmark = pytest.mark.gpu


@pytest.fixture
def policy():
    from tensorcircuit_gb300 import _native as nat

    lib = nat.load()
    prev = lib.tcg_set_tensor_policy(-1)

    def set_(p):
        lib.tcg_set_tensor_policy(p)

    yield set_
    lib.tcg_set_tensor_policy(prev)


@pytest.mark.parametrize("k,n", [(16, 32), (64, 64), (32, 256), (48, 96)])
def test_tc_mma_probe_matches_matmul(tc, k, n):
    from tensorcircuit_gb300 import _native as nat

    lib = nat.load()
    g = torch.Generator(device="cpu").manual_seed(k * 1000 + n)
    a = torch.randn(128, k, generator=g).to(torch.float16).cuda()
    b = torch.randn(n, k, generator=g).to(torch.float16).cuda()
    d = torch.full((128, n), float("nan"), device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    nat.check(lib.tcg_debug_tc_mma(a.data_ptr(), b.data_ptr(), d.data_ptr(), k, n, err.data_ptr(), st), "tc_mma")
    torch.cuda.synchronize()
    assert err.item() == 0
    want = a.float() @ b.float().T
    torch.testing.assert_close(d, want, rtol=1e-5, atol=1e-4)


def _state(c):
    return c.state()


@pytest.mark.parametrize("n,depth", [(12, 8), (16, 12), (20, 20)])
def test_tc_brickwall_matches_oracle_and_register_path(tc, policy, n, depth):
    from tensorcircuit_gb300 import circuit as cmod
    from tensorcircuit_gb300 import templates

    gl = templates.brickwall_gate_list(n, depth, 3)
    policy(1)
    c = templates.apply_gate_list(tc.Circuit(n), gl)
    psi_tc = c.state().clone()
    entry = cmod._entries[cmod._struct_key(n, c._ops)]
    ntc = entry.plan.tensor_passes()
    assert ntc == entry.plan.npasses, (ntc, entry.plan.npasses)
    entry.plan.check()
    policy(0)
    psi_reg = templates.apply_gate_list(tc.Circuit(n), gl).state()
    ref = dv.run_circuit(n, gl, "cuda")
    e_tc = torch.linalg.vector_norm(psi_tc.to(torch.complex128) - ref).item()
    e_reg = torch.linalg.vector_norm(psi_reg.to(torch.complex128) - ref).item()
    assert e_tc < 1e-5, e_tc
    assert e_reg < 1e-5, e_reg
    torch.testing.assert_close(psi_tc, psi_reg, rtol=0, atol=2e-6)


@pytest.mark.parametrize("seed", [0, 1, 2, 3])
def test_tc_random_circuits_match_oracle(tc, policy, seed):
    from tests.test_plan_replay import random_gate_list

    from tensorcircuit_gb300 import templates

    rng = np.random.default_rng(100 + seed)
    n = 12 + 2 * seed
    gl = random_gate_list(n, 150, rng)
    policy(1)
    c = templates.apply_gate_list(tc.Circuit(n), gl)
    psi = c.state()
    want = dv.run_circuit(n, gl, "cuda")
    assert torch.linalg.vector_norm(psi.to(torch.complex128) - want).item() < 1e-5
    zz = c.expectation_ps(z=[0, n - 1]).real.item()
    assert abs(zz - dv.expectation_ps(want, n, z=[0, n - 1]).real) < 1e-5


def test_tc_batched_unnormalised_inputs(tc, policy):
    """A batch of three input states of very different norms (1e-3, 1, 1e3)
    through one plan via the C ABI: every tile is rescaled before each block,
    so the result is the oracle's up to float32 rounding in all three."""
    from tensorcircuit_gb300 import _native as nat
    from tensorcircuit_gb300 import circuit as cmod
    from tensorcircuit_gb300 import templates

    lib = nat.load()
    n, B = 16, 3
    gl = templates.brickwall_gate_list(n, 12, 7)
    c = templates.apply_gate_list(tc.Circuit(n), gl)
    entry = cmod._build_entry(n, c._ops)
    mats = entry.const_block(torch.device("cuda"))
    g = torch.Generator(device="cpu").manual_seed(3)
    psi0 = torch.randn(B, 1 << n, dtype=torch.complex128, generator=g)
    psi0 /= torch.linalg.vector_norm(psi0, dim=1, keepdim=True)
    psi0 *= torch.tensor([1e-3, 1.0, 1e3], dtype=torch.float64)[:, None]
    psi = psi0.to(torch.complex64).cuda().contiguous()
    policy(1)
    st = torch.cuda.current_stream().cuda_stream
    nat.check(lib.tcg_forward(entry.plan.handle, psi.data_ptr(), B, mats.data_ptr(), 0, st), "forward")
    nat.check(lib.tcg_plan_check(entry.plan.handle, st), "plan_check")
    for b in range(B):
        ref = dv.run_circuit(n, gl, "cuda", psi0[b].to(torch.complex64).cuda())
        scale = torch.linalg.vector_norm(ref).item()
        err = torch.linalg.vector_norm(psi[b].to(torch.complex128) - ref).item() / scale
        assert err < 1e-5, (b, err)


def test_tc_zero_state_tiles(tc, policy):
    """Tiles that are exactly zero (a product state's support) pass through
    the scaling without producing NaN or Inf."""
    from tensorcircuit_gb300 import templates

    n = 14
    gl = [("any", (0, 1), {"unitary": templates.haar_unitary(4, np.random.default_rng(1))})]
    gl += [("cnot", (1, 2), {}), ("h", (3,), {})]
    policy(1)
    psi = templates.apply_gate_list(tc.Circuit(n), gl).state()
    assert torch.isfinite(torch.view_as_real(psi)).all()
    want = dv.run_circuit(n, gl, "cuda")
    assert torch.linalg.vector_norm(psi.to(torch.complex128) - want).item() < 1e-6


def _two_plans_same_structure(tc, n, depth):
    """Two brick walls with the same gate layout and different matrices: one
    plan, two rows of gate matrices."""
    from tensorcircuit_gb300 import circuit as cmod
    from tensorcircuit_gb300 import templates

    gls = [templates.brickwall_gate_list(n, depth, s) for s in (11, 12)]
    ents = [cmod._build_entry(n, templates.apply_gate_list(tc.Circuit(n), gl)._ops) for gl in gls]
    mats = [e.const_block(torch.device("cuda")) for e in ents]
    assert mats[0].shape == mats[1].shape
    return gls, ents[0].plan, mats


def test_tc_concurrent_streams_do_not_share_fused_matrices(tc, policy):
    """One plan, two streams, two different sets of gate matrices in flight
    at once: each call fuses into its own stream-ordered buffer, so both
    results match the oracle."""
    from tensorcircuit_gb300 import _native as nat

    lib = nat.load()
    n, B = 20, 4
    gls, plan, mats = _two_plans_same_structure(tc, n, 12)
    policy(1)
    assert plan.tensor_passes() == plan.npasses
    refs = [dv.run_circuit(n, gl, "cuda") for gl in gls]
    streams = [torch.cuda.Stream(), torch.cuda.Stream()]
    psis = []
    torch.cuda.synchronize()
    for rep in range(3):
        outs = []
        for k in (0, 1):
            psi = torch.zeros(B, 1 << n, dtype=torch.complex64, device="cuda")
            psi[:, 0] = 1
            outs.append(psi)
        torch.cuda.synchronize()
        for k in (0, 1):
            with torch.cuda.stream(streams[k]):
                nat.check(lib.tcg_forward(plan.handle, outs[k].data_ptr(), B, mats[k].data_ptr(), 0,
                                          streams[k].cuda_stream), "forward")
        torch.cuda.synchronize()
        psis.append(outs)
    plan.check()
    for outs in psis:
        for k in (0, 1):
            for b in range(B):
                err = torch.linalg.vector_norm(outs[k][b].to(torch.complex128) - refs[k]).item()
                assert err < 1e-5, (k, b, err)


def test_tc_forward_under_graph_capture(tc, policy):
    """A forward call captured into a CUDA graph owns its fused-matrix buffer
    (graph memory nodes): replays stay correct after eager calls with a
    larger batch in between."""
    from tensorcircuit_gb300 import _native as nat

    lib = nat.load()
    n = 16
    gls, plan, mats = _two_plans_same_structure(tc, n, 12)
    policy(1)
    refs = [dv.run_circuit(n, gl, "cuda") for gl in gls]

    def fresh(B):
        psi = torch.zeros(B, 1 << n, dtype=torch.complex64, device="cuda")
        psi[:, 0] = 1
        return psi

    def fwd(psi, k):
        st = torch.cuda.current_stream().cuda_stream
        nat.check(lib.tcg_forward(plan.handle, psi.data_ptr(), psi.shape[0], mats[k].data_ptr(), 0, st), "forward")

    # eager calls first: the plan's device program and specialised kernels
    # are set up outside the capture
    for _ in range(4):
        fwd(fresh(2), 0)
    psi_g = fresh(2)
    start = fresh(2)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        fwd(psi_g, 0)
    for rep in range(2):
        psi_g.copy_(start)
        g.replay()
        big = fresh(8)
        fwd(big, 1)
        torch.cuda.synchronize()
        for b in range(2):
            assert torch.linalg.vector_norm(psi_g[b].to(torch.complex128) - refs[0]).item() < 1e-5
        for b in range(8):
            assert torch.linalg.vector_norm(big[b].to(torch.complex128) - refs[1]).item() < 1e-5
    plan.check()
