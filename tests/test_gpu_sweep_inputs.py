"""GPU: sweeps whose first pass reads its input elsewhere.

``tcg_forward_from`` (input rows read in place, one shared row with stride 0),
``tcg_backward_from`` (output states read, working copy written) and
``tcg_pauli_accumulate_ex`` with ``TCG_ACC_OVERWRITE`` (mu written, never
read) run the same kernels as their in-place forms with other load
pointers, so their results must be bitwise equal to the in-place forms on
the same inputs -- on the generic kernels (first two calls of a plan), the
specialised ones (later calls) and the tensor-core passes.
"""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _random_gates(n, ngates, rng, grad):
    """Dense 1- and 2-qubit gates with random (unnormalised) matrices."""
    gates, off = [], 0
    from tensorcircuit_gb300 import _native as nat

    for i in range(ngates):
        if rng.random() < 0.5:
            q = (int(rng.integers(n)),)
        else:
            q = tuple(int(x) for x in rng.choice(n, 2, replace=False))
        size = 4 ** len(q)
        gates.append((nat.TCG_GATE_DENSE, q, off, off if grad else -1))
        off += size
    mats = rng.standard_normal(off) + 1j * rng.standard_normal(off)
    return gates, torch.tensor(mats, dtype=torch.complex64, device="cuda")


def _rand_states(B, n, seed):
    g = torch.Generator(device="cpu").manual_seed(seed)
    x = torch.randn(B, 1 << n, dtype=torch.complex64, generator=g)
    return (x / torch.linalg.vector_norm(x, dim=1, keepdim=True)).cuda()


@pytest.mark.parametrize("policy", [0, 1])
def test_forward_from_equals_in_place(tc, policy):
    from tensorcircuit_gb300 import _native as nat
    from tensorcircuit_gb300 import engine as eng

    lib = nat.load()
    prev = lib.tcg_set_tensor_policy(-1)
    lib.tcg_set_tensor_policy(policy)
    try:
        n, B = 14, 3
        gates, mats = _random_gates(n, 60, np.random.default_rng(1), grad=False)
        plan = eng.GatePlan(n, gates, mats.numel())
        st = torch.cuda.current_stream().cuda_stream
        rows = _rand_states(B, n, 2)
        one = _rand_states(1, n, 3)[0]
        for rep in range(4):  # generic kernels first, then the specialised ones
            for src, stride in ((rows, 1 << n), (one, 0)):
                want = (src if stride else one.expand(B, -1)).clone().contiguous()
                nat.check(lib.tcg_forward(plan.handle, want.data_ptr(), B, mats.data_ptr(), 0, st), "forward")
                got = torch.full((B, 1 << n), float("nan"), dtype=torch.complex64, device="cuda")
                src_before = src.clone()
                nat.check(lib.tcg_forward_from(plan.handle, src.data_ptr(), stride, got.data_ptr(), B,
                                               mats.data_ptr(), 0, st), "forward_from")
                torch.cuda.synchronize()
                assert torch.equal(got, want), (rep, stride)
                assert torch.equal(src, src_before)
        plan.check()
    finally:
        lib.tcg_set_tensor_policy(prev)


def test_backward_from_equals_in_place(tc):
    from tensorcircuit_gb300 import _native as nat
    from tensorcircuit_gb300 import engine as eng

    lib = nat.load()
    n, B = 13, 2
    gates, mats = _random_gates(n, 40, np.random.default_rng(4), grad=True)
    M = mats.numel()
    plan = eng.GatePlan(n, gates, M)
    st = torch.cuda.current_stream().cuda_stream
    psi_out = _rand_states(B, n, 5)
    mu0 = _rand_states(B, n, 6)
    nbytes = int(lib.tcg_backward_scratch_bytes(plan.handle, B))
    scratch = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    for rep in range(4):
        psi_a, mu_a = psi_out.clone(), mu0.clone()
        g_a = torch.zeros(B, M, dtype=torch.complex64, device="cuda")
        nat.check(lib.tcg_backward(plan.handle, psi_a.data_ptr(), mu_a.data_ptr(), B, mats.data_ptr(), 0,
                                   g_a.data_ptr(), M, scratch.data_ptr(), nbytes, st), "backward")
        psi_b = torch.full_like(psi_out, float("nan"))
        mu_b = mu0.clone()
        g_b = torch.zeros(B, M, dtype=torch.complex64, device="cuda")
        before = psi_out.clone()
        nat.check(lib.tcg_backward_from(plan.handle, psi_out.data_ptr(), psi_b.data_ptr(), mu_b.data_ptr(), B,
                                        mats.data_ptr(), 0, g_b.data_ptr(), M, scratch.data_ptr(), nbytes, st),
                  "backward_from")
        torch.cuda.synchronize()
        assert torch.equal(psi_out, before)
        assert torch.equal(psi_b, psi_a), rep
        assert torch.equal(mu_b, mu_a), rep
        assert torch.equal(g_b, g_a), rep


def test_accumulate_overwrite_equals_zero_then_add(tc):
    from tensorcircuit_gb300 import _native as nat
    from tensorcircuit_gb300 import engine as eng
    from tensorcircuit_gb300 import templates

    lib = nat.load()
    n, B = 16, 3
    terms = templates.tfim_terms(n, -1.0, -0.7)
    spec = tuple(eng.pauli_masks(n, t.get("x", []), t.get("y", []), t.get("z", [])) for _, t in terms)
    tp = eng.term_plan(n, spec)
    st = torch.cuda.current_stream().cuda_stream
    psi = _rand_states(B, n, 7)
    coef = torch.tensor(np.random.default_rng(8).standard_normal((B, len(spec))), dtype=torch.float32,
                        device="cuda")
    for rep in range(4):
        want = torch.zeros_like(psi)
        nat.check(lib.tcg_pauli_accumulate(tp.handle, psi.data_ptr(), want.data_ptr(), B, coef.data_ptr(),
                                           len(spec), st), "accumulate")
        got = torch.full_like(psi, float("nan"))
        nat.check(lib.tcg_pauli_accumulate_ex(tp.handle, psi.data_ptr(), got.data_ptr(), B, coef.data_ptr(),
                                              len(spec), nat.TCG_ACC_OVERWRITE, st), "accumulate_ex")
        torch.cuda.synchronize()
        assert torch.equal(got, want), rep
    with pytest.raises(ValueError):
        nat.check(lib.tcg_pauli_accumulate_ex(tp.handle, psi.data_ptr(), got.data_ptr(), B, coef.data_ptr(),
                                              len(spec), 2, st), "accumulate_ex")


def test_forward_from_without_gates_copies_the_input(tc):
    from tensorcircuit_gb300 import _native as nat
    from tensorcircuit_gb300 import engine as eng

    lib = nat.load()
    n, B = 8, 3
    plan = eng.GatePlan(n, [], 1)
    st = torch.cuda.current_stream().cuda_stream
    rows = _rand_states(B, n, 9)
    one = _rand_states(1, n, 10)[0]
    mats = torch.zeros(1, dtype=torch.complex64, device="cuda")
    for src, stride, want in ((rows, 1 << n, rows), (one, 0, one.expand(B, -1))):
        got = torch.full((B, 1 << n), float("nan"), dtype=torch.complex64, device="cuda")
        nat.check(lib.tcg_forward_from(plan.handle, src.data_ptr(), stride, got.data_ptr(), B, mats.data_ptr(), 0,
                                       st), "forward_from")
        torch.cuda.synchronize()
        assert torch.equal(got, want)
