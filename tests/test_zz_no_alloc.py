"""GPU: the allocation-free Pauli expectation entry point.

``tcg_expect_pauli_noalloc`` is for callers that cannot allocate device
memory (hosts whose device memory sits in a pool the C ABI cannot reach;
loops that cannot take cudaMalloc's implicit synchronisation).  It keeps its partial sums in a fixed
array inside the library.  Called through the C ABI twice in a row, it must
give what the planned entry point ``tcg_expect_pauli`` gives; oversized
requests must be refused.  (This file sorts last so that a run stopping at
its first failure has run every other test first.)
"""

import numpy as np
import pytest
import torch

from oracle import statevector as sv

pytestmark = pytest.mark.gpu


def _term_lists(n, rng, count):
    """Random Pauli strings as the reference's x/y/z qubit lists."""
    out = []
    for _ in range(count):
        q = rng.choice(n, int(rng.integers(1, min(6, n) + 1)), replace=False)
        kinds = rng.integers(1, 4, size=len(q))
        out.append({"x": [int(a) for a, k in zip(q, kinds) if k == 1],
                    "y": [int(a) for a, k in zip(q, kinds) if k == 2],
                    "z": [int(a) for a, k in zip(q, kinds) if k == 3]})
    return out


def _terms(n, rng, count, lists=None):
    from tensorcircuit_gb300 import engine as eng

    lists = _term_lists(n, rng, count) if lists is None else lists
    return [eng.pauli_masks(n, t["x"], t["y"], t["z"]) for t in lists]


def _planned(lib, nat, eng, psi, n, batch, terms):
    tp = eng.TermPlan(n, tuple(terms))
    out = torch.empty((batch, len(terms), 2), dtype=torch.float64, device="cuda")
    nbytes = int(lib.tcg_expect_scratch_bytes(tp.handle, batch))
    scratch = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    st = int(torch.cuda.current_stream().cuda_stream)
    nat.check(lib.tcg_expect_pauli(tp.handle, psi.data_ptr(), batch, out.data_ptr(), scratch.data_ptr(), nbytes, st))
    return out


def test_noalloc_expectation_matches_planned_entry_point(tc):
    from tensorcircuit_gb300 import _native as nat
    from tensorcircuit_gb300 import engine as eng

    lib = nat.load()
    rng = np.random.default_rng(77)
    n, batch = 14, 3
    lists = _term_lists(n, rng, 24)
    terms = _terms(n, rng, 24, lists)
    arr = (nat.TcgPauli * len(terms))()
    for i, (x, z) in enumerate(terms):
        arr[i].xmask, arr[i].zmask = x, z
    st = int(torch.cuda.current_stream().cuda_stream)
    for call in range(2):  # two calls in a row: the shared array keeps the last call's contents
        psi = torch.randn(batch, 1 << n, dtype=torch.complex64, device="cuda")
        psi = psi / torch.linalg.norm(psi, dim=-1, keepdim=True)
        want = _planned(lib, nat, eng, psi, n, batch, terms)
        got = torch.full((batch, len(terms), 2), float("nan"), dtype=torch.float64, device="cuda")
        rc = lib.tcg_expect_pauli_noalloc(psi.data_ptr(), n, batch, arr, len(terms), got.data_ptr(), st)
        assert rc == nat.TCG_OK, lib.tcg_status_string(rc)
        np.testing.assert_allclose(got.cpu().numpy(), want.cpu().numpy(), atol=2e-5)
        # and against the complex128 oracle's expectation_ps of the same strings
        host = psi.cpu().numpy().astype(np.complex128)
        ref = np.array([[sv.expectation_ps(host[b], n, **t) for t in lists] for b in range(batch)])
        g = got.cpu().numpy()
        np.testing.assert_allclose(g[..., 0] + 1j * g[..., 1], ref, atol=2e-5)


def test_noalloc_at_the_edge_of_its_limit(tc):
    """batch * nterms = 107 * 64 = 6848 fits the fixed array (checked against
    the planned entry point); 108 * 64 = 6912 is refused."""
    from tensorcircuit_gb300 import _native as nat
    from tensorcircuit_gb300 import engine as eng

    lib = nat.load()
    rng = np.random.default_rng(5)
    n = 6
    terms = _terms(n, rng, 64)
    arr = (nat.TcgPauli * len(terms))()
    for i, (x, z) in enumerate(terms):
        arr[i].xmask, arr[i].zmask = x, z
    st = int(torch.cuda.current_stream().cuda_stream)
    psi = torch.randn(108, 1 << n, dtype=torch.complex64, device="cuda")
    psi = psi / torch.linalg.norm(psi, dim=-1, keepdim=True)
    got = torch.full((108, 64, 2), float("nan"), dtype=torch.float64, device="cuda")
    rc = lib.tcg_expect_pauli_noalloc(psi.data_ptr(), n, 107, arr, 64, got.data_ptr(), st)
    assert rc == nat.TCG_OK, lib.tcg_status_string(rc)
    want = _planned(lib, nat, eng, psi[:107].contiguous(), n, 107, terms)
    np.testing.assert_allclose(got[:107].cpu().numpy(), want.cpu().numpy(), atol=2e-5)
    rc = lib.tcg_expect_pauli_noalloc(psi.data_ptr(), n, 108, arr, 64, got.data_ptr(), st)
    assert rc == nat.TCG_ERR_TOO_LARGE


def test_noalloc_rejects_requests_beyond_its_fixed_scratch(tc):
    from tensorcircuit_gb300 import _native as nat

    lib = nat.load()
    n = 8
    psi = torch.zeros(1 << n, dtype=torch.complex64, device="cuda")
    out = torch.empty((70, 2), dtype=torch.float64, device="cuda")
    arr = (nat.TcgPauli * 70)()
    st = int(torch.cuda.current_stream().cuda_stream)
    assert lib.tcg_expect_pauli_noalloc(psi.data_ptr(), n, 1, arr, 65, out.data_ptr(), st) == nat.TCG_ERR_TOO_LARGE
    assert b"capacity" in lib.tcg_status_string(nat.TCG_ERR_TOO_LARGE)
