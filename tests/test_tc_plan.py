"""CPU: the fused-block (tensor-core) program of forward plans, replayed in
numpy against the complex128 oracle.

Checks what the tensor-core pass kernel relies on before it runs on a GPU:
the planner's fusion of each pass's gates into blocks of at most 6 tile bits
(dependency order), the block-bit and column-bit maps (a bijection of the
tile), the gate-to-block bit positions the fusion kernel reads, and the
planar complex GEMM with its epilogue combination (Re y = D1[2i] - D2[2i+1],
Im y = D2[2i] + D1[2i+1]).  Passes that do not take the tensor-core path are
replayed with the register-path emulator.
"""

import numpy as np
import pytest

from oracle import statevector as sv
from tests.plan_emulator import Replay, dep
from tests.test_plan_replay import build_host, random_gate_list
from tensorcircuit_gb300 import _native as nat
from tensorcircuit_gb300 import templates

DENSE, DIAG, PROT = 0, 1, 2


def _sub(idx, G):
    s = np.zeros_like(idx)
    for q in range(G.k):
        s |= ((idx >> G.pos[q]) & 1) << (G.k - 1 - q)
    return s


def block_matrix(blk, gates, mats):
    """The fused 64 x 64 matrix of a block, as the fusion kernel builds it."""
    a = np.arange(64)
    F = np.eye(64, dtype=np.complex128)
    for G in gates[blk.gate_begin:blk.gate_end]:
        m = mats[G.mat_off:]
        if G.kind == DIAG:
            E = np.diag(m[_sub(a, G)].astype(np.complex128))
        elif G.kind == PROT:
            c, s = m[0].real, m[0].imag
            P = np.zeros((64, 64), np.complex128)
            sign = np.where([bin(int(x) & G.zmask).count("1") % 2 for x in a], -1.0, 1.0)
            P[a, a ^ G.xmask] = (-1j) ** G.nY * sign
            E = c * np.eye(64) - 1j * s * P
        else:
            D = 1 << G.k
            M = m[:D * D].reshape(D, D).astype(np.complex128)
            gmask = sum(1 << G.pos[q] for q in range(G.k))
            same = ((a[:, None] ^ a[None, :]) & ~gmask) == 0
            E = np.where(same, M[_sub(a, G)[:, None], _sub(a, G)[None, :]], 0)
        F = E @ F
    return F


def emulate_tc_pass(psi, P, blocks, gates, mats, n):
    lbits = [P.lbits[i] for i in range(P.L)]
    nl = [P.nlbits[i] for i in range(P.nnonlocal)]
    gl = dep(np.arange(1 << P.L), lbits)
    for blk in blocks:
        bb = [blk.bbits[i] for i in range(6)]
        cb = [blk.cbits[i] for i in range(6)]
        assert sorted(bb + cb) == list(range(12)), "block + column bits must partition the tile"
    mats_f = [block_matrix(blk, gates, mats) for blk in blocks]
    for tile in range(1 << (n - P.L)):
        base = int(dep(tile, nl))
        T = psi[base | gl].copy()
        for blk, F in zip(blocks, mats_f):
            tj = dep(np.arange(64), [blk.bbits[i] for i in range(6)])
            tn = dep(np.arange(64), [blk.cbits[i] for i in range(6)])
            idx = tj[:, None] | tn[None, :]
            assert len(np.unique(idx)) == 4096
            x = T[idx]
            A = np.empty((128, 64))
            A[0::2] = F.real
            A[1::2] = F.imag
            D1 = A @ x.real
            D2 = A @ x.imag
            y = (D1[0::2] - D2[1::2]) + 1j * (D2[0::2] + D1[1::2])
            T[idx] = y
        psi[base | gl] = T
    return psi


def emulate_forward(n, entry, mats):
    prog = nat.debug_program(entry.plan.handle, 0)
    tcp = nat.debug_tc_program(entry.plan.handle)
    by_pass = {d.pass_: d for d in tcp["passes"]}
    psi = np.zeros(1 << n, np.complex128)
    psi[0] = 1
    used = 0
    for pi, P in enumerate(prog["passes"]):
        if pi in by_pass:
            d = by_pass[pi]
            psi = emulate_tc_pass(psi, P, tcp["blocks"][d.block_begin:d.block_end], tcp["gates"], mats, n)
            used += 1
        else:
            one = dict(prog)
            one["passes"] = [P]
            psi = Replay(one, n).forward(psi, mats)
    return psi, used, tcp


@pytest.mark.parametrize("n,depth", [(12, 6), (14, 10), (16, 12)])
def test_tc_blocks_brickwall_match_oracle(n, depth):
    gl = templates.brickwall_gate_list(n, depth, 3)
    c, entry, mats, n_eng = build_host(n, gl)
    psi, used, tcp = emulate_forward(n_eng, entry, mats)
    assert used == len(nat.debug_program(entry.plan.handle, 0)["passes"]), "every brick-wall pass qualifies"
    slots = [b.slot for b in tcp["blocks"]]
    assert sorted(slots) == list(range(len(slots)))
    np.testing.assert_allclose(psi, sv.run_circuit(n, gl), atol=2e-6)


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_tc_blocks_random_circuits_match_oracle(seed):
    rng = np.random.default_rng(seed)
    n = 13 + seed
    gl = random_gate_list(n, 120, rng)
    c, entry, mats, n_eng = build_host(n, gl)
    psi, used, _ = emulate_forward(n_eng, entry, mats)
    assert used >= 1
    np.testing.assert_allclose(psi, sv.run_circuit(n, gl), atol=2e-6)


def test_tc_blocks_respect_six_bits_and_order():
    """Every block spans at most 6 tile bits of its gates and lists them in
    application order; every source gate of a tensor pass lands in exactly
    one block."""
    gl = templates.brickwall_gate_list(20, 20, 3)
    c, entry, mats, n_eng = build_host(20, gl)
    tcp = nat.debug_tc_program(entry.plan.handle)
    for blk in tcp["blocks"]:
        used = 0
        for G in tcp["gates"][blk.gate_begin:blk.gate_end]:
            for q in range(G.k):
                assert 0 <= G.pos[q] < 6
                used |= 1 << G.pos[q]
        assert bin(used).count("1") <= 6
    assert len(tcp["gates"]) == sum(b.gate_end - b.gate_begin for b in tcp["blocks"])
