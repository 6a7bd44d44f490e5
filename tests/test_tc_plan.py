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


PLANE_LO, PLANE_IM = 8192, 16448


def kmajor_off(row, k, lbo=1024):
    return (k & 7) * 2 + (row & 7) * 16 + (k >> 3) * lbo + (row >> 3) * 128


def swz(t):
    return t ^ (((t >> 5) ^ (t >> 10)) & 31)


def emulate_tc_pass(psi, P, desc, blocks, gates, mats, n, stats=None):
    """Replays the tensor-core pass kernel's data movement byte for byte:
    the tile load through the pass's load table, operand planes read the way
    the MMA descriptors address them (K-major canonical layout), the planar
    complex GEMM, and the epilogue stores through each block's XOR tables
    (two values per 32-bit word on the pairing bit) into the next block's
    planes or the fp32 tile copy.  Values are kept exact (no fp16 split):
    this checks addresses, not rounding."""
    lbits = [P.lbits[i] for i in range(P.L)]
    nl = [P.nlbits[i] for i in range(P.nnonlocal)]
    gl = dep(np.arange(1 << P.L), lbits)
    ld = [desc.ldaddr[t] for t in range(12)]
    mats_f = [block_matrix(blk, gates, mats) for blk in blocks]
    for blk in blocks:
        bb = [blk.bbits[i] for i in range(6)]
        cb = [blk.cbits[i] for i in range(6)]
        assert sorted(bb + cb) == list(range(12)), "block + column bits must partition the tile"
    NT = 256  # threads per CTA of the pass kernel: tile offset 2 * (tid + NT u) + e
    tid_bits = NT.bit_length() - 1
    tid = np.arange(NT)
    tb = np.zeros(NT, np.int64)
    for k in range(tid_bits):
        tb ^= np.where((tid >> k) & 1, ld[1 + k], 0)
    for tile in range(1 << (n - P.L)):
        base = int(dep(tile, nl))
        T = psi[base | gl].copy()
        mem = {}

        def put(off, v):
            assert 0 <= off and off + 2 <= 32832 and (off % 2) == 0
            mem[int(off)] = v

        for u in range(4096 // (2 * NT)):
            ad = tb.copy()
            for k in range(11 - tid_bits):
                if (u >> k) & 1:
                    ad ^= ld[1 + tid_bits + k]
            j = 2 * (tid + NT * u)
            for t in range(NT):
                x0, x1 = T[j[t]], T[j[t] + 1]
                a0 = int(ad[t])
                a1 = a0 + 2 if desc.ldpair else a0 ^ ld[0]
                put(a0, x0.real)
                put(a1, x1.real)
                put(PLANE_IM + a0, x0.imag)
                put(PLANE_IM + a1, x1.imag)
        for bi, (blk, F) in enumerate(zip(blocks, mats_f)):
            last = bi + 1 == len(blocks)
            k = np.arange(64)[:, None]
            nn = np.arange(64)[None, :]
            offs = kmajor_off(nn, k)
            assert len(mem) == 2 * 4096, "every operand element written once"
            xre = np.vectorize(lambda o: mem[int(o)])(offs)
            xim = np.vectorize(lambda o: mem[PLANE_IM + int(o)])(offs)
            A = np.empty((128, 64))
            A[0::2] = F.real
            A[1::2] = F.imag
            D0, D1 = A @ xre, A @ xim
            rows = np.arange(128)
            sgn = np.where(rows & 1, 1.0, -1.0)[:, None]
            V = D0 + sgn * D1[rows ^ 1]
            R = np.array([blk.raddr[i] for i in range(64)])
            C = np.array([blk.caddr[i] for i in range(64)])
            mem = {}
            pb = blk.pairbit
            for row in range(128):
                plane = PLANE_IM if row & 1 else 0
                for col in range(64):
                    off = plane + int(R[row >> 1] ^ C[col])
                    if last:
                        mem[off] = V[row, col]
                    elif pb >= 0:
                        if (col >> pb) & 1:
                            continue
                        partner = col | (1 << pb)
                        assert (off & 2) == 0 and plane + int(R[row >> 1] ^ C[partner]) == off + 2
                        mem[off] = V[row, col]
                        mem[off + 2] = V[row, partner]
                    else:
                        mem[off] = V[row, col]
            if stats is not None and not last:
                # 4-byte-word banks of one store instruction: 32 lanes = 16 rows x re/im
                worst = 1
                for q in range(4):
                    for col in range(0, 64):
                        banks = {}
                        for lane in range(32):
                            row = 32 * q + lane
                            off = (PLANE_IM if row & 1 else 0) + int(R[row >> 1] ^ C[col])
                            banks.setdefault((off >> 2) & 31, set()).add(off >> 2)
                        worst = max(worst, max(len(v) for v in banks.values()))
                stats.append(worst)
        out = np.empty(4096, np.complex128)
        for j in range(4096):
            out[j] = mem[swz(j) * 4] + 1j * mem[PLANE_IM + swz(j) * 4]
        psi[base | gl] = out
    return psi


def emulate_forward(n, entry, mats, stats=None):
    prog = nat.debug_program(entry.plan.handle, 0)
    tcp = nat.debug_tc_program(entry.plan.handle)
    by_pass = {d.pass_: d for d in tcp["passes"]}
    psi = np.zeros(1 << n, np.complex128)
    psi[0] = 1
    used = 0
    for pi, P in enumerate(prog["passes"]):
        if pi in by_pass:
            d = by_pass[pi]
            psi = emulate_tc_pass(psi, P, d, tcp["blocks"][d.block_begin:d.block_end], tcp["gates"], mats, n,
                                  stats)
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


def test_tc_epilogue_store_conflicts_brickwall():
    """Bank conflicts of the epilogue's operand-plane stores (32 lanes = 16
    output rows x re/im planes) for the n=16 brick wall: the block orders
    keep them low."""
    gl = templates.brickwall_gate_list(16, 12, 3)
    c, entry, mats, n_eng = build_host(16, gl)
    stats = []
    emulate_forward(n_eng, entry, mats, stats)
    print("epilogue store conflict ways per block:", stats)
    assert stats and max(stats) <= 4
