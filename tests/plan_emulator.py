"""CPU replay of the engine's device programs (test infrastructure).

Executes a plan's passes / stages / ops with the same index arithmetic as
tensorcircuit_gb300/csrc/pass.cuh (tile base from the non-local bits, thread
and register bit deposits, register-position gate application, diagonal and
Pauli sign rules, per-tile accumulator slots), in numpy.  It lets the CPU
suite check the planner and every index a kernel would touch -- bijective
tiles, in-range global offsets -- before anything runs on a GPU.
"""

import numpy as np

OP_DENSE1, OP_DENSE2, OP_DIAG, OP_DENSEK, OP_EXPECT, OP_PACC, OP_PROT, OP_ZRUN = 0, 1, 2, 3, 4, 5, 6, 7


def dep(v, bits):
    v = np.asarray(v, dtype=np.int64)
    out = np.zeros_like(v)
    for i, b in enumerate(bits):
        out |= ((v >> i) & 1) << int(b)
    return out


def _popc(x):
    x = np.asarray(x, dtype=np.uint64)
    c = np.zeros(x.shape, dtype=np.int64)
    while np.any(x):
        c += (x & np.uint64(1)).astype(np.int64)
        x = x >> np.uint64(1)
    return c


class Replay:
    def __init__(self, prog, n):
        self.prog = prog
        self.n = n

    def _tiles(self, P):
        n = self.n
        L = P.L
        lbits = [P.lbits[i] for i in range(L)]
        nl = [P.nlbits[i] for i in range(P.nnonlocal)]
        assert sorted(lbits + nl) == list(range(n)), "local + non-local bits must partition the index"
        j = np.arange(1 << L)
        gl = dep(j, lbits)
        for tile in range(1 << (n - L)):
            base = int(dep(tile, nl))
            assert (base & gl).max(initial=0) == 0
            yield tile, base, gl

    def _layout(self, S, P, base):
        L = P.L
        R = S.R
        nt = 1 << S.nthread_bits
        assert S.nthread_bits == L - R
        assert nt <= 256, "a CTA has at most 256 threads (kernel launch bound)"
        thr = [S.thr_tile[i] for i in range(S.nthread_bits)]
        reg = [S.reg_tile[i] for i in range(R)]
        assert sorted(thr + reg) == list(range(L)), "thread + register bits must partition the tile"
        t = np.arange(nt)[:, None]
        r = np.arange(1 << R)[None, :]
        J = dep(t, thr) | dep(r, reg)
        assert J.min() >= 0 and J.max() < (1 << L)
        assert len(np.unique(J)) == (1 << L)
        lb = np.array([P.lbits[i] for i in range(L)])
        gthr = base | dep(np.arange(nt), lb[thr])
        rg = [1 << int(lb[x]) for x in reg]
        return J, gthr, rg, R

    @staticmethod
    def _gidx(gthr, rg, R):
        r = np.arange(1 << R)
        gr = np.zeros(1 << R, dtype=np.int64)
        for i in range(R):
            gr |= ((r >> i) & 1) * rg[i]
        return gthr[:, None] | gr[None, :]

    def forward(self, psi, mats):
        psi = np.array(psi, dtype=np.complex128)
        P_list, S_list, O_list = self.prog["passes"], self.prog["stages"], self.prog["ops"]
        for P in P_list:
            for tile, base, gl in self._tiles(P):
                assert (base | gl).max() < psi.size
                T = psi[base | gl].copy()
                for s in range(P.stage_begin, P.stage_end):
                    S = S_list[s]
                    if S.smem_stage:
                        for o in range(S.op_begin, S.op_end):
                            T = self._denseK(T, P.L, O_list[o], mats, adj=False)
                        continue
                    J, gthr, rg, R = self._layout(S, P, base)
                    V = T[J]
                    G = self._gidx(gthr, rg, R)
                    for o in range(S.op_begin, S.op_end):
                        V = self._apply(V, O_list[o], mats, G, R, adj=False)
                    T[J] = V
                psi[base | gl] = T
        return psi

    def backward(self, psi, mu, mats, nout):
        psi = np.array(psi, dtype=np.complex128)
        mu = np.array(mu, dtype=np.complex128)
        grads = np.zeros(nout, dtype=np.complex128)
        P_list, S_list, O_list = self.prog["passes"], self.prog["stages"], self.prog["ops"]
        for P in P_list:
            for tile, base, gl in self._tiles(P):
                T = psi[base | gl].copy()
                U = mu[base | gl].copy()
                for s in range(P.stage_begin, P.stage_end):
                    S = S_list[s]
                    if S.smem_stage:
                        for o in range(S.op_begin, S.op_end):
                            T = self._denseK(T, P.L, O_list[o], mats, adj=True)
                            U = self._denseK(U, P.L, O_list[o], mats, adj=True)
                        continue
                    J, gthr, rg, R = self._layout(S, P, base)
                    V, W = T[J], U[J]
                    G = self._gidx(gthr, rg, R)
                    for o in range(S.op_begin, S.op_end):
                        V, W = self._apply_bwd(V, W, O_list[o], mats, G, R, grads)
                    T[J], U[J] = V, W
                psi[base | gl] = T
                mu[base | gl] = U
        return psi, mu, grads

    def measure(self, psi, nterms):
        out = np.zeros(nterms, dtype=np.complex128)
        P_list, S_list, O_list = self.prog["passes"], self.prog["stages"], self.prog["ops"]
        for P in P_list:
            for tile, base, gl in self._tiles(P):
                T = np.asarray(psi, dtype=np.complex128)[base | gl]
                for s in range(P.stage_begin, P.stage_end):
                    S = S_list[s]
                    J, gthr, rg, R = self._layout(S, P, base)
                    V = T[J]
                    for o in range(S.op_begin, S.op_end):
                        op = O_list[o]
                        if op.kind == OP_ZRUN:
                            # Z-string terms: sum_x s_t(x) |psi_x|^2, thread/register split
                            G = self._gidx(gthr, rg, R)
                            for z, sg in self._zrun_signs(op, G, R):
                                out[z.mat_off] += np.sum(sg * np.abs(V) ** 2)
                            continue
                        assert op.kind == OP_EXPECT
                        X = op.xreg
                        sbase = _popc(gthr & op.zmask) & 1
                        zr = sum(1 << i for i in range(R) if rg[i] & op.zmask)
                        r = np.arange(1 << R)
                        s = (sbase[:, None] ^ (_popc(r & zr)[None, :] & 1)) & 1
                        c = np.conj(V) * V[:, r ^ X]
                        acc = np.sum(np.where(s == 1, -c, c))
                        out[op.mat_off] += acc * (-1j) ** (op.nY % 4)
        return out

    # ------------------------------------------------------------ op helpers
    @staticmethod
    def _pauli(V, op, G, R):
        """P V for the op's Pauli string: the X/Y bits are the register mask
        xreg, the Y/Z bits the global mask zmask, phase i^nY."""
        X = op.xreg
        assert 0 <= X < (1 << R)
        r = np.arange(1 << R)
        src = G[:, r ^ X]
        sgn = 1 - 2 * (_popc(src & op.zmask) & 1)
        return (1j ** (op.nY % 4)) * sgn * V[:, r ^ X]

    def _zrun_signs(self, op, G, R):
        """(entry, s_e[thread, r]) with s_e = (-1)^parity, the parity split as
        the kernels split it: thread part from the global index of register 0
        plus popc(r & zreg)."""
        zs = self.prog["zents"][op.mat_off:op.mat_off + op.k]
        r = np.arange(1 << R)
        out = []
        for z in zs:
            pt = _popc(G[:, 0] & z.zmask) & 1
            pr = _popc(r & z.zreg) & 1
            # the register mask must match the Z bits among the register bits
            want = _popc((G[:, [1 << i for i in range(R)]] ^ G[:, [0]]) & z.zmask)
            assert np.all((want > 0) == ((z.zreg >> np.arange(R)) & 1)[None, :].astype(bool))
            out.append((z, 1 - 2 * ((pt[:, None] ^ pr[None, :]) & 1)))
        return out

    @staticmethod
    def _mat(op, mats, dim):
        return np.asarray(mats[op.mat_off:op.mat_off + dim * dim], dtype=np.complex128).reshape(dim, dim)

    def _denseK(self, T, L, op, mats, adj):
        k = op.k
        tb = [op.p[i] for i in range(k)]
        m = self._mat(op, mats, 1 << k)
        if adj:
            m = m.conj().T
        t = T.reshape([2] * L)  # axis a <-> tile bit L-1-a
        axes = [L - 1 - b for b in tb]
        g = m.reshape([2] * (2 * k))
        t = np.tensordot(g, t, axes=(list(range(k, 2 * k)), axes))
        t = np.moveaxis(t, list(range(k)), axes)
        return t.reshape(-1)

    def _apply(self, V, op, mats, G, R, adj):
        V = V.copy()
        if op.kind == OP_DENSE1:
            p = op.p[0]
            assert 0 <= p < R
            m = self._mat(op, mats, 2)
            r0 = np.array([r for r in range(1 << R) if not (r >> p) & 1])
            r1 = r0 | (1 << p)
            x0, x1 = V[:, r0].copy(), V[:, r1].copy()
            V[:, r0] = m[0, 0] * x0 + m[0, 1] * x1
            V[:, r1] = m[1, 0] * x0 + m[1, 1] * x1
        elif op.kind == OP_DENSE2:
            p0, p1 = op.p[0], op.p[1]
            assert 0 <= p0 < R and 0 <= p1 < R and p0 != p1
            m = self._mat(op, mats, 4)
            rb = np.array([r for r in range(1 << R) if not ((r >> p0) & 1 or (r >> p1) & 1)])
            idx = [rb, rb | (1 << p1), rb | (1 << p0), rb | (1 << p0) | (1 << p1)]
            x = [V[:, i].copy() for i in idx]
            for a in range(4):
                V[:, idx[a]] = sum(m[a, b] * x[b] for b in range(4))
        elif op.kind == OP_DIAG:
            k = op.k
            d = np.asarray(mats[op.mat_off:op.mat_off + (1 << k)], dtype=np.complex128)
            idx = np.zeros(G.shape, dtype=np.int64)
            for i in range(k):
                idx |= ((G >> op.p[i]) & 1) << (k - 1 - i)
            V = V * d[idx]
        elif op.kind == OP_PROT:
            z = complex(mats[op.mat_off])
            c, s = z.real, z.imag
            if adj:
                s = -s
            V = c * V - 1j * s * self._pauli(V, op, G, R)
        elif op.kind == OP_ZRUN:
            for z, sg in self._zrun_signs(op, G, R):
                phi = np.angle(complex(mats[z.mat_off]))
                V = V * np.exp((1j if adj else -1j) * phi * sg)
        else:
            raise AssertionError("unexpected op kind %d" % op.kind)
        return V

    def _apply_bwd(self, V, W, op, mats, G, R, grads):
        V, W = V.copy(), W.copy()
        if op.kind in (OP_DENSE1, OP_DENSE2):
            k = 1 if op.kind == OP_DENSE1 else 2
            m = self._mat(op, mats, 1 << k)
            a = m.conj().T
            if k == 1:
                p = op.p[0]
                rb = np.array([r for r in range(1 << R) if not (r >> p) & 1])
                idx = [rb, rb | (1 << p)]
            else:
                p0, p1 = op.p[0], op.p[1]
                rb = np.array([r for r in range(1 << R) if not ((r >> p0) & 1 or (r >> p1) & 1)])
                idx = [rb, rb | (1 << p1), rb | (1 << p0), rb | (1 << p0) | (1 << p1)]
            D = 1 << k
            x = [V[:, i].copy() for i in idx]
            y = [sum(a[i, j] * x[j] for j in range(D)) for i in range(D)]
            for i in range(D):
                V[:, idx[i]] = y[i]
            u = [W[:, i].copy() for i in idx]
            if op.slot >= 0:
                for i in range(D):
                    for j in range(D):
                        grads[op.grad_off + i * D + j] += np.sum(u[i] * np.conj(y[j]))
            for i in range(D):
                W[:, idx[i]] = sum(a[i, j] * u[j] for j in range(D))
        elif op.kind == OP_DIAG:
            k = op.k
            d = np.conj(np.asarray(mats[op.mat_off:op.mat_off + (1 << k)], dtype=np.complex128))
            idx = np.zeros(G.shape, dtype=np.int64)
            for i in range(k):
                idx |= ((G >> op.p[i]) & 1) << (k - 1 - i)
            V = V * d[idx]
            if op.slot >= 0:
                g = W * np.conj(V)
                for e in range(1 << k):
                    grads[op.grad_off + e] += np.sum(g[idx == e])
            W = W * d[idx]
        elif op.kind == OP_ZRUN:
            # the run's rotations commute: dL/dphi_e = Im <mu| Z_e |psi> at the run output
            for z, sg in self._zrun_signs(op, G, R):
                if z.slot >= 0:
                    grads[z.grad_off] += np.sum(sg * np.imag(np.conj(W) * V))
            V = self._apply(V, op, mats, G, R, adj=True)
            W = self._apply(W, op, mats, G, R, adj=True)
        elif op.kind == OP_PROT:
            # dG/dphi = -i P G, so dL/dphi = Im <mu| P |psi_out>
            if op.slot >= 0:
                grads[op.grad_off] += np.sum(np.conj(W) * self._pauli(V, op, G, R)).imag
            V = self._apply(V, op, mats, G, R, adj=True)
            W = self._apply(W, op, mats, G, R, adj=True)
        else:
            raise AssertionError("unexpected op kind %d" % op.kind)
        return V, W
