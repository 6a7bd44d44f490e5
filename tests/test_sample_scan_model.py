"""CPU: the index arithmetic of the sampling kernels (tensorcircuit_gb300/
csrc/misc.cu: block sums, block-sum scan, per-amplitude CDF in rounds,
binary search) restated in numpy and checked against the oracle's declared
CDF and sampler, including states shorter than one 4096-amplitude block.
No GPU needed; the kernels themselves are checked bit for bit on the GPU."""

import numpy as np
import pytest

from oracle import statevector as sv

THREADS, PER = 256, 16          # kScanThreads, kScanPer
BLOCK = THREADS * PER           # kScanBlock
WARPS = THREADS // 32
SCAN_THREADS = 1024             # the block-sum scan runs one CTA of 1024 threads


def _q(psi):
    a = np.asarray(psi, dtype=np.complex64)
    return sv.qweight(a.real) + sv.qweight(a.imag)


def _model_cdf(psi):
    """The three scan kernels, index for index."""
    q = _q(psi)
    n_amp = q.shape[0]
    nblocks = (n_amp + BLOCK - 1) // BLOCK
    padded = np.zeros(nblocks * BLOCK, dtype=np.uint64)
    padded[:n_amp] = q
    # [block][round][thread]: amplitude beg + r * THREADS + t (a < len, else 0)
    qb = padded.reshape(nblocks, PER, THREADS)
    # phase A: per-thread sums over its 16 rounds, then over the block
    bsum = qb.sum(axis=1, dtype=np.uint64).sum(axis=1, dtype=np.uint64)
    # phase B: contiguous chunks per thread, scan of the chunk totals, then
    # each chunk rewritten with its exclusive prefix
    per = (nblocks + SCAN_THREADS - 1) // SCAN_THREADS
    excl = np.zeros(nblocks, dtype=np.uint64)
    run_total = np.uint64(0)
    for i in range(SCAN_THREADS):
        beg = i * per
        for j in range(per):
            if beg + j < nblocks:
                excl[beg + j] = run_total
                run_total = np.uint64(run_total + bsum[beg + j])
    # phase C: 16 rounds per block; warp-inclusive scan of 32 lanes, warp
    # totals, carry across rounds
    lanes = qb.reshape(nblocks, PER, WARPS, 32)
    x = np.cumsum(lanes, axis=3, dtype=np.uint64)        # warp inclusive scan
    wsum = x[..., 31]                                      # [block][round][warp]
    pre = np.cumsum(wsum, axis=2, dtype=np.uint64) - wsum  # exclusive over warps
    tot = wsum.sum(axis=2, dtype=np.uint64)                # [block][round]
    carry = excl[:, None] + np.cumsum(tot, axis=1, dtype=np.uint64) - tot
    cdf = carry[:, :, None, None] + pre[..., None] + x
    return cdf.reshape(-1)[:n_amp]


def _model_search(cdf, u):
    total = cdf[-1]
    out = np.empty(len(u), dtype=np.int64)
    for i, ui in enumerate(np.asarray(u, dtype=np.float32)):
        t = np.floor((1.0 - np.float64(ui)) * np.float64(total))
        t = np.uint64(0) if t <= 0.0 else np.uint64(t)
        lo, hi = 0, cdf.shape[0]
        while lo < hi:
            mid = (lo + hi) >> 1
            if cdf[mid] < t:
                lo = mid + 1
            else:
                hi = mid
        out[i] = lo if lo < cdf.shape[0] else cdf.shape[0] - 1
    return out


@pytest.mark.parametrize("n", [3, 6, 11, 12, 13, 16])
def test_sampling_kernel_model_matches_declared_cdf(n):
    rng = np.random.default_rng(100 + n)
    psi = rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)
    psi[rng.choice(1 << n, max(1, (1 << n) // 8), replace=False)] = 0  # zero-probability entries
    psi /= np.linalg.norm(psi)
    cdf = _model_cdf(psi)
    np.testing.assert_array_equal(cdf, sv.declared_cdf(psi))
    u = rng.random(300).astype(np.float32)
    u[:3] = [0.0, np.float32(1.0) - np.float32(2 ** -24), 0.5]
    np.testing.assert_array_equal(_model_search(cdf, u), sv.sample_declared(psi, u))
