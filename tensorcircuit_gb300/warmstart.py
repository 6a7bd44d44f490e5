"""Learned warm start for variational ground-state searches.

Workload: random-coupling open transverse-field Ising chains
H = -sum_i J_i Z_i Z_{i+1} - sum_i h_i X_i on n=16 sites (J_i ~ U[0.5, 1.5],
h_i ~ U[0.2, 2.0]), the hardware-efficient ansatz of depth 6 (rx on every
qubit then rzz on the open chain per layer: 186 angles), Adam (lr 0.02) on the
energy.  A small network (31 -> 256 -> 256 -> 186, GELU, float32 weights,
bfloat16 activations) learns to map couplings (J, h) to good starting
angles from optimised angles that the simulator itself produces; at
inference its output replaces the random starting point, which stays the
fallback.  Both are scored against the exact ground energy (free fermions, float64).

Everything on the GPU is this project's code: the energies and gradients
come from the engine's batched adjoint sweep (``backend.vvag``), the
network's forward, backward, loss and Adam steps from the kernels in
csrc/mlp.cu (``tcg_mlp_*``, ``tcg_periodic_loss``, ``tcg_adam_update``).
The reference has no counterpart; its VQE examples start from random angles.
"""

from typing import Any, Dict, List, Optional, Sequence, Tuple

import numpy as np
import torch

from . import _native as nat
from . import templates

N_SITES, DEPTH = 16, 6
N_COUPLINGS = 2 * N_SITES - 1


def n_params(n: int = N_SITES, depth: int = DEPTH) -> int:
    return templates.hea_nparams(n, depth)


def tfim_instances(count: int, seed: int, n: int = N_SITES) -> Tuple[np.ndarray, np.ndarray]:
    """Couplings of ``count`` random open chains: J [count, n-1] ~ U[0.5, 1.5],
    h [count, n] ~ U[0.2, 2.0] (float64)."""
    rng = np.random.default_rng(seed)
    J = rng.uniform(0.5, 1.5, (count, n - 1))
    h = rng.uniform(0.2, 2.0, (count, n))
    return J, h


def free_fermion_e0(J: np.ndarray, h: np.ndarray) -> np.ndarray:
    """Exact ground energy of H = -sum J_i Z_i Z_{i+1} - sum h_i X_i (open
    chain) by the Jordan-Wigner mapping to free fermions: E0 = -sum_k s_k(B),
    s_k the singular values of the bidiagonal B = diag(h) + superdiag(J)."""
    J = np.atleast_2d(np.asarray(J, dtype=np.float64))
    h = np.atleast_2d(np.asarray(h, dtype=np.float64))
    out = np.empty(J.shape[0])
    for i in range(J.shape[0]):
        B = np.diag(h[i]) + np.diag(J[i], 1)
        out[i] = -np.linalg.svd(B, compute_uv=False).sum()
    return out


def features(J: Any, h: Any) -> torch.Tensor:
    """Network input: couplings centred on their distributions' means."""
    J = torch.as_tensor(np.asarray(J), dtype=torch.float32)
    h = torch.as_tensor(np.asarray(h), dtype=torch.float32)
    return torch.cat([(J - 1.0) / 0.29, (h - 1.1) / 0.52], -1)


# --------------------------------------------------------------- optimiser
class AdamSearch:
    """Batched Adam on circuit angles: every step is one engine ``vvag`` call
    over the batch (energies and adjoint gradients) and one Adam kernel."""

    def __init__(self, n: int = N_SITES, depth: int = DEPTH, lr: float = 0.02) -> None:
        import tensorcircuit_gb300 as tc

        self.n, self.depth, self.lr = n, depth, lr
        K = tc.set_backend("pytorch")

        def energy(p: torch.Tensor, J: torch.Tensor, h: torch.Tensor) -> torch.Tensor:
            c = templates.apply_hea(tc.Circuit(n), n, depth, p)
            e = 0.0
            for i in range(n - 1):
                e = e - J[i] * K.real(c.expectation_ps(z=[i, i + 1]))
            for i in range(n):
                e = e - h[i] * K.real(c.expectation_ps(x=[i]))
            return e

        self.vvag = K.jit(K.vvag(energy, argnums=0, vectorized_argnums=(0, 1, 2)))

    def run(self, J: np.ndarray, h: np.ndarray, init: Any, steps: int, chunk: int = 4096,
            record: bool = True) -> Tuple[np.ndarray, np.ndarray]:
        """Adam from ``init`` for ``steps`` steps; returns the final angles
        [B, P] and the energy before every step and after the last one
        [steps + 1, B] (float64 host arrays)."""
        lib = nat.load()
        dev = torch.device("cuda", torch.cuda.current_device())
        init = torch.as_tensor(np.asarray(init), dtype=torch.float32)
        B = init.shape[0]
        out_p = np.empty((B, init.shape[1]), dtype=np.float32)
        hist = np.empty((steps + 1, B))
        for s0 in range(0, B, chunk):
            s1 = min(B, s0 + chunk)
            p = init[s0:s1].to(dev).contiguous()
            Jd = torch.as_tensor(J[s0:s1], dtype=torch.float32, device=dev)
            hd = torch.as_tensor(h[s0:s1], dtype=torch.float32, device=dev)
            m = torch.zeros_like(p)
            v = torch.zeros_like(p)
            es = []
            st = torch.cuda.current_stream().cuda_stream
            for step in range(1, steps + 1):
                e, g = self.vvag(p, Jd, hd)
                if record:
                    es.append(e.detach().clone())
                g = g.contiguous()
                nat.check(lib.tcg_adam_update(nat.ptr(p), nat.ptr(g), nat.ptr(m), nat.ptr(v), p.numel(), self.lr,
                                              0.9, 0.999, 1e-8, step, st), "adam")
            e, _ = self.vvag(p, Jd, hd)
            es.append(e.detach().clone())
            out_p[s0:s1] = p.cpu().numpy()
            if record:
                hist[:, s0:s1] = torch.stack(es).double().cpu().numpy()
            else:
                hist[-1, s0:s1] = es[-1].double().cpu().numpy()
        return out_p, hist


# ----------------------------------------------------------------- network
class WarmStartMLP:
    """31 -> 256 -> 256 -> 186 network on the project's kernels: float32
    weights, bfloat16 hidden activations, GELU, periodic angle loss."""

    def __init__(self, sizes: Sequence[int] = (N_COUPLINGS, 256, 256, 186), seed: int = 0,
                 device: Optional[torch.device] = None) -> None:
        self.sizes = list(sizes)
        self.dev = device or torch.device("cuda", torch.cuda.current_device())
        g = torch.Generator().manual_seed(seed)
        self.W: List[torch.Tensor] = []
        self.b: List[torch.Tensor] = []
        for a, b in zip(self.sizes[:-1], self.sizes[1:]):
            bound = 1.0 / np.sqrt(a)
            self.W.append(((torch.rand(b, a, generator=g) * 2 - 1) * bound).to(self.dev))
            self.b.append(((torch.rand(b, generator=g) * 2 - 1) * bound).to(self.dev))
        self.params = self.W + self.b
        self.m = [torch.zeros_like(t) for t in self.params]
        self.v = [torch.zeros_like(t) for t in self.params]
        self.step = 0

    def forward(self, x: torch.Tensor, keep: bool = False) -> Tuple[torch.Tensor, List[Any]]:
        lib = nat.load()
        st = torch.cuda.current_stream().cuda_stream
        x = x.to(self.dev, torch.float32).contiguous()
        B = x.shape[0]
        acts: List[Any] = [(x, 0)]
        h, hbf = x, 0
        nl = len(self.W)
        for i, (W, b) in enumerate(zip(self.W, self.b)):
            last = i == nl - 1
            out = W.shape[0]
            pre = torch.empty(B, out, dtype=torch.float32, device=self.dev) if (keep and not last) else None
            y = torch.empty(B, out, dtype=torch.float32 if last else torch.bfloat16, device=self.dev)
            nat.check(lib.tcg_mlp_linear_forward(nat.ptr(h), hbf, nat.ptr(W), nat.ptr(b), B, W.shape[1], out,
                                                 0 if last else 1, nat.ptr(pre) if pre is not None else None,
                                                 nat.ptr(y), 0 if last else 1, st), "mlp forward")
            acts.append((pre, y))
            h, hbf = y, (0 if last else 1)
        return h, acts

    def __call__(self, x: torch.Tensor) -> torch.Tensor:
        return self.forward(x)[0]

    def gradients(self, x: torch.Tensor, target: torch.Tensor) -> Tuple[float, List[torch.Tensor]]:
        """Loss mean(1 - cos(pred - target)) and d loss / d (W..., b...)."""
        lib = nat.load()
        st = torch.cuda.current_stream().cuda_stream
        pred, acts = self.forward(x, keep=True)
        target = target.to(self.dev, torch.float32).contiguous()
        B = pred.shape[0]
        n = pred.numel()
        nblk = 64
        dpred = torch.empty_like(pred)
        part = torch.empty(nblk, dtype=torch.float32, device=self.dev)
        nat.check(lib.tcg_periodic_loss(nat.ptr(pred), nat.ptr(target), n, nat.ptr(dpred), nat.ptr(part), nblk, st))
        dW = [torch.empty_like(W) for W in self.W]
        db = [torch.empty_like(b) for b in self.b]
        dy = dpred
        nl = len(self.W)
        for i in reversed(range(nl)):
            W = self.W[i]
            out, inn = W.shape
            xin, xbf = (acts[0][0], 0) if i == 0 else (acts[i][1], 1)
            pre = acts[i + 1][0]
            act = 0 if i == nl - 1 else 1
            dz = torch.empty(B, out, dtype=torch.float32, device=self.dev)
            dx = torch.empty(B, inn, dtype=torch.float32, device=self.dev) if i > 0 else None
            nat.check(lib.tcg_mlp_linear_backward(nat.ptr(dy), nat.ptr(pre) if pre is not None else None, act,
                                                  nat.ptr(xin), xbf, nat.ptr(W), B, inn, out, nat.ptr(dz),
                                                  nat.ptr(dW[i]), nat.ptr(db[i]),
                                                  nat.ptr(dx) if dx is not None else None, st), "mlp backward")
            dy = dx
        return float(part.sum().item()), dW + db

    def train_step(self, x: torch.Tensor, target: torch.Tensor, lr: float) -> float:
        lib = nat.load()
        st = torch.cuda.current_stream().cuda_stream
        loss, grads = self.gradients(x, target)
        self.step += 1
        for p, g, m, v in zip(self.params, grads, self.m, self.v):
            nat.check(lib.tcg_adam_update(nat.ptr(p), nat.ptr(g), nat.ptr(m), nat.ptr(v), p.numel(), lr, 0.9,
                                          0.999, 1e-8, self.step, st), "adam")
        return loss

    def fit(self, x: torch.Tensor, target: torch.Tensor, epochs: int = 200, batch: int = 512, lr: float = 1e-3,
            seed: int = 0) -> List[float]:
        x = x.to(self.dev, torch.float32)
        target = target.to(self.dev, torch.float32)
        g = torch.Generator().manual_seed(seed)
        losses = []
        N = x.shape[0]
        for ep in range(epochs):
            perm = torch.randperm(N, generator=g).to(self.dev)
            tot = 0.0
            for s0 in range(0, N, batch):
                idx = perm[s0:s0 + batch]
                tot += self.train_step(x[idx], target[idx], lr) * idx.numel()
            losses.append(tot / N)
        return losses


# ------------------------------------------------------------------- study
def relative_errors(hist: np.ndarray, e0: np.ndarray) -> np.ndarray:
    return np.abs((hist - e0[None, :]) / e0[None, :])


def steps_to(rel: np.ndarray, level: float) -> np.ndarray:
    """First step at which each instance's relative error is <= level
    (rel.shape[0] when never)."""
    hit = rel <= level
    first = np.where(hit.any(0), hit.argmax(0), rel.shape[0])
    return first


LEVELS = (0.1, 0.05, 0.03, 0.02, 0.01, 5e-3, 2e-3, 1e-3)


def level_table(rel_w: np.ndarray, rel_r: np.ndarray) -> Dict[str, Any]:
    """Per relative-error level: the fraction of chains each start reaches it
    in, and -- over the chains where both do -- the median Adam steps and
    their ratio (random / warm)."""
    out = {}
    for lv in LEVELS:
        sw, sr = steps_to(rel_w, lv), steps_to(rel_r, lv)
        both = (sw < rel_w.shape[0]) & (sr < rel_r.shape[0])
        row: Dict[str, Any] = {"reached_warm": float(np.mean(sw < rel_w.shape[0])),
                               "reached_random": float(np.mean(sr < rel_r.shape[0])),
                               "chains_both": int(both.sum())}
        if both.any():
            mw, mr = float(np.median(sw[both])), float(np.median(sr[both]))
            row.update({"median_steps_warm": mw, "median_steps_random": mr, "ratio": mr / max(mw, 1.0)})
        out["%g" % lv] = row
    return out


def study(n_train: int, n_test: int, steps: int = 300, gen_steps: int = 300, epochs: int = 200,
          seed: int = 6, lr: float = 0.02, plateau_chains: int = 0, plateau_steps: int = 0) -> Dict[str, Any]:
    """Generate training angles with the simulator, train the network, and
    compare warm-started and randomly started searches on held-out chains."""
    import time

    t0 = time.perf_counter()
    P = n_params()
    J, h = tfim_instances(n_train + n_test, seed)
    Jtr, htr, Jte, hte = J[:n_train], h[:n_train], J[n_train:], h[n_train:]
    search = AdamSearch(lr=lr)
    # training targets: every training chain optimised from one shared start
    # (a fixed draw), so the optimum moves smoothly with the couplings
    shared = np.random.default_rng(seed + 1).uniform(0, 2 * np.pi, P).astype(np.float32)
    p_tr, hist_tr = search.run(Jtr, htr, np.tile(shared, (n_train, 1)), gen_steps, record=False)
    t_gen = time.perf_counter() - t0
    net = WarmStartMLP(seed=seed)
    losses = net.fit(features(Jtr, htr), torch.as_tensor(p_tr), epochs=epochs)
    t_fit = time.perf_counter() - t0 - t_gen
    e0 = free_fermion_e0(Jte, hte)
    warm = net(features(Jte, hte)).float().cpu().numpy()
    rand = np.random.default_rng(seed + 2).uniform(0, 2 * np.pi, (n_test, P)).astype(np.float32)
    _, hist_w = search.run(Jte, hte, warm, steps)
    _, hist_r = search.run(Jte, hte, rand, steps)
    rel_w = relative_errors(hist_w, e0)
    rel_r = relative_errors(hist_r, e0)
    level = float(np.median(rel_r[-1]))
    s_w = steps_to(rel_w, level)
    s_r = steps_to(rel_r, level)
    gen_e0 = free_fermion_e0(Jtr, htr)
    checkpoints = sorted({k for k in (0, 10, 50, 100, 200, steps) if k <= steps})
    plateau = None
    if plateau_chains > 0 and plateau_steps > 0:
        # long runs on the first held-out chains: where each start levels off
        # and how many steps each needs to every level both reach
        k = min(plateau_chains, n_test)
        _, pw = search.run(Jte[:k], hte[:k], warm[:k], plateau_steps)
        _, pr = search.run(Jte[:k], hte[:k], rand[:k], plateau_steps)
        lw, lr_ = relative_errors(pw, e0[:k]), relative_errors(pr, e0[:k])
        pcts = (10, 25, 50, 75, 90)
        plateau = {
            "chains": k, "steps": plateau_steps,
            "final_rel_err_percentiles_warm": {str(q): float(np.percentile(lw[-1], q)) for q in pcts},
            "final_rel_err_percentiles_random": {str(q): float(np.percentile(lr_[-1], q)) for q in pcts},
            "best_rel_err_min_warm": float(lw.min()), "best_rel_err_min_random": float(lr_.min()),
            "median_rel_err_at": {str(c): {"warm": float(np.median(lw[c])), "random": float(np.median(lr_[c]))}
                                  for c in (0, 100, 300, 1000, 2000, 3000, plateau_steps) if c <= plateau_steps},
            "levels": level_table(lw, lr_),
        }
    return {
        "n_train": n_train, "n_test": n_test, "steps": steps, "gen_steps": gen_steps, "epochs": epochs,
        "train_rel_err_median": float(np.median(np.abs((hist_tr[-1] - gen_e0) / gen_e0))),
        "fit_loss_first_last": [losses[0], losses[-1]],
        "rel_err_median_warm": {str(k): float(np.median(rel_w[k])) for k in checkpoints},
        "rel_err_median_random": {str(k): float(np.median(rel_r[k])) for k in checkpoints},
        "target_level": level,
        # median steps to fixed relative-error levels (steps + 1 = not reached)
        "steps_to_level_median": {
            "%g" % lv: {"warm": float(np.median(steps_to(rel_w, lv))),
                        "random": float(np.median(steps_to(rel_r, lv)))}
            for lv in (0.1, 0.05, 0.03, 0.02, 1e-3)},
        "steps_to_target_median_warm": float(np.median(s_w)),
        "steps_to_target_median_random": float(np.median(s_r)),
        "step_ratio": float(np.median(s_r) / max(np.median(s_w), 1.0)),
        "reached_1e-3_warm": float(np.mean(rel_w.min(0) <= 1e-3)),
        "reached_1e-3_random": float(np.mean(rel_r.min(0) <= 1e-3)),
        "levels": level_table(rel_w, rel_r),
        "plateau": plateau,
        "seconds": {"generate": t_gen, "fit": t_fit, "evaluate": time.perf_counter() - t0 - t_gen - t_fit},
    }
