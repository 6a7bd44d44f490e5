"""Benchmark: batched adjoint value+gradient of parameterized circuits.

Workload (one step): the hardware-efficient ansatz on n=20 qubits, 8 layers
(rx on every qubit then rzz on the open chain; 312 parameters), a batch of 64
parameter vectors ~U[0, 2pi) (seed 2), energy of the TFIM
H = -sum Z_i Z_{i+1} - 1.0 sum X_i, value and full gradient of every circuit
through ``backend.vvag`` -- the reference's batched VQE step.  Synthetic
inputs; states are complex64.  On one GPU the default run also times the
large-circuit gate-application workload (n=28 Haar brick wall of depth 20,
<Z0 Z27>, <X13>, 2^20 samples) and reports it under "brickwall_n28" in the
same line, with its own forward-pass roofline, CPU baseline and e2e figure,
and the uneven batch (512 QAOA MaxCut circuits, n 12..24, one persistent
launch per sweep) under "qaoa_uneven_512".

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

``--impl reference`` times the reference algorithm's CPU path (a labelled
torch restatement: per-gate tensordot + taped AD, see
oracle/reference_algo.py) on the host cores, on a bounded sample of the same
workload.  Multi-GPU runs are independent replicas (each rank runs its own
64-circuit batch; no collective on the data path) and report the aggregate.
"""

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

N_QUBITS, N_LAYERS, BATCH, SEED = 20, 8, 64, 2
METRIC = "adjoint value+grad circuits/s (n=20 HEA, 312 params, TFIM energy)"
UNIT = "circuits/s"
WORKLOAD = "hea_n20_l8_b64_tfim_vvag"


def hea_config(n_gpus):
    """The workload description both arms (engine and reference) report."""
    from tensorcircuit_gb300 import templates

    return {"workload": WORKLOAD, "n_qubits": N_QUBITS, "layers": N_LAYERS,
            "params": int(templates.hea_nparams(N_QUBITS, N_LAYERS)), "batch_per_gpu": BATCH,
            "parallelism": "replicas" if n_gpus > 1 else "single",
            "l2": "no flush: per-step working set (64 states + 64 cotangents = 1 GiB) exceeds the 129 MB L2"}


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(r[1]) for r in self.rows if len(r) > 8 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 8 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            if len(r) > 8:
                for nm, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def _traffic(key, applies):
    """DRAM bytes per launch of the dominant kernel from the ncu captures
    (profiles/traffic.json), when the run has the captured configuration."""
    if not applies:
        return None
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as fh:
            return json.load(fh).get(key)
    except Exception:
        return None


def aggregate_replicas(ms_values, units_per_rank, world, device):
    """Replicas (one independent batch per rank, no exchange on the data
    path): the step time is the maximum over ranks, the throughput the units
    of all ranks over that time.  Returns (max times in ms, units/s)."""
    if world > 1:
        import torch

        t = torch.tensor([float(x) for x in ms_values], dtype=torch.float64, device=device)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms_values = t.tolist()
    return list(ms_values), [world * units_per_rank / (m / 1e3) for m in ms_values]


def _workload_params():
    from tensorcircuit_gb300 import templates

    rng = np.random.default_rng(SEED)
    return rng.uniform(0, 2 * np.pi, (BATCH, templates.hea_nparams(N_QUBITS, N_LAYERS))).astype(np.float32)


def cpu_reference(steps, warmup, sample_circuits=1):
    """Reference-algorithm restatement on the host cores, bounded sample."""
    from oracle import reference_algo as ra
    from tensorcircuit_gb300 import templates

    threads = len(os.sched_getaffinity(0))
    params = _workload_params()[:sample_circuits]
    layout = templates.hea_layout(N_QUBITS, N_LAYERS)
    terms = templates.tfim_terms(N_QUBITS, -1.0, -1.0)

    def one_step():
        # one circuit per vvag call: the restatement's fastest form on the
        # host (a vmapped sample of four tapes ran at 0.21 circuits/s on 16
        # cores, one circuit at a time at 0.37)
        for i in range(sample_circuits):
            ra.vvag_hea(N_QUBITS, layout, terms, params[i:i + 1], threads)

    for _ in range(warmup):
        one_step()
    t0 = time.perf_counter()
    for _ in range(steps):
        one_step()
    dt = (time.perf_counter() - t0) / steps
    return {"value": sample_circuits / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "%d of the %d circuits per step, one per vvag call (labelled torch restatement of "
                      "the reference algorithm: per-gate tensordot + taped AD via torch.func vmap/grad), "
                      "%d steps" % (sample_circuits, BATCH, steps),
            "seconds_per_circuit": dt / sample_circuits, "sample_circuits": sample_circuits}


def gpu_plain_ad(sample_circuits=8, steps=2):
    """The reference algorithm's taped AD (per-gate tensordot, torch.func
    vmap/grad -- the reference's pytorch backend) placed on the same GPU,
    on a bounded sample of the batch: the 'plain AD on the same GPU' the
    adjoint kernel is compared with."""
    import torch

    from oracle import reference_algo as ra
    from tensorcircuit_gb300 import templates

    params = _workload_params()[:sample_circuits]
    layout = templates.hea_layout(N_QUBITS, N_LAYERS)
    terms = templates.tfim_terms(N_QUBITS, -1.0, -1.0)
    try:
        ra.vvag_hea(N_QUBITS, layout, terms, params, 1, device="cuda")
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(steps):
            ra.vvag_hea(N_QUBITS, layout, terms, params, 1, device="cuda")
        torch.cuda.synchronize()
        dt = (time.perf_counter() - t0) / steps
    except Exception as exc:  # e.g. out of memory for the taped states
        return {"unavailable": "%s: %s" % (type(exc).__name__, str(exc)[:200])}
    return {"value": sample_circuits / dt, "unit": UNIT,
            "sample": "%d of the %d circuits, %d steps (labelled torch restatement of the reference "
                      "algorithm: per-gate tensordot + taped AD via torch.func vmap/grad, on the GPU)" %
                      (sample_circuits, BATCH, steps)}


def run_reference_arm(args, rank):
    if rank != 0:
        return
    # two circuits per step, about 5 s on 16 cores: at most 3 timed and 2
    # warm-up steps (the restatement has no compilation to warm up)
    steps = max(1, min(args.steps, 3))
    warmup = min(args.warmup, 2)
    cb = cpu_reference(steps, warmup, sample_circuits=2)
    line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": UNIT, "n_gpus": args.gpus,
            "steps": steps, "warmup": warmup, "ms_per_step": 1000.0 * cb["sample_circuits"] / cb["value"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c64", "data": "synthetic",
            "config": hea_config(args.gpus),
            "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_gb300_arm(args, rank, world):
    import torch

    import tensorcircuit_gb300 as tc
    from tensorcircuit_gb300 import _native, engine, templates

    tc.build()
    lib = _native.load()
    dev = torch.device("cuda", torch.cuda.current_device())
    K = tc.set_backend("pytorch")
    n, nl = N_QUBITS, N_LAYERS
    terms = templates.tfim_terms(n, -1.0, -1.0)

    def f(p):
        c = templates.apply_hea(tc.Circuit(n), n, nl, p)
        return templates.energy(c, terms)

    # the reference's idiom (e.g. examples/bp_validation.py:55): K.jit(K.vvag(f));
    # jit captures the step into a CUDA graph after its eager warm-up calls
    vvag = K.jit(K.vvag(f, argnums=0, vectorized_argnums=0))
    params_host = torch.from_numpy(_workload_params()).pin_memory()
    params = params_host.to(dev)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    # warm-up: the jit wrapper runs 3 eager calls, then captures the graph;
    # every warm-up call is untimed
    warmup = max(args.warmup, 5)
    for _ in range(warmup):
        v, g = vvag(params)
    torch.cuda.synchronize()
    # engine kernels per step: count the launches of one eager step (graph
    # replays launch the same kernels without passing through the host code)
    l0 = lib.tcg_launch_count()
    K.vvag(f, argnums=0, vectorized_argnums=0)(params)
    torch.cuda.synchronize()
    launches_per_step = lib.tcg_launch_count() - l0

    # ---- device-resident value
    barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev.index) as clk:
        ev0.record()
        for _ in range(args.steps):
            v, g = vvag(params)
        ev1.record()
        torch.cuda.synchronize()
    launches = launches_per_step * args.steps
    ms = ev0.elapsed_time(ev1) / args.steps
    barrier()

    # ---- end to end: pinned host params in, values + gradients out
    vh = torch.empty((BATCH,), dtype=torch.float32).pin_memory()
    gh = torch.empty((BATCH, params.shape[1]), dtype=torch.float32).pin_memory()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        p = params_host.to(dev, non_blocking=True)
        v, g = vvag(p)
        vh.copy_(v, non_blocking=True)
        gh.copy_(g, non_blocking=True)
    e1.record()
    torch.cuda.synchronize()
    ms_e2e = e0.elapsed_time(e1) / args.steps
    h2d = params_host.numel() * 4
    d2h = (vh.numel() + gh.numel()) * 4

    # ---- dominant kernel: the adjoint sweep (tcg_backward) on the same batch,
    # called through the C ABI with the batch's gate matrices
    from tensorcircuit_gb300 import circuit as cmod
    from tensorcircuit_gb300 import gates as G

    layout = templates.hea_layout(n, nl)
    c = templates.apply_hea(tc.Circuit(n), n, nl, np.zeros(params.shape[1]))
    # the plan the vvag steps above used (specialised kernels already built)
    entry = cmod._entries.get(cmod._struct_key(n, c._ops)) or cmod._build_entry(n, c._ops)
    plan = entry.plan
    N = 1 << n
    blocks = []
    for gkey, idx, E in entry.groups:
        th = params[:, [layout[i][2] for i in idx]]
        if gkey[0] == "prot":
            blocks.append(G.build_prot(th, gkey[1]).reshape(BATCH, -1))
        else:
            blocks.append(G.FAMILIES[gkey[1]].build(th).reshape(BATCH, -1))
    mats = torch.cat(blocks, -1).to(torch.complex64).contiguous()
    M = mats.shape[-1]
    psi_out = torch.zeros(BATCH, N, dtype=torch.complex64, device=dev)
    psi_out[:, 0] = 1
    st = int(torch.cuda.current_stream().cuda_stream)
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record()
    _native.check(lib.tcg_forward(plan.handle, psi_out.data_ptr(), BATCH, mats.data_ptr(), M, st))
    f1.record()
    torch.cuda.synchronize()
    ms_fwd = f0.elapsed_time(f1)
    mu0 = torch.randn(BATCH, N, dtype=torch.complex64, device=dev)
    psi_w = psi_out.clone()
    mu_w = mu0.clone()
    grads = torch.zeros_like(mats)
    nbytes = int(lib.tcg_backward_scratch_bytes(plan.handle, BATCH))
    scratch = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    prog_b = _native.debug_program(plan.handle, 1)
    nb_pass = len(prog_b["passes"])
    reps = max(3, args.steps)

    def bwd_once():
        psi_w.copy_(psi_out)
        mu_w.copy_(mu0)

    for _ in range(2):
        bwd_once()
        _native.check(lib.tcg_backward(plan.handle, psi_w.data_ptr(), mu_w.data_ptr(), BATCH, mats.data_ptr(), M,
                                       grads.data_ptr(), M, scratch.data_ptr(), nbytes, st))
    torch.cuda.synchronize()
    tot = 0.0
    for _ in range(reps):
        bwd_once()
        b0, b1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        b0.record()
        _native.check(lib.tcg_backward(plan.handle, psi_w.data_ptr(), mu_w.data_ptr(), BATCH, mats.data_ptr(), M,
                                       grads.data_ptr(), M, scratch.data_ptr(), nbytes, st))
        b1.record()
        torch.cuda.synchronize()
        tot += b0.elapsed_time(b1)
    ms_bwd = tot / reps
    alg_bytes = nb_pass * 4 * 8 * N * BATCH  # psi and mu, read + write, per pass
    per_launch_s = ms_bwd / 1e3 / nb_pass
    achieved = (alg_bytes / nb_pass) / per_launch_s / 1e9
    peak, peak_kind = _peaks()
    traffic = _traffic("pass_kernel_bwd_bytes_per_launch", BATCH == 64)

    # ---- aggregate over ranks (replicas)
    (ms, ms_e2e), (circ_s, circ_e2e) = aggregate_replicas([ms, ms_e2e], BATCH, world, dev)
    if rank != 0:
        return
    cpu = None
    plain_ad = None
    if world == 1 and not args.no_cpu:
        cpu = cpu_reference(steps=1, warmup=1, sample_circuits=4)  # about 11 s on 16 cores
        plain_ad = gpu_plain_ad()
    line = {
        "metric": METRIC, "value": circ_s, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "c64", "data": "synthetic",
        "config": hea_config(world),
        "roofline": {"bound": "hbm", "kernel": "pass_kernel<BWD> (adjoint sweep, tcg_backward)",
                     "passes": nb_pass,
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_kind, "traffic": traffic,
                     "alg_bytes_per_launch": alg_bytes / nb_pass, "ms_per_sweep": ms_bwd,
                     "forward_sweep": {"ms": ms_fwd, "passes": plan.npasses,
                                       "GB_per_s": plan.npasses * 16 * N * BATCH / (ms_fwd / 1e3) / 1e9}},
        "cpu_baseline": cpu,
        "plain_ad_same_gpu": plain_ad,
        "e2e": {"value": circ_e2e, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "clocks": clk.summary(),
        "gpu_launches": int(launches),
        "gpu_launches_per_step": int(launches_per_step),
    }
    if world == 1 and not args.no_brickwall:
        # the large-circuit gate-application workload (n=28 Haar brick wall),
        # timed the same way after the batched step, reported beside it
        bw = measure_brickwall(args, rank, world)
        line["brickwall_n28"] = {k: bw[k] for k in ("metric", "value", "unit", "ms_per_step", "steps", "warmup",
                                                    "config", "roofline", "cpu_baseline", "e2e", "clocks",
                                                    "gpu_launches", "gpu_launches_per_step")}
    if world == 1 and not args.no_qaoa:
        # the uneven batch: 512 QAOA circuits in one persistent launch per sweep
        qb = measure_qaoa(args, rank, world, nested=True)
        qb["roofline"].pop("sweeps", None)
        line["qaoa_uneven_512"] = {k: qb[k] for k in ("metric", "value", "unit", "ms_per_step", "steps", "warmup",
                                                      "config", "roofline", "cpu_baseline", "e2e", "clocks",
                                                      "gpu_launches", "gpu_launches_per_step")}
    print(json.dumps(line), flush=True)


BW_N, BW_DEPTH, BW_SEED, BW_USEED, BW_SHOTS = 28, 20, 3, 4, 1 << 20
BW_METRIC = "gate-updates/s (n=28 Haar brick wall, depth 20; state, <Z0Z27>, <X13>, 2^20 samples)"
BW_UNIT = "gate-updates/s"
BW_WORKLOAD = "brickwall_n28_d20_haar"


def _bw_inputs():
    from tensorcircuit_gb300 import templates

    gl = templates.brickwall_gate_list(BW_N, BW_DEPTH, BW_SEED)
    u = np.random.default_rng(BW_USEED).random(BW_SHOTS, dtype=np.float32)
    return gl, u


def cpu_brickwall(n_cpu=22):
    """Reference-algorithm restatement (per-gate tensordot, complex64) on the
    host cores: the n=28 circuit holds 2 GiB states, so the bounded sample is
    the same brick wall at ``n_cpu`` qubits, scaled to gate-updates/s of
    n=28 by the amplitude count."""
    from oracle import reference_algo as ra
    from tensorcircuit_gb300 import templates

    threads = len(os.sched_getaffinity(0))
    gl = templates.brickwall_gate_list(n_cpu, BW_DEPTH, BW_SEED)
    scale = float(1 << (BW_N - n_cpu))
    ra.run_gate_list(n_cpu, gl[:4], threads)
    t0 = time.perf_counter()
    ra.run_gate_list(n_cpu, gl, threads)
    dt = time.perf_counter() - t0
    # the numpy backend's form of the same contraction (numpy.tensordot per
    # gate), reported beside it; the value is the faster of the two
    try:
        t0 = time.perf_counter()
        ra.run_gate_list_numpy(n_cpu, gl)
        dt_np = time.perf_counter() - t0
        numpy_form = {"value": len(gl) / dt_np / scale, "seconds": dt_np}
    except Exception as exc:  # reported, never fatal for the bench line
        dt_np, numpy_form = float("inf"), {"unavailable": "%s: %s" % (type(exc).__name__, str(exc)[:200])}
    best = min(dt, dt_np)
    return {"value": len(gl) / best / scale, "unit": BW_UNIT, "cores": threads, "kind": "port",
            "sample": "brick wall depth %d at n=%d (%d gates; labelled restatements of the reference's "
                      "per-gate tensordot: torch %.2f s, numpy %.2f s, the faster counts), scaled by 2^%d "
                      "amplitudes to n=%d" % (BW_DEPTH, n_cpu, len(gl), dt, dt_np, BW_N - n_cpu, BW_N),
            "torch_form": {"value": len(gl) / dt / scale, "seconds": dt}, "numpy_form": numpy_form}


def run_brickwall(args, rank, world):
    line = measure_brickwall(args, rank, world)
    if line is not None:
        print(json.dumps(line), flush=True)


def measure_brickwall(args, rank, world):
    """Large single circuit: n=28 Haar brick wall (270 gates), then <Z0 Z27>,
    <X13> and 2^20 samples from seeded uniforms, through the Circuit API.
    Returns the JSON line (rank 0) or None."""
    import torch

    import tensorcircuit_gb300 as tc
    from tensorcircuit_gb300 import _native, templates
    from tensorcircuit_gb300 import circuit as cmod

    tc.build()
    lib = _native.load()
    dev = torch.device("cuda", torch.cuda.current_device())
    n = BW_N
    gl, u_np = _bw_inputs()
    u_host = torch.from_numpy(u_np).pin_memory()
    u_dev = u_host.to(dev)

    def step(u):
        c = templates.apply_gate_list(tc.Circuit(n), gl)
        zz = c.expectation_ps(z=[0, n - 1])
        x13 = c.expectation_ps(x=[13])
        s = c.sample(batch=BW_SHOTS, allow_state=True, status=u, format="sample_int")
        return zz, x13, s

    warmup = max(args.warmup, 3)
    for _ in range(warmup):
        out = step(u_dev)
    torch.cuda.synchronize()
    l0 = lib.tcg_launch_count()
    step(u_dev)
    torch.cuda.synchronize()
    launches_per_step = lib.tcg_launch_count() - l0

    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev.index) as clk:
        ev0.record()
        for _ in range(args.steps):
            out = step(u_dev)
        ev1.record()
        torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / args.steps

    # end to end: uniforms from pinned host memory in, expectations and
    # samples back to pinned host memory, every step
    sh = torch.empty((BW_SHOTS,), dtype=torch.int64).pin_memory()
    eh = torch.empty((2,), dtype=torch.complex64).pin_memory()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        u = u_host.to(dev, non_blocking=True)
        zz, x13, s = step(u)
        eh.copy_(torch.stack([zz.reshape(()), x13.reshape(())]), non_blocking=True)
        sh.copy_(s, non_blocking=True)
    e1.record()
    torch.cuda.synchronize()
    ms_e2e = e0.elapsed_time(e1) / args.steps

    # dominant kernel: the forward sweep of the cached plan, per pass
    c = templates.apply_gate_list(tc.Circuit(n), gl)
    entry = cmod._entries[cmod._struct_key(n, c._ops)]
    plan = entry.plan
    mats = entry.const_block(dev)
    N = 1 << n
    psi = torch.zeros(N, dtype=torch.complex64, device=dev)
    st = int(torch.cuda.current_stream().cuda_stream)
    reps = max(3, args.steps)
    tot = 0.0
    for r in range(reps + 1):
        psi.zero_()
        psi[0] = 1
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record()
        _native.check(lib.tcg_forward(plan.handle, psi.data_ptr(), 1, mats.data_ptr(), mats.numel(), st))
        f1.record()
        torch.cuda.synchronize()
        if r:
            tot += f0.elapsed_time(f1)
    ms_fwd = tot / reps
    per_launch_s = ms_fwd / 1e3 / plan.npasses
    achieved = 16.0 * N / per_launch_s / 1e9
    peak, peak_kind = _peaks()
    if rank != 0:
        return
    cpu = None if args.no_cpu else cpu_brickwall()
    zz, x13, _ = out
    line = {
        "metric": BW_METRIC, "value": len(gl) / (ms / 1e3), "unit": BW_UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c64", "data": "synthetic",
        "config": {"workload": BW_WORKLOAD if n == 28 else "brickwall_n%d_d20_haar" % n, "n_qubits": n, "depth": BW_DEPTH, "gates": len(gl),
                   "shots": BW_SHOTS, "seed": BW_SEED, "uniform_seed": BW_USEED,
                   "l2": "no flush: the 2 GiB state exceeds the 129 MB L2",
                   "fwd_passes": plan.npasses, "zz_0_27": float(zz.real), "x_13": float(x13.real)},
        "roofline": {"bound": "hbm", "kernel": "forward pass (tcg_forward, one launch per pass: %d of %d passes "
                                               "on tc_pass_kernel, fused blocks on the tensor cores)" %
                                               (plan.tensor_passes(), plan.npasses),
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_kind, "traffic": _traffic("brickwall_fwd_bytes_per_launch", n == 28),
                     "alg_bytes_per_launch": 16.0 * N,
                     "ms_forward": ms_fwd, "passes": plan.npasses,
                     "amp_updates_per_s": len(gl) * N / (ms_fwd / 1e3),
                     "gate_updates_per_s_forward": len(gl) / (ms_fwd / 1e3)},
        "cpu_baseline": cpu,
        "e2e": {"value": len(gl) / (ms_e2e / 1e3), "unit": BW_UNIT, "h2d_bytes_per_step": BW_SHOTS * 4,
                "d2h_bytes_per_step": BW_SHOTS * 8 + 16},
        "clocks": clk.summary(),
        "gpu_launches": int(launches_per_step * args.steps),
        "gpu_launches_per_step": int(launches_per_step),
    }
    return line


QB_COUNT, QB_SEED = 512, 5
QB_METRIC = "adjoint value+grad circuits/s (512 uneven QAOA MaxCut circuits, n 12..24, p 1..6)"
QB_UNIT = "circuits/s"
QB_WORKLOAD = "qaoa_uneven_512"


def cpu_qaoa(specs, params, sample=3):
    """Reference-algorithm restatement (per-gate tensordot + taped AD, one
    circuit at a time) on the host cores for a bounded sample of the batch:
    circuits drawn at seed 0, scaled to the batch by the amplitude-weighted
    work (sum of 2^n * gates)."""
    from oracle import reference_algo as ra

    threads = len(os.sched_getaffinity(0))
    rng = np.random.default_rng(0)
    idx = rng.choice(len(specs), sample, replace=False)
    # amplitudes x gates (n H gates, then per layer 1.5 n edges + n rx)
    work = [(1 << s[0]) * (s[0] + (s[2] // 2) * 2.5 * s[0]) for s in specs]
    t0 = time.perf_counter()
    for i in idx:
        n, build, npar, terms, offset = specs[i]
        edges = [tuple(t["z"]) for _, t in terms]
        ra.qaoa_value_and_grad(n, edges, npar // 2, params[i], threads)
    dt = time.perf_counter() - t0
    frac = sum(work[i] for i in idx) / sum(work)
    # the whole batch would take dt / frac seconds
    return {"value": len(specs) / (dt / frac), "unit": QB_UNIT, "cores": threads, "kind": "port",
            "sample": "%d circuits (n=%s, %.2f s; labelled torch restatement: per-gate tensordot + taped AD), "
                      "scaled to the 512-circuit batch by amplitude-weighted gate count (%.4f of its work)" %
                      (sample, [specs[i][0] for i in idx], dt, frac)}


def per_circuit_loop(specs, params, sample=24):
    """The reference's way through this engine: one ``K.value_and_grad``
    per circuit (Circuit API, adjoint kernels, no batching across circuits),
    timed on a sample of the batch (seed 1) and scaled by its share of the
    amplitude-weighted work."""
    import torch

    import tensorcircuit_gb300 as tc
    from tensorcircuit_gb300 import templates

    K = tc.set_backend("pytorch")
    rng = np.random.default_rng(1)
    idx = rng.choice(len(specs), sample, replace=False)
    work = [(1 << s[0]) * (s[0] + (s[2] // 2) * 2.5 * s[0]) for s in specs]

    def run(i):
        n, build, npar, terms, offset = specs[i]

        def f(p):
            c = tc.Circuit(n)
            build(c, p)
            return templates.energy(c, terms) + offset

        return K.value_and_grad(f)(torch.tensor(params[i], device="cuda"))

    run(int(idx[0]))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in idx:
        run(int(i))
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    frac = sum(work[i] for i in idx) / sum(work)
    return {"value": len(specs) / (dt / frac), "unit": QB_UNIT,
            "sample": "%d circuits through Circuit + K.value_and_grad one at a time (%.2f s), scaled by "
                      "amplitude-weighted work (%.3f of the batch)" % (sample, dt, frac)}


def run_qaoa(args, rank, world):
    line = measure_qaoa(args, rank, world)
    if line is not None:
        print(json.dumps(line), flush=True)


def measure_qaoa(args, rank, world, nested=False):
    """Uneven batch: 512 QAOA MaxCut circuits (n ~ U{12,..,24} even, random
    3-regular graphs, p ~ U{1..6}, gamma, beta ~ U[0, pi), seed 5), energy
    and adjoint gradient of every circuit per step, one persistent launch per
    sweep replayed from a CUDA graph, tile width autotuned.  Returns the JSON
    line (rank 0) or None; ``nested`` (inside the default run) leaves out the
    per-circuit comparison loop."""
    import torch

    import tensorcircuit_gb300 as tc
    from tensorcircuit_gb300 import _native, batch, templates

    tc.build()
    lib = _native.load()
    dev = torch.device("cuda", torch.cuda.current_device())
    specs, params = templates.qaoa_uneven_workload(QB_COUNT, QB_SEED)
    t0 = time.perf_counter()
    ub = batch.UnevenBatch(specs, graph=True)
    setup_s = time.perf_counter() - t0
    flat_host = torch.from_numpy(np.concatenate(params)).pin_memory()
    flat = flat_host.to(dev)
    warmup = max(args.warmup, 3)
    for _ in range(warmup):
        e, g = ub.value_and_grad(flat)
    torch.cuda.synchronize()
    ub.check()
    l0 = lib.tcg_launch_count()
    ub.h.run(flat, e, g)  # one eager call: kernels per step (the graph replays the same ones)
    torch.cuda.synchronize()
    launches_per_step = lib.tcg_launch_count() - l0

    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev.index) as clk:
        ev0.record()
        for _ in range(args.steps):
            e, g = ub.value_and_grad(flat)
        ev1.record()
        torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / args.steps
    ub.check()

    eh = torch.empty((QB_COUNT,), dtype=torch.float32).pin_memory()
    gh = torch.empty((ub.nparams,), dtype=torch.float32).pin_memory()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        p = flat_host.to(dev, non_blocking=True)
        e, g = ub.value_and_grad(p)
        eh.copy_(e, non_blocking=True)
        gh.copy_(g, non_blocking=True)
    e1.record()
    torch.cuda.synchronize()
    ms_e2e = e0.elapsed_time(e1) / args.steps

    # value-only calls (forward + measure) to split the step into sweeps
    v0, v1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ub.value_and_grad(flat, grad=False)
    torch.cuda.synchronize()
    v0.record()
    for _ in range(max(3, args.steps)):
        ub.value_and_grad(flat, grad=False)
    v1.record()
    torch.cuda.synchronize()
    ms_val = v0.elapsed_time(v1) / max(3, args.steps)
    st = ub.stats()
    alg_total = sum(x["alg_bytes"] for x in st.values())
    alg_bwd = st["adjoint"]["alg_bytes"] + st["accumulate"]["alg_bytes"]
    peak, peak_kind = _peaks()
    achieved = alg_total / (ms / 1e3) / 1e9
    # DRAM bytes of the four sweeps per algorithmic byte, from the capture of
    # a 64-circuit prefix of the same workload (the sweeps stream every tile
    # once, so traffic grows with the algorithmic bytes)
    ratio = _traffic("batch_kernel_traffic_per_alg_byte", True)
    traffic = float(ratio) * alg_total if ratio is not None else None
    if rank != 0:
        return
    cpu = None if args.no_cpu else cpu_qaoa(specs, params)
    loop = None if nested else per_circuit_loop(specs, params)
    ns = [s[0] for s in specs]
    line = {
        "metric": QB_METRIC, "value": QB_COUNT / (ms / 1e3), "unit": QB_UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c64", "data": "synthetic",
        "config": {"workload": QB_WORKLOAD, "circuits": QB_COUNT, "seed": QB_SEED, "n_min": min(ns),
                   "n_max": max(ns), "params": int(ub.nparams), "tile_bits": ub.tile_bits,
                   "zrun_max": ub.zrun_max,
                   "autotune": "tile width x Z-rotation fusion width (0 = runs of up to 32, 1 = none); "
                               "autotune_ms lists [tile_bits, zrun_max, ms per call]",
                   "autotune_ms": getattr(ub, "tune_log", None), "setup_s": setup_s,
                   "state_gib": float(sum(1 << n for n in ns) * 8 / 2 ** 30),
                   "l2": "no flush: the 12 GiB of states exceed the 129 MB L2"},
        "roofline": {"bound": "hbm", "kernel": "batch_kernel (all four persistent sweeps of one step)",
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_kind, "traffic": traffic, "alg_bytes_per_step": alg_total,
                     "value_only_ms": ms_val,
                     "adjoint_part": {"ms": ms - ms_val, "alg_bytes": alg_bwd,
                                      "GB_per_s": alg_bwd / max(ms - ms_val, 1e-6) * 1e3 / 1e9},
                     "sweeps": st},
        "cpu_baseline": cpu,
        "per_circuit_loop_same_engine": loop,
        "e2e": {"value": QB_COUNT / (ms_e2e / 1e3), "unit": QB_UNIT, "h2d_bytes_per_step": int(ub.nparams * 4),
                "d2h_bytes_per_step": int((QB_COUNT + ub.nparams) * 4)},
        "clocks": clk.summary(),
        "gpu_launches": int(launches_per_step * args.steps),
        "gpu_launches_per_step": int(launches_per_step),
    }
    return line


MC_N, MC_LAYERS, MC_GAMMA, MC_SEED = 10, 4, 0.15, 7
MC_TRAJ = 1024
MC_NSTATUS = MC_LAYERS * (MC_N - 1) * 2
MC_METRIC = "MC-noise trajectories/s, value+grad (n=10, 4 layers, 72 phase-damping channels, <Z5>)"
MC_UNIT = "trajectories/s"
MC_WORKLOAD = "mcnoise_n10_l4_phasedamping"


def _mc_inputs():
    rng = np.random.default_rng(MC_SEED)
    params = rng.uniform(0, 2 * np.pi, (MC_LAYERS, MC_N)).astype(np.float32)
    status = rng.random((MC_TRAJ, MC_NSTATUS), dtype=np.float32)
    return params, status


def mcnoise_energy(tc, params, status):
    """examples/mcnoise_boost_v2.py:20-37 at n=10, 4 layers: H on all; per
    layer cnot(i, i+1) then phase damping (gamma 0.15, a general Kraus
    channel) on i and i+1; rx(params[j, i]) on all; <Z_5>."""
    import torch

    c = tc.Circuit(MC_N)
    for i in range(MC_N):
        c.H(i)
    s = 0
    for j in range(MC_LAYERS):
        for i in range(MC_N - 1):
            c.cnot(i, i + 1)
            c.phasedamping(i, gamma=MC_GAMMA, status=status[s])
            c.phasedamping(i + 1, gamma=MC_GAMMA, status=status[s + 1])
            s += 2
        for i in range(MC_N):
            c.rx(i, theta=params[j, i])
    return torch.real(c.expectation_ps(z=[MC_N // 2]))


def _mc_cpu_worker(chunk):
    from oracle import reference_algo as ra

    params, status = _mc_inputs()
    t0 = time.perf_counter()
    for b in chunk:
        ra.mcnoise_value_and_grad(MC_N, MC_LAYERS, MC_GAMMA, params, status[b], 1)
    return time.perf_counter() - t0


def cpu_mcnoise(per_core=48):
    """Labelled torch restatement of the reference algorithm (per-gate
    tensordot, general_kraus probabilities by contraction, taped AD), one
    trajectory per call, spread over the host cores by a spawn pool."""
    import multiprocessing as mp

    cores = len(os.sched_getaffinity(0))
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        pool.map(_mc_cpu_worker, [[b] for b in range(cores)])  # import + first-call warm-up
        chunks = [list(range(w * per_core, (w + 1) * per_core)) for w in range(cores)]
        t0 = time.perf_counter()
        pool.map(_mc_cpu_worker, chunks)
        dt = time.perf_counter() - t0
    ntraj = cores * per_core
    return {"value": ntraj / dt, "unit": MC_UNIT, "cores": cores, "kind": "port",
            "sample": "%d trajectories (%d per core, %.1f s wall; labelled torch restatement of the reference "
                      "algorithm: per-gate tensordot, general_kraus by contraction, taped AD)" %
                      (ntraj, per_core, dt)}


def run_mcnoise(args, rank, world):
    """Monte-Carlo noise trajectories: ``MC_TRAJ`` status vectors (seed 7)
    through ``K.vvag(f, argnums=params, vectorized_argnums=status)`` -- every
    trajectory's <Z_5> and the parameter gradient summed over trajectories,
    each general-Kraus channel one segment boundary of the batched sweep."""
    import torch

    import tensorcircuit_gb300 as tc
    from tensorcircuit_gb300 import _native

    tc.build()
    lib = _native.load()
    K_ = tc.set_backend("pytorch")
    dev = torch.device("cuda", torch.cuda.current_device())
    params_np, status_np = _mc_inputs()
    ntraj = args.trajectories
    status_np = np.resize(status_np, (ntraj, MC_NSTATUS))
    p_host = torch.from_numpy(params_np).pin_memory()
    s_host = torch.from_numpy(status_np).pin_memory()
    p_dev, s_dev = p_host.to(dev), s_host.to(dev)

    def f(p, st):
        return mcnoise_energy(tc, p, st)

    eager = K_.vvag(f, argnums=0, vectorized_argnums=1)
    # the reference's own trajectory examples jit the value_and_grad; here
    # the jit replays the whole step (every segment) from one CUDA graph
    step = eager if args.mc_eager else K_.jit(eager)
    warmup = max(args.warmup, 3)
    for _ in range(warmup + 1):
        v, g = step(p_dev, s_dev)
    torch.cuda.synchronize()
    # engine kernels per step, counted on one eager call (a graph replay
    # launches the same kernels without passing the host-side counter)
    l0 = lib.tcg_launch_count()
    eager(p_dev, s_dev)
    torch.cuda.synchronize()
    launches_per_step = lib.tcg_launch_count() - l0
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev.index) as clk:
        torch.cuda.synchronize()
        ev0.record()
        for _ in range(args.steps):
            v, g = step(p_dev, s_dev)
        ev1.record()
        torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / args.steps
    vh = torch.empty((ntraj,), dtype=torch.float32).pin_memory()
    gh = torch.empty(tuple(params_np.shape), dtype=torch.float32).pin_memory()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(args.steps):
        v, g = step(p_host.to(dev, non_blocking=True), s_host.to(dev, non_blocking=True))
        vh.copy_(v, non_blocking=True)
        gh.copy_(g, non_blocking=True)
    e1.record()
    torch.cuda.synchronize()
    ms_e2e = e0.elapsed_time(e1) / args.steps
    # segments: one per channel plus the last; per segment and trajectory a
    # forward pass (16 B/amp), the Pauli measurement (8), the cotangent
    # accumulation (24) and the adjoint pass (32)
    segs = MC_NSTATUS + 1
    alg = segs * 80 * (1 << MC_N) * ntraj
    peak, peak_kind = _peaks()
    achieved = alg / (ms / 1e3) / 1e9
    if rank != 0:
        return
    cpu = None if args.no_cpu else cpu_mcnoise()
    line = {
        "metric": MC_METRIC, "value": ntraj / (ms / 1e3), "unit": MC_UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c64", "data": "synthetic",
        "config": {"workload": MC_WORKLOAD, "trajectories": ntraj, "n_qubits": MC_N, "layers": MC_LAYERS,
                   "channels_per_trajectory": MC_NSTATUS, "gamma": MC_GAMMA, "seed": MC_SEED,
                   "jit": not args.mc_eager,
                   "jit_capture_errors": None if args.mc_eager else step.capture_errors(),
                   "l2": "no flush: %d trajectories x 8 KiB states stay in L2 (launch-latency bound)" % ntraj},
        "roofline": {"bound": "hbm", "kernel": "all engine sweeps of one step (segment passes)",
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_kind, "traffic": None, "alg_bytes_per_step": alg},
        "cpu_baseline": cpu,
        "e2e": {"value": ntraj / (ms_e2e / 1e3), "unit": MC_UNIT,
                "h2d_bytes_per_step": int(params_np.nbytes + status_np.nbytes),
                "d2h_bytes_per_step": int(ntraj * 4 + params_np.nbytes)},
        "clocks": clk.summary(),
        "gpu_launches": int(launches_per_step * args.steps),
        "gpu_launches_per_step": int(launches_per_step),
    }
    print(json.dumps(line), flush=True)


DM_N, DM_LAYERS, DM_P, DM_BATCH, DM_SEED = 10, 4, 0.01, 64, 8
DM_METRIC = "density-matrix value+grad circuits/s (n=10 noisy HEA, 4 layers, depolarizing 0.01, TFIM energy)"
DM_UNIT = "circuits/s"
DM_WORKLOAD = "dm_n10_l4_depol_b64_vvag"


def dm_energy(tc, params):
    """Noisy HEA on a density matrix: per layer rx on every qubit, rzz on
    the open chain, depolarizing(p, p, p) on every qubit; energy
    sum <Z_i Z_i+1> + sum <X_i>."""
    import torch

    c = tc.DMCircuit(DM_N)
    ps = params.unbind(-1)
    k = 0
    for _ in range(DM_LAYERS):
        for i in range(DM_N):
            c.rx(i, theta=ps[k])
            k += 1
        for i in range(DM_N - 1):
            c.rzz(i, i + 1, theta=ps[k])
            k += 1
        for i in range(DM_N):
            c.depolarizing(i, px=DM_P, py=DM_P, pz=DM_P)
    e = 0.0
    for i in range(DM_N - 1):
        e = e + torch.real(c.expectation_ps(z=[i, i + 1]))
    for i in range(DM_N):
        e = e + torch.real(c.expectation_ps(x=[i]))
    return e


def cpu_dm(sample=2):
    from oracle import reference_algo as ra

    threads = len(os.sched_getaffinity(0))
    rng = np.random.default_rng(DM_SEED)
    params = rng.uniform(0, 2 * np.pi, (DM_BATCH, DM_LAYERS * (2 * DM_N - 1))).astype(np.float32)
    ra.dm_value_and_grad(DM_N, 1, DM_P, params[0][: 2 * DM_N - 1], threads)  # warm-up
    t0 = time.perf_counter()
    for b in range(sample):
        ra.dm_value_and_grad(DM_N, DM_LAYERS, DM_P, params[b], threads)
    dt = time.perf_counter() - t0
    return {"value": sample / dt, "unit": DM_UNIT, "cores": threads, "kind": "port",
            "sample": "%d of the %d circuits (%.1f s; labelled torch restatement of the reference's DMCircuit2 "
                      "algorithm: per-gate tensordot on both legs of rho, superoperator channels, taped AD)" %
                      (sample, DM_BATCH, dt)}


def run_dm(args, rank, world):
    """Density matrices: ``DM_BATCH`` parameter vectors (seed 8) of the noisy
    HEA through ``K.jit(K.vvag(f))``; rho is a 20-qubit engine vector per
    circuit, each run of channels one segment boundary."""
    import torch

    import tensorcircuit_gb300 as tc
    from tensorcircuit_gb300 import _native

    tc.build()
    lib = _native.load()
    K_ = tc.set_backend("pytorch")
    dev = torch.device("cuda", torch.cuda.current_device())
    rng = np.random.default_rng(DM_SEED)
    params_np = rng.uniform(0, 2 * np.pi, (DM_BATCH, DM_LAYERS * (2 * DM_N - 1))).astype(np.float32)
    p_host = torch.from_numpy(params_np).pin_memory()
    p_dev = p_host.to(dev)
    eager = K_.vvag(lambda p: dm_energy(tc, p), argnums=0, vectorized_argnums=0)
    step = K_.jit(eager)
    warmup = max(args.warmup, 3)
    for _ in range(warmup + 1):
        v, g = step(p_dev)
    torch.cuda.synchronize()
    l0 = lib.tcg_launch_count()
    eager(p_dev)
    torch.cuda.synchronize()
    launches_per_step = lib.tcg_launch_count() - l0
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev.index) as clk:
        torch.cuda.synchronize()
        ev0.record()
        for _ in range(args.steps):
            v, g = step(p_dev)
        ev1.record()
        torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / args.steps
    vh = torch.empty((DM_BATCH,), dtype=torch.float32).pin_memory()
    gh = torch.empty(tuple(params_np.shape), dtype=torch.float32).pin_memory()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(args.steps):
        v, g = step(p_host.to(dev, non_blocking=True))
        vh.copy_(v, non_blocking=True)
        gh.copy_(g, non_blocking=True)
    e1.record()
    torch.cuda.synchronize()
    ms_e2e = e0.elapsed_time(e1) / args.steps
    if rank != 0:
        return
    cpu = None if args.no_cpu else cpu_dm()
    line = {
        "metric": DM_METRIC, "value": DM_BATCH / (ms / 1e3), "unit": DM_UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "c64", "data": "synthetic",
        "config": {"workload": DM_WORKLOAD, "n_qubits": DM_N, "engine_qubits": 2 * DM_N, "layers": DM_LAYERS,
                   "depolarizing": DM_P, "batch": DM_BATCH, "params": int(params_np.shape[1]), "seed": DM_SEED,
                   "jit_capture_errors": step.capture_errors(),
                   "l2": "no flush: 64 density matrices of 8 MiB (512 MiB) exceed the 129 MB L2"},
        "roofline": None,
        "cpu_baseline": cpu,
        "e2e": {"value": DM_BATCH / (ms_e2e / 1e3), "unit": DM_UNIT, "h2d_bytes_per_step": int(params_np.nbytes),
                "d2h_bytes_per_step": int(DM_BATCH * 4 + params_np.nbytes)},
        "clocks": clk.summary(),
        "gpu_launches": int(launches_per_step * args.steps),
        "gpu_launches_per_step": int(launches_per_step),
    }
    print(json.dumps(line), flush=True)


def run_warmstart(args, rank, world):
    """Learned warm start: random-coupling open TFIM n=16, HEA depth 6 (186
    angles), Adam lr 0.02; training angles generated by the engine's batched
    adjoint Adam (``--instances`` chains x 300 steps), the 31-256-256-186
    network trained with the project's kernels, then held-out chains
    optimised for 300 steps from the network's angles and from random ones,
    scored against the exact free-fermion ground energy."""
    import torch

    import tensorcircuit_gb300 as tc
    from tensorcircuit_gb300 import _native, warmstart as ws

    tc.build()
    lib = _native.load()
    dev = torch.device("cuda", torch.cuda.current_device())
    l0 = lib.tcg_launch_count()
    with ClockSampler(dev.index) as clk:
        r = ws.study(n_train=args.instances, n_test=args.held_out, steps=300, gen_steps=args.gen_steps,
                     epochs=args.epochs, plateau_chains=args.plateau_chains, plateau_steps=args.plateau_steps)
    launches = lib.tcg_launch_count() - l0
    if rank != 0:
        return
    gen_evals = args.instances * (args.gen_steps + 1)
    line = {
        "metric": "warm-start Adam steps to the random start's 300-step error (ratio random / warm)",
        "value": r["step_ratio"], "unit": "x fewer steps", "n_gpus": world, "steps": 1, "warmup": 0,
        "ms_per_step": 1e3 * sum(r["seconds"].values()), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "c64 simulator / bf16 network activations", "data": "synthetic",
        "config": {"workload": "tfim_n16_hea6_warmstart", "train_chains": args.instances,
                   "held_out": args.held_out, "epochs": args.epochs, "gen_steps": args.gen_steps, "seed": 6,
                   "plateau_chains": args.plateau_chains, "plateau_steps": args.plateau_steps},
        "study": r,
        "generation_throughput": {"value": gen_evals / r["seconds"]["generate"],
                                  "unit": "n=16 energy+gradient evaluations/s"},
        "cpu_baseline": None, "clocks": clk.summary(), "gpu_launches": int(launches),
    }
    print(json.dumps(line), flush=True)


def main():
    global BATCH, BW_N, QB_COUNT
    ap = argparse.ArgumentParser()
    ap.add_argument("--qaoa-circuits", type=int, default=QB_COUNT,
                    help="qaoa: circuits in the batch (512 is the configured workload; fewer for profiler captures)")
    ap.add_argument("--bw-qubits", type=int, default=BW_N,
                    help="brickwall: qubits (28 is the configured workload; fewer for profiler captures)")
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="hea", choices=["hea", "brickwall", "qaoa", "warmstart", "mcnoise", "dm"],
                    help="hea: n=20 HEA batched vvag (default); brickwall: n=28 Haar brick wall; "
                         "qaoa: 512 uneven QAOA circuits in one persistent launch per sweep; "
                         "warmstart: learned warm start for n=16 TFIM chains; "
                         "mcnoise: Monte-Carlo phase-damping trajectories, value+grad; "
                         "dm: noisy HEA on n=10 density matrices, value+grad")
    ap.add_argument("--trajectories", type=int, default=MC_TRAJ, help="mcnoise: trajectories per step")
    ap.add_argument("--mc-eager", action="store_true", help="mcnoise: run the step eagerly instead of replaying it from a CUDA graph")
    ap.add_argument("--batch", type=int, default=BATCH,
                    help="hea: parameter vectors per step (64 is the configured workload; smaller "
                         "batches are for profiler captures)")
    ap.add_argument("--instances", type=int, default=20000, help="warmstart: training chains")
    ap.add_argument("--plateau-chains", type=int, default=64, help="warmstart: held-out chains of the long runs")
    ap.add_argument("--plateau-steps", type=int, default=5000, help="warmstart: Adam steps of the long runs")
    ap.add_argument("--held-out", type=int, default=1000, help="warmstart: held-out chains")
    ap.add_argument("--epochs", type=int, default=200, help="warmstart: network training epochs")
    ap.add_argument("--gen-steps", type=int, default=2500,
                    help="warmstart: Adam steps that produce each training chain's target angles")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-brickwall", action="store_true",
                    help="default workload: skip the nested n=28 brick-wall measurement")
    ap.add_argument("--no-qaoa", action="store_true",
                    help="default workload: skip the nested 512-circuit uneven-batch measurement")
    args = ap.parse_args()
    BATCH = args.batch
    BW_N = args.bw_qubits
    QB_COUNT = args.qaoa_circuits
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        run_reference_arm(args, rank)
        return
    import torch

    if world > 1:
        local = int(os.environ.get("LOCAL_RANK", "0"))
        torch.cuda.set_device(local)
        torch.distributed.init_process_group("nccl")
    if args.workload == "brickwall":
        run_brickwall(args, rank, world)
    elif args.workload == "qaoa":
        run_qaoa(args, rank, world)
    elif args.workload == "warmstart":
        run_warmstart(args, rank, world)
    elif args.workload == "mcnoise":
        run_mcnoise(args, rank, world)
    elif args.workload == "dm":
        run_dm(args, rank, world)
    else:
        run_gb300_arm(args, rank, world)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
