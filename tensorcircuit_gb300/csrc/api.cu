// api.cu — the extern "C" entry points declared in include/tcgb300.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <vector>

#include "kernels.h"
#include "plan.h"

using namespace tcg;

namespace {

constexpr int kAbiVersion = 3;

inline cudaStream_t as_stream(void* s) { return static_cast<cudaStream_t>(s); }

int check_gate(int n, const tcg_gate& g) {
  if (g.kind != TCG_GATE_DENSE && g.kind != TCG_GATE_DIAG && g.kind != TCG_GATE_PAULI_ROT)
    return TCG_ERR_INVALID_ARG;
  if (g.kind == TCG_GATE_PAULI_ROT) {
    if (g.nq < 1 || g.nq > TCG_MAX_GATE_QUBITS) return TCG_ERR_INVALID_ARG;
    int nx = 0;
    for (int i = 0; i < g.nq; ++i) {
      if (g.pauli[i] < 1 || g.pauli[i] > 3) return TCG_ERR_INVALID_ARG;
      nx += g.pauli[i] != 3;
    }
    if (nx > kRBwd) return TCG_ERR_UNSUPPORTED;  // X/Y qubits must fit the registers
  }
  if (g.nq < 1 || g.nq > TCG_MAX_GATE_QUBITS) return TCG_ERR_INVALID_ARG;
  if (g.mat_off < 0) return TCG_ERR_INVALID_ARG;
  for (int i = 0; i < g.nq; ++i) {
    if (g.qubits[i] < 0 || g.qubits[i] >= n) return TCG_ERR_INVALID_ARG;
    for (int j = 0; j < i; ++j)
      if (g.qubits[i] == g.qubits[j]) return TCG_ERR_DUP_QUBIT;
  }
  if (g.grad_off >= 0 && g.nq > 2 && g.kind != TCG_GATE_PAULI_ROT) return TCG_ERR_UNSUPPORTED;
  return TCG_OK;
}

int cuda_rc(cudaError_t e) { return e == cudaSuccess ? TCG_OK : TCG_ERR_CUDA; }

int mplan_device(tcg_mplan* p, tcg_mplan::Dev* out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return TCG_ERR_CUDA;
  std::lock_guard<std::mutex> lk(p->mu);
  auto it = p->dev.find(dev);
  if (it != p->dev.end()) {
    *out = it->second;
    return TCG_OK;
  }
  const size_t nt = p->terms.size(), nd = p->direct.size();
  const size_t o_terms = 0;
  const size_t o_dir = (nt * sizeof(tcg_pauli) + 255) & ~size_t(255);
  const size_t o_ent = o_dir + ((nd * sizeof(int) + 255) & ~size_t(255));
  const size_t total = o_ent + nd * sizeof(int64_t) + 256;
  std::vector<char> host(total, 0);
  if (nt) std::memcpy(host.data() + o_terms, p->terms.data(), nt * sizeof(tcg_pauli));
  for (size_t i = 0; i < nd; ++i) {
    reinterpret_cast<int*>(host.data() + o_dir)[i] = p->direct[i];
    reinterpret_cast<int64_t*>(host.data() + o_ent)[i] = p->direct[i];
  }
  void* d = nullptr;
  if (cudaMalloc(&d, total) != cudaSuccess) return TCG_ERR_OOM;
  if (cudaMemcpy(d, host.data(), total, cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaFree(d);
    return TCG_ERR_CUDA;
  }
  tcg_mplan::Dev dv;
  dv.base = d;
  dv.terms = reinterpret_cast<tcg_pauli*>(static_cast<char*>(d) + o_terms);
  dv.direct = reinterpret_cast<int*>(static_cast<char*>(d) + o_dir);
  dv.direct_entries = reinterpret_cast<int64_t*>(static_cast<char*>(d) + o_ent);
  p->dev[dev] = dv;
  *out = dv;
  return TCG_OK;
}

constexpr uint32_t kDirectBlocks = 304;

// Tensor-core passes: TCG_TC=0 never, TCG_TC=1 every pass that qualifies,
// unset = the passes the planner's cost model prefers.
std::atomic<int> g_tc_policy{-1};

int tc_policy() {
  int pol = g_tc_policy.load();
  if (pol < 0) {
    const char* e = std::getenv("TCG_TC");
    pol = (e && e[0] == '0') ? 0 : (e && e[0] == '1') ? 1 : 2;
    int expect = -1;
    g_tc_policy.compare_exchange_strong(expect, pol);
    pol = g_tc_policy.load();
  }
  return pol;
}

bool tc_use_pass(const Program* P, int ps) {
  if (ps >= (int)P->tc_of_pass.size()) return false;
  const int t = P->tc_of_pass[ps];
  if (t < 0) return false;
  const int pol = tc_policy();
  return pol == 1 || (pol == 2 && P->tc_prefer[t]);
}

// Fused block matrices of one forward call (batch * slots blocks of
// kTcMatBytes, then batch * slots {1 / matrix scale, gain bound} pairs): a
// stream-ordered allocation on the call's stream, freed in stream order after
// the call's last pass, so that calls on different streams or threads never
// share one.  Outside stream capture it comes from a library pool per device
// that keeps up to kTcPoolKeep bytes between calls; under capture
// cudaMallocAsync / cudaFreeAsync become memory nodes of the graph.
constexpr uint64_t kTcPoolKeep = uint64_t(1) << 30;

int tc_pool(int dev, cudaMemPool_t* out) {
  static std::mutex mu;
  static std::map<int, cudaMemPool_t> pools;
  std::lock_guard<std::mutex> lk(mu);
  auto it = pools.find(dev);
  if (it != pools.end()) {
    *out = it->second;
    return TCG_OK;
  }
  cudaMemPoolProps props;
  std::memset(&props, 0, sizeof(props));
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = dev;
  cudaMemPool_t pool;
  if (cudaMemPoolCreate(&pool, &props) != cudaSuccess) {
    (void)cudaGetLastError();
    return TCG_ERR_CUDA;
  }
  uint64_t keep = kTcPoolKeep;
  (void)cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  pools[dev] = pool;
  *out = pool;
  return TCG_OK;
}

int tc_alloc(int64_t batch, int slots, cudaStream_t st, void** out) {
  const size_t nmat = size_t(batch) * size_t(slots);
  const size_t bytes = nmat * (size_t(kTcMatBytes) + sizeof(float2));
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cs) != cudaSuccess) {
    (void)cudaGetLastError();
    return TCG_ERR_CUDA;
  }
  cudaError_t e;
  if (cs != cudaStreamCaptureStatusNone) {
    e = cudaMallocAsync(out, bytes, st);
  } else {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return TCG_ERR_CUDA;
    cudaMemPool_t pool;
    const int rc = tc_pool(dev, &pool);
    if (rc != TCG_OK) return rc;
    e = cudaMallocFromPoolAsync(out, bytes, pool, st);
  }
  if (e != cudaSuccess) {
    (void)cudaGetLastError();  // an allocation failure is not a sticky error: clear it
    *out = nullptr;
    return TCG_ERR_OOM;
  }
  return TCG_OK;
}

// Frees a tc_alloc buffer in stream order when the call returns.
struct StreamOrderedFree {
  void* p = nullptr;
  cudaStream_t st = nullptr;
  ~StreamOrderedFree() {
    if (p) (void)cudaFreeAsync(p, st);
  }
};

// Runs every pass of a program direction: the specialised kernels when the
// JIT policy selects them for this plan (see jit.cpp), else the generic
// pass kernels of pass.cuh.
// dst[b] = src[b * stride] for batch rows of len complex entries: one copy
// when the rows are contiguous, one per row otherwise (stride 0: a shared row)
int copy_rows(float2* dst, const float2* src, int64_t stride, size_t len, int64_t batch, cudaStream_t st) {
  if (stride == int64_t(len))
    return cudaMemcpyAsync(dst, src, size_t(batch) * len * sizeof(float2), cudaMemcpyDeviceToDevice, st) ==
                   cudaSuccess
               ? TCG_OK
               : TCG_ERR_CUDA;
  for (int64_t b = 0; b < batch; ++b)
    if (cudaMemcpyAsync(dst + size_t(b) * len, src + size_t(b) * size_t(stride), len * sizeof(float2),
                        cudaMemcpyDeviceToDevice, st) != cudaSuccess)
      return TCG_ERR_CUDA;
  return TCG_OK;
}

int run_program(Program* P, int mode, int R, PassArgs& a, int64_t batch, cudaStream_t st) {
  if ((a.psi_in || a.mu_zero) && !P->passes.empty() && P->passes[0].stage_end == P->passes[0].stage_begin) {
    // a first pass without stages never loads or stores its tiles: put the
    // input where the sweep works in place instead
    const size_t len = size_t(1) << a.n;
    if (a.psi_in) {
      if (copy_rows(a.psi, a.psi_in, a.in_stride, len, batch, st) != TCG_OK) return TCG_ERR_CUDA;
      a.psi_in = nullptr;
    }
    if (a.mu_zero) {
      if (cudaMemsetAsync(a.mu, 0, size_t(batch) * len * sizeof(float2), st) != cudaSuccess) return TCG_ERR_CUDA;
      a.mu_zero = 0;
    }
  }
  JitKernels* jk = nullptr;
  {
    std::lock_guard<std::mutex> lk(P->jit_mu);
    const int pol = jit_policy();
    P->calls[mode] += 1;
    if (pol == 1 || (pol == 2 && P->calls[mode] >= 3)) {
      if (!P->jit[mode]) {
        P->jit[mode].reset(new (std::nothrow) JitKernels());
        if (P->jit[mode]) jit_build(*P, mode, R, P->jit[mode].get());
      }
      if (P->jit[mode] && !P->jit[mode]->failed) jk = P->jit[mode].get();
    }
  }
  const uint32_t ntiles = 1u << (a.n - P->L);
  // tensor-core passes of a forward sweep: fuse this call's block matrices
  bool any_tc = false;
  uint8_t* tc_fused = nullptr;
  float2* tc_scales = nullptr;
  StreamOrderedFree tc_buf;
  if (mode == MODE_FWD && !P->tc_passes.empty()) {
    for (int ps = 0; ps < (int)P->passes.size(); ++ps) any_tc = any_tc || tc_use_pass(P, ps);
    if (any_tc) {
      int rc = tc_alloc(batch, P->tc_slots, st, &tc_buf.p);
      if (rc != TCG_OK) return rc;
      tc_buf.st = st;
      tc_fused = static_cast<uint8_t*>(tc_buf.p);
      tc_scales = reinterpret_cast<float2*>(tc_fused + size_t(batch) * size_t(P->tc_slots) * kTcMatBytes);
      rc = cuda_rc(launch_tc_fuse(a.prog.tc_blocks, (int)P->tc_blocks.size(), a.prog.tc_gates, a.mats, a.mat_stride,
                                  batch, tc_fused, tc_scales, P->tc_slots, st));
      if (rc != TCG_OK) return rc;
    }
  }
  // a separate input state (psi_in) and a zero start of mu (mu_zero) apply
  // to the sweep's first pass only
  auto tc_launch = [&](int ps) -> int {
    const TcPassDesc& d = P->tc_passes[P->tc_of_pass[ps]];
    const DevPass& dp = P->passes[ps];
    return cuda_rc(launch_tc_pass(dp, d, a.prog.runs + dp.runs_off, a.prog.tc_blocks + d.block_begin, a.psi,
                                  ps == 0 ? a.psi_in : nullptr, a.in_stride, a.n, batch, tc_fused, tc_scales,
                                  P->tc_slots, a.prog.tc_err, st));
  };
  if (jk) {
    KParams_Host kp;
    kp.psi = a.psi;
    kp.mu = a.mu;
    kp.mats = a.mats;
    kp.mat_stride = a.mat_stride;
    kp.partial = a.partial;
    kp.part_stride = a.part_stride;
    kp.coef = a.coef;
    kp.coef_stride = a.coef_stride;
    kp.in_stride = a.in_stride;
    kp.pad = 0;
    for (int ps = 0; ps < (int)P->passes.size(); ++ps) {
      kp.psi_in = ps == 0 ? a.psi_in : nullptr;
      kp.mu_zero = ps == 0 ? a.mu_zero : 0;
      const int rc = (any_tc && tc_use_pass(P, ps)) ? tc_launch(ps)
                                                    : cuda_rc(jit_launch(jk, ps, kp, ntiles, batch, a.n, st));
      if (rc != TCG_OK) return rc;
    }
    return TCG_OK;
  }
  for (int ps = 0; ps < (int)P->passes.size(); ++ps) {
    PassArgs ap = a;
    ap.pass = ps;
    if (ps > 0) {
      ap.psi_in = nullptr;
      ap.mu_zero = 0;
    }
    const int rc = (any_tc && tc_use_pass(P, ps)) ? tc_launch(ps) : cuda_rc(launch_pass(mode, R, ap, P->L, batch, st));
    if (rc != TCG_OK) return rc;
  }
  return TCG_OK;
}

}  // namespace

extern "C" {

int32_t tcg_abi_version(void) { return kAbiVersion; }

int64_t tcg_launch_count(void) { return launch_count(); }

const char* tcg_status_string(int32_t s) {
  switch (s) {
    case TCG_OK: return "ok";
    case TCG_ERR_INVALID_ARG: return "invalid argument";
    case TCG_ERR_DUP_QUBIT: return "a gate lists the same qubit twice";
    case TCG_ERR_UNSUPPORTED: return "not supported by the engine";
    case TCG_ERR_CUDA: return "CUDA runtime error";
    case TCG_ERR_SCRATCH: return "scratch buffer too small";
    case TCG_ERR_OOM: return "allocation failed";
    case TCG_ERR_TOO_LARGE:
      return "request exceeds a fixed internal capacity of the entry point (see its limits in tcgb300.h)";
    case TCG_ERR_TIMEOUT: return "a bounded device-side wait ran out of time (results invalid)";
    default: return "unknown status";
  }
}

int tcg_plan_create(int32_t nqubits, const tcg_gate* gates, int32_t ngates, const tcg_plan_opts* opts,
                    tcg_plan** out) {
  if (!out) return TCG_ERR_INVALID_ARG;
  *out = nullptr;
  if (nqubits < kMinQubits || nqubits > kMaxQubits || ngates < 0 || (ngates > 0 && !gates))
    return TCG_ERR_INVALID_ARG;
  std::vector<PGate> pg;
  bool has_grad = false;
  int64_t grad_entries = 0;
  for (int i = 0; i < ngates; ++i) {
    const int rc = check_gate(nqubits, gates[i]);
    if (rc != TCG_OK) return rc;
    PGate g;
    std::memset(&g, 0, sizeof(g));
    g.kind = gates[i].kind;
    g.k = gates[i].nq;
    for (int q = 0; q < g.k; ++q) g.gbits[q] = nqubits - 1 - gates[i].qubits[q];
    g.mat_off = gates[i].mat_off;
    g.grad_off = gates[i].grad_off;
    if (g.kind == TCG_GATE_PAULI_ROT) {
      for (int q = 0; q < g.k; ++q) {
        const uint64_t bit = 1ull << g.gbits[q];
        if (gates[i].pauli[q] != 3) g.xmask |= bit;  // X or Y
        if (gates[i].pauli[q] != 1) g.zmask |= bit;  // Z or Y
      }
    }
    if (g.grad_off >= 0) {
      has_grad = true;
      const int64_t E = (g.kind == TCG_GATE_PAULI_ROT) ? 1 : (g.kind == TCG_GATE_DIAG) ? (1 << g.k) : (1 << (2 * g.k));
      grad_entries = std::max(grad_entries, g.grad_off + E);
    }
    pg.push_back(g);
  }
  PlanOpts po;
  if (opts && opts->tile_bits > 0) {
    po.tile_bits_fwd = std::min(opts->tile_bits, kRFwd + 8);  // at most 256 threads
    po.tile_bits_bwd = std::min(opts->tile_bits, kRBwd + 8);
  }
  if (opts && opts->max_stage_grad_entries > 0) po.max_stage_slots = std::max(16, opts->max_stage_grad_entries);
  if (opts && opts->zrun_max < 0) return TCG_ERR_INVALID_ARG;
  if (opts && opts->zrun_max > 0) po.zrun_max = std::min(opts->zrun_max, po.zrun_max);
  if (po.tile_bits_fwd < kRFwd + 1 || po.tile_bits_bwd < kRBwd + 1) return TCG_ERR_INVALID_ARG;
  tcg_plan* p = new (std::nothrow) tcg_plan();
  if (!p) return TCG_ERR_OOM;
  p->n = nqubits;
  p->ngates = ngates;
  p->has_grad = has_grad;
  p->grad_entries = grad_entries;
  std::vector<PGate> fwd_gates = pg;
  for (PGate& g : fwd_gates) g.grad_off = -1;
  p->fwd.zrun_max = po.zrun_max;
  p->bwd.zrun_max = po.zrun_max;
  int rc = build_gate_program(nqubits, fwd_gates, po.tile_bits_fwd, kRFwd, false, po.max_stage_slots, &p->fwd);
  if (rc == TCG_OK) plan_tensor_passes(&p->fwd, fwd_gates);
  if (rc == TCG_OK)
    rc = build_gate_program(nqubits, pg, po.tile_bits_bwd, kRBwd, true, po.max_stage_slots, &p->bwd);
  if (rc != TCG_OK) {
    delete p;
    return rc;
  }
  *out = p;
  return TCG_OK;
}

int tcg_plan_destroy(tcg_plan* plan) {
  if (!plan) return TCG_OK;
  program_free(&plan->fwd);
  program_free(&plan->bwd);
  delete plan;
  return TCG_OK;
}

int32_t tcg_set_tensor_policy(int32_t policy) {
  const int prev = tc_policy();
  if (policy >= 0 && policy <= 2) g_tc_policy.store(policy);
  return prev;
}

int tcg_plan_tensor_passes(const tcg_plan* plan) {
  if (!plan) return -1;
  int c = 0;
  for (int ps = 0; ps < (int)plan->fwd.passes.size(); ++ps) c += tc_use_pass(&plan->fwd, ps) ? 1 : 0;
  return c;
}

int tcg_plan_check(const tcg_plan* plan, void* stream) {
  if (!plan) return TCG_ERR_INVALID_ARG;
  tcg_plan* p = const_cast<tcg_plan*>(plan);
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return TCG_ERR_CUDA;
  if (cudaStreamSynchronize(as_stream(stream)) != cudaSuccess) return TCG_ERR_CUDA;
  std::lock_guard<std::mutex> lk(p->fwd.mu);
  auto it = p->fwd.dev.find(dev);
  if (it == p->fwd.dev.end()) return TCG_OK;  // never ran on this device
  unsigned int* ef = it->second.view.tc_err;
  unsigned int flag = 0;
  if (cudaMemcpy(&flag, ef, sizeof(flag), cudaMemcpyDeviceToHost) != cudaSuccess) return TCG_ERR_CUDA;
  if (flag) {
    if (cudaMemset(ef, 0, sizeof(flag)) != cudaSuccess) return TCG_ERR_CUDA;
    return TCG_ERR_TIMEOUT;
  }
  return TCG_OK;
}

int tcg_debug_tc_program(const tcg_plan* plan, const void** arrays, int64_t* counts, int64_t* sizes) {
  if (!plan || !arrays || !counts || !sizes) return TCG_ERR_INVALID_ARG;
  const Program& p = plan->fwd;
  arrays[0] = p.tc_passes.data();
  arrays[1] = p.tc_blocks.data();
  arrays[2] = p.tc_gates.data();
  arrays[3] = p.tc_prefer.data();
  counts[0] = (int64_t)p.tc_passes.size();
  counts[1] = (int64_t)p.tc_blocks.size();
  counts[2] = (int64_t)p.tc_gates.size();
  counts[3] = (int64_t)p.tc_prefer.size();
  sizes[0] = sizeof(TcPassDesc);
  sizes[1] = sizeof(TcBlock);
  sizes[2] = sizeof(TcGate);
  sizes[3] = sizeof(int);
  return TCG_OK;
}

int tcg_debug_tc_mma(const void* a, const void* b, float* d, int32_t k, int32_t n, unsigned int* err, void* stream) {
  if (!a || !b || !d || !err) return TCG_ERR_INVALID_ARG;
  if (k < 16 || k > 64 || k % 16 || n < 32 || n > 256 || n % 32) return TCG_ERR_INVALID_ARG;
  return cuda_rc(launch_tc_mma_probe(a, b, d, k, n, err, as_stream(stream)));
}

int tcg_plan_get_stats(const tcg_plan* plan, tcg_plan_stats* out) {
  if (!plan || !out) return TCG_ERR_INVALID_ARG;
  out->nqubits = plan->n;
  out->ngates = plan->ngates;
  out->npasses = (int)plan->fwd.passes.size();
  out->nstages = (int)plan->fwd.stages.size();
  out->tile_bits = plan->fwd.L;
  out->grad_entries = plan->grad_entries;
  return TCG_OK;
}

int tcg_forward(const tcg_plan* plan, void* psi, int64_t batch, const void* mats, int64_t mat_stride,
                void* stream) {
  if (!plan || !psi || batch < 0) return TCG_ERR_INVALID_ARG;
  if (batch == 0) return TCG_OK;
  if (plan->ngates > 0 && !mats) return TCG_ERR_INVALID_ARG;
  tcg_plan* p = const_cast<tcg_plan*>(plan);
  ProgramView view;
  int rc = program_device_view(&p->fwd, &view);
  if (rc != TCG_OK) return rc;
  if (plan->ngates == 0) return TCG_OK;
  PassArgs a;
  std::memset(&a, 0, sizeof(a));
  a.prog = view;
  a.n = plan->n;
  a.psi = static_cast<float2*>(psi);
  a.mats = static_cast<const float2*>(mats);
  a.mat_stride = mat_stride;
  a.max_slots = 0;
  return run_program(&p->fwd, MODE_FWD, kRFwd, a, batch, as_stream(stream));
}

int tcg_forward_from(const tcg_plan* plan, const void* psi_in, int64_t in_stride, void* psi, int64_t batch,
                     const void* mats, int64_t mat_stride, void* stream) {
  if (!plan || !psi || !psi_in || batch < 0 || in_stride < 0) return TCG_ERR_INVALID_ARG;
  if (batch == 0) return TCG_OK;
  const int64_t N = int64_t(1) << plan->n;
  if (psi_in == psi && in_stride != N) return TCG_ERR_INVALID_ARG;
  if (plan->ngates == 0 || psi_in == psi) {
    if (psi_in != psi)  // no passes: the output is the input
      return copy_rows(static_cast<float2*>(psi), static_cast<const float2*>(psi_in), in_stride, size_t(N), batch,
                       as_stream(stream));
    return tcg_forward(plan, psi, batch, mats, mat_stride, stream);
  }
  if (!mats) return TCG_ERR_INVALID_ARG;
  tcg_plan* p = const_cast<tcg_plan*>(plan);
  ProgramView view;
  int rc = program_device_view(&p->fwd, &view);
  if (rc != TCG_OK) return rc;
  PassArgs a;
  std::memset(&a, 0, sizeof(a));
  a.prog = view;
  a.n = plan->n;
  a.psi = static_cast<float2*>(psi);
  a.psi_in = static_cast<const float2*>(psi_in);
  a.in_stride = in_stride;
  a.mats = static_cast<const float2*>(mats);
  a.mat_stride = mat_stride;
  a.max_slots = 0;
  return run_program(&p->fwd, MODE_FWD, kRFwd, a, batch, as_stream(stream));
}

size_t tcg_backward_scratch_bytes(const tcg_plan* plan, int64_t batch) {
  if (!plan) return 0;
  const size_t ntiles = size_t(1) << (plan->n - plan->bwd.L);
  return size_t(batch) * size_t(std::max<int64_t>(plan->bwd.nout, 1)) * ntiles * sizeof(float2) + 256;
}

namespace {
int backward_impl(const tcg_plan* plan, const void* psi_in, void* psi, void* mu, int64_t batch, const void* mats,
                  int64_t mat_stride, void* grads, int64_t grad_stride, void* scratch, size_t scratch_bytes,
                  void* stream) {
  if (!plan || !psi || !mu || batch < 0) return TCG_ERR_INVALID_ARG;
  if (batch == 0) return TCG_OK;
  if (plan->ngates == 0) {
    if (psi_in && psi_in != psi &&
        cudaMemcpyAsync(psi, psi_in, size_t(batch) * (size_t(1) << plan->n) * sizeof(float2),
                        cudaMemcpyDeviceToDevice, as_stream(stream)) != cudaSuccess)
      return TCG_ERR_CUDA;
    return TCG_OK;
  }
  if (!mats) return TCG_ERR_INVALID_ARG;
  if (plan->has_grad && (!grads || grad_stride < plan->grad_entries)) return TCG_ERR_INVALID_ARG;
  tcg_plan* p = const_cast<tcg_plan*>(plan);
  const size_t need = tcg_backward_scratch_bytes(plan, batch);
  if (plan->has_grad && (!scratch || scratch_bytes < need)) return TCG_ERR_SCRATCH;
  ProgramView view;
  int rc = program_device_view(&p->bwd, &view);
  if (rc != TCG_OK) return rc;
  PassArgs a;
  std::memset(&a, 0, sizeof(a));
  a.prog = view;
  a.n = plan->n;
  a.psi = static_cast<float2*>(psi);
  a.mu = static_cast<float2*>(mu);
  if (psi_in && psi_in != psi) {
    a.psi_in = static_cast<const float2*>(psi_in);
    a.in_stride = int64_t(1) << plan->n;
  }
  a.mats = static_cast<const float2*>(mats);
  a.mat_stride = mat_stride;
  a.partial = static_cast<float2*>(scratch);
  a.part_stride = std::max<int64_t>(p->bwd.nout, 1);
  a.max_slots = std::max(p->bwd.max_slots, 1);
  rc = run_program(&p->bwd, MODE_BWD, kRBwd, a, batch, as_stream(stream));
  if (rc != TCG_OK) return rc;
  if (plan->has_grad) {
    const uint32_t ntiles = 1u << (plan->n - p->bwd.L);
    rc = cuda_rc(launch_reduce_partials(a.partial, a.part_stride, ntiles, view.entries, view.nentries, batch,
                                        static_cast<float2*>(grads), grad_stride, nullptr, 0,
                                        as_stream(stream)));
  }
  return rc;
}
}  // namespace

int tcg_backward(const tcg_plan* plan, void* psi, void* mu, int64_t batch, const void* mats,
                 int64_t mat_stride, void* grads, int64_t grad_stride, void* scratch, size_t scratch_bytes,
                 void* stream) {
  return backward_impl(plan, nullptr, psi, mu, batch, mats, mat_stride, grads, grad_stride, scratch, scratch_bytes,
                       stream);
}

int tcg_backward_from(const tcg_plan* plan, const void* psi_out, void* psi, void* mu, int64_t batch,
                      const void* mats, int64_t mat_stride, void* grads, int64_t grad_stride, void* scratch,
                      size_t scratch_bytes, void* stream) {
  if (!psi_out) return TCG_ERR_INVALID_ARG;
  return backward_impl(plan, psi_out, psi, mu, batch, mats, mat_stride, grads, grad_stride, scratch, scratch_bytes,
                       stream);
}

int tcg_mplan_create(int32_t nqubits, const tcg_pauli* terms, int32_t nterms, tcg_mplan** out) {
  if (!out) return TCG_ERR_INVALID_ARG;
  *out = nullptr;
  if (nqubits < kMinQubits || nqubits > kMaxQubits || nterms < 0 || (nterms > 0 && !terms))
    return TCG_ERR_INVALID_ARG;
  const uint64_t full = (nqubits >= 64) ? ~0ull : ((1ull << nqubits) - 1);
  for (int t = 0; t < nterms; ++t)
    if ((terms[t].xmask & ~full) || (terms[t].zmask & ~full)) return TCG_ERR_INVALID_ARG;
  tcg_mplan* p = new (std::nothrow) tcg_mplan();
  if (!p) return TCG_ERR_OOM;
  p->n = nqubits;
  p->nterms = nterms;
  p->terms.assign(terms, terms + nterms);
  PlanOpts po;
  int rc = build_term_program(nqubits, p->terms, po.tile_bits_fwd, kRFwd, po.max_stage_slots, &p->prog,
                              &p->direct);
  if (rc != TCG_OK) {
    delete p;
    return rc;
  }
  *out = p;
  return TCG_OK;
}

int tcg_mplan_destroy(tcg_mplan* plan) {
  if (!plan) return TCG_OK;
  program_free(&plan->prog);
  int cur = 0;
  cudaGetDevice(&cur);
  for (auto& kv : plan->dev) {
    cudaSetDevice(kv.first);
    cudaFree(kv.second.base);
  }
  cudaSetDevice(cur);
  delete plan;
  return TCG_OK;
}

int tcg_mplan_passes(const tcg_mplan* plan) {
  if (!plan) return -1;
  return (int)plan->prog.passes.size() + (int)plan->direct.size();
}

size_t tcg_expect_scratch_bytes(const tcg_mplan* plan, int64_t batch) {
  if (!plan) return 0;
  const size_t ntiles = size_t(1) << (plan->n - plan->prog.L);
  const size_t nt = std::max(plan->nterms, 1);
  return size_t(batch) * nt * (ntiles + kDirectBlocks) * sizeof(float2) + 512;
}

int tcg_expect_pauli(const tcg_mplan* plan, const void* psi, int64_t batch, double* out, void* scratch,
                     size_t scratch_bytes, void* stream) {
  if (!plan || !psi || !out || batch < 0) return TCG_ERR_INVALID_ARG;
  if (batch == 0 || plan->nterms == 0) return TCG_OK;
  if (!scratch || scratch_bytes < tcg_expect_scratch_bytes(plan, batch)) return TCG_ERR_SCRATCH;
  tcg_mplan* p = const_cast<tcg_mplan*>(plan);
  ProgramView view;
  int rc = program_device_view(&p->prog, &view);
  if (rc != TCG_OK) return rc;
  tcg_mplan::Dev dv;
  rc = mplan_device(p, &dv);
  if (rc != TCG_OK) return rc;
  const uint32_t ntiles = 1u << (plan->n - p->prog.L);
  float2* part_tiles = static_cast<float2*>(scratch);
  float2* part_direct = part_tiles + size_t(batch) * plan->nterms * ntiles;
  cudaStream_t st = as_stream(stream);
  if (!p->prog.passes.empty()) {
    PassArgs a;
    std::memset(&a, 0, sizeof(a));
    a.prog = view;
    a.n = plan->n;
    a.psi = const_cast<float2*>(static_cast<const float2*>(psi));
    a.partial = part_tiles;
    a.part_stride = plan->nterms;
    a.max_slots = std::max(p->prog.max_slots, 1);
    rc = run_program(&p->prog, MODE_MEAS, kRFwd, a, batch, st);
    if (rc != TCG_OK) return rc;
    rc = cuda_rc(launch_reduce_partials(part_tiles, plan->nterms, ntiles, view.entries, view.nentries, batch,
                                        nullptr, 0, out, plan->nterms, st));
    if (rc != TCG_OK) return rc;
  }
  if (!p->direct.empty()) {
    rc = cuda_rc(launch_direct_expect(static_cast<const float2*>(psi), plan->n, batch, dv.terms, dv.direct,
                                      (int)p->direct.size(), plan->nterms, part_direct, kDirectBlocks, st));
    if (rc != TCG_OK) return rc;
    rc = cuda_rc(launch_reduce_partials(part_direct, plan->nterms, kDirectBlocks, dv.direct_entries,
                                        (int64_t)p->direct.size(), batch, nullptr, 0, out, plan->nterms, st));
  }
  return rc;
}

int tcg_pauli_accumulate(const tcg_mplan* plan, const void* psi, void* mu, int64_t batch, const float* coef,
                         int64_t coef_stride, void* stream) {
  return tcg_pauli_accumulate_ex(plan, psi, mu, batch, coef, coef_stride, 0, stream);
}

int tcg_pauli_accumulate_ex(const tcg_mplan* plan, const void* psi, void* mu, int64_t batch, const float* coef,
                            int64_t coef_stride, int32_t flags, void* stream) {
  if (!plan || !psi || !mu || !coef || batch < 0 || (flags & ~TCG_ACC_OVERWRITE)) return TCG_ERR_INVALID_ARG;
  if (batch == 0) return TCG_OK;
  const bool overwrite = (flags & TCG_ACC_OVERWRITE) != 0;
  const size_t state_bytes = size_t(batch) * (size_t(1) << plan->n) * sizeof(float2);
  if (plan->nterms == 0) {
    if (overwrite && cudaMemsetAsync(mu, 0, state_bytes, as_stream(stream)) != cudaSuccess) return TCG_ERR_CUDA;
    return TCG_OK;
  }
  tcg_mplan* p = const_cast<tcg_mplan*>(plan);
  ProgramView view;
  int rc = program_device_view(&p->prog, &view);
  if (rc != TCG_OK) return rc;
  tcg_mplan::Dev dv;
  rc = mplan_device(p, &dv);
  if (rc != TCG_OK) return rc;
  cudaStream_t st = as_stream(stream);
  if (!p->prog.passes.empty()) {
    PassArgs a;
    std::memset(&a, 0, sizeof(a));
    a.prog = view;
    a.n = plan->n;
    a.psi = const_cast<float2*>(static_cast<const float2*>(psi));
    a.mu = static_cast<float2*>(mu);
    a.coef = coef;
    a.coef_stride = coef_stride;
    a.max_slots = 0;
    a.mu_zero = overwrite ? 1 : 0;  // the first pass writes mu instead of adding to it
    rc = run_program(&p->prog, MODE_PACC, kRFwd, a, batch, st);
    if (rc != TCG_OK) return rc;
  } else if (overwrite) {
    if (cudaMemsetAsync(mu, 0, state_bytes, st) != cudaSuccess) return TCG_ERR_CUDA;
  }
  if (!p->direct.empty())
    rc = cuda_rc(launch_direct_pacc(static_cast<const float2*>(psi), static_cast<float2*>(mu), plan->n, batch,
                                    dv.terms, dv.direct, (int)p->direct.size(), coef, coef_stride, st));
  return rc;
}

size_t tcg_sample_scratch_bytes(int32_t nqubits, int64_t batch) {
  if (nqubits < 1 || nqubits > kMaxQubits || batch < 0) return 0;
  return sample_scratch_bytes(nqubits, batch) + 256;
}

int tcg_sample(const void* psi, int32_t nqubits, int64_t batch, const float* u, int64_t u_stride,
               int64_t nshots, int64_t* out, void* scratch, size_t scratch_bytes, void* stream) {
  if (!psi || nqubits < 1 || nqubits > kMaxQubits || batch < 0 || nshots < 0 || u_stride < 0)
    return TCG_ERR_INVALID_ARG;
  if (batch == 0 || nshots == 0) return TCG_OK;
  if (!u || !out) return TCG_ERR_INVALID_ARG;
  if (!scratch || scratch_bytes < tcg_sample_scratch_bytes(nqubits, batch)) return TCG_ERR_SCRATCH;
  return cuda_rc(launch_sample(static_cast<const float2*>(psi), nqubits, batch, u, u_stride, nshots, out,
                               scratch, as_stream(stream)));
}

int tcg_kraus_pick(const void* ev, int32_t nstrings, const float* coef, int32_t nkraus, const float* x,
                   int64_t x_stride, int64_t batch, int32_t* pick, void* scale, float* p, void* stream) {
  if (batch < 0 || nstrings < 1 || nkraus < 1 || x_stride < 0) return TCG_ERR_INVALID_ARG;
  if (batch == 0) return TCG_OK;
  if (!ev || !coef || !x || !pick || !scale || !p) return TCG_ERR_INVALID_ARG;
  return cuda_rc(launch_kraus_pick(static_cast<const float2*>(ev), nstrings, coef, nkraus, x, x_stride, batch, pick,
                                   static_cast<float2*>(scale), p, as_stream(stream)));
}

int tcg_kraus_pick_backward(const void* gscale, const int32_t* pick, const float* p, int32_t nkraus,
                            const float* coef, int32_t nstrings, int64_t batch, void* gev, void* stream) {
  if (batch < 0 || nstrings < 1 || nkraus < 1) return TCG_ERR_INVALID_ARG;
  if (batch == 0) return TCG_OK;
  if (!gscale || !pick || !p || !coef || !gev) return TCG_ERR_INVALID_ARG;
  return cuda_rc(launch_kraus_pick_bwd(static_cast<const float2*>(gscale), pick, p, nkraus, coef, nstrings, batch,
                                       static_cast<float2*>(gev), as_stream(stream)));
}

int tcg_probability(const void* psi, int64_t len, float* p, void* stream) {
  if (len < 0 || (len > 0 && (!psi || !p))) return TCG_ERR_INVALID_ARG;
  return cuda_rc(launch_probability(static_cast<const float2*>(psi), len, p, as_stream(stream)));
}

size_t tcg_inner_scratch_bytes(int64_t len, int64_t batch) { return inner_scratch_bytes(len, batch) + 256; }

int tcg_inner(const void* a, const void* b, int64_t len, int64_t batch, double* out, void* scratch,
              size_t scratch_bytes, void* stream) {
  if (!a || !b || !out || len <= 0 || batch < 0) return TCG_ERR_INVALID_ARG;
  if (batch == 0) return TCG_OK;
  if (!scratch || scratch_bytes < tcg_inner_scratch_bytes(len, batch)) return TCG_ERR_SCRATCH;
  return cuda_rc(launch_inner(static_cast<const float2*>(a), static_cast<const float2*>(b), len, batch, out,
                              scratch, as_stream(stream)));
}

int tcg_debug_jit(const void* plan, int32_t which, int32_t mode, int32_t* state, char* text, int64_t cap,
                  int32_t what) {
  if (!plan || !state || mode < 0 || mode > 3) return TCG_ERR_INVALID_ARG;
  Program* p = nullptr;
  if (which == 0) p = &static_cast<tcg_plan*>(const_cast<void*>(plan))->fwd;
  else if (which == 1) p = &static_cast<tcg_plan*>(const_cast<void*>(plan))->bwd;
  else if (which == 2) p = &static_cast<tcg_mplan*>(const_cast<void*>(plan))->prog;
  else return TCG_ERR_INVALID_ARG;
  std::string s;
  {
    std::lock_guard<std::mutex> lk(p->jit_mu);
    *state = !p->jit[mode] ? 0 : (p->jit[mode]->failed ? -1 : 1);
    if (what == 0 && p->jit[mode]) s = p->jit[mode]->log;
  }
  if (what == 1) s = jit_source(*p, mode, mode == MODE_BWD ? kRBwd : kRFwd);
  if (text && cap > 0) {
    const size_t n = std::min<size_t>(s.size(), size_t(cap - 1));
    std::memcpy(text, s.data(), n);
    text[n] = 0;
  }
  return TCG_OK;
}

int tcg_debug_program(const void* plan, int32_t which, const void** arrays, int64_t* counts, int64_t* sizes) {
  if (!plan || !arrays || !counts || !sizes) return TCG_ERR_INVALID_ARG;
  const Program* p = nullptr;
  if (which == 0) p = &static_cast<const tcg_plan*>(plan)->fwd;
  else if (which == 1) p = &static_cast<const tcg_plan*>(plan)->bwd;
  else if (which == 2) p = &static_cast<const tcg_mplan*>(plan)->prog;
  else return TCG_ERR_INVALID_ARG;
  arrays[0] = p->passes.data();
  arrays[1] = p->stages.data();
  arrays[2] = p->ops.data();
  arrays[3] = p->slot_out.data();
  arrays[4] = p->runs.data();
  arrays[5] = p->zents.data();
  counts[0] = (int64_t)p->passes.size();
  counts[1] = (int64_t)p->stages.size();
  counts[2] = (int64_t)p->ops.size();
  counts[3] = (int64_t)p->slot_out.size();
  counts[4] = (int64_t)p->runs.size();
  counts[5] = (int64_t)p->zents.size();
  sizes[0] = sizeof(DevPass);
  sizes[1] = sizeof(DevStage);
  sizes[2] = sizeof(DevOp);
  sizes[3] = sizeof(SlotOut);
  sizes[4] = sizeof(uint32_t);
  sizes[5] = sizeof(ZEnt);
  return TCG_OK;
}

}  // extern "C"
