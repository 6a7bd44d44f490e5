// batch.cu — uneven batches: many parameterized circuits of different sizes
// and depths, value and adjoint gradient of each circuit's Pauli energy, with
// one persistent launch per sweep (pass.cuh: batch_kernel) instead of one
// launch per pass per circuit.
//
// One call = eight kernels in a fixed order (a CUDA graph captures it):
//   build_mats      rotation entries e^{i scale theta}, constants copied
//   init_states     |0...0> for every circuit (after a memset)
//   batch FWD       every pass of every circuit
//   batch MEAS      every circuit's Pauli terms -> per-tile partial sums
//   ragged reduce   energies (fixed-order float64)
//   batch PACC      mu = sum_t 2 coef_t P_t psi
//   batch BWD       adjoint sweep, dL/dphi per rotation -> partial sums
//   ragged reduce   parameter gradients (fixed-order float64)
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <new>
#include <vector>

#include "kernels.h"
#include "plan.h"

using namespace tcg;

namespace {

struct RedTask {
  int64_t item_begin;
  int64_t item_end;
  double offset;
};
struct RedItem {
  int64_t part_off;  // complex entries into the partial buffer
  uint32_t ntiles;
  float scale;
};

__device__ __forceinline__ double warp_sum_dbl(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// out[task] = offset + sum_items scale * sum_t Re(partial[part_off + t]);
// one warp per task, lane-strided tiles, fixed xor tree: deterministic.
__global__ void ragged_reduce_kernel(const float2* __restrict__ partial, const RedTask* __restrict__ tasks,
                                     int64_t ntasks, const RedItem* __restrict__ items, float* __restrict__ out) {
  const int64_t task = int64_t(blockIdx.x) * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (task >= ntasks) return;
  const RedTask T = tasks[task];
  double acc = 0.0;
  for (int64_t i = T.item_begin; i < T.item_end; ++i) {
    const RedItem it = items[i];
    const float2* p = partial + it.part_off;
    double s = 0.0;
    for (uint32_t t = lane; t < it.ntiles; t += 32) s += (double)p[t].x;
    acc += (double)it.scale * s;
  }
  acc = warp_sum_dbl(acc);
  if (lane == 0) out[task] = (float)(T.offset + acc);
}

// Rotation entries: (cos phi, sin phi), phi = scale * theta in float64 and
// rounded once; constant entries copied.
__global__ void build_mats_kernel(const float* __restrict__ params, const int64_t* __restrict__ pidx,
                                  const float* __restrict__ scale, const float2* __restrict__ cval, int64_t nmat,
                                  float2* __restrict__ mats) {
  for (int64_t j = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; j < nmat; j += int64_t(gridDim.x) * blockDim.x) {
    const int64_t k = pidx[j];
    if (k >= 0) {
      const double phi = (double)scale[j] * (double)params[k];
      double s, c;
      sincos(phi, &s, &c);
      mats[j] = make_float2((float)c, (float)s);
    } else {
      mats[j] = cval[j];
    }
  }
}

__global__ void init_states_kernel(float2* psi, const int64_t* __restrict__ state_off, int ncirc) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < ncirc) psi[state_off[c]] = make_float2(1.f, 0.f);
}

size_t al256(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace

struct tcg_ubatch {
  int ncirc = 0;
  int L = 0;
  int device = -1;
  std::vector<tcg_plan*> plans;
  std::vector<Program*> terms;      // measurement programs (one pass set per circuit)
  std::vector<int> nq;
  std::vector<int64_t> state_off;   // complex entries
  std::vector<int64_t> mat_base;    // complex entries
  std::vector<int64_t> param_base;
  int64_t state_total = 0, mat_total = 0, param_total = 0;
  int64_t part_total = 0;           // complex entries (max of MEAS and BWD)
  int max_slots[4] = {0, 0, 0, 0};
  int64_t nitems[4] = {0, 0, 0, 0};
  int nsegs[4] = {0, 0, 0, 0};
  int64_t n_energy_tasks = 0, n_grad_tasks = 0;
  bool lite = true;  // every program fits the lighter persistent body
  unsigned long long wait_ns = 2000000000ull;  // limit of one dependency wait

  // device tables (one allocation)
  void* dtab = nullptr;
  const BatchCirc* circ[4] = {nullptr, nullptr, nullptr, nullptr};
  const BatchSeg* segs[4] = {nullptr, nullptr, nullptr, nullptr};
  const int32_t* coarse[4] = {nullptr, nullptr, nullptr, nullptr};
  const int64_t* d_pidx = nullptr;
  const float* d_scale = nullptr;
  const float2* d_cval = nullptr;
  const float* d_coef = nullptr;
  const int64_t* d_state_off = nullptr;
  const RedTask* d_etasks = nullptr;
  const RedItem* d_eitems = nullptr;
  const RedTask* d_gtasks = nullptr;
  const RedItem* d_gitems = nullptr;

  // scratch layout (bytes)
  size_t o_psi = 0, o_mu = 0, o_mats = 0, o_part = 0, o_cnt = 0, scratch = 0;

  ~tcg_ubatch() {
    for (tcg_plan* p : plans) tcg_plan_destroy(p);
    for (Program* p : terms) {
      if (p) {
        program_free(p);
        delete p;
      }
    }
    if (dtab) cudaFree(dtab);
  }
};

namespace {

int rc_of(cudaError_t e) { return e == cudaSuccess ? TCG_OK : TCG_ERR_CUDA; }

// counters of one launch: queue, done[ncirc]
size_t counter_words(int ncirc) { return size_t(1) + size_t(ncirc); }

}  // namespace

extern "C" {

int tcg_ubatch_create(const tcg_ubatch_circuit* circuits, int32_t ncircuits, int32_t tile_bits,
                      tcg_ubatch** out) {
  tcg_plan_opts o;
  o.tile_bits = tile_bits;
  o.max_stage_grad_entries = 0;
  o.zrun_max = 0;
  return tcg_ubatch_create_ex(circuits, ncircuits, &o, out);
}

int tcg_ubatch_create_ex(const tcg_ubatch_circuit* circuits, int32_t ncircuits, const tcg_plan_opts* opts,
                         tcg_ubatch** out) {
  if (!out) return TCG_ERR_INVALID_ARG;
  *out = nullptr;
  if (!opts || opts->zrun_max < 0 || opts->max_stage_grad_entries < 0) return TCG_ERR_INVALID_ARG;
  const int tile_bits = opts->tile_bits;
  if (!circuits || ncircuits < 1 || tile_bits < kRFwd + 2 || tile_bits > kRFwd + 8) return TCG_ERR_INVALID_ARG;
  tcg_ubatch* B = new (std::nothrow) tcg_ubatch();
  if (!B) return TCG_ERR_OOM;
  B->ncirc = ncircuits;
  B->L = tile_bits;
  if (cudaGetDevice(&B->device) != cudaSuccess) {
    delete B;
    return TCG_ERR_CUDA;
  }
  const int C = ncircuits;
  // ---- per-circuit plans and measurement programs
  std::vector<RedTask> etasks, gtasks;
  std::vector<RedItem> eitems, gitems;
  std::vector<int64_t> pidx;
  std::vector<float> scale;
  std::vector<float2> cval;
  std::vector<float> coef;
  std::vector<BatchCirc> hc[4];
  int64_t meas_part = 0, bwd_part = 0, coef_total = 0;
  for (int c = 0; c < C; ++c) {
    const tcg_ubatch_circuit& U = circuits[c];
    const int n = U.nqubits;
    if (n < tile_bits || n > kMaxQubits || U.ngates < 0 || (U.ngates > 0 && !U.gates) || U.nmat < 1 ||
        !U.mat_const || !U.mat_param || !U.mat_scale || U.nparams < 0 || U.nterms < 0 ||
        (U.nterms > 0 && (!U.terms || !U.coef))) {
      delete B;
      return TCG_ERR_INVALID_ARG;
    }
    for (int g = 0; g < U.ngates; ++g) {
      const tcg_gate& G = U.gates[g];
      const int64_t E = (G.kind == TCG_GATE_PAULI_ROT) ? 1 : (G.kind == TCG_GATE_DIAG) ? (1 << G.nq) : (1 << (2 * G.nq));
      if (G.mat_off < 0 || G.mat_off + E > U.nmat) {
        delete B;
        return TCG_ERR_INVALID_ARG;
      }
      if (G.grad_off >= 0 && (G.kind != TCG_GATE_PAULI_ROT || U.mat_param[G.mat_off] < 0)) {
        delete B;
        return TCG_ERR_UNSUPPORTED;
      }
    }
    for (int64_t e = 0; e < U.nmat; ++e)
      if (U.mat_param[e] >= U.nparams) {
        delete B;
        return TCG_ERR_INVALID_ARG;
      }
    tcg_plan_opts po;
    po.tile_bits = tile_bits;
    po.max_stage_grad_entries = opts->max_stage_grad_entries;
    po.zrun_max = opts->zrun_max;
    tcg_plan* plan = nullptr;
    int rc = tcg_plan_create(n, U.gates, U.ngates, &po, &plan);
    if (rc != TCG_OK) {
      delete B;
      return rc;
    }
    B->plans.push_back(plan);
    Program* tp = new (std::nothrow) Program();
    if (!tp) {
      delete B;
      return TCG_ERR_OOM;
    }
    B->terms.push_back(tp);
    std::vector<tcg_pauli> tl(U.terms, U.terms + U.nterms);
    const uint64_t full = (1ull << n) - 1;
    for (const tcg_pauli& t : tl)
      if ((t.xmask & ~full) || (t.zmask & ~full)) {
        delete B;
        return TCG_ERR_INVALID_ARG;
      }
    std::vector<int> direct;
    PlanOpts dflt;
    rc = build_term_program(n, tl, tile_bits, kRFwd, dflt.max_stage_slots, tp, &direct);
    if (rc != TCG_OK) {
      delete B;
      return rc;
    }
    if (!direct.empty()) {  // terms with many X/Y bits need the one-pass-per-term kernel
      delete B;
      return TCG_ERR_UNSUPPORTED;
    }
    if (plan->fwd.L != tile_bits || plan->bwd.L != tile_bits || (tl.size() && tp->L != tile_bits)) {
      delete B;
      return TCG_ERR_INVALID_ARG;
    }
    B->nq.push_back(n);
    B->state_off.push_back(B->state_total);
    B->mat_base.push_back(B->mat_total);
    B->param_base.push_back(B->param_total);
    const uint32_t ntiles = 1u << (n - tile_bits);
    // matrices
    for (int64_t e = 0; e < U.nmat; ++e) {
      pidx.push_back(U.mat_param[e] >= 0 ? B->param_total + U.mat_param[e] : -1);
      scale.push_back(U.mat_scale[e]);
      cval.push_back(make_float2(U.mat_const[2 * e], U.mat_const[2 * e + 1]));
    }
    // energy task: offset + sum_t coef_t Re <P_t>
    RedTask et;
    et.item_begin = (int64_t)eitems.size();
    for (int t = 0; t < U.nterms; ++t) {
      RedItem it;
      it.part_off = meas_part + int64_t(t) * ntiles;
      it.ntiles = ntiles;
      it.scale = U.coef[t];
      eitems.push_back(it);
      coef.push_back(2.0f * U.coef[t]);
    }
    et.item_end = (int64_t)eitems.size();
    et.offset = U.offset;
    etasks.push_back(et);
    // gradient tasks: one per parameter, its rotations in gate order
    const int64_t bstride = std::max<int64_t>(plan->bwd.nout, 1);
    for (int k = 0; k < U.nparams; ++k) {
      RedTask gt;
      gt.item_begin = (int64_t)gitems.size();
      for (int g = 0; g < U.ngates; ++g) {
        const tcg_gate& G = U.gates[g];
        if (G.grad_off >= 0 && U.mat_param[G.mat_off] == k) {
          RedItem it;
          it.part_off = bwd_part + G.grad_off * int64_t(ntiles);
          it.ntiles = ntiles;
          it.scale = U.mat_scale[G.mat_off];
          gitems.push_back(it);
        }
      }
      gt.item_end = (int64_t)gitems.size();
      gt.offset = 0.0;
      gtasks.push_back(gt);
    }
    // launch descriptors (program views are filled in at upload)
    BatchCirc bc;
    std::memset(&bc, 0, sizeof(bc));
    bc.n = n;
    bc.state_off = B->state_total;
    bc.mat_off = B->mat_total;
    BatchCirc f = bc;
    f.max_slots = 0;
    hc[MODE_FWD].push_back(f);
    BatchCirc m = bc;
    m.part_off = meas_part;
    m.part_stride = std::max(U.nterms, 1);
    m.max_slots = std::max(tp->max_slots, 1);
    hc[MODE_MEAS].push_back(m);
    BatchCirc a = bc;
    a.coef_off = coef_total;
    a.max_slots = 0;
    hc[MODE_PACC].push_back(a);
    BatchCirc b = bc;
    b.part_off = bwd_part;
    b.part_stride = bstride;
    b.max_slots = std::max(plan->bwd.max_slots, 1);
    hc[MODE_BWD].push_back(b);
    B->max_slots[MODE_MEAS] = std::max(B->max_slots[MODE_MEAS], m.max_slots);
    B->max_slots[MODE_BWD] = std::max(B->max_slots[MODE_BWD], b.max_slots);
    meas_part += int64_t(std::max(U.nterms, 1)) * ntiles;
    bwd_part += bstride * ntiles;
    coef_total += U.nterms;
    B->state_total += int64_t(1) << n;
    B->mat_total += U.nmat;
    B->param_total += U.nparams;
  }
  B->part_total = std::max(meas_part, bwd_part);
  // the lighter kernel body covers 1-qubit dense gates, Pauli rotations,
  // Z-rotation runs and Pauli terms in register stages
  auto lite_ok = [](const Program& p) {
    for (const DevStage& s : p.stages)
      if (s.smem_stage) return false;
    for (const DevOp& o : p.ops)
      if (o.kind != OP_DENSE1 && o.kind != OP_PROT && o.kind != OP_ZRUN && o.kind != OP_EXPECT) return false;
    return true;
  };
  for (int c = 0; c < C; ++c)
    if (!lite_ok(B->plans[c]->fwd) || !lite_ok(B->plans[c]->bwd) || !lite_ok(*B->terms[c])) B->lite = false;
  B->n_energy_tasks = (int64_t)etasks.size();
  B->n_grad_tasks = (int64_t)gtasks.size();
  if (coef.empty()) coef.push_back(0.f);
  if (eitems.empty()) eitems.push_back(RedItem{0, 0, 0.f});
  if (gitems.empty()) gitems.push_back(RedItem{0, 0, 0.f});
  if (gtasks.empty()) gtasks.push_back(RedTask{0, 0, 0.0});

  // ---- segments: pass-major, larger circuits first within a pass
  std::vector<BatchSeg> hs[4];
  std::vector<int32_t> hcoarse[4];
  const int modes[4] = {MODE_FWD, MODE_BWD, MODE_MEAS, MODE_PACC};
  std::vector<int> order(C);
  for (int c = 0; c < C; ++c) order[c] = c;
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return B->nq[x] > B->nq[y]; });
  for (int mi = 0; mi < 4; ++mi) {
    const int mode = modes[mi];
    int maxp = 0;
    auto npass = [&](int c) -> int {
      if (mode == MODE_FWD) return (int)B->plans[c]->fwd.passes.size();
      if (mode == MODE_BWD) return (int)B->plans[c]->bwd.passes.size();
      return (int)B->terms[c]->passes.size();
    };
    for (int c = 0; c < C; ++c) maxp = std::max(maxp, npass(c));
    int64_t item = 0;
    for (int p = 0; p < maxp; ++p) {
      for (int c : order) {
        if (p >= npass(c)) continue;
        BatchSeg s;
        s.item0 = item;
        s.circ = c;
        s.pass = p;
        s.ntiles = 1u << (B->nq[c] - tile_bits);
        s.need = uint32_t(p) * s.ntiles;
        hs[mode].push_back(s);
        item += s.ntiles;
      }
    }
    if (item >= (int64_t(1) << 31)) {
      delete B;
      return TCG_ERR_TOO_LARGE;
    }
    B->nitems[mode] = item;
    B->nsegs[mode] = (int)hs[mode].size();
    if (hs[mode].empty()) hs[mode].push_back(BatchSeg{0, 0, 0, 0, 0});
    // coarse index: segment holding item k * kBatchCoarse (clamped to the last item)
    {
      const int64_t nk = item / kBatchCoarse + 2;
      hcoarse[mode].resize((size_t)nk);
      size_t sgi = 0;
      for (int64_t k = 0; k < nk; ++k) {
        const int64_t it = std::min<int64_t>(k * kBatchCoarse, std::max<int64_t>(item - 1, 0));
        while (sgi + 1 < hs[mode].size() && hs[mode][sgi + 1].item0 <= it) ++sgi;
        hcoarse[mode][(size_t)k] = (int32_t)sgi;
      }
    }
  }

  // ---- program views and one device table allocation
  for (int c = 0; c < C; ++c) {
    ProgramView vf, vb, vt;
    int rc = program_device_view(&B->plans[c]->fwd, &vf);
    if (rc == TCG_OK) rc = program_device_view(&B->plans[c]->bwd, &vb);
    if (rc == TCG_OK) rc = program_device_view(B->terms[c], &vt);
    if (rc != TCG_OK) {
      delete B;
      return rc;
    }
    hc[MODE_FWD][c].prog = vf;
    hc[MODE_BWD][c].prog = vb;
    hc[MODE_MEAS][c].prog = vt;
    hc[MODE_PACC][c].prog = vt;
  }
  size_t off = 0;
  size_t o_circ[4], o_seg[4], o_coarse[4];
  for (int m = 0; m < 4; ++m) {
    o_circ[m] = off;
    off = al256(off + hc[m].size() * sizeof(BatchCirc));
    o_seg[m] = off;
    off = al256(off + hs[m].size() * sizeof(BatchSeg));
    o_coarse[m] = off;
    off = al256(off + hcoarse[m].size() * sizeof(int32_t));
  }
  const size_t o_pidx = off;
  off = al256(off + pidx.size() * sizeof(int64_t));
  const size_t o_scale = off;
  off = al256(off + scale.size() * sizeof(float));
  const size_t o_cval = off;
  off = al256(off + cval.size() * sizeof(float2));
  const size_t o_coef = off;
  off = al256(off + coef.size() * sizeof(float));
  const size_t o_soff = off;
  off = al256(off + B->state_off.size() * sizeof(int64_t));
  const size_t o_et = off;
  off = al256(off + etasks.size() * sizeof(RedTask));
  const size_t o_ei = off;
  off = al256(off + eitems.size() * sizeof(RedItem));
  const size_t o_gt = off;
  off = al256(off + gtasks.size() * sizeof(RedTask));
  const size_t o_gi = off;
  off = al256(off + gitems.size() * sizeof(RedItem));
  std::vector<char> host(off, 0);
  auto put = [&](size_t o, const void* src, size_t bytes) {
    if (bytes) std::memcpy(host.data() + o, src, bytes);
  };
  for (int m = 0; m < 4; ++m) {
    put(o_circ[m], hc[m].data(), hc[m].size() * sizeof(BatchCirc));
    put(o_seg[m], hs[m].data(), hs[m].size() * sizeof(BatchSeg));
    put(o_coarse[m], hcoarse[m].data(), hcoarse[m].size() * sizeof(int32_t));
  }
  put(o_pidx, pidx.data(), pidx.size() * sizeof(int64_t));
  put(o_scale, scale.data(), scale.size() * sizeof(float));
  put(o_cval, cval.data(), cval.size() * sizeof(float2));
  put(o_coef, coef.data(), coef.size() * sizeof(float));
  put(o_soff, B->state_off.data(), B->state_off.size() * sizeof(int64_t));
  put(o_et, etasks.data(), etasks.size() * sizeof(RedTask));
  put(o_ei, eitems.data(), eitems.size() * sizeof(RedItem));
  put(o_gt, gtasks.data(), gtasks.size() * sizeof(RedTask));
  put(o_gi, gitems.data(), gitems.size() * sizeof(RedItem));
  if (cudaMalloc(&B->dtab, off) != cudaSuccess) {
    B->dtab = nullptr;
    delete B;
    return TCG_ERR_OOM;
  }
  if (cudaMemcpy(B->dtab, host.data(), off, cudaMemcpyHostToDevice) != cudaSuccess) {
    delete B;
    return TCG_ERR_CUDA;
  }
  char* d = static_cast<char*>(B->dtab);
  for (int m = 0; m < 4; ++m) {
    B->circ[m] = reinterpret_cast<const BatchCirc*>(d + o_circ[m]);
    B->segs[m] = reinterpret_cast<const BatchSeg*>(d + o_seg[m]);
    B->coarse[m] = reinterpret_cast<const int32_t*>(d + o_coarse[m]);
  }
  B->d_pidx = reinterpret_cast<const int64_t*>(d + o_pidx);
  B->d_scale = reinterpret_cast<const float*>(d + o_scale);
  B->d_cval = reinterpret_cast<const float2*>(d + o_cval);
  B->d_coef = reinterpret_cast<const float*>(d + o_coef);
  B->d_state_off = reinterpret_cast<const int64_t*>(d + o_soff);
  B->d_etasks = reinterpret_cast<const RedTask*>(d + o_et);
  B->d_eitems = reinterpret_cast<const RedItem*>(d + o_ei);
  B->d_gtasks = reinterpret_cast<const RedTask*>(d + o_gt);
  B->d_gitems = reinterpret_cast<const RedItem*>(d + o_gi);

  // ---- scratch layout
  size_t s = 0;
  B->o_psi = s;
  s = al256(s + size_t(B->state_total) * sizeof(float2));
  B->o_mu = s;
  s = al256(s + size_t(B->state_total) * sizeof(float2));
  B->o_mats = s;
  s = al256(s + size_t(B->mat_total) * sizeof(float2));
  B->o_part = s;
  s = al256(s + size_t(std::max<int64_t>(B->part_total, 1)) * sizeof(float2));
  B->o_cnt = s;
  s = al256(s + (4 * counter_words(C) + 2) * sizeof(unsigned));
  B->scratch = s;
  *out = B;
  return TCG_OK;
}

int tcg_ubatch_destroy(tcg_ubatch* batch) {
  delete batch;
  return TCG_OK;
}

int tcg_ubatch_info(const tcg_ubatch* batch, int64_t* nparams_total, int64_t* state_entries,
                    size_t* scratch_bytes) {
  if (!batch) return TCG_ERR_INVALID_ARG;
  if (nparams_total) *nparams_total = batch->param_total;
  if (state_entries) *state_entries = batch->state_total;
  if (scratch_bytes) *scratch_bytes = batch->scratch;
  return TCG_OK;
}

int64_t tcg_ubatch_state_offset(const tcg_ubatch* batch, int32_t c) {
  if (!batch || c < 0 || c >= batch->ncirc) return -1;
  return int64_t(batch->o_psi / sizeof(float2)) + batch->state_off[c];
}

int tcg_ubatch_value_and_grad(tcg_ubatch* batch, const float* params, float* energies, float* grads,
                              void* scratch, size_t scratch_bytes, void* stream) {
  if (!batch || !energies || (batch->param_total > 0 && !params)) return TCG_ERR_INVALID_ARG;
  if (!scratch || scratch_bytes < batch->scratch) return TCG_ERR_SCRATCH;
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) return TCG_ERR_CUDA;
  if (dev != batch->device) return TCG_ERR_INVALID_ARG;
  tcg_ubatch* B = batch;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  char* S = static_cast<char*>(scratch);
  float2* psi = reinterpret_cast<float2*>(S + B->o_psi);
  float2* mu = reinterpret_cast<float2*>(S + B->o_mu);
  float2* mats = reinterpret_cast<float2*>(S + B->o_mats);
  float2* part = reinterpret_cast<float2*>(S + B->o_part);
  unsigned* cnt = reinterpret_cast<unsigned*>(S + B->o_cnt);
  const size_t cw = counter_words(B->ncirc);
  unsigned* err = cnt + 4 * cw;      // this call's wait time-out flag
  unsigned* sticky = err + 1;        // kept until tcg_ubatch_check
  const int C = B->ncirc;

  // counters of all four launches and this call's flag
  int rc = rc_of(cudaMemsetAsync(cnt, 0, (4 * cw + 1) * sizeof(unsigned), st));
  if (rc != TCG_OK) return rc;
  {
    const int64_t nm = B->mat_total;
    const int threads = 256;
    const int blocks = (int)std::min<int64_t>((nm + threads - 1) / threads, 1184);
    count_launch();
    build_mats_kernel<<<blocks, threads, 0, st>>>(params, B->d_pidx, B->d_scale, B->d_cval, nm, mats);
    rc = rc_of(cudaGetLastError());
    if (rc != TCG_OK) return rc;
  }
  rc = rc_of(cudaMemsetAsync(psi, 0, size_t(B->state_total) * sizeof(float2), st));
  if (rc != TCG_OK) return rc;
  count_launch();
  init_states_kernel<<<(C + 255) / 256, 256, 0, st>>>(psi, B->d_state_off, C);
  rc = rc_of(cudaGetLastError());
  if (rc != TCG_OK) return rc;

  auto run = [&](int mode, float2* mu_ptr, float2* part_ptr, const float* coef_ptr) -> int {
    if (B->nitems[mode] == 0) return TCG_OK;
    BatchLaunch bl;
    std::memset(&bl, 0, sizeof(bl));
    bl.circ = B->circ[mode];
    bl.segs = B->segs[mode];
    bl.coarse = B->coarse[mode];
    bl.nsegs = B->nsegs[mode];
    bl.nitems = B->nitems[mode];
    bl.psi = psi;
    bl.mu = mu_ptr;
    bl.mats = mats;
    bl.partial = part_ptr;
    bl.coef = coef_ptr;
    bl.queue = cnt + mode * cw;
    bl.done = cnt + mode * cw + 1;
    bl.err = err;
    bl.sticky = sticky;
    bl.wait_ns = B->wait_ns;
    return rc_of(launch_batch(mode, bl, B->L, B->max_slots[mode], B->lite, st));
  };
  auto reduce = [&](const RedTask* tasks, int64_t ntasks, const RedItem* items, float* out) -> int {
    if (ntasks == 0) return TCG_OK;
    const int threads = 256, wpb = threads / 32;
    count_launch();
    ragged_reduce_kernel<<<(unsigned)((ntasks + wpb - 1) / wpb), threads, 0, st>>>(part, tasks, ntasks, items, out);
    return rc_of(cudaGetLastError());
  };

  rc = run(MODE_FWD, nullptr, nullptr, nullptr);
  if (rc == TCG_OK) rc = run(MODE_MEAS, nullptr, part, nullptr);
  if (rc == TCG_OK) rc = reduce(B->d_etasks, B->n_energy_tasks, B->d_eitems, energies);
  if (rc != TCG_OK || !grads || B->param_total == 0) return rc;
  rc = rc_of(cudaMemsetAsync(mu, 0, size_t(B->state_total) * sizeof(float2), st));
  if (rc == TCG_OK) rc = run(MODE_PACC, mu, nullptr, B->d_coef);
  if (rc == TCG_OK) rc = run(MODE_BWD, mu, part, nullptr);
  if (rc == TCG_OK) rc = reduce(B->d_gtasks, B->n_grad_tasks, B->d_gitems, grads);
  return rc;
}

int tcg_ubatch_stats(const tcg_ubatch* batch, int64_t* tiles, double* alg_bytes) {
  if (!batch) return TCG_ERR_INVALID_ARG;
  const double per_amp[4] = {16.0, 32.0, 8.0, 24.0};  // indexed by MODE_*
  for (int m = 0; m < 4; ++m) {
    if (tiles) tiles[m] = batch->nitems[m];
    if (alg_bytes) alg_bytes[m] = double(batch->nitems[m]) * double(int64_t(1) << batch->L) * per_amp[m];
  }
  return TCG_OK;
}

int tcg_ubatch_set_wait_limit(tcg_ubatch* batch, uint64_t wait_ns) {
  if (!batch || wait_ns == 0) return TCG_ERR_INVALID_ARG;
  batch->wait_ns = wait_ns;
  return TCG_OK;
}

int tcg_debug_ubatch_set_need(tcg_ubatch* batch, int32_t sweep, int32_t seg, uint32_t need) {
  if (!batch || sweep < 0 || sweep > 3 || seg < 0 || seg >= batch->nsegs[sweep]) return TCG_ERR_INVALID_ARG;
  int cur = 0;
  if (cudaGetDevice(&cur) != cudaSuccess) return TCG_ERR_CUDA;
  if (cudaSetDevice(batch->device) != cudaSuccess) return TCG_ERR_CUDA;
  BatchSeg* s = const_cast<BatchSeg*>(batch->segs[sweep]) + seg;
  const cudaError_t e = cudaMemcpy(&s->need, &need, sizeof(need), cudaMemcpyHostToDevice);
  cudaSetDevice(cur);
  return e == cudaSuccess ? TCG_OK : TCG_ERR_CUDA;
}

int tcg_ubatch_check(tcg_ubatch* batch, void* scratch, void* stream) {
  if (!batch || !scratch) return TCG_ERR_INVALID_ARG;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  unsigned* err = reinterpret_cast<unsigned*>(static_cast<char*>(scratch) + batch->o_cnt) +
                  4 * counter_words(batch->ncirc) + 1;  // sticky flag
  unsigned h = 0;
  if (cudaMemcpyAsync(&h, err, sizeof(unsigned), cudaMemcpyDeviceToHost, st) != cudaSuccess) return TCG_ERR_CUDA;
  if (cudaStreamSynchronize(st) != cudaSuccess) return TCG_ERR_CUDA;
  if (cudaMemsetAsync(err, 0, sizeof(unsigned), st) != cudaSuccess) return TCG_ERR_CUDA;
  return h ? TCG_ERR_TIMEOUT : TCG_OK;
}

}  // extern "C"
