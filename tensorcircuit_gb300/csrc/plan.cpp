// plan.cpp — host planner.  Cuts an ordered gate list into HBM passes (each a
// set of L local index bits, one CTA per 2^L-amplitude tile) and each pass
// into register stages (R register bits per thread), then flattens the result
// into the device program the pass kernels read.
//
// The reference has no counterpart: it contracts a tensor network with an
// opt_einsum greedy path (tensorcircuit/cons.py:523-631).  What must agree is
// the result, i.e. gates are applied in circuit order on the big-endian state
// (tensorcircuit/basecircuit.py:120-245).
#include "plan.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

namespace tcg {

namespace {

inline int popc64(uint64_t v) { return __builtin_popcountll(v); }

// longest OP_ZRUN (its gradients are reduced as 16 float pairs in one
// transposed warp reduction by the specialised kernels)
constexpr int kZRunMax = 32;

uint64_t gate_mask(const PGate& g) {
  uint64_t m = 0;
  for (int i = 0; i < g.k; ++i) m |= 1ull << g.gbits[i];
  return m;
}

// phys-bank position a tile bit flips under the smem swizzle
// phys(j) = j ^ (((j >> 5) ^ (j >> 10)) & 31)  (see pass.cuh)
inline int bankpos(int t) { return t < 5 ? t : (t < 10 ? t - 5 : t - 10); }

struct StageDraft {
  bool smem = false;
  uint32_t rset = 0;  // tile-bit mask of register bits
  std::vector<int> ops;  // indices into the pass op drafts
  int slots = 0;
};

struct OpDraft {
  int kind;
  int k;
  int gbits[6];
  int64_t mat_off;
  int64_t grad_off;
  // term ops
  uint64_t x = 0, z = 0;
  int term = -1;
};

// Complete a stage: pad the register set, choose thread-bit order, encode ops.
int emit_stage(Program* P, DevPass& dp, const StageDraft& sd,
               const std::vector<OpDraft>& od, const int* tile_of_gbit,
               int L, int R, bool prefer_high_pad) {
  DevStage st;
  std::memset(&st, 0, sizeof(st));
  st.op_begin = (int)P->ops.size();
  st.slot_out_begin = (int)P->slot_out.size();
  if (sd.smem) {
    st.smem_stage = 1;
    st.R = 0;
    st.nthread_bits = 0;
    for (int oi : sd.ops) {
      const OpDraft& o = od[oi];
      DevOp d;
      std::memset(&d, 0, sizeof(d));
      d.kind = OP_DENSEK;
      d.k = o.k;
      for (int i = 0; i < o.k; ++i) d.p[i] = tile_of_gbit[o.gbits[i]];
      d.slot = -1;
      d.mat_off = o.mat_off;
      d.grad_off = -1;
      P->ops.push_back(d);
    }
    st.op_end = (int)P->ops.size();
    st.slot_out_end = (int)P->slot_out.size();
    P->stages.push_back(st);
    return TCG_OK;
  }
  // pad register set to exactly R bits
  uint32_t rset = sd.rset;
  auto pad_from = [&](int lo, int hi) {
    for (int t = lo; t < hi && popc64(rset) < R; ++t)
      if (!(rset >> t & 1)) rset |= 1u << t;
  };
  if (prefer_high_pad) {
    pad_from(std::min(kLo, L), L);
    pad_from(0, L);
  } else {
    pad_from(0, L);
  }
  if (popc64(rset) != R) return TCG_ERR_INVALID_ARG;
  st.R = R;
  int ri = 0;
  for (int t = 0; t < L; ++t)
    if (rset >> t & 1) st.reg_tile[ri++] = t;
  // thread bits
  std::vector<int> tb;
  for (int t = 0; t < L; ++t)
    if (!(rset >> t & 1)) tb.push_back(t);
  st.nthread_bits = (int)tb.size();
  std::vector<int> order;
  bool low_ok = (int)tb.size() >= std::min(kLo, L - R);
  for (int i = 0; i < std::min(kLo, (int)tb.size()); ++i)
    if (tb[i] != i) low_ok = false;
  if (low_ok) {
    order = tb;
    st.lanes_low = 1;
  } else {
    std::vector<int> left = tb;
    int nl = std::min(5, (int)tb.size());
    for (int i = 0; i < nl; ++i) {
      int pick = -1;
      if (i < 4)
        for (size_t c = 0; c < left.size(); ++c)
          if (bankpos(left[c]) == i) { pick = (int)c; break; }
      if (pick < 0) pick = 0;
      order.push_back(left[pick]);
      left.erase(left.begin() + pick);
    }
    for (int t : left) order.push_back(t);
    st.lanes_low = 0;
  }
  for (size_t i = 0; i < order.size(); ++i) st.thr_tile[i] = order[i];
  // register position of each tile bit
  int regpos_of_tile[32];
  for (int i = 0; i < 32; ++i) regpos_of_tile[i] = -1;
  for (int i = 0; i < R; ++i) regpos_of_tile[st.reg_tile[i]] = i;
  int slot = 0;
  for (size_t si = 0; si < sd.ops.size(); ++si) {
    const int oi = sd.ops[si];
    const OpDraft& o = od[oi];
    // a run of >= 2 consecutive Z-string rotations (no X/Y factor) becomes
    // one OP_ZRUN: they commute, so their product is one phase per amplitude.
    // In a measurement program the same op carries Z-string Pauli terms
    // (entry mat_off = term id, every entry has a slot): all their values,
    // or their accumulated coefficients, come from one Walsh-Hadamard
    // transform per thread.
    const bool zterm = (o.kind == OP_EXPECT && o.x == 0);
    if ((o.kind == TCG_GATE_PAULI_ROT && o.x == 0) || zterm) {
      // rotation runs follow the program's fusion width; term runs the maximum
      const size_t run_max = zterm ? (size_t)kZRunMax : (size_t)std::max(1, std::min(kZRunMax, P->zrun_max));
      size_t sj = si;
      while (sj < sd.ops.size() && sj - si < run_max) {
        const OpDraft& q = od[sd.ops[sj]];
        if (q.kind != o.kind || q.x != 0) break;
        ++sj;
      }
      if (sj - si >= 2) {
        DevOp d;
        std::memset(&d, 0, sizeof(d));
        d.kind = OP_ZRUN;
        d.k = (int)(sj - si);
        d.mat_off = (int64_t)P->zents.size();
        d.grad_off = -1;
        d.slot = -1;
        for (size_t t = si; t < sj; ++t) {
          const OpDraft& q = od[sd.ops[t]];
          ZEnt z;
          std::memset(&z, 0, sizeof(z));
          z.zmask = (uint32_t)q.z;
          int zr = 0;
          for (int b = 0; b < 64; ++b)
            if (q.z >> b & 1) {
              const int tb = tile_of_gbit[b];
              const int rp = tb >= 0 ? regpos_of_tile[tb] : -1;
              if (rp >= 0) zr |= 1 << rp;
            }
          z.zreg = zr;
          z.mat_off = zterm ? q.term : q.mat_off;
          z.grad_off = zterm ? q.term : q.grad_off;
          z.slot = -1;
          if (z.grad_off >= 0) {
            if (d.slot < 0) d.slot = slot;
            z.slot = slot;
            SlotOut so;
            so.slot = slot;
            so.pad = 0;
            so.out_off = z.grad_off;
            P->slot_out.push_back(so);
            slot += 1;
          }
          P->zents.push_back(z);
        }
        P->ops.push_back(d);
        si = sj - 1;
        continue;
      }
    }
    DevOp d;
    std::memset(&d, 0, sizeof(d));
    d.slot = -1;
    d.grad_off = -1;
    d.mat_off = o.mat_off;
    d.k = o.k;
    if (o.kind == OP_EXPECT) {
      d.kind = OP_EXPECT;
      int xr = 0;
      for (int b = 0; b < 64; ++b)
        if (o.x >> b & 1) {
          int rp = regpos_of_tile[tile_of_gbit[b]];
          if (rp < 0) return TCG_ERR_INVALID_ARG;
          xr |= 1 << rp;
        }
      d.xreg = xr;
      d.zmask = (uint32_t)o.z;
      d.nY = popc64(o.x & o.z);
      d.mat_off = o.term;
      d.slot = slot;
      SlotOut so;
      so.slot = slot;
      so.pad = 0;
      so.out_off = o.term;
      P->slot_out.push_back(so);
      slot += 1;
    } else if (o.kind == TCG_GATE_PAULI_ROT) {
      d.kind = OP_PROT;
      int xr = 0;
      for (int b = 0; b < 64; ++b)
        if (o.x >> b & 1) {
          int rp = regpos_of_tile[tile_of_gbit[b]];
          if (rp < 0) return TCG_ERR_INVALID_ARG;
          xr |= 1 << rp;
        }
      d.xreg = xr;
      d.zmask = (uint32_t)o.z;
      d.nY = popc64(o.x & o.z);
      for (int i = 0; i < o.k; ++i) d.p[i] = o.gbits[i];
      if (o.grad_off >= 0) {
        d.grad_off = o.grad_off;
        d.slot = slot;
        SlotOut so;
        so.slot = slot;
        so.pad = 0;
        so.out_off = o.grad_off;
        P->slot_out.push_back(so);
        slot += 1;
      }
    } else if (o.kind == TCG_GATE_DIAG) {
      d.kind = OP_DIAG;
      for (int i = 0; i < o.k; ++i) d.p[i] = o.gbits[i];
      if (o.grad_off >= 0) {
        d.grad_off = o.grad_off;
        d.slot = slot;
        int E = 1 << o.k;
        for (int e = 0; e < E; ++e) {
          SlotOut so;
          so.slot = slot + e;
          so.pad = 0;
          so.out_off = o.grad_off + e;
          P->slot_out.push_back(so);
        }
        slot += E;
      }
    } else {  // dense on registers
      if (o.k == 1) d.kind = OP_DENSE1;
      else if (o.k == 2) d.kind = OP_DENSE2;
      else return TCG_ERR_INVALID_ARG;
      for (int i = 0; i < o.k; ++i) {
        int rp = regpos_of_tile[tile_of_gbit[o.gbits[i]]];
        if (rp < 0) return TCG_ERR_INVALID_ARG;
        d.p[i] = rp;
      }
      if (o.grad_off >= 0) {
        d.grad_off = o.grad_off;
        d.slot = slot;
        int E = 1 << (2 * o.k);
        for (int e = 0; e < E; ++e) {
          SlotOut so;
          so.slot = slot + e;
          so.pad = 0;
          so.out_off = o.grad_off + e;
          P->slot_out.push_back(so);
        }
        slot += E;
      }
    }
    P->ops.push_back(d);
  }
  st.nslots = slot;
  P->max_slots = std::max(P->max_slots, slot);
  st.op_end = (int)P->ops.size();
  st.slot_out_end = (int)P->slot_out.size();
  P->stages.push_back(st);
  return TCG_OK;
}

// Common tail: build DevPass for local set S (global-bit mask) and op drafts,
// splitting the pass ops into stages.
int emit_pass(Program* P, int n, int L, int R, uint64_t S,
              const std::vector<OpDraft>& od, int max_slots) {
  DevPass dp;
  std::memset(&dp, 0, sizeof(dp));
  dp.L = L;
  int tile_of_gbit[64];
  for (int i = 0; i < 64; ++i) tile_of_gbit[i] = -1;
  int ti = 0, ni = 0;
  for (int b = 0; b < n; ++b) {
    if (S >> b & 1) {
      dp.lbits[ti] = b;
      tile_of_gbit[b] = ti++;
    } else {
      dp.nlbits[ni++] = b;
    }
  }
  if (ti != L) return TCG_ERR_INVALID_ARG;
  dp.nnonlocal = ni;
  int lo = std::min(kLo, L);
  dp.runs_off = (int)P->runs.size();
  int nruns = 1 << (L - lo);
  for (int r = 0; r < nruns; ++r) {
    uint32_t off = 0;
    for (int i = lo; i < L; ++i)
      if (r >> (i - lo) & 1) off |= 1u << dp.lbits[i];
    P->runs.push_back(off);
  }
  dp.stage_begin = (int)P->stages.size();
  // stage drafting
  std::vector<StageDraft> drafts;
  StageDraft cur;
  auto close = [&]() {
    if (!cur.ops.empty()) drafts.push_back(cur);
    cur = StageDraft();
  };
  for (size_t oi = 0; oi < od.size(); ++oi) {
    const OpDraft& o = od[oi];
    if (o.kind == OP_EXPECT) {
      uint32_t tb = 0;
      for (int b = 0; b < n; ++b)
        if (o.x >> b & 1) tb |= 1u << tile_of_gbit[b];
      uint32_t need = tb & ~cur.rset;
      if (popc64(cur.rset | need) <= R && cur.slots + 1 <= max_slots) {
        cur.rset |= need;
      } else {
        close();
        cur.rset = tb;
      }
      cur.ops.push_back((int)oi);
      cur.slots += 1;
      continue;
    }
    if (o.kind == TCG_GATE_PAULI_ROT) {
      // X/Y bits must be register bits; Z bits may be anywhere
      const int E1 = o.grad_off >= 0 ? 1 : 0;
      uint32_t tb = 0;
      for (int b = 0; b < n; ++b)
        if (o.x >> b & 1) tb |= 1u << tile_of_gbit[b];
      if (popc64(tb) > R) return TCG_ERR_UNSUPPORTED;
      if (cur.smem) close();
      const uint32_t need = tb & ~cur.rset;
      if (popc64(cur.rset | need) <= R && cur.slots + E1 <= max_slots) {
        cur.rset |= need;
      } else {
        close();
        cur.rset = tb;
      }
      cur.ops.push_back((int)oi);
      cur.slots += E1;
      continue;
    }
    int E = 0;
    if (o.grad_off >= 0) E = (o.kind == TCG_GATE_DIAG) ? (1 << o.k) : (1 << (2 * o.k));
    if (o.kind == TCG_GATE_DIAG) {
      if (o.grad_off >= 0 && o.k > 2) return TCG_ERR_UNSUPPORTED;
      if (cur.smem || cur.slots + E > max_slots) close();
      cur.ops.push_back((int)oi);
      cur.slots += E;
      continue;
    }
    // dense
    if (o.k > 2 || o.k > R) {
      if (o.grad_off >= 0) return TCG_ERR_UNSUPPORTED;
      if (!cur.smem) close();
      cur.smem = true;
      cur.ops.push_back((int)oi);
      continue;
    }
    if (cur.smem) close();
    uint32_t tb = 0;
    for (int i = 0; i < o.k; ++i) tb |= 1u << tile_of_gbit[o.gbits[i]];
    uint32_t need = tb & ~cur.rset;
    if (popc64(cur.rset | need) <= R && cur.slots + E <= max_slots) {
      cur.rset |= need;
    } else {
      close();
      cur.rset = tb;
    }
    cur.ops.push_back((int)oi);
    cur.slots += E;
  }
  close();
  if (drafts.empty()) {  // a pass with no ops still needs a layout
    StageDraft e;
    drafts.push_back(e);
  }
  for (size_t s = 0; s < drafts.size(); ++s) {
    bool edge = (s == 0) || (s + 1 == drafts.size());
    int rc = emit_stage(P, dp, drafts[s], od, tile_of_gbit, L, R, edge || true);
    if (rc != TCG_OK) return rc;
  }
  dp.stage_end = (int)P->stages.size();
  P->passes.push_back(dp);
  return TCG_OK;
}

void finish_entries(Program* P) {
  std::vector<int64_t> e;
  for (const SlotOut& so : P->slot_out) e.push_back(so.out_off);
  std::sort(e.begin(), e.end());
  e.erase(std::unique(e.begin(), e.end()), e.end());
  P->entries = e;
}

}  // namespace

int build_gate_program(int n, const std::vector<PGate>& gates, int L, int R,
                       bool reverse, int max_slots, Program* out) {
  Program& P = *out;
  P.n = n;
  L = std::min(L, n);
  P.L = L;
  P.R = R;
  if (R > L) return TCG_ERR_INVALID_ARG;
  int lo = std::min(kLo, L);
  std::vector<int> rem;
  for (size_t i = 0; i < gates.size(); ++i) rem.push_back((int)i);
  if (reverse) std::reverse(rem.begin(), rem.end());
  int64_t nout = 0;
  for (const PGate& g : gates)
    if (g.grad_off >= 0) {
      int64_t E = (g.kind == TCG_GATE_PAULI_ROT) ? 1 : (g.kind == TCG_GATE_DIAG) ? (1 << g.k) : (1 << (2 * g.k));
      nout = std::max(nout, g.grad_off + E);
    }
  P.nout = nout;
  if (rem.empty()) {
    // identity circuit: one pass with no ops keeps the launch path uniform
    uint64_t S = 0;
    for (int b = 0; b < L; ++b) S |= 1ull << b;
    std::vector<OpDraft> none;
    P.pass_gates.emplace_back();
    return emit_pass(&P, n, L, R, S, none, max_slots);
  }
  auto need_of = [&](const PGate& g) -> uint64_t {
    return (g.kind == TCG_GATE_DENSE) ? gate_mask(g) : (g.kind == TCG_GATE_PAULI_ROT) ? g.xmask : 0;
  };
  // gates of `rem` a pass with the fixed local set S can run, in order
  // (a gate that cannot run blocks every later gate on its qubits)
  auto take_fixed = [&](uint64_t S, std::vector<int>* taken, std::vector<int>* left) {
    uint64_t blocked = 0;
    for (int gi : rem) {
      const PGate& g = gates[gi];
      const uint64_t bits = gate_mask(g);
      if ((bits & blocked) || (need_of(g) & ~S)) {
        blocked |= bits;
        if (left) left->push_back(gi);
      } else if (taken) {
        taken->push_back(gi);
      }
    }
  };
  auto count_fixed = [&](uint64_t S) -> int {
    uint64_t blocked = 0;
    int c = 0;
    for (int gi : rem) {
      const PGate& g = gates[gi];
      const uint64_t bits = gate_mask(g);
      if ((bits & blocked) || (need_of(g) & ~S)) blocked |= bits;
      else ++c;
    }
    return c;
  };
  // window candidates: the low bits plus L - lo free bits made of one or two
  // runs of consecutive index bits (a brick wall's light cone is a window)
  std::vector<uint64_t> windows;
  {
    const int w = L - lo;
    const uint64_t base = (lo >= 64) ? ~0ull : ((1ull << lo) - 1);
    auto run = [](int a, int len) -> uint64_t {
      uint64_t m = 0;
      for (int b = a; b < a + len; ++b) m |= 1ull << b;
      return m;
    };
    if (n > L && w > 0) {
      for (int a = lo; a + w <= n; ++a) windows.push_back(base | run(a, w));
      for (int w1 = 1; w1 < w; ++w1)
        for (int a = lo; a + w1 <= n; ++a)
          for (int b2 = a + w1 + 1; b2 + (w - w1) <= n; ++b2)
            windows.push_back(base | run(a, w1) | run(b2, w - w1));
    }
  }
  while (!rem.empty()) {
    uint64_t S = (lo >= 64) ? ~0ull : ((1ull << lo) - 1);
    uint64_t blocked = 0;
    std::vector<int> taken, left;
    for (int gi : rem) {
      const PGate& g = gates[gi];
      uint64_t bits = gate_mask(g);
      if (bits & blocked) {
        blocked |= bits;
        left.push_back(gi);
        continue;
      }
      uint64_t need = need_of(g) & ~S;
      if (popc64(S | need) <= L) {
        S |= need;
        taken.push_back(gi);
      } else {
        blocked |= bits;
        left.push_back(gi);
      }
    }
    if (taken.empty()) return TCG_ERR_INVALID_ARG;  // cannot happen: L >= lo + 6
    // a fixed window that runs more gates than the in-order greedy choice wins
    {
      int best = (int)taken.size();
      uint64_t bestS = 0;
      // bounded planning work: two-run windows only while they stay cheap
      const int single = std::max(0, n - (L - lo) - lo + 1);
      const size_t nw = (windows.size() * rem.size() > 2000000) ? std::min<size_t>(single, windows.size())
                                                                  : windows.size();
      for (size_t wi = 0; wi < nw; ++wi) {
        const uint64_t Wm = windows[wi];
        const int c = count_fixed(Wm);
        if (c > best) {
          best = c;
          bestS = Wm;
        }
      }
      if (bestS) {
        S = bestS;
        taken.clear();
        left.clear();
        take_fixed(S, &taken, &left);
      }
    }
    // pad S to L bits: prefer bits the next gates need
    for (int gi : left) {
      if (popc64(S) >= L) break;
      const PGate& g = gates[gi];
      if (g.kind != TCG_GATE_DENSE) continue;
      uint64_t need = gate_mask(g) & ~S;
      if (popc64(S | need) <= L) S |= need;
    }
    for (int b = 0; b < n && popc64(S) < L; ++b) S |= 1ull << b;
    // Z-string rotations commute with every gate on other qubits and with
    // all diagonal gates: move each one back to the nearest earlier Z-string
    // rotation it can reach, so that runs (one phase op each) grow long
    {
      auto is_z = [&](const PGate& g) { return g.kind == TCG_GATE_PAULI_ROT && g.xmask == 0; };
      std::vector<int> ord;
      ord.reserve(taken.size());
      for (int gi : taken) {
        const PGate& g = gates[gi];
        if (!is_z(g)) {
          ord.push_back(gi);
          continue;
        }
        const uint64_t m = gate_mask(g);
        int at = -1;
        for (int j = (int)ord.size() - 1; j >= 0; --j) {
          const PGate& h = gates[ord[j]];
          if (is_z(h)) {
            at = j + 1;
            break;
          }
          if (h.kind != TCG_GATE_DIAG && (gate_mask(h) & m)) break;  // does not commute
        }
        if (at < 0) ord.push_back(gi);
        else ord.insert(ord.begin() + at, gi);
      }
      taken.swap(ord);
    }
    std::vector<OpDraft> od;
    for (int gi : taken) {
      const PGate& g = gates[gi];
      OpDraft o;
      o.kind = g.kind;
      o.k = g.k;
      for (int i = 0; i < 6; ++i) o.gbits[i] = (i < g.k) ? g.gbits[i] : 0;
      o.mat_off = g.mat_off;
      o.grad_off = g.grad_off;
      o.x = g.xmask;
      o.z = g.zmask;
      od.push_back(o);
    }
    P.pass_gates.push_back(taken);
    int rc = emit_pass(&P, n, L, R, S, od, max_slots);
    if (rc != TCG_OK) return rc;
    rem.swap(left);
  }
  finish_entries(&P);
  return TCG_OK;
}

namespace {

// Per-pass cost model (microseconds per pass over 2^26 amplitudes, fitted to
// per-launch GB300 timings of brick-wall passes on both paths): a
// tensor-core pass costs a fixed part (tile load, split, store) plus a
// part per fused block; a register-path pass a fixed part plus a part per
// dense gate of two or more qubits.
constexpr double kTcBaseUs = 280.0;
constexpr double kTcPerBlockUs = 135.0;
constexpr double kRegBaseUs = 110.0;
constexpr double kRegPerDense2Us = 47.0;

// Fuse the gates of one pass (tile-bit masks tb, in application order) into
// blocks of at most kTcBlockBits tile bits.  A gate may join the open block
// once every earlier gate it shares a bit with is placed or in the block;
// gates that fit the block's bits are absorbed first, otherwise the ready
// gate that widens the block least joins.  Returns the blocks (gate indices
// in application order) and their bit sets.
void fuse_pass_gates(const std::vector<uint32_t>& tb, std::vector<std::vector<int>>* blocks,
                     std::vector<uint32_t>* sets) {
  const int m = (int)tb.size();
  std::vector<std::vector<int>> preds(m);
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < i; ++j)
      if (tb[j] & tb[i]) preds[i].push_back(j);
  std::vector<char> placed(m, 0), inb(m, 0);
  int nplaced = 0;
  while (nplaced < m) {
    uint32_t S = 0;
    std::vector<int> cur;
    std::fill(inb.begin(), inb.end(), 0);
    auto ready = [&](int i) {
      if (placed[i] || inb[i]) return false;
      for (int j : preds[i])
        if (!placed[j] && !inb[j]) return false;
      return true;
    };
    for (;;) {
      bool changed = false;
      for (int i = 0; i < m; ++i)
        if (ready(i) && (tb[i] & ~S) == 0) {
          inb[i] = 1;
          cur.push_back(i);
          changed = true;
        }
      if (changed) continue;
      int best = -1, bc = kTcBlockBits + 1;
      for (int i = 0; i < m; ++i)
        if (ready(i)) {
          const int c = popc64(S | tb[i]);
          if (c <= kTcBlockBits && c < bc) {
            bc = c;
            best = i;
          }
        }
      if (best < 0) break;
      inb[best] = 1;
      cur.push_back(best);
      S |= tb[best];
    }
    std::sort(cur.begin(), cur.end());
    for (int i : cur) placed[i] = 1;
    nplaced += (int)cur.size();
    blocks->push_back(cur);
    sets->push_back(S);
  }
}

// Byte-address bit, in a block's fp16 operand planes (K-major canonical
// layout: element (row n, k) at (k & 7) * 2 + (n & 7) * 16 + (k >> 3) * 1024
// + (n >> 3) * 128), of block-index bit i and of column bit i.
constexpr int kKAddrBit[6] = {1, 2, 3, 10, 11, 12};
constexpr int kNAddrBit[6] = {4, 5, 6, 7, 8, 9};

uint32_t plane_bit(const TcBlock& b, int t) {
  for (int i = 0; i < kTcBlockBits; ++i) {
    if (b.bbits[i] == t) return 1u << kKAddrBit[i];
    if (b.cbits[i] == t) return 1u << kNAddrBit[i];
  }
  return 0;
}

uint32_t plane_off(const TcBlock& b, uint32_t tile_off) {
  uint32_t o = 0;
  for (int t = 0; t < kTcTileBits; ++t)
    if (tile_off >> t & 1u) o ^= plane_bit(b, t);
  return o;
}

uint32_t expand6(uint32_t v, const int32_t* bits) {
  uint32_t o = 0;
  for (int i = 0; i < 6; ++i) o |= (v >> i & 1u) << bits[i];
  return o;
}

inline uint32_t staging_swz(uint32_t t) { return t ^ (((t >> 5) ^ (t >> 10)) & 31u); }

// Bit orders of the blocks of one pass (full[b] = the block's 6 tile bits).
// The epilogue of block b writes, per lane, output rows that differ in
// block bits 0..3 of b; those stores avoid bank conflicts when the four bits
// are, in block b+1's planes, K bits 1, 2 and column bits 0, 1 (byte-address
// bits 2..5), so block b+1 takes them there where it can.  Two outputs that
// differ only in a column bit of b which is block b+1's K bit 0 share one
// 32-bit word (the pairing bit, kept at a column position <= 3).  The first
// block orders tile bits 0..5 the same way for the load of the tile.
void order_tc_blocks(const std::vector<uint32_t>& full, std::vector<TcBlock>* out) {
  const int m = (int)full.size();
  std::vector<int> prev4;
  int pair_in = -1;
  for (int b = 0; b < m; ++b) {
    const uint32_t B = full[b], Cs = ((1u << kTcTileBits) - 1) & ~B;
    int bb[6], cb[6];
    for (int i = 0; i < 6; ++i) bb[i] = cb[i] = -1;
    auto has = [&](const int* v, int t) {
      for (int i = 0; i < 6; ++i)
        if (v[i] == t) return true;
      return false;
    };
    std::vector<int> want;
    int nslots = 2;
    if (b == 0) {
      if (B & 1u) bb[0] = 0;
      want = {1, 2, 3, 4, 5};
      nslots = 3;
    } else {
      if (pair_in >= 0) bb[0] = pair_in;
      want = prev4;
    }
    int ki = 0, ni = 0;
    for (int t : want) {
      if (t < 0 || has(bb, t) || has(cb, t)) continue;
      if ((B >> t & 1u) && ki < 2) bb[1 + ki++] = t;
      else if ((Cs >> t & 1u) && ni < nslots) cb[ni++] = t;
    }
    int pair_out = -1;
    if (b + 1 < m) {
      const uint32_t cand = Cs & full[b + 1];
      for (int pos = 0; pos < 4 && pair_out < 0; ++pos)
        if (cb[pos] >= 0 && (cand >> cb[pos] & 1u)) pair_out = cb[pos];
      for (int t = 0; t < kTcTileBits && pair_out < 0; ++t)
        if ((cand >> t & 1u) && !has(cb, t))
          for (int pos = 0; pos < 4; ++pos)
            if (cb[pos] < 0) {
              cb[pos] = t;
              pair_out = t;
              break;
            }
    }
    for (int t = 0; t < kTcTileBits; ++t) {
      int* v = (B >> t & 1u) ? bb : cb;
      if (has(v, t)) continue;
      for (int i = 0; i < 6; ++i)
        if (v[i] < 0) {
          v[i] = t;
          break;
        }
    }
    TcBlock& tb = (*out)[b];
    std::memset(&tb, 0, sizeof(tb));
    for (int i = 0; i < 6; ++i) {
      tb.bbits[i] = bb[i];
      tb.cbits[i] = cb[i];
    }
    prev4 = {bb[0], bb[1], bb[2], bb[3]};
    pair_in = pair_out;
  }
}

// Epilogue address tables of every block and the load table of the pass.
void tc_tables(std::vector<TcBlock>* tbs, TcPassDesc* pd) {
  const int m = (int)tbs->size();
  for (int b = 0; b < m; ++b) {
    TcBlock& t = (*tbs)[b];
    t.pairbit = -1;
    for (uint32_t v = 0; v < 64; ++v) {
      const uint32_t tr = expand6(v, t.bbits), tc = expand6(v, t.cbits);
      if (b + 1 < m) {
        t.raddr[v] = plane_off((*tbs)[b + 1], tr);
        t.caddr[v] = plane_off((*tbs)[b + 1], tc);
      } else {
        t.raddr[v] = staging_swz(tr) * 4u;
        t.caddr[v] = staging_swz(tc) * 4u;
      }
    }
    if (b + 1 < m)
      for (int pos = 0; pos < 4; ++pos)
        if (plane_bit((*tbs)[b + 1], t.cbits[pos]) == 2u) t.pairbit = pos;
  }
  for (int t = 0; t < kTcTileBits; ++t) pd->ldaddr[t] = plane_bit((*tbs)[0], t);
  pd->ldpair = pd->ldaddr[0] == 2u ? 1 : 0;
}

}  // namespace

void plan_tensor_passes(Program* P, const std::vector<PGate>& gates) {
  P->tc_of_pass.assign(P->passes.size(), -1);
  if (P->L != kTcTileBits) return;
  for (size_t ps = 0; ps < P->passes.size() && ps < P->pass_gates.size(); ++ps) {
    const DevPass& dp = P->passes[ps];
    const std::vector<int>& gl = P->pass_gates[ps];
    if (gl.empty()) continue;
    int tile_of_gbit[64];
    for (int i = 0; i < 64; ++i) tile_of_gbit[i] = -1;
    for (int i = 0; i < dp.L; ++i) tile_of_gbit[dp.lbits[i]] = i;
    bool ok = true;
    int ndense2 = 0;
    std::vector<uint32_t> tb(gl.size());
    for (size_t i = 0; i < gl.size() && ok; ++i) {
      const PGate& g = gates[gl[i]];
      if (g.grad_off >= 0) ok = false;
      uint32_t t = 0;
      for (int q = 0; q < g.k; ++q) {
        const int tt = tile_of_gbit[g.gbits[q]];
        if (tt < 0) ok = false;
        else t |= 1u << tt;
      }
      tb[i] = t;
      if (g.kind == TCG_GATE_DENSE && g.k >= 2) ++ndense2;
    }
    if (!ok) continue;
    std::vector<std::vector<int>> blocks;
    std::vector<uint32_t> sets;
    fuse_pass_gates(tb, &blocks, &sets);
    TcPassDesc pd;
    std::memset(&pd, 0, sizeof(pd));
    pd.pass = (int)ps;
    pd.block_begin = (int)P->tc_blocks.size();
    const int m = (int)blocks.size();
    // pad every block to 6 tile bits (identity on the extra bits)
    std::vector<uint32_t> full(m);
    for (int b = 0; b < m; ++b) {
      uint32_t Sx = sets[b];
      for (int t = 0; t < kTcTileBits && popc64(Sx) < kTcBlockBits; ++t) Sx |= 1u << t;
      full[b] = Sx;
    }
    std::vector<TcBlock> tbs(m);
    order_tc_blocks(full, &tbs);
    for (int b = 0; b < m; ++b) {
      TcBlock& tbk = tbs[b];
      int blockpos_of_tile[32];
      for (int i = 0; i < 32; ++i) blockpos_of_tile[i] = -1;
      for (int i = 0; i < kTcBlockBits; ++i) blockpos_of_tile[tbk.bbits[i]] = i;
      tbk.gate_begin = (int)P->tc_gates.size();
      for (int gi : blocks[b]) {
        const PGate& g = gates[gl[gi]];
        TcGate G;
        std::memset(&G, 0, sizeof(G));
        G.kind = g.kind;
        G.k = g.k;
        for (int q = 0; q < g.k; ++q) G.pos[q] = blockpos_of_tile[tile_of_gbit[g.gbits[q]]];
        if (g.kind == TCG_GATE_PAULI_ROT) {
          for (int bit = 0; bit < 64; ++bit) {
            if (g.xmask >> bit & 1) G.xmask |= 1 << blockpos_of_tile[tile_of_gbit[bit]];
            if (g.zmask >> bit & 1) G.zmask |= 1 << blockpos_of_tile[tile_of_gbit[bit]];
          }
          G.nY = popc64(g.xmask & g.zmask);
        }
        G.mat_off = g.mat_off;
        P->tc_gates.push_back(G);
      }
      tbk.gate_end = (int)P->tc_gates.size();
      tbk.slot = P->tc_slots++;
    }
    tc_tables(&tbs, &pd);
    for (const TcBlock& t : tbs) P->tc_blocks.push_back(t);
    pd.block_end = (int)P->tc_blocks.size();
    P->tc_of_pass[ps] = (int)P->tc_passes.size();
    P->tc_passes.push_back(pd);
    // the tensor path runs where the cost model estimates it faster
    const double t_tc = kTcBaseUs + kTcPerBlockUs * (double)blocks.size();
    const double t_reg = kRegBaseUs + kRegPerDense2Us * (double)ndense2;
    P->tc_prefer.push_back(t_tc < t_reg ? 1 : 0);
  }
}

int build_term_program(int n, const std::vector<tcg_pauli>& terms, int L, int R,
                       int max_slots, Program* out, std::vector<int>* direct) {
  Program& P = *out;
  P.n = n;
  L = std::min(L, n);
  P.L = L;
  P.R = R;
  P.nout = (int64_t)terms.size();
  int lo = std::min(kLo, L);
  std::vector<int> rem;
  for (size_t t = 0; t < terms.size(); ++t) {
    if (popc64(terms[t].xmask) > 2) direct->push_back((int)t);  // register path: <= 2 X/Y bits
    else rem.push_back((int)t);
  }
  // group equal / overlapping X masks next to each other
  std::stable_sort(rem.begin(), rem.end(), [&](int a, int b) {
    return terms[a].xmask < terms[b].xmask;
  });
  while (!rem.empty()) {
    uint64_t S = (1ull << lo) - 1;
    std::vector<int> taken, left;
    for (int t : rem) {
      uint64_t need = terms[t].xmask & ~S;
      if (popc64(S | need) <= L) {
        S |= need;
        taken.push_back(t);
      } else {
        left.push_back(t);
      }
    }
    for (int b = 0; b < n && popc64(S) < L; ++b) S |= 1ull << b;
    std::vector<OpDraft> od;
    for (int t : taken) {
      OpDraft o;
      std::memset(&o, 0, sizeof(o));
      o.kind = OP_EXPECT;
      o.k = popc64(terms[t].xmask);
      o.x = terms[t].xmask;
      o.z = terms[t].zmask;
      o.term = t;
      o.grad_off = -1;
      od.push_back(o);
    }
    int rc = emit_pass(&P, n, L, R, S, od, max_slots);
    if (rc != TCG_OK) return rc;
    rem.swap(left);
  }
  finish_entries(&P);
  return TCG_OK;
}

int program_device_view(Program* p, ProgramView* view) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return TCG_ERR_CUDA;
  std::lock_guard<std::mutex> lk(p->mu);
  auto it = p->dev.find(dev);
  if (it != p->dev.end()) {
    *view = it->second.view;
    return TCG_OK;
  }
  auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
  size_t o_pass = 0;
  size_t o_stage = al(o_pass + p->passes.size() * sizeof(DevPass));
  size_t o_op = al(o_stage + p->stages.size() * sizeof(DevStage));
  size_t o_so = al(o_op + p->ops.size() * sizeof(DevOp));
  size_t o_runs = al(o_so + p->slot_out.size() * sizeof(SlotOut));
  size_t o_ent = al(o_runs + p->runs.size() * sizeof(uint32_t));
  size_t o_z = al(o_ent + p->entries.size() * sizeof(int64_t));
  size_t o_tcp = al(o_z + p->zents.size() * sizeof(ZEnt));
  size_t o_tcb = al(o_tcp + p->tc_passes.size() * sizeof(TcPassDesc));
  size_t o_tcg = al(o_tcb + p->tc_blocks.size() * sizeof(TcBlock));
  size_t o_err = al(o_tcg + p->tc_gates.size() * sizeof(TcGate));
  size_t total = o_err + 256;
  std::vector<char> host(total, 0);
  if (!p->passes.empty()) std::memcpy(host.data() + o_pass, p->passes.data(), p->passes.size() * sizeof(DevPass));
  if (!p->stages.empty()) std::memcpy(host.data() + o_stage, p->stages.data(), p->stages.size() * sizeof(DevStage));
  if (!p->ops.empty()) std::memcpy(host.data() + o_op, p->ops.data(), p->ops.size() * sizeof(DevOp));
  if (!p->slot_out.empty()) std::memcpy(host.data() + o_so, p->slot_out.data(), p->slot_out.size() * sizeof(SlotOut));
  if (!p->runs.empty()) std::memcpy(host.data() + o_runs, p->runs.data(), p->runs.size() * sizeof(uint32_t));
  if (!p->entries.empty()) std::memcpy(host.data() + o_ent, p->entries.data(), p->entries.size() * sizeof(int64_t));
  if (!p->zents.empty()) std::memcpy(host.data() + o_z, p->zents.data(), p->zents.size() * sizeof(ZEnt));
  if (!p->tc_passes.empty())
    std::memcpy(host.data() + o_tcp, p->tc_passes.data(), p->tc_passes.size() * sizeof(TcPassDesc));
  if (!p->tc_blocks.empty())
    std::memcpy(host.data() + o_tcb, p->tc_blocks.data(), p->tc_blocks.size() * sizeof(TcBlock));
  if (!p->tc_gates.empty()) std::memcpy(host.data() + o_tcg, p->tc_gates.data(), p->tc_gates.size() * sizeof(TcGate));
  void* d = nullptr;
  if (cudaMalloc(&d, total) != cudaSuccess) return TCG_ERR_OOM;
  if (cudaMemcpy(d, host.data(), total, cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaFree(d);
    return TCG_ERR_CUDA;
  }
  Program::DevCopy c;
  c.base = d;
  char* b = (char*)d;
  c.view.passes = (const DevPass*)(b + o_pass);
  c.view.stages = (const DevStage*)(b + o_stage);
  c.view.ops = (const DevOp*)(b + o_op);
  c.view.slot_out = (const SlotOut*)(b + o_so);
  c.view.runs = (const uint32_t*)(b + o_runs);
  c.view.entries = (const int64_t*)(b + o_ent);
  c.view.nentries = (int64_t)p->entries.size();
  c.view.zents = (const ZEnt*)(b + o_z);
  c.view.tc_passes = (const TcPassDesc*)(b + o_tcp);
  c.view.tc_blocks = (const TcBlock*)(b + o_tcb);
  c.view.tc_gates = (const TcGate*)(b + o_tcg);
  c.view.tc_err = (unsigned int*)(b + o_err);
  p->dev[dev] = c;
  *view = c.view;
  return TCG_OK;
}

void program_free(Program* p) {
  std::lock_guard<std::mutex> lk(p->mu);
  int cur = 0;
  cudaGetDevice(&cur);
  for (auto& kv : p->dev) {
    cudaSetDevice(kv.first);
    cudaFree(kv.second.base);
  }
  cudaSetDevice(cur);
  p->dev.clear();
}

}  // namespace tcg
