// jit.cpp — the plan specialiser.
//
// A planned program (passes / stages / ops, see engine.h) is translated into
// one straight-line CUDA kernel per pass: register positions, tile layouts,
// swizzled shared-memory offsets, global offsets and Pauli sign masks become
// literals, diagonal gates whose sub-index bits are all outside the
// registers collapse into one per-thread factor, and no op descriptor is read
// at run time.  The kernels call the helpers of jit_device.cuh and are
// compiled for sm_103a with NVRTC (loaded with dlopen, so the library has no
// link-time dependency on it), cached as cubins on disk, and loaded with
// cudaLibraryLoadData.  When NVRTC is missing or a compile fails the caller
// keeps the generic pass kernels of pass.cuh.
#include "jit.h"

#include <dlfcn.h>
#include <nvrtc.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <sys/stat.h>
#include <unistd.h>

#include "plan.h"

namespace tcg {

namespace {

const char kJitDevice[] =
#include "jit_device.inc"
    ;

inline uint32_t host_swz(uint32_t j) { return j ^ (((j >> 5) ^ (j >> 10)) & 31u); }

// tcgkF_<pass> forward, tcgkB_ adjoint, tcgkM_ measure, tcgkP_ Pauli accumulate
std::string kernel_name(int mode, int pass) {
  const char m = mode == MODE_FWD ? 'F' : mode == MODE_BWD ? 'B' : mode == MODE_MEAS ? 'M' : 'P';
  return std::string("tcgk") + m + "_" + std::to_string(pass);
}

struct Layout {
  int R = 0, nthr = 0;
  int reg_tile[6] = {0};
  int thr_tile[16] = {0};
  bool lanes_low = false;
};

Layout layout_of(const DevStage& S) {
  Layout l;
  l.R = S.R;
  l.nthr = S.nthread_bits;
  for (int i = 0; i < 6; ++i) l.reg_tile[i] = S.reg_tile[i];
  for (int i = 0; i < 16; ++i) l.thr_tile[i] = S.thr_tile[i];
  l.lanes_low = S.lanes_low != 0;
  return l;
}

bool same_layout(const Layout& a, const Layout& b) {
  if (a.R != b.R || a.nthr != b.nthr) return false;
  for (int i = 0; i < a.R; ++i)
    if (a.reg_tile[i] != b.reg_tile[i]) return false;
  for (int i = 0; i < a.nthr; ++i)
    if (a.thr_tile[i] != b.thr_tile[i]) return false;
  return true;
}
// Host mirror of the op record the generated kernels read from constant
// memory (one per op; the kind and compile-time register positions live in
// the signature `sig`, the rest are run-time operands).
struct OpRec {
  long long off;  // matrix offset (gates) or term / coefficient index (Pauli)
  int sig;        // index of the compiled body
  int slot;       // first accumulator slot, -1 = none
  int g0, g1;     // global bits of a diagonal op's sub-index (run-time part)
  unsigned zm;    // Pauli Z/Y mask (global bits)
  int ny;         // number of Y factors
  int zr;         // register-position mask of the Z/Y bits
  int pad;
};

// How a register stage's ops are emitted: 0 = a loop over constant op
// records with a switch on the shared op bodies; 1 = straight-line code per
// stage (operands become literals, and the compiler can overlap one op's
// reduction with the next op's arithmetic); 2 = straight-line code whose
// real-valued reductions (rotation gradients, Pauli-term values) are
// collected over the stage and summed by one transpose-reduce.
// Passes above this size (ops, counted twice when mu is held) share code
// between stages of the same shape.
constexpr int kShareOps = 100;
// Rotations per pass whose shear parameters come from the CTA's table
// (8 bytes of shared memory and 12 of constant memory each); later ones
// compute their own.
constexpr int kRotTable = 1024;

int stage_code_mode() {
  const char* e = std::getenv("TCG_JIT_UNROLL");
  if (!e || !*e) return 2;
  const int v = e[0] - '0';
  return (v >= 0 && v <= 2) ? v : 2;
}

class Gen {
 public:
  Gen(const Program& P, int mode, int R) : P_(P), mode_(mode), R_(R), unroll_(stage_code_mode()) {}

  // Returns false when the op tables do not fit the 64 KiB constant bank.
  bool source(std::string* out) {
    std::ostringstream o;
    o << "// generated by the tcgb300 plan specialiser: n=" << P_.n << " mode=" << mode_ << "\n";
    o << "struct OpRec { long long off; int sig; int slot; int g0; int g1; unsigned zm; int ny; int zr; int pad; };\n";
    size_t cbytes = 0;
    for (size_t p = 0; p < P_.passes.size(); ++p) cbytes += pass(o, int(p));
    *out = o.str();
    return cbytes <= 60 * 1024;
  }

 private:
  const Program& P_;
  int mode_, R_;
  int unroll_;
  // set by op_sig when the op's real value is left in `defer_var_` for a
  // stage-level reduction (stage code mode 2) instead of reduced in place
  const char* defer_var_ = nullptr;
  bool straight_ = false;  // op_sig is emitting for straight_ops
  int pi_ = 0;             // pass being emitted
  // Modes that hold psi only keep two tile buffers in shared memory (smp,
  // smq): a layout change writes one and reads it back, and the next change
  // writes the other, so the barrier after the read-back is not needed.
  // pend_ = the buffer read last with no barrier since (-1: none); a write
  // into that buffer first takes a barrier.
  int pend_ = -1;
  void guard(std::ostream& c, int b) {
    if (pend_ == b) {
      c << "      __syncthreads();\n";
      pend_ = -1;
    }
  }
  // rotations of the pass's straight-line stages: matrix offset of (c, s)
  // and the sign of q = +-s, for the kernel prologue's shear table
  std::vector<int64_t> rot_off_;
  std::vector<int> rot_sq_;
  bool share_ = false;     // stages of the same shape share code (large passes)
  std::map<std::string, int> shape_id_;  // straight-line stage code -> id
  std::vector<std::string> shape_code_;
  const DevPass* dp_ = nullptr;
  int L_ = 0, NT_ = 0, NR_ = 0, NL_ = 0, NW_ = 0, MS_ = 1;
  bool has_mu_ = false;
  std::map<std::string, int> sig_id_;
  std::vector<std::string> sig_body_;

  bool fwd() const { return mode_ == MODE_FWD; }
  bool bwd() const { return mode_ == MODE_BWD; }
  bool meas() const { return mode_ == MODE_MEAS; }
  bool pacc() const { return mode_ == MODE_PACC; }

  uint32_t gbit(int tile_bit) const { return 1u << dp_->lbits[tile_bit]; }
  uint32_t tr(const Layout& l, int r) const {
    uint32_t o = 0;
    for (int i = 0; i < l.R; ++i)
      if ((r >> i) & 1) o |= 1u << l.reg_tile[i];
    return o;
  }
  uint32_t gr(const Layout& l, int r) const {
    uint32_t o = 0;
    for (int i = 0; i < l.R; ++i)
      if ((r >> i) & 1) o |= gbit(l.reg_tile[i]);
    return o;
  }
  int regpos(const Layout& l, int g) const {
    for (int i = 0; i < l.R; ++i)
      if (dp_->lbits[l.reg_tile[i]] == g) return i;
    return -1;
  }

  int sig(const std::string& body) {
    auto it = sig_id_.find(body);
    if (it != sig_id_.end()) return it->second;
    const int id = (int)sig_body_.size();
    sig_id_[body] = id;
    sig_body_.push_back(body);
    return id;
  }

  // ------------------------------------------------------------ data moves
  void layout_code(std::ostream& o, const Layout& l) {
    o << "      jt = 0u; gt = 0u;\n";
    for (int i = 0; i < l.nthr; ++i)
      o << "      jt |= ((tid >> " << i << ") & 1u) << " << l.thr_tile[i] << "; gt |= ((tid >> " << i
        << ") & 1u) << " << dp_->lbits[l.thr_tile[i]] << ";\n";
    o << "      sjt = swz(jt);\n";
  }
  void regs_from_smem(std::ostream& o, const Layout& l, bool mu, const char* buf = "smp") {
    for (int r = 0; r < NR_; ++r) {
      o << "      v[" << r << "] = " << buf << "[sjt ^ " << host_swz(tr(l, r)) << "u];";
      if (mu) o << " w[" << r << "] = smu[sjt ^ " << host_swz(tr(l, r)) << "u];";
      o << "\n";
    }
  }
  void regs_to_smem(std::ostream& o, const Layout& l, bool psi, bool mu, const char* buf = "smp") {
    for (int r = 0; r < NR_; ++r) {
      if (psi) o << "      " << buf << "[sjt ^ " << host_swz(tr(l, r)) << "u] = v[" << r << "];";
      if (mu) o << " smu[sjt ^ " << host_swz(tr(l, r)) << "u] = w[" << r << "];";
      o << "\n";
    }
  }
  void regs_from_global(std::ostream& o, const Layout& l, bool mu) {
    for (int r = 0; r < NR_; ++r) {
      o << "      v[" << r << "] = Sl[gt + " << gr(l, r) << "u];";
      if (mu) o << " w[" << r << "] = muz ? czero() : U[gt + " << gr(l, r) << "u];";
      o << "\n";
    }
  }
  void regs_to_global(std::ostream& o, const Layout& l, bool psi, bool mu) {
    for (int r = 0; r < NR_; ++r) {
      if (psi) o << "  S[gt + " << gr(l, r) << "u] = v[" << r << "];";
      if (mu) o << " U[gt + " << gr(l, r) << "u] = w[" << r << "];";
      o << "\n";
    }
  }
  std::string off_expr() const {
    std::ostringstream e;
    e << "(j & 31u)";
    for (int q = kLo; q < L_; ++q) e << " | (((j >> " << q << ") & 1u) << " << dp_->lbits[q] << ")";
    return e.str();
  }
  void staged_load(std::ostream& o, bool psi, bool mu) {
    o << "      for (u32 i = tid; i < " << (1u << (L_ - 1)) << "u; i += " << NT_ << "u) {\n";
    o << "        const u32 j = 2u * i; const u32 off = " << off_expr() << ";\n";
    if (psi)
      o << "        { const float4 q = *reinterpret_cast<const float4*>(Sl + off); smp[swz(j)] = "
           "make_float2(q.x, q.y); smp[swz(j + 1u)] = make_float2(q.z, q.w); }\n";
    if (mu)
      o << "        { const float4 q = muz ? make_float4(0.f, 0.f, 0.f, 0.f) : *reinterpret_cast<const float4*>(U + off); "
           "smu[swz(j)] = make_float2(q.x, q.y); smu[swz(j + 1u)] = make_float2(q.z, q.w); }\n";
    o << "      }\n";
  }
  void staged_store(std::ostream& o, bool psi, bool mu) {
    o << "  for (u32 i = tid; i < " << (1u << (L_ - 1)) << "u; i += " << NT_ << "u) {\n";
    o << "    const u32 j = 2u * i; const u32 off = " << off_expr() << ";\n";
    if (psi)
      o << "    { const float2 a = smp[swz(j)], c = smp[swz(j + 1u)]; *reinterpret_cast<float4*>(S + off) = "
           "make_float4(a.x, a.y, c.x, c.y); }\n";
    if (mu)
      o << "    { const float2 a = smu[swz(j)], c = smu[swz(j + 1u)]; *reinterpret_cast<float4*>(U + off) = "
           "make_float4(a.x, a.y, c.x, c.y); }\n";
    o << "  }\n";
  }

  // One real value (a rotation's gradient): a real butterfly; the first
  // lane writes (sum, 0) where the complex reduction would.
  std::string reduce_real(const char* var) {
    if (straight_ && unroll_ == 2 && NL_ == 32) {
      defer_var_ = var;
      return "";
    }
    std::ostringstream o;
    if (NL_ < 32) {
      o << " { const float t = warp_sum1<" << NL_ << ">(" << var
        << "); if (lane == 0) sms[op.slot] = make_float2(t, 0.f); }";
      return o.str();
    }
    o << " { const float t = warp_sum1<" << NL_ << ">(" << var << "); if (lane == 0) sms[warp * " << MS_
      << " + op.slot] = make_float2(t, 0.f); }";
    return o.str();
  }

  std::string reduce(int E, const char* arr) const {
    std::ostringstream o;
    if (NL_ < 32) {  // one partial warp: a butterfly per entry, lane 0 writes
      o << " small_reduce<" << E << ", " << NL_ << ">(" << arr << ", lane, sms + op.slot);";
      return o.str();
    }
    o << " { int ent; const float2 t = warp_reduce<" << E << ", " << NL_ << ">(" << arr
      << ", lane, ent); if (ent >= 0) sms[warp * " << MS_ << " + op.slot + ent] = t; }";
    return o.str();
  }

  // Body (signature) and record of one register-stage op.  Returns false
  // for ops without a shared body (wide diagonals): their code goes
  // straight into the stage's case.
  void op_sig(const DevOp& op, const Layout& l, OpRec* rec, bool* usesC) {
    std::memset(rec, 0, sizeof(*rec));
    defer_var_ = nullptr;
    rec->off = op.mat_off;
    rec->slot = op.slot;
    std::ostringstream b;
    if (op.kind == OP_DENSE1) {
      if (fwd()) {
        b << "const float2* m = Mt + op.off; dense1<" << NR_ << ", " << op.p[0]
          << ">(v, ld(m), ld(m + 1), ld(m + 2), ld(m + 3));";
      } else {
        const bool G = op.slot >= 0;
        b << "const float2* m = Mt + op.off; float2 acc[4] = {czero(), czero(), czero(), czero()}; dense1_bwd<"
          << NR_ << ", " << op.p[0] << ", " << (G ? "true" : "false")
          << ">(v, w, cconj(ld(m)), cconj(ld(m + 2)), cconj(ld(m + 1)), cconj(ld(m + 3)), acc);";
        if (G) b << reduce(4, "acc");
      }
    } else if (op.kind == OP_DENSE2) {
      if (fwd()) {
        b << "const float2* m = Mt + op.off; float2 mm[16];\n#pragma unroll\n for (int e = 0; e < 16; ++e) mm[e] = "
             "ld(m + e); dense2<"
          << NR_ << ", " << op.p[0] << ", " << op.p[1] << ">(v, mm);";
      } else {
        const bool G = op.slot >= 0;
        b << "const float2* m = Mt + op.off; float2 a[16];\n#pragma unroll\n for (int i = 0; i < 4; ++i)\n#pragma "
             "unroll\n for (int j = 0; j < 4; ++j) a[4 * i + j] = cconj(ld(m + 4 * j + i)); float2 acc[16];\n"
             "#pragma unroll\n for (int e = 0; e < 16; ++e) acc[e] = czero(); dense2_bwd<"
          << NR_ << ", " << op.p[0] << ", " << op.p[1] << ", " << (G ? "true" : "false") << ">(v, w, a, acc);";
        if (G) b << reduce(16, "acc");
      }
    } else if (op.kind == OP_DIAG) {
      const int k = op.k;
      int rb[6];
      for (int i = 0; i < k; ++i) rb[i] = regpos(l, op.p[i]);
      rec->g0 = op.p[0];
      rec->g1 = k > 1 ? op.p[1] : 0;
      const char* t0 = "((gthr >> op.g0) & 1u)";
      const char* t1 = "((gthr >> op.g1) & 1u)";
      if (k <= 2) {
        const bool scalar = (k == 1) ? rb[0] < 0 : (rb[0] < 0 && rb[1] < 0);
        if (fwd()) {
          if (scalar) {
            if (k == 1) b << "cmul_ip(C, ld(Mt + op.off + " << t0 << "));";
            else b << "cmul_ip(C, ld(Mt + op.off + ((" << t0 << " << 1) | " << t1 << ")));";
            *usesC = true;
          } else if (k == 1) {
            b << "diag1<" << NR_ << ", " << rb[0] << ">(v, Mt + op.off, " << t0 << ", false);";
          } else {
            b << "diag2<" << NR_ << ", " << rb[0] << ", " << rb[1] << ">(v, Mt + op.off, " << t0 << ", " << t1
              << ", false);";
          }
        } else {
          const bool G = op.slot >= 0;
          b << "float2 acc[4] = {czero(), czero(), czero(), czero()}; ";
          if (k == 1) {
            b << "diag1_bwd<" << NR_ << ", " << rb[0] << ", " << (G ? "true" : "false") << ">(v, w, Mt + op.off, "
              << t0 << ", acc);";
            if (G) b << " float2 a2[2] = {acc[0], acc[1]};" << reduce(2, "a2");
          } else {
            b << "diag2_bwd<" << NR_ << ", " << rb[0] << ", " << rb[1] << ", " << (G ? "true" : "false")
              << ">(v, w, Mt + op.off, " << t0 << ", " << t1 << ", acc);";
            if (G) b << reduce(4, "acc");
          }
        }
      } else {
        // wide diagonal (no gradient): literal per-op code
        b << "const float2* d = Mt + " << op.mat_off << "ll; const u32 rt = 0u";
        for (int i = 0; i < k; ++i)
          if (rb[i] < 0) b << " | (((gthr >> " << op.p[i] << ") & 1u) << " << (k - 1 - i) << ")";
        b << ";";
        for (int r = 0; r < NR_; ++r) {
          uint32_t c = 0;
          for (int i = 0; i < k; ++i)
            if (rb[i] >= 0 && ((r >> rb[i]) & 1)) c |= 1u << (k - 1 - i);
          if (fwd()) {
            b << " cmul_ip(v[" << r << "], ld(d + (rt | " << c << "u)));";
          } else {
            b << " { const float2 e = cconj(ld(d + (rt | " << c << "u))); cmul_ip(v[" << r << "], e); cmul_ip(w["
              << r << "], e); }";
          }
        }
      }
    } else if (op.kind == OP_PROT) {
      rec->pad = 1;  // the op loop prefetches this entry one op ahead
      int zr = 0;
      for (int i = 0; i < l.R; ++i)
        if (gbit(l.reg_tile[i]) & op.zmask) zr |= 1 << i;
      rec->zm = op.zmask;
      rec->ny = op.nY;
      rec->zr = zr;
      // the thread's part of the Z/Y parity; none when every Z/Y bit sits in
      // a register (rx, ry, rxx, ...: no Z bits at all)
      // (the forward loop prefetched the entry one op ahead into csc)
      b << (fwd() ? "const float2 cs = csc; " : "const float2 cs = ld(Mt + op.off); ");
      if ((op.zmask & ~(uint64_t)gr(l, NR_ - 1)) == 0)
        b << "const u32 sg = 0u; ";
      else
        b << "const u32 sg = __popc(gthr & op.zm) & 1u; ";
      // (in straight-line stages the body above is replaced below)
      // three in-place shears per component pair; a rotation with cos < 0
      // toggles the tile's sign bit (applied when the tile is stored)
      if (straight_ && (fwd() || bwd()) && rot_off_.size() < size_t(kRotTable)) {
        // shear parameters from the CTA's table (the kernel prologue filled
        // it and the tile's sign bit); rec->g0 = the rotation's table index
        rec->g0 = (int)rot_off_.size();
        rot_off_.push_back(op.mat_off);
        const bool neg_q = ((op.nY & 3) <= 1) != bwd();  // q = -s: (-i)^nY sign, adjoint
        rot_sq_.push_back(neg_q ? -1 : 1);
        b.str("");
        if ((op.zmask & ~(uint64_t)gr(l, NR_ - 1)) == 0)
          b << "const u32 sg = 0u; ";
        else
          b << "const u32 sg = __popc(gthr & op.zm) & 1u; ";
        b << "const float2 kt = shk[op.g0]; ";
        if (fwd()) {
          b << "float k = kt.x, t = kt.y; if (sg) { k = -k; t = -t; } prot_sh<" << NR_ << ", " << op.xreg << ", "
            << zr << ", " << (op.nY & 3) << ">(v, k, t);";
        } else {
          const bool G = op.slot >= 0;
          b << "float g = 0.f; prot_bwd_kt<" << NR_ << ", " << op.xreg << ", " << zr << ", " << (op.nY & 3) << ", "
            << (G ? "true" : "false") << ">(v, w, kt.x, kt.y, sg, g);";
          if (G) b << reduce_real("g");
        }
      } else if (fwd()) {
        b << "float k, t; pneg ^= shear_params(cs.x, prot_qv<" << (op.nY & 3) << ">(cs.y, sg, false), k, t); prot_sh<"
          << NR_ << ", " << op.xreg << ", " << zr << ", " << (op.nY & 3) << ">(v, k, t);";
      } else {
        const bool G = op.slot >= 0;
        b << "float g = 0.f; pneg ^= prot_bwd_sh<" << NR_ << ", " << op.xreg << ", " << zr << ", " << (op.nY & 3)
          << ", " << (G ? "true" : "false") << ">(v, w, cs.x, cs.y, sg, g);";
        if (G) b << reduce_real("g");
      }
    } else if (op.kind == OP_ZRUN) {
      // entries are literals: each run is its own body
      std::vector<const ZEnt*> slotted;
      for (int e = 0; e < op.k; ++e)
        if (P_.zents[op.mat_off + e].slot >= 0) slotted.push_back(&P_.zents[op.mat_off + e]);
      // per-entry values s_e * t[class_e] reduced over the block in pairs
      // (g_{2i}, g_{2i+1}) of consecutive slots
      auto emit_pairs = [&]() {
        const int KG = (int)slotted.size();
        if (KG == 0) return;
        int E2 = 1;
        while (E2 < (KG + 1) / 2) E2 <<= 1;
        b << " float2 g[" << E2 << "];";
        for (int i = 0; i < E2; ++i) {
          std::string xs = "0.f", ys = "0.f";
          for (int h = 0; h < 2; ++h) {
            const int k = 2 * i + h;
            if (k >= KG) continue;
            std::ostringstream s;
            s << "((__popc(gthr & " << slotted[k]->zmask << "u) & 1u) ? -t[" << slotted[k]->zreg << "] : t["
              << slotted[k]->zreg << "])";
            (h == 0 ? xs : ys) = s.str();
          }
          b << " g[" << i << "] = make_float2(" << xs << ", " << ys << ");";
        }
        if (NL_ < 32) {
          b << " float2 red[" << E2 << "]; small_reduce<" << E2 << ", " << NL_
            << ">(g, lane, red); if (lane == 0) { ";
          for (int k = 0; k < KG; ++k)
            b << "sms[op.slot + " << k << "] = make_float2(red[" << k / 2 << "]." << (k % 2 ? "y" : "x")
              << ", 0.f); ";
          b << "}";
        } else {
          // padding pairs (entries >= KG) hold zeros and must not be
          // written: their slots belong to other ops or other warps
          b << " int ent; const float2 s = warp_reduce<" << E2 << ", " << NL_
            << ">(g, lane, ent); if (ent >= 0 && 2 * ent < " << KG << ") { sms[warp * " << MS_
            << " + op.slot + 2 * ent] = make_float2(s.x, 0.f); if (2 * ent + 1 < " << KG << ") sms[warp * "
            << MS_ << " + op.slot + 2 * ent + 1] = make_float2(s.y, 0.f); }";
        }
      };
      if (meas()) {
        // Z-string terms: <Z_S> partials from one transform of |v_r|^2
        b << "{ float t[" << NR_ << "]; zmeas_t<" << NR_ << ">(v, t);";
        emit_pairs();
        b << " }";
      } else if (pacc()) {
        // mu += (sum_t c_t s_t(x)) psi: class sums and one transform
        b << "{ float a[" << NR_ << "];\n#pragma unroll\n for (int c = 0; c < " << NR_ << "; ++c) a[c] = 0.f;";
        for (int e = 0; e < op.k; ++e) {
          const ZEnt& z = P_.zents[op.mat_off + e];
          b << " a[" << z.zreg << "] += ((__popc(gthr & " << z.zmask << "u) & 1u) ? -1.f : 1.f) * kp.coef[b * "
            << "kp.coef_stride + " << z.mat_off << "ll];";
        }
        b << " add_walsh<" << NR_ << ">(a); zpacc_apply<" << NR_ << ">(v, w, a); }";
      } else {
        // Class products of the run's entries, then the multiplicative
        // Walsh-Hadamard transform into per-register phases.  Which entries
        // are still exactly 1 is known here, so a class nobody touches costs
        // nothing, and a butterfly against a 1 is a copy or a conjugate
        // instead of two complex products.  An entry whose Z bits all sit in
        // registers has a fixed thread parity (even): its factor is conj(u).
        const uint32_t regbits = gr(l, NR_ - 1);
        std::vector<bool> one(NR_, true);
        b << "float2 ph[" << NR_ << "];";
        for (int e = 0; e < op.k; ++e) {
          const ZEnt& z = P_.zents[op.mat_off + e];
          std::ostringstream f;
          if ((z.zmask & ~regbits) == 0)
            f << "cconj(ld(Mt + " << z.mat_off << "ll))";
          else
            f << "zrun_factor(Mt + " << z.mat_off << "ll, gthr, " << z.zmask << "u)";
          if (one[z.zreg]) {
            b << " ph[" << z.zreg << "] = " << f.str() << ";";
            one[z.zreg] = false;
          } else {
            b << " ph[" << z.zreg << "] = cmul(ph[" << z.zreg << "], " << f.str() << ");";
          }
        }
        for (int j = 1; j < NR_; j <<= 1)
          for (int c = 0; c < NR_; ++c) {
            if (c & j) continue;
            const int d = c | j;
            if (one[c] && one[d]) continue;
            if (one[d]) {
              b << " ph[" << d << "] = ph[" << c << "];";
              one[d] = false;
            } else if (one[c]) {
              b << " ph[" << c << "] = ph[" << d << "]; ph[" << d << "] = cconj(ph[" << d << "]);";
              one[c] = false;
            } else {
              b << " { const float2 x = ph[" << c << "], y = ph[" << d << "]; ph[" << c << "] = cmul(x, y); ph["
                << d << "] = cmul(x, cconj(y)); }";
            }
          }
        if (fwd()) {
          for (int r = 0; r < NR_; ++r)
            if (!one[r]) b << " cmul_ip(v[" << r << "], ph[" << r << "]);";
        } else {
          if (!slotted.empty()) {
            b << " { float t[" << NR_ << "]; zrun_grad<" << NR_ << ">(v, w, t);";
            emit_pairs();
            b << " }";
          }
          for (int r = 0; r < NR_; ++r)
            if (!one[r])
              b << " { const float2 e = cconj(ph[" << r << "]); cmul_ip(v[" << r << "], e); cmul_ip(w[" << r
                << "], e); }";
        }
      }
    } else if (op.kind == OP_EXPECT) {
      int zr = 0;
      for (int i = 0; i < l.R; ++i)
        if (gbit(l.reg_tile[i]) & op.zmask) zr |= 1 << i;
      rec->zm = op.zmask;
      rec->ny = op.nY;
      rec->zr = zr;
      // a Pauli string's value is real: one real accumulation per amplitude
      // pair component, signs and the (-i)^nY phase fixed at compile time
      const bool thread_sign = (op.zmask & ~(uint64_t)gr(l, NR_ - 1)) != 0;
      if (meas()) {
        b << "float e = expect_real<" << NR_ << ", " << op.xreg << ", " << zr << ", " << (op.nY & 3) << ">(v);";
        if (thread_sign) b << " if (__popc(gthr & op.zm) & 1) e = -e;";
        b << reduce_real("e");
      } else {
        b << "float k = kp.coef[b * kp.coef_stride + op.off];";
        if (thread_sign) b << " if (__popc(gthr & op.zm) & 1) k = -k;";
        b << " pacc_real<" << NR_ << ", " << op.xreg << ", " << zr << ", " << (op.nY & 3) << ">(v, w, k);";
      }
    }
    rec->sig = sig(b.str());
  }

  // Straight-line code of one register stage: each op's body, its record
  // read from the pass's stage-op table (SOPS_<pass>[rb + k], rb set by the
  // stage's entry code), so that stages of the same shape -- e.g. the four
  // rotations of an ansatz layer on the four register bits -- share one code
  // block and the kernel's code stays small enough for the instruction
  // cache.  In stage code mode 2 the ops' real values are kept in dv[] and
  // reduced together at the end of the stage (pairs of values in one complex
  // transpose-reduce, at most 32 values per reduction).  Returns the shape
  // id, or -1 for a stage without ops.
  // Where a deferred value of the stage's op k goes: a literal slot, or the
  // slot of the op's table record when stages share code.
  std::string slot_ref(const std::vector<OpRec>& srecs, size_t rb0, int k) const {
    if (!share_) return std::to_string(srecs[rb0 + k].slot);
    return "SOPS_" + std::to_string(pi_) + "[rb + " + std::to_string(k) + "].slot";
  }

  int straight_ops(const DevStage& S, const Layout& cur, bool* usesC, std::vector<OpRec>* srecs) {
    std::ostringstream c;
    std::vector<int> dops;  // index within the stage of each deferred value's op
    const size_t rb0 = srecs->size();
    int k = 0;
    for (int oi = S.op_begin; oi < S.op_end; ++oi, ++k) {
      OpRec r;
      straight_ = true;
      op_sig(P_.ops[oi], cur, &r, usesC);
      straight_ = false;
      srecs->push_back(r);
      if (share_)
        c << "      { const OpRec op = SOPS_" << pi_ << "[rb + " << k << "]; (void)op;";
      else
        c << "      { const OpRec op = {" << r.off << "ll, " << r.sig << ", " << r.slot << ", " << r.g0 << ", " << r.g1
          << ", " << r.zm << "u, " << r.ny << ", " << r.zr << ", " << r.pad << "}; (void)op;";
      if (sig_body_[r.sig].find("csc") != std::string::npos) c << " const float2 csc = ld(Mt + op.off);";
      c << " " << sig_body_[r.sig];
      if (defer_var_) {
        c << " dv[" << dops.size() << "] = " << defer_var_ << ";";
        dops.push_back(k);
      }
      c << " }\n";
    }
    if (k == 0) return -1;
    std::ostringstream oc;
    if (!dops.empty()) oc << "      float dv[" << dops.size() << "];\n";
    oc << c.str();
    for (size_t g0 = 0; g0 < dops.size(); g0 += 32) {
      const int K = (int)std::min<size_t>(32, dops.size() - g0);
      int E2 = 1;
      while (E2 < (K + 1) / 2) E2 <<= 1;
      oc << "      { float2 gp[" << E2 << "];";
      for (int i = 0; i < E2; ++i) {
        const int a = 2 * i, bb = 2 * i + 1;
        oc << " gp[" << i << "] = make_float2(" << (a < K ? "dv[" + std::to_string(g0 + a) + "]" : std::string("0.f"))
           << ", " << (bb < K ? "dv[" + std::to_string(g0 + bb) + "]" : std::string("0.f")) << ");";
      }
      oc << " int ent; const float2 t = warp_reduce<" << E2 << ", 32>(gp, lane, ent);\n";
      oc << "        switch (ent) {";
      for (int i = 0; i < E2 && 2 * i < K; ++i) {
        oc << " case " << i << ": sms[warp * " << MS_ << " + " << slot_ref(*srecs, rb0, dops[g0 + 2 * i])
           << "] = make_float2(t.x, 0.f);";
        if (2 * i + 1 < K)
          oc << " sms[warp * " << MS_ << " + " << slot_ref(*srecs, rb0, dops[g0 + 2 * i + 1])
             << "] = make_float2(t.y, 0.f);";
        oc << " break;";
      }
      oc << " default: break; }\n      }\n";
    }
    const std::string code = oc.str();
    auto it = shape_id_.find(code);
    if (it != shape_id_.end()) return it->second;
    const int id = (int)shape_code_.size();
    shape_id_[code] = id;
    shape_code_.push_back(code);
    return id;
  }

  // ------------------------------------------------------------------ pass
  // Emits one kernel; returns the constant-memory bytes its tables use.
  size_t pass(std::ostringstream& out, int pi) {
    dp_ = &P_.passes[pi];
    L_ = dp_->L;
    NR_ = 1 << R_;
    NT_ = 1 << (L_ - R_);
    NL_ = NT_ < 32 ? NT_ : 32;
    NW_ = (NT_ + 31) / 32;
    MS_ = P_.max_slots > 0 ? P_.max_slots : 1;
    has_mu_ = bwd() || pacc();
    sig_id_.clear();
    sig_body_.clear();
    const bool store_psi = fwd() || bwd();
    const bool store_mu = has_mu_;
    const uint64_t N = 1ull << P_.n;
    const uint32_t TILE = 1u << L_;
    const uint64_t ntiles = 1ull << (P_.n - L_);

    std::vector<OpRec> recs;
    std::vector<int> so;  // slot, out pairs
    std::ostringstream cases;  // stage-entry code, one case per stage
    std::vector<OpRec> srecs;  // op records of the straight-line stages
    shape_id_.clear();
    shape_code_.clear();
    rot_off_.clear();
    rot_sq_.clear();
    pi_ = pi;
    pend_ = -1;
    {
      // Code size: literal straight-line code costs about one op body per
      // op.  The n=20 HEA adjoint's first pass (76 ops holding psi and mu,
      // some 250 KB of code) stalled on instruction fetch; sharing code
      // between stages of the same shape halved those stalls there (that
      // pass 2 % faster, the whole step unchanged within run-to-run noise),
      // while smaller passes ran slower with table-driven operands.
      int nops = 0;
      for (int st = dp_->stage_begin; st < dp_->stage_end; ++st) nops += P_.stages[st].op_end - P_.stages[st].op_begin;
      share_ = nops * (has_mu_ ? 2 : 1) > kShareOps;
    }
    bool live = false, in_smem = false;
    Layout cur;
    const int NS = dp_->stage_end - dp_->stage_begin;
    for (int si = 0; si < NS; ++si) {
      const DevStage& S = P_.stages[dp_->stage_begin + si];
      const int ob = (int)recs.size();
      int shape = -1, rb = 0;  // straight-line code block and its first record
      bool usesC = false;
      std::ostringstream c;
      if (S.smem_stage) {
        if (live) {
          guard(c, 0);
          regs_to_smem(c, cur, true, has_mu_);
          live = false;
        } else if (!in_smem) {
          guard(c, 0);
          staged_load(c, true, has_mu_);
        }
        in_smem = true;
        c << "      __syncthreads();\n";
        pend_ = -1;
        for (int oi = S.op_begin; oi < S.op_end; ++oi) {
          const DevOp& op = P_.ops[oi];
          c << "      { const int tb[6] = {" << op.p[0] << ", " << op.p[1] << ", " << op.p[2] << ", " << op.p[3]
            << ", " << op.p[4] << ", " << op.p[5] << "};\n";
          if (fwd() || bwd())
            c << "        denseK_smem<" << op.k << ">(smp, " << L_ << ", tb, Mt + " << op.mat_off << "ll, "
              << (bwd() ? "true" : "false") << ", tid, " << NT_ << ");\n";
          if (bwd())
            c << "        denseK_smem<" << op.k << ">(smu, " << L_ << ", tb, Mt + " << op.mat_off
              << "ll, true, tid, " << NT_ << ");\n";
          c << "      }\n      __syncthreads();\n";
        }
      } else {
        const Layout nl = layout_of(S);
        if (!live) {
          cur = nl;
          layout_code(c, cur);
          if (in_smem) {
            regs_from_smem(c, cur, has_mu_);
            c << "      __syncthreads();\n";
            pend_ = -1;
          } else if (cur.lanes_low) {
            regs_from_global(c, cur, has_mu_);
          } else {
            guard(c, 0);
            staged_load(c, true, has_mu_);
            c << "      __syncthreads();\n";
            regs_from_smem(c, cur, has_mu_);
            if (has_mu_) {
              c << "      __syncthreads();\n";
              pend_ = -1;
            } else {
              pend_ = 0;
            }
          }
          live = true;
          in_smem = false;
        } else if (!same_layout(cur, nl)) {
          if (has_mu_) {
            regs_to_smem(c, cur, true, has_mu_);
            c << "      __syncthreads();\n";
            cur = nl;
            layout_code(c, cur);
            regs_from_smem(c, cur, has_mu_);
            c << "      __syncthreads();\n";
          } else {
            const int wb = pend_ == 0 ? 1 : 0;  // the buffer nobody may still read
            const char* bn = wb ? "smq" : "smp";
            regs_to_smem(c, cur, true, false, bn);
            c << "      __syncthreads();\n";
            cur = nl;
            layout_code(c, cur);
            regs_from_smem(c, cur, false, bn);
            pend_ = wb;
          }
        }
        // dense ops keep the loop: straight-line code lets the compiler load
        // several ops' matrices ahead, past the register budget
        bool dense = false;
        for (int oi = S.op_begin; oi < S.op_end; ++oi)
          dense = dense || P_.ops[oi].kind == OP_DENSE1 || P_.ops[oi].kind == OP_DENSE2;
        if (unroll_ == 0 || dense) {
          for (int oi = S.op_begin; oi < S.op_end; ++oi) {
            OpRec r;
            op_sig(P_.ops[oi], cur, &r, &usesC);
            recs.push_back(r);
          }
        } else {
          rb = (int)srecs.size();
          shape = straight_ops(S, cur, &usesC, &srecs);
        }
      }
      const int oe = (int)recs.size();
      const int sob = (int)so.size() / 2;
      if (bwd() || meas()) {
        for (int e = S.slot_out_begin; e < S.slot_out_end; ++e) {
          so.push_back(P_.slot_out[e].slot);
          so.push_back((int)P_.slot_out[e].out_off);
        }
      }
      const int soe = (int)so.size() / 2;
      cases << "    case " << si << ": {\n" << c.str() << "      ob = " << ob << "; oe = " << oe << "; sob = " << sob
            << "; soe = " << soe << "; useC = " << (usesC ? "true" : "false") << "; sh = " << shape
            << "; rb = " << rb << ";\n    } break;\n";
    }

    // constant tables
    out << "\n__constant__ OpRec OPS_" << pi << "[" << std::max<size_t>(recs.size(), 1) << "] = {";
    if (recs.empty()) out << "{0, 0, -1, 0, 0, 0u, 0, 0, 0}";
    for (size_t i = 0; i < recs.size(); ++i) {
      const OpRec& r = recs[i];
      out << (i ? ", " : "") << "{" << r.off << "ll, " << r.sig << ", " << r.slot << ", " << r.g0 << ", " << r.g1
          << ", " << r.zm << "u, " << r.ny << ", " << r.zr << ", " << r.pad << "}";
    }
    out << "};\n";
    out << "__constant__ OpRec SOPS_" << pi << "[" << std::max<size_t>(srecs.size(), 1) << "] = {";
    if (srecs.empty()) out << "{0, 0, -1, 0, 0, 0u, 0, 0, 0}";
    for (size_t i = 0; i < srecs.size(); ++i) {
      const OpRec& r = srecs[i];
      out << (i ? ", " : "") << "{" << r.off << "ll, " << r.sig << ", " << r.slot << ", " << r.g0 << ", " << r.g1
          << ", " << r.zm << "u, " << r.ny << ", " << r.zr << ", " << r.pad << "}";
    }
    out << "};\n";
    const size_t nrot = rot_off_.size();
    if (nrot > 0) {
      out << "__constant__ long long ROTO_" << pi << "[" << nrot << "] = {";
      for (size_t i = 0; i < nrot; ++i) out << (i ? ", " : "") << rot_off_[i] << "ll";
      out << "};\n__constant__ float ROTS_" << pi << "[" << nrot << "] = {";
      for (size_t i = 0; i < nrot; ++i) out << (i ? ", " : "") << (rot_sq_[i] < 0 ? "-1.f" : "1.f");
      out << "};\n";
    }
    out << "__constant__ int SO_" << pi << "[" << std::max<size_t>(so.size(), 2) << "] = {";
    if (so.empty()) out << "0, 0";
    for (size_t i = 0; i < so.size(); ++i) out << (i ? ", " : "") << so[i];
    out << "};\n";

    // kernel: three CTAs per SM for the modes that hold psi only (80
    // registers), two for the ones that also hold mu (128 registers): more
    // resident warps hide the dependent FMA chains and shuffles of these
    // issue-bound kernels.  A forward pass with Z-rotation runs (16 phases
    // live) fits 80 registers as straight-line code (n=20 HEA: 14.31 ->
    // 13.89 ms per value+grad step), not as the op loop.
    bool zrun = false;
    for (int s = dp_->stage_begin; s < dp_->stage_end; ++s)
      for (int o = P_.stages[s].op_begin; o < P_.stages[s].op_end; ++o)
        if (P_.ops[o].kind == OP_ZRUN) zrun = true;
    const int min_ctas = (has_mu_ || (zrun && fwd() && unroll_ == 0)) ? 2 : 3;
    out << "extern \"C\" __global__ void __launch_bounds__(" << NT_ << ", " << min_ctas << ") "
        << kernel_name(mode_, pi)
        << "(KParams kp) {\n";
    out << "  using namespace tk;\n  extern __shared__ __align__(16) float2 smem[];\n";
    out << "  const u32 tid = threadIdx.x;\n  const int lane = (int)(tid & 31u);\n  const int warp = (int)(tid >> 5);\n";
    out << "  (void)lane; (void)warp;\n  const u32 tile = blockIdx.x;\n  const long long b = (long long)blockIdx.y;\n";
    out << "  u32 base = 0u;\n";
    for (int i = 0; i < dp_->nnonlocal; ++i)
      out << "  base |= ((tile >> " << i << ") & 1u) << " << dp_->nlbits[i] << ";\n";
    out << "  float2* __restrict__ S = kp.psi + (unsigned long long)b * " << N << "ull + base;\n";
    if (has_mu_) out << "  float2* __restrict__ U = kp.mu + (unsigned long long)b * " << N << "ull + base;\n";
    // the first pass of a sweep may read its input state elsewhere, and the
    // first accumulation pass starts mu at zero
    out << "  const float2* __restrict__ Sl = kp.psi_in ? kp.psi_in + (unsigned long long)b * (unsigned long long)"
           "kp.in_stride + base : S;\n  (void)Sl;\n";
    out << "  const bool muz = kp.mu_zero != 0;\n  (void)muz;\n";
    if (fwd() || bwd()) out << "  const float2* __restrict__ Mt = kp.mats + b * kp.mat_stride;\n";
    out << "  float2* const smp = smem;\n";
    if (has_mu_) out << "  float2* const smu = smem + " << TILE << ";\n";
    if (!has_mu_) out << "  float2* const smq = smem + " << TILE << ";\n  (void)smq;\n";
    out << "  float2* const sms = smem + " << 2 * TILE << ";\n  (void)sms;\n";
    out << "  float2 v[" << NR_ << "];\n";
    if (has_mu_) out << "  float2 w[" << NR_ << "];\n";
    out << "  u32 jt = 0u, gt = 0u, sjt = 0u;\n  (void)jt; (void)sjt;\n";
    out << "  u32 pneg = 0u;  // the tile's sign: rotations taken as -(partner)\n  (void)pneg;\n";
    if (nrot > 0) {
      // prologue: the shear parameters of every table rotation, once per CTA,
      // and the tile sign their c < 0 cases leave
      out << "  __shared__ float2 shk[" << nrot << "];\n  __shared__ u32 shneg;\n";
      out << "  if (tid == 0u) shneg = 0u;\n  __syncthreads();\n";
      out << "  for (u32 i = tid; i < " << nrot << "u; i += " << NT_ << "u) {\n";
      out << "    const float2 cs = ld(Mt + ROTO_" << pi << "[i]);\n    float k, t;\n";
      out << "    if (shear_params(cs.x, ROTS_" << pi << "[i] * cs.y, k, t)) atomicXor(&shneg, 1u);\n";
      out << "    shk[i] = make_float2(k, t);\n  }\n  __syncthreads();\n  pneg = shneg;\n";
    }
    out << "#pragma unroll 1\n  for (int s = 0; s < " << NS << "; ++s) {\n";
    out << "    int ob = 0, oe = 0, sob = 0, soe = 0, sh = -1, rb = 0; bool useC = false; (void)rb;\n";
    out << "    switch (s) {\n" << cases.str() << "    default: break;\n    }\n";
    out << "    const u32 gthr = base | gt; (void)gthr;\n    float2 C = cone(); (void)C;\n";
    // forward: rotation entries (records with pad = 1) are loaded one op
    // ahead, so the global load overlaps the previous op's arithmetic (in the
    // adjoint, which holds twice the state, the extra live registers cost
    // more than the hidden latency: measured 9.25 -> 9.59 ms)
    if (fwd())
      out << "    float2 csn = czero();\n    if (ob < oe && OPS_" << pi << "[ob].pad) csn = ld(Mt + OPS_" << pi
          << "[ob].off);\n";
    out << "#pragma unroll 1\n    for (int o = ob; o < oe; ++o) {\n      const OpRec op = OPS_" << pi << "[o];\n";
    if (fwd())
      out << "      const float2 csc = csn; (void)csc;\n      if (o + 1 < oe && OPS_" << pi << "[o + 1].pad) csn = ld(Mt + OPS_"
          << pi << "[o + 1].off);\n";
    out << "      switch (op.sig) {\n";
    {
      // the bodies the op records use (straight-line stages inline theirs)
      std::vector<bool> used(sig_body_.size(), false);
      for (const OpRec& r : recs) used[r.sig] = true;
      for (size_t i = 0; i < sig_body_.size(); ++i)
        if (used[i]) out << "        case " << i << ": { " << sig_body_[i] << " } break;\n";
    }
    out << "        default: break;\n      }\n    }\n";
    if (!shape_code_.empty()) {
      out << "    switch (sh) {\n";
      for (size_t i = 0; i < shape_code_.size(); ++i)
        out << "    case " << i << ": {\n" << shape_code_[i] << "    } break;\n";
      out << "    default: break;\n    }\n";
    }
    out << "    if (useC) {\n#pragma unroll\n      for (int r = 0; r < " << NR_ << "; ++r) cmul_ip(v[r], C);\n    }\n";
    if (bwd() || meas()) {
      out << "    if (soe > sob) {\n      __syncthreads();\n";
      out << "      for (int e = sob + (int)tid; e < soe; e += " << NT_ << ") {\n";
      out << "        const int slot = SO_" << pi << "[2 * e], outo = SO_" << pi << "[2 * e + 1];\n";
      out << "        float2 t = czero();\n";
      out << "        for (int q = 0; q < " << NW_ << "; ++q) { const float2 x = sms[q * " << MS_
          << " + slot]; t.x += x.x; t.y += x.y; }\n";
      out << "        kp.partial[((unsigned long long)b * kp.part_stride + (unsigned long long)outo) * " << ntiles
          << "ull + tile] = t;\n      }\n      __syncthreads();\n    }\n";
    }
    out << "  }\n";
    if ((fwd() || bwd()) && (store_psi || store_mu)) {
      // undo the sign bit the shear rotations left on the whole tile
      if (live) {
        out << "  if (pneg) {\n#pragma unroll\n    for (int r = 0; r < " << NR_ << "; ++r) {";
        if (store_psi) out << " v[r] = cneg(v[r]);";
        if (store_mu && has_mu_) out << " w[r] = cneg(w[r]);";
        out << " }\n  }\n";
      } else if (in_smem) {
        out << "  if (pneg) {\n    for (u32 i = tid; i < " << TILE << "u; i += " << NT_ << "u) {";
        if (store_psi) out << " smp[i] = cneg(smp[i]);";
        if (store_mu && has_mu_) out << " smu[i] = cneg(smu[i]);";
        out << " }\n    __syncthreads();\n  }\n";
      }
    }
    if (store_psi || store_mu) {
      if (live) {
        if (cur.lanes_low) {
          regs_to_global(out, cur, store_psi, store_mu);
        } else {
          std::ostringstream tmp;
          guard(tmp, 0);
          regs_to_smem(tmp, cur, store_psi, store_mu);
          out << tmp.str() << "  __syncthreads();\n";
          staged_store(out, store_psi, store_mu);
        }
      } else if (in_smem) {
        staged_store(out, store_psi, store_mu);
      }
    }
    out << "}\n";
    return (recs.size() + srecs.size()) * sizeof(OpRec) + so.size() * sizeof(int) +
           nrot * (sizeof(long long) + sizeof(float));
  }
};

// ---------------------------------------------------------------- NVRTC
struct Nvrtc {
  bool ok = false;
  decltype(&nvrtcCreateProgram) create = nullptr;
  decltype(&nvrtcCompileProgram) compile = nullptr;
  decltype(&nvrtcGetProgramLogSize) logsize = nullptr;
  decltype(&nvrtcGetProgramLog) getlog = nullptr;
  decltype(&nvrtcGetCUBINSize) cubinsize = nullptr;
  decltype(&nvrtcGetCUBIN) getcubin = nullptr;
  decltype(&nvrtcDestroyProgram) destroy = nullptr;
  decltype(&nvrtcVersion) version = nullptr;
};

Nvrtc& nvrtc() {
  static Nvrtc n;
  static std::once_flag once;
  std::call_once(once, [] {
    const char* names[] = {"libnvrtc.so.13", "libnvrtc.so", "/usr/local/cuda/lib64/libnvrtc.so.13",
                           "/usr/local/cuda/lib64/libnvrtc.so"};
    void* h = nullptr;
    for (const char* nm : names) {
      h = dlopen(nm, RTLD_NOW | RTLD_LOCAL);
      if (h) break;
    }
    if (!h) return;
    n.create = (decltype(n.create))dlsym(h, "nvrtcCreateProgram");
    n.compile = (decltype(n.compile))dlsym(h, "nvrtcCompileProgram");
    n.logsize = (decltype(n.logsize))dlsym(h, "nvrtcGetProgramLogSize");
    n.getlog = (decltype(n.getlog))dlsym(h, "nvrtcGetProgramLog");
    n.cubinsize = (decltype(n.cubinsize))dlsym(h, "nvrtcGetCUBINSize");
    n.getcubin = (decltype(n.getcubin))dlsym(h, "nvrtcGetCUBIN");
    n.destroy = (decltype(n.destroy))dlsym(h, "nvrtcDestroyProgram");
    n.version = (decltype(n.version))dlsym(h, "nvrtcVersion");
    n.ok = n.create && n.compile && n.logsize && n.getlog && n.cubinsize && n.getcubin && n.destroy;
  });
  return n;
}

uint64_t fnv1a(const std::string& s, uint64_t h = 1469598103934665603ull) {
  for (unsigned char c : s) {
    h ^= c;
    h *= 1099511628211ull;
  }
  return h;
}

std::string cache_dir() {
  const char* e = std::getenv("TCG_JIT_CACHE");
  std::string d;
  if (e && *e) {
    d = e;
  } else {
    const char* home = std::getenv("HOME");
    d = std::string(home && *home ? home : "/tmp") + "/.cache/tcgb300";
  }
  return d;
}

void mkdirs(const std::string& d) {
  std::string cur;
  for (size_t i = 0; i < d.size(); ++i) {
    cur += d[i];
    if (d[i] == '/' && cur.size() > 1) mkdir(cur.c_str(), 0755);
  }
  mkdir(d.c_str(), 0755);
}

bool read_file(const std::string& p, std::vector<char>* out) {
  std::ifstream f(p, std::ios::binary);
  if (!f) return false;
  out->assign(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
  return !out->empty();
}

}  // namespace

int jit_policy() {
  const char* e = std::getenv("TCG_JIT");
  if (!e || !*e) return 2;
  if (e[0] == '0' || e[0] == 'n' || e[0] == 'N') return 0;
  if (e[0] == '1' || e[0] == 'y' || e[0] == 'Y' || (e[0] == 'a' && e[1] == 'l')) return 1;
  return 2;
}

std::string jit_source(const Program& P, int mode, int R) {
  Gen g(P, mode, R);
  std::string s;
  g.source(&s);
  return s;
}

bool jit_build(const Program& P, int mode, int R, JitKernels* out) {
  Nvrtc& nv = nvrtc();
  if (!nv.ok) {
    out->failed = true;
    out->log = "NVRTC not found";
    return false;
  }
  std::string body;
  {
    Gen g(P, mode, R);
    if (!g.source(&body)) {
      out->failed = true;
      out->log = "op tables exceed the constant bank";
      return false;
    }
  }
  const std::string src = std::string(kJitDevice) + "\n" + body;
  const char* opts[] = {"--gpu-architecture=sm_103a", "--std=c++17", "-lineinfo", "--ptxas-options=-v"};
  const int nopt = 4;
  int maj = 0, min = 0;
  if (nv.version) nv.version(&maj, &min);
  std::string key = src;
  for (int i = 0; i < nopt; ++i) key += opts[i];
  key += std::to_string(maj) + "." + std::to_string(min);
  char hex[32];
  std::snprintf(hex, sizeof(hex), "%016llx", (unsigned long long)fnv1a(key));
  const std::string dir = cache_dir();
  const std::string path = dir + "/" + hex + ".cubin";
  std::vector<char> cubin;
  if (!read_file(path, &cubin)) {
    nvrtcProgram prog;
    if (nv.create(&prog, src.c_str(), "tcg_pass.cu", 0, nullptr, nullptr) != NVRTC_SUCCESS) {
      out->failed = true;
      out->log = "nvrtcCreateProgram failed";
      return false;
    }
    const nvrtcResult rc = nv.compile(prog, nopt, opts);
    size_t ls = 0;
    nv.logsize(prog, &ls);
    std::string log(ls, '\0');
    if (ls) nv.getlog(prog, &log[0]);
    out->log = log;
    if (rc != NVRTC_SUCCESS) {
      nv.destroy(&prog);
      out->failed = true;
      return false;
    }
    size_t cs = 0;
    nv.cubinsize(prog, &cs);
    cubin.resize(cs);
    nv.getcubin(prog, cubin.data());
    nv.destroy(&prog);
    mkdirs(dir);
    const std::string tmp = path + ".tmp" + std::to_string(::getpid());
    {
      std::ofstream f(tmp, std::ios::binary);
      f.write(cubin.data(), (std::streamsize)cubin.size());
    }
    std::rename(tmp.c_str(), path.c_str());
  }
  if (cudaLibraryLoadData(&out->lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0) != cudaSuccess) {
    cudaGetLastError();
    out->failed = true;
    out->log += "\ncudaLibraryLoadData failed";
    return false;
  }
  const bool has_mu = (mode == MODE_BWD || mode == MODE_PACC);
  for (size_t p = 0; p < P.passes.size(); ++p) {
    cudaKernel_t k;
    const std::string nm = kernel_name(mode, int(p));
    if (cudaLibraryGetKernel(&k, out->lib, nm.c_str()) != cudaSuccess) {
      cudaGetLastError();
      out->failed = true;
      out->log += "\nmissing kernel " + nm;
      return false;
    }
    const int L = P.passes[p].L;
    const int nt = 1 << (L - R);
    const int nw = (nt + 31) / 32;
    const int ms = P.max_slots > 0 ? P.max_slots : 1;
    out->fn.push_back(k);
    out->nthreads.push_back(nt);
    // two tiles: psi and mu, or (modes holding psi only) psi's two buffers
    (void)has_mu;
    out->smem.push_back(size_t(2) * (size_t(1) << L) * 8 + size_t(nw) * ms * 8);
  }
  return true;
}

cudaError_t jit_launch(JitKernels* jk, int pass, const KParams_Host& kp, uint32_t ntiles, int64_t batch, int n,
                       cudaStream_t st) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (!jk->attr_set[dev]) {
    for (size_t p = 0; p < jk->fn.size(); ++p) {
      e = cudaFuncSetAttribute((const void*)jk->fn[p], cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)jk->smem[p]);
      if (e != cudaSuccess) return e;
    }
    jk->attr_set[dev] = true;
  }
  const size_t len = size_t(1) << n;
  for (int64_t b0 = 0; b0 < batch; b0 += 65535) {
    const int64_t nb = (batch - b0) < 65535 ? (batch - b0) : 65535;
    KParams_Host a = kp;
    a.psi = kp.psi + b0 * len;
    if (a.mu) a.mu = kp.mu + b0 * len;
    if (a.mats) a.mats = kp.mats + b0 * kp.mat_stride;
    if (a.coef) a.coef = kp.coef + b0 * kp.coef_stride;
    if (a.psi_in) a.psi_in = kp.psi_in + b0 * kp.in_stride;
    if (a.partial) a.partial = kp.partial + size_t(b0) * kp.part_stride * ntiles;
    void* args[] = {&a};
    count_launch();
    e = cudaLaunchKernel((const void*)jk->fn[pass], dim3(ntiles, (unsigned)nb), dim3(jk->nthreads[pass]), args,
                         jk->smem[pass], st);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace tcg
