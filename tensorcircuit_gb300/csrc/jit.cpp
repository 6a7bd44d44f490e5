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
// keeps the generic pass kernels of pass.cu.
#include "jit.h"

#include <dlfcn.h>
#include <nvrtc.h>

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

class Gen {
 public:
  Gen(const Program& P, int mode, int R) : P_(P), mode_(mode), R_(R) {}

  std::string source() {
    std::ostringstream& o = os_;
    o << "// generated by the tcgb300 plan specialiser: n=" << P_.n << " mode=" << mode_ << "\n";
    for (size_t p = 0; p < P_.passes.size(); ++p) pass(int(p));
    return o.str();
  }

 private:
  const Program& P_;
  int mode_, R_;
  std::ostringstream os_;
  // per-pass state
  const DevPass* dp_ = nullptr;
  int L_ = 0, NT_ = 0, NR_ = 0, NL_ = 0, NW_ = 0, MS_ = 1;
  bool has_mu_ = false;
  Layout cur_;

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
  // register position holding global bit g in layout l, or -1
  int regpos(const Layout& l, int g) const {
    for (int i = 0; i < l.R; ++i)
      if (dp_->lbits[l.reg_tile[i]] == g) return i;
    return -1;
  }

  void layout_code(const Layout& l) {
    std::ostringstream& o = os_;
    o << "  jt = 0u; gt = 0u;\n";
    for (int i = 0; i < l.nthr; ++i)
      o << "  jt |= ((tid >> " << i << ") & 1u) << " << l.thr_tile[i] << "; gt |= ((tid >> " << i
        << ") & 1u) << " << dp_->lbits[l.thr_tile[i]] << ";\n";
    o << "  sjt = swz(jt);\n";
  }
  void regs_from_smem(const Layout& l, bool mu) {
    for (int r = 0; r < NR_; ++r) {
      os_ << "  v[" << r << "] = smp[sjt ^ " << host_swz(tr(l, r)) << "u];";
      if (mu) os_ << " w[" << r << "] = smu[sjt ^ " << host_swz(tr(l, r)) << "u];";
      os_ << "\n";
    }
  }
  void regs_to_smem(const Layout& l, bool psi, bool mu) {
    for (int r = 0; r < NR_; ++r) {
      if (psi) os_ << "  smp[sjt ^ " << host_swz(tr(l, r)) << "u] = v[" << r << "];";
      if (mu) os_ << " smu[sjt ^ " << host_swz(tr(l, r)) << "u] = w[" << r << "];";
      os_ << "\n";
    }
  }
  void regs_from_global(const Layout& l, bool mu) {
    for (int r = 0; r < NR_; ++r) {
      os_ << "  v[" << r << "] = S[gt + " << gr(l, r) << "u];";
      if (mu) os_ << " w[" << r << "] = U[gt + " << gr(l, r) << "u];";
      os_ << "\n";
    }
  }
  void regs_to_global(const Layout& l, bool psi, bool mu) {
    for (int r = 0; r < NR_; ++r) {
      if (psi) os_ << "  S[gt + " << gr(l, r) << "u] = v[" << r << "];";
      if (mu) os_ << " U[gt + " << gr(l, r) << "u] = w[" << r << "];";
      os_ << "\n";
    }
  }
  std::string off_expr() const {
    std::ostringstream e;
    e << "(j & 31u)";
    for (int q = kLo; q < L_; ++q) e << " | (((j >> " << q << ") & 1u) << " << dp_->lbits[q] << ")";
    return e.str();
  }
  void staged_load(bool psi, bool mu) {
    std::ostringstream& o = os_;
    o << "  for (u32 i = tid; i < " << (1u << (L_ - 1)) << "u; i += " << NT_ << "u) {\n";
    o << "    const u32 j = 2u * i; const u32 off = " << off_expr() << ";\n";
    if (psi)
      o << "    { const float4 q = *reinterpret_cast<const float4*>(S + off); smp[swz(j)] = "
           "make_float2(q.x, q.y); smp[swz(j + 1u)] = make_float2(q.z, q.w); }\n";
    if (mu)
      o << "    { const float4 q = *reinterpret_cast<const float4*>(U + off); smu[swz(j)] = "
           "make_float2(q.x, q.y); smu[swz(j + 1u)] = make_float2(q.z, q.w); }\n";
    o << "  }\n";
  }
  void staged_store(bool psi, bool mu) {
    std::ostringstream& o = os_;
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

  void reduce_to_slot(int E, const char* arr, int slot) {
    os_ << "    { int ent; const float2 t = warp_reduce<" << E << ", " << NL_ << ">(" << arr
        << ", lane, ent); if (ent >= 0) sms[warp * " << MS_ << " + " << slot << " + ent] = t; }\n";
  }

  void op_code(const DevOp& op) {
    std::ostringstream& o = os_;
    const Layout& l = cur_;
    o << "  {\n";
    if (op.kind == OP_DENSE1) {
      o << "    const float2* m = Mt + " << op.mat_off << "ll;\n";
      if (fwd()) {
        o << "    dense1<" << NR_ << ", " << op.p[0] << ">(v, ld(m), ld(m + 1), ld(m + 2), ld(m + 3));\n";
      } else {
        const bool G = op.slot >= 0;
        o << "    float2 acc[4] = {czero(), czero(), czero(), czero()};\n";
        o << "    dense1_bwd<" << NR_ << ", " << op.p[0] << ", " << (G ? "true" : "false")
          << ">(v, w, cconj(ld(m)), cconj(ld(m + 2)), cconj(ld(m + 1)), cconj(ld(m + 3)), acc);\n";
        if (G) reduce_to_slot(4, "acc", op.slot);
      }
    } else if (op.kind == OP_DENSE2) {
      o << "    const float2* m = Mt + " << op.mat_off << "ll;\n";
      if (fwd()) {
        o << "    float2 mm[16];\n#pragma unroll\n    for (int e = 0; e < 16; ++e) mm[e] = ld(m + e);\n";
        o << "    dense2<" << NR_ << ", " << op.p[0] << ", " << op.p[1] << ">(v, mm);\n";
      } else {
        const bool G = op.slot >= 0;
        o << "    float2 a[16];\n#pragma unroll\n    for (int i = 0; i < 4; ++i)\n#pragma unroll\n"
             "      for (int j = 0; j < 4; ++j) a[4 * i + j] = cconj(ld(m + 4 * j + i));\n";
        o << "    float2 acc[16];\n#pragma unroll\n    for (int e = 0; e < 16; ++e) acc[e] = czero();\n";
        o << "    dense2_bwd<" << NR_ << ", " << op.p[0] << ", " << op.p[1] << ", " << (G ? "true" : "false")
          << ">(v, w, a, acc);\n";
        if (G) reduce_to_slot(16, "acc", op.slot);
      }
    } else if (op.kind == OP_DIAG) {
      const int k = op.k;
      int rb[6];
      for (int i = 0; i < k; ++i) rb[i] = regpos(l, op.p[i]);
      o << "    const float2* d = Mt + " << op.mat_off << "ll;\n";
      if (k <= 2) {
        std::ostringstream t0, t1;
        t0 << "((gthr >> " << op.p[0] << ") & 1u)";
        if (k == 2) t1 << "((gthr >> " << op.p[1] << ") & 1u)";
        if (fwd()) {
          bool scalar = (k == 1) ? rb[0] < 0 : (rb[0] < 0 && rb[1] < 0);
          if (scalar) {
            if (k == 1) o << "    C = cmul(C, ld(d + " << t0.str() << "));\n";
            else o << "    C = cmul(C, ld(d + ((" << t0.str() << " << 1) | " << t1.str() << ")));\n";
            uses_c_ = true;
          } else if (k == 1) {
            o << "    diag1<" << NR_ << ", " << rb[0] << ">(v, d, " << t0.str() << ", false);\n";
          } else {
            o << "    diag2<" << NR_ << ", " << rb[0] << ", " << rb[1] << ">(v, d, " << t0.str() << ", "
              << t1.str() << ", false);\n";
          }
        } else {  // BWD
          const bool G = op.slot >= 0;
          o << "    float2 acc[4] = {czero(), czero(), czero(), czero()};\n";
          if (k == 1) {
            o << "    diag1_bwd<" << NR_ << ", " << rb[0] << ", " << (G ? "true" : "false") << ">(v, w, d, "
              << t0.str() << ", acc);\n";
            if (G) {
              o << "    float2 a2[2] = {acc[0], acc[1]};\n";
              reduce_to_slot(2, "a2", op.slot);
            }
          } else {
            o << "    diag2_bwd<" << NR_ << ", " << rb[0] << ", " << rb[1] << ", " << (G ? "true" : "false")
              << ">(v, w, d, " << t0.str() << ", " << t1.str() << ", acc);\n";
            if (G) reduce_to_slot(4, "acc", op.slot);
          }
        }
      } else {
        // wide diagonal (no gradient): run-time part of the index once,
        // register part per amplitude as a literal
        o << "    const u32 rt = 0u";
        for (int i = 0; i < k; ++i)
          if (rb[i] < 0) o << " | (((gthr >> " << op.p[i] << ") & 1u) << " << (k - 1 - i) << ")";
        o << ";\n";
        for (int r = 0; r < NR_; ++r) {
          uint32_t c = 0;
          for (int i = 0; i < k; ++i)
            if (rb[i] >= 0 && ((r >> rb[i]) & 1)) c |= 1u << (k - 1 - i);
          if (fwd()) {
            o << "    v[" << r << "] = cmul(ld(d + (rt | " << c << "u)), v[" << r << "]);\n";
          } else {
            o << "    { const float2 e = cconj(ld(d + (rt | " << c << "u))); v[" << r << "] = cmul(e, v[" << r
              << "]); w[" << r << "] = cmul(e, w[" << r << "]); }\n";
          }
        }
      }
    } else if (op.kind == OP_EXPECT) {
      int zr = 0;
      for (int i = 0; i < l.R; ++i)
        if (gbit(l.reg_tile[i]) & op.zmask) zr |= 1 << i;
      if (meas()) {
        o << "    float2 acc = expect<" << NR_ << ", " << op.xreg << ", " << zr << ">(v);\n";
        o << "    if (__popc(gthr & " << op.zmask << "u) & 1) acc = cneg(acc);\n";
        o << "    acc = cmul(ypow(" << op.nY << "), acc);\n";
        o << "    float2 a1[1] = {acc};\n";
        reduce_to_slot(1, "a1", op.slot);
      } else {
        o << "    float2 cf = cmul(ypow(" << op.nY << "), make_float2(kp.coef[b * kp.coef_stride + " << op.mat_off
          << "ll], 0.f));\n";
        o << "    if (__popc(gthr & " << op.zmask << "u) & 1) cf = cneg(cf);\n";
        o << "    pacc<" << NR_ << ", " << op.xreg << ", " << zr << ">(v, w, cf);\n";
      }
    }
    o << "  }\n";
  }

  void flush_slots(const DevStage& S) {
    std::ostringstream& o = os_;
    o << "  __syncthreads();\n";
    const uint64_t ntiles = 1ull << (P_.n - L_);
    for (int e = S.slot_out_begin; e < S.slot_out_end; ++e) {
      const SlotOut& so = P_.slot_out[e];
      const int te = (e - S.slot_out_begin) % NT_;
      o << "  if (tid == " << te << "u) { float2 t = czero();";
      for (int q = 0; q < NW_; ++q)
        o << " { const float2 x = sms[" << q * MS_ + so.slot << "]; t.x += x.x; t.y += x.y; }";
      o << " kp.partial[((unsigned long long)b * kp.part_stride + " << so.out_off << "ull) * " << ntiles
        << "ull + tile] = t; }\n";
    }
    o << "  __syncthreads();\n";
  }

  bool uses_c_ = false;

  void pass(int pi) {
    std::ostringstream& o = os_;
    dp_ = &P_.passes[pi];
    L_ = dp_->L;
    NR_ = 1 << R_;
    NT_ = 1 << (L_ - R_);
    NL_ = NT_ < 32 ? NT_ : 32;
    NW_ = (NT_ + 31) / 32;
    MS_ = P_.max_slots > 0 ? P_.max_slots : 1;
    has_mu_ = bwd() || pacc();
    const bool store_psi = fwd() || bwd();
    const bool store_mu = has_mu_;
    const uint64_t N = 1ull << P_.n;
    const uint32_t TILE = 1u << L_;
    // two CTAs per SM (<= 128 registers at 256 threads) so one CTA's tile
    // load overlaps the other's arithmetic; the adjoint kernel keeps psi and
    // mu live and gets the whole register file
    o << "\nextern \"C\" __global__ void __launch_bounds__(" << NT_ << ", " << (bwd() ? 1 : 2) << ") tcgk_" << pi
      << "(KParams kp) {\n";
    o << "  using namespace tk;\n";
    o << "  extern __shared__ __align__(16) float2 smem[];\n";
    o << "  const u32 tid = threadIdx.x;\n  const int lane = (int)(tid & 31u);\n  const int warp = (int)(tid >> 5);\n";
    o << "  (void)lane; (void)warp;\n";
    o << "  const u32 tile = blockIdx.x;\n  const long long b = (long long)blockIdx.y;\n";
    o << "  u32 base = 0u;\n";
    for (int i = 0; i < dp_->nnonlocal; ++i) o << "  base |= ((tile >> " << i << ") & 1u) << " << dp_->nlbits[i] << ";\n";
    o << "  float2* __restrict__ S = kp.psi + (unsigned long long)b * " << N << "ull + base;\n";
    if (has_mu_) o << "  float2* __restrict__ U = kp.mu + (unsigned long long)b * " << N << "ull + base;\n";
    if (fwd() || bwd()) o << "  const float2* __restrict__ Mt = kp.mats + b * kp.mat_stride;\n";
    o << "  float2* const smp = smem;\n";
    if (has_mu_) o << "  float2* const smu = smem + " << TILE << ";\n";
    o << "  float2* const sms = smem + " << (has_mu_ ? 2 : 1) * TILE << ";\n  (void)sms;\n";
    o << "  float2 v[" << NR_ << "];\n";
    if (has_mu_) o << "  float2 w[" << NR_ << "];\n";
    o << "  u32 jt = 0u, gt = 0u, sjt = 0u;\n  (void)jt; (void)sjt;\n";
    bool live = false, in_smem = false;
    for (int s = dp_->stage_begin; s < dp_->stage_end; ++s) {
      const DevStage& S = P_.stages[s];
      o << "  // stage " << s << "\n";
      if (S.smem_stage) {
        if (live) {
          regs_to_smem(cur_, true, has_mu_);
          live = false;
        } else if (!in_smem) {
          staged_load(true, has_mu_);
        }
        in_smem = true;
        o << "  __syncthreads();\n";
        for (int oi = S.op_begin; oi < S.op_end; ++oi) {
          const DevOp& op = P_.ops[oi];
          o << "  { const int tb[6] = {" << op.p[0] << ", " << op.p[1] << ", " << op.p[2] << ", " << op.p[3] << ", "
            << op.p[4] << ", " << op.p[5] << "};\n";
          if (fwd() || bwd())
            o << "    denseK_smem<" << op.k << ">(smp, " << L_ << ", tb, Mt + " << op.mat_off << "ll, "
              << (bwd() ? "true" : "false") << ", tid, " << NT_ << ");\n";
          if (bwd())
            o << "    denseK_smem<" << op.k << ">(smu, " << L_ << ", tb, Mt + " << op.mat_off << "ll, true, tid, "
              << NT_ << ");\n";
          o << "  }\n  __syncthreads();\n";
        }
        continue;
      }
      const Layout nl = layout_of(S);
      if (!live) {
        cur_ = nl;
        layout_code(cur_);
        if (in_smem) {
          regs_from_smem(cur_, has_mu_);
          o << "  __syncthreads();\n";
        } else if (cur_.lanes_low) {
          regs_from_global(cur_, has_mu_);
        } else {
          staged_load(true, has_mu_);
          o << "  __syncthreads();\n";
          regs_from_smem(cur_, has_mu_);
          o << "  __syncthreads();\n";
        }
        live = true;
        in_smem = false;
      } else if (!same_layout(cur_, nl)) {
        regs_to_smem(cur_, true, has_mu_);
        o << "  __syncthreads();\n";
        cur_ = nl;
        layout_code(cur_);
        regs_from_smem(cur_, has_mu_);
        o << "  __syncthreads();\n";
      }
      o << "  {\n  const u32 gthr = base | gt; (void)gthr;\n  float2 C = cone(); (void)C;\n";
      uses_c_ = false;
      for (int oi = S.op_begin; oi < S.op_end; ++oi) op_code(P_.ops[oi]);
      if (uses_c_) {
        o << "#pragma unroll\n  for (int r = 0; r < " << NR_ << "; ++r) v[r] = cmul(C, v[r]);\n";
      }
      o << "  }\n";
      if ((bwd() || meas()) && S.nslots > 0) flush_slots(S);
    }
    if (store_psi || store_mu) {
      if (live) {
        if (cur_.lanes_low) {
          regs_to_global(cur_, store_psi, store_mu);
        } else {
          regs_to_smem(cur_, store_psi, store_mu);
          o << "  __syncthreads();\n";
          staged_store(store_psi, store_mu);
        }
      } else if (in_smem) {
        staged_store(store_psi, store_mu);
      }
    }
    o << "}\n";
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
  return g.source();
}

bool jit_build(const Program& P, int mode, int R, JitKernels* out) {
  Nvrtc& nv = nvrtc();
  if (!nv.ok) {
    out->failed = true;
    out->log = "NVRTC not found";
    return false;
  }
  const std::string body = jit_source(P, mode, R);
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
    const std::string nm = "tcgk_" + std::to_string(p);
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
    out->smem.push_back(size_t(has_mu ? 2 : 1) * (size_t(1) << L) * 8 + size_t(nw) * ms * 8);
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
