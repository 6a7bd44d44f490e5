// tcpass.cu — fused dense blocks on the tensor cores (tcgen05, sm_103a).
//
// A forward pass whose gates all act on its 12 local bits is applied as a
// short sequence of FUSED BLOCKS.  A block is the product F of consecutive
// gates of the pass on (at most) 6 tile bits: a 64 x 64 complex matrix.  For
// one tile (4096 amplitudes = 64 block entries j x 64 columns n) the block is
// the complex GEMM  y[i][n] = sum_j F[i][j] x[j][n]  run on the tensor cores:
//
//   * planar real form: A = 128 x 64 real matrix whose row 2i holds Re F[i][.]
//     and row 2i+1 holds Im F[i][.]; B_re[n][j] = Re x[j][n], B_im likewise.
//     D1 = A B_re^T and D2 = A B_im^T (128 x 64 each, fp32 in tensor memory)
//     give Re y_i = D1[2i] - D2[2i+1] and Im y_i = D2[2i] + D1[2i+1]: one lane
//     shuffle per value in the epilogue.
//   * split precision: every operand v is held as v = hi + lo with hi, lo in
//     fp16 (11 significant bits each, 22 together -- the same operand
//     precision as a 3xTF32 split), and D = A_hi B_hi + A_hi B_lo + A_lo B_hi
//     accumulates in fp32 (kind::f16 MMAs: twice the TF32 rate, half the
//     shared-memory bytes).  fp16's exponent range is handled with exact
//     power-of-two scales: the fused matrix is scaled so its largest entry
//     lies in [2^13, 2^14) (per block, by the fusion kernel) and every tile is
//     rescaled the same way before each block (per tile, from its largest
//     component), so nothing overflows and the low halves stay normal.
//
// Data path per tile (one CTA, 256 threads, three CTAs per SM): the tile is
// read from HBM once and written, split, into the first block's operand
// planes (K-major canonical layout); per block one thread issues 24
// tcgen05.mma (M=128, N=64, K=16) into tensor memory and commits them to an
// mbarrier, the fused matrix of the NEXT block streams in with one bulk TMA
// copy (cp.async.bulk) while the epilogue reads D back (tcgen05.ld) and
// writes the next block's operand planes straight from registers; after the
// last block the tile goes back to HBM once.  All device-side waits are bounded (%globaltimer); a wait that
// runs out sets an error flag (tcg_plan_check reports it), waits once more
// for the copies it issued, frees its tensor memory and ends the CTA.
//
// The reference has no kernel here: it contracts each gate into the network
// one tensordot at a time (tensorcircuit/cons.py:605-623) for gates built by
// tensorcircuit/gates.py (`any`/`unitary` at :772-791).  What must agree is
// the result of applying the gates in order.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdint>

#include "engine.h"
#include "kernels.h"

namespace tcg {

namespace {

constexpr int kTcThreads = 256;  // 512 threads at two CTAs per SM measured slower (58.8 vs 45.9 ms, n=28)
constexpr int kTcWarps = kTcThreads / 32;
constexpr int kTcLdIter = 4096 / (2 * kTcThreads);  // float4 loads per thread
constexpr unsigned long long kTcWaitNs = 2000000000ull;  // 2 s per wait

// shared-memory map of the pass kernel (bytes): three CTAs fit on an SM
constexpr uint32_t kSmA = 0;                  // fused block: hi plane, lo plane (16 KiB each)
constexpr uint32_t kSmB = 32768;              // operand planes, or the fp32 tile copy
constexpr uint32_t kSmT = kSmB + kTcBRegion;  // epilogue address tables raddr[64], caddr[64]
constexpr uint32_t kSmW = kSmT + 512;         // warp maxima [kTcWarps]
constexpr uint32_t kSmM = kSmW + 64;          // mbarriers: matrix copy, MMA completion
constexpr uint32_t kSmX = kSmM + 16;          // tensor-memory base, abort flag, copy in flight
constexpr uint32_t kSmTotal = kSmX + 16;

// canonical K-major, no-swizzle layout of a 16-bit operand: core matrices of
// 8 rows x 16 bytes (8 elements), rows 16 bytes apart; core matrices step
// SBO = 128 bytes along M/N and LBO bytes along K.
__host__ __device__ constexpr uint32_t kmajor_off(uint32_t row, uint32_t k, uint32_t lbo) {
  return (k & 7u) * 2u + (row & 7u) * 16u + (k >> 3) * lbo + (row >> 3) * 128u;
}
constexpr uint32_t kLboA = 2048;  // 128 rows -> 16 core matrices along M
constexpr uint32_t kLboB = 1024;  // 64 rows  -> 8 core matrices along N

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// shared-memory matrix descriptor (tcgen05): start, LBO, SBO in 16-byte
// units, descriptor version 1 at bit 46, no swizzle, base offset 0
__device__ __forceinline__ uint64_t make_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// instruction descriptor, kind::f16: D fp32, A/B fp16, both K-major
__host__ __device__ constexpr uint32_t make_idesc(uint32_t M, uint32_t N) {
  return (1u << 4) | ((N >> 3) << 17) | ((M >> 4) << 24);
}

__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

// One poll; a thread whose phase is not complete yet is suspended for up to
// the hint (or until the phase completes), so waiting warps do not take issue
// slots from the warps of the other CTAs on the SM.
__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t phase) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(bar), "r"(phase), "r"(20000u)
      : "memory");
  return ok != 0;
}

// bounded wait: false when the deadline passed first (the clock is read
// every 64 polls)
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t phase, unsigned long long limit_ns) {
  if (mbar_try(bar, phase)) return true;
  const unsigned long long t0 = globaltimer();
  for (uint32_t it = 1;; ++it) {
    if (mbar_try(bar, phase)) return true;
    if ((it & 63u) == 0u && globaltimer() - t0 > limit_ns) return false;
  }
}

__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}

__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_alloc(uint32_t dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst_smem), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_free(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void mma_f16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                        uint32_t accum) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accum)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// 32 consecutive columns of this warp's 32 lanes, one 32-bit value each
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}
// 16 consecutive columns of this warp's 32 lanes
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// staging swizzle: tile bit t flips bank bit (t mod 5) (the pass kernels'
// swizzle), so lanes that differ in five tile bits of distinct classes hit
// distinct banks
__device__ __forceinline__ uint32_t swz(uint32_t t) { return t ^ (((t >> 5) ^ (t >> 10)) & 31u); }

// power of two s with m * s in [2^13, 2^14) (1 for m == 0), as s and 1/s
__device__ __forceinline__ void pow2_scale(float m, float& s, float& inv) {
  if (!(m > 0.f)) {
    s = 1.f;
    inv = 1.f;
    return;
  }
  const int e = (int)((__float_as_uint(m) >> 23) & 0xFFu) - 127;  // floor(log2 m) for normal m
  int es = 13 - e;
  es = es > 126 ? 126 : (es < -126 ? -126 : es);
  s = __uint_as_float((uint32_t)(127 + es) << 23);
  inv = __uint_as_float((uint32_t)(127 - es) << 23);
}

__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

}  // namespace

// ============================================================================
// Fusion: one CTA builds one block's 64 x 64 matrix F = G_last ... G_first
// (fp32, in shared memory) from the circuit's gate matrices, then writes its
// scaled planar real form as fp16 hi/lo planes in the canonical layout the
// pass kernel copies verbatim.  grid = (blocks, batch).
__global__ void __launch_bounds__(256) tc_fuse_kernel(const TcBlock* __restrict__ blocks,
                                                       const TcGate* __restrict__ gates,
                                                       const float2* __restrict__ mats, int64_t mat_stride,
                                                       uint8_t* __restrict__ fused, float2* __restrict__ scales,
                                                       int slots) {
  __shared__ float2 F[64 * 65];  // F[i * 65 + j]: row i (output), column j (input)
  __shared__ float red[8];
  __shared__ float rowsum[64];
  const TcBlock blk = blocks[blockIdx.x];
  const int64_t b = blockIdx.y;
  const int tid = threadIdx.x;
  const float2* m_b = mats + b * mat_stride;
  for (int e = tid; e < 64 * 64; e += 256) {
    const int i = e >> 6, j = e & 63;
    F[i * 65 + j] = make_float2(i == j ? 1.f : 0.f, 0.f);
  }
  for (int g = blk.gate_begin; g < blk.gate_end; ++g) {
    const TcGate G = gates[g];
    const float2* m = m_b + G.mat_off;
    __syncthreads();
    if (G.kind == TCG_GATE_DIAG) {
      for (int e = tid; e < 64 * 64; e += 256) {
        const int i = e >> 6, j = e & 63;
        uint32_t s = 0;
        for (int q = 0; q < G.k; ++q) s |= ((uint32_t)(i >> G.pos[q]) & 1u) << (G.k - 1 - q);
        const float2 d = __ldg(m + s);
        const float2 v = F[i * 65 + j];
        F[i * 65 + j] = make_float2(d.x * v.x - d.y * v.y, d.x * v.y + d.y * v.x);
      }
    } else if (G.kind == TCG_GATE_PAULI_ROT) {
      // G = cos(phi) I - i sin(phi) P, (P v)[a] = (-i)^nY (-1)^popc(a & z) v[a ^ x]
      const float2 cs = __ldg(m);
      const uint32_t x = (uint32_t)G.xmask, z = (uint32_t)G.zmask;
      // -i sin(phi) (-i)^nY = sin(phi) * (-i)^(nY + 1)
      float2 ph;
      switch ((G.nY + 1) & 3) {
        case 0: ph = make_float2(cs.y, 0.f); break;
        case 1: ph = make_float2(0.f, -cs.y); break;
        case 2: ph = make_float2(-cs.y, 0.f); break;
        default: ph = make_float2(0.f, cs.y); break;
      }
      for (int e = tid; e < 64 * 64; e += 256) {
        const int a = e >> 6, j = e & 63;
        const uint32_t a2 = (uint32_t)a ^ x;
        if (x != 0 && a2 < (uint32_t)a) continue;  // each pair once
        const float2 va = F[a * 65 + j];
        const float2 vb = F[a2 * 65 + j];
        const float sa = (__popc(a & z) & 1) ? -1.f : 1.f;
        const float sb = (__popc(a2 & z) & 1) ? -1.f : 1.f;
        // new[a] = c v[a] + ph * sa * v[a ^ x]
        const float2 na = make_float2(cs.x * va.x + sa * (ph.x * vb.x - ph.y * vb.y),
                                      cs.x * va.y + sa * (ph.x * vb.y + ph.y * vb.x));
        if (x == 0) {
          F[a * 65 + j] = na;
        } else {
          const float2 nb = make_float2(cs.x * vb.x + sb * (ph.x * va.x - ph.y * va.y),
                                        cs.x * vb.y + sb * (ph.x * va.y + ph.y * va.x));
          F[a * 65 + j] = na;
          F[a2 * 65 + j] = nb;
        }
      }
    } else {  // dense k-qubit gate: every column j, every group of 2^k rows
      const int K = G.k, D = 1 << K;
      uint32_t gmask = 0;
      for (int q = 0; q < K; ++q) gmask |= 1u << G.pos[q];
      const int groups = 64 >> K;
      for (int task = tid; task < 64 * groups; task += 256) {
        const int j = task & 63;
        const int gi = task >> 6;
        // gi -> the rest index with the gate bits zero (deposit into non-gate bits)
        uint32_t r = 0;
        for (int bit = 0, src = 0; bit < 6; ++bit) {
          if (gmask >> bit & 1u) continue;
          r |= ((uint32_t)(gi >> src) & 1u) << bit;
          ++src;
        }
        float2 v[64];
        for (int s = 0; s < D; ++s) {
          uint32_t idx = r;
          for (int q = 0; q < K; ++q) idx |= ((uint32_t)(s >> (K - 1 - q)) & 1u) << G.pos[q];
          v[s] = F[idx * 65 + j];
        }
        for (int s2 = 0; s2 < D; ++s2) {
          float2 acc = make_float2(0.f, 0.f);
          for (int s = 0; s < D; ++s) {
            const float2 mm = __ldg(m + s2 * D + s);
            acc.x = fmaf(mm.x, v[s].x, fmaf(-mm.y, v[s].y, acc.x));
            acc.y = fmaf(mm.x, v[s].y, fmaf(mm.y, v[s].x, acc.y));
          }
          uint32_t idx = r;
          for (int q = 0; q < K; ++q) idx |= ((uint32_t)(s2 >> (K - 1 - q)) & 1u) << G.pos[q];
          F[idx * 65 + j] = acc;
        }
      }
    }
  }
  __syncthreads();
  float mx = 0.f;
  for (int e = tid; e < 64 * 64; e += 256) {
    const float2 v = F[(e >> 6) * 65 + (e & 63)];
    mx = fmaxf(mx, fmaxf(fabsf(v.x), fabsf(v.y)));
  }
  mx = warp_max(mx);
  if ((tid & 31) == 0) red[tid >> 5] = mx;
  __syncthreads();
  mx = red[0];
  for (int w = 1; w < 8; ++w) mx = fmaxf(mx, red[w]);
  float s, inv;
  pow2_scale(mx, s, inv);
  // bound on the block's gain in one component: max_i sum_j |Re F_ij| + |Im F_ij|
  if (tid < 64) {
    float r = 0.f;
    for (int j = 0; j < 64; ++j) r += fabsf(F[tid * 65 + j].x) + fabsf(F[tid * 65 + j].y);
    rowsum[tid] = r;
  }
  __syncthreads();
  const int64_t slot = b * slots + blk.slot;
  if (tid == 0) {
    float r = 0.f;
    for (int i = 0; i < 64; ++i) r = fmaxf(r, rowsum[i]);
    scales[slot] = make_float2(inv, r);
  }
  uint8_t* out = fused + slot * kTcMatBytes;
  __half* hi = reinterpret_cast<__half*>(out);
  __half* lo = reinterpret_cast<__half*>(out + kTcMatBytes / 2);
  for (int e = tid; e < 128 * 64; e += 256) {
    const int row = e >> 6, k = e & 63;
    const float2 f = F[(row >> 1) * 65 + k];
    const float v = ((row & 1) ? f.y : f.x) * s;
    const __half h = __float2half_rn(v);
    const __half l = __float2half_rn(v - __half2float(h));
    const uint32_t off = kmajor_off((uint32_t)row, (uint32_t)k, kLboA) >> 1;
    hi[off] = h;
    lo[off] = l;
  }
}

// ============================================================================
struct TcArgs {
  float2* psi;
  const float2* psi_in;  // first pass of a sweep: input tiles read here (null: psi)
  int64_t in_stride;
  int n;
  uint32_t ntiles;
  uint32_t nnonlocal;
  int32_t nlbits[kMaxQubits];
  const uint32_t* runs;
  const TcBlock* blocks;
  int nblocks;
  int ldpair;
  uint32_t ldaddr[12];
  const uint8_t* fused;
  const float2* scales;
  int slots;
  unsigned int* err;
};

namespace {

// v = hi + lo, both fp16, at shared address a (the lo plane kTcPlaneLo further);
// put2s: two values that share one 32-bit word (v0 at the lower address)
__device__ __forceinline__ void st_sh32(uint32_t a, uint32_t v) {
  asm volatile("st.shared.b32 [%0], %1;" ::"r"(a), "r"(v) : "memory");
}
__device__ __forceinline__ void st_sh16(uint32_t a, unsigned short v) {
  asm volatile("st.shared.b16 [%0], %1;" ::"r"(a), "h"(v) : "memory");
}
__device__ __forceinline__ void put2s(uint32_t a, float v0, float v1) {
  const __half2 hh = __floats2half2_rn(v0, v1);
  const float2 hf = __half22float2(hh);
  const __half2 ll = __floats2half2_rn(v0 - hf.x, v1 - hf.y);
  st_sh32(a, *reinterpret_cast<const uint32_t*>(&hh));
  st_sh32(a + kTcPlaneLo, *reinterpret_cast<const uint32_t*>(&ll));
}
__device__ __forceinline__ void put1s(uint32_t a, float v) {
  const __half h = __float2half_rn(v);
  const __half l = __float2half_rn(v - __half2float(h));
  st_sh16(a, __half_as_ushort(h));
  st_sh16(a + kTcPlaneLo, __half_as_ushort(l));
}

template <int P>
__device__ __forceinline__ void put_pairs(uint32_t pl, uint32_t R, const uint32_t (&ct)[16], const float (&v)[16]) {
#pragma unroll
  for (int c = 0; c < 16; ++c)
    if (!((c >> P) & 1)) put2s(pl + (R ^ ct[c]), v[c], v[c | (1 << P)]);
}

}  // namespace

// One tile of a tensor-core pass: 4096 amplitudes, every fused block of the
// pass, one read and one write of the tile in HBM.  256 threads, three CTAs
// per SM (66 KiB of shared memory, 128 tensor-memory columns each).
//
// Per block: one thread waits for the block's matrix (bulk copy), issues 12
// MMAs (M=128, N=64, K=16) per plane into one fp32 accumulator -- the two
// correction products first, the main product last, so the tensor core's
// truncating accumulation touches the full-size value only four times -- and
// commits them; every warp waits, thread 0 streams in the next block's
// matrix, and the epilogue turns D into the next block's split operand
// planes directly: Re/Im combination (one lane shuffle), the exact
// power-of-two rescale, fp16 hi/lo split, stores at raddr[i] ^ caddr[n]
// (two values per 32-bit word where the next block's K bit 0 is one of this
// block's column bits).  The scale for the next block comes from a bound
// (2 x max row sum of |F| x the input's largest component), so no extra
// reduction pass is needed; the exact largest output is reduced alongside
// for the block after.  The last block writes fp32 values in natural order,
// which go back to HBM as one coalesced store of the tile.
__global__ void __launch_bounds__(kTcThreads, 3) tc_pass_kernel(const TcArgs a) {
  extern __shared__ __align__(1024) uint8_t smem[];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t sbase = smem_u32(smem);
  uint8_t* bp = smem + kSmB;
  uint32_t* rtab = reinterpret_cast<uint32_t*>(smem + kSmT);
  uint32_t* ctab = rtab + 64;
  float* wmax = reinterpret_cast<float*>(smem + kSmW);
  const uint32_t bar_mat = sbase + kSmM, bar_mma = sbase + kSmM + 8;
  volatile uint32_t* sx = reinterpret_cast<volatile uint32_t*>(smem + kSmX);

  const uint32_t tile = blockIdx.x % a.ntiles;
  const int64_t b = blockIdx.x / a.ntiles;
  uint32_t base = 0;
  for (uint32_t i = 0; i < a.nnonlocal; ++i)
    if ((tile >> i) & 1u) base |= 1u << a.nlbits[i];
  float2* psi = a.psi + b * ((int64_t)1 << a.n);
  const float2* psi_ld = a.psi_in ? a.psi_in + b * a.in_stride : psi;
  const uint8_t* fused_b = a.fused + b * a.slots * (int64_t)kTcMatBytes;
  const float2* scales_b = a.scales + b * a.slots;

  if (warp == 0) tmem_alloc(sbase + kSmX, 128);
  if (tid == 0) {
    mbar_init(bar_mat, 1);
    mbar_init(bar_mma, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    sx[1] = 0;
    sx[2] = 0;
  }
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = sx[0];
  uint32_t ph_mat = 0, ph_mma = 0;
  if (tid == 0) {  // first block's matrix
    sx[2] = 1;
    mbar_expect_tx(bar_mat, kTcMatBytes);
    bulk_g2s(sbase + kSmA, fused_b + (int64_t)a.blocks[0].slot * kTcMatBytes, kTcMatBytes, bar_mat);
  }

  // ---- the tile: kTcLdIter float4 (2 amplitudes each) per thread, its largest component
  float4 xv[kTcLdIter];
  float lmax = 0.f;
#pragma unroll
  for (int u = 0; u < kTcLdIter; ++u) {
    const uint32_t j = 2u * (uint32_t)(tid + kTcThreads * u);
    const uint32_t off = __ldg(a.runs + (j >> kLo)) | (j & ((1u << kLo) - 1));
    xv[u] = __ldcg(reinterpret_cast<const float4*>(psi_ld + (base | off)));
    lmax = fmaxf(lmax, fmaxf(fmaxf(fabsf(xv[u].x), fabsf(xv[u].y)), fmaxf(fabsf(xv[u].z), fabsf(xv[u].w))));
  }
  lmax = warp_max(lmax);
  if (lane == 0) wmax[warp] = lmax;
  __syncthreads();
  float max_in = wmax[0];
  for (int w = 1; w < kTcWarps; ++w) max_in = fmaxf(max_in, wmax[w]);
  float s_in, sinv_in;
  pow2_scale(max_in, s_in, sinv_in);
  // ---- first block's operand planes: the plane offset is linear in the
  // tile offset 2 * (tid + kTcThreads u) + e
  {
    constexpr int kTidBits = kTcThreads == 512 ? 9 : 8;
    uint32_t tb = 0;
#pragma unroll
    for (int k = 0; k < kTidBits; ++k)
      if ((tid >> k) & 1) tb ^= a.ldaddr[1 + k];
#pragma unroll
    for (int u = 0; u < kTcLdIter; ++u) {
      uint32_t ad = tb;
#pragma unroll
      for (int k = 0; k < 11 - kTidBits; ++k)
        if ((u >> k) & 1) ad ^= a.ldaddr[1 + kTidBits + k];
      const float r0 = xv[u].x * s_in, i0 = xv[u].y * s_in, r1 = xv[u].z * s_in, i1 = xv[u].w * s_in;
      const uint32_t pb0 = sbase + kSmB;
      if (a.ldpair) {
        put2s(pb0 + ad, r0, r1);
        put2s(pb0 + kTcPlaneIm + ad, i0, i1);
      } else {
        const uint32_t ad1 = ad ^ a.ldaddr[0];
        put1s(pb0 + ad, r0);
        put1s(pb0 + ad1, r1);
        put1s(pb0 + kTcPlaneIm + ad, i0);
        put1s(pb0 + kTcPlaneIm + ad1, i1);
      }
    }
  }

  const uint32_t idesc = make_idesc(128, 64);
  bool abort = false;
  for (int bi = 0; bi < a.nblocks; ++bi) {
    const TcBlock& blk = a.blocks[bi];
    const bool last = bi + 1 == a.nblocks;
    if (tid < 64) rtab[tid] = blk.raddr[tid];
    else if (tid < 128) ctab[tid - 64] = blk.caddr[tid - 64];
    const float2 sc = __ldg(scales_b + blk.slot);  // {1 / matrix scale, gain bound}
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    // ---- one thread: wait for the matrix, issue the MMAs, commit
    if (tid == 0) {
      tc_fence_after();
      if (!mbar_wait(bar_mat, ph_mat, kTcWaitNs)) {
        sx[1] = 1;  // nothing is committed: the waits below run out as well
      } else {
        ph_mat ^= 1;
        sx[2] = 0;
#pragma unroll
        for (int p = 0; p < 2; ++p) {
          const uint32_t d = tmem + 64u * p;
          const uint32_t bh = sbase + kSmB + p * kTcPlaneIm, bl = bh + kTcPlaneLo;
#pragma unroll
          for (int s = 0; s < 4; ++s)
            mma_f16(d, make_desc(sbase + kSmA + s * 2 * kLboA, kLboA, 128),
                    make_desc(bl + s * 2 * kLboB, kLboB, 128), idesc, s > 0);
#pragma unroll
          for (int s = 0; s < 4; ++s)
            mma_f16(d, make_desc(sbase + kSmA + 16384 + s * 2 * kLboA, kLboA, 128),
                    make_desc(bh + s * 2 * kLboB, kLboB, 128), idesc, 1);
#pragma unroll
          for (int s = 0; s < 4; ++s)
            mma_f16(d, make_desc(sbase + kSmA + s * 2 * kLboA, kLboA, 128),
                    make_desc(bh + s * 2 * kLboB, kLboB, 128), idesc, 1);
        }
        mma_commit(bar_mma);
      }
    }
    uint32_t ok = 0;
    if (lane == 0) ok = mbar_wait(bar_mma, ph_mma, kTcWaitNs) ? 1u : 0u;
    ok = __shfl_sync(0xffffffffu, ok, 0);
    if (!ok) {
      sx[1] = 1;
    } else {
      if (tid == 0 && !last) {  // the tensor core is done with A: next matrix
        sx[2] = 1;
        mbar_expect_tx(bar_mat, kTcMatBytes);
        bulk_g2s(sbase + kSmA, fused_b + (int64_t)a.blocks[bi + 1].slot * kTcMatBytes, kTcMatBytes, bar_mat);
      }
      tc_fence_after();
      // ---- epilogue
      float s_out = 1.f, sinv_out = 1.f;
      if (!last) pow2_scale(2.f * sc.y * max_in, s_out, sinv_out);
      const float f = s_out * sc.x * sinv_in;
      // warp w reads tensor-memory lanes 32 (w % 4) ..; the 64 columns are
      // shared by the kTcWarps / 4 warps of each lane quarter
      constexpr int kCols = 64 / (kTcWarps / 4);
      const int q = warp & 3, hc = warp >> 2;
      const int row = 32 * q + lane;
      const uint32_t R = rtab[row >> 1];
      const uint32_t pl = sbase + kSmB + ((row & 1) ? kTcPlaneIm : 0u);
      const float sgn = (row & 1) ? 1.f : -1.f;
      const int pb = blk.pairbit;
      float m = 0.f;
#pragma unroll
      for (int half = 0; half < kCols / 16; ++half) {
        const int col0 = kCols * hc + 16 * half;
        const uint32_t ta = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)col0;
        float d0[16], d1[16], v[16];
        tmem_ld16(ta, d0);
        tmem_ld16(ta + 64u, d1);
        tmem_wait_ld();
#pragma unroll
        for (int c = 0; c < 16; ++c) {
          v[c] = fmaf(sgn, __shfl_xor_sync(0xffffffffu, d1[c], 1), d0[c]) * f;
          m = fmaxf(m, fabsf(v[c]));
        }
        uint32_t ct[16];
#pragma unroll
        for (int g = 0; g < 4; ++g) {
          const uint4 c4 = *reinterpret_cast<const uint4*>(ctab + col0 + 4 * g);
          ct[4 * g] = c4.x;
          ct[4 * g + 1] = c4.y;
          ct[4 * g + 2] = c4.z;
          ct[4 * g + 3] = c4.w;
        }
        if (last) {
#pragma unroll
          for (int c = 0; c < 16; ++c) st_sh32(pl + (R ^ ct[c]), __float_as_uint(v[c]));
        } else {
          switch (pb) {
            case 0: put_pairs<0>(pl, R, ct, v); break;
            case 1: put_pairs<1>(pl, R, ct, v); break;
            case 2: put_pairs<2>(pl, R, ct, v); break;
            case 3: put_pairs<3>(pl, R, ct, v); break;
            default:
#pragma unroll
              for (int c = 0; c < 16; ++c) put1s(pl + (R ^ ct[c]), v[c]);
          }
        }
      }
      m = warp_max(m);
      if (lane == 0) wmax[warp] = m * sinv_out;
      s_in = s_out;
      sinv_in = sinv_out;
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    if (sx[1]) {
      abort = true;
      break;
    }
    ph_mma ^= 1;
    max_in = wmax[0];
    for (int w = 1; w < kTcWarps; ++w) max_in = fmaxf(max_in, wmax[w]);
  }

  if (!abort) {
#pragma unroll
    for (int u = 0; u < kTcLdIter; ++u) {
      const uint32_t j = 2u * (uint32_t)(tid + kTcThreads * u);
      const uint32_t off = __ldg(a.runs + (j >> kLo)) | (j & ((1u << kLo) - 1));
      const uint32_t w0 = swz(j) * 4u, w1 = swz(j + 1) * 4u;
      const float4 o = make_float4(*reinterpret_cast<const float*>(bp + w0),
                                   *reinterpret_cast<const float*>(bp + kTcPlaneIm + w0),
                                   *reinterpret_cast<const float*>(bp + w1),
                                   *reinterpret_cast<const float*>(bp + kTcPlaneIm + w1));
      *reinterpret_cast<float4*>(psi + (base | off)) = o;
    }
  } else {
    if (tid == 0) atomicExch(a.err, 1u);
    // let the copies and MMAs this CTA issued finish before its memory goes away
    if (sx[2]) mbar_wait(bar_mat, ph_mat, kTcWaitNs);
    mbar_wait(bar_mma, ph_mma, kTcWaitNs);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_free(tmem, 128);
  }
}

// ============================================================================
// Probe of the operand layouts and the MMA: D[128][N] = A[128][K] B[N][K]^T
// for fp16 row-major A and B in global memory (K a multiple of 16 up to 64,
// N a multiple of 32 up to 256), one CTA of 128 threads, the same
// descriptors and instruction descriptor form as the pass kernel.
__global__ void __launch_bounds__(128) tc_mma_probe_kernel(const __half* __restrict__ A,
                                                            const __half* __restrict__ B, float* __restrict__ D,
                                                            int K, int N, unsigned int* err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t sbase = smem_u32(smem);
  const uint32_t lbo_b = (uint32_t)(N / 8) * 128u;
  const uint32_t offB = 16384u;  // A: 128 x 64 max = 16 KiB
  const uint32_t offX = offB + 32768u;
  volatile uint32_t* sx = reinterpret_cast<volatile uint32_t*>(smem + offX);
  const uint32_t bar = sbase + offX + 8;
  if (warp == 0) tmem_alloc(sbase + offX, 256);
  if (tid == 0) {
    mbar_init(bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  for (int e = tid; e < 128 * K; e += 128) {
    const int r = e / K, k = e % K;
    *reinterpret_cast<__half*>(smem + kmajor_off((uint32_t)r, (uint32_t)k, kLboA)) = A[e];
  }
  for (int e = tid; e < N * K; e += 128) {
    const int r = e / K, k = e % K;
    *reinterpret_cast<__half*>(smem + offB + kmajor_off((uint32_t)r, (uint32_t)k, lbo_b)) = B[e];
  }
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = sx[0];
  if (tid == 0) {
    const uint32_t idesc = make_idesc(128, (uint32_t)N);
    for (int s = 0; s < K / 16; ++s)
      mma_f16(tmem, make_desc(sbase + s * 2 * kLboA, kLboA, 128), make_desc(sbase + offB + s * 2 * lbo_b, lbo_b, 128),
              idesc, s > 0);
    mma_commit(bar);
  }
  const bool ok = mbar_wait(bar, 0, kTcWaitNs);
  if (!ok && tid == 0) atomicExch(err, 1u);
  tc_fence_after();
  if (ok) {
    for (int c0 = 0; c0 < N; c0 += 32) {
      float v[32];
      tmem_ld32(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0, v);
      tmem_wait_ld();
      const int row = 32 * warp + lane;
#pragma unroll
      for (int c = 0; c < 32; ++c) D[row * N + c0 + c] = v[c];
    }
  } else {
    mbar_wait(bar, 0, kTcWaitNs);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_free(tmem, 256);
  }
}

// ============================================================================
namespace {

// Kernel attributes are per device: one bit per device and kernel.
std::atomic<uint64_t> g_attr_pass{0}, g_attr_probe{0};

cudaError_t set_attrs_once(std::atomic<uint64_t>& done, const void* fn, int smem, bool carveout) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const uint64_t bit = uint64_t(1) << (dev & 63);
  if (done.load() & bit) return cudaSuccess;
  e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  if (carveout) {
    // the largest shared-memory carveout, so that three CTAs fit on an SM
    e = cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    if (e != cudaSuccess) return e;
  }
  done.fetch_or(bit);
  return cudaSuccess;
}

}  // namespace

cudaError_t launch_tc_fuse(const TcBlock* blocks, int nblocks, const TcGate* gates, const float2* mats,
                           int64_t mat_stride, int64_t batch, uint8_t* fused, float2* scales, int slots,
                           cudaStream_t st) {
  if (nblocks <= 0 || batch <= 0) return cudaSuccess;
  // grid.y is limited to 65535: larger batches go in chunks of circuits
  constexpr int64_t kChunk = 65535;
  for (int64_t b0 = 0; b0 < batch; b0 += kChunk) {
    const int64_t nb = std::min(kChunk, batch - b0);
    dim3 grid((unsigned)nblocks, (unsigned)nb);
    tc_fuse_kernel<<<grid, 256, 0, st>>>(blocks, gates, mats + b0 * mat_stride, mat_stride,
                                         fused + size_t(b0) * size_t(slots) * kTcMatBytes,
                                         scales + size_t(b0) * size_t(slots), slots);
    count_launch();
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t launch_tc_pass(const DevPass& pass, const TcPassDesc& desc, const uint32_t* runs_dev,
                           const TcBlock* blocks_dev, float2* psi, const float2* psi_in, int64_t in_stride, int n,
                           int64_t batch, const uint8_t* fused,
                           const float2* scales, int slots, unsigned int* err, cudaStream_t st) {
  const cudaError_t ea = set_attrs_once(g_attr_pass, (const void*)tc_pass_kernel, (int)kSmTotal, true);
  if (ea != cudaSuccess) return ea;
  // one CTA per (tile, circuit) in a 1-D grid
  if ((int64_t(1) << (n - kTcTileBits)) * batch > int64_t(0x7fffffff)) return cudaErrorInvalidConfiguration;
  TcArgs a;
  a.psi = psi;
  a.psi_in = psi_in;
  a.in_stride = in_stride;
  a.n = n;
  a.ntiles = 1u << (n - kTcTileBits);
  a.nnonlocal = (uint32_t)pass.nnonlocal;
  for (int i = 0; i < kMaxQubits; ++i) a.nlbits[i] = pass.nlbits[i];
  a.runs = runs_dev;
  a.blocks = blocks_dev;
  a.nblocks = desc.block_end - desc.block_begin;
  a.ldpair = desc.ldpair;
  for (int i = 0; i < 12; ++i) a.ldaddr[i] = desc.ldaddr[i];
  a.fused = fused;
  a.scales = scales;
  a.slots = slots;
  a.err = err;
  const int64_t grid = (int64_t)a.ntiles * batch;
  tc_pass_kernel<<<(unsigned)grid, kTcThreads, kSmTotal, st>>>(a);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_tc_mma_probe(const void* A, const void* B, float* D, int K, int N, unsigned int* err,
                                cudaStream_t st) {
  const int smem = 16384 + 32768 + 64;
  const cudaError_t ea = set_attrs_once(g_attr_probe, (const void*)tc_mma_probe_kernel, smem, false);
  if (ea != cudaSuccess) return ea;
  tc_mma_probe_kernel<<<1, 128, smem, st>>>(static_cast<const __half*>(A), static_cast<const __half*>(B), D, K, N,
                                            err);
  count_launch();
  return cudaGetLastError();
}

}  // namespace tcg
