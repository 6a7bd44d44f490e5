// noalloc.cu — Pauli expectations that allocate nothing.
//
// Some callers cannot allocate device memory: hosts whose device memory
// belongs to a pool this C ABI cannot reach (a binding or runtime that hands
// over only pre-allocated buffers and forbids allocations of its own), and
// latency-critical loops where cudaMalloc's implicit device synchronisation
// is not acceptable.  tcg_expect_pauli_noalloc serves them:
// the caller passes the state and the output, and the per-block partial sums
// live in a fixed file-scope device array instead of caller or library
// allocations.  No plan is needed (the terms travel as a kernel argument).
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "kernels.h"

namespace tcg {
namespace {

constexpr int kNaMaxTerms = 64;                  // terms per call
constexpr uint32_t kNaBlocks = 152;              // partials per (circuit, term)
constexpr int64_t kNaScratch = int64_t(1) << 20; // float2 partials: 8 MiB
// batch * nterms * kNaBlocks must not exceed kNaScratch: batch * nterms <= 6898

// The scratch.  In host code this name is a host-side stand-in, not a device
// address; the device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) float2 g_na_partials[kNaScratch];

struct NaTerms {
  tcg_pauli t[kNaMaxTerms];
};

// One block per (block index, circuit); each block covers a strided share of
// the state for every term and writes ONE partial per term: every slot the
// reduction reads is written earlier in the same call, so the array needs no
// clearing between calls.
__global__ void na_expect_kernel(const float2* __restrict__ psi, int n, NaTerms terms, int nterms,
                                 float2* partial) {
  const size_t len = size_t(1) << n;
  const int64_t b = blockIdx.y;
  const float2* s = psi + b * len;
  __shared__ float2 red[32];
  for (int q = 0; q < nterms; ++q) {
    const uint64_t x = terms.t[q].xmask, z = terms.t[q].zmask;
    float ax = 0.f, ay = 0.f;
    for (size_t a = size_t(blockIdx.x) * blockDim.x + threadIdx.x; a < len; a += size_t(gridDim.x) * blockDim.x) {
      const float2 u = s[a], v = s[a ^ x];
      const float cx = u.x * v.x + u.y * v.y, cy = u.x * v.y - u.y * v.x;
      const bool neg = __popcll((unsigned long long)(a & z)) & 1;
      ax += neg ? -cx : cx;
      ay += neg ? -cy : cy;
    }
    const int nY = __popcll((unsigned long long)(x & z)) & 3;
    float px = ax, py = ay;
    if (nY == 1) { px = ay; py = -ax; }
    else if (nY == 2) { px = -ax; py = -ay; }
    else if (nY == 3) { px = -ay; py = ax; }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      px += __shfl_xor_sync(0xffffffffu, px, o);
      py += __shfl_xor_sync(0xffffffffu, py, o);
    }
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = make_float2(px, py);
    __syncthreads();
    if (threadIdx.x < 32) {
      float2 v = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : make_float2(0.f, 0.f);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
      }
      if (threadIdx.x == 0) partial[(size_t(b) * nterms + q) * gridDim.x + blockIdx.x] = v;
    }
    __syncthreads();
  }
}

// device address of g_na_partials, looked up once per device
std::mutex g_na_mu;
void* g_na_addr[64] = {nullptr};

}  // namespace
}  // namespace tcg

using namespace tcg;

extern "C" int tcg_expect_pauli_noalloc(const void* psi, int32_t nqubits, int64_t batch, const tcg_pauli* terms,
                                        int32_t nterms, double* out, void* stream) {
  if (!psi || !out || nqubits < 1 || nqubits > kMaxQubits || batch < 0 || nterms < 0 || (nterms > 0 && !terms))
    return TCG_ERR_INVALID_ARG;
  if (batch == 0 || nterms == 0) return TCG_OK;
  if (nterms > kNaMaxTerms || batch > 65535 || batch * nterms * int64_t(kNaBlocks) > kNaScratch)
    return TCG_ERR_TOO_LARGE;
  const uint64_t full = (nqubits >= 64) ? ~0ull : ((1ull << nqubits) - 1);
  NaTerms t;
  for (int i = 0; i < kNaMaxTerms; ++i) t.t[i] = tcg_pauli{0ull, 0ull};
  for (int i = 0; i < nterms; ++i) {
    if ((terms[i].xmask & ~full) || (terms[i].zmask & ~full)) return TCG_ERR_INVALID_ARG;
    t.t[i] = terms[i];
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return TCG_ERR_CUDA;
  void* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_na_mu);
    if (!g_na_addr[dev]) {
      // first call on this device: resolve the array's device address with
      // this device current
      if (cudaGetSymbolAddress(&g_na_addr[dev], g_na_partials) != cudaSuccess) {
        g_na_addr[dev] = nullptr;
        return TCG_ERR_CUDA;
      }
    }
    scratch = g_na_addr[dev];
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  float2* part = static_cast<float2*>(scratch);
  count_launch();
  na_expect_kernel<<<dim3(kNaBlocks, (unsigned)batch), 256, 0, st>>>(static_cast<const float2*>(psi), nqubits, t,
                                                                     nterms, part);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return TCG_ERR_CUDA;
  e = launch_reduce_partials(part, nterms, kNaBlocks, nullptr, nterms, batch, nullptr, 0, out, nterms, st);
  return e == cudaSuccess ? TCG_OK : TCG_ERR_CUDA;
}
