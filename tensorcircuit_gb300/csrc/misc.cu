// misc.cu — reductions, plain-pass Pauli terms, probabilities, inner
// products and inverse-CDF sampling.
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>

#include "kernels.h"

namespace tcg {

static std::atomic<int64_t> g_launches{0};
void count_launch(int64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
int64_t launch_count() { return g_launches.load(std::memory_order_relaxed); }

namespace {

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ float2 cfma(float2 a, float2 b, float2 c) {
  return make_float2(fmaf(a.x, b.x, fmaf(-a.y, b.y, c.x)), fmaf(a.x, b.y, fmaf(a.y, b.x, c.y)));
}

// -------------------------------------------------------------- reductions
// One warp per (entry, circuit): fixed lane-strided order, then a fixed tree,
// so the sum is the same on every run.
__global__ void reduce_partials_kernel(const float2* __restrict__ partial, int64_t part_stride,
                                       uint32_t ntiles, const int64_t* __restrict__ entries,
                                       int64_t nentries, float2* out64, int64_t os64, double* out128,
                                       int64_t os128) {
  const int warps_per_block = blockDim.x >> 5;
  const int64_t ei = int64_t(blockIdx.x) * warps_per_block + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  const int64_t b = blockIdx.y;
  if (ei >= nentries) return;
  const int64_t e = entries ? entries[ei] : ei;  // null: entries 0 .. nentries-1
  const float2* p = partial + (size_t(b) * part_stride + e) * ntiles;
  // eight loads in flight per lane, summed in a fixed order
  double sx = 0.0, sy = 0.0;
  uint32_t t = lane;
  for (; t + 7 * 32 < ntiles; t += 8 * 32) {
    float2 v[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) v[k] = p[t + k * 32];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      sx += v[k].x;
      sy += v[k].y;
    }
  }
  for (; t < ntiles; t += 32) {
    const float2 v = p[t];
    sx += v.x;
    sy += v.y;
  }
  sx = warp_sum_d(sx);
  sy = warp_sum_d(sy);
  if (lane == 0) {
    if (out64) out64[b * os64 + e] = make_float2((float)sx, (float)sy);
    if (out128) {
      out128[2 * (b * os128 + e)] = sx;
      out128[2 * (b * os128 + e) + 1] = sy;
    }
  }
}

// ---------------------------------------------------------- direct Pauli terms
// <psi|P|psi> with P = (-i)^nY (-1)^{popc(a & z)} |a ^ x><a|, one pass per term.
__global__ void direct_expect_kernel(const float2* __restrict__ psi, int n,
                                     const tcg_pauli* __restrict__ terms, const int* __restrict__ ids,
                                     int nd, int64_t nterms_total, float2* partial) {
  const size_t len = size_t(1) << n;
  const int64_t b = blockIdx.y;
  const float2* s = psi + b * len;
  __shared__ float2 red[32];
  for (int q = 0; q < nd; ++q) {
    const int t = ids[q];
    const uint64_t x = terms[t].xmask, z = terms[t].zmask;
    float ax = 0.f, ay = 0.f;
    for (size_t a = size_t(blockIdx.x) * blockDim.x + threadIdx.x; a < len;
         a += size_t(gridDim.x) * blockDim.x) {
      const float2 u = s[a], v = s[a ^ x];
      const float cx = u.x * v.x + u.y * v.y, cy = u.x * v.y - u.y * v.x;
      const bool neg = __popcll((unsigned long long)(a & z)) & 1;
      ax += neg ? -cx : cx;
      ay += neg ? -cy : cy;
    }
    // phase (-i)^nY
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
      if (threadIdx.x == 0) partial[(size_t(b) * nterms_total + t) * gridDim.x + blockIdx.x] = v;
    }
    __syncthreads();
  }
}

__global__ void direct_pacc_kernel(const float2* __restrict__ psi, float2* __restrict__ mu, int n,
                                   const tcg_pauli* __restrict__ terms, const int* __restrict__ ids,
                                   int nd, const float* __restrict__ coef, int64_t coef_stride) {
  const size_t len = size_t(1) << n;
  const int64_t b = blockIdx.y;
  const float2* s = psi + b * len;
  float2* m = mu + b * len;
  for (size_t a = size_t(blockIdx.x) * blockDim.x + threadIdx.x; a < len;
       a += size_t(gridDim.x) * blockDim.x) {
    float2 acc = m[a];
    for (int q = 0; q < nd; ++q) {
      const int t = ids[q];
      const uint64_t x = terms[t].xmask, z = terms[t].zmask;
      const float c = coef[b * coef_stride + t];
      const int nY = __popcll((unsigned long long)(x & z)) & 3;
      float2 cf = make_float2(c, 0.f);
      if (nY == 1) cf = make_float2(0.f, -c);
      else if (nY == 2) cf = make_float2(-c, 0.f);
      else if (nY == 3) cf = make_float2(0.f, c);
      if (__popcll((unsigned long long)(a & z)) & 1) cf = make_float2(-cf.x, -cf.y);
      acc = cfma(cf, s[a ^ x], acc);
    }
    m[a] = acc;
  }
}

// ---------------------------------------------------------------- probability
__global__ void probability_kernel(const float2* __restrict__ psi, size_t len, float* __restrict__ p) {
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < len; i += size_t(gridDim.x) * blockDim.x) {
    const float2 v = psi[i];
    p[i] = fmaf(v.x, v.x, v.y * v.y);
  }
}

// ---------------------------------------------------------------- inner product
__global__ void inner_kernel(const float2* __restrict__ a, const float2* __restrict__ bb, size_t len,
                             double* partial) {
  const int64_t b = blockIdx.y;
  const float2* x = a + b * len;
  const float2* y = bb + b * len;
  double sx = 0.0, sy = 0.0;
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < len; i += size_t(gridDim.x) * blockDim.x) {
    const float2 u = x[i], v = y[i];
    sx += (double)fmaf(u.x, v.x, u.y * v.y);
    sy += (double)fmaf(u.x, v.y, -u.y * v.x);
  }
  __shared__ double rx[32], ry[32];
  sx = warp_sum_d(sx);
  sy = warp_sum_d(sy);
  if ((threadIdx.x & 31) == 0) {
    rx[threadIdx.x >> 5] = sx;
    ry[threadIdx.x >> 5] = sy;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    const int nw = blockDim.x >> 5;
    double vx = threadIdx.x < nw ? rx[threadIdx.x] : 0.0;
    double vy = threadIdx.x < nw ? ry[threadIdx.x] : 0.0;
    vx = warp_sum_d(vx);
    vy = warp_sum_d(vy);
    if (threadIdx.x == 0) {
      partial[2 * (size_t(b) * gridDim.x + blockIdx.x)] = vx;
      partial[2 * (size_t(b) * gridDim.x + blockIdx.x) + 1] = vy;
    }
  }
}

__global__ void inner_final_kernel(const double* partial, int nblocks, double* out) {
  const int64_t b = blockIdx.x;
  double sx = 0.0, sy = 0.0;
  for (int i = threadIdx.x; i < nblocks; i += 32) {
    sx += partial[2 * (size_t(b) * nblocks + i)];
    sy += partial[2 * (size_t(b) * nblocks + i) + 1];
  }
  sx = warp_sum_d(sx);
  sy = warp_sum_d(sy);
  if (threadIdx.x == 0) {
    out[2 * b] = sx;
    out[2 * b + 1] = sy;
  }
}

// ---------------------------------------------------------------- sampling
// Declared fixed-point weight of one amplitude component x (fp32):
// floor(x^2 * 2^60) computed exactly from the fp32 bits.  x = M * 2^(E-150)
// for a normal number, so x^2 * 2^60 = M^2 * 2^(2E-240) with M^2 < 2^48.
__device__ __forceinline__ uint64_t qweight(float x) {
  const uint32_t bits = __float_as_uint(x) & 0x7fffffffu;
  const uint32_t E = bits >> 23;
  if (E == 0) return 0ull;  // zero or subnormal: below 2^-126, weight 0
  const uint64_t M = (uint64_t)((bits & 0x7fffffu) | 0x800000u);
  const uint64_t M2 = M * M;
  const int s = 2 * (int)E - 240;
  if (s >= 0) return M2 << (s > 15 ? 15 : s);  // |x| < 2 by precondition
  return (-s) >= 64 ? 0ull : (M2 >> (-s));
}
__device__ __forceinline__ uint64_t qamp(float2 v) { return qweight(v.x) + qweight(v.y); }

constexpr int kScanThreads = 256;
constexpr int kScanPer = 16;
constexpr int kScanBlock = kScanThreads * kScanPer;  // 4096 amplitudes

// phase A: block sums (the 16 loads of a thread are issued before any sum)
__global__ void sample_blocksum_kernel(const float2* __restrict__ psi, size_t len, uint64_t* bsum,
                                       uint32_t nblocks) {
  const int64_t b = blockIdx.y;
  const float2* s = psi + b * len;
  const size_t beg = size_t(blockIdx.x) * kScanBlock;
  float2 v[kScanPer];
#pragma unroll
  for (int r = 0; r < kScanPer; ++r) {
    const size_t a = beg + size_t(r) * kScanThreads + threadIdx.x;
    v[r] = (a < len) ? s[a] : make_float2(0.f, 0.f);
  }
  uint64_t acc = 0;
#pragma unroll
  for (int r = 0; r < kScanPer; ++r) acc += qamp(v[r]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  __shared__ uint64_t red[kScanThreads / 32];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint64_t t = 0;
    for (int w = 0; w < kScanThreads / 32; ++w) t += red[w];
    bsum[size_t(b) * nblocks + blockIdx.x] = t;
  }
}

// phase B: exclusive scan of block sums, one CTA per circuit
__global__ void sample_scan_bsum_kernel(uint64_t* bsum, uint32_t nblocks) {
  const int64_t b = blockIdx.x;
  uint64_t* p = bsum + size_t(b) * nblocks;
  const int T = blockDim.x;
  const uint32_t per = (nblocks + T - 1) / T;
  const uint32_t beg = threadIdx.x * per;
  uint64_t loc = 0;
  for (uint32_t i = 0; i < per; ++i)
    if (beg + i < nblocks) loc += p[beg + i];
  __shared__ uint64_t sh[1024];
  sh[threadIdx.x] = loc;
  __syncthreads();
  // Hillis-Steele inclusive scan over thread totals
  for (int o = 1; o < T; o <<= 1) {
    const uint64_t add = (threadIdx.x >= o) ? sh[threadIdx.x - o] : 0ull;
    __syncthreads();
    sh[threadIdx.x] += add;
    __syncthreads();
  }
  uint64_t run = sh[threadIdx.x] - loc;  // exclusive prefix of this thread
  for (uint32_t i = 0; i < per; ++i) {
    if (beg + i < nblocks) {
      const uint64_t v = p[beg + i];
      p[beg + i] = run;
      run += v;
    }
  }
}

// phase C: per-amplitude inclusive CDF.  The block's 4096 amplitudes are
// scanned in 16 rounds of 256 consecutive ones: every thread loads its 16
// amplitudes up front (coalesced), then per round a warp-shuffle scan plus
// the eight warp totals from shared memory (double-buffered: one barrier per
// round) give each amplitude its prefix, stored coalesced.  (Integer sums, so
// any order gives the same bits.  A per-thread scan of 16 consecutive
// amplitudes in shared memory put every lane of a warp on the same bank:
// 16-word strides.)
__global__ void sample_cdf_kernel(const float2* __restrict__ psi, size_t len, const uint64_t* bsum,
                                  uint32_t nblocks, uint64_t* cdf) {
  const int64_t b = blockIdx.y;
  const float2* s = psi + b * len;
  uint64_t* c = cdf + b * len;
  const size_t beg = size_t(blockIdx.x) * kScanBlock;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __shared__ uint64_t wsum[2][kScanThreads / 32];
  float2 v[kScanPer];
#pragma unroll
  for (int r = 0; r < kScanPer; ++r) {
    const size_t a = beg + size_t(r) * kScanThreads + threadIdx.x;
    v[r] = (a < len) ? s[a] : make_float2(0.f, 0.f);
  }
  uint64_t carry = bsum[size_t(b) * nblocks + blockIdx.x];  // exclusive prefix of the block
#pragma unroll
  for (int r = 0; r < kScanPer; ++r) {
    uint64_t x = qamp(v[r]);
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint64_t t = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += t;
    }
    // round r writes buffer r & 1; a thread can reach round r + 2's write only
    // after every thread passed round r + 1's barrier, i.e. read round r's
    if (lane == 31) wsum[r & 1][warp] = x;
    __syncthreads();
    uint64_t pre = 0, tot = 0;
#pragma unroll
    for (int w = 0; w < kScanThreads / 32; ++w) {
      const uint64_t t = wsum[r & 1][w];
      pre += (w < warp) ? t : 0ull;
      tot += t;
    }
    const size_t a = beg + size_t(r) * kScanThreads + threadIdx.x;
    if (a < len) c[a] = carry + pre + x;
    carry += tot;
  }
}

// phase D: target t = floor((1 - u) * total) in double, then the first index
// with cdf >= t (left searchsorted), clamped to len - 1.
__global__ void sample_search_kernel(const uint64_t* __restrict__ cdf, size_t len, const float* __restrict__ u,
                                     int64_t u_stride, int64_t nshots, int64_t* out) {
  const int64_t b = blockIdx.y;
  const uint64_t* c = cdf + b * len;
  const uint64_t total = c[len - 1];
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < nshots;
       i += int64_t(gridDim.x) * blockDim.x) {
    const double wgt = 1.0 - (double)u[b * u_stride + i];
    const double tt = floor(wgt * (double)total);
    const uint64_t t = tt <= 0.0 ? 0ull : (uint64_t)tt;
    size_t lo = 0, hi = len;
    while (lo < hi) {
      const size_t mid = (lo + hi) >> 1;
      if (__ldg(reinterpret_cast<const unsigned long long*>(c + mid)) < t) lo = mid + 1;
      else hi = mid;
    }
    out[b * nshots + i] = (int64_t)(lo < len ? lo : len - 1);
  }
}

inline int grid_for(size_t work, int threads, int cap) {
  size_t g = (work + threads - 1) / threads;
  if (g > (size_t)cap) g = cap;
  if (g < 1) g = 1;
  return (int)g;
}

}  // namespace

cudaError_t launch_reduce_partials(const float2* partial, int64_t part_stride, uint32_t ntiles,
                                   const int64_t* entries_dev, int64_t nentries, int64_t batch,
                                   float2* out_c64, int64_t os64, double* out_c128, int64_t os128,
                                   cudaStream_t st) {
  if (nentries == 0 || batch == 0) return cudaSuccess;
  const int threads = 256, wpb = threads / 32;
  for (int64_t b0 = 0; b0 < batch; b0 += 65535) {
    const int64_t nb = (batch - b0) < 65535 ? (batch - b0) : 65535;
    dim3 grid((unsigned)((nentries + wpb - 1) / wpb), (unsigned)nb);
    count_launch();
    reduce_partials_kernel<<<grid, threads, 0, st>>>(
        partial + size_t(b0) * part_stride * ntiles, part_stride, ntiles, entries_dev, nentries,
        out_c64 ? out_c64 + b0 * os64 : nullptr, os64, out_c128 ? out_c128 + 2 * b0 * os128 : nullptr, os128);
  }
  return cudaGetLastError();
}

cudaError_t launch_direct_expect(const float2* psi, int n, int64_t batch, const tcg_pauli* terms_dev,
                                 const int* ids_dev, int nd, int64_t nterms_total, float2* partial,
                                 uint32_t nblocks, cudaStream_t st) {
  if (nd == 0) return cudaSuccess;
  for (int64_t b0 = 0; b0 < batch; b0 += 65535) {
    const int64_t nb = (batch - b0) < 65535 ? (batch - b0) : 65535;
    dim3 grid(nblocks, (unsigned)nb);
    count_launch();
    direct_expect_kernel<<<grid, 256, 0, st>>>(psi + b0 * (size_t(1) << n), n, terms_dev, ids_dev, nd,
                                               nterms_total, partial + size_t(b0) * nterms_total * nblocks);
  }
  return cudaGetLastError();
}

cudaError_t launch_direct_pacc(const float2* psi, float2* mu, int n, int64_t batch, const tcg_pauli* terms,
                               const int* ids, int nd, const float* coef, int64_t coef_stride,
                               cudaStream_t st) {
  if (nd == 0) return cudaSuccess;
  const size_t len = size_t(1) << n;
  for (int64_t b0 = 0; b0 < batch; b0 += 65535) {
    const int64_t nb = (batch - b0) < 65535 ? (batch - b0) : 65535;
    dim3 grid(grid_for(len, 256, 4096), (unsigned)nb);
    count_launch();
    direct_pacc_kernel<<<grid, 256, 0, st>>>(psi + b0 * len, mu + b0 * len, n, terms, ids, nd,
                                             coef + b0 * coef_stride, coef_stride);
  }
  return cudaGetLastError();
}

cudaError_t launch_probability(const float2* psi, int64_t len, float* p, cudaStream_t st) {
  if (len <= 0) return cudaSuccess;
  count_launch();
  probability_kernel<<<grid_for((size_t)len, 256, 152 * 16), 256, 0, st>>>(psi, (size_t)len, p);
  return cudaGetLastError();
}

size_t inner_scratch_bytes(int64_t len, int64_t batch) {
  (void)len;
  return size_t(batch) * 608 * 2 * sizeof(double);
}

cudaError_t launch_inner(const float2* a, const float2* b, int64_t len, int64_t batch, double* out,
                         void* scratch, cudaStream_t st) {
  const int nblocks = grid_for((size_t)len, 256, 608);
  double* part = static_cast<double*>(scratch);
  for (int64_t b0 = 0; b0 < batch; b0 += 65535) {
    const int64_t nb = (batch - b0) < 65535 ? (batch - b0) : 65535;
    dim3 grid(nblocks, (unsigned)nb);
    count_launch();
    inner_kernel<<<grid, 256, 0, st>>>(a + b0 * len, b + b0 * len, (size_t)len, part + 2 * size_t(b0) * nblocks);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  for (int64_t b0 = 0; b0 < batch; b0 += 65535) {
    const int64_t nb = (batch - b0) < 65535 ? (batch - b0) : 65535;
    count_launch();
    inner_final_kernel<<<(unsigned)nb, 32, 0, st>>>(part + 2 * size_t(b0) * nblocks, nblocks, out + 2 * b0);
  }
  return cudaGetLastError();
}

size_t sample_scratch_bytes(int n, int64_t batch) {
  const size_t len = size_t(1) << n;
  const size_t nblocks = (len + kScanBlock - 1) / kScanBlock;
  return size_t(batch) * (len + nblocks) * sizeof(uint64_t);
}

cudaError_t launch_sample(const float2* psi, int n, int64_t batch, const float* u, int64_t u_stride,
                          int64_t nshots, int64_t* out, void* scratch, cudaStream_t st) {
  const size_t len = size_t(1) << n;
  const uint32_t nblocks = (uint32_t)((len + kScanBlock - 1) / kScanBlock);
  uint64_t* cdf = static_cast<uint64_t*>(scratch);
  uint64_t* bsum = cdf + size_t(batch) * len;
  for (int64_t b0 = 0; b0 < batch; b0 += 65535) {
    const int64_t nb = (batch - b0) < 65535 ? (batch - b0) : 65535;
    const float2* p0 = psi + b0 * len;
    uint64_t* bs0 = bsum + size_t(b0) * nblocks;
    uint64_t* cdf0 = cdf + size_t(b0) * len;
    count_launch(3);
    sample_blocksum_kernel<<<dim3(nblocks, (unsigned)nb), kScanThreads, 0, st>>>(p0, len, bs0, nblocks);
    sample_scan_bsum_kernel<<<(unsigned)nb, 1024, 0, st>>>(bs0, nblocks);
    sample_cdf_kernel<<<dim3(nblocks, (unsigned)nb), kScanThreads, 0, st>>>(p0, len, bs0, nblocks, cdf0);
    if (nshots > 0) {
      dim3 g(grid_for((size_t)nshots, 256, 4096), (unsigned)nb);
      count_launch();
      sample_search_kernel<<<g, 256, 0, st>>>(cdf0, len, u + b0 * u_stride, u_stride, nshots, out + b0 * nshots);
    }
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------- Kraus pick
// One thread per trajectory.  p_i = sum_s Re(ev_s) coef[i, s] (the Pauli
// expansion of <K_i^dag K_i>), running sums c_i in index order, the pick
// r = (int)(sum_{i<K-1} sign(x - c_i) / 2 + (K - 1) / 2) and the rescale
// 1 / (sqrt(p_r) + 1e-10), written as a complex number with zero imaginary
// part.  p (K floats per trajectory) is kept for the backward.
__global__ void kraus_pick_kernel(const float2* __restrict__ ev, int S, const float* __restrict__ coef, int K,
                                  const float* __restrict__ x, int64_t x_stride, int64_t B,
                                  int32_t* __restrict__ pick, float2* __restrict__ scale, float* __restrict__ p) {
  const int64_t b = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (b >= B) return;
  const float2* e = ev + b * S;
  float* pb = p + b * K;
  const float xb = x[b * x_stride];
  float c = 0.f, sg = 0.f;
  for (int i = 0; i < K; ++i) {
    float acc = 0.f;
    for (int s = 0; s < S; ++s) acc = fmaf(e[s].x, coef[i * S + s], acc);
    pb[i] = acc;
    c += acc;
    if (i < K - 1) {
      const float d = xb - c;
      sg += d > 0.f ? 1.f : (d < 0.f ? -1.f : 0.f);
    }
  }
  int r = (int)(sg * 0.5f + float(K - 1) * 0.5f);
  r = r < 0 ? 0 : (r > K - 1 ? K - 1 : r);
  pick[b] = r;
  scale[b] = make_float2(1.f / (sqrtf(pb[r]) + 1e-10f), 0.f);
}

// d/d Re(ev_s) of the rescale: g (-1 / (sqrt(p_r) + 1e-10)^2) / (2 sqrt(p_r))
// coef[r, s]; the picks themselves carry no gradient.
__global__ void kraus_pick_bwd_kernel(const float2* __restrict__ gscale, const int32_t* __restrict__ pick,
                                      const float* __restrict__ p, int K, const float* __restrict__ coef, int S,
                                      int64_t B, float2* __restrict__ gev) {
  const int64_t b = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (b >= B) return;
  const int r = pick[b];
  const float pr = p[b * K + r];
  const float sq = sqrtf(pr);
  const float den = sq + 1e-10f;
  const float gp = -gscale[b].x / (den * den) / (2.f * sq);
  for (int s = 0; s < S; ++s) gev[b * S + s] = make_float2(gp * coef[r * S + s], 0.f);
}

cudaError_t launch_kraus_pick(const float2* ev, int S, const float* coef, int K, const float* x, int64_t x_stride,
                              int64_t B, int32_t* pick, float2* scale, float* p, cudaStream_t st) {
  if (B <= 0) return cudaSuccess;
  count_launch();
  kraus_pick_kernel<<<(unsigned)((B + 127) / 128), 128, 0, st>>>(ev, S, coef, K, x, x_stride, B, pick, scale, p);
  return cudaGetLastError();
}

cudaError_t launch_kraus_pick_bwd(const float2* gscale, const int32_t* pick, const float* p, int K,
                                  const float* coef, int S, int64_t B, float2* gev, cudaStream_t st) {
  if (B <= 0) return cudaSuccess;
  count_launch();
  kraus_pick_bwd_kernel<<<(unsigned)((B + 127) / 128), 128, 0, st>>>(gscale, pick, p, K, coef, S, B, gev);
  return cudaGetLastError();
}

}  // namespace tcg
