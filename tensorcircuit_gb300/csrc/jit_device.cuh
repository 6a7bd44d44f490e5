// jit_device.cuh — device helpers for the specialised pass kernels.
//
// The specialiser (jit.cpp) turns a planned pass into straight-line CUDA that
// calls these helpers with compile-time register positions, so every register
// index is a constant and no op descriptor is read at run time.  This header
// is compiled by NVRTC together with the generated code (it is embedded in the
// library as a string) and must stay self-contained: no host headers.
#pragma once

typedef unsigned int u32;
typedef unsigned long long u64;

struct KParams {
  float2* psi;
  float2* mu;
  const float2* mats;
  long long mat_stride;
  float2* partial;
  long long part_stride;
  const float* coef;
  long long coef_stride;
  const float2* psi_in;  // first pass of a sweep: read psi here (may be null)
  long long in_stride;
  int mu_zero;           // first pass of an accumulation: mu starts at zero
  int pad;
};

namespace tk {

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float2 cfma(float2 a, float2 b, float2 c) {
  return make_float2(fmaf(a.x, b.x, fmaf(-a.y, b.y, c.x)), fmaf(a.x, b.y, fmaf(a.y, b.x, c.y)));
}
// a * conj(b) + c
__device__ __forceinline__ float2 cfmac(float2 a, float2 b, float2 c) {
  return make_float2(fmaf(a.x, b.x, fmaf(a.y, b.y, c.x)), fmaf(a.y, b.x, fmaf(-a.x, b.y, c.y)));
}
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
// v <- p v with the cross products first and one FMA per component reading
// its own old value last, so the result can stay in v's registers (the op
// loops carry their register arrays; a result in new registers costs copies)
__device__ __forceinline__ void cmul_ip(float2& v, float2 p) {
  const float tx = p.y * v.y, ty = p.y * v.x;
  v.x = fmaf(p.x, v.x, -tx);
  v.y = fmaf(p.x, v.y, ty);
}
__device__ __forceinline__ float2 czero() { return make_float2(0.f, 0.f); }
__device__ __forceinline__ float2 cone() { return make_float2(1.f, 0.f); }
__device__ __forceinline__ float2 cneg(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 ld(const float2* p) { return __ldg(p); }
__device__ __forceinline__ u32 swz(u32 j) { return j ^ (((j >> 5) ^ (j >> 10)) & 31u); }
__device__ __forceinline__ float2 sel2(u32 i, float2 a, float2 b) { return i ? b : a; }
__device__ __forceinline__ float2 sel4(u32 i, float2 a, float2 b, float2 c, float2 d) {
  return (i & 2u) ? ((i & 1u) ? d : c) : ((i & 1u) ? b : a);
}

// ------------------------------------------------------------------ dense
template <int NR, int P>
__device__ __forceinline__ void dense1(float2 (&v)[NR], float2 m0, float2 m1, float2 m2, float2 m3) {
#pragma unroll
  for (int r = 0; r < NR; ++r) {
    if (r & (1 << P)) continue;
    const int r1 = r | (1 << P);
    const float2 x0 = v[r], x1 = v[r1];
    v[r] = cfma(m0, x0, cmul(m1, x1));
    v[r1] = cfma(m2, x0, cmul(m3, x1));
  }
}

template <int NR, int P, bool G>
__device__ __forceinline__ void dense1_bwd(float2 (&v)[NR], float2 (&w)[NR], float2 a0, float2 a1, float2 a2,
                                           float2 a3, float2 (&acc)[4]) {
#pragma unroll
  for (int r = 0; r < NR; ++r) {
    if (r & (1 << P)) continue;
    const int r1 = r | (1 << P);
    const float2 x0 = v[r], x1 = v[r1];
    const float2 y0 = cfma(a0, x0, cmul(a1, x1));
    const float2 y1 = cfma(a2, x0, cmul(a3, x1));
    v[r] = y0;
    v[r1] = y1;
    const float2 u0 = w[r], u1 = w[r1];
    if (G) {
      acc[0] = cfmac(u0, y0, acc[0]);
      acc[1] = cfmac(u0, y1, acc[1]);
      acc[2] = cfmac(u1, y0, acc[2]);
      acc[3] = cfmac(u1, y1, acc[3]);
    }
    w[r] = cfma(a0, u0, cmul(a1, u1));
    w[r1] = cfma(a2, u0, cmul(a3, u1));
  }
}

template <int NR, int P0, int P1>
__device__ __forceinline__ void dense2(float2 (&v)[NR], const float2 (&m)[16]) {
#pragma unroll
  for (int r = 0; r < NR; ++r) {
    if (r & ((1 << P0) | (1 << P1))) continue;
    const int i0 = r, i1 = r | (1 << P1), i2 = r | (1 << P0), i3 = r | (1 << P0) | (1 << P1);
    const float2 x0 = v[i0], x1 = v[i1], x2 = v[i2], x3 = v[i3];
    v[i0] = cfma(m[0], x0, cfma(m[1], x1, cfma(m[2], x2, cmul(m[3], x3))));
    v[i1] = cfma(m[4], x0, cfma(m[5], x1, cfma(m[6], x2, cmul(m[7], x3))));
    v[i2] = cfma(m[8], x0, cfma(m[9], x1, cfma(m[10], x2, cmul(m[11], x3))));
    v[i3] = cfma(m[12], x0, cfma(m[13], x1, cfma(m[14], x2, cmul(m[15], x3))));
  }
}

template <int NR, int P0, int P1, bool G>
__device__ __forceinline__ void dense2_bwd(float2 (&v)[NR], float2 (&w)[NR], const float2 (&a)[16],
                                           float2 (&acc)[16]) {
#pragma unroll
  for (int r = 0; r < NR; ++r) {
    if (r & ((1 << P0) | (1 << P1))) continue;
    const int idx[4] = {r, r | (1 << P1), r | (1 << P0), r | (1 << P0) | (1 << P1)};
    float2 y[4], u[4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
      y[i] = cfma(a[4 * i], v[idx[0]], cfma(a[4 * i + 1], v[idx[1]], cfma(a[4 * i + 2], v[idx[2]],
                                                                          cmul(a[4 * i + 3], v[idx[3]]))));
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      v[idx[i]] = y[i];
      u[i] = w[idx[i]];
    }
    if (G) {
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[4 * i + j] = cfmac(u[i], y[j], acc[4 * i + j]);
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
      w[idx[i]] = cfma(a[4 * i], u[0], cfma(a[4 * i + 1], u[1], cfma(a[4 * i + 2], u[2], cmul(a[4 * i + 3], u[3]))));
  }
}

// k-qubit dense gate applied in place on the shared-memory tile (tile bits
// tb[0..K-1], tb[0] = sub-index MSB); adj applies M^H.
template <int K>
__device__ __forceinline__ void denseK_smem(float2* tile, int L, const int* tb, const float2* m, bool adj, u32 tid,
                                            u32 nthreads) {
  constexpr int D = 1 << K;
  const u32 ngroups = 1u << (L - K);
  int srt[K];
#pragma unroll
  for (int i = 0; i < K; ++i) srt[i] = tb[i];
#pragma unroll
  for (int i = 0; i < K; ++i)
#pragma unroll
    for (int j = 0; j + 1 < K - i; ++j)
      if (srt[j] > srt[j + 1]) {
        const int t = srt[j];
        srt[j] = srt[j + 1];
        srt[j + 1] = t;
      }
  for (u32 g = tid; g < ngroups; g += nthreads) {
    u32 j0 = g;
#pragma unroll
    for (int i = 0; i < K; ++i) {
      const u32 lowm = (1u << srt[i]) - 1u;
      j0 = ((j0 & ~lowm) << 1) | (j0 & lowm);
    }
    float2 x[D];
#pragma unroll
    for (int s = 0; s < D; ++s) {
      u32 j = j0;
#pragma unroll
      for (int i = 0; i < K; ++i)
        if ((s >> (K - 1 - i)) & 1) j |= 1u << tb[i];
      x[s] = tile[swz(j)];
    }
#pragma unroll
    for (int s = 0; s < D; ++s) {
      float2 y = czero();
#pragma unroll 8
      for (int t = 0; t < D; ++t) {
        const float2 e = adj ? cconj(ld(m + t * D + s)) : ld(m + s * D + t);
        y = cfma(e, x[t], y);
      }
      u32 j = j0;
#pragma unroll
      for (int i = 0; i < K; ++i)
        if ((s >> (K - 1 - i)) & 1) j |= 1u << tb[i];
      tile[swz(j)] = y;
    }
  }
}

// ----------------------------------------------------------------- diagonal
// A k<=2 diagonal op whose sub-index bits come from register positions RB0,
// RB1 (or -1: the bit is the run-time value t0 / t1 of this thread).  The
// factor table e[] is selected once per thread; per amplitude the factor is a
// compile-time pick.
template <int RB0, int RB1>
__device__ __forceinline__ int dsub(int r) {
  return ((RB0 >= 0 ? ((r >> RB0) & 1) : 0) << 1) | (RB1 >= 0 ? ((r >> RB1) & 1) : 0);
}

template <int NR, int RB0, int RB1>
__device__ __forceinline__ void diag2(float2 (&v)[NR], const float2* d, u32 t0, u32 t1, bool conj) {
  float2 e[4];
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    const u32 b0 = RB0 >= 0 ? u32((s >> 1) & 1) : t0;
    const u32 b1 = RB1 >= 0 ? u32(s & 1) : t1;
    float2 x = ld(d + ((b0 << 1) | b1));
    e[s] = conj ? cconj(x) : x;
  }
#pragma unroll
  for (int r = 0; r < NR; ++r) cmul_ip(v[r], e[dsub<RB0, RB1>(r)]);
}

template <int NR, int RB0, int RB1, bool G>
__device__ __forceinline__ void diag2_bwd(float2 (&v)[NR], float2 (&w)[NR], const float2* d, u32 t0, u32 t1,
                                          float2 (&acc)[4]) {
  float2 e[4], g[4];
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    const u32 b0 = RB0 >= 0 ? u32((s >> 1) & 1) : t0;
    const u32 b1 = RB1 >= 0 ? u32(s & 1) : t1;
    e[s] = cconj(ld(d + ((b0 << 1) | b1)));
    g[s] = czero();
  }
#pragma unroll
  for (int r = 0; r < NR; ++r) {
    const int s = dsub<RB0, RB1>(r);
    cmul_ip(v[r], e[s]);
    if (G) g[s] = cfmac(w[r], v[r], g[s]);
    cmul_ip(w[r], e[s]);
  }
  if (G) {
    // bin s holds sub-index (b0(s) << 1 | b1(s)); move to output entries
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      const u32 b0 = RB0 >= 0 ? u32((s >> 1) & 1) : t0;
      const u32 b1 = RB1 >= 0 ? u32(s & 1) : t1;
      const u32 o = (b0 << 1) | b1;
      const bool live = (RB0 >= 0 || ((s >> 1) & 1) == 0) && (RB1 >= 0 || (s & 1) == 0);
      if (live) {
        acc[0] = (o == 0) ? make_float2(acc[0].x + g[s].x, acc[0].y + g[s].y) : acc[0];
        acc[1] = (o == 1) ? make_float2(acc[1].x + g[s].x, acc[1].y + g[s].y) : acc[1];
        acc[2] = (o == 2) ? make_float2(acc[2].x + g[s].x, acc[2].y + g[s].y) : acc[2];
        acc[3] = (o == 3) ? make_float2(acc[3].x + g[s].x, acc[3].y + g[s].y) : acc[3];
      }
    }
  }
}

// 1-qubit diagonal: same with a single sub-index bit
template <int NR, int RB>
__device__ __forceinline__ void diag1(float2 (&v)[NR], const float2* d, u32 t, bool conj) {
  float2 e0 = ld(d + (RB >= 0 ? 0u : t)), e1 = ld(d + (RB >= 0 ? 1u : t));
  if (conj) {
    e0 = cconj(e0);
    e1 = cconj(e1);
  }
#pragma unroll
  for (int r = 0; r < NR; ++r) cmul_ip(v[r], (RB >= 0 && ((r >> RB) & 1)) ? e1 : e0);
}

template <int NR, int RB, bool G>
__device__ __forceinline__ void diag1_bwd(float2 (&v)[NR], float2 (&w)[NR], const float2* d, u32 t,
                                          float2 (&acc)[4]) {
  const float2 e0 = cconj(ld(d + (RB >= 0 ? 0u : t))), e1 = cconj(ld(d + (RB >= 0 ? 1u : t)));
  float2 g0 = czero(), g1 = czero();
#pragma unroll
  for (int r = 0; r < NR; ++r) {
    const bool hi = RB >= 0 && ((r >> RB) & 1);
    cmul_ip(v[r], hi ? e1 : e0);
    if (G) {
      if (hi) g1 = cfmac(w[r], v[r], g1);
      else g0 = cfmac(w[r], v[r], g0);
    }
    cmul_ip(w[r], hi ? e1 : e0);
  }
  if (G) {
    if (RB >= 0) {
      acc[0] = g0;
      acc[1] = g1;
    } else {
      acc[0] = t ? czero() : g0;
      acc[1] = t ? g0 : czero();
    }
  }
}

// ----------------------------------------------------------------- Pauli terms
// population count usable in constant expressions (NVRTC has no
// __builtin_popcount)
__host__ __device__ constexpr int tk_popc(unsigned x) { return x ? int(x & 1u) + tk_popc(x >> 1) : 0; }

// A Pauli string's contribution over this thread's registers, as the one
// real number the term needs: P has (-1)^{popc(r & ZR)} (-i)^NY on the
// pairs (r, r ^ X), so <v|P|v> restricted to the registers is
// sgn(NY) * Re or Im of z = sum_r (-1)^{popc(r & ZR)} conj(v_r) v_{r^X}
// (Re for even NY, Im for odd; sgn = + for NY % 4 in {0, 1}).  Two FMAs per
// amplitude with the signs folded at compile time.
template <int NR, int X, int ZR, int NY>
__device__ __forceinline__ float expect_real(const float2 (&v)[NR]) {
  constexpr bool IMZ = (NY & 1) != 0;
  float acc = 0.f;
#pragma unroll
  for (int r = 0; r < NR; ++r) {
    const float2 t = v[r ^ X];
    const bool neg = (tk_popc(r & ZR) & 1) != 0;
    const float vx = neg ? -v[r].x : v[r].x;
    const float vy = neg ? -v[r].y : v[r].y;
    if (IMZ) {
      acc = fmaf(vx, t.y, acc);
      acc = fmaf(-vy, t.x, acc);
    } else {
      acc = fmaf(vx, t.x, acc);
      acc = fmaf(vy, t.y, acc);
    }
  }
  return ((NY & 3) <= 1) ? acc : -acc;
}

// w += k (-i)^NY P v on the registers (k real, the thread's sign folded in):
// (-i)^NY k is real for even NY and imaginary for odd NY, so each component
// takes one FMA, in place.
template <int NR, int X, int ZR, int NY>
__device__ __forceinline__ void pacc_real(const float2 (&v)[NR], float2 (&w)[NR], float k) {
  const float kk = ((NY & 3) == 0 || (NY & 3) == 3) ? k : -k;
#pragma unroll
  for (int r = 0; r < NR; ++r) {
    const float2 t = v[r ^ X];
    const float q = (tk_popc(r & ZR) & 1) ? -kk : kk;
    if ((NY & 1) == 0) {
      // (-i)^NY = +-1: w += q t
      w[r].x = fmaf(q, t.x, w[r].x);
      w[r].y = fmaf(q, t.y, w[r].y);
    } else {
      // (-i)^NY = -+i: w += -i q t for NY % 4 == 1 (kk = -k folds the sign)
      w[r].x = fmaf(-q, t.y, w[r].x);
      w[r].y = fmaf(q, t.x, w[r].y);
    }
  }
}

// ----------------------------------------------------------------- Pauli rotations
// G = c I - i s P with (P psi)[a] = (-i)^NY (-1)^{popc(a & zmask)} psi[a ^ x].
// X: register mask of the X/Y bits; ZR: register mask of the Z/Y bits (the
// rest of the Z/Y mask is folded into the thread sign `sgn`).
// G psi [r] = c psi[r] + (-1)^{popc(r & ZR)} q psi[r ^ X],  q = -i s (-i)^NY (-1)^sgn;
// G^H uses -q.
// q = -i s (-i)^NY is purely imaginary for even NY and purely real for odd
// NY, so the pair update a' = c a + q b, b' = c b + q' a splits into plane
// rotations [[c, -tau], [tau, c]] of two real components (tau = +-q:
// (a.x, b.y) and (a.y, b.x) for imaginary q, (a.x, b.x) and (a.y, b.y) for
// real q, (v.x, v.y) for X = 0).  Paeth's
// decomposition x -= k y; y += tau x; x -= k y with k = tau / (1 + c) does
// it with three FMAs per component pair instead of two products and two
// FMAs, each in place.  |k|, |tau| <= 1 needs c >= 0: a rotation with
// c < 0 is applied as -(the rotation by phi - pi), and the -1 -- the same
// for every amplitude of the tile -- is kept as one sign bit per thread and
// applied when the tile is stored.

// q's nonzero component for this thread (sign of P, adjoint, thread parity).
template <int NY>
__device__ __forceinline__ float prot_qv(float s, u32 sgn, bool adj) {
  float qv = ((NY & 3) <= 1) ? -s : s;
  if (adj ^ (sgn != 0u)) qv = -qv;
  return qv;
}

// Shear parameters (k, t) of the rotation with cosine c and sine q; returns
// 1 when the rotation is taken as the negative of its c >= 0 partner.
__device__ __forceinline__ u32 shear_params(float c, float q, float& k, float& t) {
  const u32 neg = c < 0.f ? 1u : 0u;
  t = neg ? -q : q;
  k = t * __frcp_rn(1.f + fabsf(c));
  return neg;
}

// One of the three shears (step 0 and 2: x += -+k y, step 1: y += +-t x).
template <int STEP>
__device__ __forceinline__ void shear_step(float& x, float& y, float k, float t, bool flip) {
  if (STEP == 1) y = fmaf(flip ? -t : t, x, y);
  else x = fmaf(flip ? k : -k, y, x);
}

// The rotation of every register pair, issued as three sweeps (all first
// shears, then all second, then all third): each sweep has 16 independent
// FMAs, so the three dependent steps of one pair never wait on each other.
template <int NR, int X, int ZR, int NY, int STEP>
__device__ __forceinline__ void prot_sh_sweep(float2 (&v)[NR], float k, float t) {
  constexpr bool QIM = (NY & 1) == 0;
#pragma unroll
  for (int r = 0; r < NR; ++r) {
    const bool sr = (tk_popc(r & ZR) & 1) != 0;  // qr = -qv
    if (X == 0) {
      shear_step<STEP>(v[r].x, v[r].y, k, t, sr);
    } else {
      const int r2 = r ^ X;
      if (r2 < r) continue;
      if (QIM) {
        shear_step<STEP>(v[r].x, v[r2].y, k, t, sr);
        shear_step<STEP>(v[r].y, v[r2].x, k, t, !sr);
      } else {
        shear_step<STEP>(v[r].x, v[r2].x, k, t, !sr);
        shear_step<STEP>(v[r].y, v[r2].y, k, t, !sr);
      }
    }
  }
}

template <int NR, int X, int ZR, int NY>
__device__ __forceinline__ void prot_sh(float2 (&v)[NR], float k, float t) {
  prot_sh_sweep<NR, X, ZR, NY, 0>(v, k, t);
  prot_sh_sweep<NR, X, ZR, NY, 1>(v, k, t);
  prot_sh_sweep<NR, X, ZR, NY, 2>(v, k, t);
}

// Adjoint step: g = Im <mu|P|psi> over this thread's amplitudes (psi, mu
// after the gate), then psi <- G^H psi, mu <- G^H mu by shears; returns the
// sign bit of the step (see above).
template <int NR, int X, int ZR, int NY, bool G>
__device__ __forceinline__ u32 prot_bwd_sh(float2 (&v)[NR], float2 (&w)[NR], float c, float s, u32 sgn, float& g) {
  if (G) {
    constexpr bool IMZ = (NY & 1) == 0;
    // four partial sums (register r into zc[r & 3]): four short FMA chains
    // instead of one of 2 NR dependent FMAs
    float zc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int r = 0; r < NR; ++r) {
      const float2 t = v[r ^ X];
      const bool neg = (tk_popc(r & ZR) & 1) != 0;
      const float wx = neg ? -w[r].x : w[r].x;
      const float wy = neg ? -w[r].y : w[r].y;
      if (IMZ) {
        zc[r & 3] = fmaf(wx, t.y, zc[r & 3]);
        zc[r & 3] = fmaf(-wy, t.x, zc[r & 3]);
      } else {
        zc[r & 3] = fmaf(wx, t.x, zc[r & 3]);
        zc[r & 3] = fmaf(wy, t.y, zc[r & 3]);
      }
    }
    const float zs = (zc[0] + zc[1]) + (zc[2] + zc[3]);
    g = ((NY & 3) == 0 || (NY & 3) == 3) ? zs : -zs;
    if (sgn) g = -g;
  }
  float k, t;
  const u32 ng = shear_params(c, prot_qv<NY>(s, sgn, true), k, t);
  // psi and mu sweeps interleaved: 32 independent FMAs per step
  prot_sh_sweep<NR, X, ZR, NY, 0>(v, k, t);
  prot_sh_sweep<NR, X, ZR, NY, 0>(w, k, t);
  prot_sh_sweep<NR, X, ZR, NY, 1>(v, k, t);
  prot_sh_sweep<NR, X, ZR, NY, 1>(w, k, t);
  prot_sh_sweep<NR, X, ZR, NY, 2>(v, k, t);
  prot_sh_sweep<NR, X, ZR, NY, 2>(w, k, t);
  return ng;
}

// The same adjoint step with the shear parameters precomputed for the
// whole CTA (k, t of the thread-parity-even case; an odd thread parity
// negates both), so no reciprocal sits at the head of each rotation.
template <int NR, int X, int ZR, int NY, bool G>
__device__ __forceinline__ void prot_bwd_kt(float2 (&v)[NR], float2 (&w)[NR], float k, float t, u32 sgn, float& g) {
  if (G) {
    constexpr bool IMZ = (NY & 1) == 0;
    float zc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int r = 0; r < NR; ++r) {
      const float2 tv = v[r ^ X];
      const bool neg = (tk_popc(r & ZR) & 1) != 0;
      const float wx = neg ? -w[r].x : w[r].x;
      const float wy = neg ? -w[r].y : w[r].y;
      if (IMZ) {
        zc[r & 3] = fmaf(wx, tv.y, zc[r & 3]);
        zc[r & 3] = fmaf(-wy, tv.x, zc[r & 3]);
      } else {
        zc[r & 3] = fmaf(wx, tv.x, zc[r & 3]);
        zc[r & 3] = fmaf(wy, tv.y, zc[r & 3]);
      }
    }
    const float zs = (zc[0] + zc[1]) + (zc[2] + zc[3]);
    g = ((NY & 3) == 0 || (NY & 3) == 3) ? zs : -zs;
    if (sgn) g = -g;
  }
  if (sgn) {
    k = -k;
    t = -t;
  }
  prot_sh_sweep<NR, X, ZR, NY, 0>(v, k, t);
  prot_sh_sweep<NR, X, ZR, NY, 0>(w, k, t);
  prot_sh_sweep<NR, X, ZR, NY, 1>(v, k, t);
  prot_sh_sweep<NR, X, ZR, NY, 1>(w, k, t);
  prot_sh_sweep<NR, X, ZR, NY, 2>(v, k, t);
  prot_sh_sweep<NR, X, ZR, NY, 2>(w, k, t);
}

// ------------------------------------------------- runs of Z-string rotations
// ph[c] holds the product of the run's entries of register class c (entry
// factor e^{-i phi} when the thread's part of the parity is even, e^{+i phi}
// when odd); the multiplicative Walsh-Hadamard transform turns it into the
// phase of every register: ph[r] = prod_c (popc(r & c) even ? A_c : conj(A_c)).
template <int NR>
__device__ __forceinline__ void mul_walsh(float2 (&a)[NR]) {
#pragma unroll
  for (int j = 1; j < NR; j <<= 1)
#pragma unroll
    for (int c = 0; c < NR; ++c)
      if (!(c & j)) {
        const float2 x = a[c], y = a[c | j];
        a[c] = cmul(x, y);
        a[c | j] = cmul(x, cconj(y));
      }
}
template <int NR>
__device__ __forceinline__ void add_walsh(float (&a)[NR]) {
#pragma unroll
  for (int j = 1; j < NR; j <<= 1)
#pragma unroll
    for (int c = 0; c < NR; ++c)
      if (!(c & j)) {
        const float x = a[c], y = a[c | j];
        a[c] = x + y;
        a[c | j] = x - y;
      }
}
// entry factor of a run: e^{i phi} at m, conjugated for an even thread parity
__device__ __forceinline__ float2 zrun_factor(const float2* m, u32 gthr, u32 zm) {
  const float2 u = ld(m);
  return (__popc(gthr & zm) & 1u) ? u : cconj(u);
}
template <int NR>
__device__ __forceinline__ void zrun_apply(float2 (&v)[NR], const float2 (&ph)[NR]) {
#pragma unroll
  for (int r = 0; r < NR; ++r) cmul_ip(v[r], ph[r]);
}
template <int NR>
__device__ __forceinline__ void zrun_unapply(float2 (&v)[NR], float2 (&w)[NR], const float2 (&ph)[NR]) {
#pragma unroll
  for (int r = 0; r < NR; ++r) {
    const float2 c = cconj(ph[r]);
    cmul_ip(v[r], c);
    cmul_ip(w[r], c);
  }
}
// t[c] = sum_r (-1)^{popc(r & c)} Im(conj(w_r) v_r)
template <int NR>
__device__ __forceinline__ void zrun_grad(const float2 (&v)[NR], const float2 (&w)[NR], float (&t)[NR]) {
#pragma unroll
  for (int r = 0; r < NR; ++r) t[r] = fmaf(w[r].x, v[r].y, -w[r].y * v[r].x);
  add_walsh<NR>(t);
}
// t[c] = sum_r (-1)^{popc(r & c)} |v_r|^2 (Z-string term partials)
template <int NR>
__device__ __forceinline__ void zmeas_t(const float2 (&v)[NR], float (&t)[NR]) {
#pragma unroll
  for (int r = 0; r < NR; ++r) t[r] = fmaf(v[r].x, v[r].x, v[r].y * v[r].y);
  add_walsh<NR>(t);
}
// w_r += a_r v_r (a_r real: the summed Z-term coefficients of register r)
template <int NR>
__device__ __forceinline__ void zpacc_apply(const float2 (&v)[NR], float2 (&w)[NR], const float (&a)[NR]) {
#pragma unroll
  for (int r = 0; r < NR; ++r) w[r] = make_float2(fmaf(a[r], v[r].x, w[r].x), fmaf(a[r], v[r].y, w[r].y));
}

// Butterfly sum of E values over the NL (< 32) lanes of a small block; lane 0
// writes value e to out[e].
template <int E, int NL>
__device__ __forceinline__ void small_reduce(const float2 (&a)[E], int lane, float2* out) {
  constexpr unsigned FULL = NL >= 32 ? 0xffffffffu : ((1u << NL) - 1u);
#pragma unroll
  for (int e = 0; e < E; ++e) {
    float2 x = a[e];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      if (o < NL) {
        x.x += __shfl_xor_sync(FULL, x.x, o);
        x.y += __shfl_xor_sync(FULL, x.y, o);
      }
    }
    if (lane == 0) out[e] = x;
  }
}

// ----------------------------------------------------------------- reductions
// Sum of one real value over the NL lanes (butterfly: every lane ends with
// the total) -- half the shuffles of the complex form, for rotation
// gradients, which are real.
template <int NL>
__device__ __forceinline__ float warp_sum1(float x) {
  constexpr unsigned FULL = NL >= 32 ? 0xffffffffu : ((1u << NL) - 1u);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
    if (o < NL) x += __shfl_xor_sync(FULL, x, o);
  return x;
}

// Sum E complex values (E a power of two <= 16) over the NL lanes of a warp.
// Returns this lane's total and sets `entry` to the entry it holds, or -1 if
// another lane writes that entry.  Full warps use a transpose-reduce (each
// step keeps half of the entries and sends the other half to the partner
// lane), which costs E + log2(32) shuffle pairs instead of E * log2(32).
template <int E, int NL>
__device__ __forceinline__ float2 warp_reduce(float2 (&a)[E], int lane, int& entry) {
  constexpr unsigned FULL = NL >= 32 ? 0xffffffffu : ((1u << NL) - 1u);
  if (E == 1 || NL < 32) {
    // plain butterfly per entry; lane e returns entry e
    entry = lane < E ? lane : -1;
    float2 mine = czero();
#pragma unroll
    for (int e = 0; e < E; ++e) {
      float2 x = a[e];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        if (o < NL) {
          x.x += __shfl_xor_sync(FULL, x.x, o);
          x.y += __shfl_xor_sync(FULL, x.y, o);
        }
      }
      if (lane == e) mine = x;
    }
    return mine;
  } else {
    // halve the entry set at each step: keep the half selected by the lane
    // bit, send the other half; lane l ends with entry l >> (5 - log2 E)
    constexpr int M = E == 2 ? 1 : E == 4 ? 2 : E == 8 ? 3 : E == 16 ? 4 : 5;
    entry = (lane & ((32 >> M) - 1)) == 0 ? (lane >> (5 - M)) : -1;
    float2 b[E];
#pragma unroll
    for (int e = 0; e < E; ++e) b[e] = a[e];
    int cnt = E;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      if (cnt > 1) {
        const int h = cnt >> 1;
        const bool up = (lane & o) != 0;
#pragma unroll
        for (int e = 0; e < E / 2; ++e) {
          if (e < h) {
            const float2 keep = up ? b[e + h] : b[e];
            const float2 send = up ? b[e] : b[e + h];
            const float rx = __shfl_xor_sync(FULL, send.x, o);
            const float ry = __shfl_xor_sync(FULL, send.y, o);
            b[e] = make_float2(keep.x + rx, keep.y + ry);
          }
        }
        cnt = h;
      } else {
        b[0].x += __shfl_xor_sync(FULL, b[0].x, o);
        b[0].y += __shfl_xor_sync(FULL, b[0].y, o);
      }
    }
    return b[0];
  }
}

}  // namespace tk
