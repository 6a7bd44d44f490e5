// pass.cuh — the tile-pass kernels (templates; instantiated per kernel family
// by pass_inst.cu, dispatched by pass.cu).
//
// One CTA = one tile = the 2^L amplitudes of one circuit that differ only in
// the pass's local index bits.  The CTA reads its tile from HBM once, runs
// every stage of the pass on it and writes it back once.  In a register stage
// each of the 2^(L-R) threads holds the 2^R amplitudes spanned by the stage's
// R register bits; gates on register bits are register-only arithmetic,
// diagonal gates work on any bit through the amplitude's global index, and
// the only shared-memory traffic is one transpose between stages whose
// register bits differ.
//
// Modes (template MODE):
//   FWD  : psi <- G_k ... G_1 psi                       (Circuit.wavefunction)
//   BWD  : adjoint sweep over psi and mu: psi <- G^H psi, gradient slot
//          += mu (x) conj(psi) over the gate's sub-indices, mu <- G^H mu
//   MEAS : Pauli expectations, psi read only
//   PACC : mu += c_t P_t psi, psi read only
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "engine.h"
#include "kernels.h"

namespace tcg {

namespace {

__device__ __forceinline__ uint32_t swz(uint32_t j) {
  return j ^ (((j >> 5) ^ (j >> 10)) & 31u);
}
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
// a * b + c
__device__ __forceinline__ float2 cfma(float2 a, float2 b, float2 c) {
  return make_float2(fmaf(a.x, b.x, fmaf(-a.y, b.y, c.x)),
                     fmaf(a.x, b.y, fmaf(a.y, b.x, c.y)));
}
// a * conj(b) + c
__device__ __forceinline__ float2 cfmac(float2 a, float2 b, float2 c) {
  return make_float2(fmaf(a.x, b.x, fmaf(a.y, b.y, c.x)),
                     fmaf(a.y, b.x, fmaf(-a.x, b.y, c.y)));
}
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
__device__ __forceinline__ float2 czero() { return make_float2(0.f, 0.f); }

__device__ __forceinline__ float2 ldm(const float2* p) {
  return __ldg(reinterpret_cast<const float2*>(p));
}

// v <- p v in place (cross products first, then one FMA per component that
// reads its own old value last: the op loop's register arrays need no copies)
__device__ __forceinline__ void cmul_ip(float2& v, float2 p) {
  const float tx = p.y * v.y, ty = p.y * v.x;
  v.x = fmaf(p.x, v.x, -tx);
  v.y = fmaf(p.x, v.y, ty);
}

// sum of one real value over the first nl lanes (gradients are real)
__device__ __forceinline__ float warp_sum1(float v, int nl) {
  const unsigned mask = nl >= 32 ? 0xffffffffu : ((1u << nl) - 1u);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
    if (o < nl) v += __shfl_xor_sync(mask, v, o);
  return v;
}

// Sum over the lanes of a warp; blocks smaller than a warp (tiny tiles) use
// only their nl = blockDim.x lanes.
__device__ __forceinline__ float2 warp_sum(float2 v, int nl) {
  const unsigned mask = nl >= 32 ? 0xffffffffu : ((1u << nl) - 1u);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    if (o < nl) {
      v.x += __shfl_xor_sync(mask, v.x, o);
      v.y += __shfl_xor_sync(mask, v.y, o);
    }
  }
  return v;
}

// ---------------------------------------------------------------- dense 1q
template <int R, int P>
__device__ __forceinline__ void dense1(float2 (&v)[1 << R], const float2 (&m)[4]) {
#pragma unroll
  for (int r = 0; r < (1 << R); ++r) {
    if (r & (1 << P)) continue;
    const int r1 = r | (1 << P);
    const float2 x0 = v[r], x1 = v[r1];
    v[r] = cfma(m[0], x0, cmul(m[1], x1));
    v[r1] = cfma(m[2], x0, cmul(m[3], x1));
  }
}

// adjoint step for a 1q gate: a = M^H
template <int R, int P, bool GRAD>
__device__ __forceinline__ void dense1_bwd(float2 (&v)[1 << R], float2 (&w)[1 << R],
                                           const float2 (&a)[4], float2 (&acc)[16]) {
#pragma unroll
  for (int r = 0; r < (1 << R); ++r) {
    if (r & (1 << P)) continue;
    const int r1 = r | (1 << P);
    const float2 x0 = v[r], x1 = v[r1];
    const float2 y0 = cfma(a[0], x0, cmul(a[1], x1));
    const float2 y1 = cfma(a[2], x0, cmul(a[3], x1));
    v[r] = y0;
    v[r1] = y1;
    const float2 u0 = w[r], u1 = w[r1];
    if (GRAD) {
      acc[0] = cfmac(u0, y0, acc[0]);
      acc[1] = cfmac(u0, y1, acc[1]);
      acc[2] = cfmac(u1, y0, acc[2]);
      acc[3] = cfmac(u1, y1, acc[3]);
    }
    w[r] = cfma(a[0], u0, cmul(a[1], u1));
    w[r1] = cfma(a[2], u0, cmul(a[3], u1));
  }
}

// ---------------------------------------------------------------- dense 2q
template <int R, int P0, int P1>
__device__ __forceinline__ void dense2(float2 (&v)[1 << R], const float2 (&m)[16]) {
#pragma unroll
  for (int r = 0; r < (1 << R); ++r) {
    if (r & ((1 << P0) | (1 << P1))) continue;
    const int i0 = r, i1 = r | (1 << P1), i2 = r | (1 << P0), i3 = r | (1 << P0) | (1 << P1);
    const float2 x0 = v[i0], x1 = v[i1], x2 = v[i2], x3 = v[i3];
    v[i0] = cfma(m[0], x0, cfma(m[1], x1, cfma(m[2], x2, cmul(m[3], x3))));
    v[i1] = cfma(m[4], x0, cfma(m[5], x1, cfma(m[6], x2, cmul(m[7], x3))));
    v[i2] = cfma(m[8], x0, cfma(m[9], x1, cfma(m[10], x2, cmul(m[11], x3))));
    v[i3] = cfma(m[12], x0, cfma(m[13], x1, cfma(m[14], x2, cmul(m[15], x3))));
  }
}

template <int R, int P0, int P1, bool GRAD>
__device__ __forceinline__ void dense2_bwd(float2 (&v)[1 << R], float2 (&w)[1 << R],
                                           const float2 (&a)[16], float2 (&acc)[16]) {
#pragma unroll
  for (int r = 0; r < (1 << R); ++r) {
    if (r & ((1 << P0) | (1 << P1))) continue;
    const int idx[4] = {r, r | (1 << P1), r | (1 << P0), r | (1 << P0) | (1 << P1)};
    float2 y[4], u[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      y[i] = cfma(a[4 * i + 0], v[idx[0]],
                  cfma(a[4 * i + 1], v[idx[1]],
                       cfma(a[4 * i + 2], v[idx[2]], cmul(a[4 * i + 3], v[idx[3]]))));
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      v[idx[i]] = y[i];
      u[i] = w[idx[i]];
    }
    if (GRAD) {
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[4 * i + j] = cfmac(u[i], y[j], acc[4 * i + j]);
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      w[idx[i]] = cfma(a[4 * i + 0], u[0],
                       cfma(a[4 * i + 1], u[1], cfma(a[4 * i + 2], u[2], cmul(a[4 * i + 3], u[3]))));
    }
  }
}

// switch helpers --------------------------------------------------------------
template <int R>
__device__ __forceinline__ void dispatch_dense1(int p, float2 (&v)[1 << R], const float2 (&m)[4]) {
  switch (p) {
    case 0: dense1<R, 0>(v, m); break;
    case 1: if (R > 1) dense1<R, (R > 1 ? 1 : 0)>(v, m); break;
    case 2: if (R > 2) dense1<R, (R > 2 ? 2 : 0)>(v, m); break;
    case 3: if (R > 3) dense1<R, (R > 3 ? 3 : 0)>(v, m); break;
    case 4: if (R > 4) dense1<R, (R > 4 ? 4 : 0)>(v, m); break;
    default: break;
  }
}

template <int R, bool G>
__device__ __forceinline__ void dispatch_dense1_bwd(int p, float2 (&v)[1 << R], float2 (&w)[1 << R],
                                                    const float2 (&a)[4], float2 (&acc)[16]) {
  switch (p) {
    case 0: dense1_bwd<R, 0, G>(v, w, a, acc); break;
    case 1: if (R > 1) dense1_bwd<R, (R > 1 ? 1 : 0), G>(v, w, a, acc); break;
    case 2: if (R > 2) dense1_bwd<R, (R > 2 ? 2 : 0), G>(v, w, a, acc); break;
    case 3: if (R > 3) dense1_bwd<R, (R > 3 ? 3 : 0), G>(v, w, a, acc); break;
    case 4: if (R > 4) dense1_bwd<R, (R > 4 ? 4 : 0), G>(v, w, a, acc); break;
    default: break;
  }
}

template <int R>
__device__ __forceinline__ void dispatch_dense2(int p0, int p1, float2 (&v)[1 << R],
                                                const float2 (&m)[16]) {
#define TCG_D2(P0, P1)                                                               \
  case (P0) * 8 + (P1):                                                              \
    if ((P0) < R && (P1) < R) dense2<R, ((P0) < R ? (P0) : 0), ((P1) < R ? (P1) : 1)>(v, m); \
    break;
  switch (p0 * 8 + p1) {
    TCG_D2(0, 1) TCG_D2(0, 2) TCG_D2(0, 3) TCG_D2(0, 4)
    TCG_D2(1, 0) TCG_D2(1, 2) TCG_D2(1, 3) TCG_D2(1, 4)
    TCG_D2(2, 0) TCG_D2(2, 1) TCG_D2(2, 3) TCG_D2(2, 4)
    TCG_D2(3, 0) TCG_D2(3, 1) TCG_D2(3, 2) TCG_D2(3, 4)
    TCG_D2(4, 0) TCG_D2(4, 1) TCG_D2(4, 2) TCG_D2(4, 3)
    default: break;
  }
#undef TCG_D2
}

template <int R, bool G>
__device__ __forceinline__ void dispatch_dense2_bwd(int p0, int p1, float2 (&v)[1 << R],
                                                    float2 (&w)[1 << R], const float2 (&a)[16],
                                                    float2 (&acc)[16]) {
#define TCG_D2B(P0, P1)                                                                 \
  case (P0) * 8 + (P1):                                                                 \
    if ((P0) < R && (P1) < R)                                                           \
      dense2_bwd<R, ((P0) < R ? (P0) : 0), ((P1) < R ? (P1) : 1), G>(v, w, a, acc);    \
    break;
  switch (p0 * 8 + p1) {
    TCG_D2B(0, 1) TCG_D2B(0, 2) TCG_D2B(0, 3) TCG_D2B(0, 4)
    TCG_D2B(1, 0) TCG_D2B(1, 2) TCG_D2B(1, 3) TCG_D2B(1, 4)
    TCG_D2B(2, 0) TCG_D2B(2, 1) TCG_D2B(2, 3) TCG_D2B(2, 4)
    TCG_D2B(3, 0) TCG_D2B(3, 1) TCG_D2B(3, 2) TCG_D2B(3, 4)
    TCG_D2B(4, 0) TCG_D2B(4, 1) TCG_D2B(4, 2) TCG_D2B(4, 3)
    default: break;
  }
#undef TCG_D2B
}

// ---------------------------------------------------------------- Pauli terms
// w[r] += cf * s(r) * v[r ^ X]   (cf complex, includes (-i)^nY and the coefficient)
template <int R, int X>
__device__ __forceinline__ void pacc_x(const float2 (&v)[1 << R], float2 (&w)[1 << R], float2 cf,
                                       int sbase, int zr) {
#pragma unroll
  for (int r = 0; r < (1 << R); ++r) {
    const int s = (sbase ^ __popc(r & zr)) & 1;
    const float2 c = s ? make_float2(-cf.x, -cf.y) : cf;
    w[r] = cfma(c, v[r ^ X], w[r]);
  }
}

// Terms reaching the register path have at most two X/Y bits (the planner
// sends wider ones to the plain kernel), so 16 compiled patterns cover them.
#define TCG_XCASES(M)                                                      \
  M(0) M(1) M(2) M(4) M(8) M(16) M(3) M(5) M(9) M(17) M(6) M(10) M(18) M(12) \
  M(20) M(24)

// acc = sum_r conj(v[r]) s(r) v[r ^ x], s(r) = (-1)^(sbase ^ popc(r & zr)).
// The measurement form: t[r] = v[r ^ x] built by one conditional exchange
// per register bit of x, then one pass over compile-time indices.  (A switch
// over the 16 compiled patterns, as the accumulation below uses, gave the
// measurement kernels a 1 KiB local-memory stack frame, and the uneven
// batch's measurement sweep 4.8x its algorithmic DRAM bytes, mostly writes.)
template <int R>
__device__ __forceinline__ float2 dispatch_expect(int x, const float2 (&v)[1 << R], int sbase, int zr) {
  float2 t[1 << R];
#pragma unroll
  for (int r = 0; r < (1 << R); ++r) t[r] = v[r];
#pragma unroll
  for (int j = 0; j < R; ++j) {
    const bool f = (x >> j) & 1;
#pragma unroll
    for (int r = 0; r < (1 << R); ++r)
      if (!((r >> j) & 1)) {
        const float2 a = t[r], b = t[r | (1 << j)];
        t[r] = f ? b : a;
        t[r | (1 << j)] = f ? a : b;
      }
  }
  float2 acc = czero();
#pragma unroll
  for (int r = 0; r < (1 << R); ++r) {
    const float2 c = make_float2(fmaf(v[r].x, t[r].x, v[r].y * t[r].y), fmaf(v[r].x, t[r].y, -v[r].y * t[r].x));
    const int s = (sbase ^ __popc(r & zr)) & 1;
    acc.x += s ? -c.x : c.x;
    acc.y += s ? -c.y : c.y;
  }
  return acc;
}

template <int R>
__device__ __forceinline__ void dispatch_pacc(int x, const float2 (&v)[1 << R], float2 (&w)[1 << R],
                                              float2 cf, int sbase, int zr) {
#define TCG_PA(XX) case XX: if ((XX) < (1 << R)) pacc_x<R, ((XX) < (1 << R) ? (XX) : 0)>(v, w, cf, sbase, zr); break;
  switch (x) {
    TCG_XCASES(TCG_PA)
    default: break;
  }
#undef TCG_PA
}

// Pauli rotation on registers: v[r] <- c v[r] + (-1)^{popc(r & zr)} q v[r ^ X]
// (q = -i s (-i)^nY with the thread's sign folded in; the adjoint passes -q).
// q is purely imaginary (QIM, even nY) or purely real, so it is carried as
// one real number qv and the update costs four operations per amplitude.
template <int R, int X, bool QIM>
__device__ __forceinline__ void prot_rt(float2 (&v)[1 << R], float c, float qv, int zr) {
  // cross terms into temporaries first, then one FMA per component reading
  // its own old value last, so results can stay in the registers they
  // replace (no copies at the end of the op)
#pragma unroll
  for (int r = 0; r < (1 << R); ++r) {
    const float qr = (__popc(r & zr) & 1) ? -qv : qv;
    if (X == 0) {
      if (QIM) {
        const float px = qr * v[r].y, py = qr * v[r].x;
        v[r].x = fmaf(c, v[r].x, -px);
        v[r].y = fmaf(c, v[r].y, py);
      } else {
        const float f = c + qr;
        v[r].x = f * v[r].x;
        v[r].y = f * v[r].y;
      }
    } else {
      const int r2 = r ^ X;
      if (r2 < r) continue;
      const float q2 = (__popc(r2 & zr) & 1) ? -qv : qv;
      if (QIM) {
        const float pax = qr * v[r2].y, pay = qr * v[r2].x;
        const float pbx = q2 * v[r].y, pby = q2 * v[r].x;
        v[r].x = fmaf(c, v[r].x, -pax);
        v[r].y = fmaf(c, v[r].y, pay);
        v[r2].x = fmaf(c, v[r2].x, -pbx);
        v[r2].y = fmaf(c, v[r2].y, pby);
      } else {
        const float pax = qr * v[r2].x, pay = qr * v[r2].y;
        const float pbx = q2 * v[r].x, pby = q2 * v[r].y;
        v[r].x = fmaf(c, v[r].x, pax);
        v[r].y = fmaf(c, v[r].y, pay);
        v[r2].x = fmaf(c, v[r2].x, pbx);
        v[r2].y = fmaf(c, v[r2].y, pby);
      }
    }
  }
}

// Im (IMZ) or Re of sum_r (-1)^{popc(r & zr)} conj(w[r]) v[r ^ X]; Z0: zr is
// known to be 0 (no Z/Y factor in the registers: rx, ry, rxx, ...), so no
// per-register sign is computed.  Four partial sums keep the FMA chains short.
template <int R, int X, bool IMZ, bool Z0>
__device__ __forceinline__ float prot_dot(const float2 (&v)[1 << R], const float2 (&w)[1 << R], int zr) {
  float z[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
  for (int r = 0; r < (1 << R); ++r) {
    const float2 t = v[r ^ X];
    const bool neg = Z0 ? false : (__popc(r & zr) & 1) != 0;
    const float wx = neg ? -w[r].x : w[r].x;
    const float wy = neg ? -w[r].y : w[r].y;
    if (IMZ) {
      z[r & 3] = fmaf(wx, t.y, z[r & 3]);
      z[r & 3] = fmaf(-wy, t.x, z[r & 3]);
    } else {
      z[r & 3] = fmaf(wx, t.x, z[r & 3]);
      z[r & 3] = fmaf(wy, t.y, z[r & 3]);
    }
  }
  return (z[0] + z[1]) + (z[2] + z[3]);
}

#define TCG_X16(M) M(0) M(1) M(2) M(3) M(4) M(5) M(6) M(7) M(8) M(9) M(10) M(11) M(12) M(13) M(14) M(15)

// Shear form of the same rotation (a rotation by (c, s) as three in-place
// shears x -= k y, y += t x, x -= k y with k = s / (1 + c): three FMAs per
// component pair instead of four operations per amplitude).  A rotation with
// c < 0 is taken as the negative of its c >= 0 partner; gshear_params
// returns 1 then, and the tile carries the sign until it is stored.
__device__ __forceinline__ uint32_t gshear_params(float c, float q, float& k, float& t) {
  const uint32_t neg = c < 0.f ? 1u : 0u;
  t = neg ? -q : q;
  k = t * __frcp_rn(1.f + fabsf(c));
  return neg;
}
template <int STEP>
__device__ __forceinline__ void gshear_step(float& x, float& y, float k, float t, bool flip) {
  if (STEP == 1) y = fmaf(flip ? -t : t, x, y);
  else x = fmaf(flip ? k : -k, y, x);
}
// one of the three shear sweeps over every register pair of the rotation
// (Z0: no Z/Y factor in the registers, so no per-register sign)
template <int R, int X, bool QIM, bool Z0, int STEP>
__device__ __forceinline__ void gshear_sweep(float2 (&v)[1 << R], float k, float t, int zr) {
#pragma unroll
  for (int r = 0; r < (1 << R); ++r) {
    const bool sr = Z0 ? false : (__popc(r & zr) & 1) != 0;
    if (X == 0) {
      gshear_step<STEP>(v[r].x, v[r].y, k, t, sr);
    } else {
      const int r2 = r ^ X;
      if (r2 < r) continue;
      if (QIM) {
        gshear_step<STEP>(v[r].x, v[r2].y, k, t, sr);
        gshear_step<STEP>(v[r].y, v[r2].x, k, t, !sr);
      } else {
        gshear_step<STEP>(v[r].x, v[r2].x, k, t, !sr);
        gshear_step<STEP>(v[r].y, v[r2].y, k, t, !sr);
      }
    }
  }
}
template <int R, int X, bool QIM, bool Z0>
__device__ __forceinline__ void gshear_rot(float2 (&v)[1 << R], float k, float t, int zr) {
  gshear_sweep<R, X, QIM, Z0, 0>(v, k, t, zr);
  gshear_sweep<R, X, QIM, Z0, 1>(v, k, t, zr);
  gshear_sweep<R, X, QIM, Z0, 2>(v, k, t, zr);
}
// psi and mu together: the sweeps interleaved for independent FMAs
template <int R, int X, bool QIM, bool Z0>
__device__ __forceinline__ void gshear_rot2(float2 (&v)[1 << R], float2 (&w)[1 << R], float k, float t, int zr) {
  gshear_sweep<R, X, QIM, Z0, 0>(v, k, t, zr);
  gshear_sweep<R, X, QIM, Z0, 0>(w, k, t, zr);
  gshear_sweep<R, X, QIM, Z0, 1>(v, k, t, zr);
  gshear_sweep<R, X, QIM, Z0, 1>(w, k, t, zr);
  gshear_sweep<R, X, QIM, Z0, 2>(v, k, t, zr);
  gshear_sweep<R, X, QIM, Z0, 2>(w, k, t, zr);
}
// X = the register-position mask of the rotation's X/Y factors (< 2^R)
#define TCG_XC(XX) ((XX) < (1 << R) ? (XX) : 0)
template <int R, bool QIM, bool Z0>
__device__ __forceinline__ void dispatch_gshear_x(int x, float2 (&v)[1 << R], float k, float t, int zr) {
#define TCG_GS(XX) case XX: if ((XX) < (1 << R)) gshear_rot<R, TCG_XC(XX), QIM, Z0>(v, k, t, zr); break;
  switch (x) {
    TCG_X16(TCG_GS)
    default: break;
  }
#undef TCG_GS
}
template <int R, bool QIM, bool Z0>
__device__ __forceinline__ void dispatch_gshear2_x(int x, float2 (&v)[1 << R], float2 (&w)[1 << R], float k, float t,
                                                   int zr) {
#define TCG_GS(XX) case XX: if ((XX) < (1 << R)) gshear_rot2<R, TCG_XC(XX), QIM, Z0>(v, w, k, t, zr); break;
  switch (x) {
    TCG_X16(TCG_GS)
    default: break;
  }
#undef TCG_GS
}
template <int R>
__device__ __forceinline__ void dispatch_gshear(int x, bool qim, float2 (&v)[1 << R], float k, float t, int zr) {
  if (qim) {
    if (zr == 0) dispatch_gshear_x<R, true, true>(x, v, k, t, zr);
    else dispatch_gshear_x<R, true, false>(x, v, k, t, zr);
  } else {
    if (zr == 0) dispatch_gshear_x<R, false, true>(x, v, k, t, zr);
    else dispatch_gshear_x<R, false, false>(x, v, k, t, zr);
  }
}
template <int R>
__device__ __forceinline__ void dispatch_gshear2(int x, bool qim, float2 (&v)[1 << R], float2 (&w)[1 << R], float k,
                                                 float t, int zr) {
  if (qim) {
    if (zr == 0) dispatch_gshear2_x<R, true, true>(x, v, w, k, t, zr);
    else dispatch_gshear2_x<R, true, false>(x, v, w, k, t, zr);
  } else {
    if (zr == 0) dispatch_gshear2_x<R, false, true>(x, v, w, k, t, zr);
    else dispatch_gshear2_x<R, false, false>(x, v, w, k, t, zr);
  }
}

template <int R>
__device__ __forceinline__ void dispatch_prot(int x, float2 (&v)[1 << R], float c, float qv, int zr, bool qim) {
  if (qim) {
#define TCG_PR(XX) case XX: if ((XX) < (1 << R)) prot_rt<R, ((XX) < (1 << R) ? (XX) : 0), true>(v, c, qv, zr); break;
    switch (x) {
      TCG_X16(TCG_PR)
      default: break;
    }
#undef TCG_PR
  } else {
#define TCG_PR(XX) case XX: if ((XX) < (1 << R)) prot_rt<R, ((XX) < (1 << R) ? (XX) : 0), false>(v, c, qv, zr); break;
    switch (x) {
      TCG_X16(TCG_PR)
      default: break;
    }
#undef TCG_PR
  }
}

template <int R, bool IMZ, bool Z0>
__device__ __forceinline__ float dispatch_prot_dot_x(int x, const float2 (&v)[1 << R], const float2 (&w)[1 << R],
                                                     int zr) {
  float z = 0.f;
#define TCG_PD(XX) case XX: if ((XX) < (1 << R)) z = prot_dot<R, TCG_XC(XX), IMZ, Z0>(v, w, zr); break;
  switch (x) {
    TCG_X16(TCG_PD)
    default: break;
  }
#undef TCG_PD
  return z;
}
template <int R>
__device__ __forceinline__ float dispatch_prot_dot(int x, const float2 (&v)[1 << R], const float2 (&w)[1 << R],
                                                   int zr, bool imz) {
  if (imz) return zr == 0 ? dispatch_prot_dot_x<R, true, true>(x, v, w, zr) : dispatch_prot_dot_x<R, true, false>(x, v, w, zr);
  return zr == 0 ? dispatch_prot_dot_x<R, false, true>(x, v, w, zr) : dispatch_prot_dot_x<R, false, false>(x, v, w, zr);
}

// (-i)^nY
__device__ __forceinline__ float2 ypow(int nY) {
  switch (nY & 3) {
    case 0: return make_float2(1.f, 0.f);
    case 1: return make_float2(0.f, -1.f);
    case 2: return make_float2(-1.f, 0.f);
    default: return make_float2(0.f, 1.f);
  }
}

// ---------------------------------------------------------------- smem dense k
template <int K>
__device__ void denseK_smem(float2* tile, int L, const int* tb, const float2* m, bool adj,
                            int tid, int nthreads) {
  constexpr int D = 1 << K;
  const uint32_t ngroups = 1u << (L - K);
  // sorted tile bits for zero insertion
  int srt[K];
#pragma unroll
  for (int i = 0; i < K; ++i) srt[i] = tb[i];
#pragma unroll
  for (int i = 0; i < K; ++i)
#pragma unroll
    for (int j = 0; j + 1 < K - i; ++j)
      if (srt[j] > srt[j + 1]) { int t = srt[j]; srt[j] = srt[j + 1]; srt[j + 1] = t; }
  for (uint32_t g = tid; g < ngroups; g += nthreads) {
    uint32_t j0 = g;
#pragma unroll
    for (int i = 0; i < K; ++i) {
      const uint32_t lowm = (1u << srt[i]) - 1u;
      j0 = ((j0 & ~lowm) << 1) | (j0 & lowm);
    }
    float2 x[D];
#pragma unroll
    for (int s = 0; s < D; ++s) {
      uint32_t j = j0;
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
        const float2 e = adj ? cconj(ldm(m + t * D + s)) : ldm(m + s * D + t);
        y = cfma(e, x[t], y);
      }
      uint32_t j = j0;
#pragma unroll
      for (int i = 0; i < K; ++i)
        if ((s >> (K - 1 - i)) & 1) j |= 1u << tb[i];
      tile[swz(j)] = y;
    }
  }
}

__device__ void dispatch_denseK(int k, float2* tile, int L, const int* tb, const float2* m, bool adj,
                                int tid, int nthreads) {
  switch (k) {
    case 1: denseK_smem<1>(tile, L, tb, m, adj, tid, nthreads); break;
    case 2: denseK_smem<2>(tile, L, tb, m, adj, tid, nthreads); break;
    case 3: denseK_smem<3>(tile, L, tb, m, adj, tid, nthreads); break;
    case 4: denseK_smem<4>(tile, L, tb, m, adj, tid, nthreads); break;
    case 5: denseK_smem<5>(tile, L, tb, m, adj, tid, nthreads); break;
    case 6: denseK_smem<6>(tile, L, tb, m, adj, tid, nthreads); break;
    default: break;
  }
}

// ------------------------------------------------- runs of Z-string rotations
// A run of commuting rotations exp(-i phi_e Z_{S_e}) multiplies amplitude x
// by prod_e e^{-i phi_e s_e(x)}, s_e = (-1)^{parity(x & S_e)}.  Per thread the
// parity splits into a thread part and a register part popc(r & c_e), c_e the
// entry's register mask ("class").  Folding each entry into its class,
// A_c = prod_{c_e = c} B_e, the phase of register r is
// prod_c (popc(r & c) even ? A_c : conj(A_c)): a multiplicative Walsh-Hadamard
// transform of A, computed with 2^R * R complex products per thread.
// Run-time class index into a register array: a switch (one indexed branch
// and one update) instead of 2^R predicated updates.
#define TCG_CASES16(M) M(0) M(1) M(2) M(3) M(4) M(5) M(6) M(7) M(8) M(9) M(10) M(11) M(12) M(13) M(14) M(15)
template <int R>
__device__ __forceinline__ void class_mul(float2 (&a)[1 << R], int c, float2 u) {
  switch (c) {
#define TCG_CM(I) case I: if ((I) < (1 << R)) a[(I) < (1 << R) ? (I) : 0] = cmul(a[(I) < (1 << R) ? (I) : 0], u); break;
    TCG_CASES16(TCG_CM)
#undef TCG_CM
    default: break;
  }
}
template <int R>
__device__ __forceinline__ void class_add(float (&a)[1 << R], int c, float x) {
  switch (c) {
#define TCG_CA(I) case I: if ((I) < (1 << R)) a[(I) < (1 << R) ? (I) : 0] += x; break;
    TCG_CASES16(TCG_CA)
#undef TCG_CA
    default: break;
  }
}
template <int R>
__device__ __forceinline__ void mul_walsh(float2 (&a)[1 << R]) {
#pragma unroll
  for (int j = 0; j < R; ++j)
#pragma unroll
    for (int c = 0; c < (1 << R); ++c)
      if (!((c >> j) & 1)) {
        const float2 x = a[c], y = a[c | (1 << j)];
        a[c] = cmul(x, y);
        a[c | (1 << j)] = cmul(x, cconj(y));
      }
}
template <int R>
__device__ __forceinline__ void add_walsh(float (&a)[1 << R]) {
#pragma unroll
  for (int j = 0; j < R; ++j)
#pragma unroll
    for (int c = 0; c < (1 << R); ++c)
      if (!((c >> j) & 1)) {
        const float x = a[c], y = a[c | (1 << j)];
        a[c] = x + y;
        a[c | (1 << j)] = x - y;
      }
}
template <int R>
__device__ __forceinline__ float class_pick(const float (&a)[1 << R], int c) {
  switch (c) {
#define TCG_CP(I) case I: return a[(I) < (1 << R) ? (I) : 0];
    TCG_CASES16(TCG_CP)
#undef TCG_CP
    default: return 0.f;
  }
}

// Per-entry sums of a Z-run (measured <Z_S> partials or rotation-angle
// gradients) written to the entries' slots of this warp.  Value of entry e:
// the Walsh coefficient t[class_e], negated for an odd thread parity.  Full
// warps reduce eight entries at once by a transpose-reduce (each butterfly
// step keeps half of the values and sends the other half to the partner
// lane; lane l ends with entry l >> 2): 9 shuffles per eight entries instead
// of 40.  Entries without a slot are skipped.
template <int R>
__device__ __forceinline__ void zrun_slot_sums(const float (&t)[1 << R], const ZEnt* __restrict__ ze, int k,
                                               uint32_t gthr, int nl, int lane, float2* wslots) {
  if (nl < 32) {
    for (int e = 0; e < k; ++e) {
      const ZEnt z = ze[e];
      if (z.slot < 0) continue;
      float g = class_pick<R>(t, z.zreg);
      if (__popc(gthr & z.zmask) & 1) g = -g;
      const float s = warp_sum1(g, nl);
      if (lane == 0) wslots[z.slot] = make_float2(s, 0.f);
    }
    return;
  }
  for (int e0 = 0; e0 < k; e0 += 8) {
    float b[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      float x = 0.f;
      if (e0 + q < k) {
        const ZEnt z = ze[e0 + q];
        if (z.slot >= 0) {
          x = class_pick<R>(t, z.zreg);
          if (__popc(gthr & z.zmask) & 1) x = -x;
        }
      }
      b[q] = x;
    }
#pragma unroll
    for (int o = 16, h = 4; o >= 4; o >>= 1, h >>= 1) {
      const bool up = (lane & o) != 0;
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        if (e < h) {
          const float keep = up ? b[e + h] : b[e];
          const float send = up ? b[e] : b[e + h];
          b[e] = keep + __shfl_xor_sync(0xffffffffu, send, o);
        }
      }
    }
    float v = b[0];
    v += __shfl_xor_sync(0xffffffffu, v, 2);
    v += __shfl_xor_sync(0xffffffffu, v, 1);
    const int my = e0 + (lane >> 2);
    if ((lane & 3) == 0 && my < k) {
      const ZEnt z = ze[my];
      if (z.slot >= 0) wslots[z.slot] = make_float2(v, 0.f);
    }
  }
}

// ------------------------------------------------------------------ tile I/O
__device__ __forceinline__ void tile_load_smem(float2* sm, const float2* __restrict__ src, uint32_t base,
                                               const uint32_t* runs, int L, int tid, int nthreads) {
  const uint32_t half = 1u << (L - 1);
  for (uint32_t i = tid; i < half; i += nthreads) {
    const uint32_t j = 2 * i;
    const uint32_t off = __ldg(runs + (j >> kLo)) | (j & ((1u << kLo) - 1));
    const float4 q = __ldcg(reinterpret_cast<const float4*>(src + (base | off)));
    sm[swz(j)] = make_float2(q.x, q.y);
    sm[swz(j + 1)] = make_float2(q.z, q.w);
  }
}

__device__ __forceinline__ void tile_store_smem(const float2* sm, float2* __restrict__ dst, uint32_t base,
                                                const uint32_t* runs, int L, int tid, int nthreads) {
  const uint32_t half = 1u << (L - 1);
  for (uint32_t i = tid; i < half; i += nthreads) {
    const uint32_t j = 2 * i;
    const uint32_t off = __ldg(runs + (j >> kLo)) | (j & ((1u << kLo) - 1));
    const float2 a = sm[swz(j)], b = sm[swz(j + 1)];
    *reinterpret_cast<float4*>(dst + (base | off)) = make_float4(a.x, a.y, b.x, b.y);
  }
}

struct Layout {
  uint32_t jt;      // tile offset of this thread's group
  uint32_t gt;      // global offset (local bits) of this thread's group
  uint32_t rt[6];   // tile offset of register bit i
  uint32_t rg[6];   // global offset of register bit i
};

template <int R>
__device__ __forceinline__ void make_layout(Layout& ly, const DevStage& S, const DevPass& P, int tid) {
  ly.jt = 0;
  ly.gt = 0;
  for (int i = 0; i < S.nthread_bits; ++i) {
    if ((tid >> i) & 1) {
      const int t = S.thr_tile[i];
      ly.jt |= 1u << t;
      ly.gt |= 1u << P.lbits[t];
    }
  }
#pragma unroll
  for (int i = 0; i < R; ++i) {
    const int t = S.reg_tile[i];
    ly.rt[i] = 1u << t;
    ly.rg[i] = 1u << P.lbits[t];
  }
}

template <int R>
__device__ __forceinline__ uint32_t roff(const Layout& ly, int r, bool global) {
  uint32_t o = 0;
#pragma unroll
  for (int i = 0; i < R; ++i)
    if ((r >> i) & 1) o |= global ? ly.rg[i] : ly.rt[i];
  return o;
}

template <int R>
__device__ __forceinline__ void regs_from_smem(float2 (&v)[1 << R], const float2* sm, const Layout& ly) {
#pragma unroll
  for (int r = 0; r < (1 << R); ++r) v[r] = sm[swz(ly.jt | roff<R>(ly, r, false))];
}
template <int R>
__device__ __forceinline__ void regs_to_smem(const float2 (&v)[1 << R], float2* sm, const Layout& ly) {
#pragma unroll
  for (int r = 0; r < (1 << R); ++r) sm[swz(ly.jt | roff<R>(ly, r, false))] = v[r];
}
template <int R>
__device__ __forceinline__ void regs_from_global(float2 (&v)[1 << R], const float2* __restrict__ src,
                                                 uint32_t base, const Layout& ly) {
#pragma unroll
  for (int r = 0; r < (1 << R); ++r) v[r] = __ldcg(src + (base | ly.gt | roff<R>(ly, r, true)));
}
template <int R>
__device__ __forceinline__ void regs_to_global(const float2 (&v)[1 << R], float2* __restrict__ dst,
                                               uint32_t base, const Layout& ly) {
#pragma unroll
  for (int r = 0; r < (1 << R); ++r) dst[base | ly.gt | roff<R>(ly, r, true)] = v[r];
}

__device__ __forceinline__ bool same_layout(const DevStage& a, const DevStage& b) {
  if (a.smem_stage || b.smem_stage || a.R != b.R || a.nthread_bits != b.nthread_bits) return false;
  for (int i = 0; i < a.R; ++i)
    if (a.reg_tile[i] != b.reg_tile[i]) return false;
  for (int i = 0; i < a.nthread_bits; ++i)
    if (a.thr_tile[i] != b.thr_tile[i]) return false;
  return true;
}

}  // namespace

// ============================================================================
// One tile of one pass: state loads go through L2 (ld.global.cg) so that a
// persistent launch may read tiles written earlier in the same launch.
// LITE drops the shared-memory stages, 2-qubit dense and diagonal ops: the
// body of programs made of 1-qubit dense gates, Pauli rotations, Z-rotation
// runs and Pauli terms needs half the registers.
constexpr int kKtMax = 256;  // ops per pass with precomputed shear parameters

template <int MODE, int R, bool LITE = false>
__device__ __forceinline__ void pass_tile(const PassArgs& A, uint32_t tile, int64_t b, uint32_t ntiles,
                                          float2* smem_raw) {
  constexpr int NR = 1 << R;
  constexpr bool HAS_MU = (MODE == MODE_BWD || MODE == MODE_PACC);
  constexpr bool STORE_PSI = (MODE == MODE_FWD || MODE == MODE_BWD);
  constexpr bool STORE_MU = HAS_MU;

  const DevPass& P = A.prog.passes[A.pass];
  const int L = P.L;
  const int tid = threadIdx.x;
  const int nthreads = blockDim.x;
  const int warp = tid >> 5;
  const int lane = tid & 31;
  const int nwarps = (nthreads + 31) >> 5;
  const int nl = nthreads < 32 ? nthreads : 32;

  float2* sm_psi = smem_raw;
  float2* sm_mu = smem_raw + (HAS_MU ? (1u << L) : 0u);
  float2* sm_slot = smem_raw + (HAS_MU ? 2u : 1u) * (1u << L);

  uint32_t base = 0;
  for (int i = 0; i < P.nnonlocal; ++i)
    if ((tile >> i) & 1u) base |= 1u << P.nlbits[i];

  const size_t state_len = size_t(1) << A.n;
  float2* psi = A.psi + b * state_len;
  float2* mu = HAS_MU ? (A.mu + b * state_len) : nullptr;
  const float2* mats = A.mats ? (A.mats + b * A.mat_stride) : nullptr;
  const uint32_t* runs = A.prog.runs + P.runs_off;
  // first pass of a sweep: the input state may sit elsewhere (psi_in), and
  // an accumulation may start mu at zero instead of reading it
  const float2* psi_ld = A.psi_in ? (A.psi_in + b * A.in_stride) : psi;
  const bool mu_zero = HAS_MU && A.mu_zero != 0;
  auto load_mu_smem = [&]() {
    if (mu_zero) {
      for (uint32_t j = tid; j < (1u << L); j += nthreads) sm_mu[j] = make_float2(0.f, 0.f);
    } else {
      tile_load_smem(sm_mu, mu, base, runs, L, tid, nthreads);
    }
  };

  float2 v[NR];
  float2 w[NR];  // mu registers; dead (and removed) in modes without mu
  uint32_t pneg = 0;  // the tile holds the negative of its true values

  // Shear parameters of the pass's Pauli rotations, computed once per tile
  // by the whole CTA instead of a reciprocal per thread and rotation: op
  // (kt_ob + i) has (k, t) at s_kt[i] for an even thread parity (an odd one
  // negates both); the c < 0 cases' tile sign goes straight into pneg.  Ops
  // past the table compute their own.
  __shared__ float2 s_kt[kKtMax];
  __shared__ uint32_t s_kneg;
  int kt_ob = 0, kt_n = 0;
  if ((MODE == MODE_FWD || MODE == MODE_BWD) && P.stage_end > P.stage_begin) {
    kt_ob = A.prog.stages[P.stage_begin].op_begin;
    kt_n = A.prog.stages[P.stage_end - 1].op_end - kt_ob;
    if (kt_n > kKtMax) kt_n = kKtMax;
    if (kt_n < 0) kt_n = 0;
    if (tid == 0) s_kneg = 0u;
    __syncthreads();
    for (int i = tid; i < kt_n; i += nthreads) {
      const DevOp& op = A.prog.ops[kt_ob + i];
      if (op.kind == OP_PROT) {
        const float2 cs = ldm(mats + op.mat_off);
        float qv = ((op.nY & 3) <= 1) ? -cs.y : cs.y;
        if (MODE == MODE_BWD) qv = -qv;  // the adjoint rotation
        float k, t;
        if (gshear_params(cs.x, qv, k, t)) atomicXor(&s_kneg, 1u);
        s_kt[i] = make_float2(k, t);
      }
    }
    __syncthreads();
    pneg = s_kneg;
  }
  bool live = false;     // registers hold the tile
  bool in_smem = false;  // smem holds the tile
  int prev = -1;
  Layout ly;

  for (int s = P.stage_begin; s < P.stage_end; ++s) {
    const DevStage& S = A.prog.stages[s];
    if (!LITE && S.smem_stage) {
      if (live) {
        regs_to_smem<R>(v, sm_psi, ly);
        if (HAS_MU) regs_to_smem<R>(w, sm_mu, ly);
        live = false;
      } else if (!in_smem) {
        tile_load_smem(sm_psi, psi_ld, base, runs, L, tid, nthreads);
        if (HAS_MU) load_mu_smem();
      }
      in_smem = true;
      __syncthreads();
      for (int o = S.op_begin; o < S.op_end; ++o) {
        const DevOp& op = A.prog.ops[o];
        const float2* m = mats + op.mat_off;
        if (MODE == MODE_FWD) {
          dispatch_denseK(op.k, sm_psi, L, op.p, m, false, tid, nthreads);
        } else if (MODE == MODE_BWD) {
          dispatch_denseK(op.k, sm_psi, L, op.p, m, true, tid, nthreads);
          dispatch_denseK(op.k, sm_mu, L, op.p, m, true, tid, nthreads);
        }
        __syncthreads();
      }
      prev = s;
      continue;
    }

    // ---- register stage: bring the tile into registers in this layout
    if (!live) {
      make_layout<R>(ly, S, P, tid);
      if (in_smem) {
        regs_from_smem<R>(v, sm_psi, ly);
        if (HAS_MU) regs_from_smem<R>(w, sm_mu, ly);
        __syncthreads();
      } else if (S.lanes_low) {
        regs_from_global<R>(v, psi_ld, base, ly);
        if (HAS_MU) {
          if (mu_zero) {
#pragma unroll
            for (int r = 0; r < NR; ++r) w[r] = make_float2(0.f, 0.f);
          } else {
            regs_from_global<R>(w, mu, base, ly);
          }
        }
      } else {
        tile_load_smem(sm_psi, psi_ld, base, runs, L, tid, nthreads);
        if (HAS_MU) load_mu_smem();
        __syncthreads();
        regs_from_smem<R>(v, sm_psi, ly);
        if (HAS_MU) regs_from_smem<R>(w, sm_mu, ly);
        __syncthreads();
      }
      live = true;
      in_smem = false;
    } else if (!same_layout(A.prog.stages[prev], S)) {
      regs_to_smem<R>(v, sm_psi, ly);
      if (HAS_MU) regs_to_smem<R>(w, sm_mu, ly);
      __syncthreads();
      make_layout<R>(ly, S, P, tid);
      regs_from_smem<R>(v, sm_psi, ly);
      if (HAS_MU) regs_from_smem<R>(w, sm_mu, ly);
      __syncthreads();
    }
    const uint32_t gthr = base | ly.gt;  // global index of register 0

    // ---- ops
    for (int o = S.op_begin; o < S.op_end; ++o) {
      const DevOp& op = A.prog.ops[o];
      const int kind = op.kind;
      if (kind == OP_DENSE1) {
        const float2* m = mats + op.mat_off;
        if (MODE == MODE_FWD) {
          const float2 mm[4] = {ldm(m), ldm(m + 1), ldm(m + 2), ldm(m + 3)};
          dispatch_dense1<R>(op.p[0], v, mm);
        } else if (MODE == MODE_BWD) {
          const float2 a[4] = {cconj(ldm(m)), cconj(ldm(m + 2)), cconj(ldm(m + 1)), cconj(ldm(m + 3))};
          float2 acc[16];
#pragma unroll
          for (int e = 0; e < 16; ++e) acc[e] = czero();
          if (op.slot >= 0) {
            dispatch_dense1_bwd<R, true>(op.p[0], v, w, a, acc);
#pragma unroll
            for (int e = 0; e < 4; ++e) {
              const float2 t = warp_sum(acc[e], nl);
              if (lane == 0) sm_slot[warp * A.max_slots + op.slot + e] = t;
            }
          } else {
            dispatch_dense1_bwd<R, false>(op.p[0], v, w, a, acc);
          }
        }
      } else if (!LITE && kind == OP_DENSE2) {
        const float2* m = mats + op.mat_off;
        if (MODE == MODE_FWD) {
          float2 mm[16];
#pragma unroll
          for (int e = 0; e < 16; ++e) mm[e] = ldm(m + e);
          dispatch_dense2<R>(op.p[0], op.p[1], v, mm);
        } else if (MODE == MODE_BWD) {
          float2 a[16];
#pragma unroll
          for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) a[4 * i + j] = cconj(ldm(m + 4 * j + i));
          float2 acc[16];
#pragma unroll
          for (int e = 0; e < 16; ++e) acc[e] = czero();
          if (op.slot >= 0) {
            dispatch_dense2_bwd<R, true>(op.p[0], op.p[1], v, w, a, acc);
#pragma unroll
            for (int e = 0; e < 16; ++e) {
              const float2 t = warp_sum(acc[e], nl);
              if (lane == 0) sm_slot[warp * A.max_slots + op.slot + e] = t;
            }
          } else {
            dispatch_dense2_bwd<R, false>(op.p[0], op.p[1], v, w, a, acc);
          }
        }
      } else if (!LITE && kind == OP_DIAG) {
        const float2* m = mats + op.mat_off;
        const int k = op.k;
        // index contribution of the fixed part and of each register bit
        int idx_t = 0;
        for (int i = 0; i < k; ++i) idx_t |= ((gthr >> op.p[i]) & 1u) << (k - 1 - i);
        int dbit[R];
#pragma unroll
        for (int ri = 0; ri < R; ++ri) {
          int d = 0;
          for (int i = 0; i < k; ++i)
            if (ly.rg[ri] == (1u << op.p[i])) d = 1 << (k - 1 - i);
          dbit[ri] = d;
        }
        if (k <= 2) {
          float2 d4[4];
#pragma unroll
          for (int e = 0; e < 4; ++e) d4[e] = (e < (1 << k)) ? ldm(m + e) : czero();
          if (MODE == MODE_FWD) {
#pragma unroll
            for (int r = 0; r < NR; ++r) {
              int idx = idx_t;
#pragma unroll
              for (int ri = 0; ri < R; ++ri)
                if ((r >> ri) & 1) idx ^= dbit[ri];
              const float2 d = (idx == 0) ? d4[0] : (idx == 1) ? d4[1] : (idx == 2) ? d4[2] : d4[3];
              v[r] = cmul(d, v[r]);
            }
          } else if (MODE == MODE_BWD) {
            float2 acc[4] = {czero(), czero(), czero(), czero()};
#pragma unroll
            for (int r = 0; r < NR; ++r) {
              int idx = idx_t;
#pragma unroll
              for (int ri = 0; ri < R; ++ri)
                if ((r >> ri) & 1) idx ^= dbit[ri];
              const float2 d = cconj((idx == 0) ? d4[0] : (idx == 1) ? d4[1] : (idx == 2) ? d4[2] : d4[3]);
              const float2 y = cmul(d, v[r]);
              v[r] = y;
              const float2 u = w[r];
              const float2 g = make_float2(fmaf(u.x, y.x, u.y * y.y), fmaf(u.y, y.x, -u.x * y.y));
              acc[0].x += (idx == 0) ? g.x : 0.f; acc[0].y += (idx == 0) ? g.y : 0.f;
              acc[1].x += (idx == 1) ? g.x : 0.f; acc[1].y += (idx == 1) ? g.y : 0.f;
              acc[2].x += (idx == 2) ? g.x : 0.f; acc[2].y += (idx == 2) ? g.y : 0.f;
              acc[3].x += (idx == 3) ? g.x : 0.f; acc[3].y += (idx == 3) ? g.y : 0.f;
              w[r] = cmul(d, u);
            }
            if (op.slot >= 0) {
              for (int e = 0; e < (1 << k); ++e) {
                const float2 t = warp_sum(acc[e], nl);
                if (lane == 0) sm_slot[warp * A.max_slots + op.slot + e] = t;
              }
            }
          }
        } else {
#pragma unroll
          for (int r = 0; r < NR; ++r) {
            int idx = idx_t;
#pragma unroll
            for (int ri = 0; ri < R; ++ri)
              if ((r >> ri) & 1) idx ^= dbit[ri];
            if (MODE == MODE_FWD) {
              v[r] = cmul(ldm(m + idx), v[r]);
            } else if (MODE == MODE_BWD) {
              const float2 d = cconj(ldm(m + idx));
              v[r] = cmul(d, v[r]);
              w[r] = cmul(d, w[r]);
            }
          }
        }
      } else if (kind == OP_PROT) {
        const int sg = __popc(gthr & op.zmask) & 1;
        int zr = 0;
#pragma unroll
        for (int ri = 0; ri < R; ++ri)
          if (ly.rg[ri] & op.zmask) zr |= 1 << ri;
        // q = (0, -s) (-i)^nY: (0, -s), (-s, 0), (0, s), (s, 0) for nY % 4 = 0..3
        const int ny = op.nY & 3;
        const bool qim = (ny & 1) == 0;
        // shear parameters of this rotation (the adjoint's for MODE_BWD)
        float k, t;
        if ((unsigned)(o - kt_ob) < (unsigned)kt_n) {
          const float2 kt = s_kt[o - kt_ob];
          k = sg ? -kt.x : kt.x;
          t = sg ? -kt.y : kt.y;
        } else {
          const float2 cs = ldm(mats + op.mat_off);  // (cos phi, sin phi)
          float qv = (ny <= 1) ? -cs.y : cs.y;
          if (sg) qv = -qv;
          pneg ^= gshear_params(cs.x, MODE == MODE_BWD ? -qv : qv, k, t);
        }
        if (MODE == MODE_FWD) {
          dispatch_gshear<R>(op.xreg, qim, v, k, t, zr);
        } else if (MODE == MODE_BWD) {
          if (op.slot >= 0) {
            // g = Im(pt z), pt = (+-)(-i)^nY: z.y, -z.x, -z.y, z.x for nY % 4 = 0..3
            float g = dispatch_prot_dot<R>(op.xreg, v, w, zr, qim);
            if (ny == 1 || ny == 2) g = -g;
            if (sg) g = -g;
            const float gs = warp_sum1(g, nl);  // (t is the shear parameter)
            if (lane == 0) sm_slot[warp * A.max_slots + op.slot] = make_float2(gs, 0.f);
          }
          dispatch_gshear2<R>(op.xreg, qim, v, w, k, t, zr);
        }
      } else if (kind == OP_ZRUN) {
        if (MODE == MODE_MEAS) {
          // <Z_S> partial = sum_x s(x) |psi_x|^2: one transform of |v_r|^2
          float t[NR];
#pragma unroll
          for (int r = 0; r < NR; ++r) t[r] = fmaf(v[r].x, v[r].x, v[r].y * v[r].y);
          add_walsh<R>(t);
          zrun_slot_sums<R>(t, A.prog.zents + op.mat_off, op.k, gthr, nl, lane, sm_slot + warp * A.max_slots);
        } else if (MODE == MODE_PACC) {
          // mu += (sum_t c_t s_t(x)) psi: class sums, one transform
          float a[NR];
#pragma unroll
          for (int c = 0; c < NR; ++c) a[c] = 0.f;
          for (int e = 0; e < op.k; ++e) {
            const ZEnt ze = A.prog.zents[op.mat_off + e];
            float cf = A.coef[b * A.coef_stride + ze.mat_off];
            if (__popc(gthr & ze.zmask) & 1) cf = -cf;
            class_add<R>(a, ze.zreg, cf);
          }
          add_walsh<R>(a);
#pragma unroll
          for (int r = 0; r < NR; ++r) w[r] = make_float2(fmaf(a[r], v[r].x, w[r].x), fmaf(a[r], v[r].y, w[r].y));
        }
        if (MODE == MODE_FWD || MODE == MODE_BWD) {
          float2 ph[NR];
#pragma unroll
          for (int c = 0; c < NR; ++c) ph[c] = make_float2(1.f, 0.f);
          for (int e = 0; e < op.k; ++e) {
            const ZEnt ze = A.prog.zents[op.mat_off + e];
            float2 u = ldm(mats + ze.mat_off);  // e^{i phi}; parity 0 takes e^{-i phi}
            if (!(__popc(gthr & ze.zmask) & 1)) u = cconj(u);
            class_mul<R>(ph, ze.zreg, u);
          }
          mul_walsh<R>(ph);
          if (MODE == MODE_FWD) {
#pragma unroll
            for (int r = 0; r < NR; ++r) cmul_ip(v[r], ph[r]);
          } else {
            if (op.slot >= 0) {
              // dL/dphi_e = sum_x s_e(x) Im(conj(mu_x) psi_x) at the run's output
              float t[NR];
#pragma unroll
              for (int r = 0; r < NR; ++r) t[r] = fmaf(w[r].x, v[r].y, -w[r].y * v[r].x);
              add_walsh<R>(t);
              zrun_slot_sums<R>(t, A.prog.zents + op.mat_off, op.k, gthr, nl, lane, sm_slot + warp * A.max_slots);
            }
#pragma unroll
            for (int r = 0; r < NR; ++r) {
              const float2 c = cconj(ph[r]);
              cmul_ip(v[r], c);
              cmul_ip(w[r], c);
            }
          }
        }
      } else if (kind == OP_EXPECT) {
        // sign bits: fixed part parity and register bits inside zmask
        const int sbase = __popc(gthr & op.zmask) & 1;
        int zr = 0;
#pragma unroll
        for (int ri = 0; ri < R; ++ri)
          if (ly.rg[ri] & op.zmask) zr |= 1 << ri;
        if (MODE == MODE_MEAS) {
          float2 acc = dispatch_expect<R>(op.xreg, v, sbase, zr);
          acc = cmul(ypow(op.nY), acc);
          acc = warp_sum(acc, nl);
          if (lane == 0) sm_slot[warp * A.max_slots + op.slot] = acc;
        } else if (MODE == MODE_PACC) {
          const float c = A.coef[b * A.coef_stride + op.mat_off];
          const float2 y = ypow(op.nY);
          const float2 cf = make_float2(c * y.x, c * y.y);
          dispatch_pacc<R>(op.xreg, v, w, cf, sbase, zr);
        }
      }
    }

    // ---- flush accumulator slots of this stage (fixed order over warps)
    if ((MODE == MODE_BWD || MODE == MODE_MEAS) && S.nslots > 0) {
      __syncthreads();
      for (int e = S.slot_out_begin + tid; e < S.slot_out_end; e += nthreads) {
        const SlotOut so = A.prog.slot_out[e];
        float2 t = czero();
        for (int q = 0; q < nwarps; ++q) {
          const float2 x = sm_slot[q * A.max_slots + so.slot];
          t.x += x.x;
          t.y += x.y;
        }
        A.partial[(size_t(b) * A.part_stride + so.out_off) * ntiles + tile] = t;
      }
      __syncthreads();
    }
    prev = s;
  }

  // ---- write the tile back (with the sign the shear rotations left pending;
  // it is the same for every thread of the tile)
  if ((MODE == MODE_FWD || MODE == MODE_BWD) && pneg) {
    if (live) {
#pragma unroll
      for (int r = 0; r < NR; ++r) {
        v[r] = make_float2(-v[r].x, -v[r].y);
        if (HAS_MU) w[r] = make_float2(-w[r].x, -w[r].y);
      }
    } else if (in_smem) {
      __syncthreads();
      for (uint32_t j = tid; j < (1u << L); j += nthreads) {
        sm_psi[j] = make_float2(-sm_psi[j].x, -sm_psi[j].y);
        if (HAS_MU) sm_mu[j] = make_float2(-sm_mu[j].x, -sm_mu[j].y);
      }
      __syncthreads();
    }
  }
  if (STORE_PSI || STORE_MU) {
    if (live) {
      const DevStage& S = A.prog.stages[prev];
      if (S.lanes_low) {
        if (STORE_PSI) regs_to_global<R>(v, psi, base, ly);
        if (STORE_MU) regs_to_global<R>(w, mu, base, ly);
      } else {
        if (STORE_PSI) regs_to_smem<R>(v, sm_psi, ly);
        if (STORE_MU) regs_to_smem<R>(w, sm_mu, ly);
        __syncthreads();
        if (STORE_PSI) tile_store_smem(sm_psi, psi, base, runs, L, tid, nthreads);
        if (STORE_MU) tile_store_smem(sm_mu, mu, base, runs, L, tid, nthreads);
      }
    } else if (in_smem) {
      if (STORE_PSI) tile_store_smem(sm_psi, psi, base, runs, L, tid, nthreads);
      if (STORE_MU) tile_store_smem(sm_mu, mu, base, runs, L, tid, nthreads);
    }
  }
}

template <int MODE, int R>
__global__ void __launch_bounds__(256, 1) pass_kernel(PassArgs A) {
  extern __shared__ __align__(16) float2 smem_raw[];
  pass_tile<MODE, R>(A, blockIdx.x, blockIdx.y, gridDim.x, smem_raw);
}

// ------------------------------------------------------ persistent batches
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// Bulk L2 prefetch of one 256-byte run (TMA unit; a hint, never faults on
// a valid address).  Runs are 256-byte aligned.
__device__ __forceinline__ void prefetch_l2_run(const float2* p) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], 256;" ::"l"(__cvta_generic_to_global(p)) : "memory");
}
__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// A dependency is always a set of items dequeued earlier by CTAs that are
// running, so waits end; the limit only guards against a broken schedule.
// After a time-out every later wait is skipped (results are then invalid and
// the error flag says so) so the launch still finishes.

template <int MODE, int R, bool LITE>
__global__ void __launch_bounds__(256, LITE ? ((MODE == MODE_FWD || MODE == MODE_PACC) ? 3 : 2) : 1)
    batch_kernel(BatchLaunch BL) {
  extern __shared__ __align__(16) float2 smem_raw[];
  __shared__ long long s_item;
  __shared__ int s_seg;
  // L2 prefetch of the chunk's next tile: its runs, psi (and mu)
  __shared__ const float2* s_pf_psi;
  __shared__ const float2* s_pf_mu;
  __shared__ const uint32_t* s_pf_runs;
  __shared__ int s_pf_n;
  long long chunk_next = 0, chunk_end = 0;  // thread 0: rest of the dequeued chunk
  int last_seg = 0;
  for (;;) {
    if (threadIdx.x == 0) {
      s_pf_n = 0;
      if (chunk_next >= chunk_end) {
        chunk_next = (long long)atomicAdd(BL.queue, (unsigned)kBatchChunk);
        chunk_end = chunk_next + kBatchChunk;
        last_seg = -1;
      }
      const long long item = chunk_next++;
      int seg = -1;
      if (item < BL.nitems) {
        if (last_seg >= 0) {
          // items of a chunk are consecutive: step forward from the last one
          seg = last_seg;
          while (seg + 1 < BL.nsegs && BL.segs[seg + 1].item0 <= item) ++seg;
        } else {
          // the coarse index brackets the binary search to a few segments
          const long long k = item / kBatchCoarse;
          int lo = BL.coarse[k], hi = BL.coarse[k + 1];
          while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (BL.segs[mid].item0 <= item) lo = mid;
            else hi = mid - 1;
          }
          seg = lo;
        }
        last_seg = seg;
        // the next tile of the chunk: its data may still be rewritten before
        // it is read (L2 stays coherent), so the prefetch is only a hint
        const long long nxt = chunk_next;
        if (nxt < chunk_end && nxt < BL.nitems) {
          int ns = seg;
          while (ns + 1 < BL.nsegs && BL.segs[ns + 1].item0 <= nxt) ++ns;
          const BatchSeg& q = BL.segs[ns];
          const BatchCirc& qc = BL.circ[q.circ];
          const DevPass& qp = qc.prog.passes[q.pass];
          const uint32_t t = (uint32_t)(nxt - q.item0);
          uint32_t base = 0;
          for (int i = 0; i < qp.nnonlocal; ++i)
            if ((t >> i) & 1u) base |= 1u << qp.nlbits[i];
          s_pf_psi = BL.psi + qc.state_off + base;
          s_pf_mu = BL.mu ? BL.mu + qc.state_off + base : nullptr;
          s_pf_runs = qc.prog.runs + qp.runs_off;
          s_pf_n = 1 << (qp.L - kLo);
        }
        const unsigned need = BL.segs[seg].need;
        const unsigned* dn = BL.done + BL.segs[seg].circ;
        if (need > 0 && ld_acquire_u32(dn) < need && ld_acquire_u32(BL.err) == 0u) {
          const unsigned long long t0 = global_ns();
          unsigned spins = 0;
          while (ld_acquire_u32(dn) < need) {
            __nanosleep(100);
            if ((++spins & 63u) == 0u && (global_ns() - t0 > BL.wait_ns || ld_acquire_u32(BL.err) != 0u)) {
              atomicOr(BL.err, 1u);
              atomicOr(BL.sticky, 1u);
              break;
            }
          }
        }
        __threadfence();
      }
      s_item = item;
      s_seg = seg;
    }
    __syncthreads();
    const long long item = s_item;
    const int seg = s_seg;
    if (seg < 0) break;
    {
      const int pn = s_pf_n;
      const float2* pp = s_pf_psi;
      const float2* pm = s_pf_mu;
      const uint32_t* pr = s_pf_runs;
      for (int k = threadIdx.x; k < pn; k += blockDim.x) {
        const uint32_t off = __ldg(pr + k);  // one 2^kLo-amplitude (256-byte) run
        prefetch_l2_run(pp + off);
        if (pm) prefetch_l2_run(pm + off);
      }
    }
    const BatchSeg sg = BL.segs[seg];
    const BatchCirc& C = BL.circ[sg.circ];
    PassArgs A;
    A.prog = C.prog;
    A.pass = sg.pass;
    A.n = C.n;
    A.psi = BL.psi + C.state_off;
    A.mu = BL.mu ? BL.mu + C.state_off : nullptr;
    A.mats = BL.mats ? BL.mats + C.mat_off : nullptr;
    A.mat_stride = 0;
    A.partial = BL.partial ? BL.partial + C.part_off : nullptr;
    A.part_stride = C.part_stride;
    A.coef = BL.coef ? BL.coef + C.coef_off : nullptr;
    A.coef_stride = 0;
    A.max_slots = C.max_slots;
    A.psi_in = nullptr;
    A.in_stride = 0;
    A.mu_zero = 0;
    pass_tile<MODE, R, LITE>(A, (uint32_t)(item - sg.item0), 0, sg.ntiles, smem_raw);
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      atomicAdd(BL.done + sg.circ, 1u);
    }
  }
}

// ---------------------------------------------------------------- launchers
template <int MODE, int R>
static cudaError_t launch_one(const PassArgs& a, int L, int64_t batch, cudaStream_t st) {
  const int nthreads = 1 << (L - R);
  const bool has_mu = (MODE == MODE_BWD || MODE == MODE_PACC);
  const int nwarps = (nthreads + 31) / 32;
  const size_t smem = size_t(has_mu ? 2 : 1) * (size_t(1) << L) * sizeof(float2) +
                      size_t(nwarps) * a.max_slots * sizeof(float2);
  if (nthreads > kMaxThreads) return cudaErrorInvalidValue;
  // the opt-in shared-memory size is a per-device function attribute: raise
  // it once per device to the largest size seen
  static int attr_smem[64] = {0};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 64 && attr_smem[dev] < (int)smem) {
    e = cudaFuncSetAttribute(pass_kernel<MODE, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    attr_smem[dev] = (int)smem;
  }
  const uint32_t ntiles = 1u << (a.n - L);
  for (int64_t b0 = 0; b0 < batch; b0 += 65535) {
    const int64_t nb = (batch - b0) < 65535 ? (batch - b0) : 65535;
    PassArgs aa = a;
    const size_t len = size_t(1) << a.n;
    aa.psi = a.psi + b0 * len;
    if (aa.mu) aa.mu = a.mu + b0 * len;
    if (aa.mats) aa.mats = a.mats + b0 * a.mat_stride;
    if (aa.coef) aa.coef = a.coef + b0 * a.coef_stride;
    if (aa.psi_in) aa.psi_in = a.psi_in + b0 * a.in_stride;
    if (aa.partial) aa.partial = a.partial + size_t(b0) * a.part_stride * ntiles;
    dim3 grid(ntiles, (unsigned)nb);
    count_launch();
    pass_kernel<MODE, R><<<grid, nthreads, smem, st>>>(aa);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

template <int MODE, int R, bool LITE>
static cudaError_t launch_batch_one(const BatchLaunch& bl, int L, int max_slots, cudaStream_t st) {
  const int nthreads = 1 << (L - R);
  if (nthreads > kMaxThreads || nthreads < 1) return cudaErrorInvalidValue;
  const bool has_mu = (MODE == MODE_BWD || MODE == MODE_PACC);
  const int nwarps = (nthreads + 31) / 32;
  const size_t smem = size_t(has_mu ? 2 : 1) * (size_t(1) << L) * sizeof(float2) +
                      size_t(nwarps) * max_slots * sizeof(float2);
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  static int attr_smem[64] = {0};
  if (dev < 64 && attr_smem[dev] < (int)smem) {
    e = cudaFuncSetAttribute(batch_kernel<MODE, R, LITE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
    if (e != cudaSuccess) return e;
    attr_smem[dev] = (int)smem;
  }
  int nsm = 0, per_sm = 0;
  e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_kernel<MODE, R, LITE>, nthreads, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  int64_t grid = int64_t(nsm) * per_sm;
  if (grid > bl.nitems) grid = bl.nitems;
  if (grid < 1) return cudaSuccess;
  count_launch();
  batch_kernel<MODE, R, LITE><<<(unsigned)grid, nthreads, smem, st>>>(bl);
  return cudaGetLastError();
}

// Per-family launchers, explicitly instantiated by pass_inst.cu.
template <int MODE>
cudaError_t launch_pass_mode(const PassArgs& a, int L, int64_t batch, cudaStream_t st) {
  return launch_one<MODE, 4>(a, L, batch, st);
}

template <int MODE, bool LITE>
cudaError_t launch_batch_mode(const BatchLaunch& bl, int L, int max_slots, cudaStream_t st) {
  return launch_batch_one<MODE, 4, LITE>(bl, L, max_slots, st);
}

}  // namespace tcg
