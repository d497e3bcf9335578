// Device building blocks of the mixed-precision determinant, shared by the
// batched kernels (lup_mixed.cu) and the persistent mixed-size kernel
// (grouped.cu). The method is described in lup_mixed.cu.
#pragma once

#include <cmath>
#include <type_traits>

#include "lup_fp64.cuh"
#include "fp64_correct.cuh"

namespace lufqhe {
namespace mixed {
// internal linkage: every translation unit that includes this gets its own copy
namespace {


constexpr int kMaxWarpsMixed = 8;
// ||E||_F / max(1, |log|det||) above which the correction may miss 1e-10
// relative accuracy. E comes from FP32 triangular solves, whose rounding
// leaves an absolute error of about 1e-6 * ||E||_F in log det(I + E)
// (measured on lowest-Landau-level matrices against a double-double oracle);
// 5e-5 keeps that near 5e-11 relative, half the 1e-10 target.
constexpr float kCorrRelCap = 5e-5f;
// The same cap after one refinement step of the back substitution
// (mixed_refine_tile): an emulation of the method on lowest-Landau-level
// matrices against a double-double oracle puts the error left in
// log det(I + E) at about 1.2e-7 ||E||_F at most, so 3e-4 keeps it near
// 4e-11 relative; above max(1, |log|det||) ~ 300 the absolute cap theta binds.
constexpr float kRefinedRelCap = 3e-4f;

// Packed FP32 pairs: one instruction for both components, each rounded
// exactly as the scalar __fadd_rn / __fsub_rn / __fmul_rn / __fmaf_rn.
__device__ __forceinline__ unsigned long long pk2(float2 a) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a.x), "f"(a.y));
  return r;
}
__device__ __forceinline__ float2 up2(unsigned long long r) {
  float2 a;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a.x), "=f"(a.y) : "l"(r));
  return a;
}
__device__ __forceinline__ float2 f2fma(float2 a, float2 b, float2 c) {
  unsigned long long r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(pk2(a)), "l"(pk2(b)), "l"(pk2(c)));
  return up2(r);
}
__device__ __forceinline__ float2 f2add(float2 a, float2 b) {
  unsigned long long r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(pk2(a)), "l"(pk2(b)));
  return up2(r);
}
__device__ __forceinline__ float2 f2sub(float2 a, float2 b) {
  unsigned long long r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(pk2(a)), "l"(pk2(b)));
  return up2(r);
}
__device__ __forceinline__ float2 f2mul(float2 a, float2 b) {
  unsigned long long r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(pk2(a)), "l"(pk2(b)));
  return up2(r);
}

// ---- float-float building blocks (never contracted: explicit _rn ops) ------
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
__device__ __forceinline__ void two_prod(float a, float b, float &p, float &e) {
  p = __fmul_rn(a, b);
  e = __fmaf_rn(a, b, -p);
}

// s + c -= l*u exactly up to the compensation's own rounding (Dot2 step), the
// real and imaginary parts side by side in packed pairs: sc.xy is the high
// part, sc.zw the compensation. A = -(lx ux, lx uy), B = (ly uy, -ly ux) with
// their exact product errors from FMAs, each added by TwoSum.
__device__ __forceinline__ void dot2_csub(float4 &sc, float2 l, float2 u) {
  const float2 lx = make_float2(l.x, l.x), lxn = make_float2(-l.x, -l.x);
  const float2 lys = make_float2(l.y, -l.y), lysn = make_float2(-l.y, l.y);
  const float2 us = make_float2(u.y, u.x);
  const float2 A = f2mul(lxn, u);       // (-p1, -p3)
  const float2 EA = f2fma(lx, u, A);    // (e1, e3), lx u = p + e
  const float2 B = f2mul(lys, us);      // (p2, -p4)
  const float2 EBn = f2fma(lysn, us, B);  // (-e2, e4)
  const float2 hi = make_float2(sc.x, sc.y);
  const float2 s1 = f2add(hi, A);
  float2 bb = f2sub(s1, hi);
  const float2 t1 = f2add(f2sub(hi, f2sub(s1, bb)), f2sub(A, bb));
  const float2 s2 = f2add(s1, B);
  bb = f2sub(s2, s1);
  const float2 t2 = f2add(f2sub(s1, f2sub(s2, bb)), f2sub(B, bb));
  const float2 lo = f2add(make_float2(sc.z, sc.w), f2add(f2sub(t1, EA), f2sub(t2, EBn)));
  sc = make_float4(s2.x, s2.y, lo.x, lo.y);
}

__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
  return make_float2(__fmaf_rn(a.x, b.x, -a.y * b.y), __fmaf_rn(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float2 cfms(float2 s, float2 l, float2 u) {  // s - l*u
  float x = __fmaf_rn(-l.x, u.x, s.x);
  x = __fmaf_rn(l.y, u.y, x);
  float y = __fmaf_rn(-l.x, u.y, s.y);
  y = __fmaf_rn(-l.y, u.x, y);
  return make_float2(x, y);
}
__device__ __forceinline__ float2 crcpf(float2 u) {
  float rd = __frcp_rn(__fmaf_rn(u.x, u.x, u.y * u.y));
  return make_float2(u.x * rd, -u.y * rd);
}
// 1/u from the hardware's approximate reciprocal (about an ulp, subnormal
// |u|^2 flushed to zero, which gives a non-finite multiplier and so a
// rejection): for the FP32 LUP of the tile path, whose multipliers need not be
// correctly rounded because the float-float residual is exact for whatever L
// and U come out. The solves and the elimination of I + E keep crcpf.
__device__ __forceinline__ float2 crcpf_approx(float2 u) {
  float rd;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(rd) : "f"(__fmaf_rn(u.x, u.x, u.y * u.y)));
  return make_float2(u.x * rd, -u.y * rd);
}

// Unbiased exponent field of the larger of |re|, |im| (-2000 for zero/subnormal).
__device__ __forceinline__ int cexp_field(double2 v) {
  int ex = (__double2hiint(v.x) >> 20) & 0x7ff;
  int ey = (__double2hiint(v.y) >> 20) & 0x7ff;
  int e = max(ex, ey);
  return e == 0 ? -2000 : e - 1023;
}

// x * 2^-s split into float hi + lo by integer operations (hi keeps the top 24
// significant bits, lo the next 24; the last <= 5 bits are dropped). The
// caller guarantees |x| * 2^-s < 2. Subnormal results flush to zero.
__device__ __forceinline__ void split_scaled(double x, int s, float &hi, float &lo) {
  unsigned long long u = (unsigned long long)__double_as_longlong(x);
  unsigned sign = (unsigned)(u >> 32) & 0x80000000u;
  int e = (int)((u >> 52) & 0x7ff);
  int E = e - 1023 - s;
  if (e == 0 || E < -126) {
    hi = __int_as_float((int)sign);
    lo = 0.0f;
    return;
  }
  unsigned long long mant = u & 0xFFFFFFFFFFFFFull;
  hi = __int_as_float((int)(sign | ((unsigned)(E + 127) << 23) | (unsigned)(mant >> 29)));
  unsigned rem = (unsigned)(mant & 0x1FFFFFFFull);
  if (rem == 0) {
    lo = 0.0f;
    return;
  }
  int p = 31 - __clz(rem);
  int El = E - 52 + p;
  if (El < -126) {
    lo = 0.0f;
    return;
  }
  unsigned lm = (p >= 23) ? (rem >> (p - 23)) : (rem << (23 - p));
  lo = __int_as_float((int)(sign | ((unsigned)(El + 127) << 23) | (lm & 0x7FFFFFu)));
}

// ---- complex float-float with a separate power-of-two exponent ------------
struct CFF {
  float xh, xl, yh, yl;
  int e;
};

__device__ __forceinline__ void ff_renorm(CFF &a) {
  float m = fmaxf(fabsf(a.xh), fabsf(a.yh));
  if (m == 0.0f) return;
  int k = ((__float_as_int(m) >> 23) & 0xff) - 127;
  // scale by 2^-k (exact): multiply by a power of two built from bits
  float sc = __int_as_float((127 - k) << 23);
  a.xh *= sc;
  a.xl *= sc;
  a.yh *= sc;
  a.yl *= sc;
  a.e += k;
}

__device__ __forceinline__ CFF ff_cmul(const CFF &a, const CFF &b) {
  float p1, e1, p2, e2, p3, e3, p4, e4, s, t;
  two_prod(a.xh, b.xh, p1, e1);
  two_prod(a.yh, b.yh, p2, e2);
  two_prod(a.xh, b.yh, p3, e3);
  two_prod(a.yh, b.xh, p4, e4);
  CFF r;
  // every operation explicit (_rn): no context-dependent FMA contraction, so
  // each kernel that uses this gets the same bits
  two_sum(p1, -p2, s, t);
  float cx = __fmaf_rn(a.xh, b.xl, __fmul_rn(a.xl, b.xh));
  float cy = __fmaf_rn(a.yh, b.yl, __fmul_rn(a.yl, b.yh));
  float lo = __fsub_rn(__fadd_rn(__fsub_rn(__fadd_rn(t, e1), e2), cx), cy);
  r.xh = __fadd_rn(s, lo);
  r.xl = __fsub_rn(lo, __fsub_rn(r.xh, s));
  two_sum(p3, p4, s, t);
  cx = __fmaf_rn(a.xh, b.yl, __fmul_rn(a.xl, b.yh));
  cy = __fmaf_rn(a.yh, b.xl, __fmul_rn(a.yl, b.xh));
  lo = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(t, e3), e4), cx), cy);
  r.yh = __fadd_rn(s, lo);
  r.yl = __fsub_rn(lo, __fsub_rn(r.yh, s));
  r.e = a.e + b.e;
  ff_renorm(r);
  return r;
}

__device__ __forceinline__ CFF shfl_cff(const CFF &a, int src_or_mask, bool xor_mode) {
  CFF r;
  if (xor_mode) {
    r.xh = __shfl_xor_sync(kFull, a.xh, src_or_mask);
    r.xl = __shfl_xor_sync(kFull, a.xl, src_or_mask);
    r.yh = __shfl_xor_sync(kFull, a.yh, src_or_mask);
    r.yl = __shfl_xor_sync(kFull, a.yl, src_or_mask);
    r.e = __shfl_xor_sync(kFull, a.e, src_or_mask);
  } else {
    r.xh = __shfl_sync(kFull, a.xh, src_or_mask);
    r.xl = __shfl_sync(kFull, a.xl, src_or_mask);
    r.yh = __shfl_sync(kFull, a.yh, src_or_mask);
    r.yl = __shfl_sync(kFull, a.yl, src_or_mask);
    r.e = __shfl_sync(kFull, a.e, src_or_mask);
  }
  return r;
}

struct MixedSmem {
  float2 *Af;   // FP32 working matrix -> L\U          [n][lds]
  float4 *SC;   // residual sum (xy) + compensation (zw); also double2 A [n][lds]
  double *hold; // FP64 fallback row scales and their reciprocals [2n]
  int *er;      // row exponents [n]
  int *ec;      // column exponents [n]
};

// Steps 4-6 on the factored F (L\\U, row stride lds) and the residual R
// (entry (i, k) at R[RS * (i * lds + k)]): E = U^-1 L^-1 R in place, the
// float-float product of diag(U), the acceptance test, and log det(I + E).
// Returns false (warp-uniform) if the matrix must be refactorised in FP64.
template <int RS>
__device__ bool mixed_finish(const float2 *F, float2 *R, int n, int lds, int lane, float theta2,
                             int exp_sum, CFF &prod, float2 &corr) {
  const int nn = n * n;
  // 4a. Y = L^-1 R (unit lower, forward)
  for (int t = 0; t + 1 < n; ++t) {
    const int rows = n - 1 - t;
    const int tot = rows * n;
    BlockWalk w(lane, n);
    for (int e = lane; e < tot; e += 32) {
      const int i = t + 1 + w.i, k = w.k;
      R[RS * (i * lds + k)] = cfms(R[RS * (i * lds + k)], F[i * lds + t], R[RS * (t * lds + k)]);
      w.next(n);
    }
    __syncwarp();
  }
  // 4b. E = U^-1 Y (backward)
  for (int t = n - 1; t >= 0; --t) {
    const float2 r = crcpf(F[t * lds + t]);
    for (int k = lane; k < n; k += 32) R[RS * (t * lds + k)] = cmulf(R[RS * (t * lds + k)], r);
    __syncwarp();
    const int tot = t * n;
    BlockWalk w(lane, n);
    for (int e = lane; e < tot; e += 32) {
      const int i = w.i, k = w.k;
      R[RS * (i * lds + k)] = cfms(R[RS * (i * lds + k)], F[i * lds + t], R[RS * (t * lds + k)]);
      w.next(n);
    }
    __syncwarp();
  }

  // 6 (first half). complex float-float product of the diagonal of U; its
  // exponent gives log2|det| to within 2 before the correction is accepted
  {
    CFF acc = {1.0f, 0.0f, 0.0f, 0.0f, 0};
    for (int t = lane; t < n; t += 32) {
      float2 u = F[t * lds + t];
      CFF v = {u.x, 0.0f, u.y, 0.0f, 0};
      ff_renorm(v);
      acc = ff_cmul(acc, v);
    }
#pragma unroll
    for (int off = 16; off; off >>= 1) acc = ff_cmul(acc, shfl_cff(acc, off, true));
    prod = shfl_cff(acc, 0, false);
  }

  // acceptance: ||E||_F <= theta, and the FP32 evaluation of log det(I+E)
  // (error ~ eps32 * ||E||_F) small against 1e-11 * max(1, |log|det||).
  // Decided on lane 0's sum so it is warp-uniform.
  {
    float f = 0.0f;
    BlockWalk w(lane, n);
    for (int e = lane; e < nn; e += 32) {
      float2 v = R[RS * (w.i * lds + w.k)];
      f = __fmaf_rn(v.x, v.x, __fmaf_rn(v.y, v.y, f));
      w.next(n);
    }
#pragma unroll
    for (int off = 16; off; off >>= 1) f += __shfl_xor_sync(kFull, f, off);
    f = __shfl_sync(kFull, f, 0);
    const float la_est = fabsf((float)(prod.e + exp_sum)) * 0.6931472f;
    const float rel_cap = kCorrRelCap * fmaxf(1.0f, la_est);
    if (!(f <= theta2) || !(f <= rel_cap * rel_cap)) return false;
  }

  // 5. log det(I + E): unpivoted LU with the identity implicit; the pivots
  //    1 + d_t stay on the diagonal and their logs are taken lane-parallel.
  for (int t = 0; t + 1 < n; ++t) {
    const float2 d = R[RS * (t * lds + t)];
    const float2 r = crcpf(make_float2(1.0f + d.x, d.y));
    for (int i = t + 1 + lane; i < n; i += 32)
      R[RS * (i * lds + t)] = cmulf(R[RS * (i * lds + t)], r);
    __syncwarp();
    const int m = n - 1 - t;
    const int mm = m * m;
    BlockWalk w(lane, m);
    for (int e = lane; e < mm; e += 32) {
      const int i = t + 1 + w.i, k = t + 1 + w.k;
      R[RS * (i * lds + k)] = cfms(R[RS * (i * lds + k)], R[RS * (i * lds + t)], R[RS * (t * lds + k)]);
      w.next(m);
    }
    __syncwarp();
  }
  float cre = 0.0f, cim = 0.0f;
  for (int t = lane; t < n; t += 32) {
    const float2 d = R[RS * (t * lds + t)];
    cre = __fmaf_rn(0.5f, log1pf(__fmaf_rn(d.x, d.x, __fmaf_rn(d.y, d.y, 2.0f * d.x))), cre);
    cim += atan2f(d.y, 1.0f + d.x);
  }
#pragma unroll
  for (int off = 16; off; off >>= 1) {
    cre += __shfl_xor_sync(kFull, cre, off);
    cim += __shfl_xor_sync(kFull, cim, off);
  }
  cre = __shfl_sync(kFull, cre, 0);
  cim = __shfl_sync(kFull, cim, 0);
  corr = make_float2(cre, cim);

  return true;
}

// Steps 1-6 for the matrix already loaded (as double2) into S.SC. Returns
// false (warp-uniform) if the matrix must be refactorised in FP64.
__device__ bool mixed_factor(const MixedSmem &S, int n, int lane, float theta2, CFF &prod,
                             int &exp_sum, float2 &corr, int &par) {
  const int lds = n + 1;
  const int nn = n * n;
  double2 *A = reinterpret_cast<double2 *>(S.SC);

  // 1. exponents: columns first (for orbital matrices the columns carry the
  //    |z|^m scales), then rows of the column-scaled matrix
  int rsum = 0, csum = 0;
  for (int k = lane; k < n; k += 32) {
    int m = -2000;
    for (int i = 0; i < n; ++i) m = max(m, cexp_field(A[i * lds + k]));
    if (m == -2000) m = 0;
    S.ec[k] = m;
    csum += m;
  }
  __syncwarp();
  for (int i = lane; i < n; i += 32) {
    int m = -2000;
    for (int k = 0; k < n; ++k) {
      int e = cexp_field(A[i * lds + k]);
      if (e != -2000) m = max(m, e - S.ec[k]);
    }
    if (m == -2000) m = 0;
    S.er[i] = m;
    rsum += m;
  }
  __syncwarp();
  // 2. split into hi (Af) and hi + lo (SC as s + c); same lane reads and writes
  {
    BlockWalk w(lane, n);
    for (int e = lane; e < nn; e += 32) {
      const int idx = w.i * lds + w.k;
      const double2 v = A[idx];
      const int s = S.er[w.i] + S.ec[w.k];
      float xh, xl, yh, yl;
      split_scaled(v.x, s, xh, xl);
      split_scaled(v.y, s, yh, yl);
      S.Af[idx] = make_float2(xh, yh);
      S.SC[idx] = make_float4(xh, yh, xl, yl);
      w.next(n);
    }
  }
#pragma unroll
  for (int off = 16; off; off >>= 1) {
    rsum += __shfl_xor_sync(kFull, rsum, off);
    csum += __shfl_xor_sync(kFull, csum, off);
  }
  exp_sum = rsum + csum;
  __syncwarp();

  // 3. FP32 LUP with the float-float residual
  par = 0;
  for (int t = 0; t < n; ++t) {
    float best = -1.0f;
    int bi = t;
    for (int i = t + lane; i < n; i += 32) {
      float2 v = S.Af[i * lds + t];
      float m = fabsf(v.x) + fabsf(v.y);
      if (m > best) {
        best = m;
        bi = i;
      }
    }
#pragma unroll
    for (int off = 16; off; off >>= 1) {
      float om = __shfl_xor_sync(kFull, best, off);
      int oi = __shfl_xor_sync(kFull, bi, off);
      if (om > best || (om == best && oi < bi)) {
        best = om;
        bi = oi;
      }
    }
    if (!(best > 0.0f) || !(best < INFINITY)) return false;  // zero/NaN/Inf pivot
    const int p = bi;
    if (p != t) {
      for (int k = lane; k < n; k += 32) {
        float2 a = S.Af[p * lds + k];
        S.Af[p * lds + k] = S.Af[t * lds + k];
        S.Af[t * lds + k] = a;
        float4 c = S.SC[p * lds + k];
        S.SC[p * lds + k] = S.SC[t * lds + k];
        S.SC[t * lds + k] = c;
      }
      par ^= 1;
    }
    __syncwarp();
    const float2 r = crcpf(S.Af[t * lds + t]);
    for (int i = t + 1 + lane; i < n; i += 32) S.Af[i * lds + t] = cmulf(S.Af[i * lds + t], r);
    __syncwarp();
    const int m = n - t;
    const int mm = m * m;
    BlockWalk w(lane, m);
    for (int e = lane; e < mm; e += 32) {
      const int i = t + w.i, k = t + w.k;
      const float2 U = S.Af[t * lds + k];
      float4 sc = S.SC[i * lds + k];
      if (i == t) {
        float s, c;
        two_sum(sc.x, -U.x, s, c);
        sc.x = s;
        sc.z = __fadd_rn(sc.z, c);
        two_sum(sc.y, -U.y, s, c);
        sc.y = s;
        sc.w = __fadd_rn(sc.w, c);
      } else {
        const float2 L = S.Af[i * lds + t];
        dot2_csub(sc, L, U);
        if (k > t) S.Af[i * lds + k] = cfms(S.Af[i * lds + k], L, U);
      }
      S.SC[i * lds + k] = sc;
      w.next(m);
    }
    __syncwarp();
  }

  // R = s + c, kept in the xy half of SC
  float2 *R = reinterpret_cast<float2 *>(S.SC);  // entry idx at R[2*idx]
  {
    BlockWalk w(lane, n);
    for (int e = lane; e < nn; e += 32) {
      const int idx = w.i * lds + w.k;
      float4 sc = S.SC[idx];
      R[2 * idx] = make_float2(__fadd_rn(sc.x, sc.z), __fadd_rn(sc.y, sc.w));
      w.next(n);
    }
  }
  __syncwarp();

  return mixed_finish<2>(S.Af, R, n, lds, lane, theta2, exp_sum, prod, corr);
}

// Deferred FP64 finalisation: lane L holds the L-th accepted matrix of the
// current group of 32; one warp-wide log/atan2 then serves all 32.
struct DeferredOut {
  long long slot_b = -1;
  CFF slot_p = {1.0f, 0.0f, 0.0f, 0.0f, 0};
  int slot_e = 0, slot_par = 0;
  float2 slot_c = make_float2(0.0f, 0.0f);
  int cnt = 0;

  __device__ __forceinline__ void flush(int lane, double *logabs, double *phase, int8_t *parity,
                                        int32_t *status) {
    if (lane < cnt && slot_b >= 0) {
      const double re = __dadd_rn((double)slot_p.xh, (double)slot_p.xl);
      const double im = __dadd_rn((double)slot_p.yh, (double)slot_p.yl);
      const double m2 = __fma_rn(re, re, __dmul_rn(im, im));
      const double la =
          __dadd_rn(__fma_rn((double)slot_e, kLn2, __dmul_rn(0.5, log(m2))), (double)slot_c.x);
      const double ph = __dadd_rn(__dadd_rn(atan2(im, re), (double)slot_c.y), slot_par ? kPi : 0.0);
      logabs[slot_b] = la;
      if (phase) phase[slot_b] = wrap_phase(ph);
      if (parity) parity[slot_b] = (int8_t)slot_par;
      if (status) status[slot_b] = 0;
    }
    slot_b = -1;
    cnt = 0;
  }
  __device__ __forceinline__ void push(int lane, long long b, const CFF &prod, int exp_sum,
                                       float2 corr, int par, double *logabs, double *phase,
                                       int8_t *parity, int32_t *status) {
    if (lane == cnt) {
      slot_b = b;
      slot_p = prod;
      slot_e = prod.e + exp_sum;
      slot_c = corr;
      slot_par = par;
    }
    if (++cnt == 32) flush(lane, logabs, phase, parity, status);
  }
};

// Route of a matrix in the batched mixed mode: true = straight to FP64. A hash
// of its first entry's bits, so the route depends on the content only.
__device__ __forceinline__ bool route_fp64_entry(double2 v, unsigned int share64k) {
  if (share64k == 0) return false;
  if (share64k >= 65536u) return true;
  unsigned long long h = (unsigned long long)__double_as_longlong(v.x) * 0x9E3779B97F4A7C15ull ^
                         (unsigned long long)__double_as_longlong(v.y);
  h ^= h >> 29;
  h *= 0xBF58476D1CE4E5B9ull;
  h ^= h >> 32;
  return (unsigned int)(h & 0xffffu) < share64k;
}

template <bool COHERENT = false>
__device__ __forceinline__ bool route_fp64(const double2 *src, unsigned int share64k) {
  if (share64k == 0) return false;
  if (share64k >= 65536u) return true;
  return route_fp64_entry(COHERENT ? __ldcg(src) : __ldg(src), share64k);
}

// A bounded wait inside the kernel ran out (never expected): NaN result.
__device__ __forceinline__ void emit_wait_timeout(int lane, long long b, double *logabs,
                                                  double *phase, int8_t *parity, int32_t *status) {
  if (lane == 0) {
    logabs[b] = NAN;
    if (phase) phase[b] = NAN;
    if (parity) parity[b] = 0;
    if (status) status[b] = LUFQHE_ST_WAIT_TIMEOUT;
  }
}

__device__ __forceinline__ void emit_nonfinite(int lane, long long b, double *logabs,
                                               double *phase, int8_t *parity, int32_t *status) {
  if (lane == 0) {
    logabs[b] = NAN;
    if (phase) phase[b] = NAN;
    if (parity) parity[b] = 0;
    if (status) status[b] = LUFQHE_ST_NONFINITE;
  }
}

// FP64 factors left for a correction pass of their own (FacList): the
// matrix's slot, its uncorrected result, the pivot order and L\U (row stride
// n), and with `copy` the matrix itself after them (for sources the pass
// cannot read again cheaply: a batch in host memory, matrices built from
// coordinates), in a call-local buffer of `cap` entries of
// fac_entry_bytes(n, copy) each.
struct FacHead {
  long long b;
  double la, ph;
  int par, flag;
};
__host__ __device__ constexpr long long fac_factors_offset(int n) {
  return (long long)sizeof(FacHead) + (((long long)n * 4 + 15) & ~15ll);
}
__host__ __device__ constexpr long long fac_copy_offset(int n) {
  return fac_factors_offset(n) + (long long)n * n * 16;
}
__host__ __device__ constexpr long long fac_entry_bytes(int n, bool copy = false) {
  return fac_copy_offset(n) + (copy ? (long long)n * n * 16 : 0ll);
}
struct FacList {
  unsigned long long *count;
  unsigned char *buf;
  long long cap;
  int copy;
};

// FP64 refactorisation of matrix sb of `src` (reloaded into M), results into
// slot b, status |= flag (FALLBACK, or FP64 for the routed share). With
// scratch (cs, 17 <= n <= 40) the log-determinant gets the extended-precision
// correction (fp64_correct_warp for n <= 32, fp64_correct_group on this one
// warp above), which brings the FP64 route within the mixed mode's error
// bound on ill-conditioned matrices. With a list (fl, n <= 32) the factors
// are listed instead, while it has room, for the correction pass
// (lup_mixed_fac_correct_kernel) to finish the result.
template <class Src, bool COHERENT = false>
__device__ void fallback_fp64_src(const Src &src, long long sb, int n, double2 *M, int lds,
                                  double *hold, int lane, long long b, double *logabs,
                                  double *phase, int8_t *parity, int32_t *status,
                                  int flag = LUFQHE_ST_FALLBACK,
                                  const CorrScratch *cs = nullptr,
                                  const FacList *fl = nullptr) {
  __syncwarp();
  src.template load<COHERENT>(sb, n, M, lds, lane);
  int par = 0;
  const bool correct = cs != nullptr && n >= kCorrectMinN && n <= kCorrectMaxN;
  int st = lup_fp64_warp<ARITH_FUSED>(M, lds, hold, n, lane, &par, correct ? cs->ints : nullptr);
  double la, ph;
  if (st == 0) {
    logdet_from_diag(M, lds, n, lane, par, &la, &ph);
    if (correct && n <= 32 && fl) {
      unsigned long long k = 0;
      if (lane == 0) k = atomicAdd(fl->count, 1ull);
      k = __shfl_sync(kFull, k, 0);
      if (k < (unsigned long long)fl->cap) {
        unsigned char *e = fl->buf + k * fac_entry_bytes(n, fl->copy != 0);
        if (lane == 0) *reinterpret_cast<FacHead *>(e) = FacHead{b, la, ph, par, flag};
        int *pe = reinterpret_cast<int *>(e + sizeof(FacHead));
        for (int i = lane; i < n; i += 32) pe[i] = cs->ints[i];
        double2 *fe = reinterpret_cast<double2 *>(e + fac_factors_offset(n));
        for (int q = lane; q < n * n; q += 32) fe[q] = M[(q / n) * lds + q % n];
        if (fl->copy) {
          double2 *ce = reinterpret_cast<double2 *>(e + fac_copy_offset(n));
          if constexpr (std::is_same<Src, DenseSource>::value) {
            for (int q = lane; q < n * n; q += 32) ce[q] = source_entry(src, sb, n, q / n, q % n);
          } else {
            // a row per lane, built once (entries rebuilt one at a time would
            // repeat their row's recurrence)
            for (int r = lane; r < n; r += 32) {
              auto it = source_row(src, sb, n, r);
              for (int c = 0; c < n; ++c) ce[r * n + c] = it.next();
            }
          }
        }
        __syncwarp();
        return;
      }
    }
    if (correct && n <= 32) {
      fp64_correct_warp(src, sb, n, M, lds, *cs, lane, &la, &ph);
    } else if (correct) {
      const double2 c = fp64_correct_one_warp(src, sb, n, M, lds, *cs, lane);
      la += c.x;
      ph += c.y;
    }
  } else if (st == LUFQHE_ST_SINGULAR) {
    la = -INFINITY;
    ph = 0.0;
  } else {
    la = NAN;
    ph = NAN;
    par = 0;
  }
  if (lane == 0) {
    logabs[b] = la;
    if (phase) phase[b] = ph;
    if (parity) parity[b] = (int8_t)par;
    if (status) status[b] = st | flag;
  }
}

// Same for one dense matrix at src (row stride lda).
template <bool COHERENT = false>
__device__ void fallback_fp64(const double2 *src, int n, int lda, double2 *M, int lds,
                              double *hold, int lane, long long b, double *logabs, double *phase,
                              int8_t *parity, int32_t *status, int flag = LUFQHE_ST_FALLBACK,
                              const CorrScratch *cs = nullptr) {
  fallback_fp64_src<DenseSource, COHERENT>(DenseSource{src, lda}, 0, n, M, lds, hold, lane, b,
                                           logabs, phase, parity, status, flag, cs);
}

// ---------------------------------------------------------------------------
// Register-tiled form of the same method for a compile-time n <= 32.
//  * FP32 LUP as above (shared memory, right-looking, rows of F and of the
//    hi/lo copy swap together).
//  * Residual: the 32 lanes form a 4 x 8 grid; lane (r, c) owns the entries
//    (4a + r, 8b + c) and accumulates their float-float Dot2 sums in registers
//    over t, reading l_it and u_tk from shared memory (operands that do not
//    contribute are zero, which leaves a Dot2 step exact and branch-free).
//  * Solves and log det(I + E): E stays in registers on the same lane grid
//    (mixed_finish_tile).
template <int N>
struct TileGeom {
  static constexpr int LDS = N + 1;
  static constexpr int SA = (N + 3) / 4;  // row slots per lane
  static constexpr int SB = (N + 7) / 8;  // column slots per lane
};

// Float-float residual for the NA row slots from a0 of the 4 x 8 lane grid:
// lane (r, c) owns entries (4a + r, 8b + c); R is written into the float2
// view of HL (row stride N + 1). a0 is a run-time value so that both halves
// of the row slots can share one copy of this (large, unrolled) code.
template <int N, int NA>
__device__ __forceinline__ void residual_rows(float4 *HL, const float2 *F, int lane, int A0) {
  constexpr int LDS = N + 1;
  constexpr int SB = TileGeom<N>::SB;
  if constexpr (NA > 0) {
    const int tr = lane >> 3, tc = lane & 7;
    float4 acc[NA][SB];
#pragma unroll
    for (int a = 0; a < NA; ++a)
#pragma unroll
      for (int b = 0; b < SB; ++b) {
        const int i = 4 * (A0 + a) + tr, k = 8 * b + tc;
        acc[a][b] = (i < N && k < N) ? HL[i * LDS + k] : make_float4(0.f, 0.f, 0.f, 0.f);
      }
    // rows of this pass end at 4 (A0 + NA); steps beyond their last row add nothing
    const int TEND = min(4 * (A0 + NA), N);
#pragma unroll 1
    for (int t = 0; t < TEND; ++t) {
      float2 Lv[NA], Uv[SB];
#pragma unroll
      for (int a = 0; a < NA; ++a) {
        const int i = 4 * (A0 + a) + tr;
        Lv[a] = make_float2(0.f, 0.f);
        if (i == t) Lv[a] = make_float2(1.f, 0.f);
        else if (i > t && i < N) Lv[a] = F[i * LDS + t];
      }
#pragma unroll
      for (int b = 0; b < SB; ++b) {
        const int k = 8 * b + tc;
        Uv[b] = make_float2(0.f, 0.f);
        if (k >= t && k < N) Uv[b] = F[t * LDS + k];
      }
      // slots whose rows and columns all lie before t have nothing left to add
#pragma unroll
      for (int a = 0; a < NA; ++a) {
        if (4 * (A0 + a) + 3 < t) continue;
#pragma unroll
        for (int b = 0; b < SB; ++b) {
          if (8 * b + 7 < t) continue;
          dot2_csub(acc[a][b], Lv[a], Uv[b]);
        }
      }
    }
    float2 *Rm = reinterpret_cast<float2 *>(HL);
    __syncwarp();
#pragma unroll
    for (int a = 0; a < NA; ++a)
#pragma unroll
      for (int b = 0; b < SB; ++b) {
        const int i = 4 * (A0 + a) + tr, k = 8 * b + tc;
        if (i < N && k < N)
          Rm[i * LDS + k] = make_float2(__fadd_rn(acc[a][b].x, acc[a][b].z),
                                        __fadd_rn(acc[a][b].y, acc[a][b].w));
      }
    __syncwarp();
  }
}

// The residual of the back substitution E1 = U^-1 Y, G = Y - U E1, in
// float-float for the NA row slots from A0 of the 4 x 8 lane grid, written
// over Y in Rm (each lane reads and writes only the entries it owns there; E1
// is read from Eb by all lanes). The same Dot2 steps as residual_rows; U is
// the upper triangle of F, so row i sums over j >= i.
template <int N, int NA>
__device__ __forceinline__ void refine_rows(float2 *Rm, const float2 *F, const float2 *Eb,
                                            int lane, int A0) {
  constexpr int LDS = N + 1;
  constexpr int SB = TileGeom<N>::SB;
  if constexpr (NA > 0) {
    const int tr = lane >> 3, tc = lane & 7;
    float4 acc[NA][SB];
#pragma unroll
    for (int a = 0; a < NA; ++a)
#pragma unroll
      for (int b = 0; b < SB; ++b) {
        const int i = 4 * (A0 + a) + tr, k = 8 * b + tc;
        const float2 y = (i < N && k < N) ? Rm[i * LDS + k] : make_float2(0.f, 0.f);
        acc[a][b] = make_float4(y.x, y.y, 0.f, 0.f);
      }
#pragma unroll 1
    for (int j = 4 * A0; j < N; ++j) {
      float2 Uv[NA], Ev[SB];
#pragma unroll
      for (int a = 0; a < NA; ++a) {
        const int i = 4 * (A0 + a) + tr;
        Uv[a] = (i <= j) ? F[i * LDS + j] : make_float2(0.f, 0.f);
      }
#pragma unroll
      for (int b = 0; b < SB; ++b) {
        const int k = 8 * b + tc;
        Ev[b] = k < N ? Eb[j * LDS + k] : make_float2(0.f, 0.f);
      }
      // slots whose rows all lie below j have nothing to add
#pragma unroll
      for (int a = 0; a < NA; ++a) {
        if (4 * (A0 + a) > j) continue;
#pragma unroll
        for (int b = 0; b < SB; ++b) dot2_csub(acc[a][b], Uv[a], Ev[b]);
      }
    }
#pragma unroll
    for (int a = 0; a < NA; ++a)
#pragma unroll
      for (int b = 0; b < SB; ++b) {
        const int i = 4 * (A0 + a) + tr, k = 8 * b + tc;
        if (i < N && k < N)
          Rm[i * LDS + k] = make_float2(__fadd_rn(acc[a][b].x, acc[a][b].z),
                                        __fadd_rn(acc[a][b].y, acc[a][b].w));
      }
  }
}

__device__ __forceinline__ float2 shfl2(float2 v, int src) {
  return make_float2(__shfl_sync(kFull, v.x, src), __shfl_sync(kFull, v.y, src));
}

// Steps 4-6 of the tile path with E in registers on the 4 x 8 lane grid of
// the residual (lane (r, c) holds entries (4a + r, 8b + c)). Every element
// update is the same cfms / cmulf as in mixed_finish, so E and log det(I + E)
// come out bit for bit as there; only the order of the ||E||_F sum differs.
//  * Step t = 4s + u of a solve or of the elimination: the outer loop over the
//    row slot s is unrolled, the inner loop over u is not, so register indices
//    are compile-time while the code stays small. Row t lives in lanes (u, *)
//    at slot s and reaches the other lanes by shuffle; l_it and u_it are
//    shared-memory reads that 8 lanes share.
//  * log det(I + E): unpivoted elimination. Rows and columns up to t are
//    never read after step t, so the update runs over whole slots without
//    masks; the pivots 1 + d_t go to `diag` and their logs are taken one per
//    lane at the end.
// Outcome of the tile path for one matrix.
// TILE_NONFINITE: a NaN or Inf entry (only for matrices whose load did not
// check it: the bulk-copied ones)
enum { TILE_REJECT = 0, TILE_ACCEPT = 1, TILE_REFINE = 2, TILE_NONFINITE = 3 };

template <int N>
struct TileRegs {
  static constexpr int LDS = N + 1;
  static constexpr int SA = (N + 3) / 4;
  static constexpr int SB = (N + 7) / 8;
};

// This lane's entries of an N x N float2 array (row stride N + 1) to or from
// registers on the lane grid; entries outside the matrix read as zero.
template <int N>
__device__ __forceinline__ void tile_load(const float2 *Rm, float2 (&Y)[TileRegs<N>::SA][TileRegs<N>::SB],
                                          int lane) {
  constexpr int LDS = N + 1, SA = TileRegs<N>::SA, SB = TileRegs<N>::SB;
  const int r = lane >> 3, c = lane & 7;
#pragma unroll
  for (int a = 0; a < SA; ++a)
#pragma unroll
    for (int b = 0; b < SB; ++b) {
      const int i = 4 * a + r, k = 8 * b + c;
      Y[a][b] = (i < N && k < N) ? Rm[i * LDS + k] : make_float2(0.f, 0.f);
    }
}
template <int N>
__device__ __forceinline__ void tile_store(float2 *Rm,
                                           const float2 (&Y)[TileRegs<N>::SA][TileRegs<N>::SB],
                                           int lane) {
  constexpr int LDS = N + 1, SA = TileRegs<N>::SA, SB = TileRegs<N>::SB;
  const int r = lane >> 3, c = lane & 7;
#pragma unroll
  for (int a = 0; a < SA; ++a)
#pragma unroll
    for (int b = 0; b < SB; ++b) {
      const int i = 4 * a + r, k = 8 * b + c;
      if (i < N && k < N) Rm[i * LDS + k] = Y[a][b];
    }
}

// 4a. Y = L^-1 Y (unit lower) in place on the lane grid.
template <int N>
__device__ __forceinline__ void tile_fwd_solve(const float2 *F,
                                               float2 (&Y)[TileRegs<N>::SA][TileRegs<N>::SB],
                                               int lane) {
  constexpr int LDS = N + 1, SA = TileRegs<N>::SA, SB = TileRegs<N>::SB;
  const int r = lane >> 3, c = lane & 7;
  const float2 zero = make_float2(0.f, 0.f);
#pragma unroll
  for (int s = 0; s < SA; ++s) {
#pragma unroll 1
    for (int u = 0; u < 4; ++u) {
      const int t = 4 * s + u;
      if (t >= N - 1) break;
      float2 yt[SB];
#pragma unroll
      for (int b = 0; b < SB; ++b) yt[b] = shfl2(Y[s][b], u * 8 + c);
      {
        const bool below = r > u && 4 * s + r < N;
        const float2 l = below ? F[(4 * s + r) * LDS + t] : zero;
#pragma unroll
        for (int b = 0; b < SB; ++b) {
          const float2 v = cfms(Y[s][b], l, yt[b]);
          Y[s][b] = below ? v : Y[s][b];
        }
      }
#pragma unroll
      for (int a = s + 1; a < SA; ++a) {
        const int i = 4 * a + r;
        const float2 l = i < N ? F[i * LDS + t] : zero;
#pragma unroll
        for (int b = 0; b < SB; ++b) Y[a][b] = cfms(Y[a][b], l, yt[b]);
      }
    }
  }
}

// 4b. E = U^-1 Y in place: row t is scaled by 1/u_tt, then removed from the
// rows above. The reciprocals of the diagonal are taken first, one per lane,
// into `rdiag` (N float2 of scratch).
template <int N>
__device__ __forceinline__ void tile_bwd_solve(const float2 *F,
                                               float2 (&Y)[TileRegs<N>::SA][TileRegs<N>::SB],
                                               float2 *rdiag, int lane) {
  constexpr int LDS = N + 1, SA = TileRegs<N>::SA, SB = TileRegs<N>::SB;
  const int r = lane >> 3, c = lane & 7;
  const float2 zero = make_float2(0.f, 0.f);
  __syncwarp();
  if (lane < N) rdiag[lane] = crcpf(F[lane * LDS + lane]);
  __syncwarp();
#pragma unroll
  for (int s = SA - 1; s >= 0; --s) {
#pragma unroll 1
    for (int u = 3; u >= 0; --u) {
      const int t = 4 * s + u;
      if (t >= N) continue;
      const float2 dinv = rdiag[t];
      float2 et[SB];
#pragma unroll
      for (int b = 0; b < SB; ++b) {
        et[b] = cmulf(shfl2(Y[s][b], u * 8 + c), dinv);
        Y[s][b] = r == u ? et[b] : Y[s][b];
      }
      {
        const bool above = r < u;
        const float2 uu = above ? F[(4 * s + r) * LDS + t] : zero;
#pragma unroll
        for (int b = 0; b < SB; ++b) {
          const float2 v = cfms(Y[s][b], uu, et[b]);
          Y[s][b] = above ? v : Y[s][b];
        }
      }
#pragma unroll
      for (int a = 0; a < s; ++a) {
        const float2 uu = F[(4 * a + r) * LDS + t];
#pragma unroll
        for (int b = 0; b < SB; ++b) Y[a][b] = cfms(Y[a][b], uu, et[b]);
      }
    }
  }
}

// 6 (first half). Complex float-float product of the diagonal of U.
template <int N>
__device__ __forceinline__ CFF tile_diag_product(const float2 *F, int lane) {
  constexpr int LDS = N + 1;
  CFF acc = {1.0f, 0.0f, 0.0f, 0.0f, 0};
  if (lane < N) {
    const float2 u = F[lane * LDS + lane];
    CFF v = {u.x, 0.0f, u.y, 0.0f, 0};
    ff_renorm(v);
    acc = ff_cmul(acc, v);
  }
#pragma unroll
  for (int off = 16; off; off >>= 1) acc = ff_cmul(acc, shfl_cff(acc, off, true));
  return shfl_cff(acc, 0, false);
}

// ||E||_F^2, summed on lane 0's order and broadcast.
template <int N>
__device__ __forceinline__ float tile_frob2(const float2 (&Y)[TileRegs<N>::SA][TileRegs<N>::SB]) {
  constexpr int SA = TileRegs<N>::SA, SB = TileRegs<N>::SB;
  float f = 0.0f;
#pragma unroll
  for (int a = 0; a < SA; ++a)
#pragma unroll
    for (int b = 0; b < SB; ++b) f = __fmaf_rn(Y[a][b].x, Y[a][b].x, __fmaf_rn(Y[a][b].y, Y[a][b].y, f));
#pragma unroll
  for (int off = 16; off; off >>= 1) f += __shfl_xor_sync(kFull, f, off);
  return __shfl_sync(kFull, f, 0);
}

// 5. log det(I + E) for an accepted E (||E||_F^2 = f). Small E: the series
// tr E - tr(E^2)/2 + r with |r| <= ||E||_F^3 / (3 (1 - ||E||_F)), taken when
// that bound is below 1e-12 max(1, |log|det||) (la_est is within 1 of
// |log|det|| here, so la_est - 1 is a safe lower bound). Otherwise the
// unpivoted elimination of I + E on the lane grid, its pivots 1 + d_t to
// `diag` and their logs taken one per lane.
template <int N>
__device__ __forceinline__ void tile_logdet_ipe(float2 *Rm, float2 *diag,
                                                float2 (&Y)[TileRegs<N>::SA][TileRegs<N>::SB],
                                                int lane, float f, float la_est, float2 &corr) {
  constexpr int LDS = N + 1, SA = TileRegs<N>::SA, SB = TileRegs<N>::SB;
  const int r = lane >> 3, c = lane & 7;
  const float2 zero = make_float2(0.f, 0.f);
  const float nf = sqrtf(f);
  if (nf * f <= 3e-12f * fmaxf(1.0f, la_est - 1.0f) * (1.0f - nf)) {
    // tr E: entry (t, t) sits in slot (t / 4, t / 8) of lane (t % 4, t % 8), so slot a
    // holds a diagonal entry in the lanes with c = 4 (a % 2) + r
    float2 tr = zero, t2 = zero;
#pragma unroll
    for (int a = 0; a < SA; ++a)
      if (c == 4 * (a & 1) + r && 4 * a + r < N) {
        tr.x += Y[a][a >> 1].x;
        tr.y += Y[a][a >> 1].y;
      }
    // tr(E^2) = sum_ik E_ik E_ki, the transposed entries through shared memory
    __syncwarp();
    tile_store<N>(Rm, Y, lane);
    __syncwarp();
#pragma unroll
    for (int a = 0; a < SA; ++a)
#pragma unroll
      for (int b = 0; b < SB; ++b) {
        const int i = 4 * a + r, k = 8 * b + c;
        if (i < N && k < N) {
          const float2 e = cmulf(Y[a][b], Rm[k * LDS + i]);
          t2.x += e.x;
          t2.y += e.y;
        }
      }
#pragma unroll
    for (int off = 16; off; off >>= 1) {
      tr.x += __shfl_xor_sync(kFull, tr.x, off);
      tr.y += __shfl_xor_sync(kFull, tr.y, off);
      t2.x += __shfl_xor_sync(kFull, t2.x, off);
      t2.y += __shfl_xor_sync(kFull, t2.y, off);
    }
    corr = make_float2(__shfl_sync(kFull, __fmaf_rn(-0.5f, t2.x, tr.x), 0),
                       __shfl_sync(kFull, __fmaf_rn(-0.5f, t2.y, tr.y), 0));
    return;
  }
#pragma unroll
  for (int s = 0; s < SA; ++s) {
    const int q = s >> 1;  // column slot of t = 4s + u (compile-time)
#pragma unroll 1
    for (int u = 0; u < 4; ++u) {
      const int t = 4 * s + u;
      if (t >= N) break;
      const int ct = 4 * (s & 1) + u;  // lane column of t
      const float2 d = shfl2(Y[s][q], u * 8 + ct);
      if (lane == 0) diag[t] = d;
      if (t == N - 1) break;
      const float2 rp = crcpf(make_float2(1.0f + d.x, d.y));
      float2 et[SB];
#pragma unroll
      for (int b = q; b < SB; ++b) et[b] = shfl2(Y[s][b], u * 8 + c);
#pragma unroll
      for (int a = s; a < SA; ++a) {
        const float2 l = cmulf(shfl2(Y[a][q], r * 8 + ct), rp);
#pragma unroll
        for (int b = q; b < SB; ++b) Y[a][b] = cfms(Y[a][b], l, et[b]);
      }
    }
  }
  __syncwarp();
  float cre = 0.0f, cim = 0.0f;
  if (lane < N) {
    const float2 d = diag[lane];
    cre = __fmaf_rn(0.5f, log1pf(__fmaf_rn(d.x, d.x, __fmaf_rn(d.y, d.y, 2.0f * d.x))), cre);
    cim += atan2f(d.y, 1.0f + d.x);
  }
#pragma unroll
  for (int off = 16; off; off >>= 1) {
    cre += __shfl_xor_sync(kFull, cre, off);
    cim += __shfl_xor_sync(kFull, cim, off);
  }
  corr = make_float2(__shfl_sync(kFull, cre, 0), __shfl_sync(kFull, cim, 0));
}

__device__ __forceinline__ float tile_la_est(const CFF &prod, int exp_sum) {
  return fabsf((float)(prod.e + exp_sum)) * 0.6931472f;
}

// Steps 4-6 of the tile path with E in registers on the 4 x 8 lane grid of
// the residual (lane (r, c) holds entries (4a + r, 8b + c)). Every element
// update is the same cfms / cmulf as in mixed_finish, so E and log det(I + E)
// come out bit for bit as there; only the order of the ||E||_F sum differs.
//  * Step t = 4s + u of a solve or of the elimination: the outer loop over the
//    row slot s is unrolled, the inner loop over u is not, so register indices
//    are compile-time while the code stays small. Row t lives in lanes (u, *)
//    at slot s and reaches the other lanes by shuffle; l_it and u_it are
//    shared-memory reads that 8 lanes share.
//  * log det(I + E): unpivoted elimination. Rows and columns up to t are
//    never read after step t, so the update runs over whole slots without
//    masks.
// REFINE: a matrix whose ||E||_F is within theta but above the relative cap
// returns TILE_REFINE with Y = L^-1 R left in Rm (for a refinement of the back
// substitution elsewhere); without it such a matrix is rejected.
template <int N, bool REFINE>
__device__ int mixed_finish_tile(const float2 *F, float2 *Rm, float2 *diag, int lane, float theta2,
                                 int exp_sum, CFF &prod, float2 &corr) {
  float2 Y[TileRegs<N>::SA][TileRegs<N>::SB];
  tile_load<N>(Rm, Y, lane);
  tile_fwd_solve<N>(F, Y, lane);
  if constexpr (REFINE) tile_store<N>(Rm, Y, lane);  // own entries only
  tile_bwd_solve<N>(F, Y, diag, lane);
  prod = tile_diag_product<N>(F, lane);
  const float f = tile_frob2<N>(Y);
  const float la_est = tile_la_est(prod, exp_sum);
  if (!(f <= theta2)) return TILE_REJECT;
  const float rel_cap = kCorrRelCap * fmaxf(1.0f, la_est);
  if (!(f <= rel_cap * rel_cap)) return REFINE ? TILE_REFINE : TILE_REJECT;
  tile_logdet_ipe<N>(Rm, diag, Y, lane, f, la_est, corr);
  return TILE_ACCEPT;
}

// One refinement step of the back substitution for a matrix the FP32 pass
// left as TILE_REFINE: F holds L\U, Rm holds Y = L^-1 R, Eb is N (N + 1)
// float2 of scratch. E1 = U^-1 Y in FP32; the residual G = Y - U E1 in
// float-float (the LU residual's Dot2 steps); E = E1 + U^-1 G. Against the
// double-double oracle the error left in log det(I + E) is then about
// 1.2e-7 ||E||_F at most on lowest-Landau-level matrices, so the relative cap
// is kRefinedRelCap instead of kCorrRelCap. True if accepted (corr set).
template <int N>
__device__ bool mixed_refine_tile(const float2 *F, float2 *Rm, float2 *Eb, float2 *diag, int lane,
                                  float theta2, float la_est, float2 &corr) {
  constexpr int LDS = N + 1, SA = TileRegs<N>::SA, SB = TileRegs<N>::SB;
  float2 Y[SA][SB];
  tile_load<N>(Rm, Y, lane);
  tile_bwd_solve<N>(F, Y, diag, lane);
  tile_store<N>(Eb, Y, lane);
  __syncwarp();
  if constexpr (SA % 2 == 0) {
#pragma unroll 1
    for (int h = 0; h < 2; ++h) refine_rows<N, SA / 2>(Rm, F, Eb, lane, h * (SA / 2));
  } else {
    refine_rows<N, SA / 2>(Rm, F, Eb, lane, 0);
    refine_rows<N, SA - SA / 2>(Rm, F, Eb, lane, SA / 2);
  }
  tile_load<N>(Rm, Y, lane);  // G, own entries
  tile_bwd_solve<N>(F, Y, diag, lane);
  const int r = lane >> 3, c = lane & 7;
#pragma unroll
  for (int a = 0; a < SA; ++a)
#pragma unroll
    for (int b = 0; b < SB; ++b) {
      const int i = 4 * a + r, k = 8 * b + c;
      if (i < N && k < N) {
        const float2 e1 = Eb[i * LDS + k];
        Y[a][b] = make_float2(__fadd_rn(e1.x, Y[a][b].x), __fadd_rn(e1.y, Y[a][b].y));
      }
    }
  const float f = tile_frob2<N>(Y);
  if (!(f <= theta2)) return false;
  const float rel_cap = kRefinedRelCap * fmaxf(1.0f, la_est);
  if (!(f <= rel_cap * rel_cap)) return false;
  tile_logdet_ipe<N>(Rm, diag, Y, lane, f, la_est, corr);
  return true;
}

template <int N, bool REFINE = false>
__device__ int mixed_factor_tile_ex(float4 *HL, float2 *F, int *er, int *ec, int lane,
                                    float theta2, CFF &prod, int &exp_sum, float2 &corr, int &par) {
  constexpr int LDS = TileGeom<N>::LDS;
  constexpr int SA = TileGeom<N>::SA;
  constexpr int SB = TileGeom<N>::SB;
  const double2 *A = reinterpret_cast<const double2 *>(HL);

  // 1. exponents, columns first (a NaN or Inf entry has the exponent field
  //    of 2^1024: the matrix is reported non-finite)
  int esum = 0;
  bool bad = false;
  if (lane < N) {
    int m = -2000;
#pragma unroll 4
    for (int i = 0; i < N; ++i) m = max(m, cexp_field(A[i * LDS + lane]));
    bad = m == 1024;
    if (m == -2000) m = 0;
    ec[lane] = m;
    esum = m;
  }
  if (__any_sync(kFull, bad)) return TILE_NONFINITE;
  __syncwarp();
  if (lane < N) {
    int m = -2000;
#pragma unroll 4
    for (int k = 0; k < N; ++k) {
      int e = cexp_field(A[lane * LDS + k]);
      if (e != -2000) m = max(m, e - ec[k]);
    }
    if (m == -2000) m = 0;
    er[lane] = m;
    esum += m;
  }
  exp_sum = __reduce_add_sync(kFull, esum);
  __syncwarp();
  // 2. split (each lane rewrites the entries it read)
  for (int e = lane; e < N * N; e += 32) {
    const int i = e / N, k = e - i * N;
    const int idx = i * LDS + k;
    const double2 v = A[idx];
    const int s = er[i] + ec[k];
    float xh, xl, yh, yl;
    split_scaled(v.x, s, xh, xl);
    split_scaled(v.y, s, yh, yl);
    F[idx] = make_float2(xh, yh);
    HL[idx] = make_float4(xh, yh, xl, yl);
  }
  __syncwarp();

  // 3. FP32 LUP. Pivot: the largest |Re| + |Im| in column t at or below row
  //    t, from one warp max over a key that holds the value's bits with the
  //    low 5 mantissa bits replaced by 31 - row (values within 2^-18 of each
  //    other tie; ties go to the smaller row). Trailing update on the 4 x 8
  //    lane grid: each lane reads l_it for its rows and u_tk for its columns
  //    once per step, zero outside the trailing block (which leaves those
  //    entries as they are), and updates its entries in the slots that reach
  //    the block.
  par = 0;
  {
    const int tr = lane >> 3, tc = lane & 7;
    const float2 zero = make_float2(0.f, 0.f);
    for (int t = 0; t < N; ++t) {
      unsigned int key = 0u;
      if (lane >= t && lane < N) {
        const float2 v = F[lane * LDS + t];
        const float m = fabsf(v.x) + fabsf(v.y);
        key = (__float_as_uint(m) & ~31u) | (31u - (unsigned int)lane);
      }
      key = __reduce_max_sync(kFull, key);
      const float best = __uint_as_float(key & ~31u);
      if (!(best > 0.0f) || !(best < INFINITY)) return TILE_REJECT;  // zero/NaN/Inf pivot
      const int bi = 31 - (int)(key & 31u);
      if (bi != t) {
        if (lane < N) {
          const float2 a = F[bi * LDS + lane];
          F[bi * LDS + lane] = F[t * LDS + lane];
          F[t * LDS + lane] = a;
          const float4 c = HL[bi * LDS + lane];
          HL[bi * LDS + lane] = HL[t * LDS + lane];
          HL[t * LDS + lane] = c;
        }
        par ^= 1;
      }
      __syncwarp();
      const float2 rp = crcpf_approx(F[t * LDS + t]);
      if (lane > t && lane < N) F[lane * LDS + t] = cmulf(F[lane * LDS + t], rp);
      __syncwarp();
      if (t + 1 < N) {
        float2 lv[SA], uv[SB];
#pragma unroll
        for (int a = 0; a < SA; ++a) {
          const int i = 4 * a + tr;
          lv[a] = (i > t && i < N) ? F[i * LDS + t] : zero;
        }
#pragma unroll
        for (int b = 0; b < SB; ++b) {
          const int k = 8 * b + tc;
          uv[b] = (k > t && k < N) ? F[t * LDS + k] : zero;
        }
#pragma unroll
        for (int a = 0; a < SA; ++a) {
          if (4 * a + 3 <= t) continue;
#pragma unroll
          for (int b = 0; b < SB; ++b) {
            if (8 * b + 7 <= t) continue;
            const int i = 4 * a + tr, k = 8 * b + tc;
            if ((N % 4 == 0 || i < N) && (N % 8 == 0 || k < N))
              F[i * LDS + k] = cfms(F[i * LDS + k], lv[a], uv[b]);
          }
        }
        __syncwarp();
      }
    }
  }

  // 4. residual R = P A^ - L U (float-float) in a 4 x 8 lane grid, in two
  //    passes over halves of the row slots (half the accumulator registers).
  //    R overwrites the front of HL as a float2 array; pass 1 writes rows
  //    below the ones pass 2 still reads, so the passes never collide.
  if constexpr (SA % 2 == 0) {
#pragma unroll 1
    for (int h = 0; h < 2; ++h) residual_rows<N, SA / 2>(HL, F, lane, h * (SA / 2));
  } else {
    residual_rows<N, SA / 2>(HL, F, lane, 0);
    residual_rows<N, SA - SA / 2>(HL, F, lane, SA / 2);
  }
  float2 *Rm = reinterpret_cast<float2 *>(HL);  // R, then E, row stride LDS

  // 5-6. solves, acceptance, log det(I + E) and the diagonal product
  // (the exponent arrays are free again: they hold the pivots of step 5)
  return mixed_finish_tile<N, REFINE>(F, Rm, reinterpret_cast<float2 *>(er), lane, theta2, exp_sum,
                                      prod, corr);
}

// Tile path for kernels that keep their FP64 refactorisations in place: a
// TILE_REFINE matrix has its back substitution refined right here (refine
// true), so the outcome is the batched call's (FP32 pass, then refinement).
template <int N>
__device__ __forceinline__ bool mixed_factor_tile(float4 *HL, float2 *F, int *er, int *ec, int lane,
                                                  float theta2, CFF &prod, int &exp_sum,
                                                  float2 &corr, int &par, bool refine) {
  const int code =
      mixed_factor_tile_ex<N, true>(HL, F, er, ec, lane, theta2, prod, exp_sum, corr, par);
  if (code == TILE_ACCEPT) return true;
  if (code != TILE_REFINE || !refine) return false;
  float2 *Rm = reinterpret_cast<float2 *>(HL);
  return mixed_refine_tile<N>(F, Rm, Rm + N * (N + 1), reinterpret_cast<float2 *>(er), lane, theta2,
                              tile_la_est(prod, exp_sum), corr);
}

template <int N>
constexpr size_t tile_smem_per_warp() {
  return (size_t)N * (N + 1) * (sizeof(float4) + sizeof(float2)) + 2 * (size_t)N * sizeof(double) +
         2 * (size_t)N * sizeof(int);
}


}  // namespace
}  // namespace mixed
}  // namespace lufqhe
