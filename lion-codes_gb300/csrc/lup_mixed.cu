// Mixed-precision batched complex LUP determinant.
//
// Per matrix (one warp, shared memory), with FP64 used only where accuracy
// needs it and almost all arithmetic on the FP32 and integer pipes, which on
// GB300 run far faster than FP64:
//  1. power-of-two column-then-row equilibration A^ = D_r^-1 A D_c^-1, chosen
//     from the exponent fields (exact; log|det D| is added back in FP64);
//  2. split of every scaled FP64 entry into float hi + lo by integer
//     operations (48 significant bits kept);
//  3. FP32 complex LUP of hi with partial pivoting on |Re|+|Im|; alongside,
//     the residual R = P A^ - L U is accumulated exactly in float-float
//     (Ogita-Rump-Oishi Dot2: TwoProd + TwoSum per real product), starting
//     from hi + lo, so R carries FP64-level accuracy although every operation
//     is an FP32 one;
//  4. E = U^-1 L^-1 R by FP32 triangular solves;
//  5. log det(I + E) by an unpivoted FP32 LU that keeps the identity implicit
//     (only the small offsets are stored), log1p/atan2 of each pivot;
//  6. log|det| = log|prod u_jj| (complex float-float product, one FP64 log
//     and atan2 per matrix, deferred and done for 32 matrices at once by the
//     32 lanes) + equilibration + Re log det(I+E); phase likewise.
// A matrix whose ||E||_F exceeds the threshold, or whose FP32 factorisation
// meets a zero or non-finite pivot, is refactorised by the FP64 warp routine
// (reference pivot rule, fused arithmetic) and flagged LUFQHE_ST_FALLBACK.
// The permutation parity reported is that of the pivoting actually used.

#include <cmath>

#include "lup_fp64.cuh"

namespace lufqhe {

namespace {

constexpr int kMaxWarpsMixed = 8;
// ||E||_F / max(1, |log|det||) above which the correction may miss 1e-10
// relative accuracy. E comes from FP32 triangular solves, whose rounding
// leaves an absolute error of about 1e-6 * ||E||_F in log det(I + E)
// (measured on lowest-Landau-level matrices against a double-double oracle);
// 5e-5 keeps that near 5e-11 relative, half the 1e-10 target.
constexpr float kCorrRelCap = 5e-5f;

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

// s + c -= l*u exactly up to the compensation's own rounding (Dot2 step).
__device__ __forceinline__ void dot2_csub(float4 &sc, float2 l, float2 u) {
  float p1, e1, p2, e2, p3, e3, p4, e4, s, t1, t2;
  two_prod(l.x, u.x, p1, e1);
  two_prod(l.y, u.y, p2, e2);
  two_prod(l.x, u.y, p3, e3);
  two_prod(l.y, u.x, p4, e4);
  // real: s - p1 + p2
  two_sum(sc.x, -p1, s, t1);
  two_sum(s, p2, sc.x, t2);
  sc.z = __fadd_rn(sc.z, __fadd_rn(__fsub_rn(t1, e1), __fadd_rn(t2, e2)));
  // imag: s - p3 - p4
  two_sum(sc.y, -p3, s, t1);
  two_sum(s, -p4, sc.y, t2);
  sc.w = __fadd_rn(sc.w, __fsub_rn(__fadd_rn(t1, t2), __fadd_rn(e3, e4)));
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
  two_sum(p1, -p2, s, t);
  float lo = t + e1 - e2 + (a.xh * b.xl + a.xl * b.xh) - (a.yh * b.yl + a.yl * b.yh);
  r.xh = __fadd_rn(s, lo);
  r.xl = __fsub_rn(lo, __fsub_rn(r.xh, s));
  two_sum(p3, p4, s, t);
  lo = t + e3 + e4 + (a.xh * b.yl + a.xl * b.yh) + (a.yh * b.xl + a.yl * b.xh);
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

  // 4a. Y = L^-1 R (unit lower, forward)
  for (int t = 0; t + 1 < n; ++t) {
    const int rows = n - 1 - t;
    const int tot = rows * n;
    BlockWalk w(lane, n);
    for (int e = lane; e < tot; e += 32) {
      const int i = t + 1 + w.i, k = w.k;
      R[2 * (i * lds + k)] = cfms(R[2 * (i * lds + k)], S.Af[i * lds + t], R[2 * (t * lds + k)]);
      w.next(n);
    }
    __syncwarp();
  }
  // 4b. E = U^-1 Y (backward)
  for (int t = n - 1; t >= 0; --t) {
    const float2 r = crcpf(S.Af[t * lds + t]);
    for (int k = lane; k < n; k += 32) R[2 * (t * lds + k)] = cmulf(R[2 * (t * lds + k)], r);
    __syncwarp();
    const int tot = t * n;
    BlockWalk w(lane, n);
    for (int e = lane; e < tot; e += 32) {
      const int i = w.i, k = w.k;
      R[2 * (i * lds + k)] = cfms(R[2 * (i * lds + k)], S.Af[i * lds + t], R[2 * (t * lds + k)]);
      w.next(n);
    }
    __syncwarp();
  }

  // 6 (first half). complex float-float product of the diagonal of U; its
  // exponent gives log2|det| to within 2 before the correction is accepted
  {
    CFF acc = {1.0f, 0.0f, 0.0f, 0.0f, 0};
    for (int t = lane; t < n; t += 32) {
      float2 u = S.Af[t * lds + t];
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
      float2 v = R[2 * (w.i * lds + w.k)];
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
    const float2 d = R[2 * (t * lds + t)];
    const float2 r = crcpf(make_float2(1.0f + d.x, d.y));
    for (int i = t + 1 + lane; i < n; i += 32)
      R[2 * (i * lds + t)] = cmulf(R[2 * (i * lds + t)], r);
    __syncwarp();
    const int m = n - 1 - t;
    const int mm = m * m;
    BlockWalk w(lane, m);
    for (int e = lane; e < mm; e += 32) {
      const int i = t + 1 + w.i, k = t + 1 + w.k;
      R[2 * (i * lds + k)] = cfms(R[2 * (i * lds + k)], R[2 * (i * lds + t)], R[2 * (t * lds + k)]);
      w.next(m);
    }
    __syncwarp();
  }
  float cre = 0.0f, cim = 0.0f;
  for (int t = lane; t < n; t += 32) {
    const float2 d = R[2 * (t * lds + t)];
    cre += 0.5f * log1pf(__fmaf_rn(d.x, d.x, __fmaf_rn(d.y, d.y, 2.0f * d.x)));
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

__global__ void __launch_bounds__(kMaxWarpsMixed * 32)
    lup_mixed_kernel(const double2 *__restrict__ A, int n, int lda, long long batch,
                     float theta2, double *__restrict__ logabs, double *__restrict__ phase,
                     int8_t *__restrict__ parity, int32_t *__restrict__ status) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int warps = blockDim.x >> 5;
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int lds = n + 1;
  const size_t nl = (size_t)n * lds;
  MixedSmem S;
  unsigned char *base = smem_raw;
  S.SC = reinterpret_cast<float4 *>(base) + warp * nl;
  base += warps * nl * sizeof(float4);
  S.Af = reinterpret_cast<float2 *>(base) + warp * nl;
  base += warps * nl * sizeof(float2);
  S.hold = reinterpret_cast<double *>(base) + warp * 2 * n;
  base += warps * 2 * (size_t)n * sizeof(double);
  S.er = reinterpret_cast<int *>(base) + warp * 2 * n;
  S.ec = S.er + n;

  // deferred finalisation: lane L holds the L-th completed matrix
  long long slot_b = -1;
  CFF slot_p = {1.0f, 0.0f, 0.0f, 0.0f, 0};
  int slot_e = 0, slot_par = 0;
  float2 slot_c = make_float2(0.0f, 0.0f);
  int cnt = 0;

  auto flush = [&]() {
    if (lane < cnt && slot_b >= 0) {
      double re = (double)slot_p.xh + (double)slot_p.xl;
      double im = (double)slot_p.yh + (double)slot_p.yl;
      double la = 0.5 * log(re * re + im * im) + (double)slot_e * kLn2 + (double)slot_c.x;
      double ph = atan2(im, re) + (double)slot_c.y + (slot_par ? kPi : 0.0);
      logabs[slot_b] = la;
      if (phase) phase[slot_b] = wrap_phase(ph);
      if (parity) parity[slot_b] = (int8_t)slot_par;
      if (status) status[slot_b] = 0;
    }
    slot_b = -1;
    cnt = 0;
  };

  for (long long b = (long long)blockIdx.x * warps + warp; b < batch;
       b += (long long)gridDim.x * warps) {
    __syncwarp();
    const double2 *src = A + (size_t)b * n * lda;
    double2 *M = reinterpret_cast<double2 *>(S.SC);
    if (load_matrix_fp64(src, n, lda, M, lds, lane)) {
      if (lane == 0) {
        logabs[b] = NAN;
        if (phase) phase[b] = NAN;
        if (parity) parity[b] = 0;
        if (status) status[b] = LUFQHE_ST_NONFINITE;
      }
      continue;
    }
    CFF prod;
    int exp_sum, par;
    float2 corr;
    if (mixed_factor(S, n, lane, theta2, prod, exp_sum, corr, par)) {
      if (lane == cnt) {
        slot_b = b;
        slot_p = prod;
        slot_e = prod.e + exp_sum;
        slot_c = corr;
        slot_par = par;
      }
      if (++cnt == 32) flush();
    } else {
      // FP64 refactorisation of the original matrix
      __syncwarp();
      load_matrix_fp64(src, n, lda, M, lds, lane);
      int st = lup_fp64_warp<ARITH_FUSED>(M, lds, S.hold, n, lane, &par);
      double la, ph;
      if (st == 0) {
        logdet_from_diag(M, lds, n, lane, par, &la, &ph);
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
        if (status) status[b] = st | LUFQHE_ST_FALLBACK;
      }
    }
  }
  flush();
}

}  // namespace

size_t mixed_smem_per_warp(int n) {
  const int lds = n + 1;
  return (size_t)n * lds * (sizeof(float2) + sizeof(float4)) + 2 * (size_t)n * sizeof(double) +
         2 * (size_t)n * sizeof(int);
}

float g_mixed_theta = 0.1f;

int launch_mixed(const double2 *A, int n, int lda, long long batch, double *logabs,
                 double *phase, int8_t *parity, int32_t *status, cudaStream_t stream) {
  if (batch == 0) return LUFQHE_SUCCESS;
  const size_t per_warp = mixed_smem_per_warp(n);
  const size_t optin = device_smem_optin();
  int warps = (int)(optin / per_warp);
  if (warps > 4) warps = 4;
  if (warps < 1) {
    set_error("n=%d needs %zu bytes of shared memory per matrix; the device offers %zu", n,
              per_warp, optin);
    return LUFQHE_ERR_UNSUPPORTED_N;
  }
  const size_t smem = per_warp * warps;
  int rc = check_cuda(cudaFuncSetAttribute(lup_mixed_kernel,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                      "cudaFuncSetAttribute(mixed)");
  if (rc) return rc;
  int per_sm = 0;
  rc = check_cuda(
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, lup_mixed_kernel, warps * 32, smem),
      "occupancy(mixed)");
  if (rc) return rc;
  if (per_sm < 1) per_sm = 1;
  long long want = (batch + warps - 1) / warps;
  long long cap = (long long)device_sm_count() * per_sm;
  int grid = (int)(want < cap ? want : cap);
  const float theta2 = g_mixed_theta * g_mixed_theta;
  lup_mixed_kernel<<<grid, warps * 32, smem, stream>>>(A, n, lda, batch, theta2, logabs, phase,
                                                       parity, status);
  return check_cuda(cudaGetLastError(), "lup_mixed_kernel launch");
}

}  // namespace lufqhe
