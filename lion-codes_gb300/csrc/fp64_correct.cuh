// Extended-precision correction of an FP64 LUP log-determinant (n <= 32, one
// warp), for the results of the mixed mode's FP64 route.
//
// FP64 LUP on ill-conditioned orbital matrices misses 1e-10 in log|det| on a
// tail of the batch (about 1 in 10^4 matrices at n = 24, 2 in 10^3 at
// n = 32): the factors are backward stable, PA = LU + R with R of rounding
// size, but log det(LU) differs from log det(PA) by
//   log det(I + E) = tr E - tr(E^2)/2 + O(|E|^3),   E = (LU)^-1 R,
// which is what this step adds back. Two parts:
//  * R exactly: every product of two doubles is an exact integer of at most
//    106 bits; the terms of one entry (A'_ij and the products L_ik U_kj) are
//    summed in a signed 128-bit fixed-point accumulator (two 64-bit words)
//    whose grid lies 114 bits below its largest term, so R_ij is exact up to the final rounding
//    to double (terms more than 2^114 below the largest are dropped, far
//    below R's own size). This is integer work (the ALU and IMAD pipes), not
//    FP64 work, whose pipe is the narrow one on this GPU.
//  * E, to a few digits, by FP32 triangular solves in the row- and
//    column-scaled frame D_r PA D_c = (D_r L D_r^-1)(D_r U D_c) (powers of
//    two from the rows of PA and the columns of D_r PA), where every quantity
//    is within float's range; E there is D_c^-1 E D_c, a similarity, so tr E
//    and tr E^2 are unchanged.
// The lanes take R's entries in steps of equal work, and columns for the
// solves (lane j: column j).
#pragma once

#include "lup_fp64.cuh"

namespace lufqhe {

// |x| = m 2^(e - 1075) with m < 2^53 an integer; e is the biased exponent
// field (1 for zero and subnormals, whose m has no implicit bit).
struct ExactDouble {
  unsigned long long m;
  int e;
  unsigned neg;
};

__device__ __forceinline__ ExactDouble exact_split(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  int e = (int)((b >> 52) & 0x7ff);
  unsigned long long m = b & 0xFFFFFFFFFFFFFull;
  if (e)
    m |= 1ull << 52;
  else
    e = 1;
  return {m, e, (unsigned)(b >> 63)};
}

__device__ __forceinline__ int exp_field(double x) {
  const int e = (int)(((unsigned long long)__double_as_longlong(x) >> 52) & 0x7ff);
  return e ? e : 1;
}
__device__ __forceinline__ int exp_field_c(double2 v) { return max(exp_field(v.x), exp_field(v.y)); }

// Signed 128-bit fixed-point accumulator as two 64-bit words (two's
// complement), with the few operations the residual needs written on the
// words: the compiler's generic 128-bit arithmetic is far slower.
struct Acc128 {
  unsigned long long lo;
  long long hi;
};

// (hi, lo) = m1 m2, exact (m1, m2 < 2^53)
__device__ __forceinline__ void mul_53x53(unsigned long long m1, unsigned long long m2,
                                          unsigned long long &hi, unsigned long long &lo) {
  lo = m1 * m2;
  hi = __umul64hi(m1, m2);
}

// acc += (-1)^neg (hi, lo) 2^sh for sh <= 8 and (hi, lo) < 2^106; bits below
// the grid dropped. Branch-free (selects only): the lanes of a warp shift by
// different amounts, and branches on them would split the warp.
__device__ __forceinline__ void acc_add_shifted(Acc128 &acc, unsigned long long hi,
                                                unsigned long long lo, int sh, bool neg) {
  // pre-shift by 8 (at most 114 bits), then a right shift by r = 8 - sh >= 0
  hi = (hi << 8) | (lo >> 56);
  lo <<= 8;
  const int r = min(8 - sh, 128);
  const bool big = r >= 64;
  const int rr = big ? min(r - 64, 63) : r;
  unsigned long long nlo = big ? (hi >> rr) : ((lo >> rr) | ((hi << 1) << (63 - rr)));
  unsigned long long nhi = big ? 0ull : (hi >> rr);
  nlo = r >= 128 ? 0ull : nlo;
  // two's complement of the term when it is subtracted
  const unsigned long long clo = ~nlo + 1ull;
  const unsigned long long chi = ~nhi + (clo == 0ull ? 1ull : 0ull);
  nlo = neg ? clo : nlo;
  nhi = neg ? chi : nhi;
  const unsigned long long slo = acc.lo + nlo;
  acc.hi = (long long)((unsigned long long)acc.hi + nhi + (slo < nlo ? 1ull : 0ull));
  acc.lo = slo;
}

// acc += (-1)^neg a b on the grid 2^(base - 2150)
__device__ __forceinline__ void exact_mac(Acc128 &acc, const ExactDouble &a, const ExactDouble &b,
                                          unsigned neg, int base) {
  unsigned long long hi, lo;
  mul_53x53(a.m, b.m, hi, lo);
  acc_add_shifted(acc, hi, lo, a.e + b.e - base, ((a.neg ^ b.neg ^ neg) & 1u) != 0);
}

// acc += a on the same grid: the mantissa placed like a product's (m 2^53,
// 106 bits), so the shift stays within acc_add_shifted's range (A' lies at
// most 2^61 grid units above a product-sized term, 8 after the placement)
__device__ __forceinline__ void exact_add(Acc128 &acc, const ExactDouble &a, int base) {
  acc_add_shifted(acc, a.m >> 11, a.m << 53, a.e + 1075 - 53 - base, (a.neg & 1u) != 0);
}

// acc >>= s (s > 0, arithmetic), the bits below the grid dropped
__device__ __forceinline__ void exact_rescale(Acc128 &acc, int s) {
  if (s >= 127) {
    acc.lo = acc.hi < 0 ? ~0ull : 0ull;
    acc.hi = acc.hi < 0 ? -1ll : 0ll;
  } else if (s >= 64) {
    acc.lo = (unsigned long long)(acc.hi >> (s - 64));
    acc.hi = acc.hi < 0 ? -1ll : 0ll;
  } else {
    acc.lo = (acc.lo >> s) | ((unsigned long long)acc.hi << (64 - s));
    acc.hi >>= s;
  }
}

// sign and magnitude apart: a negative value's two's-complement words would
// cancel in the sum (hi = -1, lo = 2^64 - |a|)
__device__ __forceinline__ double exact_to_double(Acc128 a) {
  const bool neg = a.hi < 0;
  unsigned long long lo = a.lo, hi = (unsigned long long)a.hi;
  if (neg) {  // negate
    lo = ~lo + 1ull;
    hi = ~hi + (lo == 0ull ? 1ull : 0ull);
  }
  const double v = fma((double)hi, 18446744073709551616.0, (double)lo);
  return neg ? -v : v;
}

__device__ __forceinline__ float2 cf_sub_mul(float2 s, float2 a, float2 b) {  // s - a b
  return make_float2(fmaf(a.y, b.y, fmaf(-a.x, b.x, s.x)), fmaf(-a.y, b.x, fmaf(-a.x, b.y, s.y)));
}
__device__ __forceinline__ float2 cf_mul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}

// Rows of a matrix source walked in column order (the correction re-reads
// the matrix the factorisation was given: L2-resident device matrices, or
// orbital rows rebuilt from z with the bits load() gave them).
struct DenseRow {
  const double2 *p;
  __device__ __forceinline__ double2 next() { return __ldcg(p++); }
  __device__ __forceinline__ void skip(int j) { p += j; }
};
__device__ __forceinline__ DenseRow source_row(const DenseSource &s, long long b, int n, int r) {
  return DenseRow{s.A + (size_t)b * n * s.lda + (size_t)r * s.lda};
}
__device__ __forceinline__ double2 source_entry(const DenseSource &s, long long b, int n, int r,
                                                int c) {
  return __ldcg(s.A + (size_t)b * n * s.lda + (size_t)r * s.lda + c);
}
struct Dense32Row {
  const float2 *p;
  __device__ __forceinline__ double2 next() { return Dense32Source::widen(__ldcg(p++)); }
  __device__ __forceinline__ void skip(int j) { p += j; }
};
__device__ __forceinline__ Dense32Row source_row(const Dense32Source &s, long long b, int n,
                                                 int r) {
  return Dense32Row{s.A + (size_t)b * n * s.lda + (size_t)r * s.lda};
}
__device__ __forceinline__ double2 source_entry(const Dense32Source &s, long long b, int n, int r,
                                                int c) {
  return Dense32Source::widen(__ldcg(s.A + (size_t)b * n * s.lda + (size_t)r * s.lda + c));
}
// the same operation sequence as lll_row_rn
struct LllRow {
  double2 z;
  double w, px, py;
  __device__ __forceinline__ double2 next() {
    const double2 v = make_double2(__dmul_rn(px, w), __dmul_rn(py, w));
    const double nx = __dsub_rn(__dmul_rn(px, z.x), __dmul_rn(py, z.y));
    const double ny = __dadd_rn(__dmul_rn(px, z.y), __dmul_rn(py, z.x));
    px = nx;
    py = ny;
    return v;
  }
  __device__ __forceinline__ void skip(int j) {
    for (int k = 0; k < j; ++k) next();
  }
};
__device__ __forceinline__ LllRow source_row(const LllSource &s, long long b, int n, int r) {
  LllRow it;
  it.z = __ldcg(s.Z + (size_t)b * n + r);
  it.w = exp(__dmul_rn(-__dadd_rn(__dmul_rn(it.z.x, it.z.x), __dmul_rn(it.z.y, it.z.y)), 0.25));
  it.px = 1.0;
  it.py = 0.0;
  return it;
}
// entry c of the row: the row's operation sequence up to c
__device__ __forceinline__ double2 source_entry(const LllSource &s, long long b, int n, int r,
                                                int c) {
  LllRow it = source_row(s, b, n, r);
  it.skip(c);
  return it.next();
}

// The FP64 route's error on ill-conditioned orbital matrices grows with n: at
// n <= 16 it stays two orders of magnitude inside the bound, so the small
// register-tiled kernels carry no correction code.
constexpr int kCorrectMinN = 17;

// Shared memory the correction borrows from its caller: F (n x lds float2),
// ints (2n: the pivot order, then the row scale exponents) and hold (2n
// doubles, free once the factorisation is done: the column scale exponents and
// the reciprocal diagonal of the scaled U).
struct CorrScratch {
  float2 *F;
  int *ints;
  double *hold;
};

// M: the FP64 factors of PA (L\U, row stride lds) as lup_fp64_warp leaves
// them, perm[j] the row of A in pivoted row j. On return M has been
// overwritten (with FP32 copies of the scaled factors) and (*la, *ph) carry
// the correction, unless a scaled quantity left float's range (then they are
// unchanged). Warp-uniform; n <= 32. Kept out of line: it runs on a few
// percent of the matrices, and inlined its registers would be the kernels'.
template <class Src>
__device__ __noinline__ void fp64_correct_warp(const Src src, long long sb, int n, double2 *M,
                                               int lds, const CorrScratch cs, int lane, double *la,
                                               double *ph) {
  // every pointer in a local: stores through one must not force reloads of a
  // struct the compiler cannot prove they leave alone
  float2 *const F = cs.F;
  const int *perm = cs.ints;
  int *sr = cs.ints + n;
  float2 *rd = reinterpret_cast<float2 *>(cs.hold);  // n float2, then n ints (of 16n bytes)
  int *sc = reinterpret_cast<int *>(rd + n);
  const bool row_lane = lane < n;
  // 1. scales: sr_i = exponent of the largest entry of row i of PA, sc_j that
  //    of column j of D_r PA (unbiased; the columns reduced over the warp)
  int er = -2000;
  if (row_lane) {
    auto it = source_row(src, sb, n, perm[lane]);
    for (int j = 0; j < n; ++j) er = max(er, exp_field_c(it.next()) - 1023);
    sr[lane] = er;
  }
  {
    auto it = source_row(src, sb, n, row_lane ? perm[lane] : 0);
    for (int j = 0; j < n; ++j) {
      int c = row_lane ? exp_field_c(it.next()) - 1023 - er : -4000;
#pragma unroll
      for (int off = 16; off; off >>= 1) c = max(c, __shfl_xor_sync(kFull, c, off));
      if (lane == 0) sc[j] = c;
    }
  }
  __syncwarp();
  // 2. R = PA - LU exactly, scaled into F. Entry (i, j) sums min(i, j) + 1
  //    products. The entries are dealt out by level m = min(i, j) (level m:
  //    (m, m..n-1), then (m+1..n-1, m); it starts at entry m (2n - m) of
  //    the order), 32 at a time, so the lanes of a step do equal work and
  //    stay converged (with lanes each walking their own runs, the warp had
  //    run the lanes one after another). The grid follows the largest term
  //    seen so far: a larger one shifts the accumulators down, dropping bits
  //    below the new grid.
  {
    for (int p0 = 0; p0 < n * n; p0 += 32) {
      const int p = p0 + lane;
      if (p < n * n) {
        int m = (int)((float)n - sqrtf((float)(n * n - p)));
        while (m > 0 && m * (2 * n - m) > p) --m;
        while ((m + 1) * (2 * n - m - 1) <= p) ++m;
        const int off = p - m * (2 * n - m);
        const int i = off < n - m ? m : m + 1 + (off - (n - m));
        const int j = off < n - m ? m + off : m;
        const double2 a = source_entry(src, sb, n, perm[i], j);
        const ExactDouble ar = exact_split(a.x), ai = exact_split(a.y);
        int mx = max(ar.e, ai.e) + 1022;
        Acc128 re = {0ull, 0ll}, im = {0ull, 0ll};
        exact_add(re, ar, mx - 8);
        exact_add(im, ai, mx - 8);
        for (int k = 0; k <= m; ++k) {  // k = m: the term with L_ii = 1 (i <= j) or U_jj
          const double2 u = M[k * lds + j];
          const ExactDouble ur = exact_split(u.x), ui = exact_split(u.y);
          const int eu = max(ur.e, ui.e);
          // L_ii = 1 (k == i, a select: the lanes of a step differ here)
          const double2 l = k == i ? make_double2(1.0, 0.0) : M[i * lds + k];
          const ExactDouble lr = exact_split(l.x), li = exact_split(l.y);
          const int t = max(lr.e, li.e) + eu;
          if (t > mx) {
            exact_rescale(re, t - mx);
            exact_rescale(im, t - mx);
            mx = t;
          }
          // re -= lr ur - li ui; im -= lr ui + li ur
          exact_mac(re, lr, ur, 1u, mx - 8);
          exact_mac(re, li, ui, 0u, mx - 8);
          exact_mac(im, lr, ui, 1u, mx - 8);
          exact_mac(im, li, ur, 1u, mx - 8);
        }
        const int sh = mx - 8 - 2150 - sr[i] - sc[j];
        F[i * lds + j] = make_float2(__double2float_rn(ldexp(exact_to_double(re), sh)),
                                     __double2float_rn(ldexp(exact_to_double(im), sh)));
      }
      __syncwarp();
    }
  }
  // 3. the scaled factors in FP32, in place over M (entry q of the float2
  //    view overlaps entry q/2 of the double2 view, which an earlier chunk, or
  //    this one before the barrier, has read)
  float2 *Mf = reinterpret_cast<float2 *>(M);
  for (int q0 = 0; q0 < n * lds; q0 += 32) {
    const int q = q0 + lane;
    float2 v = make_float2(0.f, 0.f);
    if (q < n * lds) {
      const int i = q / lds, k = q - i * lds;
      if (k < n) {
        const double2 d = M[q];
        const int s = k < i ? sr[k] - sr[i] : -sr[i] - sc[k];
        v = make_float2(__double2float_rn(ldexp(d.x, s)), __double2float_rn(ldexp(d.y, s)));
      }
    }
    __syncwarp();
    if (q < n * lds) Mf[q] = v;
    __syncwarp();
  }
  if (row_lane) {
    const float2 d = Mf[lane * lds + lane];
    const float r = 1.0f / fmaf(d.x, d.x, d.y * d.y);
    rd[lane] = make_float2(d.x * r, -d.y * r);
  }
  __syncwarp();
  // 4. E = U^-1 L^-1 R in the scaled frame, column j on lane j, in place in F
  //    (two partial sums per row, so the loads of one step overlap the
  //    arithmetic of the other)
  if (row_lane) {
    const int j = lane;
    for (int i = 1; i < n; ++i) {
      float2 s0 = F[i * lds + j], s1 = make_float2(0.f, 0.f);
      int k = 0;
#pragma unroll 2
      for (; k + 1 < i; k += 2) {
        s0 = cf_sub_mul(s0, Mf[i * lds + k], F[k * lds + j]);
        s1 = cf_sub_mul(s1, Mf[i * lds + k + 1], F[(k + 1) * lds + j]);
      }
      if (k < i) s0 = cf_sub_mul(s0, Mf[i * lds + k], F[k * lds + j]);
      F[i * lds + j] = make_float2(s0.x + s1.x, s0.y + s1.y);
    }
    for (int i = n - 1; i >= 0; --i) {
      float2 s0 = F[i * lds + j], s1 = make_float2(0.f, 0.f);
      int k = i + 1;
#pragma unroll 2
      for (; k + 1 < n; k += 2) {
        s0 = cf_sub_mul(s0, Mf[i * lds + k], F[k * lds + j]);
        s1 = cf_sub_mul(s1, Mf[i * lds + k + 1], F[(k + 1) * lds + j]);
      }
      if (k < n) s0 = cf_sub_mul(s0, Mf[i * lds + k], F[k * lds + j]);
      F[i * lds + j] = cf_mul(make_float2(s0.x + s1.x, s0.y + s1.y), rd[i]);
    }
  }
  __syncwarp();
  // 5. tr E and tr E^2
  float2 t1 = make_float2(0.f, 0.f), t2 = make_float2(0.f, 0.f);
  if (row_lane) {
    const int j = lane;
    t1 = F[j * lds + j];
    for (int i = 0; i < n; ++i) {
      const float2 p = cf_mul(F[i * lds + j], F[j * lds + i]);
      t2.x += p.x;
      t2.y += p.y;
    }
  }
#pragma unroll
  for (int off = 16; off; off >>= 1) {
    t1.x += __shfl_xor_sync(kFull, t1.x, off);
    t1.y += __shfl_xor_sync(kFull, t1.y, off);
    t2.x += __shfl_xor_sync(kFull, t2.x, off);
    t2.y += __shfl_xor_sync(kFull, t2.y, off);
  }
  const double dx = (double)t1.x - 0.5 * (double)t2.x;
  const double dy = (double)t1.y - 0.5 * (double)t2.y;
  if (isfinite(dx) && isfinite(dy)) {
    *la += dx;
    *ph += dy;
  }
  __syncwarp();
}

}  // namespace lufqhe
