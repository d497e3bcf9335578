// Extended-precision correction of an FP64 LUP log-determinant (n <= 32 by
// one warp, up to kCorrectMaxN by a warp group or one warp), for the results
// of the mixed mode's FP64 route.
//
// FP64 LUP on ill-conditioned orbital matrices misses 1e-10 in log|det| on a
// tail of the batch (about 1 in 10^4 matrices at n = 24, 2 in 10^3 at
// n = 32): the factors are backward stable, PA = LU + R with R of rounding
// size, but log det(LU) differs from log det(PA) by
//   log det(I + E) = tr E - tr(E^2)/2 + O(|E|^3),   E = (LU)^-1 R,
// which is what this step adds back. Two parts:
//  * R exactly: every product of two doubles is an exact integer of at most
//    106 bits; the terms of one entry (A'_ij and the products L_ik U_kj) are
//    summed modulo 2^64 on a fixed-point grid placed from the backward-error
//    bound of the factorisation (mod_mac below), so R_ij comes out exact up
//    to the final rounding to double (and a truncation 2^-45 below its
//    typical size). This is integer work (the ALU and IMAD pipes), not FP64
//    work, whose pipe is the narrow one on this GPU.
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

// R_ij is small next to the terms that produce it: LUP with partial pivoting
// is backward stable, |R_ij| <= n u sum_k |L_ik| |U_kj| <= n^2 2^-53 2^T for
// terms below 2^T. So the terms are summed in a 64-bit accumulator modulo
// 2^64 on a grid 2^(T - 103): the bits of every term above the window cancel
// exactly (the sum's are known to be zero), and the result, below
// 2^(T - 43) for n <= 32, is the accumulator read as a signed integer (3
// bits of margin); truncating each term below the grid costs at most n grid
// units, 2^-45 of a typical |R_ij|. T is the top-bit position of the entry's
// largest term, found by an exponent pass first.
//
// acc += (-1)^neg (m1 m2 >> r) mod 2^64, r >= 0 (m1, m2 < 2^53)
__device__ __forceinline__ void mod_mac(unsigned long long &acc, unsigned long long m1,
                                        unsigned long long m2, int r, bool neg) {
  const unsigned long long lo = m1 * m2, hi = __umul64hi(m1, m2);
  const int rr = min(r, 127);
  const unsigned long long v =
      rr >= 64 ? (hi >> (rr - 64)) : ((lo >> rr) | ((hi << 1) << (63 - rr)));
  acc = neg ? acc - v : acc + v;
}
// acc += (-1)^neg (m << s) mod 2^64 (s < 64; s < 0 shifts right)
__device__ __forceinline__ void mod_add(unsigned long long &acc, unsigned long long m, int s,
                                        bool neg) {
  const unsigned long long v = s >= 0 ? (m << s) : (s > -64 ? (m >> -s) : 0ull);
  acc = neg ? acc - v : acc + v;
}

// x 2^e rounded to float. For -1022 <= e <= 1023 the power of two is a normal
// double built from its bits and the product is the correctly rounded x 2^e,
// which is ldexp's result; ldexp (a longer FP64 sequence) covers the rest.
__device__ __forceinline__ float scale_to_float(double x, int e) {
  const double y = (e >= -1022 && e <= 1023)
                       ? __dmul_rn(x, __longlong_as_double((long long)(e + 1023) << 52))
                       : ldexp(x, e);
  return __double2float_rn(y);
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
// register-tiled kernels carry no correction code. Above n = 40 the scaled
// factors of the worst LLL matrices (z ~ CN(0, n)) are too ill-conditioned
// for the FP32 solves: on GB300, 8192 matrices per size, the correction took
// the results above 1e-10 from 7 to 0 at n = 33 and 38 to 2 at n = 40, but
// only 75 to 45 at n = 48 and 120 to 119 at n = 64, at 2.5-3x the cost of
// the factorisation; those sizes are left uncorrected.
constexpr int kCorrectMinN = 17;
constexpr int kCorrectMaxN = 40;

// Grid of the residual sums: 2^(T - 106 + bias) for an entry whose largest
// term is below 2^T. |R_ij| <= n^2 2^-53 2^T is n^2 2^(53 - bias) grid units,
// so the sum read as a signed 64-bit integer keeps 3 bits of margin with
// bias 3 for n <= 32 and bias 5 for n <= 64.
constexpr int kGridBias32 = 3;
constexpr int kGridBias64 = 5;

// Entry p of the level order (see fp64_correct_warp, step 2): R_ij = (PA -
// LU)_ij summed exactly modulo 2^64 on the grid, then scaled by the row and
// column scales into F[i * lds + j].
template <class Src>
__device__ __forceinline__ void residual_entry(const Src &src, long long sb, int n,
                                               const double2 *M, int lds, const int *perm,
                                               const int *sr, const int *sc, int p, int bias,
                                               float2 *F) {
  int m = (int)((float)n - sqrtf((float)(n * n - p)));
  while (m > 0 && m * (2 * n - m) > p) --m;
  while ((m + 1) * (2 * n - m - 1) <= p) ++m;
  const int off = p - m * (2 * n - m);
  const int i = off < n - m ? m : m + 1 + (off - (n - m));
  const int j = off < n - m ? m + off : m;
  const double2 a = source_entry(src, sb, n, perm[i], j);
  const ExactDouble ar = exact_split(a.x), ai = exact_split(a.y);
  // exponent pass: mx = the largest e(l) + e(u) (or A's, placed like a
  // product's), biased fields
  int mx = max(ar.e, ai.e) + 1022;
  for (int k = 0; k <= m; ++k) {  // k = m: the term with L_ii = 1 (i <= j) or U_jj
    const int el = k == i ? 1023 : exp_field_c(M[i * lds + k]);
    mx = max(mx, el + exp_field_c(M[k * lds + j]));
  }
  // grid unit 2^g, g = mx - 2150 + bias: a product m1 m2 2^(e1 + e2 - 2150)
  // is shifted right by g - (e1 + e2 - 2150), A's m 2^(e - 1075) left by
  // (e - 1075) - g
  unsigned long long re = 0ull, im = 0ull;
  mod_add(re, ar.m, ar.e - mx + 1075 - bias, ar.neg != 0u);
  mod_add(im, ai.m, ai.e - mx + 1075 - bias, ai.neg != 0u);
  for (int k = 0; k <= m; ++k) {
    const double2 u = M[k * lds + j];
    // L_ii = 1 (k == i, a select: the lanes of a step differ here)
    const double2 l = k == i ? make_double2(1.0, 0.0) : M[i * lds + k];
    const ExactDouble ur = exact_split(u.x), ui = exact_split(u.y);
    const ExactDouble lr = exact_split(l.x), li = exact_split(l.y);
    // re -= lr ur - li ui; im -= lr ui + li ur
    const int r0 = mx + bias;
    mod_mac(re, lr.m, ur.m, r0 - lr.e - ur.e, (lr.neg ^ ur.neg ^ 1u) != 0u);
    mod_mac(re, li.m, ui.m, r0 - li.e - ui.e, (li.neg ^ ui.neg) != 0u);
    mod_mac(im, lr.m, ui.m, r0 - lr.e - ui.e, (lr.neg ^ ui.neg ^ 1u) != 0u);
    mod_mac(im, li.m, ur.m, r0 - li.e - ur.e, (li.neg ^ ur.neg ^ 1u) != 0u);
  }
  const int sh = mx - 2150 + bias - sr[i] - sc[j];
  F[i * lds + j] = make_float2(scale_to_float((double)(long long)re, sh),
                               scale_to_float((double)(long long)im, sh));
}

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
  //    run the lanes one after another).
  for (int p0 = 0; p0 < n * n; p0 += 32) {
    const int p = p0 + lane;
    if (p < n * n) residual_entry(src, sb, n, M, lds, perm, sr, sc, p, kGridBias32, F);
    __syncwarp();
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
        v = make_float2(scale_to_float(d.x, s), scale_to_float(d.y, s));
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

// Barrier of a single warp, for fp64_correct_group run by one warp.
struct WarpBarrier {
  __device__ __forceinline__ void sync() const { __syncwarp(); }
};

// The same correction by the nthr threads of a warp group (a multiple of 32,
// synchronised by bar, as in lup_fp64_group), or by one warp (WarpBarrier),
// for n <= kCorrectMaxN (n <= 64 fits its grid), on FP64 factors of either
// routine; for n <= 32 its result is fp64_correct_warp's bit for bit (the
// same operations per entry and per column; the trace partials of warps
// without a column are zero). red: 4 floats of shared scratch per warp
// (unused, and may be null, for one warp). Returns the correction to add to
// (log|det|, phase), the same value in every thread, or (0, 0) if a scaled
// quantity left float's range. The steps are those of fp64_correct_warp with
// rows, columns and residual entries dealt over the group; the column scales
// are reduced per warp, then across warps with shared atomics. Inlined into
// its callers: compiled out of line, its warp-group form returned wrong
// corrections in one kernel of the library (n = 24, three warps), while the
// same code inlined, or out of line in a module of its own, was right on the
// same matrices.
template <class Src, class Bar>
__device__ __forceinline__ double2 fp64_correct_group(const Src src, long long sb, int n,
                                                   double2 *M, int lds, const CorrScratch cs,
                                                   int tid, int nthr, Bar bar, float *red) {
  float2 *const F = cs.F;
  const int *perm = cs.ints;
  int *sr = cs.ints + n;
  float2 *rd = reinterpret_cast<float2 *>(cs.hold);
  int *sc = reinterpret_cast<int *>(rd + n);
  const int lane = tid & 31, warp = tid >> 5, nw = nthr >> 5;
  // 1. scales
  for (int j = tid; j < n; j += nthr) sc[j] = -4000;
  for (int i = tid; i < n; i += nthr) {
    auto it = source_row(src, sb, n, perm[i]);
    int er = -2000;
    for (int j = 0; j < n; ++j) er = max(er, exp_field_c(it.next()) - 1023);
    sr[i] = er;
  }
  bar.sync();
  for (int i0 = 0; i0 < n; i0 += nthr) {
    if (i0 + warp * 32 >= n) continue;  // warp-uniform: no row of this warp
    const int i = i0 + tid;
    const bool live = i < n;
    auto it = source_row(src, sb, n, perm[live ? i : i0]);
    const int er = live ? sr[i] : 0;
    for (int j = 0; j < n; ++j) {
      const int c = __reduce_max_sync(kFull, live ? exp_field_c(it.next()) - 1023 - er : -4000);
      if (lane == 0) atomicMax(&sc[j], c);
    }
  }
  bar.sync();
  // 2. R = PA - LU exactly, scaled into F, level-dealt over the group
  for (int p0 = 0; p0 < n * n; p0 += nthr) {
    const int p = p0 + tid;
    if (p < n * n)
      residual_entry(src, sb, n, M, lds, perm, sr, sc, p, n <= 32 ? kGridBias32 : kGridBias64,
                     F);
    __syncwarp();
  }
  bar.sync();
  // 3. the scaled factors in FP32, in place over M (reads of a chunk before
  //    its writes, which overlap entries of this chunk or earlier ones)
  float2 *Mf = reinterpret_cast<float2 *>(M);
  for (int q0 = 0; q0 < n * lds; q0 += nthr) {
    const int q = q0 + tid;
    float2 v = make_float2(0.f, 0.f);
    if (q < n * lds) {
      const int i = q / lds, k = q - i * lds;
      if (k < n) {
        const double2 d = M[q];
        const int sh = k < i ? sr[k] - sr[i] : -sr[i] - sc[k];
        v = make_float2(scale_to_float(d.x, sh), scale_to_float(d.y, sh));
      }
    }
    bar.sync();
    if (q < n * lds) Mf[q] = v;
    bar.sync();
  }
  for (int i = tid; i < n; i += nthr) {
    const float2 d = Mf[i * lds + i];
    const float r = 1.0f / fmaf(d.x, d.x, d.y * d.y);
    rd[i] = make_float2(d.x * r, -d.y * r);
  }
  bar.sync();
  // 4. E = U^-1 L^-1 R in the scaled frame, column j by thread j
  for (int j = tid; j < n; j += nthr) {
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
  bar.sync();
  // 5. tr E and tr E^2: per thread, per warp, then the warps in order
  float2 t1 = make_float2(0.f, 0.f), t2 = make_float2(0.f, 0.f);
  for (int j = tid; j < n; j += nthr) {
    const float2 e = F[j * lds + j];
    t1.x += e.x;
    t1.y += e.y;
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
  float4 t = make_float4(t1.x, t1.y, t2.x, t2.y);
  if (nw > 1) {
    if (lane == 0) {
      red[4 * warp] = t1.x;
      red[4 * warp + 1] = t1.y;
      red[4 * warp + 2] = t2.x;
      red[4 * warp + 3] = t2.y;
    }
    bar.sync();
    t = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int w = 0; w < nw; ++w) {
      t.x += red[4 * w];
      t.y += red[4 * w + 1];
      t.z += red[4 * w + 2];
      t.w += red[4 * w + 3];
    }
    bar.sync();
  }
  const double dx = (double)t.x - 0.5 * (double)t.z;
  const double dy = (double)t.y - 0.5 * (double)t.w;
  return (isfinite(dx) && isfinite(dy)) ? make_double2(dx, dy) : make_double2(0.0, 0.0);
}

// The one-warp form (synchronised by __syncwarp only), kept out of line: it
// runs on a few percent of the matrices of the kernels that call it.
template <class Src>
__device__ __noinline__ double2 fp64_correct_one_warp(const Src src, long long sb, int n,
                                                      double2 *M, int lds, const CorrScratch cs,
                                                      int lane) {
  return fp64_correct_group(src, sb, n, M, lds, cs, lane, 32, WarpBarrier(),
                            static_cast<float *>(nullptr));
}

}  // namespace lufqhe
