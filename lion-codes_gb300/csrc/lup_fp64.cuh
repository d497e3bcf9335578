// Warp-cooperative FP64 complex LUP of one matrix held in shared memory.
//
// Used by the plain kernels and as the FP64 refactorisation of the mixed
// kernel. The pivot rule and arithmetic are the reference's CPU Crout
// (LU-fqhe/src/LUCoreCPU.cu:112-267):
//   row scale   holder_i = max_k |Re a_ik|                     (:145-160)
//   pivot       argmax_i |Re a_ij| / holder_i, ties to last i   (:189-213)
//   swap        rows j <-> p, holder_p = holder_j, d = -d        (:216-232)
//   multipliers a_ij /= a_jj for i > j                           (:234-251)
// Right-looking elimination subtracts the products l_ik*u_kj from every
// entry in the same order k = 0, 1, ... as Crout's left-looking sums, so with
// ARITH_REF the factors are bit-identical to the reference's arithmetic.
#pragma once

#include "lufqhe_internal.cuh"

namespace lufqhe {

// Walk the row-major index e = i*m + k of an m-column block in steps of 32
// starting at `lane`, without a division per step.
struct BlockWalk {
  int i, k, di, dk;
  __device__ __forceinline__ BlockWalk(int lane, int m) {
    i = lane / m;
    k = lane - i * m;
    di = 32 / m;
    dk = 32 - di * m;
  }
  __device__ __forceinline__ void next(int m) {
    k += dk;
    i += di;
    if (k >= m) {
      k -= m;
      ++i;
    }
  }
};

// The same walk for any step (threads of a warp group).
struct StrideWalk {
  int i, k, di, dk;
  __device__ __forceinline__ StrideWalk(int start, int step, int m) {
    i = start / m;
    k = start - i * m;
    di = step / m;
    dk = step - di * m;
  }
  __device__ __forceinline__ void next(int m) {
    k += dk;
    i += di;
    if (k >= m) {
      k -= m;
      ++i;
    }
  }
};

// Coalesced load of an n x n complex128 matrix (row stride lda) into shared
// memory (row stride lds). Returns true (warp-uniform) if any entry is NaN/Inf.
// COHERENT loads through L2 only (no read-only / L1 path), for matrices that
// a long-running kernel itself rewrites between reads.
template <bool COHERENT = false>
__device__ __forceinline__ bool load_matrix_fp64(const double2 *__restrict__ src, int n, int lda,
                                                 double2 *M, int lds, int lane) {
  bool bad = false;
  const int nn = n * n;
  BlockWalk w(lane, n);
  for (int e = lane; e < nn; e += 32) {
    const double2 *p = src + (size_t)w.i * lda + w.k;
    double2 v = COHERENT ? __ldcg(p) : __ldg(p);
    bad |= !finite_c(v);
    M[w.i * lds + w.k] = v;
    w.next(n);
  }
  bad = __any_sync(kFull, bad);
  __syncwarp();
  return bad;
}

// Row of a lowest-Landau-level orbital matrix: M_ik = z^k exp(-|z|^2/4) for
// k < n, by repeated complex multiplication. Every operation is explicitly
// rounded (no contraction), so every kernel that builds a row gets the same
// bits. Returns false if an entry is NaN/Inf.
__device__ __forceinline__ bool lll_row_rn(double2 z, int n, double2 *row) {
  const double w = exp(__dmul_rn(-__dadd_rn(__dmul_rn(z.x, z.x), __dmul_rn(z.y, z.y)), 0.25));
  double px = 1.0, py = 0.0;
  bool ok = true;
  for (int k = 0; k < n; ++k) {
    const double2 v = make_double2(__dmul_rn(px, w), __dmul_rn(py, w));
    ok &= finite_c(v);
    row[k] = v;
    const double nx = __dsub_rn(__dmul_rn(px, z.x), __dmul_rn(py, z.y));
    const double ny = __dadd_rn(__dmul_rn(px, z.y), __dmul_rn(py, z.x));
    px = nx;
    py = ny;
  }
  return ok;
}

// Where the batched kernels take matrix b from.
//  * DenseSource: n x n complex128 matrices in the reference layout (matrix b
//    at b*n*lda, row stride lda).
//  * LllSource: LLL orbital matrices built in shared memory from n particle
//    coordinates per matrix (z of matrix b at b*n), so a call reads 16n bytes
//    per matrix instead of 16n^2.
// load() fills M (row stride lds) and returns true (warp-uniform) if an entry
// is NaN/Inf; first() is entry (0,0), which the FP64 routing hashes.
struct DenseSource {
  const double2 *A;
  int lda;
  template <bool COHERENT = false>
  __device__ __forceinline__ bool load(long long b, int n, double2 *M, int lds, int lane) const {
    return load_matrix_fp64<COHERENT>(A + (size_t)b * n * lda, n, lda, M, lds, lane);
  }
  __device__ __forceinline__ double2 first(long long b, int n) const {
    return __ldg(A + (size_t)b * n * lda);
  }
  // all threads of the CTA; true (CTA-uniform) if an entry is NaN/Inf
  __device__ __forceinline__ bool load_group(long long b, int n, double2 *M, int lds, int tid,
                                             int nthr) const {
    const double2 *src = A + (size_t)b * n * lda;
    bool bad = false;
    StrideWalk w(tid, nthr, n);
    for (int e = tid; e < n * n; e += nthr) {
      const double2 v = __ldg(src + (size_t)w.i * lda + w.k);
      bad |= !finite_c(v);
      M[w.i * lds + w.k] = v;
      w.next(n);
    }
    return __syncthreads_or(bad);
  }
};

// complex64 matrices in the reference layout: the reference's own buffer type
// (LUCoreGPU::CALL takes float2 matrices, LU-fqhe/inc/LUCoreGPU.h:47). Each
// entry is widened to FP64 as it is loaded, which is exact, so a complex64
// batch gives the results of its complex128 copy bit for bit.
struct Dense32Source {
  const float2 *A;
  int lda;
  __device__ __forceinline__ static double2 widen(float2 v) {
    return make_double2((double)v.x, (double)v.y);
  }
  template <bool COHERENT = false>
  __device__ __forceinline__ bool load(long long b, int n, double2 *M, int lds, int lane) const {
    const float2 *src = A + (size_t)b * n * lda;
    bool bad = false;
    BlockWalk w(lane, n);
    for (int e = lane; e < n * n; e += 32) {
      const float2 *p = src + (size_t)w.i * lda + w.k;
      const double2 v = widen(COHERENT ? __ldcg(p) : __ldg(p));
      bad |= !finite_c(v);
      M[w.i * lds + w.k] = v;
      w.next(n);
    }
    bad = __any_sync(kFull, bad);
    __syncwarp();
    return bad;
  }
  __device__ __forceinline__ double2 first(long long b, int n) const {
    return widen(__ldg(A + (size_t)b * n * lda));
  }
  __device__ __forceinline__ bool load_group(long long b, int n, double2 *M, int lds, int tid,
                                             int nthr) const {
    const float2 *src = A + (size_t)b * n * lda;
    bool bad = false;
    StrideWalk w(tid, nthr, n);
    for (int e = tid; e < n * n; e += nthr) {
      const double2 v = widen(__ldg(src + (size_t)w.i * lda + w.k));
      bad |= !finite_c(v);
      M[w.i * lds + w.k] = v;
      w.next(n);
    }
    return __syncthreads_or(bad);
  }
};

// Store of an FP64 entry into a caller's matrix of either element type (the
// in-place factors of the reference-shaped call; complex64 rounds to nearest).
__device__ __forceinline__ void store_entry(double2 *p, double2 v) { *p = v; }
__device__ __forceinline__ void store_entry(float2 *p, double2 v) {
  *p = make_float2(__double2float_rn(v.x), __double2float_rn(v.y));
}

struct LllSource {
  const double2 *Z;
  template <bool COHERENT = false>
  __device__ __forceinline__ bool load(long long b, int n, double2 *M, int lds, int lane) const {
    bool bad = false;
    for (int i = lane; i < n; i += 32) {
      const double2 z = COHERENT ? __ldcg(Z + (size_t)b * n + i) : __ldg(Z + (size_t)b * n + i);
      bad |= !lll_row_rn(z, n, M + i * lds);
    }
    bad = __any_sync(kFull, bad);
    __syncwarp();
    return bad;
  }
  __device__ __forceinline__ double2 first(long long b, int n) const {
    const double2 z = __ldg(Z + (size_t)b * n);
    const double w = exp(__dmul_rn(-__dadd_rn(__dmul_rn(z.x, z.x), __dmul_rn(z.y, z.y)), 0.25));
    return make_double2(__dmul_rn(1.0, w), __dmul_rn(0.0, w));
  }
  __device__ __forceinline__ bool load_group(long long b, int n, double2 *M, int lds, int tid,
                                             int nthr) const {
    bool bad = false;
    for (int i = tid; i < n; i += nthr) bad |= !lll_row_rn(__ldg(Z + (size_t)b * n + i), n, M + i * lds);
    return __syncthreads_or(bad);
  }
};

// RN(a / b) for b > 0 given y = RN(1/b): Markstein's correction (P. Markstein,
// IBM J. Res. Dev. 34(1), 1990): q0 = RN(a*y) is refined once to a faithful
// q1, then q2 = RN(q1 + RN(a - b*q1)*y) is the correctly rounded quotient when
// nothing over- or underflows. Outside the guarded ranges, and for a = 0, the
// quotient is taken from the hardware-independent IEEE division instead, so
// every result equals the correctly rounded a / b.
__device__ __forceinline__ double div_rn_markstein(double a, double b, double y, bool b_safe) {
  const long long lo = 0x0370000000000000ll;  // 2^-968
  const long long hi = 0x7c70000000000000ll;  // 2^+968
  const long long ab = abs_bits(a);
  if (ab == 0) return __dmul_rn(a, y);         // signed zero, exact
  if (!b_safe || ab < lo || ab > hi) return __ddiv_rn(a, b);
  const double q0 = __dmul_rn(a, y);
  const long long qb = abs_bits(q0);
  if (qb < lo || qb > hi) return __ddiv_rn(a, b);
  const double r0 = __fma_rn(-b, q0, a);
  const double q1 = __fma_rn(r0, y, q0);
  const double r1 = __fma_rn(-b, q1, a);
  return __fma_rn(r1, y, q1);
}

// Factor M in place. hold has 2n doubles: the row scales holder_i and their
// reciprocals. Returns 0, LUFQHE_ST_SCALE_TINY or LUFQHE_ST_SINGULAR
// (warp-uniform); *parity receives the swap count mod 2.
//
// Pivot search: the reference compares q_i = RN(|Re a_ij| / holder_i). The
// kernel first ranks a_i = RN(|Re a_ij| * RN(1/holder_i)), whose relative
// distance from q_i is below 3u (u = 2^-53). When the largest a_m beats every
// other a_k by more than 16 ulps, RN(q_m) > RN(q_k) for all k, so m is the
// reference's choice; otherwise (near-ties, zero or extreme quotients) the
// exact quotients are computed and compared with the reference's rule.
//
// perm (optional, n ints of shared memory): perm[j] receives the original row
// of pivoted row j, for callers that keep the factors for later solves.
template <int ARITH>
__device__ int lup_fp64_warp(double2 *M, int lds, double *hold, int n, int lane, int *parity,
                             int *perm = nullptr) {
  int par = 0;
  double *rhold = hold + n;
  if (perm)
    for (int i = lane; i < n; i += 32) perm[i] = i;
  {
    bool tiny = false;
    const long long tiny_bits = __double_as_longlong(1e-24);
    for (int i = lane; i < n; i += 32) {
      long long big = 0;
      for (int k = 0; k < n; ++k) big = max(big, abs_bits(M[i * lds + k].x));
      const double h = __longlong_as_double(big);
      hold[i] = h;
      rhold[i] = __drcp_rn(h);
      tiny |= big < tiny_bits;
    }
    if (__any_sync(kFull, tiny)) {
      *parity = 0;
      return LUFQHE_ST_SCALE_TINY;
    }
    __syncwarp();
  }
  const long long safe_lo = 0x0170000000000000ll;  // 2^-1000
  const long long safe_hi = 0x7e70000000000000ll;  // 2^+1000
  for (int j = 0; j < n; ++j) {
    // screened pivot search: approximate quotients, ties to the larger i
    long long bk = -1;
    int bi = j;
    for (int i = j + lane; i < n; i += 32) {
      double a = __dmul_rn(fabs(M[i * lds + j].x), rhold[i]);
      long long key = (a == a) ? __double_as_longlong(a) : -2ll;
      if (key >= bk) {
        bk = key;
        bi = i;
      }
    }
#pragma unroll
    for (int off = 16; off; off >>= 1) {
      long long ok = __shfl_xor_sync(kFull, bk, off);
      int oi = __shfl_xor_sync(kFull, bi, off);
      if (ok > bk || (ok == bk && oi > bi)) {
        bk = ok;
        bi = oi;
      }
    }
    unsigned near = 0;
    for (int i = j + lane; i < n; i += 32) {
      double a = __dmul_rn(fabs(M[i * lds + j].x), rhold[i]);
      long long key = (a == a) ? __double_as_longlong(a) : -2ll;
      near += key >= bk - 16;
    }
    near = __reduce_add_sync(kFull, near);
    if (near != 1 || bk < safe_lo || bk > safe_hi) {
      // exact path: the reference's comparison on correctly rounded quotients;
      // a NaN quotient is never chosen (key -2 < initial -1)
      bk = -1;
      bi = j;
      for (int i = j + lane; i < n; i += 32) {
        double q = __ddiv_rn(fabs(M[i * lds + j].x), hold[i]);
        long long key = (q == q) ? __double_as_longlong(q) : -2ll;
        if (key >= bk) {
          bk = key;
          bi = i;
        }
      }
#pragma unroll
      for (int off = 16; off; off >>= 1) {
        long long ok = __shfl_xor_sync(kFull, bk, off);
        int oi = __shfl_xor_sync(kFull, bi, off);
        if (ok > bk || (ok == bk && oi > bi)) {
          bk = ok;
          bi = oi;
        }
      }
    }
    const int p = bi;
    if (p != j) {
      for (int k = lane; k < n; k += 32) {
        double2 t = M[p * lds + k];
        M[p * lds + k] = M[j * lds + k];
        M[j * lds + k] = t;
      }
      if (lane == 0) {
        hold[p] = hold[j];
        rhold[p] = rhold[j];
        if (perm) {
          const int t = perm[p];
          perm[p] = perm[j];
          perm[j] = t;
        }
      }
      par ^= 1;
    }
    __syncwarp();
    const double2 piv = M[j * lds + j];
    if (is_zero_c(piv)) {
      *parity = par;
      return LUFQHE_ST_SINGULAR;
    }
    if (j == n - 1) break;
    if (ARITH == ARITH_REF) {
      const double den = pivot_den<ARITH_REF>(piv);
      const double y = __drcp_rn(den);
      const long long db = abs_bits(den);
      const bool den_safe = db >= 0x03f0000000000000ll && db <= 0x7bf0000000000000ll;  // [2^-960, 2^960]
      for (int i = j + 1 + lane; i < n; i += 32) {
        const double2 a = M[i * lds + j];
        const double nx = __dadd_rn(__dmul_rn(a.x, piv.x), __dmul_rn(a.y, piv.y));
        const double ny = __dsub_rn(__dmul_rn(a.y, piv.x), __dmul_rn(a.x, piv.y));
        M[i * lds + j] = make_double2(div_rn_markstein(nx, den, y, den_safe),
                                      div_rn_markstein(ny, den, y, den_safe));
      }
    } else {
      const double d = pivot_den<ARITH>(piv);
      for (int i = j + 1 + lane; i < n; i += 32)
        M[i * lds + j] = cdiv_pivot<ARITH>(M[i * lds + j], piv, d);
    }
    __syncwarp();
    // trailing update a_ik -= l_ij * u_jk on the m x m block
    const int m = n - 1 - j;
    const int mm = m * m;
    const int j1 = j + 1;
    BlockWalk w(lane, m);
    for (int e = lane; e < mm; e += 32) {
      const int ii = j1 + w.i, kk = j1 + w.k;
      M[ii * lds + kk] = cmsub<ARITH>(M[ii * lds + kk], M[ii * lds + j], M[j * lds + kk]);
      w.next(m);
    }
    __syncwarp();
  }
  *parity = par;
  return 0;
}

// Warps of the CTA that factorises one matrix for n >= kFp64GroupMinN.
constexpr int kFp64GroupWarps = 4;
constexpr int kFp64GroupMinN = 33;

// Barrier of the threads that factorise one matrix together: the whole CTA,
// or a named barrier (id 1..15) of `count` threads, a multiple of 32, so that
// several warp groups of one CTA can factorise different matrices.
struct CtaBarrier {
  __device__ __forceinline__ void sync() const { __syncthreads(); }
  __device__ __forceinline__ bool sync_or(bool v) const { return __syncthreads_or(v) != 0; }
};
struct NamedBarrier {
  int id, count;
  __device__ __forceinline__ void sync() const {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
  }
  __device__ __forceinline__ bool sync_or(bool v) const {
    unsigned r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\tsetp.ne.u32 q, %1, 0;\n\t"
        "bar.red.or.pred p, %2, %3, q;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(r)
        : "r"((unsigned)v), "r"(id), "r"(count)
        : "memory");
    return r != 0;
  }
};

// The same factorisation by all threads of a warp group (a CTA, or part of
// one behind a named barrier), for n > 32 where one warp per matrix leaves too
// few warps on an SM to keep the FP64 pipe busy. Every pivot decision is taken
// on the same candidate keys with the same rule (ties to the larger row) and
// every entry sees the same operations in the same order as in lup_fp64_warp,
// so the factors, pivots and parity are bit-identical to it. `red` is
// 3 x (warps) words of shared scratch for the cross-warp reductions; tid and
// nthr number the group's threads. Group-uniform return value.
template <int ARITH, class Bar = CtaBarrier>
__device__ int lup_fp64_group(double2 *M, int lds, double *hold, int n, int tid, int nthr,
                              long long *red, int *parity, Bar bar = Bar(), int *perm = nullptr) {
  const int lane = tid & 31, warp = tid >> 5, nw = nthr >> 5;
  if (perm)
    for (int i = tid; i < n; i += nthr) perm[i] = i;
  long long *red_k = red;
  int *red_i = reinterpret_cast<int *>(red + nw);
  unsigned *red_n = reinterpret_cast<unsigned *>(red_i + nw);
  int par = 0;
  double *rhold = hold + n;
  {
    bool tiny = false;
    const long long tiny_bits = __double_as_longlong(1e-24);
    for (int i = tid; i < n; i += nthr) {
      long long big = 0;
      for (int k = 0; k < n; ++k) big = max(big, abs_bits(M[i * lds + k].x));
      const double h = __longlong_as_double(big);
      hold[i] = h;
      rhold[i] = __drcp_rn(h);
      tiny |= big < tiny_bits;
    }
    if (bar.sync_or(tiny)) {
      *parity = 0;
      return LUFQHE_ST_SCALE_TINY;
    }
  }
  // argmax over the CTA of (key, row), ties to the larger row
  auto argmax = [&](long long &bk, int &bi) {
#pragma unroll
    for (int off = 16; off; off >>= 1) {
      long long ok = __shfl_xor_sync(kFull, bk, off);
      int oi = __shfl_xor_sync(kFull, bi, off);
      if (ok > bk || (ok == bk && oi > bi)) {
        bk = ok;
        bi = oi;
      }
    }
    if (lane == 0) {
      red_k[warp] = bk;
      red_i[warp] = bi;
    }
    bar.sync();
    bk = red_k[0];
    bi = red_i[0];
    for (int q = 1; q < nw; ++q) {
      if (red_k[q] > bk || (red_k[q] == bk && red_i[q] > bi)) {
        bk = red_k[q];
        bi = red_i[q];
      }
    }
    bar.sync();
  };
  const long long safe_lo = 0x0170000000000000ll;  // 2^-1000
  const long long safe_hi = 0x7e70000000000000ll;  // 2^+1000
  for (int j = 0; j < n; ++j) {
    long long bk = -1;
    int bi = j;
    for (int i = j + tid; i < n; i += nthr) {
      double a = __dmul_rn(fabs(M[i * lds + j].x), rhold[i]);
      long long key = (a == a) ? __double_as_longlong(a) : -2ll;
      if (key >= bk) {
        bk = key;
        bi = i;
      }
    }
    argmax(bk, bi);
    unsigned near = 0;
    for (int i = j + tid; i < n; i += nthr) {
      double a = __dmul_rn(fabs(M[i * lds + j].x), rhold[i]);
      long long key = (a == a) ? __double_as_longlong(a) : -2ll;
      near += key >= bk - 16;
    }
    near = __reduce_add_sync(kFull, near);
    if (lane == 0) red_n[warp] = near;
    bar.sync();
    near = 0;
    for (int q = 0; q < nw; ++q) near += red_n[q];
    bar.sync();
    if (near != 1 || bk < safe_lo || bk > safe_hi) {
      bk = -1;
      bi = j;
      for (int i = j + tid; i < n; i += nthr) {
        double q = __ddiv_rn(fabs(M[i * lds + j].x), hold[i]);
        long long key = (q == q) ? __double_as_longlong(q) : -2ll;
        if (key >= bk) {
          bk = key;
          bi = i;
        }
      }
      argmax(bk, bi);
    }
    const int p = bi;
    if (p != j) {
      for (int k = tid; k < n; k += nthr) {
        double2 t = M[p * lds + k];
        M[p * lds + k] = M[j * lds + k];
        M[j * lds + k] = t;
      }
      if (tid == 0) {
        hold[p] = hold[j];
        rhold[p] = rhold[j];
        if (perm) {
          const int t = perm[p];
          perm[p] = perm[j];
          perm[j] = t;
        }
      }
      par ^= 1;
    }
    bar.sync();
    const double2 piv = M[j * lds + j];
    if (is_zero_c(piv)) {
      *parity = par;
      return LUFQHE_ST_SINGULAR;
    }
    if (j == n - 1) break;
    if (ARITH == ARITH_REF) {
      const double den = pivot_den<ARITH_REF>(piv);
      const double y = __drcp_rn(den);
      const long long db = abs_bits(den);
      const bool den_safe = db >= 0x03f0000000000000ll && db <= 0x7bf0000000000000ll;
      for (int i = j + 1 + tid; i < n; i += nthr) {
        const double2 a = M[i * lds + j];
        const double nx = __dadd_rn(__dmul_rn(a.x, piv.x), __dmul_rn(a.y, piv.y));
        const double ny = __dsub_rn(__dmul_rn(a.y, piv.x), __dmul_rn(a.x, piv.y));
        M[i * lds + j] = make_double2(div_rn_markstein(nx, den, y, den_safe),
                                      div_rn_markstein(ny, den, y, den_safe));
      }
    } else {
      const double d = pivot_den<ARITH>(piv);
      for (int i = j + 1 + tid; i < n; i += nthr)
        M[i * lds + j] = cdiv_pivot<ARITH>(M[i * lds + j], piv, d);
    }
    bar.sync();
    const int m = n - 1 - j;
    const int mm = m * m;
    const int j1 = j + 1;
    StrideWalk w(tid, nthr, m);
    for (int e = tid; e < mm; e += nthr) {
      const int ii = j1 + w.i, kk = j1 + w.k;
      M[ii * lds + kk] = cmsub<ARITH>(M[ii * lds + kk], M[ii * lds + j], M[j * lds + kk]);
      w.next(m);
    }
    bar.sync();
  }
  *parity = par;
  return 0;
}

// log|det| and phase from the diagonal of a factored M (all lanes get them).
__device__ __forceinline__ void logdet_from_diag(const double2 *M, int lds, int n, int lane,
                                                 int par, double *la_out, double *ph_out) {
  double la = 0.0, ph = 0.0;
  for (int j = lane; j < n; j += 32) {
    double lg, ar;
    log_arg_c(M[j * lds + j], lg, ar);
    la += lg;
    ph += ar;
  }
#pragma unroll
  for (int off = 16; off; off >>= 1) {
    la += __shfl_xor_sync(kFull, la, off);
    ph += __shfl_xor_sync(kFull, ph, off);
  }
  if (par) ph += kPi;
  *la_out = la;
  *ph_out = wrap_phase(ph);
}

}  // namespace lufqhe
