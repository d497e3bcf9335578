// O(n^2) single-particle moves for the serving loop.
//
// A Monte Carlo move resamples one particle i: row i of each of the walker's
// matrices is replaced, A' = A + e_i d^T with d = r' - r (r' the new row).
// The matrix determinant lemma gives det A' = det A (1 + d^T A^-1 e_i), so a
// move needs one solve with A, not a new factorisation. The reference's loop
// refactorises every matrix every step (LU-fqhe/src/MonteCarloLoop.cu:216-335).
//
// Per matrix the walker keeps, in its HBM block:
//   A     the current matrix (row-major n x n)
//   LU    the FP64 L\U factors of A0, the matrix at the last refactorisation
//         (pivoted rows), and perm[j], the row of A0 in pivoted row j
//   W, V  for the m moves since then: W[s] = A0^-1 e_{i_s}, V[s] = d_s
//   Ci    the inverse of the m x m capacitance matrix C = I + V^T W
//   st    log|det A|, arg det A and m
// so that A = A0 + sum_s e_{i_s} d_s^T and, by Woodbury,
//   A^-1 e_i = c - W Ci V^T c,   c = A0^-1 e_i   (two triangular solves).
// Accepting a move borders C with the column V^T c, the row d^T W and the
// corner 1 + d^T c; the Schur complement of that border is 1 + d^T x, the
// determinant ratio itself, so Ci grows by a rank-one update and a border
// (O(m^2), lane-parallel) instead of being refactorised.
// Each move is checked before its ratio is used. With y = A^-T d (a
// transposed solve against the same factors and history) and s = A x - e_i
// the residual of the solve against the resident current matrix, the ratio's
// first-order error is y^T s, so the ratio is taken as 1 + d^T x - y^T s and
// its error estimated as |y^T s| + 3 u (sum_p |y_p|^2 (|A| |x|)_p^2)^(1/2),
// the second term the typical size of y^T times the rounding of s itself (a
// worst-case bound, u sum_p |y_p| (|A| |x|)_p n, exceeds the errors actually
// made by two to three orders of magnitude on these matrices and refuses
// nearly every move at n >= 32). A move whose estimate exceeds the tolerance
// times |ratio|, or that finds the history full (m = K), refactorises A' in
// FP64 instead and restarts from it. (A residual test alone does not suffice:
// on ill-conditioned orbital matrices a solve with a residual at rounding
// level can still carry a forward error of 1e-5 in the direction of d.)
// The work per accepted move is O(n^2 + n K + K^2), against O(n^3) for a new
// factorisation.
//
// On this GPU a warp's FP64 instruction costs the FP64 pipe the same time
// whether one lane or 32 are active, so the code counts FP64 instructions,
// not flops: the matrices are staged into shared memory by asynchronous
// copies issued all at once, the diagonal reciprocals of U are taken
// lane-parallel before the back substitution, the residual is formed one row
// per lane from shared memory (no reductions), the K dot products against the
// history run in K lane groups at once, and nothing runs on one lane alone.
#pragma once

#include "lup_fp64.cuh"

namespace lufqhe {

struct MoveState {
  double la, ph;  // log|det A|, arg det A (unwrapped)
  int m;          // moves since the last refactorisation
  int pad;
};

// One matrix's arrays (device memory).
struct MoveArrays {
  double2 *A;
  double2 *LU;
  int *perm;
  double2 *W;   // K x n
  double2 *V;   // K x n
  double2 *Ci;  // K x K, row-major: the inverse capacitance matrix
  MoveState *st;
};

// the typical rounding of a residual formed in FP64, per unit of |A| |x|
// (three standard deviations of u)
constexpr double kMoveNoise = 3.0 * 1.1102230246251565e-16;

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(__fma_rn(a.x, b.x, -__dmul_rn(a.y, b.y)),
                      __fma_rn(a.x, b.y, __dmul_rn(a.y, b.x)));
}
__device__ __forceinline__ double2 csubmul(double2 s, double2 a, double2 b) {  // s - a b
  return cmsub<ARITH_FUSED>(s, a, b);
}
__device__ __forceinline__ void cmac(double2 &s, double2 a, double2 b) {  // s += a b
  s.x = __fma_rn(a.x, b.x, s.x);
  s.x = __fma_rn(-a.y, b.y, s.x);
  s.y = __fma_rn(a.x, b.y, s.y);
  s.y = __fma_rn(a.y, b.x, s.y);
}
__device__ __forceinline__ double cabs1(double2 a) { return fabs(a.x) + fabs(a.y); }
// 1 / b to within a few ulps (one reciprocal), for the solves, whose result is
// checked by its residual
__device__ __forceinline__ double2 crcp(double2 b) {
  const double r = __drcp_rn(__fma_rn(b.x, b.x, __dmul_rn(b.y, b.y)));
  return make_double2(__dmul_rn(b.x, r), -__dmul_rn(b.y, r));
}

__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int off = 16; off; off >>= 1) v = fmax(v, __shfl_xor_sync(kFull, v, off));
  return v;
}
__device__ __forceinline__ double2 warp_sum2(double2 v) {
#pragma unroll
  for (int off = 16; off; off >>= 1) {
    v.x += __shfl_xor_sync(kFull, v.x, off);
    v.y += __shfl_xor_sync(kFull, v.y, off);
  }
  return v;
}

// An n x n complex128 matrix (row-major, contiguous) from global memory into
// shared memory (row stride lds) by asynchronous 16-byte copies: every lane
// issues all of its copies before waiting once, so the loads overlap instead
// of one round trip each.
__device__ __forceinline__ void stage_matrix_async(double2 *dst, int lds, const double2 *src, int n,
                                                   int lane) {
  BlockWalk w(lane, n);
  for (int e = lane; e < n * n; e += 32) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst + w.i * lds + w.k);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src + e) : "memory");
    w.next(n);
  }
  asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
  __syncwarp();
}

// The same staging followed by a scan for NaN/Inf entries (warp-uniform
// result: true if there is one).
__device__ __forceinline__ bool stage_matrix_checked(double2 *dst, int lds, const double2 *src,
                                                     int n, int lane) {
  stage_matrix_async(dst, lds, src, n, lane);
  bool bad = false;
  BlockWalk w(lane, n);
  for (int e = lane; e < n * n; e += 32) {
    bad |= !finite_c(dst[w.i * lds + w.k]);
    w.next(n);
  }
  return __any_sync(kFull, bad);
}

// out[s] = sum_p X[s n + p] b[p] for s < m (m <= K; X in global memory, b in
// shared memory): the warp splits into K groups of 32 / K lanes, group s
// forms dot s over a stride of p, and the groups reduce side by side. out is
// shared memory.
template <int K>
__device__ __forceinline__ void group_dots(const double2 *X, const double2 *b, int n, int m,
                                           int lane, double2 *out) {
  static_assert(32 % K == 0, "K divides the warp");
  constexpr int G = 32 / K;
  const int s = lane / G, r = lane % G;
  double2 acc = make_double2(0.0, 0.0);
  if (s < m)
    for (int p = r; p < n; p += G) cmac(acc, __ldcg(X + (size_t)s * n + p), b[p]);
#pragma unroll
  for (int off = G / 2; off; off >>= 1) {
    acc.x += __shfl_xor_sync(kFull, acc.x, off);
    acc.y += __shfl_xor_sync(kFull, acc.y, off);
  }
  if (r == 0 && s < m) out[s] = acc;
  __syncwarp();
}

// Shared-memory scratch of one move, after the n x lds factor area.
struct MoveScratch {
  double2 *c, *x, *r, *d, *y, *rd;  // n each
  double2 *b, *z, *g, *h;           // K each: V^T c, Ci b, W^T d, Ci^T g
  int *perm;                        // n
  static constexpr size_t bytes(int n, int K) {
    return (6 * (size_t)n + 4 * (size_t)K) * sizeof(double2) + (size_t)n * sizeof(int);
  }
  __device__ void bind(unsigned char *p, int n, int K) {
    c = reinterpret_cast<double2 *>(p);
    x = c + n;
    r = x + n;
    d = r + n;
    y = d + n;
    rd = y + n;
    b = rd + n;
    z = b + K;
    g = z + K;
    h = g + K;
    perm = reinterpret_cast<int *>(h + K);
  }
};

// Try the move of row i to the new row r' (in S.r) for one matrix, one warp.
// Ls (row stride lds) receives the factors, then the current matrix. True
// (warp-uniform) if the move was accepted: the state, W, V, Ci and row i of A
// are updated and (*la, *ph) is the new log-determinant. False: only row i of
// A has been rewritten; the caller refactorises A.
template <int K>
__device__ bool move_warp(const MoveArrays &a, int n, int i, double2 *Ls, int lds,
                          const MoveScratch &S, int lane, double tol, double *la_out,
                          double *ph_out) {
  const MoveState st = *a.st;
  const int m = st.m;
  bool ok = m < K && st.la == st.la;
  // 1. the factors of A0 into shared memory (rows in pivoted order); d = r' -
  //    r_i from the current row i in global memory meanwhile
  for (int p = lane; p < n; p += 32) S.perm[p] = __ldcg(a.perm + p);
  for (int k = lane; k < n; k += 32) {
    const double2 ri = __ldcg(a.A + (size_t)i * n + k);
    S.d[k] = make_double2(__dsub_rn(S.r[k].x, ri.x), __dsub_rn(S.r[k].y, ri.y));
  }
  stage_matrix_async(Ls, lds, a.LU, n, lane);
  // q: the pivoted position of row i
  int q = n;
  for (int p = lane; p < n; p += 32)
    if (S.perm[p] == i) q = p;
#pragma unroll
  for (int off = 16; off; off >>= 1) q = min(q, __shfl_xor_sync(kFull, q, off));
  ok = ok && q < n;
  if (ok) {
    // 2. c = U^-1 L^-1 e_q: forward from q (unit lower), then backward; the
    //    reciprocals of U's diagonal first, lane-parallel
    for (int p = lane; p < n; p += 32) {
      S.c[p] = make_double2(p == q ? 1.0 : 0.0, 0.0);
      S.rd[p] = crcp(Ls[p * lds + p]);
    }
    __syncwarp();
    for (int j = q; j + 1 < n; ++j) {
      const double2 yj = S.c[j];
      for (int p = j + 1 + lane; p < n; p += 32) S.c[p] = csubmul(S.c[p], Ls[p * lds + j], yj);
      __syncwarp();
    }
    for (int j = n - 1; j >= 0; --j) {
      const double2 cj = cmul(S.c[j], S.rd[j]);
      __syncwarp();
      if (lane == 0) S.c[j] = cj;
      for (int p = lane; p < j; p += 32) S.c[p] = csubmul(S.c[p], Ls[p * lds + j], cj);
      __syncwarp();
    }
    // 3. x = c - W z, z = Ci V^T c (lane s forms z_s); g = W^T d, h = Ci^T g
    group_dots<K>(a.V, S.c, n, m, lane, S.b);
    group_dots<K>(a.W, S.d, n, m, lane, S.g);
    if (lane < m) {
      double2 t = make_double2(0.0, 0.0), u2 = make_double2(0.0, 0.0);
      for (int u = 0; u < m; ++u) {
        cmac(t, __ldcg(a.Ci + lane * K + u), S.b[u]);
        cmac(u2, S.g[u], __ldcg(a.Ci + u * K + lane));
      }
      S.z[lane] = t;
      S.h[lane] = u2;
    }
    __syncwarp();
    // x, and d' = d - V h (into S.y) for the transposed solve
    for (int p = lane; p < n; p += 32) {
      double2 t = S.c[p], e = S.d[p];
      for (int u = 0; u < m; ++u) {
        t = csubmul(t, __ldcg(a.W + (size_t)u * n + p), S.z[u]);
        e = csubmul(e, __ldcg(a.V + (size_t)u * n + p), S.h[u]);
      }
      S.x[p] = t;
      S.y[p] = e;
    }
    __syncwarp();
    // 4. y = A^-T d = P^T L^-T U^-T d': with A0 = P^T L U, forward through
    //    U^T (rows of U as axpys), then backward through L^T (rows of L)
    for (int j = 0; j < n; ++j) {
      const double2 tj = cmul(S.y[j], S.rd[j]);
      __syncwarp();
      if (lane == 0) S.y[j] = tj;
      for (int p = j + 1 + lane; p < n; p += 32) S.y[p] = csubmul(S.y[p], Ls[j * lds + p], tj);
      __syncwarp();
    }
    for (int j = n - 1; j > 0; --j) {
      const double2 wj = S.y[j];
      for (int p = lane; p < j; p += 32) S.y[p] = csubmul(S.y[p], Ls[j * lds + p], wj);
      __syncwarp();
    }
    // y_perm[j] = w_j, in place through registers (n <= 64); |x_k| into S.rd
    // (the reciprocals are done with) for the residual's bound
    double2 wv[2];
    int wp[2];
#pragma unroll
    for (int t = 0; t < 2; ++t) {
      const int j = lane + 32 * t;
      wv[t] = j < n ? S.y[j] : make_double2(0.0, 0.0);
      wp[t] = j < n ? S.perm[j] : 0;
    }
    __syncwarp();
#pragma unroll
    for (int t = 0; t < 2; ++t)
      if (lane + 32 * t < n) S.y[wp[t]] = wv[t];
    for (int k = lane; k < n; k += 32) S.rd[k].x = cabs1(S.x[k]);
    // 5. the current matrix replaces the factors; residual s = A x - e_i and
    //    q = |A| |x|, one row per lane; the ratio's first-order error y^T s
    //    and the size of y^T times the rounding of s, (sum |y_p|^2 q_p^2)^(1/2)
    __syncwarp();
    stage_matrix_async(Ls, lds, a.A, n, lane);
    double noise2 = 0.0;
    double2 yts = make_double2(0.0, 0.0), dx = make_double2(0.0, 0.0);
    for (int p = lane; p < n; p += 32) {
      double2 sres = make_double2(p == i ? -1.0 : 0.0, 0.0);
      double qa = 0.0;
      for (int k = 0; k < n; ++k) {
        const double2 v = Ls[p * lds + k];
        const double2 xk = S.x[k];
        cmac(sres, v, xk);
        qa = __fma_rn(cabs1(v), S.rd[k].x, qa);
      }
      const double2 yp = S.y[p];
      const double yq = __dmul_rn(cabs1(yp), qa);
      noise2 = __fma_rn(yq, yq, noise2);
      cmac(yts, yp, sres);
      cmac(dx, S.d[p], S.x[p]);
    }
    noise2 = warp_sum2(make_double2(noise2, 0.0)).x;
    yts = warp_sum2(yts);
    dx = warp_sum2(dx);
    // 6. the ratio, first-order corrected; taken if within the bound
    const double2 sigma = make_double2(1.0 + dx.x, dx.y);  // the Schur complement
    const double2 ratio = make_double2(sigma.x - yts.x, sigma.y - yts.y);
    const double rmag = fmax(fabs(ratio.x), fabs(ratio.y));
    const double est = __fma_rn(kMoveNoise, sqrt(noise2), cabs1(yts));
    ok = finite_d(est) && finite_c(ratio) && est <= tol * rmag && rmag > 0.0;
    ok = __shfl_sync(kFull, ok, 0);
    if (ok) {
      // 7. accept: the log-determinant; the history (W[m] = c, V[m] = d);
      //    Ci bordered by the Schur complement sigma = 1 + d^T x: with
      //    s = 1 / sigma, Ci += z s h^T, column m = -z s, row m = -s h^T,
      //    corner s
      double lg, ar;
      log_arg_c(ratio, lg, ar);
      const double la = st.la + lg, ph = st.ph + ar;
      for (int k = lane; k < n; k += 32) {
        a.W[(size_t)m * n + k] = S.c[k];
        a.V[(size_t)m * n + k] = S.d[k];
      }
      const double2 sr = crcp(sigma);
      const int m1 = m + 1;
      for (int e = lane; e < m1 * m1; e += 32) {
        const int u = e / m1, v = e - u * m1;
        double2 val;
        if (u < m && v < m)
          val = csubmul(__ldcg(a.Ci + u * K + v), cmul(S.z[u], sr), make_double2(-S.h[v].x, -S.h[v].y));
        else if (u < m)
          val = cmul(S.z[u], make_double2(-sr.x, -sr.y));
        else if (v < m)
          val = cmul(make_double2(-sr.x, -sr.y), S.h[v]);
        else
          val = sr;
        a.Ci[u * K + v] = val;
      }
      if (lane == 0) {
        MoveState ns;
        ns.la = la;
        ns.ph = ph;
        ns.m = m + 1;
        ns.pad = 0;
        *a.st = ns;
      }
      *la_out = la;
      *ph_out = ph;
    }
  }
  ok = __shfl_sync(kFull, ok, 0);
  // row i of A becomes the new row either way
  __syncwarp();
  for (int k = lane; k < n; k += 32) a.A[(size_t)i * n + k] = S.r[k];
  __syncwarp();
  return ok;
}

}  // namespace lufqhe
