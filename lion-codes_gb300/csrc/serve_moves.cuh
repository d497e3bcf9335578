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
//   C     the m x m capacitance matrix I + V^T W
//   st    log|det A|, arg det A and m
// so that A = A0 + sum_s e_{i_s} d_s^T and, by Woodbury,
//   A^-1 e_i = c - W C^-1 V^T c,   c = A0^-1 e_i   (two triangular solves).
// Each move is checked before its ratio is used: the residual
// A x - e_i of the solve against the resident current matrix, and the
// cancellation in 1 + d^T x. A move that fails a check, or finds the
// history full (m = K), refactorises A' in FP64 instead and restarts from it.
// The work per accepted move is O(n^2 + n K + K^3), against O(n^3) for a new
// factorisation.
//
// A move is a chain of short dependent steps on one warp, so the code keeps
// that chain short: the matrices are staged into shared memory by
// asynchronous copies issued all at once, the diagonal reciprocals of U are
// taken lane-parallel before the back substitution, the residual is formed
// one row per lane from shared memory (no reductions), and the m dot products
// against the history are reduced side by side.
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
  double2 *W;  // K x n
  double2 *V;  // K x n
  double2 *C;  // K x K, row-major
  MoveState *st;
};

// A move is accepted when max_p |(A x - e_i)_p| <= kMoveResTol ||A||_inf ||x||_inf
// and |1 + d^T x| >= kMoveCancel max(1, |d^T x|).
constexpr double kMoveResTol = 1e-14;
constexpr double kMoveCancel = 1e-2;

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(__fma_rn(a.x, b.x, -__dmul_rn(a.y, b.y)),
                      __fma_rn(a.x, b.y, __dmul_rn(a.y, b.x)));
}
__device__ __forceinline__ double2 csubmul(double2 s, double2 a, double2 b) {  // s - a b
  return cmsub<ARITH_FUSED>(s, a, b);
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
// shared memory): each lane accumulates all m partial sums, then the m warp
// reductions run side by side. out is shared memory, written by lane 0.
template <int K>
__device__ __forceinline__ void warp_dots(const double2 *X, const double2 *b, int n, int m,
                                          int lane, double2 *out) {
  double2 acc[K];
#pragma unroll
  for (int s = 0; s < K; ++s) acc[s] = make_double2(0.0, 0.0);
  for (int p = lane; p < n; p += 32) {
    const double2 bp = b[p];
#pragma unroll
    for (int s = 0; s < K; ++s) {
      if (s < m) {
        const double2 t = cmul(__ldcg(X + (size_t)s * n + p), bp);
        acc[s].x += t.x;
        acc[s].y += t.y;
      }
    }
  }
#pragma unroll
  for (int off = 16; off; off >>= 1)
#pragma unroll
    for (int s = 0; s < K; ++s) {
      acc[s].x += __shfl_xor_sync(kFull, acc[s].x, off);
      acc[s].y += __shfl_xor_sync(kFull, acc[s].y, off);
    }
  if (lane == 0)
#pragma unroll
    for (int s = 0; s < K; ++s)
      if (s < m) out[s] = acc[s];
  __syncwarp();
}

// Shared-memory scratch of one move, after the n x lds factor area.
struct MoveScratch {
  double2 *c, *x, *r;  // n each
  double2 *Cs;         // K x K
  double2 *rhs;        // K
  int *perm;           // n
  static constexpr size_t bytes(int n, int K) {
    return (3 * (size_t)n + (size_t)K * K + K) * sizeof(double2) + (size_t)n * sizeof(int);
  }
  __device__ void bind(unsigned char *p, int n, int K) {
    c = reinterpret_cast<double2 *>(p);
    x = c + n;
    r = x + n;
    Cs = r + n;
    rhs = Cs + K * K;
    perm = reinterpret_cast<int *>(rhs + K);
  }
};

// Try the move of row i to the new row r' (in S.r) for one matrix, one warp.
// Ls (row stride lds) receives the factors, then the current matrix. True
// (warp-uniform) if the move was accepted: the state, W, V, C and row i of A
// are updated and (*la, *ph) is the new log-determinant. False: only row i of
// A has been rewritten; the caller refactorises A.
template <int K>
__device__ bool move_warp(const MoveArrays &a, int n, int i, double2 *Ls, int lds,
                          const MoveScratch &S, int lane, double *la_out, double *ph_out) {
  const MoveState st = *a.st;
  const int m = st.m;
  bool ok = m < K && st.la == st.la;
  // 1. the factors of A0 into shared memory (rows in pivoted order)
  for (int p = lane; p < n; p += 32) S.perm[p] = __ldcg(a.perm + p);
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
    //    reciprocals of U's diagonal first, lane-parallel, into S.x (free
    //    until step 3), so each backward step is a multiply
    for (int p = lane; p < n; p += 32) {
      S.c[p] = make_double2(p == q ? 1.0 : 0.0, 0.0);
      S.x[p] = crcp(Ls[p * lds + p]);
    }
    __syncwarp();
    for (int j = q; j + 1 < n; ++j) {
      const double2 yj = S.c[j];
      for (int p = j + 1 + lane; p < n; p += 32) S.c[p] = csubmul(S.c[p], Ls[p * lds + j], yj);
      __syncwarp();
    }
    for (int j = n - 1; j >= 0; --j) {
      const double2 cj = cmul(S.c[j], S.x[j]);
      __syncwarp();
      if (lane == 0) S.c[j] = cj;
      for (int p = lane; p < j; p += 32) S.c[p] = csubmul(S.c[p], Ls[p * lds + j], cj);
      __syncwarp();
    }
    // 3. x = c - W C^-1 V^T c (the m dot products reduced together)
    warp_dots<K>(a.V, S.c, n, m, lane, S.rhs);
    for (int e = lane; e < m * m; e += 32) S.Cs[e] = __ldcg(a.C + (e / m) * K + (e % m));
    __syncwarp();
    if (lane == 0 && m > 0) {
      // C z = V^T c by Gaussian elimination with partial pivoting (m <= K);
      // each pivot is kept as its reciprocal
      double2 *Cm = S.Cs;
      double2 *z = S.rhs;
      for (int j = 0; j < m; ++j) {
        int p = j;
        for (int r = j + 1; r < m; ++r)
          if (cabs1(Cm[r * m + j]) > cabs1(Cm[p * m + j])) p = r;
        if (p != j) {
          for (int k = 0; k < m; ++k) {
            const double2 t = Cm[p * m + k];
            Cm[p * m + k] = Cm[j * m + k];
            Cm[j * m + k] = t;
          }
          const double2 t = z[p];
          z[p] = z[j];
          z[j] = t;
        }
        const double2 rj = crcp(Cm[j * m + j]);
        Cm[j * m + j] = rj;
        for (int r = j + 1; r < m; ++r) {
          const double2 l = cmul(Cm[r * m + j], rj);
          for (int k = j + 1; k < m; ++k) Cm[r * m + k] = csubmul(Cm[r * m + k], l, Cm[j * m + k]);
          z[r] = csubmul(z[r], l, z[j]);
        }
      }
      for (int j = m - 1; j >= 0; --j) {
        double2 t = z[j];
        for (int k = j + 1; k < m; ++k) t = csubmul(t, Cm[j * m + k], z[k]);
        z[j] = cmul(t, Cm[j * m + j]);
      }
    }
    __syncwarp();
    for (int p = lane; p < n; p += 32) {
      double2 t = S.c[p];
      for (int s = 0; s < m; ++s) t = csubmul(t, __ldcg(a.W + (size_t)s * n + p), S.rhs[s]);
      S.x[p] = t;
    }
    // 4. a-posteriori check of x against the current matrix: the residual
    //    A x - e_i, relative to ||A||_inf ||x||_inf. The factors are done
    //    with: A takes their place in shared memory, and each lane forms whole
    //    rows (no reductions).
    __syncwarp();
    stage_matrix_async(Ls, lds, a.A, n, lane);
    double res = 0.0, anorm = 0.0, xnorm = 0.0;
    for (int p = lane; p < n; p += 32) {
      xnorm = fmax(xnorm, cabs1(S.x[p]));
      double2 s = make_double2(p == i ? -1.0 : 0.0, 0.0);
      double rs = 0.0;
      for (int k = 0; k < n; ++k) {
        const double2 v = Ls[p * lds + k];
        const double2 t = cmul(v, S.x[k]);
        s.x += t.x;
        s.y += t.y;
        rs += cabs1(v);
      }
      res = fmax(res, cabs1(s));
      anorm = fmax(anorm, rs);
    }
    res = warp_max(res);
    anorm = warp_max(anorm);
    xnorm = warp_max(xnorm);
    // 5. d = r' - r_i, the ratio 1 + d^T x and its cancellation; d replaces x
    //    in shared memory (each lane its own entries)
    double2 dx = make_double2(0.0, 0.0);
    for (int k = lane; k < n; k += 32) {
      const double2 ri = Ls[i * lds + k];
      const double2 d = make_double2(__dsub_rn(S.r[k].x, ri.x), __dsub_rn(S.r[k].y, ri.y));
      const double2 t = cmul(d, S.x[k]);
      dx.x += t.x;
      dx.y += t.y;
      S.x[k] = d;
    }
    dx = warp_sum2(dx);
    __syncwarp();
    const double2 ratio = make_double2(1.0 + dx.x, dx.y);
    const double rmag = fmax(fabs(ratio.x), fabs(ratio.y));
    ok = (res <= kMoveResTol * anorm * xnorm) && finite_d(res) &&
         rmag >= kMoveCancel * fmax(1.0, cabs1(dx)) && finite_c(ratio);
    ok = __shfl_sync(kFull, ok, 0);
    if (ok) {
      // 6. accept: the log-determinant, then the history (W[m] = c, V[m] = d,
      //    the new row and column of C), then row i of A
      double lg, ar;
      log_arg_c(ratio, lg, ar);
      const double la = st.la + lg, ph = st.ph + ar;
      for (int k = lane; k < n; k += 32) {
        a.W[(size_t)m * n + k] = S.c[k];
        a.V[(size_t)m * n + k] = S.x[k];
      }
      // C[m][s] = d^T W[s] and C[s][m] = V[s]^T c for s < m; C[m][m] = 1 + d^T c
      // (the m x 2 dot products reduced together; S.rhs and S.Cs are free)
      warp_dots<K>(a.W, S.x, n, m, lane, S.rhs);
      warp_dots<K>(a.V, S.c, n, m, lane, S.Cs);
      for (int s = lane; s < m; s += 32) {
        a.C[m * K + s] = S.rhs[s];
        a.C[s * K + m] = S.Cs[s];
      }
      double2 dd = make_double2(0.0, 0.0);
      for (int k = lane; k < n; k += 32) {
        const double2 t = cmul(S.x[k], S.c[k]);
        dd.x += t.x;
        dd.y += t.y;
      }
      dd = warp_sum2(dd);
      if (lane == 0) {
        a.C[m * K + m] = make_double2(1.0 + dd.x, dd.y);
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
