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

// Coalesced load of an n x n complex128 matrix (row stride lda) into shared
// memory (row stride lds). Returns true (warp-uniform) if any entry is NaN/Inf.
__device__ __forceinline__ bool load_matrix_fp64(const double2 *__restrict__ src, int n, int lda,
                                                 double2 *M, int lds, int lane) {
  bool bad = false;
  const int nn = n * n;
  BlockWalk w(lane, n);
  for (int e = lane; e < nn; e += 32) {
    double2 v = __ldg(src + (size_t)w.i * lda + w.k);
    bad |= !finite_c(v);
    M[w.i * lds + w.k] = v;
    w.next(n);
  }
  bad = __any_sync(kFull, bad);
  __syncwarp();
  return bad;
}

// Factor M in place. Returns 0, LUFQHE_ST_SCALE_TINY or LUFQHE_ST_SINGULAR
// (warp-uniform); *parity receives the swap count mod 2.
template <int ARITH>
__device__ int lup_fp64_warp(double2 *M, int lds, double *hold, int n, int lane, int *parity) {
  int par = 0;
  {
    bool tiny = false;
    const long long tiny_bits = __double_as_longlong(1e-24);
    for (int i = lane; i < n; i += 32) {
      long long big = 0;
      for (int k = 0; k < n; ++k) big = max(big, abs_bits(M[i * lds + k].x));
      hold[i] = __longlong_as_double(big);
      tiny |= big < tiny_bits;
    }
    if (__any_sync(kFull, tiny)) {
      *parity = 0;
      return LUFQHE_ST_SCALE_TINY;
    }
    __syncwarp();
  }
  for (int j = 0; j < n; ++j) {
    // pivot: max of |Re a_ij| / holder_i over i >= j, ties to the larger i;
    // a NaN quotient is never chosen (key -2 < initial -1).
    long long bk = -1;
    int bi = j;
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
    const int p = bi;
    if (p != j) {
      for (int k = lane; k < n; k += 32) {
        double2 t = M[p * lds + k];
        M[p * lds + k] = M[j * lds + k];
        M[j * lds + k] = t;
      }
      if (lane == 0) hold[p] = hold[j];
      par ^= 1;
    }
    __syncwarp();
    const double2 piv = M[j * lds + j];
    if (is_zero_c(piv)) {
      *parity = par;
      return LUFQHE_ST_SINGULAR;
    }
    if (j == n - 1) break;
    const double d = pivot_den<ARITH>(piv);
    for (int i = j + 1 + lane; i < n; i += 32)
      M[i * lds + j] = cdiv_pivot<ARITH>(M[i * lds + j], piv, d);
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

// log|det| and phase from the diagonal of a factored M (all lanes get them).
__device__ __forceinline__ void logdet_from_diag(const double2 *M, int lds, int n, int lane,
                                                 int par, double *la_out, double *ph_out) {
  double la = 0.0, ph = 0.0;
  for (int j = lane; j < n; j += 32) {
    double2 u = M[j * lds + j];
    la += log(hypot(u.x, u.y));
    ph += atan2(u.y, u.x);
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
