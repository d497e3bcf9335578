// Composite-fermion (CF) matrices built in the kernels from one configuration's
// particle angles and a batch of permutations: the on-device matrix builder
// that the reference sketches and compiles out (LU-fqhe/src/mkMatrixElements.cu
// :26-363, under #if 0), restated in FP64.
//
// A configuration has np particles with
//   u_p = (cos theta_p cos phi_p, cos theta_p sin phi_p),
//   v_p = (sin theta_p cos phi_p, -sin theta_p sin phi_p)       (:91-101)
// and a table T of np x n orbital values, Q = (n - 3) / 2 (n odd, 2Q + 3 = n):
//   T[p][Q+1]   = (cos theta_p sin theta_p)^Q,
//   T[p][Q+1+j] = T[p][Q+j] * (u_p / v_p),  T[p][Q+1-j] = T[p][Q+2-j] * (v_p / u_p),
// j = 1..Q+1 (setupM_Matrix, :169-194). Matrix b takes the n particles its
// permutation lists (1-based, row stride perm_stride; the reference's
// devPermutations, :301); row r with particle p = perm[r] - 1 is
//   columns c < n - 2:  T[p][c]
//   column n - 2:       T[p][Q+1+mu] * sum_{s != r} (k1 u_p v_q + k2 u_q v_p) / (u_p v_q - u_q v_p)
//   column n - 1:       T[p][Q+1+nu] * sum_{s != r} (r1 u_p v_q + r2 u_q v_p) / (u_p v_q - u_q v_p)
// with q = perm[s] - 1, the sum taken over s < r, then s > r (calculateElement,
// :196-293). The reference returns the sum of both terms in both last columns:
// the column masks that would keep one term each are commented out (:251,
// :285), and without them the two columns are equal and every matrix singular.
// Here each column takes its own term, as the masks intend.
//
// The table and u, v are computed once per configuration on the host (cf.cu)
// and read by every row. The sums are formed on the device, in a pre-pass of
// one thread per row, with every operation explicitly rounded, so a host
// restatement of the same operation order reproduces their bits. A
// permutation entry outside 1..np gives a NaN row (status NONFINITE), never a
// read out of range; a repeated particle gives 0 * inf in its sums, also NaN.
#pragma once

#include "lup_fp64.cuh"

namespace lufqhe {

__device__ __forceinline__ double2 cd_mul(double2 a, double2 b) {
  return make_double2(__dsub_rn(__dmul_rn(a.x, b.x), __dmul_rn(a.y, b.y)),
                      __dadd_rn(__dmul_rn(a.x, b.y), __dmul_rn(a.y, b.x)));
}

// The parameters of a configuration's last two columns.
struct CfParams {
  const double2 *tab;  // np x n
  const double2 *uv;   // u[0..np), then v[0..np)
  const short *perm;   // batch x pstride, 1-based
  int pstride;
  int np;
  int cmu, cnu;        // table columns Q+1+mu, Q+1+nu
  double k1, k2, r1, r2;

  __device__ __forceinline__ int particle(long long b, int r) const {
    const int p = (int)__ldg(perm + (size_t)b * pstride + r) - 1;
    return (p >= 0 && p < np) ? p : -1;
  }
  // Entries (r, n-2) and (r, n-1) of matrix b. Per pair (p, q):
  //   a = u_p v_q, c = u_q v_p, d = a - c, w = RN(1 / |d|^2),
  //   S1 += ((k1 a + k2 c) conj d) w,  S2 += ((r1 a + r2 c) conj d) w,
  // one reciprocal for both sums (the reference's (k1 u_p) v_q + (k2 u_q) v_p
  // over u_p v_q - u_q v_p, equal up to rounding).
  __device__ void last_columns(long long b, int n, int r, double2 &e1, double2 &e2) const {
    const int p = particle(b, r);
    e1 = e2 = make_double2(NAN, NAN);
    if (p < 0) return;
    const double2 ui = __ldg(uv + p), vi = __ldg(uv + np + p);
    double2 s1 = make_double2(0.0, 0.0), s2 = make_double2(0.0, 0.0);
    for (int s = 0; s < n; ++s) {
      if (s == r) continue;
      const int q = particle(b, s);
      if (q < 0) return;
      const double2 a = cd_mul(ui, __ldg(uv + np + q));
      const double2 c = cd_mul(__ldg(uv + q), vi);
      const double dx = __dsub_rn(a.x, c.x), dy = __dsub_rn(a.y, c.y);
      const double w = __drcp_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
      const double n1x = __dadd_rn(__dmul_rn(k1, a.x), __dmul_rn(k2, c.x));
      const double n1y = __dadd_rn(__dmul_rn(k1, a.y), __dmul_rn(k2, c.y));
      const double n2x = __dadd_rn(__dmul_rn(r1, a.x), __dmul_rn(r2, c.x));
      const double n2y = __dadd_rn(__dmul_rn(r1, a.y), __dmul_rn(r2, c.y));
      s1.x = __dadd_rn(s1.x, __dmul_rn(__dadd_rn(__dmul_rn(n1x, dx), __dmul_rn(n1y, dy)), w));
      s1.y = __dadd_rn(s1.y, __dmul_rn(__dsub_rn(__dmul_rn(n1y, dx), __dmul_rn(n1x, dy)), w));
      s2.x = __dadd_rn(s2.x, __dmul_rn(__dadd_rn(__dmul_rn(n2x, dx), __dmul_rn(n2y, dy)), w));
      s2.y = __dadd_rn(s2.y, __dmul_rn(__dsub_rn(__dmul_rn(n2y, dx), __dmul_rn(n2x, dy)), w));
    }
    e1 = cd_mul(s1, __ldg(tab + (size_t)p * n + cmu));
    e2 = cd_mul(s2, __ldg(tab + (size_t)p * n + cnu));
  }
};

// The matrices as the factorising kernels read them: columns c < n - 2 from
// the table, the last two from cols (2 per row, row-major over the batch),
// which a pre-pass fills with every lane busy (built per row inside the
// factorisation, one lane per row did all of a row's O(n) divisions while the
// rest of the warp waited, and the correction's re-reads repeated them).
struct CfSource {
  static constexpr bool kOddN = true;  // n = 2Q + 3: no even-n tile kernels
  const double2 *tab;   // np x n
  const short *perm;    // batch x pstride, 1-based
  const double2 *cols;  // batch x n x 2
  int pstride;
  int np;

  __device__ __forceinline__ int particle(long long b, int r) const {
    const int p = (int)__ldg(perm + (size_t)b * pstride + r) - 1;
    return (p >= 0 && p < np) ? p : -1;
  }
  // entry (r, c) of matrix b
  __device__ __forceinline__ double2 entry(long long b, int n, int r, int c) const {
    if (c >= n - 2) return __ldg(cols + ((size_t)b * n + r) * 2 + (c - (n - 2)));
    const int p = particle(b, r);
    return p < 0 ? make_double2(NAN, NAN) : __ldg(tab + (size_t)p * n + c);
  }
  // row r of matrix b into out[0..n) (any element type store_entry takes);
  // false if an entry is NaN or infinite
  template <class T>
  __device__ bool row(long long b, int n, int r, T *out) const {
    const int p = particle(b, r);
    const double2 *t = tab + (size_t)(p < 0 ? 0 : p) * n;
    bool ok = p >= 0;
    for (int c = 0; c < n - 2; ++c) {
      const double2 v = p < 0 ? make_double2(NAN, NAN) : __ldg(t + c);
      ok &= finite_c(v);
      store_entry(out + c, v);
    }
    const double2 *e = cols + ((size_t)b * n + r) * 2;
    for (int c = 0; c < 2; ++c) {
      const double2 v = __ldg(e + c);
      ok &= finite_c(v);
      store_entry(out + n - 2 + c, v);
    }
    return ok;
  }
  template <bool COHERENT = false>
  __device__ __forceinline__ bool load(long long b, int n, double2 *M, int lds, int lane) const {
    bool bad = false;
    for (int r = lane; r < n; r += 32) bad |= !row(b, n, r, M + r * lds);
    bad = __any_sync(kFull, bad);
    __syncwarp();
    return bad;
  }
  __device__ __forceinline__ double2 first(long long b, int n) const { return entry(b, n, 0, 0); }
  __device__ __forceinline__ bool load_group(long long b, int n, double2 *M, int lds, int tid,
                                             int nthr) const {
    bool bad = false;
    for (int r = tid; r < n; r += nthr) bad |= !row(b, n, r, M + r * lds);
    return __syncthreads_or(bad);
  }
};

// Rows for the extended-precision correction (fp64_correct.cuh), which
// re-reads the matrix it corrects.
struct CfRow {
  const double2 *t;  // the particle's table row (nullptr: a NaN row)
  const double2 *e;  // its two last-column entries
  int n, c;
  __device__ __forceinline__ double2 next() {
    const int k = c++;
    if (k >= n - 2) return __ldg(e + (k - (n - 2)));
    return t ? __ldg(t + k) : make_double2(NAN, NAN);
  }
  __device__ __forceinline__ void skip(int j) { c += j; }
};
__device__ __forceinline__ CfRow source_row(const CfSource &s, long long b, int n, int r) {
  const int p = s.particle(b, r);
  return CfRow{p < 0 ? nullptr : s.tab + (size_t)p * n, s.cols + ((size_t)b * n + r) * 2, n, 0};
}
__device__ __forceinline__ double2 source_entry(const CfSource &s, long long b, int n, int r,
                                                int c) {
  return s.entry(b, n, r, c);
}

// Host: u, v (2 np) and the table (np x n) of a configuration.
void cf_tables(const double *phi, const double *theta, int np, int n, double2 *uv, double2 *tab);

int launch_plain_cf(const CfSource &src, int n, long long batch, int arith, double *logabs,
                    double *phase, int8_t *parity, int32_t *status, cudaStream_t stream,
                    int status_or = 0);
int launch_mixed_cf(const CfSource &src, int n, long long batch, double *logabs, double *phase,
                    int8_t *parity, int32_t *status, cudaStream_t stream);

}  // namespace lufqhe
