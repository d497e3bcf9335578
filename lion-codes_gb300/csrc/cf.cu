// Composite-fermion determinants: matrices built inside the factorising
// kernels from one configuration's angles and a batch of permutations
// (cf_source.cuh), the C-ABI entry points, and a builder that writes the
// matrices out as the reference's mkMatrixElements does
// (LU-fqhe/src/mkMatrixElements.cu:295-358).

#include <algorithm>
#include <cmath>
#include <vector>

#include "cf_source.cuh"
#include "mixed_kernels.cuh"

namespace lufqhe {

namespace {

// Host complex arithmetic for the tables (the host code is compiled without
// contraction, so each operation is rounded once, on any host).
inline double2 h_mul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
inline double2 h_div(double2 a, double2 b) {
  const double den = b.x * b.x + b.y * b.y;
  return make_double2((a.x * b.x + a.y * b.y) / den, (a.y * b.x - a.x * b.y) / den);
}

__global__ void cf_columns_kernel(CfParams prm, double2 *cols, int n, long long batch) {
  const long long total = batch * n;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const long long b = e / n;
    const int r = (int)(e - b * n);
    double2 e1, e2;
    prm.last_columns(b, n, r, e1, e2);
    cols[2 * e] = e1;
    cols[2 * e + 1] = e2;
  }
}

template <class T>
__global__ void gen_cf_kernel(CfSource src, T *A, int n, int lda, long long batch) {
  const long long total = batch * n;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const long long b = e / n;
    const int r = (int)(e - b * n);
    src.row(b, n, r, A + (size_t)b * n * lda + (size_t)r * lda);
  }
}

int grid_for(long long threads) {
  long long g = (threads + 255) / 256;
  const long long cap = (long long)device_sm_count() * 8;
  return (int)(g < cap ? (g < 1 ? 1 : g) : cap);
}

// One call's device state: the configuration's tables and, for a chunk of
// the batch at a time, the last two columns of its matrices, both from the
// library's pool. The tables are uploaded from pageable memory, which orders
// the call after the stream's earlier work (and cannot be captured).
struct CfCall {
  static constexpr long long kColsBytes = 1ll << 31;  // per chunk
  void *mem = nullptr;
  CfParams prm{};
  double2 *cols = nullptr;
  int n = 0;
  long long chunk = 0;
  int open(const double *phi, const double *theta, int np, int n_, double k1, double k2,
           double r1, double r2, int mu, int nu, const int16_t *perm, int perm_stride,
           long long batch, cudaStream_t s) {
    n = n_;
    chunk = std::max<long long>(1, kColsBytes / (32ll * n));
    chunk = std::min(chunk, batch);
    const size_t tab_elems = (size_t)np * n + 2 * (size_t)np;
    std::vector<double2> host(tab_elems);
    double2 *uv = host.data(), *tab = uv + 2 * (size_t)np;
    cf_tables(phi, theta, np, n, uv, tab);
    const size_t tab_bytes = (tab_elems * sizeof(double2) + 255) & ~(size_t)255;
    int rc = lib_malloc_async(&mem, tab_bytes + (size_t)chunk * n * 2 * sizeof(double2), s);
    if (rc) return rc;
    rc = check_cuda(cudaMemcpyAsync(mem, host.data(), tab_elems * sizeof(double2),
                                    cudaMemcpyHostToDevice, s),
                    "cudaMemcpyAsync (CF tables)");
    if (rc) return rc;
    const double2 *d = static_cast<const double2 *>(mem);
    cols = reinterpret_cast<double2 *>(static_cast<char *>(mem) + tab_bytes);
    const int q1 = (n - 3) / 2 + 1;
    prm = CfParams{d + 2 * (size_t)np,
                   d,
                   static_cast<const short *>(device_address(perm)),
                   perm_stride,
                   np,
                   q1 + mu,
                   q1 + nu,
                   k1,
                   k2,
                   r1,
                   r2};
    return LUFQHE_SUCCESS;
  }
  // the last two columns of matrices [off, off + m), and their source
  int columns(long long off, long long m, CfSource *src, cudaStream_t s) {
    CfParams p = prm;
    p.perm += (size_t)off * prm.pstride;
    {
      KernelTimer timer("cf_columns_kernel", n, s);
      cf_columns_kernel<<<grid_for(m * n), 256, 0, s>>>(p, cols, n, m);
      timer.stop();
    }
    *src = CfSource{prm.tab, p.perm, cols, prm.pstride, prm.np};
    return check_cuda(cudaGetLastError(), "cf_columns_kernel launch");
  }
  int close(cudaStream_t s, int rc) {
    if (mem) {
      const int rf = lib_free_async(mem, s);
      mem = nullptr;
      if (!rc) rc = rf;
    }
    return rc;
  }
};

int check_cf(const char *fn, const double *phi, const double *theta, int np, int n, int mu,
             int nu, const int16_t *perm, int perm_stride, long long batch) {
  if (!phi || !theta || batch < 0 || (batch > 0 && !perm) || n < 3 || (n & 1) == 0 ||
      np < n || np > 32767 || perm_stride < n) {
    set_error("%s: invalid argument (n=%d must be odd and >= 3, np=%d in [n, 32767], "
              "perm_stride=%d >= n, batch=%lld)",
              fn, n, np, perm_stride, batch);
    return LUFQHE_ERR_INVALID_ARG;
  }
  if (n > LUFQHE_MAX_N) {
    set_error("%s: n=%d exceeds the supported maximum %d", fn, n, LUFQHE_MAX_N);
    return LUFQHE_ERR_UNSUPPORTED_N;
  }
  const int q1 = (n - 3) / 2 + 1;
  if (q1 + mu < 0 || q1 + mu >= n || q1 + nu < 0 || q1 + nu >= n) {
    set_error("%s: mu=%d, nu=%d must lie in [%d, %d]", fn, mu, nu, -q1, n - 1 - q1);
    return LUFQHE_ERR_INVALID_ARG;
  }
  if ((reinterpret_cast<uintptr_t>(perm) & 1) != 0) {
    set_error("%s: perm must be 2-byte aligned", fn);
    return LUFQHE_ERR_INVALID_ARG;
  }
  return LUFQHE_SUCCESS;
}

}  // namespace

void cf_tables(const double *phi, const double *theta, int np, int n, double2 *uv,
               double2 *tab) {
  const int Q = (n - 3) / 2;
  for (int p = 0; p < np; ++p) {
    const double ct = std::cos(theta[p]), st = std::sin(theta[p]);
    const double cp = std::cos(phi[p]), sp = std::sin(phi[p]);
    const double2 u = make_double2(ct * cp, ct * sp);
    const double2 v = make_double2(st * cp, -(st * sp));
    uv[p] = u;
    uv[np + p] = v;
    const double2 zplus = h_div(u, v), zminus = h_div(v, u);
    double2 *t = tab + (size_t)p * n;
    t[Q + 1] = make_double2(std::pow(ct * st, (double)Q), 0.0);
    for (int j = 1; j < Q + 2; ++j) {
      t[Q + 1 + j] = h_mul(t[Q + j], zplus);
      t[Q + 1 - j] = h_mul(t[Q + 2 - j], zminus);
    }
  }
}

int launch_mixed_cf(const CfSource &src, int n, long long batch, double *logabs, double *phase,
                    int8_t *parity, int32_t *status, cudaStream_t stream) {
  return launch_mixed_src(src, n, batch, logabs, phase, parity, status, stream, [&] {
    return launch_plain_cf(src, n, batch, ARITH_FUSED, logabs, phase, parity, status, stream,
                           LUFQHE_ST_FP64);
  });
}

}  // namespace lufqhe

using namespace lufqhe;

extern "C" int lufqhe_cf_tables(const double *phi, const double *theta, int np, int n,
                                double *uv, double *tab) {
  if (!phi || !theta || !uv || !tab || n < 3 || (n & 1) == 0 || np < 1) {
    set_error("lufqhe_cf_tables: invalid argument");
    return LUFQHE_ERR_INVALID_ARG;
  }
  cf_tables(phi, theta, np, n, reinterpret_cast<double2 *>(uv), reinterpret_cast<double2 *>(tab));
  return LUFQHE_SUCCESS;
}

extern "C" int lufqhe_gen_cf(const double *phi, const double *theta, int np, int n, double k1,
                             double k2, double r1, double r2, int mu, int nu,
                             const int16_t *d_perm, int perm_stride, long long batch, void *d_A,
                             int lda, int dtype, void *stream) {
  int rc = check_cf("lufqhe_gen_cf", phi, theta, np, n, mu, nu, d_perm, perm_stride, batch);
  if (rc) return rc;
  if (!dtype_bytes(dtype) || (batch > 0 && !d_A) || lda < n ||
      (reinterpret_cast<uintptr_t>(d_A) & (dtype_bytes(dtype) - 1)) != 0) {
    set_error("lufqhe_gen_cf: invalid output (A=%p lda=%d dtype=%d)", d_A, lda, dtype);
    return LUFQHE_ERR_INVALID_ARG;
  }
  if (batch == 0) return LUFQHE_SUCCESS;
  cudaStream_t s = (cudaStream_t)stream;
  CfCall call;
  rc = call.open(phi, theta, np, n, k1, k2, r1, r2, mu, nu, d_perm, perm_stride, batch, s);
  char *A = static_cast<char *>(const_cast<void *>(device_address(d_A)));
  for (long long off = 0; !rc && off < batch; off += call.chunk) {
    const long long m = std::min(call.chunk, batch - off);
    CfSource src;
    rc = call.columns(off, m, &src, s);
    if (rc) break;
    void *Ab = A + (size_t)off * n * lda * dtype_bytes(dtype);
    if (dtype == LUFQHE_C128)
      gen_cf_kernel<double2><<<grid_for(m * n), 256, 0, s>>>(src, static_cast<double2 *>(Ab), n,
                                                              lda, m);
    else
      gen_cf_kernel<float2><<<grid_for(m * n), 256, 0, s>>>(src, static_cast<float2 *>(Ab), n,
                                                             lda, m);
    rc = check_cuda(cudaGetLastError(), "gen_cf_kernel launch");
  }
  return call.close(s, rc);
}

extern "C" int lufqhe_cf_det(const double *phi, const double *theta, int np, int n, double k1,
                             double k2, double r1, double r2, int mu, int nu,
                             const int16_t *d_perm, int perm_stride, long long batch, int mode,
                             double *d_logabs, double *d_phase, int8_t *d_parity,
                             int32_t *d_status, void *stream) {
  int rc = check_cf("lufqhe_cf_det", phi, theta, np, n, mu, nu, d_perm, perm_stride, batch);
  if (rc) return rc;
  if (batch > 0 && !d_logabs) {
    set_error("lufqhe_cf_det: logabs is null");
    return LUFQHE_ERR_INVALID_ARG;
  }
  if (mode != LUFQHE_MODE_PLAIN_FP64 && mode != LUFQHE_MODE_PLAIN_FP64_FUSED &&
      mode != LUFQHE_MODE_MIXED) {
    set_error("lufqhe_cf_det: unknown mode %d", mode);
    return LUFQHE_ERR_UNSUPPORTED_MODE;
  }
  if (batch == 0) return LUFQHE_SUCCESS;
  cudaStream_t s = (cudaStream_t)stream;
  d_logabs = static_cast<double *>(const_cast<void *>(device_address(d_logabs)));
  d_phase = static_cast<double *>(const_cast<void *>(device_address(d_phase)));
  d_parity = static_cast<int8_t *>(const_cast<void *>(device_address(d_parity)));
  d_status = static_cast<int32_t *>(const_cast<void *>(device_address(d_status)));
  CfCall call;
  rc = call.open(phi, theta, np, n, k1, k2, r1, r2, mu, nu, d_perm, perm_stride, batch, s);
  for (long long off = 0; !rc && off < batch; off += call.chunk) {
    const long long m = std::min(call.chunk, batch - off);
    CfSource src;
    rc = call.columns(off, m, &src, s);
    if (rc) break;
    auto at = [off](auto *p) { return p ? p + off : p; };  // optional outputs stay null
    if (mode == LUFQHE_MODE_MIXED)
      rc = launch_mixed_cf(src, n, m, d_logabs + off, at(d_phase), at(d_parity), at(d_status), s);
    else
      rc = launch_plain_cf(src, n, m, mode == LUFQHE_MODE_PLAIN_FP64 ? ARITH_REF : ARITH_FUSED,
                           d_logabs + off, at(d_phase), at(d_parity), at(d_status), s);
  }
  return call.close(s, rc);
}
