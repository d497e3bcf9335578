// Plain FP64 batched complex LUP determinant.
//
// One warp factorises one matrix at a time, looping over the batch with a
// grid stride. The matrix sits in shared memory (row stride n+1 complex so a
// column read by 32 lanes hits 32 different banks); the right-looking update
// of the (n-1-j)^2 trailing block is spread over all 32 lanes, so the FP64
// pipe runs with full lanes until the block is smaller than a warp. The
// factorisation itself (pivot rule, arithmetic) lives in lup_fp64.cuh.
// The determinant is returned in log-polar form: the reference multiplies the
// diagonal directly (LU-fqhe/src/LUCoreCPU.cu:256-265), which overflows for
// lowest-Landau-level matrices.

#include <cmath>

#include <type_traits>

#include "bulk_copy.cuh"
#include "cf_source.cuh"
#include "fp64_correct.cuh"
#include "lup_fp64.cuh"

namespace lufqhe {

namespace {

constexpr int kMaxWarpsPlain = 8;

// Out: element type of the in-place factors (double2, or float2 for the
// reference's complex64 buffers). CORRECT: the mixed mode's FP64 route for
// 17 <= n <= 32 (this warp kernel's sizes), whose log-determinants get the
// extended-precision correction (fp64_correct_warp; its scratch follows the
// row scales in shared memory).
template <int ARITH, class Src, class Out = double2, bool CORRECT = false>
__global__ void __launch_bounds__(kMaxWarpsPlain * 32)
    lup_plain_kernel(Src src, Out *__restrict__ Aout, int n, int lda,
                     long long batch, double *__restrict__ logabs, double *__restrict__ phase,
                     int8_t *__restrict__ parity, int32_t *__restrict__ status,
                     int status_or, int bulk) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int warps = blockDim.x >> 5;
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int lds = n + 1;
  double2 *M = reinterpret_cast<double2 *>(smem_raw) + (size_t)warp * n * lds;
  double *hold_all = reinterpret_cast<double *>(reinterpret_cast<double2 *>(smem_raw) +
                                                (size_t)warps * n * lds);
  double *hold = hold_all + warp * 2 * n;
  CorrScratch cs{};
  if constexpr (CORRECT) {
    float2 *F_all = reinterpret_cast<float2 *>(hold_all + (size_t)warps * 2 * n);
    cs = CorrScratch{F_all + (size_t)warp * n * lds,
                     reinterpret_cast<int *>(F_all + (size_t)warps * n * lds) + warp * 2 * n,
                     hold};
  }
  const int nn = n * n;

  // complex128 device batches: each matrix staged by bulk copies (bulk != 0),
  // the next one prefetched into L2 meanwhile
  constexpr bool BULK = std::is_same<Src, DenseSource>::value;
  __shared__ __align__(8) uint64_t bars[kMaxWarpsPlain];
  WarpBulk wb;
  if constexpr (BULK)
    if (bulk) wb.init(&bars[warp], lane);
  const long long stride = (long long)gridDim.x * warps;
  for (long long b = (long long)blockIdx.x * warps + warp; b < batch; b += stride) {
    __syncwarp();
    int par = 0;
    int st = -1;
    if constexpr (BULK) {
      if (bulk && !wb.broken) {
        if (b + stride < batch && lane == 0)
          prefetch_matrix_l2(src.A + (size_t)(b + stride) * n * src.lda, n, src.lda);
        if (wb.load(src.A + (size_t)b * n * src.lda, n, src.lda, M, lds, lane)) {
          bool bad = false;
          BlockWalk w(lane, n);
          for (int e = lane; e < nn; e += 32) {
            bad |= !finite_c(M[w.i * lds + w.k]);
            w.next(n);
          }
          st = __any_sync(kFull, bad) ? LUFQHE_ST_NONFINITE : 0;
        } else {
          st = LUFQHE_ST_WAIT_TIMEOUT;
        }
      }
    }
    if (st < 0) st = src.load(b, n, M, lds, lane) ? LUFQHE_ST_NONFINITE : 0;
    if (!st) st = lup_fp64_warp<ARITH>(M, lds, hold, n, lane, &par, CORRECT ? cs.ints : nullptr);

    double la, ph;
    if (st == 0) {
      logdet_from_diag(M, lds, n, lane, par, &la, &ph);
      if constexpr (CORRECT) fp64_correct_warp(src, b, n, M, lds, cs, lane, &la, &ph);
    } else if (st == LUFQHE_ST_SINGULAR) {
      la = -INFINITY;
      ph = 0.0;
    } else {
      la = NAN;
      ph = NAN;
      par = 0;
    }

    if (Aout && (st == 0 || st == LUFQHE_ST_SINGULAR)) {
      Out *dst = Aout + (size_t)b * n * lda;
      BlockWalk w(lane, n);
      for (int e = lane; e < nn; e += 32) {
        store_entry(dst + (size_t)w.i * lda + w.k, M[w.i * lds + w.k]);
        w.next(n);
      }
    }
    if (lane == 0) {
      logabs[b] = la;
      if (phase) phase[b] = ph;
      if (parity) parity[b] = (int8_t)par;
      if (status) status[b] = st | status_or;
    }
  }
}

// Writes exp(logabs + i*phase) into element (0,0); with pair_product the even
// matrix of each pair gets the product of the pair's determinants
// (LU-fqhe/src/LUCoreGPU.cu:403-435).
template <class T>
__global__ void write_det_kernel(T *A, int n, int lda, long long batch,
                                 const double *logabs, const double *phase,
                                 const int32_t *status, int pair_product) {
  long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= batch) return;
  double la = logabs[b], ph = phase[b];
  if (pair_product && (b % 2 == 0) && b + 1 < batch) {
    la += logabs[b + 1];
    ph += phase[b + 1];
  }
  double2 v;
  if (la != la || ph != ph) {
    v = make_double2(NAN, NAN);
  } else {
    double m = exp(la);
    double s, c;
    sincos(ph, &s, &c);
    v = make_double2(m * c, m * s);
  }
  store_entry(A + (size_t)b * n * lda, v);
}

}  // namespace

// n > 32: one matrix per CTA of kGroupWarps warps (lup_fp64_group). With one
// warp per matrix an SM holds only the 3-4 matrices its shared memory fits
// (n=64: 66 KB each), too few warps to cover the FP64 pipe's latency.
constexpr int kGroupWarps = kFp64GroupWarps;
constexpr int kGroupMinN = kFp64GroupMinN;

// CORRECT: the mixed mode's FP64 route, whose log-determinants get the
// extended-precision correction (fp64_correct_group; its scratch follows the
// row scales in shared memory).
template <int ARITH, class Src, class Out = double2, bool CORRECT = false>
__global__ void __launch_bounds__(kGroupWarps * 32)
    lup_plain_group_kernel(Src src, Out *__restrict__ Aout, int n, int lda, long long batch,
                           double *__restrict__ logabs, double *__restrict__ phase,
                           int8_t *__restrict__ parity, int32_t *__restrict__ status,
                           int status_or) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ long long red[3 * kGroupWarps];
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int lds = n + 1;
  double2 *M = reinterpret_cast<double2 *>(smem_raw);
  double *hold = reinterpret_cast<double *>(M + (size_t)n * lds);
  CorrScratch cs{};
  if constexpr (CORRECT) {
    float2 *F = reinterpret_cast<float2 *>(hold + 2 * n);
    cs = CorrScratch{F, reinterpret_cast<int *>(F + (size_t)n * lds), hold};
  }
  for (long long b = blockIdx.x; b < batch; b += gridDim.x) {
    __syncthreads();
    int par = 0;
    int st = src.load_group(b, n, M, lds, tid, nthr) ? LUFQHE_ST_NONFINITE : 0;
    if (!st)
      st = lup_fp64_group<ARITH>(M, lds, hold, n, tid, nthr, red, &par, CtaBarrier(),
                                 CORRECT ? cs.ints : nullptr);
    __syncthreads();
    if (Aout && (st == 0 || st == LUFQHE_ST_SINGULAR)) {
      Out *dst = Aout + (size_t)b * n * lda;
      StrideWalk w(tid, nthr, n);
      for (int e = tid; e < n * n; e += nthr) {
        store_entry(dst + (size_t)w.i * lda + w.k, M[w.i * lds + w.k]);
        w.next(n);
      }
    }
    double la = 0.0, ph = 0.0;
    if (tid < 32) {
      // warp 0, with the warp routine's own summation order
      if (st == 0) {
        logdet_from_diag(M, lds, n, tid, par, &la, &ph);
      } else if (st == LUFQHE_ST_SINGULAR) {
        la = -INFINITY;
        ph = 0.0;
      } else {
        la = NAN;
        ph = NAN;
        par = 0;
      }
    }
    if constexpr (CORRECT) {
      if (st == 0) {
        __syncthreads();  // the diagonal is read before the correction overwrites M
        const double2 c = fp64_correct_group(src, b, n, M, lds, cs, tid, nthr, CtaBarrier(),
                                             reinterpret_cast<float *>(red));
        la += c.x;
        ph += c.y;
      }
    }
    if (tid == 0) {
      logabs[b] = la;
      if (phase) phase[b] = ph;
      if (parity) parity[b] = (int8_t)par;
      if (status) status[b] = st | status_or;
    }
  }
}

// the bulk-copy staging for complex128 matrices in device memory only
inline int bulk_for(const DenseSource &s) { return g_bulk_loads && is_device_memory(s.A); }
template <class S>
inline int bulk_for(const S &) {
  return 0;
}

size_t plain_smem_per_warp(int n) {
  return (size_t)n * (n + 1) * sizeof(double2) + 2 * (size_t)n * sizeof(double);
}

template <class Src, class Out = double2>
int launch_plain_src(Src src, Out *Aout, int n, int lda, long long batch, int arith,
                     double *logabs, double *phase, int8_t *parity, int32_t *status,
                     cudaStream_t stream, int status_or) {
  if (batch == 0) return LUFQHE_SUCCESS;
  // the mixed mode's FP64 route (status_or set, no factors written back)
  const bool correct = status_or != 0 && arith == ARITH_FUSED && Aout == nullptr &&
                       n >= kCorrectMinN && n <= kCorrectMaxN;
  const size_t corr_smem = (size_t)n * (n + 1) * sizeof(float2) + 2 * (size_t)n * sizeof(int);
  if (n >= kGroupMinN) {
    const size_t smem = (size_t)n * (n + 1) * sizeof(double2) + 2 * (size_t)n * sizeof(double) +
                        (correct ? corr_smem : 0);
    auto kern = correct              ? lup_plain_group_kernel<ARITH_FUSED, Src, Out, true>
                : arith == ARITH_REF ? lup_plain_group_kernel<ARITH_REF, Src, Out>
                                     : lup_plain_group_kernel<ARITH_FUSED, Src, Out>;
    int rc = check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem),
                        "cudaFuncSetAttribute(plain group)");
    if (rc) return rc;
    int per_sm = 0;
    rc = check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kGroupWarps * 32,
                                                                  smem),
                    "occupancy(plain group)");
    if (rc) return rc;
    if (per_sm < 1) {
      set_error("n=%d needs %zu bytes of shared memory per matrix", n, smem);
      return LUFQHE_ERR_UNSUPPORTED_N;
    }
    const long long cap = (long long)device_sm_count() * per_sm;
    const int grid = (int)(batch < cap ? batch : cap);
    KernelTimer timer(arith == ARITH_REF ? "lup_plain_group_kernel_ref" : "lup_plain_group_kernel",
                      n, stream);
    kern<<<grid, kGroupWarps * 32, smem, stream>>>(src, Aout, n, lda, batch, logabs, phase, parity,
                                                   status, status_or);
    timer.stop();
    return check_cuda(cudaGetLastError(), "lup_plain_group_kernel launch");
  }
  const size_t per_warp = plain_smem_per_warp(n) + (correct ? corr_smem : 0);
  const size_t optin = device_smem_optin();
  int warps = (int)(optin / per_warp);
  if (warps > 4) warps = 4;
  if (warps < 1) {
    set_error("n=%d needs %zu bytes of shared memory per matrix; the device offers %zu", n,
              per_warp, optin);
    return LUFQHE_ERR_UNSUPPORTED_N;
  }
  const size_t smem = per_warp * warps;
  auto kern = correct              ? lup_plain_kernel<ARITH_FUSED, Src, Out, true>
              : arith == ARITH_REF ? lup_plain_kernel<ARITH_REF, Src, Out>
                                   : lup_plain_kernel<ARITH_FUSED, Src, Out>;
  int rc = check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem),
                      "cudaFuncSetAttribute(plain)");
  if (rc) return rc;
  int per_sm = 0;
  rc = check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, warps * 32, smem),
                  "occupancy(plain)");
  if (rc) return rc;
  if (per_sm < 1) per_sm = 1;
  long long want = (batch + warps - 1) / warps;
  long long cap = (long long)device_sm_count() * per_sm;
  int grid = (int)(want < cap ? want : cap);
  KernelTimer timer(arith == ARITH_REF ? "lup_plain_kernel_ref" : "lup_plain_kernel", n, stream);
  kern<<<grid, warps * 32, smem, stream>>>(src, Aout, n, lda, batch, logabs, phase, parity, status,
                                           status_or, bulk_for(src));
  timer.stop();
  return check_cuda(cudaGetLastError(), "lup_plain_kernel launch");
}

int launch_plain(const double2 *A, double2 *Aout, int n, int lda, long long batch, int arith,
                 double *logabs, double *phase, int8_t *parity, int32_t *status,
                 cudaStream_t stream, int status_or) {
  return launch_plain_src(DenseSource{A, lda}, Aout, n, lda, batch, arith, logabs, phase, parity,
                          status, stream, status_or);
}

int launch_plain32(const float2 *A, float2 *Aout, int n, int lda, long long batch, int arith,
                   double *logabs, double *phase, int8_t *parity, int32_t *status,
                   cudaStream_t stream, int status_or) {
  return launch_plain_src(Dense32Source{A, lda}, Aout, n, lda, batch, arith, logabs, phase,
                          parity, status, stream, status_or);
}

int launch_plain_lll(const double2 *Z, int n, long long batch, int arith, double *logabs,
                     double *phase, int8_t *parity, int32_t *status, cudaStream_t stream,
                     int status_or) {
  return launch_plain_src(LllSource{Z}, static_cast<double2 *>(nullptr), n, n, batch, arith,
                          logabs, phase, parity, status, stream, status_or);
}

int launch_plain_cf(const CfSource &src, int n, long long batch, int arith, double *logabs,
                    double *phase, int8_t *parity, int32_t *status, cudaStream_t stream,
                    int status_or) {
  return launch_plain_src(src, static_cast<double2 *>(nullptr), n, n, batch, arith, logabs, phase,
                          parity, status, stream, status_or);
}

template <class T>
int launch_write_det_t(T *A, int n, int lda, long long batch, const double *logabs,
                       const double *phase, const int32_t *status, int pair_product,
                       cudaStream_t stream) {
  if (batch == 0) return LUFQHE_SUCCESS;
  int threads = 256;
  long long blocks = (batch + threads - 1) / threads;
  write_det_kernel<T><<<(unsigned)blocks, threads, 0, stream>>>(A, n, lda, batch, logabs, phase,
                                                                status, pair_product);
  return check_cuda(cudaGetLastError(), "write_det_kernel launch");
}

int launch_write_det(double2 *A, int n, int lda, long long batch, const double *logabs,
                     const double *phase, const int32_t *status, int pair_product,
                     cudaStream_t stream) {
  return launch_write_det_t(A, n, lda, batch, logabs, phase, status, pair_product, stream);
}

int launch_write_det32(float2 *A, int n, int lda, long long batch, const double *logabs,
                       const double *phase, const int32_t *status, int pair_product,
                       cudaStream_t stream) {
  return launch_write_det_t(A, n, lda, batch, logabs, phase, status, pair_product, stream);
}

}  // namespace lufqhe
