// Wavefunction assembly step after the determinants: the sum over pairs
//   S = sum_i det(A_2i) * det(A_2i+1),   i < batch/2 (an odd last matrix is
// dropped, as LUCoreCPU::CALL does at LU-fqhe/src/LUCoreCPU.cu:83),
// which the reference forms by a pair product in the LU kernel
// (LU-fqhe/src/LUCoreGPU.cu:403-425) and a multi-pass tree sum
// (LU-fqhe/src/LUCoreGPU.cu:113-156, :444-557). Here it is one launch over the
// log-polar determinants, as a complex log-sum-exp so that it cannot
// overflow: S = exp(M) * sum_i exp(l_i - M) e^{i theta_i} with M = max l_i.
// One CTA of 1024 threads; fixed thread-to-pair mapping and a fixed tree
// order make the result reproducible.
#include <algorithm>
#include <cmath>

#include "lufqhe_internal.cuh"

namespace lufqhe {
namespace {

constexpr int kThreads = 1024;

__global__ void __launch_bounds__(kThreads)
    pair_sum_kernel(const double *logabs, const double *phase, long long npair, double *out) {
  __shared__ double smax[kThreads / 32];
  __shared__ double sre[kThreads / 32], sim[kThreads / 32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // pass 1: maximum of l_i = log|det A_2i| + log|det A_2i+1|
  double m = -INFINITY;
  for (long long i = tid; i < npair; i += kThreads) {
    const double l = logabs[2 * i] + logabs[2 * i + 1];
    if (l > m) m = l;  // NaN never wins
  }
  for (int off = 16; off; off >>= 1) m = fmax(m, __shfl_xor_sync(kFull, m, off));
  if (lane == 0) smax[warp] = m;
  __syncthreads();
  if (warp == 0) {
    m = smax[lane];
    for (int off = 16; off; off >>= 1) m = fmax(m, __shfl_xor_sync(kFull, m, off));
    if (lane == 0) smax[0] = m;
  }
  __syncthreads();
  const double M = smax[0];
  // pass 2: sum of exp(l_i - M) e^{i theta_i}
  double re = 0.0, im = 0.0;
  if (M > -INFINITY && M < INFINITY) {
    for (long long i = tid; i < npair; i += kThreads) {
      const double l = logabs[2 * i] + logabs[2 * i + 1] - M;
      const double th = phase[2 * i] + phase[2 * i + 1];
      const double w = exp(l);
      double s, c;
      sincos(th, &s, &c);
      re += w * c;
      im += w * s;
    }
  }
  for (int off = 16; off; off >>= 1) {
    re += __shfl_xor_sync(kFull, re, off);
    im += __shfl_xor_sync(kFull, im, off);
  }
  if (lane == 0) {
    sre[warp] = re;
    sim[warp] = im;
  }
  __syncthreads();
  if (warp == 0) {
    re = sre[lane];
    im = sim[lane];
    for (int off = 16; off; off >>= 1) {
      re += __shfl_xor_sync(kFull, re, off);
      im += __shfl_xor_sync(kFull, im, off);
    }
    if (lane == 0) {
      out[0] = (M > -INFINITY && M < INFINITY) ? M + log(hypot(re, im)) : M;
      out[1] = atan2(im, re);
    }
  }
}

}  // namespace
}  // namespace lufqhe

using namespace lufqhe;

extern "C" int lufqhe_pair_sum(const double *d_logabs, const double *d_phase, long long batch,
                               double *d_out, void *stream) {
  if (batch < 0 || !d_out || (batch > 1 && (!d_logabs || !d_phase))) {
    set_error("lufqhe_pair_sum: invalid argument");
    return LUFQHE_ERR_INVALID_ARG;
  }
  pair_sum_kernel<<<1, kThreads, 0, (cudaStream_t)stream>>>(d_logabs, d_phase, batch / 2, d_out);
  return check_cuda(cudaGetLastError(), "pair_sum_kernel launch");
}

// ---------------------------------------------------------------------------
// The same sum fused into the factorisation (plain modes): the reference forms
// the pair product inside its LU kernel (LU-fqhe/src/LUCoreGPU.cu:403-425)
// before a separate tree sum; here each warp factorises both matrices of a
// pair, adds the pair's product to its own running complex log-sum-exp, and
// the partial sums never leave the chip until one per CTA is written; the last
// CTA to finish combines them in CTA order. No per-matrix result is written,
// so a Monte Carlo step that needs only the wavefunction sum reads 16 n^2
// bytes per matrix and writes 16 bytes in all.
#include "lup_fp64.cuh"

namespace lufqhe {
namespace {

// exp(m) * (re + i im), streaming: a term larger than the running maximum
// rescales what was summed so far. A NaN term makes the sum NaN; a -inf term
// (a singular matrix) adds nothing.
struct LseAcc {
  double m = -INFINITY, re = 0.0, im = 0.0;
  __device__ __forceinline__ void add_vec(double l, double x, double y) {
    if (l != l) {
      re = im = NAN;
      return;
    }
    if (l == -INFINITY) return;
    if (l > m) {
      const double s = exp(m - l);  // 0 when m = -inf
      re = __fma_rn(re, s, x);
      im = __fma_rn(im, s, y);
      m = l;
    } else {
      const double w = exp(l - m);
      re = __fma_rn(w, x, re);
      im = __fma_rn(w, y, im);
    }
  }
  __device__ __forceinline__ void add(double l, double th) {
    double s, c;
    sincos(th, &s, &c);
    add_vec(l, c, s);
  }
  __device__ __forceinline__ void merge(const LseAcc &o) {
    if (o.re != o.re || o.im != o.im) {
      re = im = NAN;
      return;
    }
    add_vec(o.m, o.re, o.im);
  }
};

__device__ __forceinline__ LseAcc shfl_lse(const LseAcc &a, int off) {
  LseAcc r;
  r.m = __shfl_xor_sync(kFull, a.m, off);
  r.re = __shfl_xor_sync(kFull, a.re, off);
  r.im = __shfl_xor_sync(kFull, a.im, off);
  return r;
}

constexpr int kFusedWarps = 4;

// Per call, in the library's pool: [counter (8 B, zeroed)][pad][3 doubles per CTA]
struct FusedScratch {
  unsigned int done;
  unsigned int pad[63];
};

template <int ARITH, class Src>
__global__ void __launch_bounds__(kFusedWarps * 32)
    pair_sum_fused_kernel(Src src, int n, long long npair, FusedScratch *scratch, double *out) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double part[kFusedWarps][3];
  __shared__ bool last;
  const int warps = blockDim.x >> 5;
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int lds = n + 1;
  double2 *M = reinterpret_cast<double2 *>(smem_raw) + (size_t)warp * n * lds;
  double *hold = reinterpret_cast<double *>(reinterpret_cast<double2 *>(smem_raw) +
                                            (size_t)warps * n * lds) +
                 warp * 2 * n;
  LseAcc acc;  // identical on every lane of the warp
  const long long stride = (long long)gridDim.x * warps;
  for (long long p = (long long)blockIdx.x * warps + warp; p < npair; p += stride) {
    double l = 0.0, th = 0.0;
    for (int h = 0; h < 2; ++h) {
      __syncwarp();
      int par = 0;
      int st = src.load(2 * p + h, n, M, lds, lane) ? LUFQHE_ST_NONFINITE : 0;
      if (!st) st = lup_fp64_warp<ARITH>(M, lds, hold, n, lane, &par);
      double la, ph;
      if (st == 0) {
        logdet_from_diag(M, lds, n, lane, par, &la, &ph);
      } else if (st == LUFQHE_ST_SINGULAR) {
        la = -INFINITY;
        ph = 0.0;
      } else {
        la = NAN;
        ph = NAN;
      }
      l += la;
      th += ph;
    }
    acc.add(l, th);
  }
  if (lane == 0) {
    part[warp][0] = acc.m;
    part[warp][1] = acc.re;
    part[warp][2] = acc.im;
  }
  __syncthreads();
  double *cta_parts = reinterpret_cast<double *>(scratch + 1);
  if (threadIdx.x == 0) {
    LseAcc c;
    for (int w = 0; w < warps; ++w) {
      LseAcc o;
      o.m = part[w][0];
      o.re = part[w][1];
      o.im = part[w][2];
      c.merge(o);
    }
    cta_parts[3 * blockIdx.x] = c.m;
    cta_parts[3 * blockIdx.x + 1] = c.re;
    cta_parts[3 * blockIdx.x + 2] = c.im;
    __threadfence();
    last = atomicAdd(&scratch->done, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last || warp != 0) return;
  // the last CTA: every lane folds a fixed stride of the CTA partials, then a
  // fixed butterfly; the order depends on the grid only, so the sum is
  // reproducible
  __threadfence();
  LseAcc c;
  for (unsigned int b = lane; b < gridDim.x; b += 32) {
    LseAcc o;
    o.m = __ldcg(cta_parts + 3 * b);
    o.re = __ldcg(cta_parts + 3 * b + 1);
    o.im = __ldcg(cta_parts + 3 * b + 2);
    c.merge(o);
  }
#pragma unroll
  for (int off = 16; off; off >>= 1) {
    const LseAcc o = shfl_lse(c, off);
    c.merge(o);
  }
  if (lane == 0) {  // lane 0 merged in a fixed order
    const bool empty = !(c.m > -INFINITY);
    out[0] = (c.re != c.re) ? NAN : empty ? -INFINITY : c.m + log(hypot(c.re, c.im));
    out[1] = (c.re != c.re) ? NAN : empty ? 0.0 : atan2(c.im, c.re);
  }
}

template <class Src>
int launch_pair_sum_fused(Src src, int n, long long npair, int arith, double *out,
                          cudaStream_t stream) {
  const size_t per_warp = (size_t)n * (n + 1) * sizeof(double2) + 2 * (size_t)n * sizeof(double);
  const size_t smem = per_warp * kFusedWarps;
  auto kern = arith == ARITH_REF ? pair_sum_fused_kernel<ARITH_REF, Src>
                                 : pair_sum_fused_kernel<ARITH_FUSED, Src>;
  int rc = check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem),
                      "cudaFuncSetAttribute(pair sum fused)");
  if (rc) return rc;
  int per_sm = 0;
  rc = check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kFusedWarps * 32,
                                                                smem),
                  "occupancy(pair sum fused)");
  if (rc) return rc;
  if (per_sm < 1) {
    set_error("lufqhe_batch_pair_sum: n=%d does not fit one warp per matrix", n);
    return LUFQHE_ERR_UNSUPPORTED_N;
  }
  const long long want = (npair + kFusedWarps - 1) / kFusedWarps;
  const long long cap = (long long)device_sm_count() * per_sm;
  const int grid = (int)std::max<long long>(1, want < cap ? want : cap);
  FusedScratch *scratch = nullptr;
  rc = lib_malloc_async((void **)&scratch, sizeof(FusedScratch) + 3 * sizeof(double) * grid,
                        stream);
  if (rc) return rc;
  rc = check_cuda(cudaMemsetAsync(scratch, 0, sizeof(FusedScratch), stream), "memset(pair sum)");
  if (!rc) {
    KernelTimer timer("pair_sum_fused_kernel", n, stream);
    kern<<<grid, kFusedWarps * 32, smem, stream>>>(src, n, npair, scratch, out);
    timer.stop();
    rc = check_cuda(cudaGetLastError(), "pair_sum_fused_kernel launch");
  }
  const int r2 = lib_free_async(scratch, stream);
  return rc ? rc : r2;
}

}  // namespace
}  // namespace lufqhe

extern "C" int lufqhe_batch_pair_sum(const void *d_A, int n, int lda, long long batch, int dtype,
                                     int mode, double *d_out, void *stream) {
  const size_t eb = dtype_bytes(dtype);
  if (!eb) {
    set_error("lufqhe_batch_pair_sum: unknown dtype %d", dtype);
    return LUFQHE_ERR_UNSUPPORTED_MODE;
  }
  if (!d_out || n < 1 || lda < n || batch < 0 || (batch > 1 && !d_A) ||
      (reinterpret_cast<uintptr_t>(d_A) & (eb - 1)) != 0) {
    set_error("lufqhe_batch_pair_sum: invalid argument");
    return LUFQHE_ERR_INVALID_ARG;
  }
  if (n > LUFQHE_MAX_N) {
    set_error("lufqhe_batch_pair_sum: n=%d exceeds %d", n, LUFQHE_MAX_N);
    return LUFQHE_ERR_UNSUPPORTED_N;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const long long npair = batch / 2;
  if (mode == LUFQHE_MODE_PLAIN_FP64 || mode == LUFQHE_MODE_PLAIN_FP64_FUSED) {
    const int arith = mode == LUFQHE_MODE_PLAIN_FP64 ? ARITH_REF : ARITH_FUSED;
    if (n <= 32) {
      if (dtype == LUFQHE_C64)
        return launch_pair_sum_fused(Dense32Source{static_cast<const float2 *>(d_A), lda}, n,
                                     npair, arith, d_out, s);
      return launch_pair_sum_fused(DenseSource{static_cast<const double2 *>(d_A), lda}, n, npair,
                                   arith, d_out, s);
    }
  } else if (mode != LUFQHE_MODE_MIXED) {
    set_error("lufqhe_batch_pair_sum: unknown mode %d", mode);
    return LUFQHE_ERR_UNSUPPORTED_MODE;
  }
  // mixed mode (its determinants come from more than one kernel) and n > 32
  // (one matrix per warp group): the batched call into pool temporaries, then
  // the log-sum-exp pass over them
  const long long nm = 2 * npair;
  double *tmp = nullptr;
  int rc = lib_malloc_async((void **)&tmp, sizeof(double) * 2 * std::max(1ll, nm), s);
  if (rc) return rc;
  if (nm > 0)
    rc = batch_det_device(d_A, dtype, n, lda, nm, mode, tmp, tmp + nm, nullptr, nullptr, s,
                          false);
  if (!rc) {
    pair_sum_kernel<<<1, kThreads, 0, s>>>(tmp, tmp + nm, npair, d_out);
    rc = check_cuda(cudaGetLastError(), "pair_sum_kernel launch");
  }
  const int r2 = lib_free_async(tmp, s);
  return rc ? rc : r2;
}
