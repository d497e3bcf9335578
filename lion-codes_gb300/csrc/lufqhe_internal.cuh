// Internal helpers shared by the lufqhe CUDA translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "lufqhe.h"

namespace lufqhe {

constexpr unsigned kFull = 0xffffffffu;
constexpr double kPi = 3.14159265358979323846;
constexpr double kTwoPi = 6.28318530717958647692;
constexpr double kLn2 = 0.69314718055994530942;

// ---- error reporting (host) ------------------------------------------------
void set_error(const char *fmt, ...);
int check_cuda(cudaError_t e, const char *what);
int device_sm_count();
size_t device_smem_optin();
// Device address of p: p itself for device memory, the mapped view for
// page-locked host memory (which kernels then read and write over the host link).
const void *device_address(const void *p);
// True if p points into device memory (not mapped host memory): the bulk-copy
// loads are used only there.
bool is_device_memory(const void *p);
extern int g_bulk_loads;  // option LUFQHE_OPT_BULK_LOADS
// Stream-ordered device memory from the library's own pool.
int lib_malloc_async(void **p, size_t bytes, cudaStream_t s);
int lib_free_async(void *p, cudaStream_t s);
// Bytes a batched mixed call of this n and batch takes from that pool.
size_t mixed_workspace_bytes(int n, long long batch);

// Per-kernel timing for measurement (option LUFQHE_OPT_KERNEL_TIMING): while
// it is on, a KernelTimer records a CUDA event on the launching stream before
// and after the launch it brackets, and files the pair under the kernel's
// name (with n) for lufqhe_kernel_times. Off (the default), or while the
// stream is being captured, it does nothing.
class KernelTimer {
 public:
  KernelTimer(const char *name, int n, cudaStream_t stream);
  void stop();
  ~KernelTimer() { stop(); }

 private:
  const char *name_;
  int n_;
  cudaStream_t stream_;
  cudaEvent_t e0_ = nullptr;
};

// ---- IEEE helpers ----------------------------------------------------------
__device__ __forceinline__ bool finite_d(double v) {
  return (__double2hiint(v) & 0x7ff00000) != 0x7ff00000;
}
__device__ __forceinline__ bool finite_c(double2 v) { return finite_d(v.x) && finite_d(v.y); }
__device__ __forceinline__ bool is_zero_c(double2 v) {
  return ((__double_as_longlong(v.x) | __double_as_longlong(v.y)) << 1) == 0;
}
// |x| bit pattern; for non-negative doubles the integer order is the numeric order.
__device__ __forceinline__ long long abs_bits(double v) {
  return __double_as_longlong(v) & 0x7fffffffffffffffll;
}

// Wrap an angle to (-pi, pi]. k*2pi is formed inside the fma, so the result
// equals the exactly rounded x - k*2pi.
__device__ __forceinline__ double wrap_phase(double x) {
  double k = rint(x * (1.0 / kTwoPi));
  double r = __fma_rn(-k, kTwoPi, x);
  if (r > kPi) r -= kTwoPi;
  if (r <= -kPi) r += kTwoPi;
  return r;
}

// ---- compact FP64 log|u| and arg u --------------------------------------------
// Per-entry logs of an LU diagonal cost as much FP64-pipe time as a sizeable
// share of the factorisation itself at n <= 32 (each is one SIMT pass of the
// whole routine). These routines are shorter than the library's log(hypot())
// and atan2: no hypot, quotients as a * RN(1/b), short series after exact
// range reductions. Both are accurate to a few ulps. Entries with a component
// outside [2^-500, 2^500] (where |u|^2 or 1/max(|x|,|y|) could leave the
// normal range) take the library routines.
//
// log m for m in [1, 2) (k: the caller's power of two): m > sqrt(2) is halved
// into [sqrt(1/2), sqrt(2)); log m = 2 atanh(s) = 2 (s + s^3/3 + ...),
// s = (m - 1) / (m + 1), |s| <= 0.1716; the terms to s^23 leave a relative
// remainder below 1e-19.
__device__ __forceinline__ double log_mantissa(double a, int &k) {
  long long bits = __double_as_longlong(a);
  k = (int)((bits >> 52) & 0x7ff) - 1023;
  bits = (bits & 0x000fffffffffffffll) | 0x3ff0000000000000ll;  // m in [1, 2)
  double m = __longlong_as_double(bits);
  if (m > 1.4142135623730951) {
    m = __dmul_rn(m, 0.5);
    k += 1;
  }
  const double s = __dmul_rn(__dadd_rn(m, -1.0), __drcp_rn(__dadd_rn(m, 1.0)));
  const double z = __dmul_rn(s, s);
  double t = 1.0 / 23.0;
#pragma unroll
  for (int j = 21; j >= 1; j -= 2) t = __fma_rn(t, z, 1.0 / (double)j);
  return __dmul_rn(2.0 * s, t);
}

// atan2(y, x) for (x, y) != (0, 0) with max(|x|, |y|) in [2^-500, 2^500].
// Octant reduction to t = min(|x|,|y|) / max(|x|,|y|) in [0, 1]; with
// c_i = tan(i pi/16) the nearest of five points (i = 0..4),
// atan t = i pi/16 + atan v, v = (t - c_i) / (1 + t c_i), |v| <= tan(pi/32)
// < 0.0985, and the Taylor series v - v^3/3 + ... to v^17 (remainder below
// 5e-21).
__device__ __forceinline__ double atan2_reduced(double y, double x) {
  const double ax = fabs(x), ay = fabs(y);
  const bool swap = ay > ax;
  const double t = __dmul_rn(swap ? ax : ay, __drcp_rn(swap ? ay : ax));
  // the midpoints tan((2i + 1) pi/32) pick the nearest c_i
  const int i = (t > 0.09849140335716425) + (t > 0.3033466836073424) +
                (t > 0.5345111359507916) + (t > 0.8206787908286602);
  const double c = i == 0   ? 0.0
                   : i == 1 ? 0.198912367379658
                   : i == 2 ? 0.41421356237309503
                   : i == 3 ? 0.6681786379192989
                            : 1.0;
  const double v = __dmul_rn(__dadd_rn(t, -c), __drcp_rn(__fma_rn(t, c, 1.0)));
  const double z = __dmul_rn(v, v);
  double p = 1.0 / 17.0;
#pragma unroll
  for (int j = 15; j >= 1; j -= 2) p = __fma_rn(p, -z, 1.0 / (double)j);
  double r = __fma_rn(v, p, (double)i * (kPi / 16.0));
  if (swap) r = __dadd_rn(0.5 * kPi, -r);
  if (x < 0.0) r = __dadd_rn(kPi, -r);
  return y < 0.0 ? -r : r;
}

// log|u| and arg u of a nonzero finite complex number.
__device__ __forceinline__ void log_arg_c(double2 u, double &lg, double &ar) {
  const long long big = max(abs_bits(u.x), abs_bits(u.y));
  if (big >= 0x20b0000000000000ll && big < 0x5f30000000000000ll) {  // [2^-500, 2^500)
    int k;
    const double lm = log_mantissa(__fma_rn(u.x, u.x, __dmul_rn(u.y, u.y)), k);
    lg = __fma_rn((double)k, 0.5 * kLn2, __dmul_rn(0.5, lm));
    ar = atan2_reduced(u.y, u.x);
  } else {
    lg = log(hypot(u.x, u.y));
    ar = atan2(u.y, u.x);
  }
}

// ---- complex arithmetic in the two operation orders -------------------------
// ARITH_REF reproduces the reference's CPU Crout arithmetic
// (LU-fqhe/src/LUCoreCPU.cu:173-177 and :243-247) operation for operation:
// every product and sum is rounded on its own; the explicit _rn intrinsics
// keep the compiler from contracting them into FMAs.
// ARITH_FUSED uses FMAs and one reciprocal per column.
enum { ARITH_REF = 0, ARITH_FUSED = 1 };

template <int ARITH>
__device__ __forceinline__ double2 cmsub(double2 s, double2 l, double2 u) {
  if (ARITH == ARITH_REF) {
    double tx = __dsub_rn(__dmul_rn(l.x, u.x), __dmul_rn(l.y, u.y));
    double ty = __dadd_rn(__dmul_rn(l.y, u.x), __dmul_rn(l.x, u.y));
    return make_double2(__dsub_rn(s.x, tx), __dsub_rn(s.y, ty));
  } else {
    double sx = __fma_rn(-l.x, u.x, s.x);
    sx = __fma_rn(l.y, u.y, sx);
    double sy = __fma_rn(-l.y, u.x, s.y);
    sy = __fma_rn(-l.x, u.y, sy);
    return make_double2(sx, sy);
  }
}

// Per-column constant of the multiplier division.
template <int ARITH>
__device__ __forceinline__ double pivot_den(double2 p) {
  if (ARITH == ARITH_REF) return __dadd_rn(__dmul_rn(p.x, p.x), __dmul_rn(p.y, p.y));
  return __drcp_rn(__fma_rn(p.x, p.x, __dmul_rn(p.y, p.y)));  // reciprocal of |p|^2
}

// a / p given pivot_den(p).
template <int ARITH>
__device__ __forceinline__ double2 cdiv_pivot(double2 a, double2 p, double d) {
  if (ARITH == ARITH_REF) {
    double nx = __dadd_rn(__dmul_rn(a.x, p.x), __dmul_rn(a.y, p.y));
    double ny = __dsub_rn(__dmul_rn(a.y, p.x), __dmul_rn(a.x, p.y));
    return make_double2(__ddiv_rn(nx, d), __ddiv_rn(ny, d));
  } else {
    double nx = __fma_rn(a.x, p.x, __dmul_rn(a.y, p.y));
    double ny = __fma_rn(a.y, p.x, -__dmul_rn(a.x, p.y));
    return make_double2(__dmul_rn(nx, d), __dmul_rn(ny, d));
  }
}

// ---- seeded counter-based RNG (SplitMix64 finaliser) ------------------------
__host__ __device__ __forceinline__ unsigned long long mix64(unsigned long long x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}
// Uniform in (0,1) from a 64-bit counter under a seed.
__host__ __device__ __forceinline__ double uniform01(unsigned long long key,
                                                     unsigned long long ctr) {
  unsigned long long r = mix64(key + ctr * 0xD2B74407B1CE6E93ull);
  return ((double)(r >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}
__host__ __device__ __forceinline__ unsigned long long seed_key(unsigned long long seed) {
  return mix64(seed ^ 0x5851F42D4C957F2Dull);
}

// ---- launches implemented in the .cu files ---------------------------------
// status_or: bits OR-ed into every status (mixed mode's FP64 route)
int launch_plain(const double2 *A, double2 *Aout, int n, int lda, long long batch, int arith,
                 double *logabs, double *phase, int8_t *parity, int32_t *status,
                 cudaStream_t stream, int status_or = 0);
// Mixed mode's precision policy: the share (in 1/65536) of n x n matrices
// sent straight to the FP64 kernel, chosen by content hash.
unsigned int fp64_share_64k(int n);
// Same kernels on LLL orbital matrices built from n coordinates per matrix.
int launch_plain_lll(const double2 *Z, int n, long long batch, int arith, double *logabs,
                     double *phase, int8_t *parity, int32_t *status, cudaStream_t stream,
                     int status_or = 0);
int launch_mixed_lll(const double2 *Z, int n, long long batch, double *logabs, double *phase,
                     int8_t *parity, int32_t *status, cudaStream_t stream);
// inplace: FP64 refactorisations stay in the FP32 pass (no second kernel);
// used when A is read over the host link.
int launch_mixed(const double2 *A, int n, int lda, long long batch, double *logabs,
                 double *phase, int8_t *parity, int32_t *status, cudaStream_t stream,
                 bool inplace = false);
int launch_write_det(double2 *A, int n, int lda, long long batch, const double *logabs,
                     const double *phase, const int32_t *status, int pair_product,
                     cudaStream_t stream);
// complex64 batches (the reference's float2 buffers): widened to FP64 on load
int launch_plain32(const float2 *A, float2 *Aout, int n, int lda, long long batch, int arith,
                   double *logabs, double *phase, int8_t *parity, int32_t *status,
                   cudaStream_t stream, int status_or = 0);
int launch_mixed32(const float2 *A, int n, int lda, long long batch, double *logabs,
                   double *phase, int8_t *parity, int32_t *status, cudaStream_t stream);
int launch_write_det32(float2 *A, int n, int lda, long long batch, const double *logabs,
                       const double *phase, const int32_t *status, int pair_product,
                       cudaStream_t stream);
// Batched call on device (or mapped) memory of either element type.
int batch_det_device(const void *A, int dtype, int n, int lda, long long batch, int mode,
                     double *logabs, double *phase, int8_t *parity, int32_t *status,
                     cudaStream_t s, bool host_link);
// Bytes of one matrix element of dtype (LUFQHE_C128 / LUFQHE_C64), 0 if unknown.
inline size_t dtype_bytes(int dtype) {
  return dtype == LUFQHE_C128 ? 16 : dtype == LUFQHE_C64 ? 8 : 0;
}

}  // namespace lufqhe
