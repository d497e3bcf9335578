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
int launch_mixed(const double2 *A, int n, int lda, long long batch, double *logabs,
                 double *phase, int8_t *parity, int32_t *status, cudaStream_t stream);
int launch_write_det(double2 *A, int n, int lda, long long batch, const double *logabs,
                     const double *phase, const int32_t *status, int pair_product,
                     cudaStream_t stream);

}  // namespace lufqhe
