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
