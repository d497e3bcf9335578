// FMA-pipe peak probes: the FP64 and FP32 FMA throughput of the current
// device, measured with dependent-chain kernels (8 independent chains per
// thread, 8 warps per SM scheduler). The plain kernels are bound by the FP64
// pipe and the mixed kernel by the FP32 pipe; these figures are the
// denominators of their roofline fractions.
#include "lufqhe_internal.cuh"

namespace lufqhe {
namespace {

constexpr int kProbeIters = 4096;

template <typename T>
__global__ void fma_probe_kernel(T *out, T a, T b) {
  T x0 = (T)threadIdx.x, x1 = x0 + (T)1, x2 = x0 + (T)2, x3 = x0 + (T)3;
  T x4 = x0 + (T)4, x5 = x0 + (T)5, x6 = x0 + (T)6, x7 = x0 + (T)7;
#pragma unroll 4
  for (int i = 0; i < kProbeIters; ++i) {
    x0 = fma(x0, a, b);
    x1 = fma(x1, a, b);
    x2 = fma(x2, a, b);
    x3 = fma(x3, a, b);
    x4 = fma(x4, a, b);
    x5 = fma(x5, a, b);
    x6 = fma(x6, a, b);
    x7 = fma(x7, a, b);
  }
  // one store per thread into a buffer sized blocks*threads: always in bounds
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

template <typename T>
int probe(double *tflops, cudaStream_t s) {
  const int threads = 256;
  const int blocks = device_sm_count() * 8;
  T *buf = nullptr;
  int rc = check_cuda(cudaMallocAsync((void **)&buf, sizeof(T) * blocks * threads, s),
                      "probe alloc");
  if (rc) return rc;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  fma_probe_kernel<T><<<blocks, threads, 0, s>>>(buf, (T)0.999, (T)0.001);
  cudaEventRecord(e0, s);
  const int reps = 3;
  for (int r = 0; r < reps; ++r) fma_probe_kernel<T><<<blocks, threads, 0, s>>>(buf, (T)0.999, (T)0.001);
  cudaEventRecord(e1, s);
  rc = check_cuda(cudaEventSynchronize(e1), "probe sync");
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFreeAsync(buf, s);
  cudaStreamSynchronize(s);
  if (rc) return rc;
  const double fmas = (double)blocks * threads * kProbeIters * 8.0 * reps;
  *tflops = 2.0 * fmas / (ms * 1e-3) * 1e-12;
  return LUFQHE_SUCCESS;
}

}  // namespace
}  // namespace lufqhe

using namespace lufqhe;

extern "C" int lufqhe_probe_fma_peak(int kind, double *tflops, void *stream) {
  if (!tflops || (kind != 0 && kind != 1)) {
    set_error("lufqhe_probe_fma_peak: kind must be 0 (FP64) or 1 (FP32)");
    return LUFQHE_ERR_INVALID_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  return kind == 0 ? probe<double>(tflops, s) : probe<float>(tflops, s);
}
