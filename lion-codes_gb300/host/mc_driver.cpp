// A C++ host of the kind LU-fqhe's Monte Carlo driver is
// (LU-fqhe/src/MonteCarloLoop.cu:120-430), calling the determinants only
// through the C-ABI of liblufqhe.so (include/lufqhe.h).
//
// Each Monte Carlo step: new particle configurations for `nmat` matrices are
// built on the device (lowest-Landau-level orbitals), their determinants are
// taken in one batched call, and the wavefunction sum over determinant pairs
// (LUCoreCPU::CALL, LU-fqhe/src/LUCoreCPU.cu:82-98) is reduced on the device
// and copied back as one complex number in log-polar form. The reference does
// the same step with cudaMemcpyAsync + LUCoreGPU::CALL + globalReduction
// (LU-fqhe/src/MonteCarloLoop.cu:316-329).
//
// usage: mc_driver [n=24] [nmat=32768] [steps=5] [mode=2]
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>

#include "lufqhe.h"

#define CHECK_CUDA(x)                                                        \
  do {                                                                       \
    cudaError_t e_ = (x);                                                    \
    if (e_ != cudaSuccess) {                                                 \
      std::fprintf(stderr, "%s: %s\n", #x, cudaGetErrorString(e_));          \
      return 1;                                                              \
    }                                                                        \
  } while (0)
#define CHECK_LU(x)                                                          \
  do {                                                                       \
    int r_ = (x);                                                            \
    if (r_ != LUFQHE_SUCCESS) {                                              \
      std::fprintf(stderr, "%s -> %d: %s\n", #x, r_, lufqhe_last_error());   \
      return 1;                                                              \
    }                                                                        \
  } while (0)

int main(int argc, char **argv) {
  const int n = argc > 1 ? std::atoi(argv[1]) : 24;
  const long long nmat = argc > 2 ? std::atoll(argv[2]) : 32768;
  const int steps = argc > 3 ? std::atoi(argv[3]) : 5;
  const int mode = argc > 4 ? std::atoi(argv[4]) : LUFQHE_MODE_MIXED;
  cudaStream_t stream;
  CHECK_CUDA(cudaStreamCreate(&stream));
  double *A = nullptr, *logabs = nullptr, *phase = nullptr, *sum = nullptr;
  int32_t *status = nullptr;
  int8_t *parity = nullptr;
  CHECK_CUDA(cudaMalloc(&A, sizeof(double) * 2 * n * n * nmat));
  CHECK_CUDA(cudaMalloc(&logabs, sizeof(double) * nmat));
  CHECK_CUDA(cudaMalloc(&phase, sizeof(double) * nmat));
  CHECK_CUDA(cudaMalloc(&status, sizeof(int32_t) * nmat));
  CHECK_CUDA(cudaMalloc(&parity, nmat));
  CHECK_CUDA(cudaMalloc(&sum, sizeof(double) * 2));
  cudaEvent_t e0, e1;
  CHECK_CUDA(cudaEventCreate(&e0));
  CHECK_CUDA(cudaEventCreate(&e1));
  for (int step = 0; step < steps; ++step) {
    CHECK_LU(lufqhe_gen_lll(A, nullptr, n, n, nmat, 1000 + step, 0.0 + __builtin_sqrt((double)n),
                            stream));
    CHECK_CUDA(cudaEventRecord(e0, stream));
    CHECK_LU(lufqhe_batch_lup_det(A, n, n, nmat, LUFQHE_C128, mode, logabs, phase, parity, status,
                                  stream));
    CHECK_LU(lufqhe_pair_sum(logabs, phase, nmat, sum, stream));
    CHECK_CUDA(cudaEventRecord(e1, stream));
    double h[2];
    CHECK_CUDA(cudaMemcpyAsync(h, sum, sizeof(h), cudaMemcpyDeviceToHost, stream));
    CHECK_CUDA(cudaStreamSynchronize(stream));
    float ms = 0.0f;
    CHECK_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    std::printf("RESULT step %d  log|psi| %.12f  arg psi %.12f  %.3f ms  %.3e dets/s\n", step, h[0],
                h[1], ms, nmat / (ms * 1e-3));
  }
  cudaFree(A);
  cudaFree(logabs);
  cudaFree(phase);
  cudaFree(status);
  cudaFree(parity);
  cudaFree(sum);
  cudaStreamDestroy(stream);
  return 0;
}
