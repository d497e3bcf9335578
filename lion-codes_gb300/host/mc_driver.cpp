// A C++ host of the kind LU-fqhe's Monte Carlo driver is
// (LU-fqhe/src/MonteCarloLoop.cu:120-430), calling the determinants only
// through the C-ABI of liblufqhe.so (include/lufqhe.h).
//
// Each Monte Carlo step: the batch of `nmat` matrices is split over `devices`
// GPUs by factorisation cost (lufqhe_shard_by_cost, pair-aligned); on each
// device the shard's lowest-Landau-level orbital matrices are built and the
// shard's wavefunction sum over determinant pairs (LUCoreCPU::CALL,
// LU-fqhe/src/LUCoreCPU.cu:82-98) comes from one lufqhe_batch_pair_sum call
// (pair products and the sum fused into the factorisation in the plain
// modes); the per-device sums, one complex number each in log-polar form, are
// combined on the host by lufqhe_combine_log_sums. The reference does the step
// with cudaMemcpyAsync + LUCoreGPU::CALL + globalReduction per GPU thread and
// an MPI_Reduce (LU-fqhe/src/MonteCarloLoop.cu:299-392).
//
// usage: mc_driver [n=24] [nmat=32768] [steps=5] [mode=2] [devices=1]
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

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

struct Shard {
  int dev = 0;
  long long count = 0;
  cudaStream_t stream = nullptr;
  double *A = nullptr;
  double *sum = nullptr;  // device: log|S|, arg S
  cudaEvent_t e0 = nullptr, e1 = nullptr;
};

int main(int argc, char **argv) {
  const int n = argc > 1 ? std::atoi(argv[1]) : 24;
  const long long nmat = argc > 2 ? std::atoll(argv[2]) : 32768;
  const int steps = argc > 3 ? std::atoi(argv[3]) : 5;
  const int mode = argc > 4 ? std::atoi(argv[4]) : LUFQHE_MODE_MIXED;
  const int devices = argc > 5 ? std::atoi(argv[5]) : 1;
  int have = 0;
  CHECK_CUDA(cudaGetDeviceCount(&have));
  if (devices < 1 || devices > have) {
    std::fprintf(stderr, "asked for %d devices, %d present\n", devices, have);
    return 1;
  }
  // one group of nmat n x n matrices, split by cost into `devices` shards
  std::vector<long long> begin(devices), end(devices);
  const long long count = nmat;
  CHECK_LU(lufqhe_shard_by_cost(&n, &count, 1, devices, 1, begin.data(), end.data()));
  std::vector<Shard> sh(devices);
  for (int d = 0; d < devices; ++d) {
    Shard &s = sh[d];
    s.dev = d;
    s.count = end[d] - begin[d];
    CHECK_CUDA(cudaSetDevice(d));
    CHECK_CUDA(cudaStreamCreate(&s.stream));
    CHECK_CUDA(cudaMalloc(&s.A, sizeof(double) * 2 * n * n * (s.count > 0 ? s.count : 1)));
    CHECK_CUDA(cudaMalloc(&s.sum, sizeof(double) * 2));
    CHECK_CUDA(cudaEventCreate(&s.e0));
    CHECK_CUDA(cudaEventCreate(&s.e1));
  }
  for (int step = 0; step < steps; ++step) {
    std::vector<double> parts(2 * devices);
    for (Shard &s : sh) {  // issue every device's work before waiting on any
      CHECK_CUDA(cudaSetDevice(s.dev));
      CHECK_LU(lufqhe_gen_lll(s.A, nullptr, n, n, s.count, 1000 + 64 * step + s.dev,
                              std::sqrt((double)n), s.stream));
      CHECK_CUDA(cudaEventRecord(s.e0, s.stream));
      CHECK_LU(lufqhe_batch_pair_sum(s.A, n, n, s.count, LUFQHE_C128, mode, s.sum, s.stream));
      CHECK_CUDA(cudaEventRecord(s.e1, s.stream));
      CHECK_CUDA(cudaMemcpyAsync(&parts[2 * s.dev], s.sum, 2 * sizeof(double),
                                 cudaMemcpyDeviceToHost, s.stream));
    }
    float ms = 0.0f;
    for (Shard &s : sh) {
      CHECK_CUDA(cudaSetDevice(s.dev));
      CHECK_CUDA(cudaStreamSynchronize(s.stream));
      float t = 0.0f;
      CHECK_CUDA(cudaEventElapsedTime(&t, s.e0, s.e1));
      if (t > ms) ms = t;
    }
    double psi[2];
    CHECK_LU(lufqhe_combine_log_sums(parts.data(), devices, psi));
    std::printf("RESULT step %d  log|psi| %.12f  arg psi %.12f  %.3f ms  %.3e dets/s  devices %d\n",
                step, psi[0], psi[1], ms, nmat / (ms * 1e-3), devices);
  }
  for (Shard &s : sh) {
    cudaSetDevice(s.dev);
    cudaFree(s.A);
    cudaFree(s.sum);
    cudaEventDestroy(s.e0);
    cudaEventDestroy(s.e1);
    cudaStreamDestroy(s.stream);
  }
  return 0;
}
