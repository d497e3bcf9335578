/*
 * Harness around the reference's own float32 CPU determinant
 * (LUCoreCPU::determinant, LU-fqhe/src/LUCoreCPU.cu:112-267), compiled unmodified
 * from the reference sources by oracle/Makefile into oracle/_ref/. TEST
 * INFRASTRUCTURE ONLY: it pins the restatement and can serve as a timed CPU
 * baseline. Nothing in the product links it.
 *
 * LUCoreCPU.cu's CALL refers to RunInfo::getMatSide/getLoadSize
 * (LU-fqhe/inc/RunInfo.h:33-34); only `determinant` is driven here, so the two
 * getters are given trivial bodies to satisfy the link.
 */
#include <cstring>
#include <vector>
#include <omp.h>
#include "LUCoreCPU.h"
#include "RunInfo.h"

int RunInfo::getMatSide() { return matSide; }
int RunInfo::getLoadSize() { return loadSize; }

// det: 2 floats per matrix. factors (optional): the matrix as determinant()
// leaves it (L\U in pivoted row order), n x n complex64 per matrix, row stride n.
extern "C" int ref_lucorecpu_factor_batch(const float *A, int n, int lda, long long batch,
                                          float *det, float *factors, int nthreads) {
  if (n < 1 || lda < n || batch < 0) return -1;
  int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel num_threads(nt)
  {
    std::vector<float2> buf((size_t)n * lda);
#pragma omp for schedule(static)
    for (long long b = 0; b < batch; ++b) {
      std::memcpy(buf.data(), A + (size_t)b * n * lda * 2, sizeof(float2) * (size_t)n * lda);
      float2 d;
      LUCoreCPU::determinant(buf.data(), &d, n, lda);
      det[2 * b] = d.x;
      det[2 * b + 1] = d.y;
      if (factors)
        for (int i = 0; i < n; ++i)
          std::memcpy(factors + ((size_t)b * n + i) * n * 2, buf.data() + (size_t)i * lda,
                      sizeof(float2) * (size_t)n);
    }
  }
  return 0;
}

extern "C" int ref_lucorecpu_det_batch(const float *A, int n, int lda, long long batch,
                                       float *det, int nthreads) {
  return ref_lucorecpu_factor_batch(A, n, lda, batch, det, nullptr, nthreads);
}
