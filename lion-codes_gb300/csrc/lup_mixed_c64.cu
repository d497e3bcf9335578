// Mixed-precision batched determinant of complex64 matrices, the element type
// of the reference's own buffers (LUCoreGPU::CALL takes float2 matrices,
// LU-fqhe/inc/LUCoreGPU.h:47). The kernels are those of the complex128 path
// (mixed_kernels.cuh) on a source that widens each float entry to FP64 as it
// is loaded (exact): the split then gives hi = the float entry and lo = 0, and
// the results equal those of the batch's complex128 copy bit for bit. Its own
// translation unit, so that the complex64 instantiations compile in parallel
// with the others.

#include "mixed_kernels.cuh"

namespace lufqhe {

int launch_mixed32(const float2 *A, int n, int lda, long long batch, double *logabs,
                   double *phase, int8_t *parity, int32_t *status, cudaStream_t stream) {
  return launch_mixed_src(Dense32Source{A, lda}, n, batch, logabs, phase, parity, status, stream,
                          [&] {
                            return launch_plain32(A, nullptr, n, lda, batch, ARITH_FUSED, logabs,
                                                  phase, parity, status, stream, LUFQHE_ST_FP64);
                          });
}

}  // namespace lufqhe
