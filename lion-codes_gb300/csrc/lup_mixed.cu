// Mixed-precision batched complex LUP determinant: complex128 and
// lowest-Landau-level entry points, the precision policy and the options.
// The method and its kernels are described in mixed_kernels.cuh.

#include <cstddef>

#include "mixed_kernels.cuh"

namespace lufqhe {

int g_tile_warps = 0;
extern int g_mixed_refine;  // refinement of the back substitution (option 5)
float g_fp64_share = -1.0f;  // < 0: per-n default

// Share of matrices routed straight to FP64, per n, in 1/65536 units. The
// defaults come from sweeps on GB300 (the share at which the FP64 pipe and the
// FP32 pipes finish together); a caller may override them.
unsigned int fp64_share_64k(int n) {
  float s = g_fp64_share;
  if (s < 0.0f) {
    // n <= 32: the FP32 path (register-tiled or generic) is fastest; on
    // GB300 at n = 25..31 the generic mixed kernel beat the corrected FP64
    // route by 1.2-2.0x on Gaussian, LLL and CF matrices alike. Above 32 the
    // FP64 warp-group kernel beats the generic mixed kernel.
    s = n <= 32 ? 0.0f : 1.0f;
  }
  if (s <= 0.0f) return 0u;
  if (s >= 1.0f) return 65536u;
  return (unsigned int)(s * 65536.0f);
}

size_t mixed_smem_per_warp(int n) {
  const int lds = n + 1;
  return (size_t)n * lds * (sizeof(float2) + sizeof(float4)) + 2 * (size_t)n * sizeof(double) +
         2 * (size_t)n * sizeof(int);
}

float g_mixed_theta = 0.1f;
int g_mixed_refine = 1;

// Device memory a batched mixed call takes from the library's pool while it
// runs, its state block (CallState): the head, for n >= 24 the pending list
// (one entry per matrix) and, for n = 24 and 32, the saved matrices.
size_t mixed_workspace_bytes(int n, long long batch) {
  if (fp64_share_64k(n) >= 65536u || batch == 0) return 0;
  auto up = [](size_t v) { return (v + 255) & ~(size_t)255; };
  if (n < kDeferMinN) return kHeadBytes;  // at most the work counter
  size_t bytes = kHeadBytes + up((size_t)batch * sizeof(unsigned int));
  if (g_mixed_refine && (n == 24 || n == 32)) {
    long long cap = std::max<long long>(256, (long long)(kRefineShare * (double)batch));
    cap = std::min<long long>(cap, batch);
    bytes += up((size_t)cap * (n == 24 ? refine_entry_bytes<24>() : refine_entry_bytes<32>()));
  }
  return bytes;
}

int launch_mixed(const double2 *A, int n, int lda, long long batch, double *logabs,
                 double *phase, int8_t *parity, int32_t *status, cudaStream_t stream,
                 bool inplace) {
  return launch_mixed_src(
      DenseSource{A, lda}, n, batch, logabs, phase, parity, status, stream,
      [&] {
        return launch_plain(A, nullptr, n, lda, batch, ARITH_FUSED, logabs, phase, parity, status,
                            stream, LUFQHE_ST_FP64);
      },
      inplace);
}

// A mixed plan's correction pass: the FP64 factorisations its grouped kernel
// listed for size n, each entry with its matrix (the plan's groups have no
// common source). head is the list's header block (kHeadBytes, zeroed before
// the plan's passes); the corrections are those of the batched mixed mode, on
// a whole CTA per entry.
int launch_listed_corrections(int n, const void *head, const unsigned char *list, long long cap,
                              double *logabs, double *phase, int8_t *parity, int32_t *status,
                              cudaStream_t stream) {
  const CallHead *h = static_cast<const CallHead *>(head);
  switch (n) {
    case 24:
      return launch_fac_correct<24, DenseSource, true>(DenseSource{nullptr, 24}, h, list, cap,
                                                       logabs, phase, parity, status, stream);
    case 32:
      return launch_fac_correct<32, DenseSource, true>(DenseSource{nullptr, 32}, h, list, cap,
                                                       logabs, phase, parity, status, stream);
    default:
      set_error("listed corrections: n=%d has no correction pass", n);
      return LUFQHE_ERR_UNSUPPORTED_N;
  }
}
size_t listed_count_offset() { return offsetof(CallHead, corr_count); }
size_t head_bytes() { return kHeadBytes; }

int launch_mixed_lll(const double2 *Z, int n, long long batch, double *logabs, double *phase,
                     int8_t *parity, int32_t *status, cudaStream_t stream) {
  return launch_mixed_src(LllSource{Z}, n, batch, logabs, phase, parity, status, stream, [&] {
    return launch_plain_lll(Z, n, batch, ARITH_FUSED, logabs, phase, parity, status, stream,
                            LUFQHE_ST_FP64);
  });
}

}  // namespace lufqhe
