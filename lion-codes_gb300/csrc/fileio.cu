// Reader for the reference's raw matrix files: `count` matrices of n x n
// complex64, row-major, interleaved (re, im) float32, back to back, as
// PermHandler reads them with MPI-IO (LU-fqhe/src/PermHandler.cpp:91-170; the
// shipped fixture LU-fqhe/inc/1000_16x16.bin is 1000 such 16 x 16 matrices).
// Matrices [first, first + count) are widened to complex128 with row stride
// lda (>= n) into host memory, ready for a host-to-device copy.
#include <cstdio>

#include "lufqhe_internal.cuh"

using namespace lufqhe;

extern "C" long long lufqhe_read_matrices_f32(const char *path, int n, long long first,
                                              long long count, int lda, double *out) {
  if (!path || n < 1 || first < 0 || count < 0 || lda < n || (count > 0 && !out)) {
    set_error("lufqhe_read_matrices_f32: invalid argument");
    return LUFQHE_ERR_INVALID_ARG;
  }
  FILE *f = std::fopen(path, "rb");
  if (!f) {
    set_error("lufqhe_read_matrices_f32: cannot open %s", path);
    return LUFQHE_ERR_INVALID_ARG;
  }
  const long long per = 2LL * n * n;  // floats per matrix
  if (std::fseek(f, (long)(first * per * (long long)sizeof(float)), SEEK_SET) != 0) {
    std::fclose(f);
    set_error("lufqhe_read_matrices_f32: seek failed");
    return LUFQHE_ERR_INVALID_ARG;
  }
  float row[2 * LUFQHE_MAX_N * 8];
  long long done = 0;
  for (; done < count; ++done) {
    double *dst = out + done * 2LL * n * lda;
    bool ok = true;
    for (int i = 0; i < n && ok; ++i) {
      ok = std::fread(row, sizeof(float), 2 * (size_t)n, f) == 2 * (size_t)n;
      for (int k = 0; ok && k < 2 * n; ++k) dst[2LL * i * lda + k] = (double)row[k];
    }
    if (!ok) break;  // short file: return the number of whole matrices read
  }
  std::fclose(f);
  return done;
}
