// Reference-shaped determinant call that never allocates device memory.
//
// lufqhe_lucoregpu_call keeps its per-matrix temporaries (log|det|, phase and
// status, 20 bytes per matrix) in stream-ordered allocations. Some callers may
// not allocate at all once they are running: a Monte Carlo driver that sizes
// all of its device memory when it starts and treats any later allocation as a
// broken budget, a serving process that admits work against a fixed HBM
// figure, or a host that pre-binds every buffer to a memory pool it owns. For
// them this variant keeps the temporaries in one file-scope device array of
// fixed size, so a call only launches kernels.
//
// The array (kNoAllocMaxMatrices * 20 bytes, 5 MiB) lives on every device that
// loads the library, until the process exits. All calls on a device share it
// and it keeps the last call's values; calls whose kernels overlap on the GPU
// (different streams, no ordering between them) race on it, so a caller must
// order them, e.g. by issuing them on one stream. Nothing in it needs to start
// at zero: each call writes the entries it reads first.
//
// Its device address is looked up once per device, with that device current,
// on the first call made on that device; make that first call before any
// stream capture begins. The address is kept for the life of the process, so
// the library must not be used across a cudaDeviceReset.

#include <mutex>

#include "lufqhe_internal.cuh"

namespace lufqhe {

namespace {

constexpr long long kNoAllocMaxMatrices = LUFQHE_NOALLOC_MAX_MATRICES;
constexpr size_t kNoAllocBytes = (size_t)kNoAllocMaxMatrices * (2 * sizeof(double) + sizeof(int32_t));

// log|det| [max] | phase [max] | status [max]
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
void *g_noalloc_ptr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device (cached per device).
int noalloc_scratch(void **out) {
  int dev = 0;
  int rc = check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
  if (rc) return rc;
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("lufqhe_lucoregpu_call_noalloc: device ordinal %d beyond %d", dev, kMaxDevices);
    return LUFQHE_ERR_INVALID_ARG;
  }
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void *p = nullptr;
    rc = check_cuda(cudaGetSymbolAddress(&p, g_noalloc_scratch),
                    "cudaGetSymbolAddress(no-allocation scratch)");
    if (rc) return rc;
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
  return LUFQHE_SUCCESS;
}

}  // namespace
}  // namespace lufqhe

using namespace lufqhe;

extern "C" int lufqhe_lucoregpu_call_noalloc(void *d_matrices, int n_mat, int mat_side,
                                             int load_size, int pair_product, void *stream) {
  if (!d_matrices || n_mat < 0 || mat_side < 1 || load_size < mat_side) {
    set_error("lufqhe_lucoregpu_call_noalloc: invalid argument");
    return LUFQHE_ERR_INVALID_ARG;
  }
  if (mat_side > LUFQHE_MAX_N) {
    set_error("lufqhe_lucoregpu_call_noalloc: matSide=%d exceeds %d", mat_side, LUFQHE_MAX_N);
    return LUFQHE_ERR_UNSUPPORTED_N;
  }
  if ((long long)n_mat > kNoAllocMaxMatrices) {
    set_error("lufqhe_lucoregpu_call_noalloc: nMat=%d exceeds the fixed scratch capacity of "
              "%lld matrices; split the batch or use lufqhe_lucoregpu_call",
              n_mat, kNoAllocMaxMatrices);
    return LUFQHE_ERR_INVALID_ARG;
  }
  if (n_mat == 0) return LUFQHE_SUCCESS;
  void *scratch = nullptr;
  int rc = noalloc_scratch(&scratch);
  if (rc) return rc;
  double *la = static_cast<double *>(scratch);
  double *ph = la + kNoAllocMaxMatrices;
  int32_t *st = reinterpret_cast<int32_t *>(ph + kNoAllocMaxMatrices);
  cudaStream_t s = (cudaStream_t)stream;
  double2 *A = reinterpret_cast<double2 *>(d_matrices);
  rc = launch_plain(A, A, mat_side, load_size, n_mat, ARITH_REF, la, ph, nullptr, st, s);
  if (!rc) rc = launch_write_det(A, mat_side, load_size, n_mat, la, ph, st, pair_product, s);
  return rc;
}
