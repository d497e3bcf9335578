// extern "C" entry points of liblufqhe: argument checks, dispatch, errors.

#include <cstdarg>
#include <cstdio>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "lufqhe_internal.cuh"

namespace lufqhe {

namespace {
thread_local char g_err[512] = "";

struct DeviceProps {
  int dev = -1;
  int sms = 0;
  size_t smem_optin = 0;
};
thread_local DeviceProps g_props;

const DeviceProps &props() {
  int dev = 0;
  cudaGetDevice(&dev);
  if (g_props.dev != dev) {
    cudaDeviceProp p;
    if (cudaGetDeviceProperties(&p, dev) == cudaSuccess) {
      g_props.dev = dev;
      g_props.sms = p.multiProcessorCount;
      g_props.smem_optin = p.sharedMemPerBlockOptin;
    }
  }
  return g_props;
}
}  // namespace

void set_error(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

int check_cuda(cudaError_t e, const char *what) {
  if (e == cudaSuccess) return LUFQHE_SUCCESS;
  set_error("%s: %s", what, cudaGetErrorString(e));
  return LUFQHE_ERR_CUDA;
}

// ---- per-kernel timing (measurement) ----------------------------------------
int g_kernel_timing = 0;

namespace {
struct TimedLaunch {
  std::string name;
  cudaEvent_t e0, e1;
};
std::mutex g_timing_mu;
std::vector<TimedLaunch> g_timed;
}  // namespace

KernelTimer::KernelTimer(const char *name, int n, cudaStream_t stream)
    : name_(name), n_(n), stream_(stream) {
  if (!g_kernel_timing) return;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(stream, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone) {
    cudaGetLastError();
    return;
  }
  if (cudaEventCreate(&e0_) != cudaSuccess || cudaEventRecord(e0_, stream) != cudaSuccess) {
    if (e0_) cudaEventDestroy(e0_);
    e0_ = nullptr;
    cudaGetLastError();
  }
}

void KernelTimer::stop() {
  if (!e0_) return;
  cudaEvent_t e1 = nullptr;
  if (cudaEventCreate(&e1) != cudaSuccess || cudaEventRecord(e1, stream_) != cudaSuccess) {
    cudaEventDestroy(e0_);
    if (e1) cudaEventDestroy(e1);
    e0_ = nullptr;
    cudaGetLastError();
    return;
  }
  char label[96];
  snprintf(label, sizeof(label), "%s<%d>", name_, n_);
  std::lock_guard<std::mutex> lock(g_timing_mu);
  g_timed.push_back({label, e0_, e1});
  e0_ = nullptr;
}

int device_sm_count() {
  int s = props().sms;
  return s > 0 ? s : 1;
}

size_t device_smem_optin() { return props().smem_optin; }

}  // namespace lufqhe

using namespace lufqhe;

namespace {

int check_common(const void *A, int n, int lda, long long batch, const double *logabs,
                 const char *fn, size_t align = 16) {
  if ((batch > 0 && (!A || !logabs)) || n < 1 || lda < n || batch < 0) {
    set_error("%s: invalid argument (A=%p logabs=%p n=%d lda=%d batch=%lld)", fn, A,
              (const void *)logabs, n, lda, batch);
    return LUFQHE_ERR_INVALID_ARG;
  }
  if (n > LUFQHE_MAX_N) {
    set_error("%s: n=%d exceeds the supported maximum %d", fn, n, LUFQHE_MAX_N);
    return LUFQHE_ERR_UNSUPPORTED_N;
  }
  if ((reinterpret_cast<uintptr_t>(A) & (align - 1)) != 0) {  // element alignment
    set_error("%s: A must be %zu-byte aligned", fn, align);
    return LUFQHE_ERR_INVALID_ARG;
  }
  return LUFQHE_SUCCESS;
}

}  // namespace

namespace lufqhe {

// The library's own stream-ordered memory pool, per device: blocks freed on
// a stream stay in the pool for the next call instead of going back to the
// driver at the next synchronisation (the default pool's release threshold
// is 0, which made every first call after a synchronise map its memory again).
// lufqhe_release_workspace trims them.
namespace {
std::mutex g_pool_mu;
cudaMemPool_t g_pools[64] = {};
}  // namespace

int lib_malloc_async(void **p, size_t bytes, cudaStream_t s) {
  // under stream capture the allocation becomes a graph memory node (graph-
  // owned memory, its own for every instantiated graph)
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cap) != cudaSuccess) cudaGetLastError();
  if (cap == cudaStreamCaptureStatusActive)
    return check_cuda(cudaMallocAsync(p, bytes, s), "cudaMallocAsync (captured)");
  std::mutex &mu = g_pool_mu;
  cudaMemPool_t *pools = g_pools;
  int dev = 0;
  int rc = check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
  if (rc) return rc;
  if (dev < 0 || dev >= 64) {
    set_error("device %d out of range", dev);
    return LUFQHE_ERR_CUDA;
  }
  cudaMemPool_t pool;
  {
    std::lock_guard<std::mutex> lock(mu);
    if (!pools[dev]) {
      cudaMemPoolProps props{};
      props.allocType = cudaMemAllocationTypePinned;
      props.location.type = cudaMemLocationTypeDevice;
      props.location.id = dev;
      rc = check_cuda(cudaMemPoolCreate(&pools[dev], &props), "cudaMemPoolCreate");
      if (rc) {
        pools[dev] = nullptr;
        return rc;
      }
      unsigned long long keep = ~0ull;
      rc = check_cuda(cudaMemPoolSetAttribute(pools[dev], cudaMemPoolAttrReleaseThreshold, &keep),
                      "cudaMemPoolSetAttribute");
      if (rc) return rc;
    }
    pool = pools[dev];
  }
  return check_cuda(cudaMallocFromPoolAsync(p, bytes, pool, s), "cudaMallocFromPoolAsync");
}

int lib_free_async(void *p, cudaStream_t s) {
  return check_cuda(cudaFreeAsync(p, s), "cudaFreeAsync");
}

int g_bulk_loads = 1;
int g_serve_moves = 0;
double g_move_tol = 1e-12;

bool is_device_memory(const void *p) {
  if (!p) return false;
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice;
}

const void *device_address(const void *p) {
  if (!p) return p;
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();  // clear the error some drivers report for unregistered memory
    return p;
  }
  return (a.type == cudaMemoryTypeHost && a.devicePointer) ? a.devicePointer : p;
}

int batch_det_device(const void *Av, int dtype, int n, int lda, long long batch, int mode,
                     double *logabs, double *phase, int8_t *parity, int32_t *status,
                     cudaStream_t s, bool host_link) {
  if (dtype == LUFQHE_C64) {
    const float2 *A = static_cast<const float2 *>(Av);
    switch (mode) {
      case LUFQHE_MODE_PLAIN_FP64:
        return launch_plain32(A, nullptr, n, lda, batch, ARITH_REF, logabs, phase, parity, status,
                              s);
      case LUFQHE_MODE_PLAIN_FP64_FUSED:
        return launch_plain32(A, nullptr, n, lda, batch, ARITH_FUSED, logabs, phase, parity,
                              status, s);
      case LUFQHE_MODE_MIXED:
        return launch_mixed32(A, n, lda, batch, logabs, phase, parity, status, s);
      default:
        set_error("lufqhe_batch_lup_det: unknown mode %d", mode);
        return LUFQHE_ERR_UNSUPPORTED_MODE;
    }
  }
  const double2 *A = static_cast<const double2 *>(Av);
  switch (mode) {
    case LUFQHE_MODE_PLAIN_FP64:
      return launch_plain(A, nullptr, n, lda, batch, ARITH_REF, logabs, phase, parity, status, s);
    case LUFQHE_MODE_PLAIN_FP64_FUSED:
      return launch_plain(A, nullptr, n, lda, batch, ARITH_FUSED, logabs, phase, parity, status,
                          s);
    case LUFQHE_MODE_MIXED:
      return launch_mixed(A, n, lda, batch, logabs, phase, parity, status, s, host_link);
    default:
      set_error("lufqhe_batch_lup_det: unknown mode %d", mode);
      return LUFQHE_ERR_UNSUPPORTED_MODE;
  }
}

}  // namespace lufqhe

extern "C" int lufqhe_batch_lup_det(const void *d_A, int n, int lda, long long batch, int dtype,
                                    int mode, double *d_logabs, double *d_phase,
                                    int8_t *d_parity, int32_t *d_status, void *stream) {
  if (!dtype_bytes(dtype)) {
    set_error("lufqhe_batch_lup_det: unknown dtype %d", dtype);
    return LUFQHE_ERR_UNSUPPORTED_MODE;
  }
  int rc = check_common(d_A, n, lda, batch, d_logabs, "lufqhe_batch_lup_det", dtype_bytes(dtype));
  if (rc) return rc;
  return batch_det_device(d_A, dtype, n, lda, batch, mode, d_logabs, d_phase, d_parity, d_status,
                          (cudaStream_t)stream, false);
}

extern "C" int lufqhe_lll_det(const void *d_z, int n, long long batch, int mode,
                              double *d_logabs, double *d_phase, int8_t *d_parity,
                              int32_t *d_status, void *stream) {
  int rc = check_common(d_z, n, n, batch, d_logabs, "lufqhe_lll_det");
  if (rc) return rc;
  if (batch == 0) return LUFQHE_SUCCESS;
  cudaStream_t s = (cudaStream_t)stream;
  // page-locked host coordinates and results: their device views
  const double2 *Z = reinterpret_cast<const double2 *>(device_address(d_z));
  d_logabs = static_cast<double *>(const_cast<void *>(device_address(d_logabs)));
  d_phase = static_cast<double *>(const_cast<void *>(device_address(d_phase)));
  d_parity = static_cast<int8_t *>(const_cast<void *>(device_address(d_parity)));
  d_status = static_cast<int32_t *>(const_cast<void *>(device_address(d_status)));
  switch (mode) {
    case LUFQHE_MODE_PLAIN_FP64:
      return launch_plain_lll(Z, n, batch, ARITH_REF, d_logabs, d_phase, d_parity, d_status, s);
    case LUFQHE_MODE_PLAIN_FP64_FUSED:
      return launch_plain_lll(Z, n, batch, ARITH_FUSED, d_logabs, d_phase, d_parity, d_status,
                              s);
    case LUFQHE_MODE_MIXED:
      return launch_mixed_lll(Z, n, batch, d_logabs, d_phase, d_parity, d_status, s);
    default:
      set_error("lufqhe_lll_det: unknown mode %d", mode);
      return LUFQHE_ERR_UNSUPPORTED_MODE;
  }
}

extern "C" int lufqhe_batch_lup_factor_inplace(void *d_A, int n, int lda, long long batch,
                                               int mode, double *d_logabs, double *d_phase,
                                               int8_t *d_parity, int32_t *d_status,
                                               void *stream) {
  int rc = check_common(d_A, n, lda, batch, d_logabs, "lufqhe_batch_lup_factor_inplace");
  if (rc) return rc;
  if (mode != LUFQHE_MODE_PLAIN_FP64 && mode != LUFQHE_MODE_PLAIN_FP64_FUSED) {
    set_error("lufqhe_batch_lup_factor_inplace: mode %d has no in-place form", mode);
    return LUFQHE_ERR_UNSUPPORTED_MODE;
  }
  double2 *A = reinterpret_cast<double2 *>(d_A);
  return launch_plain(A, A, n, lda, batch,
                      mode == LUFQHE_MODE_PLAIN_FP64 ? ARITH_REF : ARITH_FUSED, d_logabs,
                      d_phase, d_parity, d_status, (cudaStream_t)stream);
}

extern "C" int lufqhe_lucoregpu_call(void *d_matrices, int n_mat, int mat_side, int load_size,
                                     int pair_product, void *stream) {
  if (!d_matrices || n_mat < 0 || mat_side < 1 || load_size < mat_side) {
    set_error("lufqhe_lucoregpu_call: invalid argument");
    return LUFQHE_ERR_INVALID_ARG;
  }
  if (mat_side > LUFQHE_MAX_N) {
    set_error("lufqhe_lucoregpu_call: matSide=%d exceeds %d", mat_side, LUFQHE_MAX_N);
    return LUFQHE_ERR_UNSUPPORTED_N;
  }
  if (n_mat == 0) return LUFQHE_SUCCESS;
  cudaStream_t s = (cudaStream_t)stream;
  // Per-matrix results live in stream-ordered temporaries; the reference keeps
  // them in the matrices themselves (element (0,0)), which is also the output here.
  void *tmp = nullptr;
  size_t bytes = (size_t)n_mat * (2 * sizeof(double) + sizeof(int32_t));
  int rc = lib_malloc_async(&tmp, bytes, s);
  if (rc) return rc;
  double *la = static_cast<double *>(tmp);
  double *ph = la + n_mat;
  int32_t *st = reinterpret_cast<int32_t *>(ph + n_mat);
  double2 *A = reinterpret_cast<double2 *>(d_matrices);
  rc = launch_plain(A, A, mat_side, load_size, n_mat, ARITH_REF, la, ph, nullptr, st, s);
  if (!rc) rc = launch_write_det(A, mat_side, load_size, n_mat, la, ph, st, pair_product, s);
  int rc2 = lib_free_async(tmp, s);
  return rc ? rc : rc2;
}

extern "C" int lufqhe_lucoregpu_call_c64(void *d_matrices, int n_mat, int mat_side,
                                         int load_size, int pair_product, void *stream) {
  if (!d_matrices || n_mat < 0 || mat_side < 1 || load_size < mat_side ||
      (reinterpret_cast<uintptr_t>(d_matrices) & 7) != 0) {
    set_error("lufqhe_lucoregpu_call_c64: invalid argument");
    return LUFQHE_ERR_INVALID_ARG;
  }
  if (mat_side > LUFQHE_MAX_N) {
    set_error("lufqhe_lucoregpu_call_c64: matSide=%d exceeds %d", mat_side, LUFQHE_MAX_N);
    return LUFQHE_ERR_UNSUPPORTED_N;
  }
  if (n_mat == 0) return LUFQHE_SUCCESS;
  cudaStream_t s = (cudaStream_t)stream;
  void *tmp = nullptr;
  size_t bytes = (size_t)n_mat * (2 * sizeof(double) + sizeof(int32_t));
  int rc = lib_malloc_async(&tmp, bytes, s);
  if (rc) return rc;
  double *la = static_cast<double *>(tmp);
  double *ph = la + n_mat;
  int32_t *st = reinterpret_cast<int32_t *>(ph + n_mat);
  float2 *A = reinterpret_cast<float2 *>(d_matrices);
  rc = launch_plain32(A, A, mat_side, load_size, n_mat, ARITH_REF, la, ph, nullptr, st, s);
  if (!rc) rc = launch_write_det32(A, mat_side, load_size, n_mat, la, ph, st, pair_product, s);
  int rc2 = lib_free_async(tmp, s);
  return rc ? rc : rc2;
}

namespace lufqhe {
extern float g_mixed_theta;
extern int g_kernel_timing;
extern int g_tile_warps;
extern float g_fp64_share;
extern int g_host_chunk_mb;
extern int g_mixed_refine;
}

extern "C" int lufqhe_set_option(int option, double value) {
  if (option == LUFQHE_OPT_MIXED_THRESHOLD) {
    if (!(value >= 0.0)) {
      set_error("lufqhe_set_option: threshold must be >= 0");
      return LUFQHE_ERR_INVALID_ARG;
    }
    g_mixed_theta = (float)value;
    return LUFQHE_SUCCESS;
  }
  if (option == LUFQHE_OPT_TILE_WARPS) {
    if (!(value >= 0.0 && value <= 8.0)) {
      set_error("lufqhe_set_option: tile warps must be 0..8");
      return LUFQHE_ERR_INVALID_ARG;
    }
    g_tile_warps = (int)value;
    return LUFQHE_SUCCESS;
  }
  if (option == LUFQHE_OPT_FP64_SHARE) {
    if (!(value <= 1.0)) {
      set_error("lufqhe_set_option: FP64 share must be <= 1 (negative = default)");
      return LUFQHE_ERR_INVALID_ARG;
    }
    g_fp64_share = (float)value;
    return LUFQHE_SUCCESS;
  }
  if (option == LUFQHE_OPT_HOST_CHUNK_MB) {
    if (!(value >= 1.0 && value <= 1024.0)) {
      set_error("lufqhe_set_option: host chunk must be 1..1024 MiB");
      return LUFQHE_ERR_INVALID_ARG;
    }
    g_host_chunk_mb = (int)value;
    return LUFQHE_SUCCESS;
  }
  if (option == LUFQHE_OPT_MIXED_REFINE) {
    if (!(value == 0.0 || value == 1.0)) {
      set_error("lufqhe_set_option: refine must be 0 or 1");
      return LUFQHE_ERR_INVALID_ARG;
    }
    g_mixed_refine = (int)value;
    return LUFQHE_SUCCESS;
  }
  if (option == LUFQHE_OPT_SERVE_MOVES) {
    if (!(value == 0.0 || value == 1.0 || value == 2.0)) {
      set_error("lufqhe_set_option: serve moves must be 0, 1 or 2");
      return LUFQHE_ERR_INVALID_ARG;
    }
    g_serve_moves = (int)value;
    return LUFQHE_SUCCESS;
  }
  if (option == LUFQHE_OPT_MOVE_TOL) {
    if (!(value > 0.0 && value < 1.0)) {
      set_error("lufqhe_set_option: move error bound must be in (0, 1)");
      return LUFQHE_ERR_INVALID_ARG;
    }
    g_move_tol = value;
    return LUFQHE_SUCCESS;
  }
  if (option == LUFQHE_OPT_BULK_LOADS) {
    if (!(value == 0.0 || value == 1.0)) {
      set_error("lufqhe_set_option: bulk loads must be 0 or 1");
      return LUFQHE_ERR_INVALID_ARG;
    }
    g_bulk_loads = (int)value;
    return LUFQHE_SUCCESS;
  }
  if (option == LUFQHE_OPT_KERNEL_TIMING) {
    if (!(value == 0.0 || value == 1.0)) {
      set_error("lufqhe_set_option: kernel timing must be 0 or 1");
      return LUFQHE_ERR_INVALID_ARG;
    }
    g_kernel_timing = (int)value;
    return LUFQHE_SUCCESS;
  }
  set_error("lufqhe_set_option: unknown option %d", option);
  return LUFQHE_ERR_INVALID_ARG;
}

extern "C" double lufqhe_get_option(int option) {
  if (option == LUFQHE_OPT_MIXED_THRESHOLD) return (double)g_mixed_theta;
  if (option == LUFQHE_OPT_TILE_WARPS) return (double)g_tile_warps;
  if (option == LUFQHE_OPT_FP64_SHARE) return (double)g_fp64_share;
  if (option == LUFQHE_OPT_HOST_CHUNK_MB) return (double)g_host_chunk_mb;
  if (option == LUFQHE_OPT_MIXED_REFINE) return (double)g_mixed_refine;
  if (option == LUFQHE_OPT_KERNEL_TIMING) return (double)g_kernel_timing;
  if (option == LUFQHE_OPT_BULK_LOADS) return (double)g_bulk_loads;
  if (option == LUFQHE_OPT_SERVE_MOVES) return (double)g_serve_moves;
  if (option == LUFQHE_OPT_MOVE_TOL) return g_move_tol;
  return NAN;
}

extern "C" int lufqhe_release_workspace(void) {
  std::lock_guard<std::mutex> lock(lufqhe::g_pool_mu);
  for (cudaMemPool_t pool : lufqhe::g_pools) {
    if (!pool) continue;
    const int rc = check_cuda(cudaMemPoolTrimTo(pool, 0), "cudaMemPoolTrimTo");
    if (rc) return rc;
  }
  return LUFQHE_SUCCESS;
}

extern "C" int lufqhe_kernel_times(char *json, size_t len) {
  if (!json || len == 0) {
    set_error("lufqhe_kernel_times: invalid argument");
    return LUFQHE_ERR_INVALID_ARG;
  }
  std::vector<TimedLaunch> recs;
  {
    std::lock_guard<std::mutex> lock(lufqhe::g_timing_mu);
    recs.swap(lufqhe::g_timed);
  }
  std::map<std::string, std::pair<long long, double>> agg;
  int rc = LUFQHE_SUCCESS;
  for (const TimedLaunch &r : recs) {
    float ms = 0.0f;
    if (!rc) rc = check_cuda(cudaEventSynchronize(r.e1), "cudaEventSynchronize(kernel timing)");
    if (!rc) rc = check_cuda(cudaEventElapsedTime(&ms, r.e0, r.e1), "cudaEventElapsedTime");
    cudaEventDestroy(r.e0);
    cudaEventDestroy(r.e1);
    if (!rc) {
      auto &a = agg[r.name];
      a.first += 1;
      a.second += ms;
    }
  }
  if (rc) return rc;
  std::string out = "{";
  for (const auto &kv : agg) {
    char item[192];
    snprintf(item, sizeof(item), "%s\"%s\": {\"launches\": %lld, \"ms\": %.6f}",
             out.size() > 1 ? ", " : "", kv.first.c_str(), kv.second.first, kv.second.second);
    out += item;
  }
  out += "}";
  if (out.size() + 1 > len) {
    set_error("lufqhe_kernel_times: buffer of %zu bytes holds less than %zu", len,
              out.size() + 1);
    return LUFQHE_ERR_INVALID_ARG;
  }
  memcpy(json, out.c_str(), out.size() + 1);
  return LUFQHE_SUCCESS;
}

extern "C" size_t lufqhe_workspace_bytes(int n, long long batch, int mode) {
  if (n < 1 || batch < 0) return 0;
  return mode == LUFQHE_MODE_MIXED ? mixed_workspace_bytes(n, batch) : 0;
}

extern "C" const char *lufqhe_last_error(void) { return g_err; }

extern "C" const char *lufqhe_version(void) { return "0.1.0"; }
