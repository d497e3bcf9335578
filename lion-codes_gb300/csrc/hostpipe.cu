// Host-buffer form of the batched determinant.
//
// Mixed mode on a page-locked batch: no copies at all. The kernels read the
// matrices over the host link themselves (the mapped device view of the
// pinned buffer) and keep their FP64 refactorisations in the FP32 pass: the
// pass waits on the link (about 210 GB/s host-to-device on GB300, against
// about 1.3 TB/s of matrices the FP32 pass could take from HBM), so it has
// compute to spare for them, and a second kernel would re-read the rejected
// matrices after the link has gone idle. Results go straight to pinned output
// arrays, or to device memory and back by copies. There is no pipeline fill
// or drain and no chunk tail.
//
// Otherwise (pageable input, or the plain modes, whose kernels are
// compute-bound and gain nothing from the link): a chunked copy / compute /
// copy pipeline over three internal streams.
//
// The reference's Monte Carlo loop copies the batch to the device, runs the
// LU kernel and copies the result back, one step after the other on one
// stream (LU-fqhe/src/MonteCarloLoop.cu:316-329). Here chunk c goes to stream
// c % 3 with its own staging buffer: H2D copy, the batched kernels, D2H copy
// of its results. Each stream's steps stay in order; with three streams the
// H2D copies of the next two chunks queue behind each other on the copy
// engine while a chunk is factorised, and one chunk's kernels fill the tail of
// another's, so the link (about 210 GB/s host-to-device on GB300) stays busy. The
// caller's stream is forked into the two streams at entry and joined at exit;
// staging memory comes from the library's stream-ordered pool on the caller's
// stream and is freed there after the join.

#include <mutex>

#include "lufqhe_internal.cuh"

namespace lufqhe {
namespace {

constexpr int kMaxDevices = 64;

constexpr int kPipe = 3;

struct PipeStreams {
  cudaStream_t s[kPipe] = {};
};

int pipe_streams(PipeStreams *out) {
  static std::mutex mu;
  static PipeStreams per_dev[kMaxDevices];
  int dev = 0;
  int rc = check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
  if (rc) return rc;
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("device %d out of range", dev);
    return LUFQHE_ERR_CUDA;
  }
  std::lock_guard<std::mutex> lock(mu);
  for (int i = 0; i < kPipe && !rc; ++i)
    if (!per_dev[dev].s[i])
      rc = check_cuda(cudaStreamCreateWithFlags(&per_dev[dev].s[i], cudaStreamNonBlocking),
                      "pipeline stream");
  *out = per_dev[dev];
  return rc;
}

}  // namespace

int g_host_chunk_mb = 32;  // input bytes per chunk, MiB

namespace {

// Device view of page-locked host memory, or null (pageable, device or null p).
void *mapped_view(const void *p) {
  if (!p) return nullptr;
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();  // clear the error some drivers report for unregistered memory
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// Mixed mode on a pinned batch: one launch reading over the host link.
int det_over_link(const void *dA, int dtype, int n, int lda, long long batch, double *h_logabs,
                  double *h_phase, int8_t *h_parity, int32_t *h_status, cudaStream_t s) {
  double *la = static_cast<double *>(mapped_view(h_logabs));
  double *ph = static_cast<double *>(mapped_view(h_phase));
  int8_t *pa = static_cast<int8_t *>(mapped_view(h_parity));
  int32_t *st = static_cast<int32_t *>(mapped_view(h_status));
  if (la && (!h_phase || ph) && (!h_parity || pa) && (!h_status || st))
    return batch_det_device(dA, dtype, n, lda, batch, LUFQHE_MODE_MIXED, la, ph, pa, st, s, true);
  // pageable outputs: device results, then copies
  const size_t nb = (size_t)batch;
  unsigned char *buf = nullptr;
  int rc = lib_malloc_async((void **)&buf,
                            nb * (2 * sizeof(double) + sizeof(int32_t) + sizeof(int8_t)), s);
  if (rc) return rc;
  double *dla = reinterpret_cast<double *>(buf);
  double *dph = dla + nb;
  int32_t *dst = reinterpret_cast<int32_t *>(dph + nb);
  int8_t *dpa = reinterpret_cast<int8_t *>(dst + nb);
  rc = batch_det_device(dA, dtype, n, lda, batch, LUFQHE_MODE_MIXED, dla, h_phase ? dph : nullptr,
                        h_parity ? dpa : nullptr, h_status ? dst : nullptr, s, true);
  if (!rc)
    rc = check_cuda(cudaMemcpyAsync(h_logabs, dla, nb * sizeof(double), cudaMemcpyDeviceToHost, s),
                    "D2H logabs");
  if (!rc && h_phase)
    rc = check_cuda(cudaMemcpyAsync(h_phase, dph, nb * sizeof(double), cudaMemcpyDeviceToHost, s),
                    "D2H phase");
  if (!rc && h_status)
    rc = check_cuda(cudaMemcpyAsync(h_status, dst, nb * sizeof(int32_t), cudaMemcpyDeviceToHost, s),
                    "D2H status");
  if (!rc && h_parity)
    rc = check_cuda(cudaMemcpyAsync(h_parity, dpa, nb * sizeof(int8_t), cudaMemcpyDeviceToHost, s),
                    "D2H parity");
  const int r2 = lib_free_async(buf, s);
  return rc ? rc : r2;
}

}  // namespace

}  // namespace lufqhe

using namespace lufqhe;

extern "C" int lufqhe_batch_lup_det_host(const void *h_A, int n, int lda, long long batch,
                                         int dtype, int mode, double *h_logabs, double *h_phase,
                                         int8_t *h_parity, int32_t *h_status, void *stream) {
  if ((batch > 0 && (!h_A || !h_logabs)) || n < 1 || lda < n || batch < 0) {
    set_error("lufqhe_batch_lup_det_host: invalid argument");
    return LUFQHE_ERR_INVALID_ARG;
  }
  if (n > LUFQHE_MAX_N) {
    set_error("lufqhe_batch_lup_det_host: n=%d exceeds the supported maximum %d", n,
              LUFQHE_MAX_N);
    return LUFQHE_ERR_UNSUPPORTED_N;
  }
  if (!dtype_bytes(dtype)) {
    set_error("lufqhe_batch_lup_det_host: unknown dtype %d", dtype);
    return LUFQHE_ERR_UNSUPPORTED_MODE;
  }
  if (mode != LUFQHE_MODE_PLAIN_FP64 && mode != LUFQHE_MODE_PLAIN_FP64_FUSED &&
      mode != LUFQHE_MODE_MIXED) {
    set_error("lufqhe_batch_lup_det_host: unknown mode %d", mode);
    return LUFQHE_ERR_UNSUPPORTED_MODE;
  }
  if (batch == 0) return LUFQHE_SUCCESS;
  cudaStream_t user = (cudaStream_t)stream;
  if (mode == LUFQHE_MODE_MIXED)
    if (const void *dA = mapped_view(h_A))
      return det_over_link(dA, dtype, n, lda, batch, h_logabs, h_phase, h_parity, h_status, user);
  PipeStreams ps;
  int rc = pipe_streams(&ps);
  if (rc) return rc;

  const size_t mat_bytes = (size_t)n * lda * dtype_bytes(dtype);
  long long per_chunk = (long long)(((size_t)g_host_chunk_mb << 20) / mat_bytes);
  if (per_chunk < 1) per_chunk = 1;
  const long long chunks = (batch + per_chunk - 1) / per_chunk;
  const int nbuf = chunks < kPipe ? (int)chunks : kPipe;
  // per staging buffer: the chunk's matrices and its four result arrays
  const size_t in_bytes = (size_t)per_chunk * mat_bytes;
  const size_t out_bytes = (size_t)per_chunk * (2 * sizeof(double) + sizeof(int8_t) + sizeof(int32_t));
  const size_t buf_bytes = ((in_bytes + 255) & ~(size_t)255) + ((out_bytes + 255) & ~(size_t)255);
  unsigned char *stage = nullptr;
  rc = lib_malloc_async((void **)&stage, buf_bytes * nbuf, user);
  if (rc) return rc;

  cudaEvent_t fork = nullptr, done[kPipe] = {};
  rc = check_cuda(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming), "event");
  for (int i = 0; i < nbuf && !rc; ++i)
    rc = check_cuda(cudaEventCreateWithFlags(&done[i], cudaEventDisableTiming), "event");
  if (!rc) rc = check_cuda(cudaEventRecord(fork, user), "fork record");
  for (int i = 0; i < nbuf && !rc; ++i)
    rc = check_cuda(cudaStreamWaitEvent(ps.s[i], fork, 0), "fork wait");

  const unsigned char *hA = reinterpret_cast<const unsigned char *>(h_A);
  for (long long c = 0; c < chunks && !rc; ++c) {
    const int k = (int)(c % nbuf);
    cudaStream_t s = ps.s[k];
    const long long lo = c * per_chunk;
    const long long cnt = (lo + per_chunk <= batch) ? per_chunk : batch - lo;
    unsigned char *buf = stage + (size_t)k * buf_bytes;
    void *dA = buf;
    double *dla = reinterpret_cast<double *>(buf + ((in_bytes + 255) & ~(size_t)255));
    double *dph = dla + per_chunk;
    int32_t *dst = reinterpret_cast<int32_t *>(dph + per_chunk);
    int8_t *dpa = reinterpret_cast<int8_t *>(dst + per_chunk);
    rc = check_cuda(cudaMemcpyAsync(dA, hA + (size_t)lo * mat_bytes, (size_t)cnt * mat_bytes,
                                    cudaMemcpyHostToDevice, s),
                    "H2D chunk");
    if (!rc)
      rc = batch_det_device(dA, dtype, n, lda, cnt, mode, dla, h_phase ? dph : nullptr,
                            h_parity ? dpa : nullptr, h_status ? dst : nullptr, s, false);
    if (!rc)
      rc = check_cuda(cudaMemcpyAsync(h_logabs + lo, dla, (size_t)cnt * sizeof(double),
                                      cudaMemcpyDeviceToHost, s),
                      "D2H logabs");
    if (!rc && h_phase)
      rc = check_cuda(cudaMemcpyAsync(h_phase + lo, dph, (size_t)cnt * sizeof(double),
                                      cudaMemcpyDeviceToHost, s),
                      "D2H phase");
    if (!rc && h_status)
      rc = check_cuda(cudaMemcpyAsync(h_status + lo, dst, (size_t)cnt * sizeof(int32_t),
                                      cudaMemcpyDeviceToHost, s),
                      "D2H status");
    if (!rc && h_parity)
      rc = check_cuda(cudaMemcpyAsync(h_parity + lo, dpa, (size_t)cnt * sizeof(int8_t),
                                      cudaMemcpyDeviceToHost, s),
                      "D2H parity");
  }
  // join both streams back into the caller's stream, then release the staging
  for (int i = 0; i < nbuf; ++i) {
    if (!done[i]) continue;
    int r2 = check_cuda(cudaEventRecord(done[i], ps.s[i]), "join record");
    if (!r2) r2 = check_cuda(cudaStreamWaitEvent(user, done[i], 0), "join wait");
    if (!rc) rc = r2;
  }
  int r3 = lib_free_async(stage, user);
  if (!rc) rc = r3;
  if (fork) cudaEventDestroy(fork);
  for (int i = 0; i < kPipe; ++i)
    if (done[i]) cudaEventDestroy(done[i]);
  return rc;
}
