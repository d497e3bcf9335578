/*
 * lufqhe: batched LUP determinants of small complex matrices on GB300 (sm_103a).
 *
 * C-ABI drop-in for the GPU batch-LUP call of lion-codes' LU-fqhe application.
 * Every entry point takes plain pointers and sizes; no C++ or framework types
 * cross the boundary. Device pointers are CUDA device addresses; `stream` is a
 * cudaStream_t passed as an opaque pointer (NULL = legacy default stream).
 * Calls are asynchronous on `stream` unless stated, re-entrant, and safe to
 * issue concurrently on different streams: all geometry travels as kernel
 * arguments (the reference keeps it in __constant__ memory set by
 * cudaMemcpyToSymbol, LU-fqhe/src/LUCoreGPU.cu:33,53-76, which races when two
 * host threads share a device with different n).
 *
 * Matrix layout (the reference's, LU-fqhe/src/LUCoreCPU.cu:85 and
 * LU-fqhe/inc/LUCoreGPU.h:24-40): matrix b starts at element b*n*lda, row i at
 * element i*lda, entries are interleaved (re, im) complex128 ("double2") or
 * complex64 ("float2"). lda is the reference's loadSize (= n, or p2Above(n)
 * with __PADDED__, LU-fqhe/src/RunInfo.cpp:72-76).
 *
 * Outputs per matrix (all optional except logabs):
 *   logabs  log|det A|                      (float64)
 *   phase   arg det A in (-pi, pi], permutation sign included  (float64)
 *   parity  number of row swaps mod 2       (int8)
 *   status  LUFQHE_ST_* flags, 0 = ok       (int32)
 * Errors are returned, never exit(): the reference exits on a too-large grid
 * (LU-fqhe/src/LUCoreGPU.cu:102-105) and on a near-zero row
 * (LU-fqhe/src/LUCoreCPU.cu:158).
 */
#ifndef LUFQHE_H_
#define LUFQHE_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- return codes ---- */
#define LUFQHE_SUCCESS 0
#define LUFQHE_ERR_INVALID_ARG (-1)
#define LUFQHE_ERR_UNSUPPORTED_N (-2)
#define LUFQHE_ERR_CUDA (-3)
#define LUFQHE_ERR_UNSUPPORTED_MODE (-4)
#define LUFQHE_ERR_BUSY (-5)
#define LUFQHE_ERR_TIMEOUT (-6)
#define LUFQHE_ERR_NO_MEMORY (-7)

/* ---- per-matrix status flags ---- */
#define LUFQHE_ST_SCALE_TINY 1 /* a row's max |Re| < 1e-24: the reference exits here (LUCoreCPU.cu:158) */
#define LUFQHE_ST_SINGULAR 2   /* exact zero pivot: logabs = -inf, phase = 0 */
#define LUFQHE_ST_NONFINITE 4  /* NaN/Inf in the input: logabs = phase = NaN */
#define LUFQHE_ST_FALLBACK 8   /* mixed mode: refactorised in FP64 (result is the FP64 one) */
#define LUFQHE_ST_FP64 16      /* mixed mode: routed straight to the FP64 routine so the FP64
                                  pipe works beside the FP32 pipes (result is the FP64 one) */
#define LUFQHE_ST_WAIT_TIMEOUT 32 /* a bounded wait inside the kernel (for the copy engine's
                                     staging of the matrix) ran out: logabs = phase = NaN */

/* ---- element types ---- */
#define LUFQHE_C128 0
#define LUFQHE_C64 1

/* ---- methods ---- */
/* FP64 LUP with the reference's pivot rule (implicit row scaling, pivot on
 * |Re|/scale, ties to the last row) and the reference's arithmetic: every
 * product and sum rounded separately, one division per multiplier. The
 * L\U factors are bit-identical to the reference's CPU Crout restated in FP64. */
#define LUFQHE_MODE_PLAIN_FP64 0
/* Same pivot rule with fused multiply-adds and one reciprocal per column. */
#define LUFQHE_MODE_PLAIN_FP64_FUSED 1
/* FP32 complex LUP after power-of-two equilibration, FP64-accurate residual
 * R = PA - LU (float-float on FP32 pipes), log det(I + U^-1 L^-1 R) correction,
 * FP64 log|det|/phase accumulation, and a full FP64 refactorisation for any
 * matrix whose correction norm exceeds the threshold (status FALLBACK; sizes
 * above 32 go to FP64 directly, status FP64). For 17 <= n <= 40 the FP64
 * results get an extended-precision correction of their own (an exact
 * residual of the FP64 factors, log det(I + E)). */
#define LUFQHE_MODE_MIXED 2

/* Largest n the batched entry points accept. */
#define LUFQHE_MAX_N 64

/*
 * Batched determinant. Replaces LUCoreGPU::CALL
 * (LU-fqhe/inc/LUCoreGPU.h:47, LU-fqhe/src/LUCoreGPU.cu:38-106): device batch
 * pointer, n and batch count in; per-matrix determinant out. The input is not
 * modified. Asynchronous on `stream`; no host synchronisation.
 * dtype LUFQHE_C64 takes the reference's own float2 buffers (8-byte aligned)
 * as they are: each entry is widened to FP64 as it is loaded (exact), so the
 * results equal those of the batch's complex128 copy bit for bit, in every mode.
 */
int lufqhe_batch_lup_det(const void *d_A, int n, int lda, long long batch, int dtype, int mode,
                         double *d_logabs, double *d_phase, int8_t *d_parity, int32_t *d_status,
                         void *stream);

/*
 * Determinants of lowest-Landau-level orbital matrices built on the device
 * from particle coordinates: matrix b is M_ik = z_i^k exp(-|z_i|^2/4) with
 * z = d_z[b*n .. b*n+n) (complex128). The matrices are built in shared memory
 * by the factorising kernels themselves, so a call reads 16n bytes per matrix
 * instead of 16n^2. This is the reference's intended on-device matrix-element
 * builder (LU-fqhe/src/mkMatrixElements.cu:169-358, compiled out there) fused
 * into the LUP prologue; the results are bit-identical to lufqhe_gen_lll's
 * matrices passed to lufqhe_batch_lup_det. Modes and outputs as there.
 * d_z and the outputs may also be page-locked host memory, which the kernels
 * then read and write over the host link (16n bytes in, 21 out per matrix).
 */
int lufqhe_lll_det(const void *d_z, int n, long long batch, int mode, double *d_logabs,
                   double *d_phase, int8_t *d_parity, int32_t *d_status, void *stream);

/*
 * Determinants of composite-fermion (CF) matrices built inside the
 * factorising kernels: one configuration of np particles (host arrays phi,
 * theta of np angles) and a batch of permutations (d_perm: batch rows of
 * perm_stride int16, the first n of each a 1-based particle list). Row r of
 * matrix b belongs to particle p = perm[r] - 1, with
 *   u_p = (cos theta cos phi, cos theta sin phi), v_p = (sin theta cos phi, -sin theta sin phi),
 *   Q = (n - 3) / 2 (n odd), a table T[p][Q+1] = (cos theta sin theta)^Q,
 *   T[p][Q+1+j] = T[p][Q+j] u_p / v_p, T[p][Q+1-j] = T[p][Q+2-j] v_p / u_p;
 *   columns c < n - 2: T[p][c];
 *   column n - 2: T[p][Q+1+mu] sum_{s != r} (k1 u_p v_q + k2 u_q v_p) / (u_p v_q - u_q v_p);
 *   column n - 1: T[p][Q+1+nu] sum_{s != r} (r1 u_p v_q + r2 u_q v_p) / (u_p v_q - u_q v_p),
 *   q = perm[s] - 1.
 * This is the reference's compiled-out matrix-element builder
 * (mkMatrixElements, LU-fqhe/src/mkMatrixElements.cu:46-50, 169-358, same
 * argument order) followed by LUCoreGPU::CALL, in FP64 and with each of the
 * last two columns taking its own term (the reference's column masks are
 * commented out, :251 and :285, which makes the two columns equal). Needs
 * n odd in [3, 64], np in [n, 32767], perm_stride >= n and Q+1+mu, Q+1+nu in
 * [0, n). A permutation entry outside 1..np, or a repeated particle, gives
 * status LUFQHE_ST_NONFINITE for that matrix. Modes and outputs as
 * lufqhe_batch_lup_det; d_perm and the outputs may be page-locked host memory.
 * The tables are uploaded from pageable memory, which orders the call after
 * the stream's earlier work; the call cannot be captured into a graph.
 */
int lufqhe_cf_det(const double *phi, const double *theta, int np, int n, double k1, double k2,
                  double r1, double r2, int mu, int nu, const int16_t *d_perm, int perm_stride,
                  long long batch, int mode, double *d_logabs, double *d_phase, int8_t *d_parity,
                  int32_t *d_status, void *stream);

/*
 * Same call on HOST buffers: the batch and the four result arrays are in host
 * memory. Replaces the copy-in / LUCoreGPU::CALL / copy-out sequence of the
 * reference's Monte Carlo loop (LU-fqhe/src/MonteCarloLoop.cu:316-329).
 * In mixed mode with a page-locked batch (cudaHostAlloc / cudaHostRegister)
 * the kernels read the matrices over the host link themselves, with no copy,
 * and write page-locked result arrays directly (pageable result arrays are
 * filled by copies from device memory). Otherwise the batch is cut into
 * chunks that three internal streams carry through host-to-device copy, the
 * batched kernels and device-to-host copy, so copies of one chunk overlap the
 * factorisation of another; pageable memory works but serialises the copies.
 * Device memory comes from the stream-ordered allocator and is released on
 * `stream`. Results are bit-identical to lufqhe_batch_lup_det's either way.
 * dtype LUFQHE_C64 takes complex64 host matrices (half the bytes to move).
 * Asynchronous on `stream`: the results are in host memory once `stream` has
 * completed, and the batch must stay unchanged until then.
 * d_parity / d_status may be NULL as in lufqhe_batch_lup_det.
 */
int lufqhe_batch_lup_det_host(const void *h_A, int n, int lda, long long batch, int dtype,
                              int mode, double *h_logabs, double *h_phase, int8_t *h_parity,
                              int32_t *h_status, void *stream);

/*
 * In-place variant: overwrites each matrix with its L\U factors (unit-lower L
 * below the diagonal, U on and above it, rows in pivoted order) exactly as the
 * reference kernel leaves global memory (LU-fqhe/src/LUCoreGPU.cu:318-377).
 * Plain modes only; complex128 only.
 */
int lufqhe_batch_lup_factor_inplace(void *d_A, int n, int lda, long long batch, int mode,
                                    double *d_logabs, double *d_phase, int8_t *d_parity,
                                    int32_t *d_status, void *stream);

/*
 * Reference-shaped call: LUCoreGPU::CALL with WRITE_DET (and PERFORM_PROD when
 * pair_product != 0), LU-fqhe/src/LUCoreGPU.cu:384-435. For every matrix the
 * complex determinant is written into its element (0,0); with pair_product,
 * element (0,0) of matrix 2i receives det(A_2i)*det(A_2i+1). The rest of each
 * matrix is left as L\U factors. complex128, plain FP64 reference arithmetic.
 * A determinant outside the FP64 range becomes +-inf / 0 as the reference's
 * direct product would.
 */
int lufqhe_lucoregpu_call(void *d_matrices, int n_mat, int mat_side, int load_size,
                          int pair_product, void *stream);

/*
 * The same reference-shaped call on the reference's own element type: float2
 * matrices, exactly what LUCoreGPU::CALL(float2 **d_Matrices, ...) receives
 * (LU-fqhe/inc/LUCoreGPU.h:47) and what its Monte Carlo loop copies to the
 * device (LU-fqhe/src/MonteCarloLoop.cu:316-325), so that caller links
 * unchanged. The factorisation runs in FP64 on the widened entries (plain FP64
 * reference arithmetic); element (0,0) of every matrix receives its complex64
 * determinant (or, with pair_product, matrix 2i the pair's product), rounded
 * to nearest, +-inf / 0 outside the float range as the reference's float
 * product would be; the rest of each matrix is left as L\U factors rounded to
 * float.
 */
int lufqhe_lucoregpu_call_c64(void *d_matrices, int n_mat, int mat_side, int load_size,
                              int pair_product, void *stream);

/*
 * Same call as lufqhe_lucoregpu_call, for callers that cannot allocate device
 * memory once they run: a Monte Carlo driver that fixes its whole device
 * budget at start-up, a server that admits work against a fixed HBM figure,
 * or a host whose buffers all belong to a memory pool it owns. The per-matrix
 * temporaries (log|det|, phase, status: 20 bytes per matrix) live in one
 * fixed 5 MiB file-scope device array, held by every device that loads the
 * library until the process exits, instead of stream-ordered allocations.
 * n_mat above LUFQHE_NOALLOC_MAX_MATRICES is rejected with
 * LUFQHE_ERR_INVALID_ARG. All calls on a device share that array and it keeps
 * the last call's contents: calls whose kernels overlap on the GPU race, so
 * order them (one stream). The array's device address is looked up once per
 * device, on the first call made with that device current; make that first
 * call before any stream capture, and do not use the library across a
 * cudaDeviceReset (the looked-up address would be stale).
 */
#define LUFQHE_NOALLOC_MAX_MATRICES 262144
int lufqhe_lucoregpu_call_noalloc(void *d_matrices, int n_mat, int mat_side, int load_size,
                                  int pair_product, void *stream);

/*
 * Wavefunction sum over determinant pairs, S = sum_i det(A_2i) det(A_2i+1)
 * for i < batch/2 (an odd last matrix is dropped, LU-fqhe/src/LUCoreCPU.cu:83),
 * from log-polar determinants. Replaces the pair product in the LU kernel
 * (LU-fqhe/src/LUCoreGPU.cu:403-425) plus LUCoreGPU::globalReduction
 * (LU-fqhe/src/LUCoreGPU.cu:113-156). d_out receives log|S| and arg S (two
 * doubles, device memory). One launch; reproducible order.
 */
int lufqhe_pair_sum(const double *d_logabs, const double *d_phase, long long batch, double *d_out,
                    void *stream);

/*
 * The same wavefunction sum straight from the matrices, the pair product and
 * the sum fused into the factorisation: replaces LUCoreGPU::CALL with
 * PERFORM_PROD (LU-fqhe/src/LUCoreGPU.cu:403-425) followed by
 * LUCoreGPU::globalReduction (LU-fqhe/src/LUCoreGPU.cu:113-156, :444-557).
 * In the plain modes at n <= 32 one kernel does it all: each warp factorises
 * both matrices of a pair and adds their product to a running complex
 * log-sum-exp; no per-matrix result is written. In mixed mode, and for
 * n > 32, the batched call writes log-polar determinants to pool temporaries
 * and one log-sum-exp pass reduces them. d_out (device, 2 doubles) receives
 * log|S| and arg S (-inf and 0 for S = 0, NaN if any matrix is not finite).
 * Layout, dtype and modes as lufqhe_batch_lup_det; an odd last matrix is
 * dropped (LU-fqhe/src/LUCoreCPU.cu:83). Reproducible for a given device.
 */
int lufqhe_batch_pair_sum(const void *d_A, int n, int lda, long long batch, int dtype, int mode,
                          double *d_out, void *stream);

/* ---- several devices: the host side (plain C, no device call) ---- */
/*
 * Complex log-sum-exp of k partial sums given as (log|S_r|, arg S_r) pairs in
 * parts[2r], parts[2r+1]: out = (log|sum_r S_r|, arg sum_r S_r). The
 * reduction of per-device (or per-rank) wavefunction sums, which the
 * reference does with MPI_Reduce on direct complex values
 * (LU-fqhe/src/MonteCarloLoop.cu:373-392). -inf parts add nothing; a NaN part
 * gives NaN.
 */
int lufqhe_combine_log_sums(const double *parts, long long k, double *out);

/*
 * Split a batch made of `ngroups` groups of same-size matrices (group g: count[g]
 * matrices of side n[g], in this order) into `nshards` contiguous shards of
 * nearly equal factorisation cost (the flops of one n x n LUP per matrix),
 * for one device each. Shard s takes matrices [begin[s*ngroups+g],
 * end[s*ngroups+g]) of group g. With pair_aligned, every boundary inside a
 * group falls on an even index, so no determinant pair of the wavefunction sum
 * is split. The reference splits by matrix count (LU-fqhe/src/RunInfo.cpp:53,
 * LU-fqhe/src/MonteCarloLoop.cu:141-148).
 */
int lufqhe_shard_by_cost(const int *n, const long long *count, int ngroups, int nshards,
                         int pair_aligned, long long *begin, long long *end);

/* ---- mixed-size batches: one persistent launch, autotuned, graph-captured ---- */
/* One group of same-size matrices of a mixed-size batch. Its results go to
 * indices out_offset .. out_offset + count - 1 of the output arrays. */
typedef struct {
  const void *A;        /* device or page-locked host pointer, complex128, layout as above */
  int n;
  int lda;
  long long count;
  long long out_offset;
} lufqhe_group_t;

typedef struct lufqhe_plan_s lufqhe_plan_t;

/* Tune tile sizes per n and warps per CTA by timing candidate launches. */
#define LUFQHE_PLAN_AUTOTUNE 1

/*
 * Build a plan for fixed groups and output buffers (length = max out_offset +
 * count). Inputs and outputs are device memory or page-locked host memory;
 * the kernels read and write page-locked host memory over the host link, so a
 * plan on host buffers needs no copies. The work list (tiles of same-n matrices, largest n
 * first) and a CUDA graph of the persistent launch are made once; the input
 * matrices may change between executions, their addresses may not. The
 * reference factorises one size per CALL (LU-fqhe/src/LUCoreGPU.cu:38-106);
 * this has no counterpart there. Synchronises `stream` while building.
 */
int lufqhe_plan_create(lufqhe_plan_t **plan, const lufqhe_group_t *groups, int ngroups, int mode,
                       double *d_logabs, double *d_phase, int8_t *d_parity, int32_t *d_status,
                       int flags, void *stream);
/* Replay the captured graph on `stream` (asynchronous). A plan's work
 * counters and lists (a mixed plan's pending FP64 refactorisations and factor
 * lists) are its own device memory, reset by each execution: executions of
 * one plan must not overlap on the GPU (order them on one stream); different
 * plans may run side by side. */
int lufqhe_plan_execute(lufqhe_plan_t *plan, void *stream);
/* The same work as lufqhe_plan_execute, launched directly instead of via the graph. */
int lufqhe_plan_launch_direct(lufqhe_plan_t *plan, void *stream);
/* JSON text of the chosen tiles and launch shape (and tuning timings). */
int lufqhe_plan_describe(const lufqhe_plan_t *plan, char *buf, size_t len);
int lufqhe_plan_destroy(lufqhe_plan_t *plan);

/* ---- serving: device-resident walkers and a persistent request loop ---- */
/*
 * A walker is k matrices of one size n, resident in HBM for its lifetime; each
 * move resamples particle `particle` (new z per matrix), the GPU rebuilds that
 * row of every matrix (M_ik = z^k exp(-|z|^2/4)) and recomputes the k
 * determinants. One persistent kernel per size class polls a tile ring in
 * mapped host memory (bounded waits; it exits after 0.2 s idle and is
 * relaunched on demand), so requests from many walkers share the GPU and
 * overlap without a batch boundary. Walkers are admitted against the HBM
 * budget. No counterpart in the reference, whose Monte Carlo loop re-sends
 * and refactorises every matrix each step (LU-fqhe/src/MonteCarloLoop.cu:216-335).
 */
typedef struct lufqhe_server_s lufqhe_server_t;
/* class_n: sizes served (8, 16, 32, 64); class_sms: SMs given to each (NULL =
 * equal shares); max_k: most matrices per walker; tile: matrices per work tile
 * for the classes n <= 16 (a larger class takes max(1, tile * 16^3 / n^3), the
 * same factorisation work per tile, so a request's matrices spread over more
 * warps).
 * mode: LUFQHE_MODE_MIXED or LUFQHE_MODE_PLAIN_FP64_FUSED. */
int lufqhe_server_create(lufqhe_server_t **server, size_t hbm_budget_bytes, int mode,
                         const int *class_n, const int *class_sms, int nclasses, int max_k,
                         int tile);
/* z_host: k*n complex128 particle coordinates. LUFQHE_ERR_BUSY when the HBM
 * budget is exhausted. Uploads the coordinates (synchronously); the matrices
 * are built on the device by the walker's first request. */
int lufqhe_server_walker_create(lufqhe_server_t *server, int n, int k, const double *z_host,
                                int *walker_id);
int lufqhe_server_walker_destroy(lufqhe_server_t *server, int walker_id);
/* One move: znew_host holds the k new coordinates of `particle` (particle < 0
 * recomputes the determinants without a move). LUFQHE_ERR_BUSY when the walker
 * already has a move in flight or the request ring is full. */
int lufqhe_server_submit(lufqhe_server_t *server, int walker_id, int particle,
                         const double *znew_host, long long *ticket);
/* 0 = done (k results copied to the host arrays if given), LUFQHE_ERR_BUSY =
 * not yet (wait_us = 0), LUFQHE_ERR_TIMEOUT = not within wait_us. */
int lufqhe_server_poll(lufqhe_server_t *server, long long ticket, int wait_us, double *logabs,
                       double *phase, int32_t *status);
int lufqhe_server_destroy(lufqhe_server_t *server);
/* Simulated walker stream: Poisson move arrivals at rate_hz, k log-uniform in
 * [k_min, k_max], n uniform over the classes, `moves` moves per walker.
 * Walker shapes (n, k) come in the same sequence in every run. Writes
 * per-request latency (us, arrival to completion), n and k (rec_n, rec_k may
 * be NULL); returns the number of records, *elapsed_s the wall time,
 * *matrices the determinants. */
long long lufqhe_server_run_stream(lufqhe_server_t *server, double rate_hz, long long nrequests,
                                   int moves, int k_min, int k_max, unsigned long long seed,
                                   double *lat_us, int *rec_n, int *rec_k, long long max_records,
                                   double *elapsed_s, long long *matrices);
/* Closed loop: `walkers` live walkers (k log-uniform in [k_min, k_max], n
 * uniform over the classes) each submit their next move when the previous one
 * completes; a walker retires after `moves` moves and a new one (whose first
 * request builds its matrices) takes its place. The first builds are made
 * before the clock starts. Returns the requests completed; *elapsed_s the
 * wall time, *matrices the determinants: the server's capacity for the open
 * stream's work mix. */
long long lufqhe_server_run_closed(lufqhe_server_t *server, int walkers, long long nrequests,
                                   int moves, int k_min, int k_max, unsigned long long seed,
                                   double *elapsed_s, long long *matrices);
/* Since the server was created, for its class of size class_n (0: all
 * classes): matrix moves taken by the O(n^2) path, and matrix moves that
 * refactorised instead (a failed check, or a full history). Synchronous. */
int lufqhe_server_stats(lufqhe_server_t *server, int class_n, long long *moved,
                        long long *refactored);

/* ---- on-device synthetic inputs (seeded; identical on every device) ---- */
/* i.i.d. complex Gaussian entries, Re and Im ~ N(0, sigma^2/2). */
int lufqhe_gen_gaussian(double *d_A, int n, int lda, long long batch, unsigned long long seed,
                        double sigma, void *stream);
/* Lowest-Landau-level orbital matrices M_ij = z_i^j exp(-|z_i|^2/4),
 * z_i complex Gaussian with E|z|^2 = sigma^2 (d_z receives the z_i, may be NULL). */
int lufqhe_gen_lll(double *d_A, double *d_z, int n, int lda, long long batch,
                   unsigned long long seed, double sigma, void *stream);
/* The CF matrices of lufqhe_cf_det written out (the reference's makeMatrices
 * kernel, LU-fqhe/src/mkMatrixElements.cu:295-358): matrix b at
 * d_A + b*n*lda, row stride lda, dtype LUFQHE_C128 or LUFQHE_C64 (rounded
 * from the FP64 entries). lufqhe_cf_det's results equal lufqhe_batch_lup_det's
 * on the complex128 matrices bit for bit. */
int lufqhe_gen_cf(const double *phi, const double *theta, int np, int n, double k1, double k2,
                  double r1, double r2, int mu, int nu, const int16_t *d_perm, int perm_stride,
                  long long batch, void *d_A, int lda, int dtype, void *stream);
/* Host: the per-configuration tables those calls upload: uv = u[0..np) then
 * v[0..np) (2 np complex128), tab = T (np x n complex128). */
int lufqhe_cf_tables(const double *phi, const double *theta, int np, int n, double *uv,
                     double *tab);

/* Same generators on the host (bit-identical draws; libm's exp/sin/cos/log may
 * differ from the device's in the last place). */
int lufqhe_gen_gaussian_host(double *A, int n, int lda, long long batch, unsigned long long seed,
                             double sigma);
int lufqhe_gen_lll_host(double *A, double *z, int n, int lda, long long batch,
                        unsigned long long seed, double sigma);

/* ---- reference input files ---- */
/* Reads matrices [first, first + count) of a raw file of n x n complex64
 * matrices (interleaved float32, row-major, back to back: the format
 * PermHandler reads, LU-fqhe/src/PermHandler.cpp:91-170) into host memory as
 * complex128 with row stride lda. Returns the number of whole matrices read
 * (fewer at the end of the file) or a negative error. n <= 512. */
long long lufqhe_read_matrices_f32(const char *path, int n, long long first, long long count,
                                   int lda, double *out);

/* ---- options (process-wide, read when a call is issued) ---- */
/* ||E||_F above which the mixed mode refactorises a matrix in FP64 (default
 * 0.1; 0 sends every matrix to the FP64 path, +inf disables the fallback
 * except for zero or non-finite FP32 pivots). */
#define LUFQHE_OPT_MIXED_THRESHOLD 1
/* Warps per CTA of the register-tiled mixed kernels (n in {6,8,12,16,24,32});
 * 0 = library default. */
#define LUFQHE_OPT_TILE_WARPS 2
/* Fraction (0..1) of the matrices the batched mixed mode sends straight to the
 * FP64 routine, chosen by a hash of each matrix's first entry (so a matrix
 * takes the same path wherever it sits); the FP64 pipe then works beside the
 * FP32 pipes. A negative value restores the per-n default. */
#define LUFQHE_OPT_FP64_SHARE 3
/* Input bytes per chunk of lufqhe_batch_lup_det_host, in MiB (1..1024; default
 * 32). */
#define LUFQHE_OPT_HOST_CHUNK_MB 4
/* Mixed mode, n = 24 and 32: 1 (default) refines the back substitution of the
 * matrices whose correction the FP32 solves cannot carry to 1e-10 but whose
 * ||E||_F is within the threshold, in a pass of its own, before sending the
 * rest to FP64; 0 sends them all to FP64. */
#define LUFQHE_OPT_MIXED_REFINE 5
/* 1: the batched entry points record a CUDA event pair around every kernel
 * they launch, on the launching stream, for lufqhe_kernel_times (not while
 * the stream is being captured); 0 (default): no events. */
#define LUFQHE_OPT_KERNEL_TIMING 6
/* 1 (default): the plain FP64 warp kernel and the n >= 24 mixed FP32 pass
 * stage each complex128 matrix from device memory into shared memory with
 * the copy engine's bulk copies (one per row, completing on an mbarrier) and
 * prefetch the next matrix into L2; 0: per-lane vector loads. Same bits. */
#define LUFQHE_OPT_BULK_LOADS 7
/* Servers created while this is 1 keep each walker matrix's FP64
 * L\U factors and take a move's determinant ratio from an O(n^2) solve
 * against them (matrix determinant lemma, Woodbury over the moves since the
 * last factorisation), checked before use (an error estimate of the ratio, see
 * LUFQHE_OPT_MOVE_TOL); a move that fails the check, or the 9th since the last
 * factorisation, refactorises in FP64. Every factorisation of such a class is
 * then FP64 (status LUFQHE_ST_FP64 in mixed mode). 2: the classes with
 * n <= 16 only (on ill-conditioned orbital matrices the check refuses most
 * moves at n >= 32). 0 (default): every move refactorises (mixed mode's FP32
 * path where the policy allows). On GB300, whose FP64 pipe is narrow, a mixed
 * refactorisation of an n <= 16 orbital matrix costs less than an FP64 move
 * with its check: in a mixed walker stream at 70% of the offline rate the
 * n = 8 requests' median latency was 0.08 ms refactorising against 0.5 ms
 * with moves, and a closed loop of walkers ran 3.3 times as many
 * determinants per second. */
#define LUFQHE_OPT_SERVE_MOVES 8
/* Error tolerance of the O(n^2) moves, read when a server is created: a move
 * is taken only if the a-posteriori estimate of its determinant ratio's
 * relative error (the solve's first-order error, from its residual and the
 * transposed solve A^-T d, plus the typical effect of the residual's own
 * rounding) is at most this value; otherwise it refactorises. Default 1e-12
 * (the 8 moves between factorisations add about 8e-12 to log|det|);
 * 0 < value < 1. */
#define LUFQHE_OPT_MOVE_TOL 9
int lufqhe_set_option(int option, double value);
double lufqhe_get_option(int option);

/* ---- measurement ---- */
/* Measured FMA-pipe peak of the current device in TFLOP/s (2 flops per FMA):
 * kind 0 = FP64, kind 1 = FP32. Synchronises `stream`. No counterpart in the
 * reference; it supplies the roofline denominators of the benchmark. */
int lufqhe_probe_fma_peak(int kind, double *tflops, void *stream);

/* Per-kernel device times recorded while LUFQHE_OPT_KERNEL_TIMING was on:
 * waits for the recorded events, writes a JSON object
 * {"<kernel><n>": {"launches": L, "ms": total}, ...} into json (len bytes) and
 * clears the record. No counterpart in the reference; it lets a benchmark
 * time the dominant kernel of a multi-kernel call with CUDA events on the
 * launching stream. */
int lufqhe_kernel_times(char *json, size_t len);

/* ---- misc ---- */
/* Bytes of device memory a lufqhe_batch_lup_det call of this n, batch and mode
 * takes, stream-ordered, from the library's own memory pool while it runs
 * (mixed mode at n = 24 and 32: the matrices saved for the refinement of the
 * back substitution, room for a quarter of the batch; 0 otherwise). The pool
 * keeps freed blocks for the next call. */
size_t lufqhe_workspace_bytes(int n, long long batch, int mode);
/* Return the library pool's unused device memory to the driver, on every
 * device the library has used. Blocks still held by work in flight stay
 * until it completes: synchronise the streams the library ran on first to
 * give everything back. Later calls allocate again as needed. No counterpart
 * in the reference, whose calls take no workspace. */
int lufqhe_release_workspace(void);
/* Text for the last error on the calling host thread. */
const char *lufqhe_last_error(void);
/* Library version as "major.minor.patch". */
const char *lufqhe_version(void);

#ifdef __cplusplus
}
#endif

#endif /* LUFQHE_H_ */
