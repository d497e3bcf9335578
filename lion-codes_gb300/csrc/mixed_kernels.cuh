// Kernels of the mixed-precision batched complex LUP determinant, shared by
// the complex128 (lup_mixed.cu) and complex64 (lup_mixed_c64.cu) entry points.
//
// Per matrix (one warp, shared memory), with FP64 used only where accuracy
// needs it and almost all arithmetic on the FP32 and integer pipes, which on
// GB300 run far faster than FP64:
//  1. power-of-two column-then-row equilibration A^ = D_r^-1 A D_c^-1, chosen
//     from the exponent fields (exact; log|det D| is added back in FP64);
//  2. split of every scaled FP64 entry into float hi + lo by integer
//     operations (48 significant bits kept);
//  3. FP32 complex LUP of hi with partial pivoting on |Re|+|Im|; alongside,
//     the residual R = P A^ - L U is accumulated exactly in float-float
//     (Ogita-Rump-Oishi Dot2: TwoProd + TwoSum per real product, the real
//     and imaginary parts as packed FP32 pairs), starting from hi + lo, so R
//     carries FP64-level accuracy although every operation is an FP32 one;
//  4. E = U^-1 L^-1 R by FP32 triangular solves;
//  5. log det(I + E) by an unpivoted FP32 LU that keeps the identity implicit
//     (only the small offsets are stored), log1p/atan2 of each pivot, or, for
//     the register-tiled sizes when ||E|| is small enough that the dropped
//     terms stay below 1e-12 max(1, |log|det||), by tr E - tr(E^2)/2;
//  6. log|det| = log|prod u_jj| (complex float-float product, one FP64 log
//     and atan2 per matrix, deferred and done for 32 matrices at once by the
//     32 lanes) + equilibration + Re log det(I+E); phase likewise.
// A matrix whose ||E||_F exceeds the threshold, or whose FP32 factorisation
// meets a zero or non-finite pivot, is refactorised by the FP64 warp routine
// (reference pivot rule, fused arithmetic) and flagged LUFQHE_ST_FALLBACK.
// The permutation parity reported is that of the pivoting actually used.
//
// Warps take matrices from a work counter rather than a fixed grid stride: a
// matrix refactorised in FP64 costs many times an accepted one, and a fixed
// share of the batch per warp would leave the kernel waiting on the warps
// that drew the most of them. For n >= 24 the refinements and FP64
// refactorisations run after the FP32 pass, in a second kernel on the same
// stream that has the whole GPU: the FP32 pass saves a matrix whose
// correction is within theta but beyond what FP32 solves carry (its L\U and
// Y = L^-1 R) for one refinement step of the back substitution, and appends
// the index of a rejected matrix to the call's pending list; the second
// kernel deals the list's entries out to its warps at a fixed stride for FP64
// while the other warps refine the saved matrices, so the FP64 and FP32 pipes
// work side by side. For n < 24 the FP64 refactorisations are cheap and rare enough that
// the second launch costs more than it saves; there the FP32 pass refines and
// refactorises in place, and so does the n >= 24 variant that reads its batch
// over the host link (INPLACE). The kernels take their matrices from a source:
// dense matrices in the reference layout, or lowest-Landau-level orbital
// matrices built from particle coordinates.
//
// Every call owns its state: the work counter, the pending list (room for the
// whole batch) and the saved matrices sit in one block from the library's
// stream-ordered pool whose head is zeroed on the call's stream before the
// first kernel. Nothing is shared between calls, so any number of them may be
// in flight on any streams, and a captured call replays on its own memory. A
// call whose batch fits in two strides of its grid needs no counter (warps
// take matrices at a fixed stride) and takes no block.

#pragma once

#include <algorithm>
#include <cmath>
#include <type_traits>

#include "bulk_copy.cuh"
#include "mixed_core.cuh"

namespace lufqhe {

extern int g_tile_warps;     // warps per CTA of the tile kernels (option 2)
extern int g_mixed_refine;   // refinement of the back substitution (option 5)
extern float g_mixed_theta;  // ||E||_F threshold (option 1)
unsigned int fp64_share_64k(int n);
size_t mixed_smem_per_warp(int n);

namespace {

using namespace mixed;

// Warps per CTA and CTAs per SM the register-tiled kernels are compiled for:
// the register budget this leaves (65536 / (32 warps blocks)) is what lets the
// SM hold that many warps, whichever of registers or shared memory binds.
// n = 24: 3-warp CTAs, 5 per SM (15 KB of shared memory per warp); n <= 16:
// 4-warp CTAs, 4 per SM; n = 32: shared memory allows 8 warps whatever the
// registers.
constexpr int tile_max_warps(int n) { return n == 24 ? 3 : 4; }
constexpr int tile_min_ctas(int n) { return n == 24 ? 5 : n == 32 ? 1 : 4; }

// Head of a call's state block (zeroed on the call's stream before the first
// kernel). Behind it: the pending list of the FP64 pass (one entry per matrix
// of the batch at most), then the saved matrices of the refinement.
struct CallHead {
  unsigned long long claim;           // FP32 pass: claims after each warp's first matrix
  unsigned long long refine_saved;    // saved matrices (may exceed the capacity)
  unsigned long long refine_claimed;  // claimed by the finish kernel
  unsigned int pend_count;            // entries of the pending list
  unsigned int pad;
  unsigned long long corr_count;      // host-link variant: matrices listed for the correction
};
constexpr size_t kHeadBytes = 256;

// A warp's first matrix is its own index in the grid; later ones come from the
// call's counter (after the grid's warps), or, for a call without one (a batch
// within two strides of the grid), at the grid's stride. Small batches, where
// most warps take one matrix, then make no same-address atomics at the start
// (n=8, 4096 matrices: 31.0 -> 28.9 us).
__device__ __forceinline__ long long claim_matrix(CallHead *head, int lane, long long prev) {
  const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
  if (prev < 0) return (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (!head) return prev + warps;
  unsigned long long b = 0;
  if (lane == 0) b = atomicAdd(&head->claim, 1ull);
  return (long long)__shfl_sync(kFull, b, 0) + warps;
}

// List entries: the matrix index, with this bit set for the FP64 route (status
// flag LUFQHE_ST_FP64) rather than a rejection (LUFQHE_ST_FALLBACK).
constexpr unsigned int kPendRouted = 0x80000000u;

constexpr int kDeferMinN = 24;
// Warps of the FP64 pass's CTA (one CTA per SM).
constexpr int kFallbackMaxWarps = 20;
// Warps of a CTA of the correction pass after the finish kernel.
constexpr int kFacCorrectWarps = 4;

// Hand matrix b to the FP64 pass (the list has room for every matrix).
__device__ __forceinline__ void defer_fp64(CallHead *head, unsigned int *pend, long long b,
                                           int lane, bool routed) {
  if (lane == 0) {
    const unsigned int pos = atomicAdd(&head->pend_count, 1u);
    pend[pos] = (unsigned int)b | (routed ? kPendRouted : 0u);
  }
}

// Matrices the FP32 pass leaves for a refinement of the back substitution
// (TILE_REFINE): per matrix a header and the warp's L\U and Y = L^-1 R as they
// lie in shared memory (row stride N + 1), in the call's state block (counted
// by the head's refine_saved / refine_claimed).
struct RefineHead {
  long long b;
  int exp_sum, par, prod_e, pad;
  float xh, xl, yh, yl;
};
template <int N>
constexpr size_t refine_entry_bytes() {
  return (sizeof(RefineHead) + 2 * (size_t)N * (N + 1) * sizeof(float2) + 15) & ~(size_t)15;
}
// Share of a batch the refinement buffer has room for (the rest go straight
// to the FP64 pass): on lowest-Landau-level n = 24 matrices about 9% qualify.
constexpr double kRefineShare = 0.25;

// The host-link variant refactorises rejected matrices in place (it waits on
// the link and has compute to spare) but hands their extended-precision
// correction, whose latency would hold the warp off the link for the length
// of several factorisations, to a pass of its own (the factor list with the
// matrix from the warp's device copy, FacList); the device path's finish
// kernel lists its factorisations the same way, without the copy. Share of a
// batch the list has room for (beyond it the warp corrects in place):
constexpr double kCorrShare = 0.25;
// Sources whose matrices the correction pass reads from a copy in the list:
// all but a dense device batch (rows built from coordinates would be built
// again entry by entry for the residual).
template <class Src>
constexpr int fac_copies() {
  return std::is_same<Src, DenseSource>::value ? 0 : 1;
}

// Save a TILE_REFINE matrix; false (warp-uniform) if the buffer is full.
template <int N>
__device__ bool save_refine(CallHead *head, unsigned char *buf, long long cap, long long b,
                            const float2 *F, const float2 *Rm, const CFF &prod, int exp_sum,
                            int par, int lane) {
  constexpr int NL = N * (N + 1);
  unsigned long long k = 0;
  if (lane == 0) k = atomicAdd(&head->refine_saved, 1ull);
  k = __shfl_sync(kFull, k, 0);
  if (k >= (unsigned long long)cap) return false;
  unsigned char *e = buf + k * refine_entry_bytes<N>();
  float2 *dF = reinterpret_cast<float2 *>(e + sizeof(RefineHead));
  float2 *dY = dF + NL;
  for (int q = lane; q < NL; q += 32) {
    dF[q] = F[q];
    dY[q] = Rm[q];
  }
  if (lane == 0) {
    RefineHead h;
    h.b = b;
    h.exp_sum = exp_sum;
    h.par = par;
    h.prod_e = prod.e;
    h.pad = 0;
    h.xh = prod.xh;
    h.xl = prod.xl;
    h.yh = prod.yh;
    h.yl = prod.yl;
    *reinterpret_cast<RefineHead *>(e) = h;
  }
  return true;
}

template <class Src>
__global__ void __launch_bounds__(kMaxWarpsMixed * 32)
    lup_mixed_kernel(Src src, int n, long long batch,
                     float theta2, unsigned int share64k, CallHead *head, unsigned int *pend,
                     double *__restrict__ logabs, double *__restrict__ phase,
                     int8_t *__restrict__ parity, int32_t *__restrict__ status) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int warps = blockDim.x >> 5;
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int lds = n + 1;
  const size_t nl = (size_t)n * lds;
  MixedSmem S;
  unsigned char *base = smem_raw;
  S.SC = reinterpret_cast<float4 *>(base) + warp * nl;
  base += warps * nl * sizeof(float4);
  S.Af = reinterpret_cast<float2 *>(base) + warp * nl;
  base += warps * nl * sizeof(float2);
  S.hold = reinterpret_cast<double *>(base) + warp * 2 * n;
  base += warps * 2 * (size_t)n * sizeof(double);
  S.er = reinterpret_cast<int *>(base) + warp * 2 * n;
  S.ec = S.er + n;
  const CorrScratch cs{S.Af, S.er, S.hold};

  DeferredOut out;
  for (long long b = claim_matrix(head, lane, -1); b < batch; b = claim_matrix(head, lane, b)) {
    __syncwarp();
    double2 *M = reinterpret_cast<double2 *>(S.SC);
    if (share64k && route_fp64_entry(src.first(b, n), share64k)) {
      fallback_fp64_src(src, b, n, M, lds, S.hold, lane, b, logabs, phase, parity, status,
                        LUFQHE_ST_FP64, &cs);
      continue;
    }
    if (src.load(b, n, M, lds, lane)) {
      emit_nonfinite(lane, b, logabs, phase, parity, status);
      continue;
    }
    CFF prod;
    int exp_sum, par;
    float2 corr;
    if (mixed_factor(S, n, lane, theta2, prod, exp_sum, corr, par))
      out.push(lane, b, prod, exp_sum, corr, par, logabs, phase, parity, status);
    else if (pend)
      defer_fp64(head, pend, b, lane, false);
    else
      fallback_fp64_src(src, b, n, M, lds, S.hold, lane, b, logabs, phase, parity, status,
                        LUFQHE_ST_FALLBACK, &cs);
  }
  out.flush(lane, logabs, phase, parity, status);
}


template <int N, class Src, bool INPLACE = false>
__global__ void __launch_bounds__(tile_max_warps(N) * 32, tile_min_ctas(N))
    lup_mixed_tile_kernel(Src src, long long batch, float theta2,
                          unsigned int share64k, CallHead *head, unsigned int *pend,
                          double2 *spill, unsigned char *refine, long long refine_cap,
                          unsigned char *corr_list, long long corr_cap, int bulk,
                          double *__restrict__ logabs,
                          double *__restrict__ phase, int8_t *__restrict__ parity,
                          int32_t *__restrict__ status) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // n >= 24: every FP64 factorisation goes to the FP64 pass, so this kernel
  // carries no FP64 factorisation code (a smaller instruction footprint).
  // INPLACE keeps them in this kernel: for a batch read over the host link,
  // where the FP32 pass waits on the link and has compute to spare.
  constexpr bool DEFER = !INPLACE && N >= kDeferMinN;
  // complex128 device batches: the matrix is staged by bulk copies (bulk != 0)
  constexpr bool BULK = !INPLACE && std::is_same<Src, DenseSource>::value;
  constexpr int LDS = N + 1;
  constexpr size_t NL = (size_t)N * LDS;
  const int warps = blockDim.x >> 5;
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  unsigned char *base = smem_raw;
  float4 *HL = reinterpret_cast<float4 *>(base) + warp * NL;
  base += warps * NL * sizeof(float4);
  float2 *F = reinterpret_cast<float2 *>(base) + warp * NL;
  base += warps * NL * sizeof(float2);
  double *hold = reinterpret_cast<double *>(base) + warp * 2 * N;
  base += warps * 2 * (size_t)N * sizeof(double);
  int *er = reinterpret_cast<int *>(base) + warp * 2 * N;
  int *ec = er + N;
  const CorrScratch cs{F, er, hold};
  // INPLACE: this warp's copy of its current matrix in global memory (a few
  // KB per warp, so the copies stay in L2); an FP64 refactorisation reloads
  // it from there instead of reading the matrix over the host link again
  double2 *own = INPLACE ? spill + ((size_t)blockIdx.x * warps + warp) * N * N : nullptr;
  __shared__ __align__(8) uint64_t bars[kMaxWarpsMixed];
  WarpBulk wb;
  if constexpr (BULK)
    if (bulk) wb.init(&bars[warp], lane);

  DeferredOut out;
  // the next matrix is claimed one ahead, so that its bytes can be on their
  // way to L2 while the current one is factorised
  long long b = claim_matrix(head, lane, -1);
  long long nb = b < batch ? claim_matrix(head, lane, b) : batch;
  for (; b < batch; b = nb, nb = b < batch ? claim_matrix(head, lane, b) : batch) {
    __syncwarp();
    double2 *M = reinterpret_cast<double2 *>(HL);
    if constexpr (BULK)
      if (bulk && nb < batch && lane == 0)
        prefetch_matrix_l2(src.A + (size_t)nb * N * src.lda, N, src.lda);
    if (share64k && route_fp64_entry(src.first(b, N), share64k)) {
      if constexpr (DEFER)
        defer_fp64(head, pend, b, lane, true);
      else
        fallback_fp64_src(src, b, N, M, LDS, hold, lane, b, logabs, phase, parity, status,
                          LUFQHE_ST_FP64, &cs);
      continue;
    }
    bool staged = false;
    if constexpr (BULK) {
      if (bulk && !wb.broken) {
        if (!wb.load(src.A + (size_t)b * N * src.lda, N, src.lda, M, LDS, lane)) {
          emit_wait_timeout(lane, b, logabs, phase, parity, status);
          continue;
        }
        staged = true;  // finite check: in the exponent pass
      }
    }
    if (!staged && src.load(b, N, M, LDS, lane)) {
      emit_nonfinite(lane, b, logabs, phase, parity, status);
      continue;
    }
    if constexpr (INPLACE) {
      BlockWalk w(lane, N);
      for (int e = lane; e < N * N; e += 32) {
        own[e] = M[w.i * LDS + w.k];
        w.next(N);
      }
    }
    CFF prod;
    int exp_sum, par;
    float2 corr;
    if constexpr (DEFER) {
      const int code =
          mixed_factor_tile_ex<N, true>(HL, F, er, ec, lane, theta2, prod, exp_sum, corr, par);
      if (code == TILE_ACCEPT)
        out.push(lane, b, prod, exp_sum, corr, par, logabs, phase, parity, status);
      else if (code == TILE_NONFINITE)
        emit_nonfinite(lane, b, logabs, phase, parity, status);
      // a matrix within theta but above the FP32 solves' cap gets its back
      // substitution refined in the next pass, if the buffer has room
      else if (!(code == TILE_REFINE && refine &&
                 save_refine<N>(head, refine, refine_cap, b, F,
                                reinterpret_cast<const float2 *>(HL), prod, exp_sum, par, lane)))
        defer_fp64(head, pend, b, lane, false);
    } else {
      // in place: the refinement (refine_cap != 0), then FP64 (n < 24, where
      // both are rare, and the host-link variant, which has compute to spare)
      const int code =
          mixed_factor_tile_ex<N, true>(HL, F, er, ec, lane, theta2, prod, exp_sum, corr, par);
      if (code == TILE_NONFINITE) {  // a staged matrix (the others were checked on load)
        emit_nonfinite(lane, b, logabs, phase, parity, status);
        continue;
      }
      if (code == TILE_ACCEPT ||
          (code == TILE_REFINE && refine_cap != 0 &&
           mixed_refine_tile<N>(F, reinterpret_cast<float2 *>(HL),
                                reinterpret_cast<float2 *>(HL) + N * (N + 1),
                                reinterpret_cast<float2 *>(er), lane, theta2,
                                tile_la_est(prod, exp_sum), corr)))
        out.push(lane, b, prod, exp_sum, corr, par, logabs, phase, parity, status);
      else if constexpr (INPLACE) {
        // the factors (and the warp's copy of the matrix) are listed for the
        // correction pass, so that no warp stops reading the link for one
        const FacList fl{&head->corr_count, corr_list, corr_cap, 1};
        fallback_fp64_src<DenseSource, true>(DenseSource{own, N}, 0, N, M, LDS, hold, lane, b,
                                             logabs, phase, parity, status, LUFQHE_ST_FALLBACK,
                                             &cs, corr_list != nullptr ? &fl : nullptr);
      }
      else
        fallback_fp64_src(src, b, N, M, LDS, hold, lane, b, logabs, phase, parity, status,
                          LUFQHE_ST_FALLBACK, &cs);
    }
  }
  out.flush(lane, logabs, phase, parity, status);
}

// The passes after the FP32 pass, as one kernel in the FP32 pass's
// shared-memory layout (n >= 24): the FP64 refactorisations of the matrices
// the FP32 pass rejected, dealt out at a fixed stride over the grid's warps
// first, while the warps without one refine the saved matrices (claimed one at
// a time; a refinement that fails is refactorised in FP64 on the spot). The
// FP64 pipe and the FP32 pipes then work side by side instead of one pass
// after the other.
template <int N, class Src>
__global__ void __launch_bounds__(tile_max_warps(N) * 32, tile_min_ctas(N))
    lup_mixed_finish_kernel(Src src, CallHead *head, const unsigned int *pend,
                            const unsigned char *refine, long long refine_cap, float theta2,
                            unsigned char *fac, long long fac_cap,
                            double *__restrict__ logabs, double *__restrict__ phase,
                            int8_t *__restrict__ parity, int32_t *__restrict__ status) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int LDS = N + 1;
  constexpr size_t NL = (size_t)N * LDS;
  const int warps = blockDim.x >> 5;
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  unsigned char *base = smem_raw;
  float4 *HL = reinterpret_cast<float4 *>(base) + warp * NL;
  double2 *M = reinterpret_cast<double2 *>(HL);
  float2 *Rm = reinterpret_cast<float2 *>(HL);
  base += warps * NL * sizeof(float4);
  float2 *F = reinterpret_cast<float2 *>(base) + warp * NL;
  base += warps * NL * sizeof(float2);
  double *hold = reinterpret_cast<double *>(base) + warp * 2 * N;
  base += warps * 2 * (size_t)N * sizeof(double);
  float2 *diag = reinterpret_cast<float2 *>(reinterpret_cast<int *>(base) + warp * 2 * N);
  const CorrScratch cs{F, reinterpret_cast<int *>(diag), hold};
  // the corrections of the FP64 factorisations go to lup_mixed_fac_correct_kernel
  const FacList fl{&head->corr_count, fac, fac_cap, fac_copies<Src>()};
  // 1. the FP32 pass's rejections, dealt out
  const unsigned long long listed = head->pend_count;
  const unsigned long long stride = (unsigned long long)warps * gridDim.x;
  for (unsigned long long j = (unsigned long long)warp * gridDim.x + blockIdx.x; j < listed;
       j += stride) {
    const unsigned int e = pend[j];
    const long long b = e & ~kPendRouted;
    fallback_fp64_src(src, b, N, M, LDS, hold, lane, b, logabs, phase, parity, status,
                      (e & kPendRouted) ? LUFQHE_ST_FP64 : LUFQHE_ST_FALLBACK, &cs, &fl);
  }
  // 2. the saved matrices, claimed; a failed refinement is refactorised here
  DeferredOut out;
  if (refine) {
    unsigned long long *claimed = const_cast<unsigned long long *>(&head->refine_claimed);
    const unsigned long long saved = min(head->refine_saved, (unsigned long long)refine_cap);
    for (;;) {
      unsigned long long k = saved;
      if (lane == 0 && *(volatile unsigned long long *)claimed < saved)
        k = atomicAdd(claimed, 1ull);
      k = __shfl_sync(kFull, k, 0);
      if (k >= saved) break;
      const unsigned char *e = refine + k * refine_entry_bytes<N>();
      const RefineHead h = *reinterpret_cast<const RefineHead *>(e);
      const float2 *sF = reinterpret_cast<const float2 *>(e + sizeof(RefineHead));
      const float2 *sY = sF + NL;
      __syncwarp();
      for (int q = lane; q < (int)NL; q += 32) {
        F[q] = __ldcg(sF + q);
        Rm[q] = __ldcg(sY + q);
      }
      __syncwarp();
      const CFF prod = {h.xh, h.xl, h.yh, h.yl, h.prod_e};
      float2 corr;
      if (mixed_refine_tile<N>(F, Rm, Rm + NL, diag, lane, theta2, tile_la_est(prod, h.exp_sum),
                               corr))
        out.push(lane, h.b, prod, h.exp_sum, corr, h.par, logabs, phase, parity, status);
      else
        fallback_fp64_src(src, h.b, N, M, LDS, hold, lane, h.b, logabs, phase, parity, status,
                          LUFQHE_ST_FALLBACK, &cs, &fl);
    }
  }
  out.flush(lane, logabs, phase, parity, status);
}

// The corrections of the finish kernel's FP64 factorisations (n = 24, 32):
// entry j of the list by CTA j % grid with all its warps (the inlined
// fp64_correct_group, whose result is fp64_correct_warp's bit for bit), on the
// listed L\U and pivot order and the source's matrix. One warp per matrix,
// the factorisation (~92 us on a sub-partition's shared FP64 pipe) and then
// the correction (120-177 us) on the same warp had been the finish kernel's
// critical path.
// COPY: the entries carry the matrix (the host-link variant's list), which is
// the source of the residual instead of src.
template <int N, class Src, bool COPY = false>
__global__ void __launch_bounds__(kFacCorrectWarps * 32)
    lup_mixed_fac_correct_kernel(Src src, const CallHead *head, const unsigned char *fac,
                                 long long fac_cap, double *__restrict__ logabs,
                                 double *__restrict__ phase, int8_t *__restrict__ parity,
                                 int32_t *__restrict__ status) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ long long red[3 * kFacCorrectWarps];
  constexpr int LDS = N + 1;
  const int tid = threadIdx.x, nthr = blockDim.x;
  double2 *M = reinterpret_cast<double2 *>(smem_raw);
  double *hold = reinterpret_cast<double *>(M + (size_t)N * LDS);
  float2 *F = reinterpret_cast<float2 *>(hold + 2 * N);
  int *ints = reinterpret_cast<int *>(F + (size_t)N * LDS);
  const CorrScratch cs{F, ints, hold};
  const unsigned long long listed = min(head->corr_count, (unsigned long long)fac_cap);
  for (unsigned long long j = blockIdx.x; j < listed; j += gridDim.x) {
    const unsigned char *e = fac + j * fac_entry_bytes(N, COPY);
    const FacHead h = *reinterpret_cast<const FacHead *>(e);
    const int *pe = reinterpret_cast<const int *>(e + sizeof(FacHead));
    const double2 *fe = reinterpret_cast<const double2 *>(e + fac_factors_offset(N));
    __syncthreads();  // the previous entry's correction is done with the scratch
    for (int i = tid; i < N; i += nthr) ints[i] = __ldcg(pe + i);
    for (int q = tid; q < N * N; q += nthr) M[(q / N) * LDS + q % N] = __ldcg(fe + q);
    __syncthreads();
    double2 c;
    if constexpr (COPY)
      c = fp64_correct_group(DenseSource{reinterpret_cast<const double2 *>(e + fac_copy_offset(N)),
                                         N},
                             0, N, M, LDS, cs, tid, nthr, CtaBarrier(),
                             reinterpret_cast<float *>(red));
    else
      c = fp64_correct_group(src, h.b, N, M, LDS, cs, tid, nthr, CtaBarrier(),
                             reinterpret_cast<float *>(red));
    if (tid == 0) {
      logabs[h.b] = h.la + c.x;
      if (phase) phase[h.b] = h.ph + c.y;
      if (parity) parity[h.b] = (int8_t)h.par;
      if (status) status[h.b] = h.flag;
    }
  }
}

// The FP64 pass of the generic mixed kernel (n >= 24 without a register-tiled
// kernel): one CTA per SM; its warps refactorise the pending list's matrices
// (reference pivot rule, fused arithmetic, status flag LUFQHE_ST_FALLBACK, or
// LUFQHE_ST_FP64 for the routed share). Every factorisation of one n costs the
// same, so the entries are dealt out at a fixed stride: entry j goes to warp
// j / G of CTA j % G (G CTAs), so the first G entries land on warp 0 of every
// SM, the next G on warp 1 (the next SM sub-partition), and no sub-partition's
// FP64 pipe holds more than ceil(count / (4 G)) of them when the list is
// short. (First-come claims piled up to five matrices on some sub-partitions
// while others idled.)
template <class Src>
__global__ void __launch_bounds__(kFallbackMaxWarps * 32)
    lup_mixed_fallback_kernel(Src src, int n, const CallHead *head, const unsigned int *pend,
                              double *__restrict__ logabs, double *__restrict__ phase,
                              int8_t *__restrict__ parity, int32_t *__restrict__ status) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int warps = blockDim.x >> 5;
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int lds = n + 1;
  double2 *M = reinterpret_cast<double2 *>(smem_raw) + (size_t)warp * n * lds;
  double *hold_all = reinterpret_cast<double *>(reinterpret_cast<double2 *>(smem_raw) +
                                                (size_t)warps * n * lds);
  double *hold = hold_all + warp * 2 * n;
  // n <= kCorrectMaxN: the correction's scratch after the row scales
  // (fallback_smem_per_warp)
  float2 *F_all = reinterpret_cast<float2 *>(hold_all + (size_t)warps * 2 * n);
  const CorrScratch cs{F_all + (size_t)warp * n * lds,
                       reinterpret_cast<int *>(F_all + (size_t)warps * n * lds) + warp * 2 * n,
                       hold};
  const unsigned long long listed = head->pend_count;
  const unsigned long long stride = (unsigned long long)warps * gridDim.x;
  for (unsigned long long j = (unsigned long long)warp * gridDim.x + blockIdx.x; j < listed;
       j += stride) {
    const unsigned int e = pend[j];
    const long long b = e & ~kPendRouted;
    fallback_fp64_src(src, b, n, M, lds, hold, lane, b, logabs, phase, parity, status,
                      (e & kPendRouted) ? LUFQHE_ST_FP64 : LUFQHE_ST_FALLBACK,
                      n <= kCorrectMaxN ? &cs : nullptr);
  }
}

// the bulk-copy staging for complex128 matrices in device memory only
inline int bulk_for(const DenseSource &s) { return g_bulk_loads && is_device_memory(s.A); }
template <class S>
inline int bulk_for(const S &) {
  return 0;
}

// A call's state block: the head, the pending list (pend_cap entries), the
// saved matrices of the refinement (refine_bytes) and the host-link copies
// (spill_bytes), each 256-byte aligned; the head is zeroed on `stream`.
struct CallState {
  unsigned char *block = nullptr;
  CallHead *head = nullptr;
  unsigned int *pend = nullptr;
  unsigned char *refine = nullptr;
  double2 *spill = nullptr;
  unsigned char *corr = nullptr;

  int acquire(size_t pend_cap, size_t refine_bytes, size_t spill_bytes, cudaStream_t stream,
              size_t corr_bytes = 0) {
    auto up = [](size_t v) { return (v + 255) & ~(size_t)255; };
    const size_t pend_bytes = up(pend_cap * sizeof(unsigned int));
    const size_t total =
        kHeadBytes + pend_bytes + up(refine_bytes) + up(spill_bytes) + up(corr_bytes);
    int rc = lib_malloc_async((void **)&block, total, stream);
    if (rc) return rc;
    head = reinterpret_cast<CallHead *>(block);
    unsigned char *p = block + kHeadBytes;
    pend = pend_cap ? reinterpret_cast<unsigned int *>(p) : nullptr;
    p += pend_bytes;
    refine = refine_bytes ? p : nullptr;
    p += up(refine_bytes);
    spill = spill_bytes ? reinterpret_cast<double2 *>(p) : nullptr;
    p += up(spill_bytes);
    corr = corr_bytes ? p : nullptr;
    return check_cuda(cudaMemsetAsync(block, 0, kHeadBytes, stream), "memset(call state)");
  }
  int release(cudaStream_t stream, int rc) {
    if (!block) return rc;
    const int r2 = lib_free_async(block, stream);
    block = nullptr;
    return rc ? rc : r2;
  }
};

// Whether warps must claim matrices from a counter: a batch beyond two strides
// of the grid. (A call that takes a state block anyway, for its pending list
// or host-link copies, claims from the block's zeroed counter regardless.)
inline bool needs_counter(long long batch, long long grid_warps) {
  return batch > 2 * grid_warps;
}

// Shared memory of one warp of the FP64 pass: the matrix and its row scales;
// for n <= kCorrectMaxN also the correction's float2 matrix and 2n ints.
inline size_t fallback_smem_per_warp(int n) {
  size_t b = (size_t)n * (n + 1) * sizeof(double2) + 2 * (size_t)n * sizeof(double);
  if (n <= kCorrectMaxN) b += (size_t)n * (n + 1) * sizeof(float2) + 2 * (size_t)n * sizeof(int);
  return b;
}

template <class Src>
int launch_fallback(Src src, int n, const CallHead *head, const unsigned int *pend,
                    long long batch, double *logabs, double *phase, int8_t *parity,
                    int32_t *status, cudaStream_t stream) {
  const size_t per_warp = fallback_smem_per_warp(n);
  int warps = (int)(device_smem_optin() / per_warp);
  if (warps > kFallbackMaxWarps) warps = kFallbackMaxWarps;
  if (warps < 1) warps = 1;
  const size_t smem = per_warp * warps;
  auto kern = lup_mixed_fallback_kernel<Src>;
  int rc = check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem),
                      "cudaFuncSetAttribute(mixed fallback)");
  if (rc) return rc;
  int per_sm = 0;
  rc = check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, warps * 32, smem),
                  "occupancy(mixed fallback)");
  if (rc) return rc;
  if (per_sm < 1) {
    set_error("mixed fallback: n=%d does not fit on an SM", n);
    return LUFQHE_ERR_UNSUPPORTED_N;
  }
  // one CTA per SM (the list's length is known only on the device)
  long long want = (batch + warps - 1) / warps;
  long long cap = (long long)device_sm_count();
  int grid = (int)(want < cap ? want : cap);
  KernelTimer timer("lup_mixed_fallback_kernel", n, stream);
  kern<<<grid, warps * 32, smem, stream>>>(src, n, head, pend, logabs, phase, parity, status);
  timer.stop();
  return check_cuda(cudaGetLastError(), "lup_mixed_fallback_kernel launch");
}

// The correction pass over a factor list of capacity cap (its length is
// known only on the device): as many CTAs as fit, at most one per entry.
template <int N, class Src, bool COPY>
int launch_fac_correct(Src src, const CallHead *head, const unsigned char *list, long long cap,
                       double *logabs, double *phase, int8_t *parity, int32_t *status,
                       cudaStream_t stream) {
  auto k = lup_mixed_fac_correct_kernel<N, Src, COPY>;
  const size_t smem = fallback_smem_per_warp(N);
  int rc = check_cuda(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem),
                      "cudaFuncSetAttribute(mixed fac correct)");
  int per_sm = 0;
  if (!rc)
    rc = check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k,
                                                                  kFacCorrectWarps * 32, smem),
                    "occupancy(mixed fac correct)");
  if (rc) return rc;
  const long long fit = (long long)device_sm_count() * std::max(1, per_sm);
  const int grid = (int)std::min<long long>(cap, fit);
  KernelTimer timer(COPY ? "lup_mixed_fac_correct_kernel_hostlink" : "lup_mixed_fac_correct_kernel",
                    N, stream);
  k<<<grid, kFacCorrectWarps * 32, smem, stream>>>(src, head, list, cap, logabs, phase, parity,
                                                   status);
  timer.stop();
  return check_cuda(cudaGetLastError(), "lup_mixed_fac_correct_kernel launch");
}

template <int N, class Src>
int launch_mixed_tile(Src src, long long batch, float theta2, double *logabs, double *phase,
                      int8_t *parity, int32_t *status, cudaStream_t stream, bool inplace) {
  // only dense batches of the deferring sizes have an in-place variant
  constexpr bool kHasInplace = N >= kDeferMinN && std::is_same<Src, DenseSource>::value;
  if (!kHasInplace) inplace = false;
  const size_t per_warp = tile_smem_per_warp<N>();
  // small CTAs: the register-heavy residual tile limits residency, and
  // smaller CTAs let the scheduler fill an SM with several of them
  int warps = (int)(device_smem_optin() / per_warp);
  int wcap = tile_max_warps(N);
  if (g_tile_warps > 0 && g_tile_warps < wcap) wcap = g_tile_warps;
  if (warps > wcap) warps = wcap;
  const size_t smem = per_warp * warps;
  auto kern = lup_mixed_tile_kernel<N, Src, false>;
  if constexpr (kHasInplace)
    if (inplace) kern = lup_mixed_tile_kernel<N, Src, true>;
  int rc = check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem),
                      "cudaFuncSetAttribute(mixed tile)");
  if (rc) return rc;
  int per_sm = 0;
  rc = check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, warps * 32, smem),
                  "occupancy(mixed tile)");
  if (rc) return rc;
  if (per_sm < 1) per_sm = 1;
  long long want = (batch + warps - 1) / warps;
  long long cap = (long long)device_sm_count() * per_sm;
  int grid = (int)(want < cap ? want : cap);
  // n >= 24 from device memory: the refinements and FP64 refactorisations go
  // to the finish kernel through the call's pending list and saved matrices
  const bool two_pass = N >= kDeferMinN && !inplace;
  long long refine_cap = 0;
  size_t refine_bytes = 0;
  if (two_pass && g_mixed_refine) {
    refine_cap = std::max<long long>(256, (long long)(kRefineShare * (double)batch));
    refine_cap = std::min<long long>(refine_cap, batch);
    refine_bytes = (size_t)refine_cap * refine_entry_bytes<N>();
  }
  const size_t spill_bytes = inplace ? (size_t)grid * warps * N * N * sizeof(double2) : 0;
  // the host-link variant's correction list (sizes with a corrected FP64 route)
  long long corr_cap = 0;
  if (inplace && N >= kCorrectMinN) {
    corr_cap = std::max<long long>(256, (long long)(kCorrShare * (double)batch));
    corr_cap = std::min<long long>(corr_cap, batch);
  }
  // the device path's list of FP64 factors for the correction pass (an
  // overflow is corrected in the finish kernel itself)
  long long fac_cap = 0;
  if (two_pass && N >= kCorrectMinN && N <= kCorrectMaxN) {
    fac_cap = std::max<long long>(256, (long long)(kCorrShare * (double)batch));
    fac_cap = std::min<long long>(fac_cap, batch);
  }
  CallState cs;
  if (two_pass || inplace || needs_counter(batch, (long long)grid * warps)) {
    rc = cs.acquire(two_pass ? (size_t)batch : 0, refine_bytes, spill_bytes, stream,
                    inplace ? (size_t)corr_cap * (size_t)fac_entry_bytes(N, true)
                            : (size_t)fac_cap * (size_t)fac_entry_bytes(N, fac_copies<Src>()));
    if (rc) return cs.release(stream, rc);
  }
  // in-place kernels: refine_cap says whether the refinement is on
  if (!two_pass) refine_cap = g_mixed_refine;
  {
    KernelTimer timer(inplace ? "lup_mixed_tile_kernel_hostlink" : "lup_mixed_tile_kernel", N,
                      stream);
    kern<<<grid, warps * 32, smem, stream>>>(src, batch, theta2, fp64_share_64k(N), cs.head, cs.pend,
                                             cs.spill, cs.refine, refine_cap, cs.corr, corr_cap,
                                             bulk_for(src), logabs, phase, parity, status);
    timer.stop();
  }
  rc = check_cuda(cudaGetLastError(), "lup_mixed_tile_kernel launch");
  if (!rc && corr_cap > 0) {
    if constexpr (kHasInplace && N >= kCorrectMinN && N <= kCorrectMaxN)
      rc = launch_fac_correct<N, Src, true>(src, cs.head, cs.corr, corr_cap, logabs, phase,
                                            parity, status, stream);
  }
  // the refinements and the FP64 refactorisations, side by side in one kernel,
  // then the corrections of those refactorisations, each by a whole CTA
  if (!rc && two_pass) {
    if constexpr (N >= kDeferMinN) {
      auto fk = lup_mixed_finish_kernel<N, Src>;
      rc = check_cuda(cudaFuncSetAttribute(fk, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem),
                      "cudaFuncSetAttribute(mixed finish)");
      if (!rc) {
        KernelTimer timer("lup_mixed_finish_kernel", N, stream);
        fk<<<grid, warps * 32, smem, stream>>>(src, cs.head, cs.pend, cs.refine, refine_cap,
                                               theta2, cs.corr, fac_cap, logabs, phase, parity,
                                               status);
        timer.stop();
        rc = check_cuda(cudaGetLastError(), "lup_mixed_finish_kernel launch");
      }
      if (!rc && fac_cap > 0)
        rc = launch_fac_correct<N, Src, fac_copies<Src>() != 0>(src, cs.head, cs.corr, fac_cap,
                                                                logabs, phase, parity, status,
                                                                stream);
    }
  }
  return cs.release(stream, rc);
}

// Sources whose matrices are always of odd order (CF matrices, n = 2Q + 3)
// never reach the register-tiled kernels, which exist for even n only.
template <class S, class = void>
struct has_even_n : std::true_type {};
template <class S>
struct has_even_n<S, std::void_t<decltype(S::kOddN)>> : std::false_type {};

// plain_fp64: the plain fused kernel on the same source (the all-FP64 route)
template <class Src, class PlainFn>
int launch_mixed_src(Src src, int n, long long batch, double *logabs, double *phase,
                     int8_t *parity, int32_t *status, cudaStream_t stream, PlainFn plain_fp64,
                     bool inplace = false) {
  if (batch == 0) return LUFQHE_SUCCESS;
  // every matrix on the FP64 route: the plain fused kernel, whose shared
  // memory layout holds more warps per SM than the mixed kernels'
  if (fp64_share_64k(n) >= 65536u)
    return plain_fp64();
  const float th2 = g_mixed_theta * g_mixed_theta;
  if constexpr (has_even_n<Src>::value) {
    switch (n) {
      case 6: return launch_mixed_tile<6>(src, batch, th2, logabs, phase, parity, status, stream, inplace);
      case 8: return launch_mixed_tile<8>(src, batch, th2, logabs, phase, parity, status, stream, inplace);
      case 12: return launch_mixed_tile<12>(src, batch, th2, logabs, phase, parity, status, stream, inplace);
      case 16: return launch_mixed_tile<16>(src, batch, th2, logabs, phase, parity, status, stream, inplace);
      case 24: return launch_mixed_tile<24>(src, batch, th2, logabs, phase, parity, status, stream, inplace);
      case 32: return launch_mixed_tile<32>(src, batch, th2, logabs, phase, parity, status, stream, inplace);
      default: break;
    }
  }
  const size_t per_warp = mixed_smem_per_warp(n);
  const size_t optin = device_smem_optin();
  int warps = (int)(optin / per_warp);
  if (warps > 4) warps = 4;
  if (warps < 1) {
    set_error("n=%d needs %zu bytes of shared memory per matrix; the device offers %zu", n,
              per_warp, optin);
    return LUFQHE_ERR_UNSUPPORTED_N;
  }
  const size_t smem = per_warp * warps;
  auto kern = lup_mixed_kernel<Src>;
  int rc = check_cuda(cudaFuncSetAttribute(kern,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                      "cudaFuncSetAttribute(mixed)");
  if (rc) return rc;
  int per_sm = 0;
  rc = check_cuda(
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, warps * 32, smem),
      "occupancy(mixed)");
  if (rc) return rc;
  if (per_sm < 1) per_sm = 1;
  long long want = (batch + warps - 1) / warps;
  long long cap = (long long)device_sm_count() * per_sm;
  int grid = (int)(want < cap ? want : cap);
  const float theta2 = g_mixed_theta * g_mixed_theta;
  // n >= 24: rejected matrices go to the FP64 pass through the call's list
  const bool two_pass = n >= kDeferMinN;
  const bool counter = needs_counter(batch, (long long)grid * warps);
  CallState cs;
  if (two_pass || counter) {
    rc = cs.acquire(two_pass ? (size_t)batch : 0, 0, 0, stream);
    if (rc) return cs.release(stream, rc);
  }
  {
    KernelTimer timer("lup_mixed_kernel", n, stream);
    kern<<<grid, warps * 32, smem, stream>>>(src, n, batch, theta2, fp64_share_64k(n),
                                             cs.head, cs.pend, logabs, phase, parity, status);
    timer.stop();
  }
  rc = check_cuda(cudaGetLastError(), "lup_mixed_kernel launch");
  if (!rc && two_pass)
    rc = launch_fallback(src, n, cs.head, cs.pend, batch, logabs, phase, parity, status, stream);
  return cs.release(stream, rc);
}

}  // namespace

}  // namespace lufqhe
