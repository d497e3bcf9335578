// Mixed-size batches in one persistent launch.
//
// A batch made of groups of same-size matrices (n differs between groups) is
// cut into work items: tiles of T(n) consecutive matrices of one group. The
// items are ordered largest n first (longest-processing-time first, so the
// short small-n items fill the tail), stored in device memory, and consumed
// by a persistent kernel: each warp takes the next item with one atomicAdd on
// a device counter and runs the per-n device routine (the register-tiled
// mixed routine for n in {6, 8, 12, 16, 24, 32}, the generic one otherwise,
// or the FP64 routines in the plain modes). Shared memory per warp is sized
// for the largest n of the batch.
//
// A plan (lufqhe_plan_create) fixes the groups and output buffers, chooses the
// tile sizes and the warps per CTA with an autotuner that times candidate
// launches on the plan's own data, and captures its launch in a CUDA graph
// that lufqhe_plan_execute replays:
//  - the counter and list resets;
//  - its passes, each a persistent kernel (see Launch);
//  - for a mixed plan, the pending FP64 refactorisations of its n = 24..32
//    matrices and the correction passes of their listed factors, as the
//    batched mixed mode runs them.

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "mixed_core.cuh"

namespace lufqhe {

// The plan's correction passes (lup_mixed.cu, where the correction kernel is
// built): corrections of the FP64 factorisations listed for size n, each
// entry with its matrix; head is the list's zeroed header block.
int launch_listed_corrections(int n, const void *head, const unsigned char *list, long long cap,
                              double *logabs, double *phase, int8_t *parity, int32_t *status,
                              cudaStream_t stream);
size_t listed_count_offset();
size_t head_bytes();


namespace {

using namespace mixed;

// Sizes whose FP64 factorisations a mixed plan lists for its correction pass
// (the register-tiled sizes the correction kernel is built for): lists is an
// array of kListMaxN + 1 FacLists indexed by n.
constexpr int kListMaxN = 32;

// A matrix that a mixed plan's warp pass sends to FP64 (rejected by the FP32
// path, or routed), for the plan's pending pass.
struct PendEntry {
  const double2 *A;  // the matrix
  long long ob;      // its output index
  int n, lda, flag, pad;
};

// A mixed plan's device extras, passed to its kernels by value: the factor
// lists by n, and the pending FP64 refactorisations of its n >= kPlanDeferMinN
// matrices (pend null: each is refactorised by the warp that rejected it).
struct PlanAux {
  const FacList *lists;
  PendEntry *pend;
  unsigned int *pend_count;
  unsigned int pend_cap;
};

// Sizes whose FP64 refactorisations a mixed plan leaves to its pending pass
// (as the batched mixed mode leaves them to its finish kernel from n = 24).
constexpr int kPlanDeferMinN = 24;

// A plan's passes (see Launch), and the largest n of a mixed plan's small
// pass: its own build of the grouped kernel, whose register-tiled cases stop
// at n = 16, takes under 128 registers and runs two 8-warp CTAs per SM where
// the build with the n = 24 and 32 cases (190 registers) runs one.
constexpr int kPlanPasses = 4;
constexpr int kSmallPassMaxN = 16;

struct WorkItem {
  const double2 *A;  // group base
  long long first;   // first matrix of the tile within the group
  long long out;     // output index of that matrix
  int count;         // matrices in the tile
  int n;
  int lda;
  unsigned int share64k;  // mixed mode: share routed straight to FP64 (1/65536)
  int status_or;          // bits OR-ed into each status (FP64 route of a mixed plan)
};

// Shared memory of one warp, contiguous: [matrix area][F][hold][er, ec].
//  * matrix area: the FP64 matrix (double2, nf x (nf+1)) for the FP64 routine,
//    aliased by the FP32 path's hi/lo copy (float4, nm x (nm+1));
//  * F: the FP32 factor (float2, nm x (nm+1)); hold: 2 nf doubles; er, ec:
//    2 nm ints.
// nf is the largest n of the plan, nm the largest n that takes the FP32 path
// (0 in the plain modes and for groups the precision policy sends to FP64),
// so a group that only runs the FP64 routine costs the plain kernel's bytes.
struct WarpLayout {
  size_t area, f, hold, total;
};

__host__ __device__ inline WarpLayout warp_layout(int nm, int nf) {
  WarpLayout L;
  const size_t a_fp64 = (size_t)nf * (nf + 1) * sizeof(double2);
  const size_t a_fp32 = (size_t)nm * (nm + 1) * sizeof(float4);
  L.area = a_fp64 > a_fp32 ? a_fp64 : a_fp32;
  L.f = (size_t)nm * (nm + 1) * sizeof(float2);
  L.hold = 2 * (size_t)nf * sizeof(double);
  const size_t ints = 2 * (size_t)nm * sizeof(int);
  L.total = (L.area + L.f + L.hold + ints + 15) & ~(size_t)15;
  return L;
}

// FP64 refactorisation of a matrix of a mixed plan's warp pass: appended to
// the pending list when the plan has one for this size and it has room, else
// done here (its factors listed for the correction pass when fl has room).
__device__ void plan_fp64(const double2 *src, int n, int lda, long long ob, double2 *M,
                          double *hold, int lane, int flag, const CorrScratch &cs,
                          const FacList *fl, const PlanAux &aux, double *logabs, double *phase,
                          int8_t *parity, int32_t *status) {
  // (the pending pass's shared memory holds the plan's largest n <= kListMaxN)
  if (aux.pend && n >= kPlanDeferMinN && n <= kListMaxN) {
    unsigned int k = 0;
    if (lane == 0) k = atomicAdd(aux.pend_count, 1u);
    k = __shfl_sync(kFull, k, 0);
    if (k < aux.pend_cap) {
      if (lane == 0) aux.pend[k] = PendEntry{src, ob, n, lda, flag, 0};
      return;
    }
  }
  fallback_fp64_src(DenseSource{src, lda}, 0, n, M, n + 1, hold, lane, ob, logabs, phase, parity,
                    status, flag, &cs, fl);
}

template <int MODE, bool SMALL = false>
__device__ void process_matrix(const double2 *src, int n, int lda, long long ob, float4 *HL,
                               float2 *F, double *hold, int *er, int *ec, int nm, int lane,
                               float theta2, bool refine, unsigned int share64k, int status_or,
                               const FacList *fl, const PlanAux &aux, DeferredOut &out,
                               double *logabs, double *phase, int8_t *parity, int32_t *status) {
  const int lds = n + 1;
  double2 *M = reinterpret_cast<double2 *>(HL);
  // a group on the FP32 path has F and 2n ints (n <= nm) for the correction;
  // a mixed plan defers its FP64 refactorisations and lists their factors for
  // its correction pass, while its lists have room
  const CorrScratch cs{F, er, hold};
  if (MODE == LUFQHE_MODE_MIXED && route_fp64(src, share64k)) {
    plan_fp64(src, n, lda, ob, M, hold, lane, LUFQHE_ST_FP64, cs, fl, aux, logabs, phase, parity,
              status);
    return;
  }
  if (load_matrix_fp64(src, n, lda, M, lds, lane)) {
    emit_nonfinite(lane, ob, logabs, phase, parity, status);
    return;
  }
  if (MODE == LUFQHE_MODE_MIXED) {
    CFF prod;
    int exp_sum = 0, par = 0;
    float2 corr;
    bool ok;
    switch (n) {
      case 6: ok = mixed_factor_tile<6>(HL, F, er, ec, lane, theta2, prod, exp_sum, corr, par, refine); break;
      case 8: ok = mixed_factor_tile<8>(HL, F, er, ec, lane, theta2, prod, exp_sum, corr, par, refine); break;
      case 12: ok = mixed_factor_tile<12>(HL, F, er, ec, lane, theta2, prod, exp_sum, corr, par, refine); break;
      case 16: ok = mixed_factor_tile<16>(HL, F, er, ec, lane, theta2, prod, exp_sum, corr, par, refine); break;
      // (never reached in the small pass, n <= kSmallPassMaxN)
      case 24:
        if constexpr (SMALL) ok = false;
        else ok = mixed_factor_tile<24>(HL, F, er, ec, lane, theta2, prod, exp_sum, corr, par, refine);
        break;
      case 32:
        if constexpr (SMALL) ok = false;
        else ok = mixed_factor_tile<32>(HL, F, er, ec, lane, theta2, prod, exp_sum, corr, par, refine);
        break;
      default: {
        MixedSmem S;
        S.SC = HL;
        S.Af = F;
        S.hold = hold;
        S.er = er;
        S.ec = ec;
        ok = mixed_factor(S, n, lane, theta2, prod, exp_sum, corr, par);
      }
    }
    if (ok)
      out.push(lane, ob, prod, exp_sum, corr, par, logabs, phase, parity, status);
    else
      plan_fp64(src, n, lda, ob, M, hold, lane, LUFQHE_ST_FALLBACK, cs, fl, aux, logabs, phase,
                parity, status);
  } else {
    // a mixed plan's FP64 route (status_or set) gets the correction where the
    // batched mixed mode does; its pass reserves the scratch (nm >= n)
    const bool correct = MODE == LUFQHE_MODE_PLAIN_FP64_FUSED && status_or != 0 && nm >= n &&
                         n >= kCorrectMinN && n <= 32;
    int par = 0;
    int st = MODE == LUFQHE_MODE_PLAIN_FP64
                 ? lup_fp64_warp<ARITH_REF>(M, lds, hold, n, lane, &par)
                 : lup_fp64_warp<ARITH_FUSED>(M, lds, hold, n, lane, &par,
                                              correct ? er : nullptr);
    double la, ph;
    if (st == 0) {
      logdet_from_diag(M, lds, n, lane, par, &la, &ph);
      if (correct) fp64_correct_warp(DenseSource{src, lda}, 0, n, M, lds, cs, lane, &la, &ph);
    } else if (st == LUFQHE_ST_SINGULAR) {
      la = -INFINITY;
      ph = 0.0;
    } else {
      la = NAN;
      ph = NAN;
      par = 0;
    }
    if (lane == 0) {
      logabs[ob] = la;
      if (phase) phase[ob] = ph;
      if (parity) parity[ob] = (int8_t)par;
      if (status) status[ob] = st | status_or;
    }
  }
}

template <int MODE, bool SMALL = false>
__global__ void __launch_bounds__(kMaxWarpsMixed * 32, SMALL ? 2 : 1)
    grouped_kernel(const WorkItem *__restrict__ items, int nitems, unsigned int *counter, int nm,
                   int nf,
                   float theta2, int refine, double *__restrict__ logabs, double *__restrict__ phase,
                   int8_t *__restrict__ parity, int32_t *__restrict__ status, PlanAux aux) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int warps = blockDim.x >> 5;
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  (void)warps;
  const WarpLayout L = warp_layout(nm, nf);
  unsigned char *base = smem_raw + (size_t)warp * L.total;
  float4 *HL = reinterpret_cast<float4 *>(base);
  float2 *F = reinterpret_cast<float2 *>(base + L.area);
  double *hold = reinterpret_cast<double *>(base + L.area + L.f);
  int *er = reinterpret_cast<int *>(base + L.area + L.f + L.hold);
  int *ec = er + nm;

  DeferredOut out;
  for (;;) {
    unsigned int it = 0;
    if (lane == 0) it = atomicAdd(counter, 1u);
    it = __shfl_sync(kFull, it, 0);
    if (it >= (unsigned int)nitems) break;
    const WorkItem w = items[it];
    // the plan's factor list for this size (lists[n].count null: none)
    const FacList *fl = nullptr;
    if (MODE == LUFQHE_MODE_MIXED && aux.lists && w.n <= kListMaxN && aux.lists[w.n].count)
      fl = aux.lists + w.n;
    for (int j = 0; j < w.count; ++j) {
      __syncwarp();
      const long long b = w.first + j;
      process_matrix<MODE, SMALL>(w.A + (size_t)b * w.n * w.lda, w.n, w.lda, w.out + j, HL, F, hold, er,
                           ec, nm, lane, theta2, refine != 0, w.share64k, w.status_or, fl, aux,
                           out, logabs, phase, parity, status);
    }
  }
  out.flush(lane, logabs, phase, parity, status);
}

using GroupedKernel = void (*)(const WorkItem *, int, unsigned int *, int, int, float, int,
                               double *, double *, int8_t *, int32_t *, PlanAux);

GroupedKernel kernel_for(int mode, bool small = false) {
  switch (mode) {
    case LUFQHE_MODE_PLAIN_FP64: return grouped_kernel<LUFQHE_MODE_PLAIN_FP64>;
    case LUFQHE_MODE_PLAIN_FP64_FUSED: return grouped_kernel<LUFQHE_MODE_PLAIN_FP64_FUSED>;
    default:
      return small ? grouped_kernel<LUFQHE_MODE_MIXED, true> : grouped_kernel<LUFQHE_MODE_MIXED>;
  }
}

// Default tile: about 64 n=8-equivalents of work per item (flops scale ~n^3).
int default_tile(int n) {
  double t = 64.0 * std::pow(8.0 / (double)n, 3.0);
  int v = (int)std::lround(t);
  return std::max(1, std::min(256, v));
}

// Warp-group form of the grouped kernel for the FP64 route at n > 32: each CTA
// claims work items and factorises their matrices with all its threads
// (lup_fp64_group), as the batched plain kernel does for those sizes.
// CORRECT (a mixed plan's pass): the results of items with n <= nm get the
// extended-precision correction (fp64_correct_group), as the batched mixed
// mode's FP64 route does; its scratch (nm x (nm + 1) float2 and 2 nm ints)
// follows the row scales.
template <int ARITH, bool CORRECT = false>
__global__ void __launch_bounds__(kFp64GroupWarps * 32)
    grouped_group_kernel(const WorkItem *__restrict__ items, int nitems, unsigned int *counter,
                         int nm, int nf, float theta2, int refine, double *__restrict__ logabs,
                         double *__restrict__ phase, int8_t *__restrict__ parity,
                         int32_t *__restrict__ status, PlanAux aux) {
  (void)theta2;
  (void)refine;
  (void)aux;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ long long red[3 * kFp64GroupWarps];
  __shared__ unsigned int item;
  const int tid = threadIdx.x, nthr = blockDim.x;
  double2 *M = reinterpret_cast<double2 *>(smem_raw);
  double *hold = reinterpret_cast<double *>(M + (size_t)nf * (nf + 1));
  float2 *F = reinterpret_cast<float2 *>(hold + 2 * nf);   // nm x (nm + 1)
  int *ints = reinterpret_cast<int *>(F + (size_t)nm * (nm + 1));
  for (;;) {
    __syncthreads();
    if (tid == 0) item = atomicAdd(counter, 1u);
    __syncthreads();
    const unsigned int it = item;
    if (it >= (unsigned int)nitems) break;
    const WorkItem w = items[it];
    const int n = w.n, lds = n + 1;
    const DenseSource src{w.A, w.lda};
    for (int j = 0; j < w.count; ++j) {
      __syncthreads();
      const long long ob = w.out + j;
      int par = 0;
      const bool correct = CORRECT && w.status_or != 0 && n <= nm;
      int st = src.load_group(w.first + j, n, M, lds, tid, nthr) ? LUFQHE_ST_NONFINITE : 0;
      if (!st)
        st = lup_fp64_group<ARITH>(M, lds, hold, n, tid, nthr, red, &par, CtaBarrier(),
                                   correct ? ints : nullptr);
      __syncthreads();
      double la = 0.0, ph = 0.0;
      if (tid < 32) {
        if (st == 0) {
          logdet_from_diag(M, lds, n, tid, par, &la, &ph);
        } else if (st == LUFQHE_ST_SINGULAR) {
          la = -INFINITY;
          ph = 0.0;
        } else {
          la = NAN;
          ph = NAN;
          par = 0;
        }
      }
      if (correct && st == 0) {
        __syncthreads();  // the diagonal is read before the correction overwrites M
        const double2 c = fp64_correct_group(src, w.first + j, n, M, lds,
                                             CorrScratch{F, ints, hold}, tid, nthr, CtaBarrier(),
                                             reinterpret_cast<float *>(red));
        la += c.x;
        ph += c.y;
      }
      if (tid == 0) {
        logabs[ob] = la;
        if (phase) phase[ob] = ph;
        if (parity) parity[ob] = (int8_t)par;
        if (status) status[ob] = st | w.status_or;
      }
    }
  }
}

// A mixed plan's pending pass: the FP64 refactorisations its warp pass left
// (n >= kPlanDeferMinN), one warp per matrix, in shared memory sized for the
// largest of them (the matrix, row scales, and the correction's scratch)
// rather than the warp pass's FP32-path layout and registers. Each
// factorisation is listed for the correction pass while its size's list has
// room, else corrected here.
constexpr int kPendWarps = 4;

__host__ __device__ inline size_t pending_warp_bytes(int n) {
  const size_t b = (size_t)n * (n + 1) * sizeof(double2) + 2 * (size_t)n * sizeof(double) +
                   (size_t)n * (n + 1) * sizeof(float2) + 2 * (size_t)n * sizeof(int);
  return (b + 15) & ~(size_t)15;
}

__global__ void __launch_bounds__(kPendWarps * 32)
    grouped_pending_kernel(PlanAux aux, int nmax, double *__restrict__ logabs,
                           double *__restrict__ phase, int8_t *__restrict__ parity,
                           int32_t *__restrict__ status) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int warps = blockDim.x >> 5;
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  unsigned char *base = smem_raw + (size_t)warp * pending_warp_bytes(nmax);
  double2 *M = reinterpret_cast<double2 *>(base);
  double *hold = reinterpret_cast<double *>(M + (size_t)nmax * (nmax + 1));
  float2 *F = reinterpret_cast<float2 *>(hold + 2 * nmax);
  int *ints = reinterpret_cast<int *>(F + (size_t)nmax * (nmax + 1));
  const CorrScratch cs{F, ints, hold};
  const unsigned int listed = min(*aux.pend_count, aux.pend_cap);
  const unsigned int stride = (unsigned int)(gridDim.x * warps);
  for (unsigned int j = blockIdx.x * warps + warp; j < listed; j += stride) {
    const PendEntry e = aux.pend[j];
    const FacList *fl = nullptr;
    if (aux.lists && e.n <= kListMaxN && aux.lists[e.n].count) fl = aux.lists + e.n;
    fallback_fp64_src(DenseSource{e.A, e.lda}, 0, e.n, M, e.n + 1, hold, lane, e.ob, logabs,
                      phase, parity, status, e.flag, &cs, fl);
  }
}

// correct: a mixed plan's pass (its layout reserves the correction's scratch)
GroupedKernel group_kernel_for(int mode, bool correct) {
  if (correct) return grouped_group_kernel<ARITH_FUSED, true>;
  return mode == LUFQHE_MODE_PLAIN_FP64 ? grouped_group_kernel<ARITH_REF>
                                        : grouped_group_kernel<ARITH_FUSED>;
}

// One pass of a plan: a grouped kernel over its own work list. A plan runs up
// to three passes back to back:
//  0. the plan's mode over the groups on the warp-per-matrix path (a mixed
//     plan's FP32-path groups; a plain plan's groups with n <= 32);
//  1. (mixed plans) the plain fused kernel over the groups with n <= 32 that
//     the precision policy sends to FP64;
//  2. the warp-group kernel over the FP64-route groups with n > 32 (fused
//     arithmetic for a mixed plan, the plan's arithmetic for a plain one);
//  3. (mixed plans) the small build of the mixed kernel over the FP32-path
//     groups with n <= kSmallPassMaxN, at twice pass 0's occupancy.
// Groups routed to FP64 need neither the FP32 path's shared memory nor its
// registers, and get the plain kernels' occupancy. After the passes a mixed
// plan runs its pending pass (grouped_pending_kernel) and the correction
// passes of its factor lists.
struct Launch {
  int mode = LUFQHE_MODE_MIXED;
  int nm = 0, nf = 1;  // warp_layout of the pass
  int warps = 4;
  int ctas = 0;        // grid size
  size_t smem = 0;
  int first = 0;       // first work item of the pass in the device list
  int nitems = 0;
};

}  // namespace

}  // namespace lufqhe

using namespace lufqhe;

struct lufqhe_plan_s {
  std::vector<lufqhe_group_t> groups;
  int mode = LUFQHE_MODE_MIXED;
  int nmax = 1;      // largest n of any group
  long long total = 0;
  double *logabs = nullptr, *phase = nullptr;
  int8_t *parity = nullptr;
  int32_t *status = nullptr;
  float theta2 = 0.01f;
  int refine = 1;  // in-place refinement of the tile path (option 5)
  // per-group tile size and FP64 share (1/65536) chosen by the tuner
  std::vector<int> tile;
  std::vector<unsigned int> share;
  Launch launch[kPlanPasses];
  // device state
  WorkItem *d_items = nullptr;
  unsigned int *d_counter = nullptr;
  int nitems = 0;
  size_t items_cap = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaStream_t cap_stream = nullptr;
  std::string report;
  // a mixed plan's factor lists (n = 24 and 32): the FP64 factorisations of
  // its FP32-path groups, corrected after the passes by a whole CTA each, as
  // in the batched mixed mode (a warp correcting its own in place had made
  // the plan's warp pass 1.9 times the batched calls' time). d_lists is the
  // device array by n that the grouped kernel reads.
  struct PlanList {
    int n = 0;
    unsigned char *head = nullptr, *buf = nullptr;
    long long cap = 0;
  };
  std::vector<PlanList> lists;
  lufqhe::mixed::FacList *d_lists = nullptr;
  // its pending FP64 refactorisations (n = 24..32) and their pass's launch
  lufqhe::PendEntry *d_pend = nullptr;
  unsigned int *d_pend_count = nullptr;
  unsigned int pend_cap = 0;
  int pend_nmax = 0, pend_ctas = 0;
  size_t pend_smem = 0;
};

namespace {

// Pass of group g: 2 for an FP64-route group with n >= kFp64GroupMinN, 1 for
// a mixed plan's other FP64-only groups, else 0.
int pass_of(const lufqhe_plan_s *p, size_t g) {
  const bool fp64 = p->mode != LUFQHE_MODE_MIXED || p->share[g] >= 65536u;
  if (fp64 && p->groups[g].n >= kFp64GroupMinN) return 2;
  if (p->mode == LUFQHE_MODE_MIXED && fp64) return 1;
  return p->mode == LUFQHE_MODE_MIXED && p->groups[g].n <= kSmallPassMaxN ? 3 : 0;
}

int build_items(lufqhe_plan_s *p, cudaStream_t s) {
  std::vector<int> order(p->groups.size());
  for (size_t i = 0; i < order.size(); ++i) order[i] = (int)i;
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int b) { return p->groups[a].n > p->groups[b].n; });
  std::vector<WorkItem> items[kPlanPasses];
  for (int g : order) {
    const lufqhe_group_t &G = p->groups[g];
    const int T = p->tile[g];
    const int pass = pass_of(p, g);
    for (long long f = 0; f < G.count; f += T) {
      WorkItem w;
      w.A = reinterpret_cast<const double2 *>(G.A);
      w.first = f;
      w.out = G.out_offset + f;
      w.count = (int)std::min<long long>(T, G.count - f);
      w.n = G.n;
      w.lda = G.lda;
      const bool fp32_path = pass == 0 || pass == 3;
      w.share64k = p->mode == LUFQHE_MODE_MIXED && fp32_path ? p->share[g] : 0u;
      w.status_or = p->mode == LUFQHE_MODE_MIXED && !fp32_path ? LUFQHE_ST_FP64 : 0;
      items[pass].push_back(w);
    }
  }
  std::vector<WorkItem> all;
  for (int q = 0; q < kPlanPasses; ++q) {
    p->launch[q].first = (int)all.size();
    p->launch[q].nitems = (int)items[q].size();
    all.insert(all.end(), items[q].begin(), items[q].end());
  }
  p->nitems = (int)all.size();
  if (all.size() > p->items_cap) {
    if (p->d_items) cudaFree(p->d_items);
    p->d_items = nullptr;
    int rc = check_cuda(cudaMalloc(&p->d_items, sizeof(WorkItem) * std::max<size_t>(1, all.size())),
                        "cudaMalloc(work items)");
    if (rc) return rc;
    p->items_cap = all.size();
  }
  if (!all.empty()) {
    int rc = check_cuda(cudaMemcpyAsync(p->d_items, all.data(), sizeof(WorkItem) * all.size(),
                                        cudaMemcpyHostToDevice, s),
                        "cudaMemcpyAsync(work items)");
    if (rc) return rc;
  }
  return check_cuda(cudaStreamSynchronize(s), "sync(work items)");
}

// Set up pass `pass` for its groups: layout, shared memory, grid. A pass
// without groups is left empty.
int configure_pass(lufqhe_plan_s *p, int pass, int warps) {
  Launch &L = p->launch[pass];
  L.mode = (pass == 1 || pass == 2) && p->mode == LUFQHE_MODE_MIXED ? LUFQHE_MODE_PLAIN_FP64_FUSED
                                                                    : p->mode;
  L.nm = 0;
  L.nf = 0;
  for (size_t g = 0; g < p->groups.size(); ++g) {
    const lufqhe_group_t &G = p->groups[g];
    if (G.count == 0 || pass_of(p, g) != pass) continue;
    L.nf = std::max(L.nf, G.n);
    if (L.mode == LUFQHE_MODE_MIXED) L.nm = std::max(L.nm, G.n);
    // a mixed plan's FP64 route with corrected sizes: the correction's
    // scratch (the FP32 path's F and ints) in the layout
    if (pass == 1 && p->mode == LUFQHE_MODE_MIXED && G.n >= kCorrectMinN && G.n <= 32)
      L.nm = std::max(L.nm, G.n);
  }
  L.warps = warps;
  L.ctas = 0;
  L.smem = 0;
  if (L.nf == 0) return LUFQHE_SUCCESS;
  if (pass == 2) {
    // one matrix per CTA of kFp64GroupWarps warps; a mixed plan's results
    // with n <= kCorrectMaxN are corrected (nm: the largest such n, for the
    // correction's scratch)
    if (p->mode == LUFQHE_MODE_MIXED)
      for (size_t g = 0; g < p->groups.size(); ++g)
        if (p->groups[g].count && pass_of(p, g) == 2 && p->groups[g].n <= kCorrectMaxN)
          L.nm = std::max(L.nm, p->groups[g].n);
    GroupedKernel k = group_kernel_for(L.mode, L.nm > 0);
    const size_t smem =
        (size_t)L.nf * (L.nf + 1) * sizeof(double2) + 2 * (size_t)L.nf * sizeof(double) +
        (size_t)L.nm * (L.nm + 1) * sizeof(float2) + 2 * (size_t)L.nm * sizeof(int);
    int rc = check_cuda(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem),
                        "cudaFuncSetAttribute(grouped group)");
    if (rc) return rc;
    int per_sm = 0;
    rc = check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k,
                                                                  kFp64GroupWarps * 32, smem),
                    "occupancy(grouped group)");
    if (rc) return rc;
    if (per_sm < 1) {
      set_error("plan: n=%d needs %zu bytes of shared memory per matrix", L.nf, smem);
      return LUFQHE_ERR_UNSUPPORTED_N;
    }
    L.warps = kFp64GroupWarps;
    L.smem = smem;
    L.ctas = device_sm_count() * per_sm;
    return LUFQHE_SUCCESS;
  }
  GroupedKernel k = kernel_for(L.mode, pass == 3);
  const size_t per_warp = warp_layout(L.nm, L.nf).total;
  const size_t optin = device_smem_optin();
  int w = std::min<int>(warps, (int)(optin / per_warp));
  if (w < 1) {
    set_error("plan: n=%d needs %zu bytes of shared memory per warp; the device offers %zu",
              L.nf, per_warp, optin);
    return LUFQHE_ERR_UNSUPPORTED_N;
  }
  const size_t smem = per_warp * w;
  int rc = check_cuda(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem),
                      "cudaFuncSetAttribute(grouped)");
  if (rc) return rc;
  int per_sm = 0;
  rc = check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, w * 32, smem),
                  "occupancy(grouped)");
  if (rc) return rc;
  if (per_sm < 1) per_sm = 1;
  L.warps = w;
  L.smem = smem;
  L.ctas = device_sm_count() * per_sm;
  return LUFQHE_SUCCESS;
}

int configure_launch(lufqhe_plan_s *p, int warps) {
  int rc = 0;
  for (int pass = 0; pass < kPlanPasses && !rc; ++pass) rc = configure_pass(p, pass, warps);
  return rc;
}

PlanAux aux_of(const lufqhe_plan_s *p) {
  return PlanAux{p->d_lists, p->d_pend, p->d_pend_count, p->pend_cap};
}

int launch_once(lufqhe_plan_s *p, cudaStream_t s) {
  int rc = check_cuda(cudaMemsetAsync(p->d_counter, 0, kPlanPasses * sizeof(unsigned int), s),
                      "memset(counter)");
  for (const auto &l : p->lists)
    if (!rc) rc = check_cuda(cudaMemsetAsync(l.head, 0, head_bytes(), s), "memset(list head)");
  if (!rc && p->d_pend_count)
    rc = check_cuda(cudaMemsetAsync(p->d_pend_count, 0, sizeof(unsigned int), s),
                    "memset(pending count)");
  for (int pass = 0; pass < kPlanPasses && !rc; ++pass) {
    const Launch &L = p->launch[pass];
    if (L.nitems == 0 || L.ctas == 0) continue;
    GroupedKernel k =
        pass == 2 ? group_kernel_for(L.mode, L.nm > 0) : kernel_for(L.mode, pass == 3);
    // a warp-group CTA takes one item at a time
    const long long want = pass == 2 ? L.nitems : (L.nitems + L.warps - 1) / L.warps;
    const int grid = (int)std::min<long long>(L.ctas, want);
    static const char *names[kPlanPasses] = {"grouped_kernel", "grouped_kernel_fp64",
                                             "grouped_group_kernel", "grouped_kernel_small"};
    KernelTimer timer(names[pass], L.nf, s);
    k<<<std::max(1, grid), L.warps * 32, L.smem, s>>>(p->d_items + L.first, L.nitems,
                                                       p->d_counter + pass, L.nm, L.nf, p->theta2,
                                                       p->refine,
                                                       p->logabs, p->phase, p->parity, p->status,
                                                       aux_of(p));
    timer.stop();
    rc = check_cuda(cudaGetLastError(), "grouped_kernel launch");
  }
  if (!rc && p->pend_cap) {
    KernelTimer timer("grouped_pending_kernel", p->pend_nmax, s);
    grouped_pending_kernel<<<p->pend_ctas, kPendWarps * 32, p->pend_smem, s>>>(
        aux_of(p), p->pend_nmax, p->logabs, p->phase, p->parity, p->status);
    timer.stop();
    rc = check_cuda(cudaGetLastError(), "grouped_pending_kernel launch");
  }
  for (const auto &l : p->lists)
    if (!rc)
      rc = launch_listed_corrections(l.n, l.head, l.buf, l.cap, p->logabs, p->phase, p->parity,
                                     p->status, s);
  return rc;
}

// A mixed plan's factor lists: for n = 24 and 32, room for kPlanListShare of
// the plan's matrices of that size (the FP32 path rejects 4-5% of n = 24 and
// ~18% of n = 32 LLL matrices); a factorisation beyond it is corrected in
// place by its warp.
constexpr double kPlanListShare = 0.3;

int alloc_lists(lufqhe_plan_s *p) {
  if (p->mode != LUFQHE_MODE_MIXED) return LUFQHE_SUCCESS;
  std::vector<mixed::FacList> host(kListMaxN + 1, mixed::FacList{nullptr, nullptr, 0, 0});
  for (int n : {24, 32}) {
    long long count = 0;
    for (const auto &G : p->groups)
      if (G.n == n) count += G.count;
    const long long cap = (long long)std::ceil(kPlanListShare * (double)count);
    if (cap < 1) continue;
    lufqhe_plan_s::PlanList l;
    l.n = n;
    l.cap = cap;
    int rc = check_cuda(cudaMalloc(&l.head, head_bytes()), "cudaMalloc(list head)");
    if (!rc)
      rc = check_cuda(cudaMalloc(&l.buf, (size_t)cap * mixed::fac_entry_bytes(n, true)),
                      "cudaMalloc(factor list)");
    if (rc) {
      if (l.head) cudaFree(l.head);
      return rc;
    }
    p->lists.push_back(l);
    host[n] = mixed::FacList{
        reinterpret_cast<unsigned long long *>(l.head + listed_count_offset()), l.buf, cap, 1};
  }
  int rc = LUFQHE_SUCCESS;
  if (!p->lists.empty()) {
    rc = check_cuda(cudaMalloc(&p->d_lists, host.size() * sizeof(mixed::FacList)),
                    "cudaMalloc(lists)");
    if (!rc)
      rc = check_cuda(cudaMemcpy(p->d_lists, host.data(), host.size() * sizeof(mixed::FacList),
                                 cudaMemcpyHostToDevice),
                      "copy(lists)");
  }
  // the pending list: room for kPlanListShare of the matrices with
  // kPlanDeferMinN <= n <= 32 (the FP32 path's sizes that defer)
  long long count = 0;
  for (const auto &G : p->groups)
    if (G.n >= kPlanDeferMinN && G.n <= kListMaxN) {
      count += G.count;
      p->pend_nmax = std::max(p->pend_nmax, G.n);
    }
  const long long cap = (long long)std::ceil(kPlanListShare * (double)count);
  if (rc || cap < 1) return rc;
  rc = check_cuda(cudaMalloc(&p->d_pend, (size_t)cap * sizeof(PendEntry)), "cudaMalloc(pending)");
  if (!rc)
    rc = check_cuda(cudaMalloc(&p->d_pend_count, sizeof(unsigned int)), "cudaMalloc(pending count)");
  if (rc) return rc;
  p->pend_smem = kPendWarps * pending_warp_bytes(p->pend_nmax);
  rc = check_cuda(cudaFuncSetAttribute(grouped_pending_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)p->pend_smem),
                  "cudaFuncSetAttribute(pending)");
  int per_sm = 0;
  if (!rc)
    rc = check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                        &per_sm, grouped_pending_kernel, kPendWarps * 32, p->pend_smem),
                    "occupancy(pending)");
  if (rc) return rc;
  p->pend_ctas = device_sm_count() * std::max(1, per_sm);
  p->pend_cap = (unsigned int)cap;
  return LUFQHE_SUCCESS;
}

// Time one launch (ms) after one warm-up launch.
int time_launch(lufqhe_plan_s *p, cudaStream_t s, float *ms) {
  int rc = launch_once(p, s);
  if (rc) return rc;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, s);
  rc = launch_once(p, s);
  cudaEventRecord(e1, s);
  if (!rc) rc = check_cuda(cudaEventSynchronize(e1), "tune sync");
  if (!rc) cudaEventElapsedTime(ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return rc;
}

// Autotuner: per group (alone), the tile size T from {1/4, 1/2, 1, 2, 4} x the
// default; then, for the whole batch, the warps per CTA from {2, 4, 8}.
int autotune(lufqhe_plan_s *p, cudaStream_t s) {
  char line[256];
  p->report = "{\"tiles\": {";
  const std::vector<lufqhe_group_t> all = p->groups;
  std::vector<int> base_tile = p->tile;
  const int all_nmax = p->nmax;
  int rc = configure_launch(p, 4);
  if (rc) return rc;
  std::vector<unsigned int> base_share = p->share;
  for (size_t g = 0; g < all.size(); ++g) {
    if (all[g].count == 0) continue;
    p->groups.assign(1, all[g]);
    p->nmax = all[g].n;
    float best = 1e30f;
    int best_t = base_tile[g];
    unsigned int best_s = base_share[g];
    // precision policy: the default FP64 share, half, or everything in FP64
    std::vector<unsigned int> shares = {base_share[g]};
    if (p->mode == LUFQHE_MODE_MIXED) {
      if (base_share[g] != 32768u) shares.push_back(32768u);
      shares.push_back(65536u);
    }
    for (unsigned int sh : shares) {
      for (double f : {0.25, 0.5, 1.0, 2.0, 4.0}) {
        int T = std::max(1, std::min(1024, (int)std::lround(base_tile[g] * f)));
        p->tile.assign(1, T);
        p->share.assign(1, sh);
        rc = configure_launch(p, 4);
        if (rc) return rc;
        rc = build_items(p, s);
        if (rc) return rc;
        float ms = 0.0f;
        rc = time_launch(p, s, &ms);
        if (rc) return rc;
        if (ms < best) {
          best = ms;
          best_t = T;
          best_s = sh;
        }
      }
    }
    base_tile[g] = best_t;
    base_share[g] = best_s;
    snprintf(line, sizeof(line),
             "%s\"%d\": {\"tile\": %d, \"fp64_share\": %.3f, \"ms_alone\": %.4f, \"count\": %lld}",
             g ? ", " : "", all[g].n, best_t, best_s / 65536.0, best, all[g].count);
    p->report += line;
  }
  p->share = base_share;
  p->groups = all;
  p->tile = base_tile;
  p->nmax = all_nmax;
  rc = build_items(p, s);
  if (rc) return rc;
  float best = 1e30f;
  int best_w = 4;
  p->report += "}, \"warps\": {";
  bool first = true;
  for (int w : {2, 4, 8}) {
    rc = configure_launch(p, w);
    if (rc) return rc;
    if (p->launch[0].warps != w && p->launch[1].warps != w && p->launch[3].warps != w)
      continue;  // does not fit
    float ms = 0.0f;
    rc = time_launch(p, s, &ms);
    if (rc) return rc;
    snprintf(line, sizeof(line), "%s\"%d\": %.4f", first ? "" : ", ", w, ms);
    first = false;
    p->report += line;
    if (ms < best) {
      best = ms;
      best_w = w;
    }
  }
  rc = configure_launch(p, best_w);
  if (rc) return rc;
  snprintf(line, sizeof(line),
           "}, \"chosen_warps\": %d, \"ctas\": %d, \"fp64_pass_ctas\": %d, "
           "\"group_pass_ctas\": %d, \"small_pass_ctas\": %d}",
           p->launch[0].warps, p->launch[0].ctas, p->launch[1].ctas, p->launch[2].ctas,
           p->launch[3].ctas);
  p->report += line;
  return LUFQHE_SUCCESS;
}

int capture_graph(lufqhe_plan_s *p) {
  if (p->exec) {
    cudaGraphExecDestroy(p->exec);
    p->exec = nullptr;
  }
  if (p->graph) {
    cudaGraphDestroy(p->graph);
    p->graph = nullptr;
  }
  int rc = check_cuda(cudaStreamBeginCapture(p->cap_stream, cudaStreamCaptureModeThreadLocal),
                      "cudaStreamBeginCapture");
  if (rc) return rc;
  int lrc = launch_once(p, p->cap_stream);
  rc = check_cuda(cudaStreamEndCapture(p->cap_stream, &p->graph), "cudaStreamEndCapture");
  if (lrc) return lrc;
  if (rc) return rc;
  return check_cuda(cudaGraphInstantiate(&p->exec, p->graph, 0), "cudaGraphInstantiate");
}

void destroy_plan(lufqhe_plan_s *p) {
  if (!p) return;
  if (p->exec) cudaGraphExecDestroy(p->exec);
  if (p->graph) cudaGraphDestroy(p->graph);
  if (p->d_items) cudaFree(p->d_items);
  if (p->d_counter) cudaFree(p->d_counter);
  for (const auto &l : p->lists) {
    cudaFree(l.head);
    cudaFree(l.buf);
  }
  if (p->d_lists) cudaFree(p->d_lists);
  if (p->d_pend) cudaFree(p->d_pend);
  if (p->d_pend_count) cudaFree(p->d_pend_count);
  if (p->cap_stream) cudaStreamDestroy(p->cap_stream);
  delete p;
}

}  // namespace

namespace lufqhe {
extern float g_mixed_theta;
extern int g_mixed_refine;
}

extern "C" int lufqhe_plan_create(lufqhe_plan_t **plan, const lufqhe_group_t *groups, int ngroups,
                                  int mode, double *d_logabs, double *d_phase, int8_t *d_parity,
                                  int32_t *d_status, int flags, void *stream) {
  if (!plan || (ngroups > 0 && !groups) || ngroups < 0 || !d_logabs) {
    set_error("lufqhe_plan_create: invalid argument");
    return LUFQHE_ERR_INVALID_ARG;
  }
  if (mode != LUFQHE_MODE_PLAIN_FP64 && mode != LUFQHE_MODE_PLAIN_FP64_FUSED &&
      mode != LUFQHE_MODE_MIXED) {
    set_error("lufqhe_plan_create: unknown mode %d", mode);
    return LUFQHE_ERR_UNSUPPORTED_MODE;
  }
  *plan = nullptr;
  lufqhe_plan_s *p = new lufqhe_plan_s();
  p->mode = mode;
  // outputs and inputs may be page-locked host memory: kernels use its device view
  p->logabs = static_cast<double *>(const_cast<void *>(device_address(d_logabs)));
  p->phase = static_cast<double *>(const_cast<void *>(device_address(d_phase)));
  p->parity = static_cast<int8_t *>(const_cast<void *>(device_address(d_parity)));
  p->status = static_cast<int32_t *>(const_cast<void *>(device_address(d_status)));
  p->theta2 = g_mixed_theta * g_mixed_theta;
  p->refine = g_mixed_refine;
  for (int g = 0; g < ngroups; ++g) {
    const lufqhe_group_t &G = groups[g];
    if (G.count < 0 || G.n < 1 || G.lda < G.n || G.out_offset < 0 || (G.count > 0 && !G.A) ||
        (reinterpret_cast<uintptr_t>(G.A) & 15) != 0) {
      set_error("lufqhe_plan_create: group %d is invalid", g);
      delete p;
      return LUFQHE_ERR_INVALID_ARG;
    }
    if (G.n > LUFQHE_MAX_N) {
      set_error("lufqhe_plan_create: group %d has n=%d > %d", g, G.n, LUFQHE_MAX_N);
      delete p;
      return LUFQHE_ERR_UNSUPPORTED_N;
    }
    p->groups.push_back(G);
    p->groups.back().A = device_address(G.A);
    p->tile.push_back(default_tile(G.n));
    // the per-n FP64 share of the batched mixed kernels
    p->share.push_back(fp64_share_64k(G.n));
    p->nmax = std::max(p->nmax, G.n);
    p->total += G.count;
  }
  cudaStream_t s = (cudaStream_t)stream;
  int rc = check_cuda(cudaStreamCreateWithFlags(&p->cap_stream, cudaStreamNonBlocking),
                      "cudaStreamCreate(plan)");
  if (!rc)
    rc = check_cuda(cudaMalloc(&p->d_counter, kPlanPasses * sizeof(unsigned int)),
                    "cudaMalloc(counter)");
  if (!rc) rc = check_cuda(cudaStreamSynchronize(s), "sync(plan inputs)");
  if (!rc) rc = alloc_lists(p);
  if (!rc && (flags & LUFQHE_PLAN_AUTOTUNE) && p->total > 0) rc = autotune(p, p->cap_stream);
  if (!rc) rc = build_items(p, p->cap_stream);
  if (!rc && !(flags & LUFQHE_PLAN_AUTOTUNE)) {
    rc = configure_launch(p, 4);
    char line[160];
    snprintf(line, sizeof(line), "{\"tiles\": \"default\", \"chosen_warps\": %d, \"ctas\": %d}",
             p->launch[0].warps, p->launch[0].ctas);
    p->report = line;
  }
  if (!rc) rc = capture_graph(p);
  if (rc) {
    destroy_plan(p);
    return rc;
  }
  *plan = p;
  return LUFQHE_SUCCESS;
}

extern "C" int lufqhe_plan_execute(lufqhe_plan_t *plan, void *stream) {
  if (!plan || !plan->exec) {
    set_error("lufqhe_plan_execute: invalid plan");
    return LUFQHE_ERR_INVALID_ARG;
  }
  return check_cuda(cudaGraphLaunch(plan->exec, (cudaStream_t)stream), "cudaGraphLaunch");
}

extern "C" int lufqhe_plan_launch_direct(lufqhe_plan_t *plan, void *stream) {
  if (!plan) {
    set_error("lufqhe_plan_launch_direct: invalid plan");
    return LUFQHE_ERR_INVALID_ARG;
  }
  return launch_once(plan, (cudaStream_t)stream);
}

extern "C" int lufqhe_plan_describe(const lufqhe_plan_t *plan, char *buf, size_t len) {
  if (!plan || !buf || len == 0) {
    set_error("lufqhe_plan_describe: invalid argument");
    return LUFQHE_ERR_INVALID_ARG;
  }
  // the report is one JSON object: add the kernels one execution launches
  // the pending and correction passes
  int kernels = (int)plan->lists.size() + (plan->pend_cap ? 1 : 0);
  for (const Launch &L : plan->launch) kernels += (L.nitems > 0 && L.ctas > 0) ? 1 : 0;
  std::string r = plan->report;
  const size_t close = r.rfind('}');
  if (close != std::string::npos)
    r.insert(close, std::string(r.size() > 2 ? ", " : "") + "\"kernels\": " +
                        std::to_string(kernels));
  snprintf(buf, len, "%s", r.c_str());
  return LUFQHE_SUCCESS;
}

extern "C" int lufqhe_plan_destroy(lufqhe_plan_t *plan) {
  destroy_plan(plan);
  return LUFQHE_SUCCESS;
}
