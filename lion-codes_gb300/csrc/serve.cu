// Serving: device-resident Monte Carlo walkers and a persistent request loop.
//
// A walker is k matrices of one size n (the Slater-type matrices of one
// Monte Carlo configuration set) that stay in HBM for its whole life. A move
// resamples particle i of every matrix: the host sends only the k new z_i and
// the GPU rebuilds row i (M_ik = z^k exp(-|z|^2/4)) in place, then recomputes
// the k determinants. Walkers are admitted against an HBM byte budget.
//
// Each size class (n) has its own persistent kernel on its own stream, sized
// to a share of the SMs, so all classes are resident at once. A request
// (one move of one walker) is cut into tiles of matrices; the host appends the
// tiles to the class's ring in mapped host memory and publishes them with a
// release store. Warps of the class kernel claim published tile indices one
// at a time, process the tile and count it against its request; the warp that finishes a request's last tile
// writes the request's completion flag to mapped host memory. Tiles of
// different requests are in flight at the same time on different warps: new
// requests are admitted as soon as ring slots and HBM free up, without waiting
// for a batch boundary.
//
// A warp claims only a published index (compare-and-swap on the class's claim
// counter while it is below the published count), so a warp that leaves the
// loop never strands a tile. Every device wait is bounded: when no warp of the
// class has claimed a tile for kIdleNs (a class-wide timestamp), the warps
// leave together and the kernel exits; the host relaunches it, continuing
// from the claim counter, the next time it publishes work or polls a request
// of that class.

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <mutex>
#include <random>
#include <thread>
#include <vector>

#include "mixed_core.cuh"
#include "serve_moves.cuh"

namespace lufqhe {

namespace {

using namespace mixed;

// Moves kept per matrix between refactorisations (the O(n^2) move path)
constexpr int kMoveK = 8;
// With moves on by size (option 8 = 2, the default), the classes that keep
// factors: on the orbital matrices of the serving workload the moves' error
// estimate refuses most moves at n >= 32 (their conditioning), where a
// refactorisation is then as fast or faster (measured closed-loop capacity
// per class: n = 8 8.1M moves vs 7.4M refactorising, n = 16 12.0M vs 10.7M,
// n = 32 4.1M vs 8.9M, n = 64 1.0M vs 1.4M dets/s)
constexpr int kMovesAutoMaxN = 16;

constexpr unsigned kRing = 1u << 16;                  // tiles per class ring
constexpr unsigned long long kIdleNs = 200000000ull;  // 0.2 s without a claim
// Warps per class CTA (its register budget follows from it). Every class CTA
// asks for more than half of an SM's shared memory, so exactly one CTA of any
// class fits on an SM: with the class shares summing to the SM count, all
// class loops are resident together however the scheduler places them.
constexpr int serve_max_warps(int n) { return n <= 8 ? 16 : n <= 16 ? 12 : n <= 32 ? 8 : 4; }

struct ServeTile {
  double2 *mats;             // first matrix of the tile (device)
  double2 *z;                // its particle coordinates (device, n per matrix)
  const double2 *znew;       // new coordinate of `particle` per matrix (mapped host), or null
  double *logabs;            // outputs for the tile's first matrix (mapped host)
  double *phase;
  int32_t *status;
  unsigned int *req_done;    // tiles finished, per request slot (device)
  unsigned int *completion;  // request completion flag (mapped host)
  unsigned int seq;          // value stored into *completion
  unsigned int req_tiles;
  int count;
  int particle;
  int build;                 // 1: build every row from z first (a walker's first request)
  int moves;                 // 1: O(n^2) moves against kept factors (the arrays below)
  // per-matrix move arrays of the tile's first matrix (serve_moves.cuh)
  double2 *lu;               // n x n each
  int *perm;                 // n each
  double2 *w, *v;            // kMoveK x n each
  double2 *cap;              // kMoveK x kMoveK each (inverse capacitance)
  MoveState *mst;
};

struct ClassCtl {                // device memory, one per class
  unsigned int claimed;          // tiles claimed so far (see claim_tile)
  unsigned int exited;           // warps that left the loop
  unsigned long long last_ns;    // %globaltimer of the class's latest claim
  unsigned int pub_seen;         // device mirror of the host's published count
  unsigned int ahead;            // adds that claimed a tile not yet published (see claim_tile)
  unsigned long long moved;      // moves taken by the O(n^2) path
  unsigned long long refactored; // moves that refactorised instead
  double move_tol;               // the moves' error bound
};

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ unsigned int ld_acquire_sys(const unsigned int *p) {
  unsigned int v;
  asm volatile("ld.acquire.sys.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_sys(unsigned int *p, unsigned int v) {
  asm volatile("st.release.sys.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned int ld_acquire_gpu(const unsigned int *p) {
  unsigned int v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Claim the next published tile of a class (one thread): a compare-and-swap
// on the claim counter while it is below the published count. Returns false
// when the class has had no claim for kIdleNs or the server is stopping.
// The host's published count lives in mapped host memory, and every read of
// it crosses the host link: thousands of idle warps reading it in a loop had
// saturated that link and slowed every tile's own host-memory traffic. So
// the count is mirrored in device memory (ctl->pub_seen): a claim looks at the
// mirror first, and only when the mirror shows nothing to claim does the
// thread read the host count (acquire) and raise the mirror (after a fence, so
// a tile claimed through the mirror is ordered after the host's writes of it).
// Idle threads back off exponentially between host reads, up to ~8 us.
// Under a deep backlog (the mirror at least `backlog_add` tiles ahead of the
// claims, twice the class's claimers) a tile is claimed with an add instead.
// Every successful swap costs its contenders about one L2 round trip, so a
// class claiming only by swaps topped out near 1.3M tiles/s, below the n = 32
// and n = 64 classes' rates at one matrix per tile; an add always succeeds.
// Between its reads and its add a claimer waits less than any tile takes to
// process, so each other claimer adds at most once in that window and the
// add lands below the published count. Should it land above (ctl->ahead
// counts those), the claimer keeps the tile and waits for its publication.
__device__ bool wait_published(const unsigned int *published, const unsigned int *stop,
                               ClassCtl *ctl, unsigned int t);

__device__ bool claim_tile(const unsigned int *published, const unsigned int *stop, ClassCtl *ctl,
                           unsigned int backlog_add, unsigned int &idx) {
  const unsigned long long t0 = global_ns();
  volatile unsigned int *claimed = &ctl->claimed;
  unsigned int backoff = 128;
  for (;;) {
    const unsigned int c = *claimed;
    const unsigned int p = ld_acquire_gpu(&ctl->pub_seen);
    if ((int)(p - c) > 0) {
      if (p - c >= backlog_add) {
        const unsigned int t = atomicAdd(&ctl->claimed, 1u);
        atomicMax(&ctl->last_ns, global_ns());
        idx = t;
        if ((int)(p - t) > 0) return true;
        atomicAdd(&ctl->ahead, 1u);
        return wait_published(published, stop, ctl, t);
      }
      if (atomicCAS(&ctl->claimed, c, c + 1u) == c) {
        idx = c;
        atomicMax(&ctl->last_ns, global_ns());
        return true;
      }
      continue;
    }
    const unsigned int ph = ld_acquire_sys(published);
    if ((int)(ph - p) > 0) {
      __threadfence();
      unsigned int old = p;
      while ((int)(ph - old) > 0) {  // raise the mirror (wrap-safe)
        const unsigned int prev = atomicCAS(&ctl->pub_seen, old, ph);
        if (prev == old) break;
        old = prev;
      }
      backoff = 128;
      continue;
    }
    if (ld_acquire_sys(stop)) return false;
    const unsigned long long now = global_ns();
    const unsigned long long last = *(volatile unsigned long long *)&ctl->last_ns;
    if (now - (last > t0 ? last : t0) > kIdleNs) return false;
    __nanosleep(backoff);
    backoff = backoff < 8192u ? 2u * backoff : 8192u;
  }
}


// A tile claimed by an add ahead of its publication: wait until the host has
// published it (raising the mirror as claim_tile does). Bounded: the server
// stopping, or kTicketWaitNs without the publication, gives up; the tile is
// then never processed and its request's poll times out on the host.
constexpr unsigned long long kTicketWaitNs = 10000000000ull;  // 10 s

__device__ bool wait_published(const unsigned int *published, const unsigned int *stop,
                               ClassCtl *ctl, unsigned int t) {
  const unsigned long long t0 = global_ns();
  unsigned int backoff = 128;
  for (;;) {
    const unsigned int p = ld_acquire_gpu(&ctl->pub_seen);
    if ((int)(p - t) > 0) return true;
    const unsigned int ph = ld_acquire_sys(published);
    if ((int)(ph - p) > 0) {
      __threadfence();
      unsigned int old = p;
      while ((int)(ph - old) > 0) {  // raise the mirror (wrap-safe)
        const unsigned int prev = atomicCAS(&ctl->pub_seen, old, ph);
        if (prev == old) break;
        old = prev;
      }
      continue;
    }
    if (ld_acquire_sys(stop) || global_ns() - t0 > kTicketWaitNs) return false;
    __nanosleep(backoff);
    backoff = backoff < 8192u ? 2u * backoff : 8192u;
  }
}

// Apply the move to the tile's matrices: z_particle <- znew, then rebuild that
// row (lane j handles matrix j); with t.build every row of every matrix is
// built from z instead (lanes over rows), which is how a walker's matrices are
// first made, inside the loop so no other kernel needs an SM. With t.moves the
// row is left to the move path, which needs the old row too.
__device__ void apply_move(const ServeTile &t, int n, int lane) {
  if (t.particle >= 0 && t.znew) {
    for (int j0 = 0; j0 < t.count; j0 += 32) {
      const int j = j0 + lane;
      if (j < t.count) {
        const double2 z = __ldcv(t.znew + j);
        t.z[(size_t)j * n + t.particle] = z;
        if (!t.build && !t.moves)
          lll_row_rn(z, n, t.mats + (size_t)j * n * n + (size_t)t.particle * n);
      }
    }
    __syncwarp();
  }
  if (t.build) {
    for (int j = 0; j < t.count; ++j)
      for (int i = lane; i < n; i += 32)
        lll_row_rn(__ldcg(t.z + (size_t)j * n + i), n, t.mats + (size_t)j * n * n + (size_t)i * n);
  }
  __syncwarp();
  __threadfence_block();
}

// Shared memory per warp: the FP64 matrix (as double2, aliased by the FP32
// path's hi/lo copy) and the row scales come first; the FP32 factor and the
// exponents follow and are left out when every matrix takes the FP64 kernel.
// With moves (every factorisation FP64, its factors kept) the FP32 arrays give
// way to the move path's scratch.
size_t serve_smem_per_warp(int n, bool fp64_only, bool moves) {
  const size_t nl = (size_t)n * (n + 1);
  size_t b = nl * sizeof(float4) + 2 * (size_t)n * sizeof(double);
  if (moves) return b + ((MoveScratch::bytes(n, kMoveK) + 15) & ~(size_t)15);
  if (!fp64_only) b += nl * sizeof(float2) + 2 * (size_t)n * sizeof(int);
  return b;
}

// Matrix j of a tile with moves: its arrays.
__device__ __forceinline__ MoveArrays move_arrays(const ServeTile &t, int n, int j) {
  MoveArrays a;
  a.A = t.mats + (size_t)j * n * n;
  a.LU = t.lu + (size_t)j * n * n;
  a.perm = t.perm + (size_t)j * n;
  a.W = t.w + (size_t)j * kMoveK * n;
  a.V = t.v + (size_t)j * kMoveK * n;
  a.Ci = t.cap + (size_t)j * kMoveK * kMoveK;
  a.st = t.mst + j;
  return a;
}

// The new row of particle i of matrix j (lane 0 builds it; all lanes see it).
__device__ __forceinline__ void move_new_row(const ServeTile &t, int n, int j, double2 *r,
                                             int lane) {
  if (lane == 0) lll_row_rn(__ldcg(t.z + (size_t)j * n + t.particle), n, r);
  __syncwarp();
}

// Outputs of matrix j of a tile: log|det|, wrapped phase, status.
__device__ __forceinline__ void serve_emit(const ServeTile &t, int j, double la, double ph,
                                           int st) {
  t.logabs[j] = la;
  t.phase[j] = (la == la && la > -INFINITY) ? wrap_phase(ph) : ph;
  t.status[j] = st;
}

// FP64 factorisation of the tile's matrix j (already in M) by one warp, keeping
// its factors, pivot order and log-determinant for later moves.
__device__ void refactor_keep_warp(const MoveArrays &a, int n, double2 *M, int lds, double *hold,
                                   int *perm, int lane, double *la, double *ph, int *st) {
  int par = 0;
  *st = lup_fp64_warp<ARITH_FUSED>(M, lds, hold, n, lane, &par, perm);
  if (*st == 0) {
    logdet_from_diag(M, lds, n, lane, par, la, ph);
  } else if (*st == LUFQHE_ST_SINGULAR) {
    *la = -INFINITY;
    *ph = 0.0;
  } else {
    *la = NAN;
    *ph = NAN;
  }
  __syncwarp();
  BlockWalk w(lane, n);
  for (int e = lane; e < n * n; e += 32) {
    a.LU[e] = M[w.i * lds + w.k];
    w.next(n);
  }
  for (int p = lane; p < n; p += 32) a.perm[p] = perm[p];
  if (lane == 0) {
    MoveState s;
    s.la = *st == 0 ? *la : NAN;  // a singular matrix is refactorised again next move
    s.ph = *ph;
    s.m = 0;
    s.pad = 0;
    *a.st = s;
  }
}

template <int NC>
__global__ void __launch_bounds__(serve_max_warps(NC) * 32, 1)
    serve_kernel(const ServeTile *ring, const unsigned int *published, const unsigned int *stop,
                 ClassCtl *ctl, int mode, float theta2, unsigned int share64k, int refine,
                 int moves) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int LDS = NC + 1;
  constexpr size_t NL = (size_t)NC * LDS;
  const int warps = blockDim.x >> 5;
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  unsigned char *base = smem_raw;
  float4 *HL = reinterpret_cast<float4 *>(base) + warp * NL;
  base += warps * NL * sizeof(float4);
  double *hold = reinterpret_cast<double *>(base) + warp * 2 * NC;
  base += warps * 2 * (size_t)NC * sizeof(double);
  // FP32-path arrays: only addressed when some matrix takes the FP32 path
  // (never with moves, whose scratch takes their place)
  float2 *F = reinterpret_cast<float2 *>(base) + warp * NL;
  int *er = reinterpret_cast<int *>(reinterpret_cast<unsigned char *>(base) +
                                    warps * NL * sizeof(float2)) +
            warp * 2 * NC;
  int *ec = er + NC;
  MoveScratch S;
  constexpr size_t kScratch = (MoveScratch::bytes(NC, kMoveK) + 15) & ~(size_t)15;
  S.bind(base + warp * kScratch, NC, kMoveK);
  (void)moves;

  for (;;) {
    // claim the next published tile; give up when the class has been idle
    unsigned int idx = 0;
    int give_up = 0;
    if (lane == 0)
      give_up = claim_tile(published, stop, ctl, 2u * gridDim.x * (unsigned int)warps, idx) ? 0 : 1;
    idx = __shfl_sync(kFull, idx, 0);
    give_up = __shfl_sync(kFull, give_up, 0);
    if (give_up) {
      if (lane == 0) atomicAdd(&ctl->exited, 1u);
      return;
    }
    __syncwarp();  // order every lane's reads after lane 0's acquire
    ServeTile t;
    {
      // the ring lives in mapped host memory: read it uncached, word by word
      const unsigned long long *srcw =
          reinterpret_cast<const unsigned long long *>(ring + (idx % kRing));
      unsigned long long *dstw = reinterpret_cast<unsigned long long *>(&t);
#pragma unroll
      for (int q = 0; q < (int)(sizeof(ServeTile) / 8); ++q) dstw[q] = __ldcv(srcw + q);
    }
    apply_move(t, NC, lane);
    DeferredOut out;
    for (int j = 0; j < t.count; ++j) {
      __syncwarp();
      const double2 *src = t.mats + (size_t)j * NC * NC;
      double2 *M = reinterpret_cast<double2 *>(HL);
      if (t.moves) {
        // O(n^2) move against the kept factors; an FP64 refactorisation (its
        // factors kept) for a walker's first request, a recompute, or a move
        // that fails its checks
        const MoveArrays a = move_arrays(t, NC, j);
        const int flag = mode == LUFQHE_MODE_MIXED ? LUFQHE_ST_FP64 : 0;
        double la = 0.0, ph = 0.0;
        bool done = false;
        if (!t.build && t.particle >= 0) {
          move_new_row(t, NC, j, S.r, lane);
          done = move_warp<kMoveK>(a, NC, t.particle, M, LDS, S, lane, ctl->move_tol, &la,
                                   &ph);
          __syncwarp();
          if (lane == 0) atomicAdd(done ? &ctl->moved : &ctl->refactored, 1ull);
        }
        int st = 0;
        if (!done) {
          if (stage_matrix_checked(M, LDS, src, NC, lane)) {
            st = LUFQHE_ST_NONFINITE;
            la = ph = NAN;
            if (lane == 0) a.st->la = NAN;  // refactorised again by the next move
          } else {
            refactor_keep_warp(a, NC, M, LDS, hold, S.perm, lane, &la, &ph, &st);
            st |= flag;
          }
        } else {
          st = flag;
        }
        if (lane == 0) serve_emit(t, j, la, ph, st);
        continue;
      }
      if (load_matrix_fp64<true>(src, NC, NC, M, LDS, lane)) {
        emit_nonfinite(lane, j, t.logabs, t.phase, nullptr, t.status);
        continue;
      }
      // mixed mode: the per-n precision policy may send the matrix to FP64
      const bool mixed = mode == LUFQHE_MODE_MIXED && !route_fp64<true>(src, share64k);
      if (mixed) {
        CFF prod;
        int exp_sum = 0, par = 0;
        float2 corr;
        bool ok;
        if constexpr (NC <= 32) {
          ok = mixed_factor_tile<NC>(HL, F, er, ec, lane, theta2, prod, exp_sum, corr, par,
                                     refine != 0);
        } else {
          MixedSmem S;
          S.SC = HL;
          S.Af = F;
          S.hold = hold;
          S.er = er;
          S.ec = ec;
          ok = mixed_factor(S, NC, lane, theta2, prod, exp_sum, corr, par);
        }
        if (ok) {
          out.push(lane, j, prod, exp_sum, corr, par, t.logabs, t.phase, nullptr, t.status);
        } else {
          const CorrScratch cs{F, er, hold};
          fallback_fp64<true>(src, NC, NC, M, LDS, hold, lane, j, t.logabs, t.phase, nullptr,
                              t.status, LUFQHE_ST_FALLBACK, &cs);
        }
      } else {
        int par = 0;
        int st = lup_fp64_warp<ARITH_FUSED>(M, LDS, hold, NC, lane, &par);
        double la, ph;
        if (st == 0) {
          logdet_from_diag(M, LDS, NC, lane, par, &la, &ph);
        } else if (st == LUFQHE_ST_SINGULAR) {
          la = -INFINITY;
          ph = 0.0;
        } else {
          la = NAN;
          ph = NAN;
        }
        if (lane == 0) {
          t.logabs[j] = la;
          t.phase[j] = ph;
          t.status[j] = st | (mode == LUFQHE_MODE_MIXED ? LUFQHE_ST_FP64 : 0);
        }
      }
    }
    out.flush(lane, t.logabs, t.phase, nullptr, t.status);
    __threadfence_system();  // each lane's result stores before the count
    __syncwarp();
    if (lane == 0) {
      const unsigned int done = atomicAdd(t.req_done, 1u) + 1u;
      if (done == t.req_tiles) {
        // last tile of the request: re-arm the counter for the slot's next
        // request, then publish completion
        atomicExch(t.req_done, 0u);
        __threadfence_system();
        st_release_sys(t.completion, t.seq);
      }
    }
  }
}

// FP64-only classes with n >= kFp64GroupMinN: the CTA's warps work in groups
// of kFp64GroupWarps. Each group claims tiles like a warp of serve_kernel and
// factorises their matrices one at a time with all its threads
// (lup_fp64_group behind the group's named barrier), as the batched FP64
// kernel does for these sizes: with one warp per n=64 matrix only three warps
// fit in an SM's shared memory and the FP64 pipe starves. Results are
// bit-identical to the warp routine's.
constexpr int kServeGroupsMax = 4;

template <int NC>
__global__ void __launch_bounds__(kServeGroupsMax * kFp64GroupWarps * 32, 1)
    serve_group_kernel(const ServeTile *ring, const unsigned int *published,
                       const unsigned int *stop, ClassCtl *ctl, int mode, float theta2,
                       unsigned int share64k, int refine, int moves) {
  (void)theta2;
  (void)share64k;
  (void)refine;
  (void)moves;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int LDS = NC + 1;
  constexpr size_t NL = (size_t)NC * LDS;
  constexpr int GT = kFp64GroupWarps * 32;  // threads per group
  constexpr int TW = (int)(sizeof(ServeTile) / 8);
  __shared__ long long red_s[kServeGroupsMax][3 * kFp64GroupWarps];
  __shared__ unsigned long long tile_s[kServeGroupsMax][TW];
  __shared__ int go_s[kServeGroupsMax];
  __shared__ int moved_s[kServeGroupsMax];
  const int groups = blockDim.x / GT;
  const int g = threadIdx.x / GT;
  const int tid = threadIdx.x - g * GT, lane = tid & 31;
  double2 *M = reinterpret_cast<double2 *>(smem_raw) + g * NL;
  double *hold =
      reinterpret_cast<double *>(reinterpret_cast<double2 *>(smem_raw) + groups * NL) + g * 2 * NC;
  // the move path's scratch, one per group, after the row scales
  constexpr size_t kScratch = (MoveScratch::bytes(NC, kMoveK) + 15) & ~(size_t)15;
  MoveScratch S;
  S.bind(reinterpret_cast<unsigned char *>(reinterpret_cast<double *>(
             reinterpret_cast<double2 *>(smem_raw) + groups * NL) + groups * 2 * NC) +
             g * kScratch,
         NC, kMoveK);
  const NamedBarrier bar{1 + g, GT};
  for (;;) {
    if (tid == 0) {
      unsigned int idx = 0;
      const bool go =
          claim_tile(published, stop, ctl, 2u * gridDim.x * (unsigned int)groups, idx);
      go_s[g] = go;
      if (go) {
        // the ring lives in mapped host memory: read it uncached, word by word
        const unsigned long long *srcw =
            reinterpret_cast<const unsigned long long *>(ring + (idx % kRing));
#pragma unroll
        for (int q = 0; q < TW; ++q) tile_s[g][q] = __ldcv(srcw + q);
      }
    }
    bar.sync();
    if (!go_s[g]) {
      if (tid == 0) atomicAdd(&ctl->exited, 1u);
      return;
    }
    ServeTile t;
    {
      unsigned long long *dstw = reinterpret_cast<unsigned long long *>(&t);
#pragma unroll
      for (int q = 0; q < TW; ++q) dstw[q] = tile_s[g][q];
    }
    if (tid < 32) apply_move(t, NC, lane);
    for (int j = 0; j < t.count; ++j) {
      bar.sync();  // the move's rows are written; M is free again
      const double2 *src = t.mats + (size_t)j * NC * NC;
      if (t.moves) {
        // one warp of the group tries the O(n^2) move; if it is refused (or
        // this is a walker's first request or a recompute) the group
        // refactorises in FP64 and keeps the factors. Group g moves with its
        // warp g mod 4, so the groups of a CTA move on different SM
        // sub-partitions (warp w runs on sub-partition w mod 4) and their FP64
        // work does not queue on one FP64 unit.
        const MoveArrays a = move_arrays(t, NC, j);
        const int flag = mode == LUFQHE_MODE_MIXED ? LUFQHE_ST_FP64 : 0;
        if ((tid >> 5) == g % kFp64GroupWarps) {
          double la = 0.0, ph = 0.0;
          bool done = false;
          if (!t.build && t.particle >= 0) {
            move_new_row(t, NC, j, S.r, lane);
            done = move_warp<kMoveK>(a, NC, t.particle, M, LDS, S, lane, ctl->move_tol, &la,
                                     &ph);
            if (lane == 0) atomicAdd(done ? &ctl->moved : &ctl->refactored, 1ull);
          }
          if (done && lane == 0) serve_emit(t, j, la, ph, flag);
          if (lane == 0) moved_s[g] = done;
        }
        bar.sync();
        if (moved_s[g]) continue;
        bool bad = false;
        StrideWalk w(tid, GT, NC);
        for (int e = tid; e < NC * NC; e += GT) {
          const double2 v = __ldcg(src + (size_t)w.i * NC + w.k);
          bad |= !finite_c(v);
          M[w.i * LDS + w.k] = v;
          w.next(NC);
        }
        bad = bar.sync_or(bad);
        int par = 0;
        const int st = bad ? LUFQHE_ST_NONFINITE
                           : lup_fp64_group<ARITH_FUSED>(M, LDS, hold, NC, tid, GT, red_s[g], &par,
                                                         bar, S.perm);
        bar.sync();
        StrideWalk w2(tid, GT, NC);
        for (int e = tid; e < NC * NC; e += GT) {
          a.LU[e] = M[w2.i * LDS + w2.k];
          w2.next(NC);
        }
        for (int p = tid; p < NC; p += GT) a.perm[p] = S.perm[p];
        if (tid < 32) {
          double la, ph;
          if (st == 0) {
            logdet_from_diag(M, LDS, NC, lane, par, &la, &ph);
          } else if (st == LUFQHE_ST_SINGULAR) {
            la = -INFINITY;
            ph = 0.0;
          } else {
            la = NAN;
            ph = NAN;
          }
          if (lane == 0) {
            MoveState s;
            s.la = st == 0 ? la : NAN;
            s.ph = ph;
            s.m = 0;
            s.pad = 0;
            *a.st = s;
            serve_emit(t, j, la, ph, bad ? st : st | flag);
          }
        }
        continue;
      }
      bool bad = false;
      StrideWalk w(tid, GT, NC);
      for (int e = tid; e < NC * NC; e += GT) {
        const double2 v = __ldcg(src + (size_t)w.i * NC + w.k);
        bad |= !finite_c(v);
        M[w.i * LDS + w.k] = v;
        w.next(NC);
      }
      bad = bar.sync_or(bad);
      int par = 0;
      const int st = bad ? LUFQHE_ST_NONFINITE
                         : lup_fp64_group<ARITH_FUSED>(M, LDS, hold, NC, tid, GT, red_s[g], &par,
                                                       bar);
      bar.sync();
      if (tid < 32) {
        double la, ph;
        if (st == 0) {
          logdet_from_diag(M, LDS, NC, lane, par, &la, &ph);
        } else if (st == LUFQHE_ST_SINGULAR) {
          la = -INFINITY;
          ph = 0.0;
        } else {
          la = NAN;
          ph = NAN;
        }
        if (tid == 0) {
          t.logabs[j] = la;
          t.phase[j] = ph;
          // a non-finite input carries no route flag, as in serve_kernel
          t.status[j] = bad ? st : st | (mode == LUFQHE_MODE_MIXED ? LUFQHE_ST_FP64 : 0);
        }
      }
    }
    if (tid == 0) {
      __threadfence_system();  // the result stores before the count
      const unsigned int done = atomicAdd(t.req_done, 1u) + 1u;
      if (done == t.req_tiles) {
        atomicExch(t.req_done, 0u);
        __threadfence_system();
        st_release_sys(t.completion, t.seq);
      }
    }
    bar.sync();  // tile_s and go_s are rewritten by the next claim
  }
}

using ServeKernel = void (*)(const ServeTile *, const unsigned int *, const unsigned int *,
                             ClassCtl *, int, float, unsigned int, int, int);

// A walker's block in the HBM pool: its matrices and coordinates, and with
// moves the per-matrix move arrays, each part 256-byte aligned.
struct WalkerLayout {
  size_t mats, z, lu, perm, w, v, cap, mst, total;
  WalkerLayout(int n, int k, bool moves) {
    auto up = [](size_t v) { return (v + 255) & ~(size_t)255; };
    size_t o = 0;
    mats = o;
    o += up((size_t)k * n * n * sizeof(double2));
    z = o;
    o += up((size_t)k * n * sizeof(double2));
    lu = perm = w = v = cap = mst = o;
    if (moves) {
      lu = o;
      o += up((size_t)k * n * n * sizeof(double2));
      perm = o;
      o += up((size_t)k * n * sizeof(int));
      w = o;
      o += up((size_t)k * kMoveK * n * sizeof(double2));
      v = o;
      o += up((size_t)k * kMoveK * n * sizeof(double2));
      cap = o;
      o += up((size_t)k * kMoveK * kMoveK * sizeof(double2));
      mst = o;
      o += up((size_t)k * sizeof(MoveState));
    }
    total = o;
  }
};

ServeKernel serve_group_kernel_for(int n) {
  switch (n) {
    case 64: return serve_group_kernel<64>;
    default: return nullptr;
  }
}

size_t serve_group_smem(int n) {
  return (size_t)n * (n + 1) * sizeof(double2) + 2 * (size_t)n * sizeof(double);
}

ServeKernel serve_kernel_for(int n) {
  switch (n) {
    case 8: return serve_kernel<8>;
    case 16: return serve_kernel<16>;
    case 32: return serve_kernel<32>;
    case 64: return serve_kernel<64>;
    default: return nullptr;
  }
}


// ---- host side -------------------------------------------------------------

constexpr int kReqSlots = 1024;   // requests in flight at once (all classes)

double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

struct Walker {
  bool live = false;
  int n = 0;
  int k = 0;
  int cls = -1;
  size_t offset = 0;     // in the HBM pool
  size_t bytes = 0;
  bool busy = false;     // a move is in flight
  bool built = false;    // matrices made from z by the loop (first request)
};

struct ReqSlot {
  bool used = false;
  int walker = -1;
  int k = 0;
  unsigned int seq = 0;
  unsigned int first_tile = 0, last_tile = 0;
  int cls = -1;
};

struct SClass {
  int n = 0;
  int sms = 0;
  ServeKernel kern = nullptr;
  cudaStream_t stream = nullptr;
  ServeTile *ring_h = nullptr;     // mapped host
  ServeTile *ring_d = nullptr;     // device view of the same memory
  unsigned int *pub_h = nullptr;   // published count (mapped host)
  unsigned int *pub_d = nullptr;
  ClassCtl *ctl = nullptr;         // device
  unsigned int published = 0;     // host copy
  int grid = 0, warps = 1;
  size_t smem = 0;
  bool running = false;
  unsigned int relaunches = 0;
  unsigned int share64k = 0;       // FP64 routing share, fixed at creation
  int moves = 0;                   // this class keeps factors and takes O(n^2) moves
  int tile = 8;                    // matrices per tile (class_tile)
  double last_query = 0.0;         // when the loop was last seen running (host clock)
};

// Matrices per tile of class n: the server's tile for n <= 16, fewer above so
// that a tile holds no more factorisation work (n^3) than `tile` matrices of
// n = 16 (one at n = 32 and 64 for the default 8). A warp (or warp group)
// works through its tile's matrices one after another, so at n = 32 a tile of
// 8 kept a request of 8 matrices on one warp for 8 serial factorisations
// (~1.5 ms); with one matrix per tile they run side by side. The cost is in
// claims: each tile is a compare-and-swap on the class's claim counter, and a
// class tops out near 1.3M claims/s (about one L2 round trip per successful
// swap among its contenders), below the n = 32 class's factorisation rate on
// the whole GPU but above what its share of the SMs takes in a mix.
int class_tile(int tile, int n) {
  const long long scaled = (long long)tile * 4096 / ((long long)n * n * n);
  return (int)std::max(1LL, std::min((long long)tile, scaled));
}

}  // namespace
}  // namespace lufqhe

using namespace lufqhe;

struct lufqhe_server_s {
  int mode = LUFQHE_MODE_MIXED;
  int max_k = 4096;
  int tile = 8;
  float theta2 = 0.01f;
  int refine = 1;  // in-place refinement of the tile path (option 5)
  int moves = 0;   // O(n^2) moves: 0 off, 1 every class, 2 classes n <= kMovesAutoMaxN (option 8)
  std::vector<SClass> classes;
  // HBM pool with a first-fit free list
  unsigned char *pool = nullptr;
  size_t pool_bytes = 0;
  std::vector<std::pair<size_t, size_t>> free_list;  // (offset, bytes), sorted by offset
  std::vector<Walker> walkers;
  // request slots: staging (mapped host) and results (mapped host)
  double2 *znew_h = nullptr, *znew_d = nullptr;        // kReqSlots * max_k
  double *la_h = nullptr, *la_d = nullptr;
  double *ph_h = nullptr, *ph_d = nullptr;
  int32_t *st_h = nullptr, *st_d = nullptr;
  unsigned int *comp_h = nullptr, *comp_d = nullptr;   // completion flags (mapped)
  unsigned int *req_done = nullptr;                    // device counters
  unsigned int *stop_h = nullptr, *stop_d = nullptr;
  cudaStream_t setup = nullptr;   // walker uploads (the class streams hold the loops)
  std::vector<ReqSlot> slots;
  unsigned int next_seq = 1;
  long long next_ticket = 1;
  std::mutex mu;
};

namespace {

int pool_alloc(lufqhe_server_s *s, size_t bytes, size_t *off) {
  bytes = (bytes + 255) & ~(size_t)255;
  for (size_t i = 0; i < s->free_list.size(); ++i) {
    if (s->free_list[i].second >= bytes) {
      *off = s->free_list[i].first;
      s->free_list[i].first += bytes;
      s->free_list[i].second -= bytes;
      if (s->free_list[i].second == 0) s->free_list.erase(s->free_list.begin() + i);
      return LUFQHE_SUCCESS;
    }
  }
  return LUFQHE_ERR_BUSY;
}

void pool_free(lufqhe_server_s *s, size_t off, size_t bytes) {
  bytes = (bytes + 255) & ~(size_t)255;
  auto it = std::lower_bound(s->free_list.begin(), s->free_list.end(),
                             std::make_pair(off, (size_t)0));
  it = s->free_list.insert(it, {off, bytes});
  // coalesce with neighbours
  size_t i = it - s->free_list.begin();
  if (i + 1 < s->free_list.size() &&
      s->free_list[i].first + s->free_list[i].second == s->free_list[i + 1].first) {
    s->free_list[i].second += s->free_list[i + 1].second;
    s->free_list.erase(s->free_list.begin() + i + 1);
  }
  if (i > 0 && s->free_list[i - 1].first + s->free_list[i - 1].second == s->free_list[i].first) {
    s->free_list[i - 1].second += s->free_list[i].second;
    s->free_list.erase(s->free_list.begin() + i);
  }
}

int class_index(lufqhe_server_s *s, int n) {
  for (size_t c = 0; c < s->classes.size(); ++c)
    if (s->classes[c].n == n) return (int)c;
  return -1;
}

// (Re)launch a class kernel if it is not running.
// A running loop exits only after kIdleNs without a claim, so while it has
// been seen running within the last kQueryGapS its stream is not queried again
// (a driver call per submit and poll had capped a server at a few thousand
// requests per second); a tile published in the race with an exit waits at
// most that long for the relaunch.
constexpr double kQueryGapS = 1e-3;

int ensure_running(lufqhe_server_s *s, SClass &c) {
  if (c.running) {
    const double t = now_s();
    if (t - c.last_query < kQueryGapS) return LUFQHE_SUCCESS;
    c.last_query = t;
    cudaError_t q = cudaStreamQuery(c.stream);
    if (q == cudaErrorNotReady) return LUFQHE_SUCCESS;
    c.running = false;
    if (q != cudaSuccess) return check_cuda(q, "serve kernel");
  }
  // every claimed tile was processed before its warp left, so the new loop
  // continues from the claim counter as it stands
  // (the shared memory of an FP64-only class holds no FP32 arrays, so the
  // share is the one fixed when the class was created)
  c.kern<<<c.grid, c.warps * 32, c.smem, c.stream>>>(c.ring_d, c.pub_d, s->stop_d, c.ctl, s->mode,
                                                     s->theta2, c.share64k, s->refine, c.moves);
  int rc = check_cuda(cudaGetLastError(), "serve kernel launch");
  if (rc) return rc;
  c.running = true;
  c.last_query = now_s();
  ++c.relaunches;
  return LUFQHE_SUCCESS;
}

void destroy_server(lufqhe_server_s *s) {
  if (!s) return;
  if (s->stop_h) __atomic_store_n(s->stop_h, 1u, __ATOMIC_RELEASE);
  for (auto &c : s->classes) {
    if (c.stream) {
      cudaStreamSynchronize(c.stream);
      cudaStreamDestroy(c.stream);
    }
    if (c.ring_h) cudaFreeHost(c.ring_h);
    if (c.pub_h) cudaFreeHost(c.pub_h);
    if (c.ctl) cudaFree(c.ctl);
  }
  if (s->pool) cudaFree(s->pool);
  if (s->znew_h) cudaFreeHost(s->znew_h);
  if (s->la_h) cudaFreeHost(s->la_h);
  if (s->ph_h) cudaFreeHost(s->ph_h);
  if (s->st_h) cudaFreeHost(s->st_h);
  if (s->comp_h) cudaFreeHost(s->comp_h);
  if (s->stop_h) cudaFreeHost(s->stop_h);
  if (s->req_done) cudaFree(s->req_done);
  if (s->setup) cudaStreamDestroy(s->setup);
  delete s;
}

template <typename T>
int host_mapped(T **h, T **d, size_t count, const char *what) {
  int rc = check_cuda(cudaHostAlloc((void **)h, sizeof(T) * count, cudaHostAllocMapped), what);
  if (rc) return rc;
  memset(*h, 0, sizeof(T) * count);
  return check_cuda(cudaHostGetDevicePointer((void **)d, *h, 0), what);
}

}  // namespace

namespace lufqhe {
extern float g_mixed_theta;
extern int g_mixed_refine;
extern int g_serve_moves;
extern double g_move_tol;
}

extern "C" int lufqhe_server_create(lufqhe_server_t **server, size_t hbm_budget_bytes, int mode,
                                    const int *class_n, const int *class_sms, int nclasses,
                                    int max_k, int tile) {
  if (!server || nclasses < 1 || !class_n || max_k < 1 || tile < 1 || hbm_budget_bytes == 0) {
    set_error("lufqhe_server_create: invalid argument");
    return LUFQHE_ERR_INVALID_ARG;
  }
  if (mode != LUFQHE_MODE_MIXED && mode != LUFQHE_MODE_PLAIN_FP64_FUSED) {
    set_error("lufqhe_server_create: mode must be MIXED or PLAIN_FP64_FUSED");
    return LUFQHE_ERR_UNSUPPORTED_MODE;
  }
  *server = nullptr;
  lufqhe_server_s *s = new lufqhe_server_s();
  s->mode = mode;
  s->max_k = max_k;
  s->tile = tile;
  s->theta2 = g_mixed_theta * g_mixed_theta;
  s->refine = g_mixed_refine;
  s->moves = g_serve_moves;
  s->slots.resize(kReqSlots);
  int rc = LUFQHE_SUCCESS;
  const int sms = device_sm_count();
  int sms_left = sms;
  for (int c = 0; c < nclasses && !rc; ++c) {
    SClass sc;
    sc.n = class_n[c];
    sc.kern = serve_kernel_for(sc.n);
    if (!sc.kern) {
      set_error("lufqhe_server_create: class n=%d not offered (8, 16, 32, 64)", sc.n);
      rc = LUFQHE_ERR_UNSUPPORTED_N;
      break;
    }
    int want = class_sms ? class_sms[c] : std::max(1, sms / nclasses);
    sc.sms = std::max(1, std::min(want, sms_left - (nclasses - 1 - c)));
    sms_left -= sc.sms;
    sc.share64k = mode == LUFQHE_MODE_MIXED ? fp64_share_64k(sc.n) : 0u;
    // with moves every factorisation is FP64 (its factors are kept)
    sc.moves = s->moves == 1 || (s->moves == 2 && sc.n <= kMovesAutoMaxN);
    sc.tile = class_tile(tile, sc.n);
    if ((max_k + sc.tile - 1) / sc.tile > (int)kRing) {
      set_error("lufqhe_server_create: max_k=%d needs more than the %u tiles of class n=%d's ring",
                max_k, kRing, sc.n);
      rc = LUFQHE_ERR_INVALID_ARG;
      break;
    }
    const bool fp64_only = mode != LUFQHE_MODE_MIXED || sc.share64k >= 65536u || sc.moves;
    const size_t optin = device_smem_optin();
    size_t used = 0;
    if (fp64_only && serve_group_kernel_for(sc.n)) {
      // warp groups, one matrix each
      sc.kern = serve_group_kernel_for(sc.n);
      const size_t per_group = serve_group_smem(sc.n) +
                               ((MoveScratch::bytes(sc.n, kMoveK) + 15) & ~(size_t)15);
      const int groups = std::min<int>(kServeGroupsMax, (int)((optin - 4096) / per_group));
      if (groups < 1) {
        set_error("lufqhe_server_create: n=%d needs %zu bytes of shared memory per matrix", sc.n,
                  per_group);
        rc = LUFQHE_ERR_UNSUPPORTED_N;
        break;
      }
      sc.warps = groups * kFp64GroupWarps;
      used = per_group * groups;
    } else {
      const size_t per_warp = serve_smem_per_warp(sc.n, fp64_only, sc.moves != 0);
      sc.warps = std::max(1, std::min<int>(serve_max_warps(sc.n), (int)(optin / per_warp)));
      if (per_warp * sc.warps > optin) {
        set_error("lufqhe_server_create: n=%d needs %zu bytes of shared memory per warp", sc.n,
                  per_warp);
        rc = LUFQHE_ERR_UNSUPPORTED_N;
        break;
      }
      used = per_warp * sc.warps;
    }
    // above half the SM's shared memory: one class CTA per SM
    sc.smem = std::max(used, optin / 2 + 1024);
    rc = check_cuda(cudaFuncSetAttribute(sc.kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)sc.smem),
                    "cudaFuncSetAttribute(serve)");
    if (rc) break;
    int per_sm = 0;
    rc = check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sc.kern, sc.warps * 32,
                                                                  sc.smem),
                    "occupancy(serve)");
    if (rc) break;
    sc.grid = std::max(1, sc.sms * std::max(1, per_sm));
    rc = check_cuda(cudaStreamCreateWithFlags(&sc.stream, cudaStreamNonBlocking), "serve stream");
    if (!rc) rc = host_mapped(&sc.ring_h, &sc.ring_d, kRing, "serve ring");
    if (!rc) rc = host_mapped(&sc.pub_h, &sc.pub_d, 1, "serve published");
    if (!rc) rc = check_cuda(cudaMalloc(&sc.ctl, sizeof(ClassCtl)), "serve ctl");
    if (!rc) {
      ClassCtl z{};
      z.move_tol = g_move_tol;
      rc = check_cuda(cudaMemcpy(sc.ctl, &z, sizeof(z), cudaMemcpyHostToDevice), "serve ctl init");
    }
    s->classes.push_back(sc);
  }
  if (!rc) rc = check_cuda(cudaMalloc(&s->pool, hbm_budget_bytes), "cudaMalloc(walker pool)");
  if (!rc) {
    s->pool_bytes = hbm_budget_bytes;
    s->free_list.push_back({0, hbm_budget_bytes});
  }
  const size_t slot_elems = (size_t)kReqSlots * max_k;
  if (!rc) rc = host_mapped(&s->znew_h, &s->znew_d, slot_elems, "serve staging");
  if (!rc) rc = host_mapped(&s->la_h, &s->la_d, slot_elems, "serve logabs");
  if (!rc) rc = host_mapped(&s->ph_h, &s->ph_d, slot_elems, "serve phase");
  if (!rc) rc = host_mapped(&s->st_h, &s->st_d, slot_elems, "serve status");
  if (!rc) rc = host_mapped(&s->comp_h, &s->comp_d, kReqSlots, "serve completion");
  if (!rc) rc = host_mapped(&s->stop_h, &s->stop_d, 1, "serve stop");
  if (!rc) rc = check_cuda(cudaMalloc(&s->req_done, sizeof(unsigned int) * kReqSlots), "req_done");
  if (!rc) rc = check_cuda(cudaMemset(s->req_done, 0, sizeof(unsigned int) * kReqSlots), "req_done");
  if (!rc) rc = check_cuda(cudaStreamCreateWithFlags(&s->setup, cudaStreamNonBlocking), "setup stream");
  if (!rc) rc = check_cuda(cudaDeviceSynchronize(), "serve init");
  if (rc) {
    destroy_server(s);
    return rc;
  }
  *server = s;
  return LUFQHE_SUCCESS;
}

extern "C" int lufqhe_server_walker_create(lufqhe_server_t *s, int n, int k, const double *z_host,
                                           int *walker_id) {
  if (!s || !z_host || !walker_id || k < 1 || k > s->max_k) {
    set_error("lufqhe_server_walker_create: invalid argument (k must be 1..%d)", s ? s->max_k : 0);
    return LUFQHE_ERR_INVALID_ARG;
  }
  std::lock_guard<std::mutex> lock(s->mu);
  const int cls = class_index(s, n);
  if (cls < 0) {
    set_error("lufqhe_server_walker_create: no class for n=%d", n);
    return LUFQHE_ERR_UNSUPPORTED_N;
  }
  const WalkerLayout lay(n, k, s->classes[cls].moves != 0);
  const size_t bytes = lay.total;
  size_t off = 0;
  if (pool_alloc(s, bytes, &off) != LUFQHE_SUCCESS) {
    set_error("lufqhe_server_walker_create: HBM budget exhausted (%zu bytes needed)", bytes);
    return LUFQHE_ERR_BUSY;
  }
  int id = -1;
  for (size_t w = 0; w < s->walkers.size(); ++w)
    if (!s->walkers[w].live) {
      id = (int)w;
      break;
    }
  if (id < 0) {
    id = (int)s->walkers.size();
    s->walkers.emplace_back();
  }
  Walker &W = s->walkers[id];
  W.live = true;
  W.n = n;
  W.k = k;
  W.cls = cls;
  W.offset = off;
  W.bytes = bytes;
  W.busy = false;
  W.built = false;
  double2 *z = reinterpret_cast<double2 *>(s->pool + off + lay.z);
  // only the coordinates cross now (copy engine); the matrices are built by
  // the class loop when the walker's first request runs
  cudaStream_t st = s->setup;
  int rc = check_cuda(cudaMemcpyAsync(z, z_host, (size_t)k * n * sizeof(double2),
                                      cudaMemcpyHostToDevice, st),
                      "walker z upload");
  if (!rc) rc = check_cuda(cudaStreamSynchronize(st), "walker z upload");
  if (rc) {
    pool_free(s, off, bytes);
    W.live = false;
    return rc;
  }
  *walker_id = id;
  return LUFQHE_SUCCESS;
}

extern "C" int lufqhe_server_walker_destroy(lufqhe_server_t *s, int walker_id) {
  if (!s) return LUFQHE_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lock(s->mu);
  if (walker_id < 0 || walker_id >= (int)s->walkers.size() || !s->walkers[walker_id].live) {
    set_error("lufqhe_server_walker_destroy: unknown walker %d", walker_id);
    return LUFQHE_ERR_INVALID_ARG;
  }
  Walker &W = s->walkers[walker_id];
  if (W.busy) {
    set_error("lufqhe_server_walker_destroy: walker %d has a move in flight", walker_id);
    return LUFQHE_ERR_BUSY;
  }
  pool_free(s, W.offset, W.bytes);
  W.live = false;
  return LUFQHE_SUCCESS;
}

extern "C" int lufqhe_server_submit(lufqhe_server_t *s, int walker_id, int particle,
                                    const double *znew_host, long long *ticket) {
  if (!s || !ticket) return LUFQHE_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lock(s->mu);
  if (walker_id < 0 || walker_id >= (int)s->walkers.size() || !s->walkers[walker_id].live) {
    set_error("lufqhe_server_submit: unknown walker %d", walker_id);
    return LUFQHE_ERR_INVALID_ARG;
  }
  Walker &W = s->walkers[walker_id];
  if (W.busy) {
    set_error("lufqhe_server_submit: walker %d already has a move in flight", walker_id);
    return LUFQHE_ERR_BUSY;
  }
  if (particle >= W.n || (particle >= 0 && !znew_host)) {
    set_error("lufqhe_server_submit: bad particle %d", particle);
    return LUFQHE_ERR_INVALID_ARG;
  }
  // a free request slot
  int slot = -1;
  for (int r = 0; r < kReqSlots; ++r)
    if (!s->slots[r].used) {
      slot = r;
      break;
    }
  if (slot < 0) {
    set_error("lufqhe_server_submit: all %d request slots in flight", kReqSlots);
    return LUFQHE_ERR_BUSY;
  }
  SClass &C = s->classes[W.cls];
  const unsigned int ntiles = (unsigned int)((W.k + C.tile - 1) / C.tile);
  if (ntiles > kRing) {
    set_error("lufqhe_server_submit: %u tiles exceed the class ring (%u)", ntiles, kRing);
    return LUFQHE_ERR_INVALID_ARG;
  }
  // ring space: tiles of the oldest in-flight request of this class bound the reuse
  unsigned int oldest = C.published;
  for (int r = 0; r < kReqSlots; ++r)
    if (s->slots[r].used && s->slots[r].cls == W.cls) oldest = std::min(oldest, s->slots[r].first_tile);
  if (C.published + ntiles - oldest > kRing) {
    set_error("lufqhe_server_submit: tile ring of class n=%d is full", W.n);
    return LUFQHE_ERR_BUSY;
  }
  const size_t sbase = (size_t)slot * s->max_k;
  if (particle >= 0) memcpy(s->znew_h + sbase, znew_host, sizeof(double2) * W.k);
  ReqSlot &R = s->slots[slot];
  R.used = true;
  R.walker = walker_id;
  R.k = W.k;
  R.cls = W.cls;
  R.seq = s->next_seq++;
  if (s->next_seq == 0) s->next_seq = 1;
  R.first_tile = C.published;
  R.last_tile = C.published + ntiles;
  __atomic_store_n(&s->comp_h[slot], 0u, __ATOMIC_RELAXED);
  const WalkerLayout lay(W.n, W.k, s->classes[W.cls].moves != 0);
  unsigned char *blk = s->pool + W.offset;
  double2 *mats = reinterpret_cast<double2 *>(blk + lay.mats);
  double2 *z = reinterpret_cast<double2 *>(blk + lay.z);
  for (unsigned int t = 0; t < ntiles; ++t) {
    const int first = (int)t * C.tile;
    ServeTile T;
    T.moves = s->classes[W.cls].moves;
    T.lu = reinterpret_cast<double2 *>(blk + lay.lu) + (size_t)first * W.n * W.n;
    T.perm = reinterpret_cast<int *>(blk + lay.perm) + (size_t)first * W.n;
    T.w = reinterpret_cast<double2 *>(blk + lay.w) + (size_t)first * kMoveK * W.n;
    T.v = reinterpret_cast<double2 *>(blk + lay.v) + (size_t)first * kMoveK * W.n;
    T.cap = reinterpret_cast<double2 *>(blk + lay.cap) + (size_t)first * kMoveK * kMoveK;
    T.mst = reinterpret_cast<MoveState *>(blk + lay.mst) + first;
    T.mats = mats + (size_t)first * W.n * W.n;
    T.z = z + (size_t)first * W.n;
    T.znew = particle >= 0 ? s->znew_d + sbase + first : nullptr;
    T.logabs = s->la_d + sbase + first;
    T.phase = s->ph_d + sbase + first;
    T.status = s->st_d + sbase + first;
    T.req_done = s->req_done + slot;
    T.completion = s->comp_d + slot;
    T.seq = R.seq;
    T.req_tiles = ntiles;
    T.count = std::min(C.tile, W.k - first);
    T.particle = particle;
    T.build = W.built ? 0 : 1;
    s->classes[W.cls].ring_h[(C.published + t) % kRing] = T;
  }
  std::atomic_thread_fence(std::memory_order_seq_cst);
  C.published += ntiles;
  __atomic_store_n(C.pub_h, C.published, __ATOMIC_RELEASE);
  int rc = ensure_running(s, C);
  if (rc) return rc;
  W.busy = true;
  W.built = true;
  *ticket = ((long long)R.seq << 16) | slot;
  return LUFQHE_SUCCESS;
}

// 0 = done (results copied if pointers given), LUFQHE_ERR_BUSY = not yet,
// LUFQHE_ERR_TIMEOUT = not done within wait_us.
extern "C" int lufqhe_server_poll(lufqhe_server_t *s, long long ticket, int wait_us,
                                  double *logabs, double *phase, int32_t *status) {
  if (!s) return LUFQHE_ERR_INVALID_ARG;
  const int slot = (int)(ticket & 0xffff);
  const unsigned int seq = (unsigned int)(ticket >> 16);
  if (slot < 0 || slot >= kReqSlots) return LUFQHE_ERR_INVALID_ARG;
  const double t0 = now_s();
  int spins = 0;
  for (;;) {
    if (__atomic_load_n(&s->comp_h[slot], __ATOMIC_ACQUIRE) == seq) break;
    // a class loop that gave up while idle (racing a publish) is relaunched
    if ((spins++ & 255) == 0) {
      std::lock_guard<std::mutex> lock(s->mu);
      ReqSlot &R = s->slots[slot];
      if (R.used && R.seq == seq) {
        int rc = ensure_running(s, s->classes[R.cls]);
        if (rc) return rc;
      }
    }
    if (wait_us == 0) return LUFQHE_ERR_BUSY;
    if ((now_s() - t0) * 1e6 > wait_us) return LUFQHE_ERR_TIMEOUT;
  }
  std::lock_guard<std::mutex> lock(s->mu);
  ReqSlot &R = s->slots[slot];
  if (!R.used || R.seq != seq) {
    set_error("lufqhe_server_poll: stale ticket");
    return LUFQHE_ERR_INVALID_ARG;
  }
  const size_t sbase = (size_t)slot * s->max_k;
  if (logabs) memcpy(logabs, s->la_h + sbase, sizeof(double) * R.k);
  if (phase) memcpy(phase, s->ph_h + sbase, sizeof(double) * R.k);
  if (status) memcpy(status, s->st_h + sbase, sizeof(int32_t) * R.k);
  s->walkers[R.walker].busy = false;
  R.used = false;
  return LUFQHE_SUCCESS;
}

extern "C" int lufqhe_server_destroy(lufqhe_server_t *s) {
  destroy_server(s);
  return LUFQHE_SUCCESS;
}

extern "C" int lufqhe_server_stats(lufqhe_server_t *s, int class_n, long long *moved,
                                   long long *refactored) {
  if (!s || !moved || !refactored) {
    set_error("lufqhe_server_stats: invalid argument");
    return LUFQHE_ERR_INVALID_ARG;
  }
  std::lock_guard<std::mutex> lock(s->mu);
  *moved = *refactored = 0;
  for (SClass &c : s->classes) {
    if (class_n > 0 && c.n != class_n) continue;
    ClassCtl ctl{};
    // a plain copy: the class loop keeps running on its own (non-blocking) stream
    const int rc = check_cuda(cudaMemcpy(&ctl, c.ctl, sizeof(ctl), cudaMemcpyDeviceToHost),
                              "server stats");
    if (rc) return rc;
    *moved += (long long)ctl.moved;
    *refactored += (long long)ctl.refactored;
  }
  return LUFQHE_SUCCESS;
}

namespace {
// Walker shapes for the simulated clients: n uniform over the server's
// classes, k log-uniform in [k_min, k_max], from a generator of their own and
// taken in order, a shape staying next until a walker of it is admitted. The
// clients' other draws (particles, coordinates, arrival binding) depend on
// timing, and the shapes of the walkers a window sees set the determinants it
// asks for, so every run sees the same sequence.
struct WalkerShapes {
  struct Shape {
    int n, k;
  };
  WalkerShapes(const lufqhe_server_s *srv, unsigned long long seed, int kmin, int kmax)
      : s(srv), rng(seed ^ 0x5deece66dull), k_min(kmin), k_max(kmax) {}
  Shape peek() {
    if (!have) {
      const int nclass = (int)s->classes.size();
      next.n = s->classes[(int)(uni(rng) * nclass) % nclass].n;
      const double lk = std::log((double)k_min) +
                        uni(rng) * (std::log((double)k_max + 1.0) - std::log((double)k_min));
      next.k = std::max(k_min, std::min(k_max, (int)std::floor(std::exp(lk))));
      have = true;
    }
    return next;
  }
  void take() { have = false; }

 private:
  const lufqhe_server_s *s;
  std::mt19937_64 rng;
  std::uniform_real_distribution<double> uni{0.0, 1.0};
  int k_min, k_max;
  Shape next{0, 0};
  bool have = false;
};
}  // namespace

// Simulated Monte Carlo walker stream (Poisson arrivals of move requests).
// Walkers: k log-uniform in [k_min, k_max], n uniform over the server's
// classes; each makes `moves` single-particle moves; a request arrives at the
// Poisson schedule time (rate `rate_hz`) or, if its walker's previous move is
// still running, when that move completes. Walkers are admitted against the HBM
// budget (a walker that does not fit waits for one to finish). Per request the
// latency from its arrival to its completion is written to lat_us (capacity
// max_records), and the request's n and k to rec_n and rec_k (either may be
// null). Returns the number recorded;
// *elapsed_s gets the wall time and *matrices the determinants computed.
extern "C" long long lufqhe_server_run_stream(lufqhe_server_t *s, double rate_hz,
                                              long long nrequests, int moves, int k_min, int k_max,
                                              unsigned long long seed, double *lat_us, int *rec_n,
                                              int *rec_k, long long max_records, double *elapsed_s,
                                              long long *matrices) {
  if (!s || rate_hz <= 0 || nrequests < 1 || moves < 1 || k_min < 1 || k_max < k_min ||
      k_max > s->max_k) {
    set_error("lufqhe_server_run_stream: invalid argument");
    return LUFQHE_ERR_INVALID_ARG;
  }
  std::mt19937_64 rng(seed);
  WalkerShapes shapes(s, seed, k_min, k_max);
  std::exponential_distribution<double> gap(rate_hz);
  std::uniform_real_distribution<double> uni(0.0, 1.0);
  std::normal_distribution<double> gauss(0.0, 1.0);
  struct Active {
    int id;
    int n, k;
    int moves_left;
    long long ticket;
    double arrival;
    bool in_flight;
  };
  std::vector<Active> act;
  const int nclass = (int)s->classes.size();
  // The client's coordinates come from tables of Gaussian draws made before
  // the clock starts (one per class, scaled by its sigma, in page-locked
  // memory), read at a rolling offset: drawing up to 2 k n normals per new
  // walker inside the loop took milliseconds of host time and delayed every
  // other request's submission and completion polling.
  const size_t kTable = (size_t)1 << 20;
  std::vector<double *> table(nclass, nullptr);
  std::vector<size_t> table_off(nclass, 0);
  auto release_tables = [&] {
    for (double *t : table)
      if (t) cudaFreeHost(t);
  };
  for (int c = 0; c < nclass; ++c) {
    int rc = check_cuda(cudaMallocHost((void **)&table[c], kTable * sizeof(double)),
                        "run_stream tables");
    if (rc) {
      release_tables();
      return rc;
    }
    const double sig = std::sqrt((double)s->classes[c].n / 2.0);
    for (size_t i = 0; i < kTable; ++i) table[c][i] = gauss(rng) * sig;
  }
  auto draws = [&](int n, size_t count) -> const double * {
    const int c = class_index(s, n);
    if (table_off[c] + count > kTable) table_off[c] = 0;
    const double *p = table[c] + table_off[c];
    table_off[c] += count;
    return p;
  };
  long long issued = 0, recorded = 0, mats = 0;
  double next_arrival = now_s();
  const double start = next_arrival;
  // pending arrivals not yet bound to a walker (arrival times)
  std::vector<double> pending;
  while (recorded < nrequests) {
    const double t = now_s();
    // arrivals due
    while (issued < nrequests && next_arrival <= t) {
      pending.push_back(next_arrival);
      next_arrival += gap(rng);
      ++issued;
    }
    // bind pending arrivals: to an idle walker with moves left, else a new walker
    for (size_t p = 0; p < pending.size();) {
      int use = -1;
      for (size_t a = 0; a < act.size(); ++a)
        if (!act[a].in_flight && act[a].moves_left > 0) {
          use = (int)a;
          break;
        }
      if (use < 0) {
        const WalkerShapes::Shape sh = shapes.peek();
        int id = -1;
        int rc = lufqhe_server_walker_create(s, sh.n, sh.k, draws(sh.n, (size_t)2 * sh.k * sh.n),
                                             &id);
        if (rc == LUFQHE_ERR_BUSY && act.empty()) {
          release_tables();
          set_error("lufqhe_server_run_stream: the HBM budget admits no walker of n=%d, k=%d",
                    sh.n, sh.k);
          return rc;
        }
        if (rc == LUFQHE_ERR_BUSY) break;  // HBM budget: wait for walkers to finish
        if (rc) {
          release_tables();
          return rc;
        }
        shapes.take();
        act.push_back({id, sh.n, sh.k, moves, 0, 0.0, false});
        use = (int)act.size() - 1;
      }
      Active &A = act[use];
      const int particle = (int)(uni(rng) * A.n) % A.n;
      long long ticket = 0;
      int rc = lufqhe_server_submit(s, A.id, particle, draws(A.n, (size_t)2 * A.k), &ticket);
      if (rc == LUFQHE_ERR_BUSY) break;  // ring or slots full: retry next pass
      if (rc) {
        release_tables();
        return rc;
      }
      A.ticket = ticket;
      A.arrival = pending[p];
      A.in_flight = true;
      pending.erase(pending.begin() + p);
    }
    // completions
    for (size_t a = 0; a < act.size();) {
      Active &A = act[a];
      if (A.in_flight) {
        int rc = lufqhe_server_poll(s, A.ticket, 0, nullptr, nullptr, nullptr);
        if (rc == LUFQHE_SUCCESS) {
          const double done = now_s();
          if (recorded < max_records) {
            lat_us[recorded] = (done - A.arrival) * 1e6;
            if (rec_n) rec_n[recorded] = A.n;
            if (rec_k) rec_k[recorded] = A.k;
          }
          ++recorded;
          mats += A.k;
          A.in_flight = false;
          if (--A.moves_left == 0) {
            rc = lufqhe_server_walker_destroy(s, A.id);
            if (rc) {
              release_tables();
              return rc;
            }
            act.erase(act.begin() + a);
            continue;
          }
        } else if (rc != LUFQHE_ERR_BUSY) {
          release_tables();
          return rc;
        }
      }
      ++a;
    }
  }
  if (elapsed_s) *elapsed_s = now_s() - start;
  if (matrices) *matrices = mats;
  // retire the remaining walkers
  for (auto &A : act) lufqhe_server_walker_destroy(s, A.id);
  release_tables();
  return std::min(recorded, max_records);
}

// Closed-loop walker population: `walkers` walkers (k log-uniform in
// [k_min, k_max], n uniform over the classes) each submit their next move as
// soon as the previous one completes; a walker that has made `moves` moves is
// retired and replaced by a new one, whose first request builds and factorises
// its matrices. The first `walkers` requests (the initial builds) are made
// before the clock starts. Returns the requests completed in the timed part;
// *elapsed_s the wall time and *matrices the determinants. This is the
// server's capacity for the same work mix as the open stream.
extern "C" long long lufqhe_server_run_closed(lufqhe_server_t *s, int walkers, long long nrequests,
                                              int moves, int k_min, int k_max,
                                              unsigned long long seed, double *elapsed_s,
                                              long long *matrices) {
  if (!s || walkers < 1 || nrequests < 1 || moves < 1 || k_min < 1 || k_max < k_min ||
      k_max > s->max_k) {
    set_error("lufqhe_server_run_closed: invalid argument");
    return LUFQHE_ERR_INVALID_ARG;
  }
  std::mt19937_64 rng(seed);
  WalkerShapes shapes(s, seed, k_min, k_max);
  std::uniform_real_distribution<double> uni(0.0, 1.0);
  std::normal_distribution<double> gauss(0.0, 1.0);
  std::vector<double> zbuf;
  auto fill = [&](int n, size_t count) -> const double * {
    zbuf.resize(count);
    const double sig = std::sqrt((double)n / 2.0);
    for (size_t i = 0; i < count; ++i) zbuf[i] = gauss(rng) * sig;
    return zbuf.data();
  };
  // A walker is empty (id < 0), waiting to submit (its build or its next
  // move), or in flight. A submit refused for want of ring space or request
  // slots leaves the walker waiting, and the sweep goes on polling the others:
  // ring space and slots are returned only when their requests are polled, so
  // a client that spun on the refused submit waited for itself.
  struct W {
    int id = -1, n = 0, k = 0, left = 0;
    bool waiting = false, build = false;
    long long ticket = 0;
  };
  std::vector<W> pop(walkers);
  // a new walker (LUFQHE_ERR_BUSY while the HBM budget is spent: tried again
  // on a later sweep, after others have retired)
  auto spawn = [&](W &w) -> int {
    const WalkerShapes::Shape sh = shapes.peek();
    int id = -1;
    const int rc = lufqhe_server_walker_create(s, sh.n, sh.k, fill(sh.n, (size_t)2 * sh.k * sh.n),
                                               &id);
    if (rc) return rc;
    shapes.take();
    w.id = id;
    w.n = sh.n;
    w.k = sh.k;
    w.left = moves;
    w.waiting = true;
    w.build = true;
    return LUFQHE_SUCCESS;
  };
  // one submit attempt: LUFQHE_ERR_BUSY leaves the walker waiting
  auto submit = [&](W &w) -> int {
    const int particle = w.build ? -1 : (int)(uni(rng) * w.n) % w.n;
    const int rc = lufqhe_server_submit(s, w.id, particle,
                                        w.build ? nullptr : fill(w.n, (size_t)2 * w.k), &w.ticket);
    if (rc == LUFQHE_SUCCESS) w.waiting = false;
    return rc;
  };
  // the initial builds, untimed (as many walkers as the budget admits), each
  // polled until it has completed; the first moves go out in the timed loop,
  // which polls every request it submits (first moves submitted here and left
  // unpolled could fill the ring ahead of builds still waiting for space)
  int started = 0;
  for (W &w : pop) {
    const int rc = spawn(w);
    if (rc == LUFQHE_ERR_BUSY) break;
    if (rc) return rc;
    ++started;
  }
  if (started == 0) {
    set_error("lufqhe_server_run_closed: the HBM budget admits no walker");
    return LUFQHE_ERR_BUSY;
  }
  for (int built = 0; built < started;) {
    for (W &w : pop) {
      if (w.id < 0 || !w.build) continue;  // empty, or built
      int rc = LUFQHE_SUCCESS;
      if (w.waiting) {
        rc = submit(w);
        if (rc && rc != LUFQHE_ERR_BUSY) return rc;
        continue;
      }
      rc = lufqhe_server_poll(s, w.ticket, 0, nullptr, nullptr, nullptr);
      if (rc == LUFQHE_ERR_BUSY) continue;
      if (rc) return rc;
      w.build = false;  // built: its first move waits for the clock
      w.waiting = true;
      ++built;
    }
  }
  long long done = 0, mats = 0, issued = started;
  const double start = now_s();
  for (;;) {
    bool live = false, held = false, refused = false;
    for (W &w : pop) {
      int rc = LUFQHE_SUCCESS;
      if (w.id < 0) {
        if (issued >= nrequests) continue;
        live = true;
        rc = spawn(w);
        if (rc == LUFQHE_ERR_BUSY) {
          refused = true;
          continue;
        }
        if (rc) return rc;
        ++issued;  // its build is part of the mix
      }
      held = true;
      live = true;
      if (w.waiting) {
        rc = submit(w);
        if (rc && rc != LUFQHE_ERR_BUSY) return rc;
        continue;
      }
      rc = lufqhe_server_poll(s, w.ticket, 0, nullptr, nullptr, nullptr);
      if (rc == LUFQHE_ERR_BUSY) continue;
      if (rc) return rc;
      ++done;
      mats += w.k;
      w.build = false;
      if (--w.left == 0 || issued >= nrequests) {
        rc = lufqhe_server_walker_destroy(s, w.id);
        w.id = -1;
        if (rc) return rc;
      } else {
        w.waiting = true;
        ++issued;
        rc = submit(w);
        if (rc && rc != LUFQHE_ERR_BUSY) return rc;
      }
    }
    if (refused && !held) {
      const WalkerShapes::Shape sh = shapes.peek();
      set_error("lufqhe_server_run_closed: the HBM budget admits no walker of n=%d, k=%d", sh.n,
                sh.k);
      return LUFQHE_ERR_BUSY;
    }
    if (!live) break;
  }
  if (elapsed_s) *elapsed_s = now_s() - start;
  if (matrices) *matrices = mats;
  return done;
}
