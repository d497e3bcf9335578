// Host-side pieces of a multi-device Monte Carlo step, in C so that a C++
// driver needs nothing else: splitting a (mixed-size) batch of independent
// matrices over devices by cost, and combining the devices' wavefunction sums.
//
// The reference splits its batch between GPUs and CPU threads by matrix count
// (LU-fqhe/src/RunInfo.cpp:53, LU-fqhe/src/MonteCarloLoop.cu:141-148) and adds
// the per-rank sums with MPI_Reduce (LU-fqhe/src/MonteCarloLoop.cu:373-392).
// Here the split is weighted by the flops of one n x n LUP, so that shards of
// different sizes finish together, and the sums are combined in log-polar
// form, where the reference's direct products would overflow.

#include <cmath>
#include <vector>

#include "lufqhe_internal.cuh"

namespace {

// Algorithmic flops of one n x n complex LUP (trailing-update complex MACs at
// 8 flops plus the multiplier scalings at 6); at least 1 so n = 1 has a cost.
double lup_cost(int n) {
  const double d = n;
  const double f = 4.0 * (d - 1.0) * d * (2.0 * d - 1.0) / 3.0 + 3.0 * d * (d - 1.0);
  return f > 1.0 ? f : 1.0;
}

}  // namespace

using namespace lufqhe;

extern "C" int lufqhe_combine_log_sums(const double *parts, long long k, double *out) {
  if (k < 0 || !out || (k > 0 && !parts)) {
    set_error("lufqhe_combine_log_sums: invalid argument");
    return LUFQHE_ERR_INVALID_ARG;
  }
  double m = -INFINITY;
  bool nan = false;
  for (long long r = 0; r < k; ++r) {
    const double l = parts[2 * r];
    if (l != l || parts[2 * r + 1] != parts[2 * r + 1]) nan = true;
    else if (l > m) m = l;
  }
  if (nan) {
    out[0] = out[1] = NAN;
    return LUFQHE_SUCCESS;
  }
  if (!(m > -INFINITY)) {  // no part, or every part zero
    out[0] = -INFINITY;
    out[1] = 0.0;
    return LUFQHE_SUCCESS;
  }
  double re = 0.0, im = 0.0;
  for (long long r = 0; r < k; ++r) {
    const double l = parts[2 * r];
    if (l == -INFINITY) continue;
    const double w = std::exp(l - m);
    re += w * std::cos(parts[2 * r + 1]);
    im += w * std::sin(parts[2 * r + 1]);
  }
  out[0] = m + std::log(std::hypot(re, im));
  out[1] = std::atan2(im, re);
  return LUFQHE_SUCCESS;
}

extern "C" int lufqhe_shard_by_cost(const int *n, const long long *count, int ngroups,
                                    int nshards, int pair_aligned, long long *begin,
                                    long long *end) {
  if (ngroups < 0 || nshards < 1 || (ngroups > 0 && (!n || !count || !begin || !end))) {
    set_error("lufqhe_shard_by_cost: invalid argument");
    return LUFQHE_ERR_INVALID_ARG;
  }
  for (int g = 0; g < ngroups; ++g) {
    if (n[g] < 1 || count[g] < 0) {
      set_error("lufqhe_shard_by_cost: group %d has n=%d count=%lld", g, n[g], count[g]);
      return LUFQHE_ERR_INVALID_ARG;
    }
  }
  // cost before each group
  std::vector<double> before(ngroups + 1, 0.0);
  for (int g = 0; g < ngroups; ++g) before[g + 1] = before[g] + (double)count[g] * lup_cost(n[g]);
  const double total = before[ngroups];
  // boundary s (between shard s-1 and s) as (group, index within the group)
  std::vector<int> bg(nshards + 1, 0);
  std::vector<long long> bi(nshards + 1, 0);
  bg[nshards] = ngroups;  // the end
  for (int s = 1; s < nshards; ++s) {
    const double target = total * (double)s / (double)nshards;
    int g = 0;
    while (g < ngroups - 1 && before[g + 1] <= target) ++g;
    long long idx = 0;
    if (ngroups > 0) {
      idx = std::llround((target - before[g]) / lup_cost(n[g]));
      if (pair_aligned) idx &= ~1ll;
      if (idx < 0) idx = 0;
      if (idx > count[g]) idx = count[g];
    }
    // boundaries never move backwards
    if (g < bg[s - 1] || (g == bg[s - 1] && idx < bi[s - 1])) {
      g = bg[s - 1];
      idx = bi[s - 1];
    }
    bg[s] = g;
    bi[s] = idx;
  }
  for (int s = 0; s < nshards; ++s) {
    for (int g = 0; g < ngroups; ++g) {
      // the part of group g between boundary s and boundary s + 1
      long long lo, hi;
      if (g < bg[s]) lo = count[g];
      else if (g == bg[s]) lo = bi[s];
      else lo = 0;
      if (g < bg[s + 1]) hi = count[g];
      else if (g == bg[s + 1]) hi = (s + 1 == nshards) ? count[g] : bi[s + 1];
      else hi = 0;
      if (hi < lo) hi = lo;
      begin[(size_t)s * ngroups + g] = lo;
      end[(size_t)s * ngroups + g] = hi;
    }
  }
  return LUFQHE_SUCCESS;
}
