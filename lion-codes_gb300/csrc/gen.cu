// Seeded synthetic inputs: i.i.d. complex Gaussian matrices and
// lowest-Landau-level (LLL) orbital matrices M_ij = z_i^j exp(-|z_i|^2/4).
//
// Every draw comes from a counter-based generator (SplitMix64 finaliser of
// seed-key + counter), so the uniform variates are identical on the host and
// on any device, and independent of the launch shape. Gaussians use
// Box-Muller. The LLL construction stands in for the reference's on-device
// matrix-element builder, which is compiled out (LU-fqhe/src/mkMatrixElements.cu:26-363).

#include <cmath>

#include "lup_fp64.cuh"

namespace lufqhe {

namespace {

// Pair of independent N(0,1) variates for counter `ctr`.
__host__ __device__ inline void gauss2(unsigned long long key, unsigned long long ctr, double *g0,
                                       double *g1) {
  double u1 = uniform01(key, 2 * ctr);
  double u2 = uniform01(key, 2 * ctr + 1);
  double r = sqrt(-2.0 * log(u1));
  double s, c;
#ifdef __CUDA_ARCH__
  sincospi(2.0 * u2, &s, &c);
#else
  s = sin(2.0 * kPi * u2);
  c = cos(2.0 * kPi * u2);
#endif
  *g0 = r * c;
  *g1 = r * s;
}

// Entry (i,k) of Gaussian matrix b: counter b*n*n + i*n + k.
__host__ __device__ inline double2 gauss_entry(unsigned long long key, long long b, int n, int i,
                                               int k, double scale) {
  double g0, g1;
  gauss2(key, (unsigned long long)b * n * n + (unsigned long long)i * n + k, &g0, &g1);
  return make_double2(g0 * scale, g1 * scale);
}

// Particle i of LLL matrix b: counter b*n + i.
__host__ __device__ inline double2 lll_z(unsigned long long key, long long b, int n, int i,
                                         double scale) {
  double g0, g1;
  gauss2(key, (unsigned long long)b * n + i, &g0, &g1);
  return make_double2(g0 * scale, g1 * scale);
}

// Row i of an LLL matrix on the host: M_ik = z^k exp(-|z|^2/4) by repeated
// multiplication, the same steps as the device's lll_row_rn (the host compiler
// may fuse some of them, so host and device agree to rounding, not in bits).
inline void lll_row(double2 z, int n, double2 *row, int stride) {
  double w = exp(-(z.x * z.x + z.y * z.y) * 0.25);
  double px = 1.0, py = 0.0;
  for (int k = 0; k < n; ++k) {
    row[(size_t)k * stride] = make_double2(px * w, py * w);
    double nx = px * z.x - py * z.y;
    double ny = px * z.y + py * z.x;
    px = nx;
    py = ny;
  }
}

__global__ void gen_gaussian_kernel(double2 *A, int n, int lda, long long batch,
                                    unsigned long long key, double scale) {
  long long total = batch * n * n;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    long long b = e / ((long long)n * n);
    int r = (int)(e - b * n * n);
    int i = r / n, k = r - (r / n) * n;
    A[(size_t)b * n * lda + (size_t)i * lda + k] = gauss_entry(key, b, n, i, k, scale);
  }
}

__global__ void gen_lll_kernel(double2 *A, double2 *Z, int n, int lda, long long batch,
                               unsigned long long key, double scale) {
  long long total = batch * n;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    long long b = e / n;
    int i = (int)(e - b * n);
    double2 z = lll_z(key, b, n, i, scale);
    if (Z) Z[e] = z;
    // the same explicitly rounded row as the kernels that build rows from z
    lll_row_rn(z, n, A + (size_t)b * n * lda + (size_t)i * lda);
  }
}

int grid_for(long long work) {
  long long g = (work + 255) / 256;
  long long cap = (long long)device_sm_count() * 8;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (int)g;
}

}  // namespace

}  // namespace lufqhe

using namespace lufqhe;

extern "C" int lufqhe_gen_gaussian(double *d_A, int n, int lda, long long batch,
                                   unsigned long long seed, double sigma, void *stream) {
  if (!d_A || n < 1 || lda < n || batch < 0) {
    set_error("lufqhe_gen_gaussian: bad arguments");
    return LUFQHE_ERR_INVALID_ARG;
  }
  if (batch == 0) return LUFQHE_SUCCESS;
  gen_gaussian_kernel<<<grid_for(batch * n * n), 256, 0, (cudaStream_t)stream>>>(
      reinterpret_cast<double2 *>(d_A), n, lda, batch, seed_key(seed), sigma * sqrt(0.5));
  return check_cuda(cudaGetLastError(), "gen_gaussian_kernel launch");
}

extern "C" int lufqhe_gen_lll(double *d_A, double *d_z, int n, int lda, long long batch,
                              unsigned long long seed, double sigma, void *stream) {
  if (!d_A || n < 1 || lda < n || batch < 0) {
    set_error("lufqhe_gen_lll: bad arguments");
    return LUFQHE_ERR_INVALID_ARG;
  }
  if (batch == 0) return LUFQHE_SUCCESS;
  gen_lll_kernel<<<grid_for(batch * n), 256, 0, (cudaStream_t)stream>>>(
      reinterpret_cast<double2 *>(d_A), reinterpret_cast<double2 *>(d_z), n, lda, batch,
      seed_key(seed), sigma * sqrt(0.5));
  return check_cuda(cudaGetLastError(), "gen_lll_kernel launch");
}

extern "C" int lufqhe_gen_gaussian_host(double *A, int n, int lda, long long batch,
                                        unsigned long long seed, double sigma) {
  if (!A || n < 1 || lda < n || batch < 0) {
    set_error("lufqhe_gen_gaussian_host: bad arguments");
    return LUFQHE_ERR_INVALID_ARG;
  }
  unsigned long long key = seed_key(seed);
  double scale = sigma * sqrt(0.5);
  double2 *M = reinterpret_cast<double2 *>(A);
  for (long long b = 0; b < batch; ++b)
    for (int i = 0; i < n; ++i)
      for (int k = 0; k < n; ++k)
        M[(size_t)b * n * lda + (size_t)i * lda + k] = gauss_entry(key, b, n, i, k, scale);
  return LUFQHE_SUCCESS;
}

extern "C" int lufqhe_gen_lll_host(double *A, double *z, int n, int lda, long long batch,
                                   unsigned long long seed, double sigma) {
  if (!A || n < 1 || lda < n || batch < 0) {
    set_error("lufqhe_gen_lll_host: bad arguments");
    return LUFQHE_ERR_INVALID_ARG;
  }
  unsigned long long key = seed_key(seed);
  double scale = sigma * sqrt(0.5);
  double2 *M = reinterpret_cast<double2 *>(A);
  double2 *Z = reinterpret_cast<double2 *>(z);
  for (long long b = 0; b < batch; ++b)
    for (int i = 0; i < n; ++i) {
      double2 zz = lll_z(key, b, n, i, scale);
      if (Z) Z[(size_t)b * n + i] = zz;
      lll_row(zz, n, M + (size_t)b * n * lda + (size_t)i * lda, 1);
    }
  return LUFQHE_SUCCESS;
}
