/*
 * CPU oracle for the batched LUP determinant: TEST INFRASTRUCTURE ONLY.
 *
 * This file is a restatement, in IEEE double precision, of the reference's CPU
 * Crout/LUP determinant `LUCoreCPU::determinant` (LU-fqhe/src/LUCoreCPU.cu:112-267).
 * Only the tests, the smoke check and the CPU-baseline leg of the benchmark may
 * load it; the product library never links or calls it.
 *
 * The reference is float32-only (its __DPREC__ branch does not compile), so the
 * FP64 version is a restatement, not a recompilation. Its steps, each following
 * the cited reference lines:
 *   1. row scale holder[i] = max_j |Re a_ij|                 (LUCoreCPU.cu:145-160)
 *      a scale below 1e-24 makes the reference exit(0)      (LUCoreCPU.cu:158);
 *      here the matrix gets status LUFQHE_ST_SCALE_TINY.
 *   2. Crout upper part u_ij = a_ij - sum_{k<i} l_ik u_kj    (LUCoreCPU.cu:164-182)
 *   3. lower part + pivot search on dum = |Re|/holder[i],
 *      ties to the LAST row (`dum >= big`)                   (LUCoreCPU.cu:189-213)
 *   4. row swap, d = -d, holder[imax] = holder[j]            (LUCoreCPU.cu:216-232)
 *   5. divide the sub-column by the pivot                     (LUCoreCPU.cu:234-251)
 *   6. det = d * prod u_jj                                    (LUCoreCPU.cu:256-265),
 *      returned here as log|det| = sum log|u_jj| and
 *      phase = sum arg(u_jj) + pi*[d<0], wrapped to (-pi, pi].
 *
 * Two arithmetic modes share the algorithm and the pivot rule:
 *   ARITH_LITERAL (0): the reference's operation sequence: complex products as
 *       two roundings then a subtraction, and one division per element by
 *       den = |pivot|^2. Built with -ffp-contract=off so nothing is fused.
 *   ARITH_KERNEL  (1): the exact IEEE operation sequence the GPU kernel uses:
 *       fused multiply-adds for the multiply-subtract, and one correctly
 *       rounded reciprocal of den per column followed by multiplies. With it the
 *       GPU's in-place LU factors can be compared bit for bit.
 * The pivot quotient |Re|/holder is a correctly rounded division in both modes,
 * which is what the kernel's pivot search reproduces exactly.
 *
 * Parity is UNPINNED by the reference: it ships no golden outputs or tests.
 * The restatement is checked against numpy slogdet, closed-form known answers
 * and the reference's own float32 determinant compiled from its sources.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define LUFQHE_ST_SCALE_TINY 1
#define LUFQHE_ST_SINGULAR 2
#define LUFQHE_ST_NONFINITE 4

#define ARITH_LITERAL 0
#define ARITH_KERNEL 1

typedef struct { double x, y; } cplx;

static const double kPi = 3.14159265358979323846;

static double wrap_phase(double ph) {
  double r = fmod(ph, 2.0 * kPi);
  if (r > kPi) r -= 2.0 * kPi;
  if (r <= -kPi) r += 2.0 * kPi;
  return r;
}

/* sum -= l*u, reference operation order (LUCoreCPU.cu:173-177) */
static inline void cmsub_literal(cplx *s, cplx l, cplx u) {
  double tx = l.x * u.x - l.y * u.y;
  double ty = l.y * u.x + l.x * u.y;
  s->x = s->x - tx;
  s->y = s->y - ty;
}

/* sum -= l*u, the kernel's fused operation order */
static inline void cmsub_kernel(cplx *s, cplx l, cplx u) {
  double sx = fma(-l.x, u.x, s->x);
  sx = fma(l.y, u.y, sx);
  double sy = fma(-l.y, u.x, s->y);
  sy = fma(-l.x, u.y, sy);
  s->x = sx;
  s->y = sy;
}

static inline int finite_c(cplx a) { return isfinite(a.x) && isfinite(a.y); }

/*
 * Factor one matrix in place (work is n*n, row stride n). Returns the status;
 * fills *parity (0/1) and, if piv != NULL, piv[j] = imax of step j.
 * On success the diagonal of `work` holds u_jj.
 */
static int factor_one(cplx *work, int n, int arith, double *holder, int *parity_out,
                      int *piv, int *steps_done) {
  int d = 1;
  *steps_done = 0;
  for (int i = 0; i < n * n; ++i)
    if (!finite_c(work[i])) { *parity_out = 0; return LUFQHE_ST_NONFINITE; }

  for (int i = 0; i < n; ++i) {               /* LUCoreCPU.cu:145-160 */
    double big = 0.0;
    for (int j = 0; j < n; ++j) {
      double t = fabs(work[i * n + j].x);
      if (t > big) big = t;
    }
    if (big < 1e-24) { *parity_out = 0; return LUFQHE_ST_SCALE_TINY; }
    holder[i] = big;
  }

  for (int j = 0; j < n; ++j) {
    for (int i = 0; i < j; ++i) {               /* LUCoreCPU.cu:164-182 */
      cplx s = work[i * n + j];
      for (int k = 0; k < i; ++k) {
        if (arith == ARITH_LITERAL) cmsub_literal(&s, work[i * n + k], work[k * n + j]);
        else cmsub_kernel(&s, work[i * n + k], work[k * n + j]);
      }
      work[i * n + j] = s;
    }
    double big = 0.0;
    int imax = j;
    for (int i = j; i < n; ++i) {               /* LUCoreCPU.cu:189-213 */
      cplx s = work[i * n + j];
      for (int k = 0; k < j; ++k) {
        if (arith == ARITH_LITERAL) cmsub_literal(&s, work[i * n + k], work[k * n + j]);
        else cmsub_kernel(&s, work[i * n + k], work[k * n + j]);
      }
      work[i * n + j] = s;
      double dum = fabs(s.x) / holder[i];
      if (dum >= big) { big = dum; imax = i; }
    }
    if (piv) piv[j] = imax;
    if (j != imax) {                            /* LUCoreCPU.cu:216-232 */
      for (int k = 0; k < n; ++k) {
        cplx t = work[imax * n + k];
        work[imax * n + k] = work[j * n + k];
        work[j * n + k] = t;
      }
      d = -d;
      holder[imax] = holder[j];
    }
    cplx p = work[j * n + j];
    *steps_done = j + 1;
    if (p.x == 0.0 && p.y == 0.0) {
      /* exact zero pivot: the reference would divide by zero; stop here */
      *parity_out = d < 0;
      return LUFQHE_ST_SINGULAR;
    }
    if (j != n - 1) {                           /* LUCoreCPU.cu:234-251 */
      if (arith == ARITH_LITERAL) {
        double den = p.x * p.x + p.y * p.y;
        for (int i = j + 1; i < n; ++i) {
          cplx a = work[i * n + j];
          cplx t;
          t.x = (a.x * p.x + a.y * p.y) / den;
          t.y = (a.y * p.x - a.x * p.y) / den;
          work[i * n + j] = t;
        }
      } else {
        double den = fma(p.x, p.x, p.y * p.y);
        double r = 1.0 / den;
        for (int i = j + 1; i < n; ++i) {
          cplx a = work[i * n + j];
          cplx t;
          t.x = fma(a.x, p.x, a.y * p.y) * r;
          t.y = fma(a.y, p.x, -(a.x * p.y)) * r;
          work[i * n + j] = t;
        }
      }
    }
  }
  *parity_out = d < 0;
  return 0;
}

/*
 * Batched FP64 oracle. A: `batch` matrices of complex128 (interleaved re,im),
 * row-major with row stride lda (elements) and matrix stride n*lda, exactly the
 * reference layout (&matrices[i*matSide*loadSize], LUCoreCPU.cu:85).
 * Outputs per matrix: logabs, phase (radians, (-pi,pi], includes the
 * permutation sign), parity (0/1 swaps mod 2), status (flags above).
 * Optional: piv (batch*n ints, imax per step) and factors (batch*n*n complex,
 * the in-place L\U result with row stride n).
 * nthreads <= 0 uses all OpenMP threads. Returns 0, or -1 on bad arguments.
 */
int lufqhe_oracle_lup_det_fp64(const double *A, int n, int lda, long long batch, int arith,
                               double *logabs, double *phase, signed char *parity,
                               int *status, int *piv, double *factors, int nthreads) {
  if (n < 1 || lda < n || batch < 0 || !A || (arith != 0 && arith != 1)) return -1;
#ifdef _OPENMP
  int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel num_threads(nt)
#endif
  {
    cplx *work = (cplx *)malloc(sizeof(cplx) * (size_t)n * n);
    double *holder = (double *)malloc(sizeof(double) * (size_t)n);
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
    for (long long b = 0; b < batch; ++b) {
      const double *src = A + (size_t)b * n * lda * 2;
      for (int i = 0; i < n; ++i)
        memcpy(work + (size_t)i * n, src + (size_t)i * lda * 2, sizeof(cplx) * n);
      int par = 0, steps = 0;
      int st = factor_one(work, n, arith, holder, &par, piv ? piv + (size_t)b * n : NULL, &steps);
      double la, ph;
      if (st == LUFQHE_ST_NONFINITE || st == LUFQHE_ST_SCALE_TINY) {
        la = NAN; ph = NAN;
      } else if (st == LUFQHE_ST_SINGULAR) {
        la = -INFINITY; ph = 0.0;
      } else {
        la = 0.0; ph = 0.0;
        for (int j = 0; j < n; ++j) {           /* LUCoreCPU.cu:256-265 in log-polar form */
          cplx u = work[j * n + j];
          la += log(hypot(u.x, u.y));
          ph += atan2(u.y, u.x);
        }
        if (par) ph += kPi;
        ph = wrap_phase(ph);
      }
      if (piv && steps < n)
        for (int j = steps; j < n; ++j) piv[(size_t)b * n + j] = -1;
      if (logabs) logabs[b] = la;
      if (phase) phase[b] = ph;
      if (parity) parity[b] = (signed char)par;
      if (status) status[b] = st;
      if (factors) memcpy(factors + (size_t)b * n * n * 2, work, sizeof(cplx) * (size_t)n * n);
    }
    free(work);
    free(holder);
  }
  return 0;
}

/* ------------------------------------------------------------------------- */
/* Float32 restatement: the same steps in the reference's own precision, to   */
/* pin the restatement bit for bit against the reference's compiled code.     */
/* Every operation follows LUCoreCPU::determinant (LU-fqhe/src/LUCoreCPU.cu:   */
/* 112-267) in float, in the same order, with nothing fused (this file is     */
/* built with -ffp-contract=off):                                              */
/*   scale  big = max_j fabs(Re a_ij), compared in double with 1e-24 (:145-160) */
/*   Crout  tmp = (l.x u.x - l.y u.y, l.y u.x + l.x u.y); sum -= tmp (:164-205) */
/*   pivot  dum = fabs(sum.x) / holder[i] in float, `dum >= big`    (:207-212) */
/*   swap   rows j <-> imax, d = -d, holder[imax] = holder[j]        (:215-232) */
/*   divide den = p.x p.x + p.y p.y; ((a.x p.x + a.y p.y)/den,                 */
/*          (a.y p.x - a.x p.y)/den)                                 (:234-251) */
/*   det    det = det * u_jj left to right from (1, 0), then d * det (:256-265) */
/* The factors are left in place (pivoted row order) as the reference leaves  */
/* them. A row scale below 1e-24 (where the reference calls exit(0)) gives     */
/* status LUFQHE_ST_SCALE_TINY and det = NaN; an exact zero pivot (where the   */
/* reference divides by zero) is carried through the same IEEE divisions.      */
/* ------------------------------------------------------------------------- */
typedef struct { float x, y; } cplxf;

static int factor_one_f32(cplxf *a, int n, float *holder, int *piv, cplxf *det_out) {
  float d = 1.0f;
  int imax = 0;
  for (int i = 0; i < n; ++i) {
    float big = 0.0f;
    for (int j = 0; j < n; ++j) {
      float t = fabsf(a[i * n + j].x);
      if (t > big) big = t;
    }
    if ((double)big < 1e-24) {
      det_out->x = NAN;
      det_out->y = NAN;
      return LUFQHE_ST_SCALE_TINY;
    }
    holder[i] = big;
  }
  for (int j = 0; j < n; ++j) {
    for (int i = 0; i < j; ++i) {
      cplxf s = a[i * n + j];
      for (int k = 0; k < i; ++k) {
        cplxf l = a[i * n + k], u = a[k * n + j];
        float tx = l.x * u.x - l.y * u.y;
        float ty = l.y * u.x + l.x * u.y;
        s.x = s.x - tx;
        s.y = s.y - ty;
      }
      a[i * n + j] = s;
    }
    float big = 0.0f;
    for (int i = j; i < n; ++i) {
      cplxf s = a[i * n + j];
      for (int k = 0; k < j; ++k) {
        cplxf l = a[i * n + k], u = a[k * n + j];
        float tx = l.x * u.x - l.y * u.y;
        float ty = l.y * u.x + l.x * u.y;
        s.x = s.x - tx;
        s.y = s.y - ty;
      }
      a[i * n + j] = s;
      float dum = fabsf(s.x) / holder[i];
      if (dum >= big) {
        big = dum;
        imax = i;
      }
    }
    if (piv) piv[j] = imax;
    if (j != imax) {
      for (int k = 0; k < n; ++k) {
        cplxf t = a[imax * n + k];
        a[imax * n + k] = a[j * n + k];
        a[j * n + k] = t;
      }
      d = -d;
      holder[imax] = holder[j];
    }
    if (j != n - 1) {
      cplxf p = a[j * n + j];
      for (int i = j + 1; i < n; ++i) {
        float den = p.x * p.x + p.y * p.y;
        cplxf v = a[i * n + j], t;
        t.x = (v.x * p.x + v.y * p.y) / den;
        t.y = (v.y * p.x - v.x * p.y) / den;
        a[i * n + j] = t;
      }
    }
  }
  cplxf det = {1.0f, 0.0f};
  for (int i = 0; i < n; ++i) {
    cplxf u = a[i * n + i], t;
    t.x = det.x * u.x - det.y * u.y;
    t.y = det.y * u.x + det.x * u.y;
    det = t;
  }
  det_out->x = d * det.x;
  det_out->y = d * det.y;
  return 0;
}

/*
 * Batched float32 restatement. A: `batch` complex64 matrices (interleaved
 * floats), row stride lda, matrix stride n*lda. det: one complex64 per matrix
 * (the reference's direct product). Optional: factors (batch*n*n complex64,
 * row stride n, the in-place result), piv (batch*n), status (batch).
 */
int lufqhe_oracle_lup_det_f32(const float *A, int n, int lda, long long batch, float *det,
                              float *factors, int *piv, int *status, int nthreads) {
  if (n < 1 || lda < n || batch < 0 || !A || !det) return -1;
#ifdef _OPENMP
  int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel num_threads(nt)
#endif
  {
    cplxf *work = (cplxf *)malloc(sizeof(cplxf) * (size_t)n * n);
    float *holder = (float *)malloc(sizeof(float) * (size_t)n);
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
    for (long long b = 0; b < batch; ++b) {
      const float *src = A + (size_t)b * n * lda * 2;
      for (int i = 0; i < n; ++i)
        memcpy(work + (size_t)i * n, src + (size_t)i * lda * 2, sizeof(cplxf) * n);
      cplxf dt;
      int st = factor_one_f32(work, n, holder, piv ? piv + (size_t)b * n : NULL, &dt);
      det[2 * b] = dt.x;
      det[2 * b + 1] = dt.y;
      if (status) status[b] = st;
      if (factors) memcpy(factors + (size_t)b * n * n * 2, work, sizeof(cplxf) * (size_t)n * n);
    }
    free(work);
    free(holder);
  }
  return 0;
}

/* ------------------------------------------------------------------------- */
/* Seeded synthetic inputs: the same draws as the library's host generators   */
/* (counter-based SplitMix64 uniforms, Box-Muller Gaussians, lowest-Landau-   */
/* level rows by repeated multiplication), so that the CPU reference arm of   */
/* the benchmark builds its workload without loading the product library.     */
/* Bit-identical to lufqhe_gen_gaussian_host / lufqhe_gen_lll_host (a CPU     */
/* test checks it); both are compiled without floating-point contraction.     */
/* ------------------------------------------------------------------------- */
static uint64_t gen_mix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}
static double gen_uniform01(uint64_t key, uint64_t ctr) {
  uint64_t r = gen_mix64(key + ctr * 0xD2B74407B1CE6E93ull);
  return ((double)(r >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}
static uint64_t gen_seed_key(uint64_t seed) { return gen_mix64(seed ^ 0x5851F42D4C957F2Dull); }
static void gen_gauss2(uint64_t key, uint64_t ctr, double *g0, double *g1) {
  double u1 = gen_uniform01(key, 2 * ctr);
  double u2 = gen_uniform01(key, 2 * ctr + 1);
  double r = sqrt(-2.0 * log(u1));
  double s = sin(2.0 * kPi * u2);
  double c = cos(2.0 * kPi * u2);
  *g0 = r * c;
  *g1 = r * s;
}

/* i.i.d. complex Gaussian entries, Re and Im ~ N(0, sigma^2/2). */
int lufqhe_oracle_gen_gaussian(double *A, int n, int lda, long long batch,
                               unsigned long long seed, double sigma) {
  if (!A || n < 1 || lda < n || batch < 0) return -1;
  uint64_t key = gen_seed_key(seed);
  double scale = sigma * sqrt(0.5);
  for (long long b = 0; b < batch; ++b)
    for (int i = 0; i < n; ++i)
      for (int k = 0; k < n; ++k) {
        double g0, g1;
        gen_gauss2(key, (uint64_t)b * n * n + (uint64_t)i * n + k, &g0, &g1);
        double *e = A + 2 * ((size_t)b * n * lda + (size_t)i * lda + k);
        e[0] = g0 * scale;
        e[1] = g1 * scale;
      }
  return 0;
}

/* M_ik = z_i^k exp(-|z_i|^2/4), z_i complex Gaussian with E|z|^2 = sigma^2
 * (z may be NULL). */
int lufqhe_oracle_gen_lll(double *A, double *z, int n, int lda, long long batch,
                          unsigned long long seed, double sigma) {
  if (!A || n < 1 || lda < n || batch < 0) return -1;
  uint64_t key = gen_seed_key(seed);
  double scale = sigma * sqrt(0.5);
  for (long long b = 0; b < batch; ++b)
    for (int i = 0; i < n; ++i) {
      double g0, g1;
      gen_gauss2(key, (uint64_t)b * n + i, &g0, &g1);
      double zx = g0 * scale, zy = g1 * scale;
      if (z) {
        z[2 * ((size_t)b * n + i)] = zx;
        z[2 * ((size_t)b * n + i) + 1] = zy;
      }
      double w = exp(-(zx * zx + zy * zy) * 0.25);
      double px = 1.0, py = 0.0;
      double *row = A + 2 * ((size_t)b * n * lda + (size_t)i * lda);
      for (int k = 0; k < n; ++k) {
        row[2 * k] = px * w;
        row[2 * k + 1] = py * w;
        double nx = px * zx - py * zy;
        double ny = px * zy + py * zx;
        px = nx;
        py = ny;
      }
    }
  return 0;
}

/* ------------------------------------------------------------------------- */
/* Double-double "truth" oracle. FP64 LU with the reference's |Re| pivot rule  */
/* loses up to ~1e-10 relative in log|det| on ill-conditioned lowest-Landau-   */
/* level matrices, so the error of the mixed-precision path is measured       */
/* against this one: complex LU in double-double (~32 digits) with partial    */
/* pivoting on |Re|+|Im|. It is not a restatement of the reference; it is the */
/* accuracy yardstick for every FP64 and mixed result.                        */
/* ------------------------------------------------------------------------- */
typedef struct { double hi, lo; } dd;

static inline dd dd_two_sum(double a, double b) {
  double s = a + b;
  double bb = s - a;
  double e = (a - (s - bb)) + (b - bb);
  dd r = {s, e};
  return r;
}
static inline dd dd_norm(double hi, double lo) {
  double s = hi + lo;
  double e = lo - (s - hi);
  dd r = {s, e};
  return r;
}
static inline dd dd_add(dd a, dd b) {
  dd s = dd_two_sum(a.hi, b.hi);
  dd t = dd_two_sum(a.lo, b.lo);
  s.lo += t.hi;
  s = dd_norm(s.hi, s.lo);
  s.lo += t.lo;
  return dd_norm(s.hi, s.lo);
}
static inline dd dd_neg(dd a) { dd r = {-a.hi, -a.lo}; return r; }
static inline dd dd_sub(dd a, dd b) { return dd_add(a, dd_neg(b)); }
static inline dd dd_mul(dd a, dd b) {
  double p = a.hi * b.hi;
  double e = fma(a.hi, b.hi, -p);
  e += a.hi * b.lo + a.lo * b.hi;
  return dd_norm(p, e);
}
static inline dd dd_div(dd a, dd b) {
  double q1 = a.hi / b.hi;
  dd r = dd_sub(a, dd_mul((dd){q1, 0.0}, b));
  double q2 = r.hi / b.hi;
  r = dd_sub(r, dd_mul((dd){q2, 0.0}, b));
  double q3 = r.hi / b.hi;
  dd q = dd_norm(q1, q2);
  return dd_add(q, (dd){q3, 0.0});
}
typedef struct { dd x, y; } cdd;
static inline cdd cdd_mul(cdd a, cdd b) {
  cdd r = {dd_sub(dd_mul(a.x, b.x), dd_mul(a.y, b.y)), dd_add(dd_mul(a.x, b.y), dd_mul(a.y, b.x))};
  return r;
}
static inline dd dd_ldexp(dd a, int e) { dd r = {ldexp(a.hi, e), ldexp(a.lo, e)}; return r; }
static inline cdd cdd_div(cdd a, cdd b) {
  /* scale both by 2^-e (exact) so |b|^2 cannot overflow or underflow */
  int e;
  frexp(fmax(fabs(b.x.hi), fabs(b.y.hi)), &e);
  a.x = dd_ldexp(a.x, -e); a.y = dd_ldexp(a.y, -e);
  b.x = dd_ldexp(b.x, -e); b.y = dd_ldexp(b.y, -e);
  dd den = dd_add(dd_mul(b.x, b.x), dd_mul(b.y, b.y));
  dd nx = dd_add(dd_mul(a.x, b.x), dd_mul(a.y, b.y));
  dd ny = dd_sub(dd_mul(a.y, b.x), dd_mul(a.x, b.y));
  cdd r = {dd_div(nx, den), dd_div(ny, den)};
  return r;
}

/*
 * log|det| and phase of each matrix to ~1e-25 relative, same layout as
 * lufqhe_oracle_lup_det_fp64. status: 0, LUFQHE_ST_SINGULAR, LUFQHE_ST_NONFINITE.
 */
int lufqhe_oracle_logdet_dd(const double *A, int n, int lda, long long batch, double *logabs,
                            double *phase, int *status, int nthreads) {
  if (n < 1 || lda < n || batch < 0 || !A) return -1;
#ifdef _OPENMP
  int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel num_threads(nt)
#endif
  {
    cdd *w = (cdd *)malloc(sizeof(cdd) * (size_t)n * n);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 16)
#endif
    for (long long b = 0; b < batch; ++b) {
      const double *src = A + (size_t)b * n * lda * 2;
      int st = 0, sgn = 0;
      for (int i = 0; i < n; ++i)
        for (int k = 0; k < n; ++k) {
          double re = src[(size_t)(i * lda + k) * 2], im = src[(size_t)(i * lda + k) * 2 + 1];
          if (!isfinite(re) || !isfinite(im)) st = LUFQHE_ST_NONFINITE;
          cdd v = {{re, 0.0}, {im, 0.0}};
          w[i * n + k] = v;
        }
      double la = 0.0, ph = 0.0;
      for (int j = 0; j < n && !st; ++j) {
        int p = j;
        double best = -1.0;
        for (int i = j; i < n; ++i) {
          double m = fabs(w[i * n + j].x.hi) + fabs(w[i * n + j].y.hi);
          if (m > best) { best = m; p = i; }
        }
        if (best == 0.0) { st = LUFQHE_ST_SINGULAR; break; }
        if (p != j) {
          for (int k = 0; k < n; ++k) { cdd t = w[p * n + k]; w[p * n + k] = w[j * n + k]; w[j * n + k] = t; }
          sgn ^= 1;
        }
        cdd piv = w[j * n + j];
        for (int i = j + 1; i < n; ++i) {
          cdd l = cdd_div(w[i * n + j], piv);
          for (int k = j + 1; k < n; ++k) {
            cdd t = cdd_mul(l, w[j * n + k]);
            w[i * n + k].x = dd_sub(w[i * n + k].x, t.x);
            w[i * n + k].y = dd_sub(w[i * n + k].y, t.y);
          }
        }
        /* log|u| = 0.5*log(|u|^2) with |u|^2 in dd, split to avoid overflow */
        double sc = fmax(fabs(piv.x.hi), fabs(piv.y.hi));
        int e;
        frexp(sc, &e);
        dd ux = {ldexp(piv.x.hi, -e), ldexp(piv.x.lo, -e)};
        dd uy = {ldexp(piv.y.hi, -e), ldexp(piv.y.lo, -e)};
        dd m2 = dd_add(dd_mul(ux, ux), dd_mul(uy, uy));
        la += 0.5 * (log(m2.hi) + log1p(m2.lo / m2.hi)) + e * 0.69314718055994530942;
        ph += atan2(piv.y.hi + piv.y.lo, piv.x.hi + piv.x.lo);
      }
      if (st == LUFQHE_ST_NONFINITE) { la = NAN; ph = NAN; }
      else if (st == LUFQHE_ST_SINGULAR) { la = -INFINITY; ph = 0.0; }
      else { if (sgn) ph += kPi; ph = wrap_phase(ph); }
      if (logabs) logabs[b] = la;
      if (phase) phase[b] = ph;
      if (status) status[b] = st;
    }
    free(w);
  }
  return 0;
}

/*
 * The reference's pair-product sum (LUCoreCPU::CALL, LU-fqhe/src/LUCoreCPU.cu:82-98):
 * sum over i < batch/2 of det(A_{2i}) * det(A_{2i+1}), an odd last matrix
 * dropped as the reference does (:83). Returned as a complex log-sum-exp
 * (log|sum|, arg sum) so it does not overflow. Uses the literal arithmetic.
 */
int lufqhe_oracle_pair_sum(const double *A, int n, int lda, long long batch, double *log_abs_sum,
                           double *arg_sum, int nthreads) {
  if (batch < 0 || n < 1) return -1;
  long long npair = batch / 2;
  double *la = (double *)malloc(sizeof(double) * (size_t)(2 * npair + 1));
  double *ph = (double *)malloc(sizeof(double) * (size_t)(2 * npair + 1));
  int *st = (int *)malloc(sizeof(int) * (size_t)(2 * npair + 1));
  int rc = lufqhe_oracle_lup_det_fp64(A, n, lda, 2 * npair, ARITH_LITERAL, la, ph, NULL, st, NULL,
                                      NULL, nthreads);
  double mx = -INFINITY;
  for (long long i = 0; i < npair && rc == 0; ++i) {
    double l = la[2 * i] + la[2 * i + 1];
    if (l > mx) mx = l;
  }
  double sx = 0.0, sy = 0.0;
  for (long long i = 0; i < npair && rc == 0; ++i) {
    double l = la[2 * i] + la[2 * i + 1] - mx;
    double p = ph[2 * i] + ph[2 * i + 1];
    double m = exp(l);
    sx += m * cos(p);
    sy += m * sin(p);
  }
  *log_abs_sum = mx + log(hypot(sx, sy));
  *arg_sum = atan2(sy, sx);
  free(la); free(ph); free(st);
  return rc;
}
