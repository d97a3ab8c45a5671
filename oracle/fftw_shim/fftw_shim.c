/*
 * Project-written FFTW3-API stand-in (see fftw3.h). TEST INFRASTRUCTURE ONLY:
 * it exists so the reference C library can be compiled and run as the parity
 * checker on machines without FFTW. Nothing in the product links it.
 *
 * Transforms are unnormalised, FFTW_FORWARD = e^{-2 pi i jk/n}, as FFTW's.
 * Every line of every transform is computed in double: radix-2 iterative
 * Cooley-Tukey for power-of-two lengths, Bluestein's chirp-z convolution
 * (through a power-of-two transform of length >= 2n - 1) for the rest.
 * Plans are immutable after creation, so execution is re-entrant and the
 * reference may call them from many OpenMP threads at once.
 */
#include "fftw3.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
  double re, im;
} cplx;

/* One 1-D complex transform of length n and one direction. */
typedef struct {
  int n;
  int sign;
  int pow2;
  cplx* tw;    /* pow2: e^{sign 2 pi i k / n}, k < n/2 */
  int m;       /* Bluestein: power-of-two convolution length */
  cplx* chirp; /* e^{sign i pi k^2 / n}, k < n */
  cplx* bhat;  /* forward transform of the conjugate chirp, length m */
  cplx* mtw_f; /* forward twiddles of length m */
  cplx* mtw_b; /* backward twiddles of length m */
} engine_t;

static int is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

static cplx* twiddles(int n, int sign) {
  const int h = n / 2 > 0 ? n / 2 : 1;
  cplx* t = malloc(sizeof(cplx) * (size_t)h);
  for (int k = 0; k < h; k++) {
    const double a = (double)sign * 2.0 * M_PI * (double)k / (double)n;
    t[k].re = cos(a);
    t[k].im = sin(a);
  }
  return t;
}

/* In place, length n a power of two, twiddles from twiddles(n, sign). */
static void fft_pow2(cplx* a, int n, const cplx* tw) {
  for (int i = 1, j = 0; i < n; i++) {
    int bit = n >> 1;
    for (; j & bit; bit >>= 1)
      j ^= bit;
    j ^= bit;
    if (i < j) {
      const cplx t = a[i];
      a[i] = a[j];
      a[j] = t;
    }
  }
  for (int len = 2; len <= n; len <<= 1) {
    const int half = len >> 1;
    const int step = n / len;
    for (int i = 0; i < n; i += len) {
      for (int k = 0; k < half; k++) {
        const cplx w = tw[k * step];
        const cplx u = a[i + k];
        const cplx v = a[i + k + half];
        const cplx vw = {v.re * w.re - v.im * w.im, v.re * w.im + v.im * w.re};
        a[i + k].re = u.re + vw.re;
        a[i + k].im = u.im + vw.im;
        a[i + k + half].re = u.re - vw.re;
        a[i + k + half].im = u.im - vw.im;
      }
    }
  }
}

static engine_t* engine_new(int n, int sign) {
  engine_t* e = calloc(1, sizeof(engine_t));
  e->n = n;
  e->sign = sign;
  e->pow2 = is_pow2(n);
  if (e->pow2) {
    e->tw = twiddles(n, sign);
    return e;
  }
  int m = 1;
  while (m < 2 * n - 1)
    m <<= 1;
  e->m = m;
  e->chirp = malloc(sizeof(cplx) * (size_t)n);
  for (int k = 0; k < n; k++) {
    /* k^2 mod 2n keeps the angle small, so it stays exact in double. */
    const long long q = ((long long)k * k) % (2LL * n);
    const double a = (double)sign * M_PI * (double)q / (double)n;
    e->chirp[k].re = cos(a);
    e->chirp[k].im = sin(a);
  }
  e->mtw_f = twiddles(m, -1);
  e->mtw_b = twiddles(m, +1);
  e->bhat = calloc((size_t)m, sizeof(cplx));
  for (int k = 0; k < n; k++) {
    const cplx c = {e->chirp[k].re, -e->chirp[k].im};
    e->bhat[k] = c;
    if (k > 0)
      e->bhat[m - k] = c;
  }
  fft_pow2(e->bhat, m, e->mtw_f);
  return e;
}

static void engine_free(engine_t* e) {
  if (!e)
    return;
  free(e->tw);
  free(e->chirp);
  free(e->bhat);
  free(e->mtw_f);
  free(e->mtw_b);
  free(e);
}

/* In place on a[0..n); `work` holds at least m entries for Bluestein. */
static void engine_run(const engine_t* e, cplx* a, cplx* work) {
  const int n = e->n;
  if (e->pow2) {
    fft_pow2(a, n, e->tw);
    return;
  }
  const int m = e->m;
  for (int k = 0; k < n; k++) {
    const cplx c = e->chirp[k];
    work[k].re = a[k].re * c.re - a[k].im * c.im;
    work[k].im = a[k].re * c.im + a[k].im * c.re;
  }
  for (int k = n; k < m; k++)
    work[k].re = work[k].im = 0.0;
  fft_pow2(work, m, e->mtw_f);
  for (int k = 0; k < m; k++) {
    const cplx b = e->bhat[k];
    const cplx w = work[k];
    work[k].re = w.re * b.re - w.im * b.im;
    work[k].im = w.re * b.im + w.im * b.re;
  }
  fft_pow2(work, m, e->mtw_b);
  const double inv_m = 1.0 / (double)m;
  for (int k = 0; k < n; k++) {
    const cplx c = e->chirp[k];
    const double re = work[k].re * inv_m, im = work[k].im * inv_m;
    a[k].re = re * c.re - im * c.im;
    a[k].im = re * c.im + im * c.re;
  }
}

static size_t engine_work(const engine_t* e) {
  return e->pow2 ? 1 : (size_t)e->m;
}

/* --- plans --- */

enum { KIND_MANY = 0, KIND_R2C, KIND_C2R };

struct shim_fft_plan {
  int kind;
  int is_float;
  /* KIND_MANY */
  int n, howmany, istride, idist, ostride, odist;
  /* KIND_R2C / KIND_C2R: real dims, row-major, last fastest */
  int rank;
  int dims[3];
  engine_t* eng[3]; /* one per axis, in the plan's direction */
  void* in;
  void* out;
};

static struct shim_fft_plan* plan_alloc(int kind, int is_float) {
  struct shim_fft_plan* p = calloc(1, sizeof(*p));
  p->kind = kind;
  p->is_float = is_float;
  return p;
}

static void plan_destroy(struct shim_fft_plan* p) {
  if (!p)
    return;
  for (int d = 0; d < 3; d++)
    engine_free(p->eng[d]);
  free(p);
}

/* Loads element i of an interleaved complex array of the plan's precision. */
static inline cplx load_c(const void* base, int is_float, size_t i) {
  cplx c;
  if (is_float) {
    const float* f = (const float*)base;
    c.re = f[2 * i];
    c.im = f[2 * i + 1];
  } else {
    const double* d = (const double*)base;
    c.re = d[2 * i];
    c.im = d[2 * i + 1];
  }
  return c;
}

static inline void store_c(void* base, int is_float, size_t i, cplx c) {
  if (is_float) {
    float* f = (float*)base;
    f[2 * i] = (float)c.re;
    f[2 * i + 1] = (float)c.im;
  } else {
    double* d = (double*)base;
    d[2 * i] = c.re;
    d[2 * i + 1] = c.im;
  }
}

static void exec_many(const struct shim_fft_plan* p, const void* in, void* out) {
  const int n = p->n;
  cplx* line = malloc(sizeof(cplx) * (size_t)n);
  cplx* work = malloc(sizeof(cplx) * engine_work(p->eng[0]));
  for (int k = 0; k < p->howmany; k++) {
    for (int j = 0; j < n; j++)
      line[j] = load_c(
        in, p->is_float, (size_t)k * p->idist + (size_t)j * p->istride);
    engine_run(p->eng[0], line, work);
    for (int j = 0; j < n; j++)
      store_c(
        out, p->is_float, (size_t)k * p->odist + (size_t)j * p->ostride, line[j]);
  }
  free(line);
  free(work);
}

/* C2C along axis `ax` of a double complex array of shape `shape` (rank r). */
static void pass_axis(cplx* a, const int* shape, int r, int ax, const engine_t* e) {
  size_t stride = 1;
  for (int d = ax + 1; d < r; d++)
    stride *= (size_t)shape[d];
  const size_t len = (size_t)shape[ax];
  size_t outer = 1;
  for (int d = 0; d < ax; d++)
    outer *= (size_t)shape[d];
  /* Every line is independent: a team shares them when OpenMP is on. */
#pragma omp parallel
  {
    cplx* line = malloc(sizeof(cplx) * len);
    cplx* work = malloc(sizeof(cplx) * engine_work(e));
#pragma omp for schedule(static) collapse(2)
    for (size_t o = 0; o < outer; o++) {
      for (size_t s = 0; s < stride; s++) {
        cplx* base = a + o * len * stride + s;
        for (size_t j = 0; j < len; j++)
          line[j] = base[j * stride];
        engine_run(e, line, work);
        for (size_t j = 0; j < len; j++)
          base[j * stride] = line[j];
      }
    }
    free(line);
    free(work);
  }
}

static void exec_r2c(const struct shim_fft_plan* p, const void* in, void* out) {
  const int r = p->rank;
  const int nl = p->dims[r - 1];
  const int half = nl / 2 + 1;
  size_t rows = 1;
  for (int d = 0; d < r - 1; d++)
    rows *= (size_t)p->dims[d];
  int shape[3];
  for (int d = 0; d < r - 1; d++)
    shape[d] = p->dims[d];
  shape[r - 1] = half;

  cplx* spec = malloc(sizeof(cplx) * rows * (size_t)half);
#pragma omp parallel
  {
    cplx* line = malloc(sizeof(cplx) * (size_t)nl);
    cplx* work = malloc(sizeof(cplx) * engine_work(p->eng[r - 1]));
#pragma omp for schedule(static)
    for (size_t row = 0; row < rows; row++) {
      for (int j = 0; j < nl; j++) {
        const size_t i = row * (size_t)nl + (size_t)j;
        line[j].re = p->is_float ? (double)((const float*)in)[i]
                                 : ((const double*)in)[i];
        line[j].im = 0.0;
      }
      engine_run(p->eng[r - 1], line, work);
      memcpy(spec + row * (size_t)half, line, sizeof(cplx) * (size_t)half);
    }
    free(line);
    free(work);
  }
  for (int ax = r - 2; ax >= 0; ax--)
    pass_axis(spec, shape, r, ax, p->eng[ax]);
  for (size_t i = 0; i < rows * (size_t)half; i++)
    store_c(out, p->is_float, i, spec[i]);
  free(spec);
}

static void exec_c2r(const struct shim_fft_plan* p, const void* in, void* out) {
  const int r = p->rank;
  const int nl = p->dims[r - 1];
  const int half = nl / 2 + 1;
  size_t rows = 1;
  for (int d = 0; d < r - 1; d++)
    rows *= (size_t)p->dims[d];
  int shape[3];
  for (int d = 0; d < r - 1; d++)
    shape[d] = p->dims[d];
  shape[r - 1] = half;

  cplx* spec = malloc(sizeof(cplx) * rows * (size_t)half);
  for (size_t i = 0; i < rows * (size_t)half; i++)
    spec[i] = load_c(in, p->is_float, i);
  for (int ax = 0; ax <= r - 2; ax++)
    pass_axis(spec, shape, r, ax, p->eng[ax]);

#pragma omp parallel
  {
  cplx* line = malloc(sizeof(cplx) * (size_t)nl);
  cplx* work = malloc(sizeof(cplx) * engine_work(p->eng[r - 1]));
#pragma omp for schedule(static)
  for (size_t row = 0; row < rows; row++) {
    const cplx* s = spec + row * (size_t)half;
    /* The Hermitian completion; the imaginary parts of the self-conjugate
     * modes drop out of the real part, as in FFTW's c2r. */
    for (int k = 0; k < half; k++)
      line[k] = s[k];
    for (int k = half; k < nl; k++) {
      line[k].re = s[nl - k].re;
      line[k].im = -s[nl - k].im;
    }
    engine_run(p->eng[r - 1], line, work);
    for (int j = 0; j < nl; j++) {
      const size_t i = row * (size_t)nl + (size_t)j;
      if (p->is_float)
        ((float*)out)[i] = (float)line[j].re;
      else
        ((double*)out)[i] = line[j].re;
    }
  }
  free(line);
  free(work);
  }
  free(spec);
}

static struct shim_fft_plan* plan_real(
  int kind, int is_float, int rank, const int* dims, void* in, void* out) {
  for (int d = 0; d < rank; d++)
    if (dims[d] <= 0)
      return NULL;
  struct shim_fft_plan* p = plan_alloc(kind, is_float);
  p->rank = rank;
  const int sign = kind == KIND_R2C ? FFTW_FORWARD : FFTW_BACKWARD;
  for (int d = 0; d < rank; d++) {
    p->dims[d] = dims[d];
    p->eng[d] = engine_new(dims[d], sign);
  }
  p->in = in;
  p->out = out;
  return p;
}

static void plan_execute(const struct shim_fft_plan* p, const void* in, void* out) {
  if (!p)
    return;
  switch (p->kind) {
  case KIND_MANY:
    exec_many(p, in, out);
    break;
  case KIND_R2C:
    exec_r2c(p, in, out);
    break;
  default:
    exec_c2r(p, in, out);
    break;
  }
}

#define SHIM_FFTW_DEFINE(X, R, IS_FLOAT)                                        \
  int X##_init_threads(void) { return 1; }                                      \
  void X##_plan_with_nthreads(int nthreads) { (void)nthreads; }                 \
  void X##_cleanup_threads(void) {}                                             \
  void X##_cleanup(void) {}                                                     \
  int X##_import_wisdom_from_filename(const char* filename) {                   \
    (void)filename;                                                             \
    return 0;                                                                   \
  }                                                                             \
  int X##_export_wisdom_to_filename(const char* filename) {                     \
    (void)filename;                                                             \
    return 0;                                                                   \
  }                                                                             \
  char* X##_export_wisdom_to_string(void) {                                     \
    char* s = malloc(1);                                                        \
    if (s)                                                                      \
      s[0] = '\0';                                                              \
    return s;                                                                   \
  }                                                                             \
  void X##_forget_wisdom(void) {}                                               \
  void* X##_malloc(size_t n) {                                                  \
    void* p = NULL;                                                             \
    if (posix_memalign(&p, 64, n ? n : 1) != 0)                                 \
      return NULL;                                                              \
    return p;                                                                   \
  }                                                                             \
  void X##_free(void* p) { free(p); }                                           \
  int X##_alignment_of(R* p) { return (int)((uintptr_t)p % 16u); }              \
  void X##_destroy_plan(X##_plan p) { plan_destroy(p); }                        \
  void X##_execute(const X##_plan p) {                                          \
    if (p)                                                                      \
      plan_execute(p, p->in, p->out);                                           \
  }                                                                             \
  X##_plan X##_plan_dft_r2c_2d(                                                 \
    int n0, int n1, R* in, X##_complex* out, unsigned flags) {                  \
    (void)flags;                                                                \
    const int d[2] = {n0, n1};                                                  \
    return plan_real(KIND_R2C, IS_FLOAT, 2, d, in, out);                        \
  }                                                                             \
  X##_plan X##_plan_dft_c2r_2d(                                                 \
    int n0, int n1, X##_complex* in, R* out, unsigned flags) {                  \
    (void)flags;                                                                \
    const int d[2] = {n0, n1};                                                  \
    return plan_real(KIND_C2R, IS_FLOAT, 2, d, in, out);                        \
  }                                                                             \
  X##_plan X##_plan_dft_r2c_3d(                                                 \
    int n0, int n1, int n2, R* in, X##_complex* out, unsigned flags) {          \
    (void)flags;                                                                \
    const int d[3] = {n0, n1, n2};                                              \
    return plan_real(KIND_R2C, IS_FLOAT, 3, d, in, out);                        \
  }                                                                             \
  X##_plan X##_plan_dft_c2r_3d(                                                 \
    int n0, int n1, int n2, X##_complex* in, R* out, unsigned flags) {          \
    (void)flags;                                                                \
    const int d[3] = {n0, n1, n2};                                              \
    return plan_real(KIND_C2R, IS_FLOAT, 3, d, in, out);                        \
  }                                                                             \
  X##_plan X##_plan_many_dft(int rank, const int* n, int howmany,               \
    X##_complex* in, const int* inembed, int istride, int idist,                \
    X##_complex* out, const int* onembed, int ostride, int odist, int sign,     \
    unsigned flags) {                                                           \
    (void)inembed;                                                              \
    (void)onembed;                                                              \
    (void)flags;                                                                \
    if (rank != 1 || n[0] <= 0 || howmany <= 0)                                 \
      return NULL;                                                              \
    struct shim_fft_plan* p = plan_alloc(KIND_MANY, IS_FLOAT);                  \
    p->n = n[0];                                                                \
    p->howmany = howmany;                                                       \
    p->istride = istride;                                                       \
    p->idist = idist;                                                           \
    p->ostride = ostride;                                                       \
    p->odist = odist;                                                           \
    p->eng[0] = engine_new(n[0], sign);                                         \
    p->in = in;                                                                 \
    p->out = out;                                                               \
    return p;                                                                   \
  }                                                                             \
  void X##_execute_dft(const X##_plan p, X##_complex* in, X##_complex* out) {   \
    plan_execute(p, in, out);                                                   \
  }                                                                             \
  void X##_execute_dft_r2c(const X##_plan p, R* in, X##_complex* out) {         \
    plan_execute(p, in, out);                                                   \
  }                                                                             \
  void X##_execute_dft_c2r(const X##_plan p, X##_complex* in, R* out) {         \
    plan_execute(p, in, out);                                                   \
  }

SHIM_FFTW_DEFINE(fftw, double, 0)
SHIM_FFTW_DEFINE(fftwf, float, 1)
