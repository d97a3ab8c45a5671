/*
 * A small FFTW3-API stand-in, written for this project.
 *
 * TEST INFRASTRUCTURE ONLY. FFTW is not installed on the build or GPU machines,
 * so the reference C library (sif) is linked against this shim when it is
 * compiled as the parity checker. It declares the subset of the FFTW3 API that
 * sif's src/math/fft.c and src/core/system.c call (plans: r2c/c2r in 2-D and
 * 3-D, batched 1-D complex via plan_many_dft; new-array execution; wisdom and
 * thread hooks as no-ops) in both precisions. The transforms run in double
 * internally (radix-2 for powers of two, Bluestein otherwise), so the spectra
 * agree with FFTW's to rounding, not to the bit.
 */
#ifndef SIF_ORACLE_FFTW_SHIM_H
#define SIF_ORACLE_FFTW_SHIM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FFTW_FORWARD  (-1)
#define FFTW_BACKWARD (+1)

#define FFTW_MEASURE         (0U)
#define FFTW_DESTROY_INPUT   (1U << 0)
#define FFTW_UNALIGNED       (1U << 1)
#define FFTW_CONSERVE_MEMORY (1U << 2)
#define FFTW_EXHAUSTIVE      (1U << 3)
#define FFTW_PRESERVE_INPUT  (1U << 4)
#define FFTW_PATIENT         (1U << 5)
#define FFTW_ESTIMATE        (1U << 6)
#define FFTW_WISDOM_ONLY     (1U << 21)

struct shim_fft_plan;

#define SHIM_FFTW_DECLARE(X, R)                                                 \
  typedef R X##_complex[2];                                                     \
  typedef struct shim_fft_plan* X##_plan;                                       \
  int X##_init_threads(void);                                                   \
  void X##_plan_with_nthreads(int nthreads);                                    \
  void X##_cleanup_threads(void);                                               \
  void X##_cleanup(void);                                                       \
  int X##_import_wisdom_from_filename(const char* filename);                    \
  int X##_export_wisdom_to_filename(const char* filename);                      \
  char* X##_export_wisdom_to_string(void);                                      \
  void X##_forget_wisdom(void);                                                 \
  void* X##_malloc(size_t n);                                                   \
  void X##_free(void* p);                                                       \
  int X##_alignment_of(R* p);                                                   \
  void X##_destroy_plan(X##_plan p);                                            \
  void X##_execute(const X##_plan p);                                           \
  X##_plan X##_plan_dft_r2c_2d(int n0, int n1, R* in, X##_complex* out,         \
    unsigned flags);                                                            \
  X##_plan X##_plan_dft_c2r_2d(int n0, int n1, X##_complex* in, R* out,         \
    unsigned flags);                                                            \
  X##_plan X##_plan_dft_r2c_3d(int n0, int n1, int n2, R* in,                   \
    X##_complex* out, unsigned flags);                                          \
  X##_plan X##_plan_dft_c2r_3d(int n0, int n1, int n2, X##_complex* in,         \
    R* out, unsigned flags);                                                    \
  X##_plan X##_plan_many_dft(int rank, const int* n, int howmany,               \
    X##_complex* in, const int* inembed, int istride, int idist,                \
    X##_complex* out, const int* onembed, int ostride, int odist, int sign,     \
    unsigned flags);                                                            \
  void X##_execute_dft(const X##_plan p, X##_complex* in, X##_complex* out);    \
  void X##_execute_dft_r2c(const X##_plan p, R* in, X##_complex* out);          \
  void X##_execute_dft_c2r(const X##_plan p, X##_complex* in, R* out);

SHIM_FFTW_DECLARE(fftw, double)
SHIM_FFTW_DECLARE(fftwf, float)

#undef SHIM_FFTW_DECLARE

#ifdef __cplusplus
}
#endif

#endif /* SIF_ORACLE_FFTW_SHIM_H */
