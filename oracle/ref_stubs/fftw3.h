/* FFTW3 API subset used by the reference airwave boundary (airbc_init_free.c:45-49,
 * 115-118,153,161,188), backed by the self-written transform in oracle/fft2d.c.
 * FFTW itself is not installed; this header declares only what the reference calls.
 * fftw_complex is the C99 double complex, as FFTW defines it when <complex.h> is
 * included first (the reference includes cstd.h, hence complex.h, before fftw3.h). */
#ifndef CSEM_ORACLE_FFTW3_SHIM_H
#define CSEM_ORACLE_FFTW3_SHIM_H
#include <stddef.h>
#include <complex.h>
typedef double _Complex fftw_complex;
typedef struct csem_fft_plan_s *fftw_plan;
#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_ESTIMATE (1U << 6)
void *fftw_malloc(size_t n);
void fftw_free(void *p);
fftw_plan fftw_plan_dft_2d(int n0, int n1, fftw_complex *in, fftw_complex *out,
                           int sign, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);
#endif
