/* Self-written 2-D complex DFT for the CPU oracle (test infrastructure only).
 *
 * The reference's airwave boundary calls FFTW's fftw_plan_dft_2d(n1fft, n2fft, ...)
 * with FFTW_FORWARD / FFTW_BACKWARD and executes it in place
 * (airbc_init_free.c:48-49,153,161,188). FFTW is a third-party dependency that is
 * neither vendored nor version-pinned by the reference (Makefile:28, "-lfftw3"), and
 * it is not installed here. This file restates the published definition FFTW
 * implements: the unnormalised 2-D DFT of a row-major array a[n0][n1] (n1 fastest),
 *     A[k0][k1] = sum_{j0,j1} a[j0][j1] * exp(sign * 2*pi*i * (j0*k0/n0 + j1*k1/n1)),
 * sign = -1 forward, +1 backward. Power-of-two lengths use an iterative radix-2
 * Cooley-Tukey transform (Cooley & Tukey 1965); other lengths a direct O(n^2) sum.
 * The result matches FFTW to rounding, not bit for bit: parity at the FFT boundary
 * is therefore unpinned, and tests compare airwave results with a tolerance.
 *
 * Arithmetic is written on separate real/imaginary doubles and the file is built
 * with -ffp-contract=off, so x86-64 and aarch64 builds give identical bits.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "fft2d.h"

static int is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

/* One 1-D transform of length n on data with stride `stride` (in complex elements).
 * re/im are interleaved doubles (complex layout). work holds 2*n doubles. */
static void dft1d(double *data, int n, int stride, int sign, double *work,
                  const double *tw_re, const double *tw_im)
{
  int i, j, k;
  if (n == 1) return;
  for (i = 0; i < n; i++) {
    work[2 * i] = data[2 * (size_t)i * stride];
    work[2 * i + 1] = data[2 * (size_t)i * stride + 1];
  }
  if (is_pow2(n)) {
    /* bit-reversal permutation */
    for (i = 1, j = 0; i < n; i++) {
      int bit = n >> 1;
      for (; j & bit; bit >>= 1) j ^= bit;
      j ^= bit;
      if (i < j) {
        double tr = work[2 * i], ti = work[2 * i + 1];
        work[2 * i] = work[2 * j];
        work[2 * i + 1] = work[2 * j + 1];
        work[2 * j] = tr;
        work[2 * j + 1] = ti;
      }
    }
    /* butterflies; twiddle for span len at index k is w_n^(k*n/len) */
    for (int len = 2; len <= n; len <<= 1) {
      int half = len >> 1, step = n / len;
      for (i = 0; i < n; i += len) {
        for (k = 0; k < half; k++) {
          double wr = tw_re[k * step], wi = sign < 0 ? -tw_im[k * step] : tw_im[k * step];
          double *u = &work[2 * (i + k)], *v = &work[2 * (i + k + half)];
          double vr = v[0] * wr - v[1] * wi;
          double vi = v[0] * wi + v[1] * wr;
          double ur = u[0], ui = u[1];
          u[0] = ur + vr;
          u[1] = ui + vi;
          v[0] = ur - vr;
          v[1] = ui - vi;
        }
      }
    }
    for (i = 0; i < n; i++) {
      data[2 * (size_t)i * stride] = work[2 * i];
      data[2 * (size_t)i * stride + 1] = work[2 * i + 1];
    }
  } else {
    for (k = 0; k < n; k++) {
      double sr = 0, si = 0;
      for (j = 0; j < n; j++) {
        int m = (int)(((long long)j * k) % n);
        double wr = tw_re[m], wi = sign < 0 ? -tw_im[m] : tw_im[m];
        double ar = work[2 * j], ai = work[2 * j + 1];
        sr += ar * wr - ai * wi;
        si += ar * wi + ai * wr;
      }
      data[2 * (size_t)k * stride] = sr;
      data[2 * (size_t)k * stride + 1] = si;
    }
  }
}

/* twiddles w_n^m = cos(2 pi m/n) + i sin(2 pi m/n), m = 0..n-1 */
static void make_twiddles(int n, double *re, double *im)
{
  for (int m = 0; m < n; m++) {
    double a = 2.0 * 3.14159265358979323846264 * (double)m / (double)n;
    re[m] = cos(a);
    im[m] = sin(a);
  }
}

void csem_fft2d(int n0, int n1, double *data, int sign)
{
  int nmax = n0 > n1 ? n0 : n1;
  double *work = (double *)malloc(sizeof(double) * 2 * (size_t)nmax);
  double *t0r = (double *)malloc(sizeof(double) * (size_t)n0);
  double *t0i = (double *)malloc(sizeof(double) * (size_t)n0);
  double *t1r = (double *)malloc(sizeof(double) * (size_t)n1);
  double *t1i = (double *)malloc(sizeof(double) * (size_t)n1);
  make_twiddles(n0, t0r, t0i);
  make_twiddles(n1, t1r, t1i);
  /* rows (contiguous, length n1) then columns (stride n1, length n0) */
  for (int r = 0; r < n0; r++) dft1d(data + 2 * (size_t)r * n1, n1, 1, sign, work, t1r, t1i);
  for (int c = 0; c < n1; c++) dft1d(data + 2 * (size_t)c, n0, n1, sign, work, t0r, t0i);
  free(work);
  free(t0r);
  free(t0i);
  free(t1r);
  free(t1i);
}
