/* Model, acquisition and output set-up on the host (run once per model).
 *
 * The grid construction is arithmetic-for-arithmetic the reference's, because the
 * stencil coefficients it produces decide every digit downstream:
 *   - reading:     emf_init_free.c:77-166
 *   - stretching:  create_nugrid.c:46-70 (fixed-point ratio), extend_model.c:72-108
 *   - staggering:  extend_model.c:8-21
 *   - padding:     extend_model.c:126-177, including its quirks: the top nb cells
 *                  are always air, and the bottom padding copies row j=k of the last
 *                  interior layer rather than row j (extend_model.c:169,171,173)
 *   - averaging:   extend_model.c:180-252 (sigma33 averaged as resistivity)
 *   - airwave:     airbc_init_free.c:30-105
 * The file is built with -ffp-contract=off so no multiply-add is fused.
 */
#include <complex.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "../../include/csem_host.h"
#include "../../include/csem_gpu.h" /* CSEM_ST_* */

#define CSEM_PI 3.14159265358979323846264

static __thread char g_err[512];

const char *csem_last_error(void) { return g_err; }

int csem_set_error(int code, const char *fmt, ...)
{
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return code;
}

/* find k with x[k] <= val < x[k+1] by bisection (find_index.c:9-30) */
int csem_find_index(int n, const double *x, double val)
{
  int low = 0, high = n - 1;
  while (low < high) {
    int i = (low + high) / 2;
    if (x[i] <= val) low = i;
    if (x[i] > val) high = i;
    if (low == high || low == high - 1) break;
  }
  return low;
}

static float *read_floats(const char *path, long *count)
{
  FILE *fp = fopen(path, "rb");
  if (!fp) return NULL;
  fseek(fp, 0, SEEK_END);
  long size = ftell(fp);
  rewind(fp);
  long n = size / (long)sizeof(float);
  float *buf = (float *)malloc(sizeof(float) * (size_t)(n > 0 ? n : 1));
  long got = (long)fread(buf, sizeof(float), (size_t)n, fp);
  fclose(fp);
  *count = got;
  return buf;
}

static void model_minmax(csem_grid_t *g)
{
  long n = (long)g->nx * g->ny * g->nz;
  g->rhomax = g->rho11[0];
  g->rhomin = g->rho11[0];
  for (long c = 0; c < n; c++) {
    float a = g->rho11[c], b = g->rho22[c], d = g->rho33[c];
    g->rhomax = g->rhomax > a ? g->rhomax : a;
    g->rhomin = g->rhomin < a ? g->rhomin : a;
    g->rhomax = g->rhomax > b ? g->rhomax : b;
    g->rhomin = g->rhomin < b ? g->rhomin : b;
    g->rhomax = g->rhomax > d ? g->rhomax : d;
    g->rhomin = g->rhomin < d ? g->rhomin : d;
  }
  g->rho_water = g->rhomin; /* emf_init_free.c:166: input model has no air */
}

int csem_grid_read(csem_grid_t *g, const char *fx1, const char *fx2, const char *fx3,
                   const char *frho11, const char *frho22, const char *frho33)
{
  memset(g, 0, sizeof(*g));
  long n1, n2, n3;
  const char *fx[3] = {fx1, fx2, fx3};
  float **xn[3] = {&g->x1node, &g->x2node, &g->x3node};
  long *cnt[3] = {&n1, &n2, &n3};
  for (int a = 0; a < 3; a++) {
    *xn[a] = read_floats(fx[a], cnt[a]);
    if (!*xn[a]) return csem_set_error(CSEM_EIO, "cannot open file fx%d=%s", a + 1, fx[a]);
    if (*cnt[a] < 2) return csem_set_error(CSEM_EIO, "fx%d=%s holds fewer than 2 nodes", a + 1, fx[a]);
  }
  g->nx = (int)n1 - 1;
  g->ny = (int)n2 - 1;
  g->nz = (int)n3 - 1;
  long n = (long)g->nx * g->ny * g->nz;
  const char *fr[3] = {frho11, frho22, frho33};
  float **rr[3] = {&g->rho11, &g->rho22, &g->rho33};
  for (int a = 0; a < 3; a++) {
    FILE *fp = fopen(fr[a], "rb");
    if (!fp) return csem_set_error(CSEM_EIO, "cannot open file frho%d%d=%s", a + 1, a + 1, fr[a]);
    *rr[a] = (float *)malloc(sizeof(float) * (size_t)n);
    long got = (long)fread(*rr[a], sizeof(float), (size_t)n, fp);
    fclose(fp);
    if (got != n)
      return csem_set_error(CSEM_EIO, "size not match frho%d%d: file=%ld nx*ny*nz=%ld", a + 1, a + 1, got, n);
  }
  model_minmax(g);
  return CSEM_OK;
}

int csem_grid_set(csem_grid_t *g, int nx, int ny, int nz, const float *x1node,
                  const float *x2node, const float *x3node, const float *rho11,
                  const float *rho22, const float *rho33)
{
  if (nx < 1 || ny < 1 || nz < 1) return csem_set_error(CSEM_EINVAL, "model needs nx,ny,nz >= 1");
  memset(g, 0, sizeof(*g));
  g->nx = nx;
  g->ny = ny;
  g->nz = nz;
  size_t n = (size_t)nx * ny * nz;
  g->x1node = (float *)malloc(sizeof(float) * (size_t)(nx + 1));
  g->x2node = (float *)malloc(sizeof(float) * (size_t)(ny + 1));
  g->x3node = (float *)malloc(sizeof(float) * (size_t)(nz + 1));
  memcpy(g->x1node, x1node, sizeof(float) * (size_t)(nx + 1));
  memcpy(g->x2node, x2node, sizeof(float) * (size_t)(ny + 1));
  memcpy(g->x3node, x3node, sizeof(float) * (size_t)(nz + 1));
  g->rho11 = (float *)malloc(sizeof(float) * n);
  g->rho22 = (float *)malloc(sizeof(float) * n);
  g->rho33 = (float *)malloc(sizeof(float) * n);
  memcpy(g->rho11, rho11, sizeof(float) * n);
  memcpy(g->rho22, rho22, sizeof(float) * n);
  memcpy(g->rho33, rho33, sizeof(float) * n);
  model_minmax(g);
  return CSEM_OK;
}

/* geometric padding ratio by fixed-point iteration (create_nugrid.c:46-70) */
static double nugrid_ratio(int n, double len, double dx, int istretch)
{
  if (n * dx >= len || !istretch) return 1;
  double q = 1.1, qq;
  for (int iter = 0; iter < 100; ++iter) {
    qq = pow(len * (q - 1.) / dx + 1., 1. / n);
    if (fabs(qq - q) < 1e-15) break;
    q = qq;
  }
  return q;
}

static void staggered(int n, const double *x, double *xs, double *d, double *ds)
{
  for (int i = 0; i < n; i++) {
    ds[i] = x[i + 1] - x[i];
    xs[i] = 0.5 * (x[i] + x[i + 1]);
  }
  ds[n] = ds[n - 1];
  xs[n] = x[n] + 0.5 * ds[n - 1];
  for (int i = 1; i <= n; i++) d[i] = xs[i] - xs[i - 1];
  d[0] = d[1];
}

int csem_grid_extend(csem_grid_t *g, int nb, float lextend, float rho_air, int istretch)
{
  if (nb < 0) return csem_set_error(CSEM_EINVAL, "nb must be >= 0");
  g->nb = nb;
  g->rho_air = rho_air;
  g->istretch = istretch;
  int nx = g->nx, ny = g->ny, nz = g->nz;
  int n1 = nx + 2 * nb, n2 = ny + 2 * nb, n3 = nz + 2 * nb;
  g->n1 = n1;
  g->n2 = n2;
  g->n3 = n3;
  const float *x1n = g->x1node, *x2n = g->x2node, *x3n = g->x3node;
  double dx;
  g->d1min = x1n[1] - x1n[0];
  for (int i = 0; i < nx; i++) { double t = x1n[i + 1] - x1n[i]; g->d1min = g->d1min < t ? g->d1min : t; }
  g->d2min = x2n[1] - x2n[0];
  for (int j = 0; j < ny; j++) { double t = x2n[j + 1] - x2n[j]; g->d2min = g->d2min < t ? g->d2min : t; }
  g->d3min = x3n[1] - x3n[0];
  for (int k = 0; k < nz; k++) { double t = x3n[k + 1] - x3n[k]; g->d3min = g->d3min < t ? g->d3min : t; }

  /* extend_model.c:43-51: default 40 km, at least 2.2x each model length */
  g->lextend = lextend >= 0 ? lextend : (nb > 0 ? 40e3f : 0.f);
  if (nb > 0) {
    double t;
    dx = x1n[nx] - x1n[0];
    t = 2.2 * dx;
    g->lextend = (float)(g->lextend > t ? (double)g->lextend : t);
    dx = x2n[ny] - x2n[0];
    t = 2.2 * dx;
    g->lextend = (float)(g->lextend > t ? (double)g->lextend : t);
    dx = x3n[nz] - x3n[0];
    t = 2.2 * dx;
    g->lextend = (float)(g->lextend > t ? (double)g->lextend : t);
  }

  size_t b1 = sizeof(double) * (size_t)(n1 + 1), b2 = sizeof(double) * (size_t)(n2 + 1),
         b3 = sizeof(double) * (size_t)(n3 + 1);
  g->x1 = (double *)calloc(1, b1); g->x2 = (double *)calloc(1, b2); g->x3 = (double *)calloc(1, b3);
  g->x1s = (double *)calloc(1, b1); g->x2s = (double *)calloc(1, b2); g->x3s = (double *)calloc(1, b3);
  g->d1 = (double *)calloc(1, b1); g->d2 = (double *)calloc(1, b2); g->d3 = (double *)calloc(1, b3);
  g->d1s = (double *)calloc(1, b1); g->d2s = (double *)calloc(1, b2); g->d3s = (double *)calloc(1, b3);
  for (int i = 0; i <= nx; i++) g->x1[i + nb] = x1n[i];
  for (int j = 0; j <= ny; j++) g->x2[j + nb] = x2n[j];
  for (int k = 0; k <= nz; k++) g->x3[k + nb] = x3n[k];
  if (nb > 0) {
    double len = g->lextend, r;
    dx = x1n[1] - x1n[0];
    r = g->rstretch[0] = (float)nugrid_ratio(nb, len, dx, istretch); /* emf->rstretch is a float */
    for (int i = 0; i < nb; i++) g->x1[nb - 1 - i] = g->x1[nb - i] - dx * pow(r, i);
    dx = x1n[nx] - x1n[nx - 1];
    r = g->rstretch[1] = (float)nugrid_ratio(nb, len, dx, istretch); /* emf->rstretch is a float */
    for (int i = 0; i < nb; i++) g->x1[nb + nx + 1 + i] = g->x1[nb + nx + i] + dx * pow(r, i);
    dx = x2n[1] - x2n[0];
    r = g->rstretch[2] = (float)nugrid_ratio(nb, len, dx, istretch); /* emf->rstretch is a float */
    for (int j = 0; j < nb; j++) g->x2[nb - 1 - j] = g->x2[nb - j] - dx * pow(r, j);
    dx = x2n[ny] - x2n[ny - 1];
    r = g->rstretch[3] = (float)nugrid_ratio(nb, len, dx, istretch); /* emf->rstretch is a float */
    for (int j = 0; j < nb; j++) g->x2[nb + ny + 1 + j] = g->x2[nb + ny + j] + dx * pow(r, j);
    dx = x3n[1] - x3n[0];
    r = g->rstretch[4] = (float)nugrid_ratio(nb, len, dx, istretch); /* emf->rstretch is a float */
    for (int k = 0; k < nb; k++) g->x3[nb - 1 - k] = g->x3[nb - k] - dx * pow(r, k);
    dx = x3n[nz] - x3n[nz - 1];
    r = g->rstretch[5] = (float)nugrid_ratio(nb, len, dx, istretch); /* emf->rstretch is a float */
    for (int k = 0; k < nb; k++) g->x3[nb + nz + 1 + k] = g->x3[nb + nz + k] + dx * pow(r, k);
  }
  staggered(n1, g->x1, g->x1s, g->d1, g->d1s);
  staggered(n2, g->x2, g->x2s, g->d2, g->d2s);
  staggered(n3, g->x3, g->x3s, g->d3, g->d3s);

  /* cell-centred padded parameters [n3][n2][n1] */
  size_t nc = (size_t)n1 * n2 * n3;
  double *s11 = (double *)calloc(nc, sizeof(double));
  double *s22 = (double *)calloc(nc, sizeof(double));
  double *r33 = (double *)calloc(nc, sizeof(double));
#define C3(a, k, j, i) a[((size_t)(k) * n2 + (j)) * n1 + (i)]
  for (int k = 0; k < nz; k++)
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++) {
        size_t src = ((size_t)k * ny + j) * nx + i;
        C3(s11, k + nb, j + nb, i + nb) = 1. / g->rho11[src];
        C3(s22, k + nb, j + nb, i + nb) = 1. / g->rho22[src];
        C3(r33, k + nb, j + nb, i + nb) = g->rho33[src];
      }
  if (nb > 0) {
    for (int k = 0; k < n3; k++)
      for (int j = 0; j < n2; j++)
        for (int i = 0; i < nb; i++) {
          C3(s11, k, j, i) = C3(s11, k, j, nb);
          C3(s11, k, j, n1 - 1 - i) = C3(s11, k, j, n1 - 1 - nb);
          C3(s22, k, j, i) = C3(s22, k, j, nb);
          C3(s22, k, j, n1 - 1 - i) = C3(s22, k, j, n1 - 1 - nb);
          C3(r33, k, j, i) = C3(r33, k, j, nb);
          C3(r33, k, j, n1 - 1 - i) = C3(r33, k, j, n1 - 1 - nb);
        }
    for (int k = 0; k < n3; k++)
      for (int j = 0; j < nb; j++)
        for (int i = 0; i < n1; i++) {
          C3(s11, k, j, i) = C3(s11, k, nb, i);
          C3(s11, k, n2 - 1 - j, i) = C3(s11, k, n2 - 1 - nb, i);
          C3(s22, k, j, i) = C3(s22, k, nb, i);
          C3(s22, k, n2 - 1 - j, i) = C3(s22, k, n2 - 1 - nb, i);
          C3(r33, k, j, i) = C3(r33, k, nb, i);
          C3(r33, k, n2 - 1 - j, i) = C3(r33, k, n2 - 1 - nb, i);
        }
    /* top: always air; bottom: row j=k of the deepest interior layer (sic) */
    for (int k = 0; k < nb; k++)
      for (int j = 0; j < n2; j++)
        for (int i = 0; i < n1; i++) {
          C3(s11, k, j, i) = 1. / rho_air;
          C3(s11, n3 - 1 - k, j, i) = C3(s11, n3 - 1 - nb, k, i);
          C3(s22, k, j, i) = 1. / rho_air;
          C3(s22, n3 - 1 - k, j, i) = C3(s22, n3 - 1 - nb, k, i);
          C3(r33, k, j, i) = rho_air;
          C3(r33, n3 - 1 - k, j, i) = C3(r33, n3 - 1 - nb, k, i);
        }
  }

  const double *d1 = g->d1, *d2 = g->d2, *d3 = g->d3, *d1s = g->d1s, *d2s = g->d2s, *d3s = g->d3s;
  g->sigma11 = (double *)calloc((size_t)n1 * (n2 + 1) * (n3 + 1), sizeof(double));
  g->sigma22 = (double *)calloc((size_t)(n1 + 1) * n2 * (n3 + 1), sizeof(double));
  g->sigma33 = (double *)calloc((size_t)(n1 + 1) * (n2 + 1) * n3, sizeof(double));
#define S11(k, j, i) g->sigma11[((size_t)(k) * (n2 + 1) + (j)) * n1 + (i)]
#define S22(k, j, i) g->sigma22[((size_t)(k) * n2 + (j)) * (n1 + 1) + (i)]
#define S33(k, j, i) g->sigma33[((size_t)(k) * (n2 + 1) + (j)) * (n1 + 1) + (i)]
  for (int k = 1; k < n3; k++) {
    int km1 = k - 1;
    for (int j = 1; j < n2; j++) {
      int jm1 = j - 1;
      for (int i = 0; i < n1; i++)
        S11(k, j, i) = 0.25 * ((d2s[j] * C3(s11, k, j, i) + d2s[jm1] * C3(s11, k, jm1, i)) * d3s[k] +
                               (d2s[j] * C3(s11, km1, j, i) + d2s[jm1] * C3(s11, km1, jm1, i)) * d3s[km1]) /
                       (d2[j] * d3[k]);
    }
  }
  for (int j = 0; j <= n2; j++)
    for (int i = 0; i < n1; i++) {
      S11(0, j, i) = S11(1, j, i);
      S11(n3, j, i) = S11(n3 - 1, j, i);
    }
  for (int k = 0; k <= n3; k++)
    for (int i = 0; i < n1; i++) {
      S11(k, 0, i) = S11(k, 1, i);
      S11(k, n2, i) = S11(k, n2 - 1, i);
    }
  for (int k = 1; k < n3; k++) {
    int km1 = k - 1;
    for (int j = 0; j < n2; j++)
      for (int i = 1; i < n1; i++) {
        int im1 = i - 1;
        S22(k, j, i) = 0.25 * ((d1s[i] * C3(s22, k, j, i) + d1s[im1] * C3(s22, k, j, im1)) * d3s[k] +
                               (d1s[i] * C3(s22, km1, j, i) + d1s[im1] * C3(s22, km1, j, im1)) * d3s[km1]) /
                       (d1[i] * d3[k]);
      }
  }
  for (int j = 0; j < n2; j++)
    for (int i = 0; i <= n1; i++) {
      S22(0, j, i) = S22(1, j, i);
      S22(n3, j, i) = S22(n3 - 1, j, i);
    }
  for (int k = 0; k <= n3; k++)
    for (int j = 0; j < n2; j++) {
      S22(k, j, 0) = S22(k, j, 1);
      S22(k, j, n1) = S22(k, j, n1 - 1);
    }
  for (int k = 0; k < n3; k++)
    for (int j = 1; j < n2; j++) {
      int jm1 = j - 1;
      for (int i = 1; i < n1; i++) {
        int im1 = i - 1;
        S33(k, j, i) = 0.25 * ((d1s[i] * C3(r33, k, j, i) + d1s[im1] * C3(r33, k, j, im1)) * d2s[j] +
                               (d1s[i] * C3(r33, k, jm1, i) + d1s[im1] * C3(r33, k, jm1, im1)) * d2s[jm1]) /
                       (d1[i] * d2[j]);
        S33(k, j, i) = 1. / S33(k, j, i);
      }
    }
  for (int k = 0; k < n3; k++)
    for (int j = 0; j <= n2; j++) {
      S33(k, j, 0) = S33(k, j, 1);
      S33(k, j, n1) = S33(k, j, n1 - 1);
    }
  for (int k = 0; k < n3; k++)
    for (int i = 0; i <= n1; i++) {
      S33(k, 0, i) = S33(k, 1, i);
      S33(k, n2, i) = S33(k, n2 - 1, i);
    }
#undef S11
#undef S22
#undef S33
#undef C3
  free(s11);
  free(s22);
  free(r33);
  return CSEM_OK;
}

int csem_grid_airbc(csem_grid_t *g, int n1fft, int n2fft)
{
  if (g->nb <= 0) return csem_set_error(CSEM_EINVAL, "airbc=1 assumes input model without air, you must ensure nb>0");
  g->n1fft = n1fft > 0 ? n1fft : 1024;
  g->n2fft = n2fft > 0 ? n2fft : 1024;
  int n1 = g->n1, n2 = g->n2, N1 = g->n1fft, N2 = g->n2fft;
  if (N1 < 2 || N2 < 2) return csem_set_error(CSEM_EINVAL, "n1fft, n2fft must be >= 2");
  g->d1fft = (g->x1[n1] - g->x1[0]) / (N1 - 1);
  g->d2fft = (g->x2[n2] - g->x2[0]) / (N2 - 1);
  g->d3fft = g->x3node[1] - g->x3node[0];
  free(g->sH1);
  free(g->sH2);
  g->sH1 = (double *)malloc(sizeof(double) * 2 * (size_t)N1 * N2);
  g->sH2 = (double *)malloc(sizeof(double) * 2 * (size_t)N1 * N2);
  double dkx = 2.0 * CSEM_PI / (g->d1fft * N1);
  double dky = 2.0 * CSEM_PI / (g->d2fft * N2);
  for (int i2 = 0; i2 < N2; i2++) {
    double ky = (i2 <= N2 / 2) ? i2 * dky : (i2 - N2) * dky;
    for (int i1 = 0; i1 < N1; i1++) {
      double kx = (i1 <= N1 / 2) ? i1 * dkx : (i1 - N1) * dkx;
      double kz = sqrt(kx * kx + ky * ky);
      /* same expression shapes as airbc_init_free.c:77-80 so every rounding matches */
      double _Complex s1 = exp(-kz * 0.5 * g->d3fft) * I * kx / (kz + 1.e-15);
      double _Complex s2 = exp(-kz * 0.5 * g->d3fft) * I * ky / (kz + 1.e-15);
      s1 *= cexp(-I * kx * 0.5 * g->d1s[0]);
      s2 *= cexp(-I * ky * 0.5 * g->d2s[0]);
      size_t o = 2 * ((size_t)i2 * N1 + i1);
      g->sH1[o] = creal(s1);
      g->sH1[o + 1] = cimag(s1);
      g->sH2[o] = creal(s2);
      g->sH2[o + 1] = cimag(s2);
    }
  }
  free(g->jx); free(g->jy); free(g->wx); free(g->wy);
  g->jx = (int *)calloc((size_t)N1, sizeof(int));
  g->jy = (int *)calloc((size_t)N2, sizeof(int));
  g->wx = (double *)calloc((size_t)N1, sizeof(double));
  g->wy = (double *)calloc((size_t)N2, sizeof(double));
  for (int i1 = 0; i1 < N1; i1++) {
    double x1 = g->x1s[0] + i1 * g->d1fft;
    if (x1 < g->x1s[n1 - 1]) {
      int j1 = csem_find_index(n1 + 1, g->x1s, x1);
      g->jx[i1] = j1;
      g->wx[i1] = (x1 - g->x1s[j1]) / (g->x1s[j1 + 1] - g->x1s[j1]);
    }
  }
  for (int i2 = 0; i2 < N2; i2++) {
    double x2 = g->x2s[0] + i2 * g->d2fft;
    if (x2 < g->x2s[n2 - 1]) {
      int j2 = csem_find_index(n2 + 1, g->x2s, x2);
      g->jy[i2] = j2;
      g->wy[i2] = (x2 - g->x2s[j2]) / (g->x2s[j2 + 1] - g->x2s[j2]);
    }
  }
  return CSEM_OK;
}

void csem_grid_free(csem_grid_t *g)
{
  void *ptrs[] = {g->x1node, g->x2node, g->x3node, g->rho11, g->rho22, g->rho33,
                  g->x1, g->x2, g->x3, g->x1s, g->x2s, g->x3s, g->d1, g->d2, g->d3,
                  g->d1s, g->d2s, g->d3s, g->sigma11, g->sigma22, g->sigma33,
                  g->sH1, g->sH2, g->jx, g->jy, g->wx, g->wy};
  for (size_t i = 0; i < sizeof(ptrs) / sizeof(ptrs[0]); i++) free(ptrs[i]);
  memset(g, 0, sizeof(*g));
}

int csem_grid_write_extended(const csem_grid_t *g, const char *dir)
{
  /* rebuild the padded cell arrays the way extend_model.c:126-177 holds them and
   * write them as resistivity (extend_model.c:254-289) */
  char path[4096];
  int n1 = g->n1, n2 = g->n2, n3 = g->n3, nb = g->nb;
  size_t nc = (size_t)n1 * n2 * n3;
  double *a[3];
  for (int c = 0; c < 3; c++) a[c] = (double *)calloc(nc, sizeof(double));
  const float *rho[3] = {g->rho11, g->rho22, g->rho33};
  for (int c = 0; c < 3; c++) {
    double *s = a[c];
#define C3(k, j, i) s[((size_t)(k) * n2 + (j)) * n1 + (i)]
    for (int k = 0; k < g->nz; k++)
      for (int j = 0; j < g->ny; j++)
        for (int i = 0; i < g->nx; i++) {
          double v = rho[c][((size_t)k * g->ny + j) * g->nx + i];
          C3(k + nb, j + nb, i + nb) = c < 2 ? 1. / v : v;
        }
    if (nb > 0) {
      for (int k = 0; k < n3; k++)
        for (int j = 0; j < n2; j++)
          for (int i = 0; i < nb; i++) {
            C3(k, j, i) = C3(k, j, nb);
            C3(k, j, n1 - 1 - i) = C3(k, j, n1 - 1 - nb);
          }
      for (int k = 0; k < n3; k++)
        for (int j = 0; j < nb; j++)
          for (int i = 0; i < n1; i++) {
            C3(k, j, i) = C3(k, nb, i);
            C3(k, n2 - 1 - j, i) = C3(k, n2 - 1 - nb, i);
          }
      for (int k = 0; k < nb; k++)
        for (int j = 0; j < n2; j++)
          for (int i = 0; i < n1; i++) {
            C3(k, j, i) = c < 2 ? 1. / g->rho_air : g->rho_air;
            C3(n3 - 1 - k, j, i) = C3(n3 - 1 - nb, k, i);
          }
    }
    if (c < 2)
      for (size_t q = 0; q < nc; q++) s[q] = 1. / s[q];
#undef C3
  }
  const char *names[3] = {"frho11_extended", "frho22_extended", "frho33_extended"};
  for (int c = 0; c < 3; c++) {
    snprintf(path, sizeof(path), "%s/%s", dir, names[c]);
    FILE *fp = fopen(path, "wb");
    if (!fp) return csem_set_error(CSEM_EIO, "cannot write %s", path);
    fwrite(a[c], sizeof(double), nc, fp);
    fclose(fp);
    free(a[c]);
  }
  const double *xs[3] = {g->x1, g->x2, g->x3};
  int ns[3] = {n1, n2, n3};
  const char *xn[3] = {"fx1_extended", "fx2_extended", "fx3_extended"};
  for (int c = 0; c < 3; c++) {
    snprintf(path, sizeof(path), "%s/%s", dir, xn[c]);
    FILE *fp = fopen(path, "wb");
    if (!fp) return csem_set_error(CSEM_EIO, "cannot write %s", path);
    fwrite(xs[c], sizeof(double), (size_t)ns[c] + 1, fp);
    fclose(fp);
  }
  return CSEM_OK;
}

/* ------------------------------------------------------------ acquisition */
static int read_rows(const char *path, float *rows, int *count)
{
  FILE *fp = fopen(path, "r");
  if (!fp) return csem_set_error(CSEM_EIO, "file does not exist! (%s)", path);
  float x, y, z, hd, pit;
  int idx, n = 0;
  if (fscanf(fp, "%*[^\n]\n") == EOF) { fclose(fp); *count = 0; return CSEM_OK; }
  while (1) {
    int st = fscanf(fp, "%f %f %f %f %f %d", &x, &y, &z, &hd, &pit, &idx);
    if (st == EOF) break;
    if (n >= CSEM_MAX_ACQ_ROWS) {
      fclose(fp);
      return csem_set_error(CSEM_ETOOBIG, "%s holds more than %d rows", path, CSEM_MAX_ACQ_ROWS);
    }
    if (st < 5) { /* a malformed row would make the reference loop forever; refuse it */
      fclose(fp);
      return csem_set_error(CSEM_EIO, "%s: malformed row %d", path, n + 2);
    }
    rows[5 * n + 0] = x; rows[5 * n + 1] = y; rows[5 * n + 2] = z;
    rows[5 * n + 3] = hd; rows[5 * n + 4] = pit;
    n++;
  }
  fclose(fp);
  *count = n;
  return CSEM_OK;
}

int csem_acq_read(csem_acq_t *a, const char *fsrc, const char *frec)
{
  memset(a, 0, sizeof(*a));
  float *buf = (float *)malloc(sizeof(float) * 5 * CSEM_MAX_ACQ_ROWS);
  int n, rc = read_rows(fsrc, buf, &n);
  if (rc) { free(buf); return rc; }
  if (n < 1) { free(buf); return csem_set_error(CSEM_EIO, "%s holds no source row", fsrc); }
  a->nsrc = n;
  a->src = (float *)malloc(sizeof(float) * 5 * (size_t)n);
  memcpy(a->src, buf, sizeof(float) * 5 * (size_t)n);
  rc = read_rows(frec, buf, &n);
  if (rc) { free(buf); return rc; }
  a->nrec = n;
  a->rec = (float *)malloc(sizeof(float) * 5 * (size_t)(n > 0 ? n : 1));
  memcpy(a->rec, buf, sizeof(float) * 5 * (size_t)n);
  free(buf);
  return CSEM_OK;
}

int csem_acq_check(const csem_acq_t *a, const csem_grid_t *g)
{
  /* the reference bounds only source 0 and the receivers (acq_init_free.c:84-138);
   * every source row is checked here because every row may be solved */
  float mn[3], mx[3];
  for (int c = 0; c < 3; c++) mn[c] = mx[c] = a->src[c];
  for (int s = 0; s < a->nsrc; s++)
    for (int c = 0; c < 3; c++) {
      float v = a->src[5 * s + c];
      mn[c] = mn[c] < v ? mn[c] : v;
      mx[c] = mx[c] > v ? mx[c] : v;
    }
  for (int r = 0; r < a->nrec; r++)
    for (int c = 0; c < 3; c++) {
      float v = a->rec[5 * r + c];
      mn[c] = mn[c] < v ? mn[c] : v;
      mx[c] = mx[c] > v ? mx[c] : v;
    }
  const float *node[3] = {g->x1node, g->x2node, g->x3node};
  int nn[3] = {g->nx, g->ny, g->nz};
  for (int c = 0; c < 3; c++) {
    if (node[c][0] > mn[c]) return csem_set_error(CSEM_EDOMAIN, "x%d origin > acq->x%dmin", c + 1, c + 1);
    if (node[c][nn[c]] < mx[c]) return csem_set_error(CSEM_EDOMAIN, "x%d end < acq->x%dmin", c + 1, c + 1);
  }
  return CSEM_OK;
}

void csem_acq_free(csem_acq_t *a)
{
  free(a->src);
  free(a->rec);
  memset(a, 0, sizeof(*a));
}

/* ------------------------------------------------------------------ output */
int csem_history_logged(int algopt, int preco, int status, int nh)
{
  if (nh <= 0 || status == CSEM_ST_ZERO_RHS) return 0;
  if (algopt == 1) return nh > 1 ? nh - 1 : 1;
  return preco == 0 && status == CSEM_ST_CONVERGED ? nh - 1 : nh;
}

int csem_write_emf(const char *fname, int isrc, int nchrec, int nfreq, int nrec, const float *dcal)
{
  FILE *fp = fopen(fname, "w");
  if (!fp) return csem_set_error(CSEM_EIO, "error opening file for writing");
  fprintf(fp, "iTx \t iRx    ichrec  ifreq \t emf_real \t emf_imag\n");
  for (int ic = 0; ic < nchrec; ic++)
    for (int f = 0; f < nfreq; f++)
      for (int r = 0; r < nrec; r++) {
        size_t o = 2 * (((size_t)ic * nfreq + f) * nrec + r);
        float re = dcal[o], im = dcal[o + 1];
        fprintf(fp, "%d \t %d \t %d \t %d \t %e \t %e\n", isrc, r + 1, ic + 1, f + 1, re, im);
      }
  fclose(fp);
  return CSEM_OK;
}

static int cmp_bits(const void *a, const void *b)
{
  int x, y;
  memcpy(&x, a, sizeof(int));
  memcpy(&y, b, sizeof(int));
  return x - y;
}

void csem_sort_freqs(float *freqs, int n) { qsort(freqs, (size_t)n, sizeof(float), cmp_bits); }
