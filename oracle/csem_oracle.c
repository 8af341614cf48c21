/* CPU oracle for the GB300 CSEM solver - TEST INFRASTRUCTURE ONLY (see csem_oracle.h).
 * Each routine names the reference lines it restates. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "csem_oracle.h"
#include "fft2d.h"

#define ORC_PI 3.14159265358979323846264
#define ORC_MU0 (4. * ORC_PI * 1e-7)

typedef struct { double re, im; } cz;

static inline cz mk(double re, double im) { cz r = {re, im}; return r; }
static inline cz cadd(cz a, cz b) { return mk(a.re + b.re, a.im + b.im); }
static inline cz csub(cz a, cz b) { return mk(a.re - b.re, a.im - b.im); }
static inline cz cmul(cz a, cz b) { return mk(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re); }
static inline cz cdivr(cz a, double d) { return mk(a.re / d, a.im / d); }
static inline cz rmul(double s, cz a) { return mk(s * a.re, s * a.im); }
static inline cz cneg(cz a) { return mk(-a.re, -a.im); }
static inline cz cconj(cz a) { return mk(a.re, -a.im); }
/* Smith 1962 */
static inline cz cdiv(cz a, cz b)
{
  double r, den;
  if (fabs(b.re) < fabs(b.im)) {
    r = b.re / b.im;
    den = b.re * r + b.im;
    return mk((a.re * r + a.im) / den, (a.im * r - a.re) / den);
  }
  r = b.im / b.re;
  den = b.im * r + b.re;
  return mk((a.im * r + a.re) / den, (a.im - a.re * r) / den);
}
static inline double cabs_(cz a) { return hypot(a.re, a.im); }

static inline cz ld(const double *v, long i) { return mk(v[2 * i], v[2 * i + 1]); }
static inline void st(double *v, long i, cz a) { v[2 * i] = a.re; v[2 * i + 1] = a.im; }

struct orc_ctx {
  orc_desc_t d;
  int n1, n2, n3;               /* operator grid */
  int kstart;                   /* nb when airbc, else 0 */
  long lEx, lEy, lEz, lE, lHx, lHy, lHz, lH, lv;
  cz iom;                       /* I omega mu0 */
  double *xh;                   /* H = [Hx | Hy | Hz] (fdfd.c:58-61 lengths) */
  double *hxkm1, *hykm1;        /* airwave ghosts */
  double *kxky, *kxky0;         /* uniform airwave grid (+1 zero guard row) */
  double *xx, *yy;              /* LU-SGS full-grid scratch (fdfd.c:41-48) */
  double *v, *bv;               /* A-phi node potential (fdfd.c:33-39) */
  double *gw;                   /* inner GMRES workspace */
  int gm;
};

orc_ctx_t *orc_create(const orc_desc_t *d)
{
  orc_ctx_t *c = (orc_ctx_t *)calloc(1, sizeof(orc_ctx_t));
  c->d = *d;
  int n1 = d->n1, n2 = d->n2;
  /* fdfd.c:40-62 */
  int n3full = d->n3f;
  long lExf = (long)n1 * (n2 + 1) * (n3full + 1), lEyf = (long)(n1 + 1) * n2 * (n3full + 1),
       lEzf = (long)(n1 + 1) * (n2 + 1) * n3full;
  c->xx = (double *)calloc(2 * (size_t)(lExf + lEyf + lEzf), sizeof(double));
  c->yy = (double *)calloc(2 * (size_t)(lExf + lEyf + lEzf), sizeof(double));
  int n3 = d->airbc ? d->nz + d->nb : n3full;
  c->n1 = n1;
  c->n2 = n2;
  c->n3 = n3;
  c->kstart = d->airbc ? d->nb : 0;
  c->lEx = (long)n1 * (n2 + 1) * (n3 + 1);
  c->lEy = (long)(n1 + 1) * n2 * (n3 + 1);
  c->lEz = (long)(n1 + 1) * (n2 + 1) * n3;
  c->lE = c->lEx + c->lEy + c->lEz;
  c->lHx = (long)(n1 + 1) * n2 * n3;
  c->lHy = (long)n1 * (n2 + 1) * n2; /* sic: fdfd.c:59 uses n2 for the last factor */
  c->lHz = (long)n1 * n2 * (n3 + 1);
  c->lH = c->lHx + c->lHy + c->lHz;
  c->lv = (long)(n1 + 1) * (n2 + 1) * (n3 + 1);
  /* Hy is written up to n1*(n2+1)*n3 past its start; size the buffer for that, and for
     the corrected Hy length (orc_set_hy_length) */
  long hneed = c->lHx + (long)n1 * (n2 + 1) * (n3 > n2 ? n3 : n2) + c->lHz;
  c->xh = (double *)calloc(2 * (size_t)hneed, sizeof(double));
  c->v = (double *)calloc(2 * (size_t)c->lv, sizeof(double));
  c->bv = (double *)calloc(2 * (size_t)c->lv, sizeof(double));
  if (d->airbc) {
    c->hxkm1 = (double *)calloc(2 * (size_t)(n1 + 1) * n2, sizeof(double));
    c->hykm1 = (double *)calloc(2 * (size_t)n1 * (n2 + 1), sizeof(double));
    size_t nf = (size_t)d->n1fft * d->n2fft + (size_t)d->n1fft + 1;
    c->kxky = (double *)calloc(2 * nf, sizeof(double));
    c->kxky0 = (double *)calloc(2 * nf, sizeof(double));
  }
  return c;
}

void orc_destroy(orc_ctx_t *c)
{
  if (!c) return;
  free(c->xh); free(c->hxkm1); free(c->hykm1); free(c->kxky); free(c->kxky0);
  free(c->xx); free(c->yy); free(c->v); free(c->bv); free(c->gw);
  free(c);
}

void orc_set_iom(orc_ctx_t *c, double re, double im) { c->iom = mk(re, im); }

void orc_set_freq(orc_ctx_t *c, float freq)
{
  /* main.c:95: I*2.*PI*freq*mu0, evaluated left to right on (0,1) */
  cz z = mk(0.0, 1.0);
  z = rmul(2., z);
  z = rmul(ORC_PI, z);
  z = rmul((double)freq, z);
  z = rmul(ORC_MU0, z);
  c->iom = mk(z.re, z.im);
}

void orc_sizes(const orc_ctx_t *c, long *o)
{
  o[0] = c->lE; o[1] = c->lEx; o[2] = c->lEy; o[3] = c->lEz; o[4] = c->lH; o[5] = c->lv; o[6] = c->n3;
}

void orc_set_hy_length(orc_ctx_t *c, int sic)
{
  /* sic != 0: fdfd.c:59's n1*(n2+1)*n2, so that Hz starts inside Hy when n2 < n3 and the
     two overlap; sic == 0: n1*(n2+1)*n3, disjoint. Identical whenever n2 == n3, and the
     overlap is absent whenever n2 >= n3. */
  c->lHy = (long)c->n1 * (c->n2 + 1) * (sic ? c->n2 : c->n3);
  c->lH = c->lHx + c->lHy + c->lHz;
}

void orc_get_h(const orc_ctx_t *c, double *h) { memcpy(h, c->xh, sizeof(double) * 2 * (size_t)c->lH); }

static cz iwmu_of(const orc_ctx_t *c) { return cdiv(mk(1.0, 0.0), c->iom); }

/* ------------------------------------------------------------ airwave */
void orc_airbc_apply(orc_ctx_t *c, const double *H3k, double *H1km1, double *H2km1)
{
  /* airbc_init_free.c:130-209 */
  const orc_desc_t *d = &c->d;
  int n1 = c->n1, n2 = c->n2, N1 = d->n1fft, N2 = d->n2fft;
  double *K = c->kxky, *K0 = c->kxky0;
  for (int i2 = 0; i2 < N2; i2++) {
    double x2 = d->x2s[0] + i2 * d->d2fft;
    for (int i1 = 0; i1 < N1; i1++) {
      double x1 = d->x1s[0] + i1 * d->d1fft;
      cz val = mk(0., 0.);
      if (x1 < d->x1s[n1 - 1] && x2 < d->x2s[n2 - 1]) {
        int j1 = d->jx[i1], j2 = d->jy[i2];
        double w1 = d->wx[i1], w2 = d->wy[i2];
        cz a = rmul((1. - w1) * (1. - w2), ld(H3k, j1 + (long)n1 * j2));
        cz b = rmul(w1 * (1. - w2), ld(H3k, j1 + 1 + (long)n1 * j2));
        cz e = rmul((1. - w1) * w2, ld(H3k, j1 + (long)n1 * (j2 + 1)));
        cz f = rmul(w1 * w2, ld(H3k, j1 + 1 + (long)n1 * (j2 + 1)));
        val = cadd(cadd(cadd(a, b), e), f);
      }
      st(K, i1 + (long)N1 * i2, val);
    }
  }
  csem_fft2d(N1, N2, K, -1);
  memcpy(K0, K, sizeof(double) * 2 * (size_t)N1 * N2);
  for (int pass = 0; pass < 2; pass++) {
    const double *filt = pass == 0 ? d->sH1 : d->sH2;
    for (long q = 0; q < (long)N1 * N2; q++) st(K, q, cmul(ld(K0, q), ld(filt, q)));
    csem_fft2d(N1, N2, K, +1);
    double nn = (double)(N1 * N2);
    for (long q = 0; q < (long)N1 * N2; q++) st(K, q, cdivr(ld(K, q), nn));
    /* the guard row past the end stays zero (reads of j+1 == N at the last node) */
    if (pass == 0) {
      for (int i2 = 0; i2 < n2; i2++) {
        double s2 = d->x2s[i2] - d->x2s[0];
        int j2 = (int)(s2 / d->d2fft);
        double w2 = s2 / d->d2fft - j2;
        for (int i1 = 0; i1 <= n1; i1++) {
          double s1 = d->x1[i1] - d->x1[0];
          int j1 = (int)(s1 / d->d1fft);
          double w1 = s1 / d->d1fft - j1;
          cz a = rmul((1. - w1) * (1. - w2), ld(K, j1 + (long)N1 * j2));
          cz b = rmul(w1 * (1. - w2), ld(K, j1 + 1 + (long)N1 * j2));
          cz e = rmul((1. - w1) * w2, ld(K, j1 + (long)N1 * (j2 + 1)));
          cz f = rmul(w1 * w2, ld(K, j1 + 1 + (long)N1 * (j2 + 1)));
          st(H1km1, i1 + (long)(n1 + 1) * i2, cadd(cadd(cadd(a, b), e), f));
        }
      }
    } else {
      for (int i2 = 0; i2 <= n2; i2++) {
        double s2 = d->x2[i2] - d->x2[0];
        int j2 = (int)(s2 / d->d2fft);
        double w2 = s2 / d->d2fft - j2;
        for (int i1 = 0; i1 < n1; i1++) {
          double s1 = d->x1s[i1] - d->x1s[0];
          int j1 = (int)(s1 / d->d1fft);
          double w1 = s1 / d->d1fft - j1;
          cz a = rmul((1. - w1) * (1. - w2), ld(K, j1 + (long)N1 * j2));
          cz b = rmul(w1 * (1. - w2), ld(K, j1 + 1 + (long)N1 * j2));
          cz e = rmul((1. - w1) * w2, ld(K, j1 + (long)N1 * (j2 + 1)));
          cz f = rmul(w1 * w2, ld(K, j1 + 1 + (long)N1 * (j2 + 1)));
          st(H2km1, i1 + (long)n1 * i2, cadd(cadd(cadd(a, b), e), f));
        }
      }
    }
  }
}

/* ------------------------------------------------------------ operator */
void orc_fdfd_apply(orc_ctx_t *c, const double *x, double *y)
{
  /* fdfd.c:86-205 */
  const orc_desc_t *D = &c->d;
  int n1 = c->n1, n2 = c->n2, n3 = c->n3, ks = c->kstart;
  const double *d1 = D->d1, *d2 = D->d2, *d3 = D->d3 + ks, *d1s = D->d1s, *d2s = D->d2s, *d3s = D->d3s + ks;
  const double *s11 = D->sigma11 + (long)ks * (n2 + 1) * n1;
  const double *s22 = D->sigma22 + (long)ks * n2 * (n1 + 1);
  const double *s33 = D->sigma33 + (long)ks * (n2 + 1) * (n1 + 1);
  const double *Ex = x, *Ey = x + 2 * c->lEx, *Ez = x + 2 * (c->lEx + c->lEy);
  double *Hx = c->xh, *Hy = c->xh + 2 * c->lHx, *Hz = c->xh + 2 * (c->lHx + c->lHy);
  double *bx = y, *by = y + 2 * c->lEx, *bz = y + 2 * (c->lEx + c->lEy);
  cz iwmu = iwmu_of(c);
#define I1(k, j, i) ((i) + (long)n1 * ((j) + (long)(n2 + 1) * (k)))
#define I2(k, j, i) ((i) + (long)(n1 + 1) * ((j) + (long)n2 * (k)))
#define I3(k, j, i) ((i) + (long)(n1 + 1) * ((j) + (long)(n2 + 1) * (k)))
#define IX(k, j, i) ((i) + (long)(n1 + 1) * ((j) + (long)n2 * (k)))
#define IY(k, j, i) ((i) + (long)n1 * ((j) + (long)(n2 + 1) * (k)))
#define IZ(k, j, i) ((i) + (long)n1 * ((j) + (long)n2 * (k)))
  memset(y, 0, sizeof(double) * 2 * (size_t)c->lE);
  for (int k = 0; k <= n3; k++)
    for (int j = 0; j <= n2; j++)
      for (int i = 0; i <= n1; i++) {
        if (j < n2 && k < n3) {
          cz t1 = cdivr(csub(ld(Ez, I3(k, j + 1, i)), ld(Ez, I3(k, j, i))), d2s[j]);
          cz t2 = cdivr(csub(ld(Ey, I2(k + 1, j, i)), ld(Ey, I2(k, j, i))), d3s[k]);
          st(Hx, IX(k, j, i), cmul(csub(t1, t2), iwmu));
        }
        if (i < n1 && k < n3) {
          cz t1 = cdivr(csub(ld(Ex, I1(k + 1, j, i)), ld(Ex, I1(k, j, i))), d3s[k]);
          cz t2 = cdivr(csub(ld(Ez, I3(k, j, i + 1)), ld(Ez, I3(k, j, i))), d1s[i]);
          st(Hy, IY(k, j, i), cmul(csub(t1, t2), iwmu));
        }
        if (i < n1 && j < n2) {
          cz t1 = cdivr(csub(ld(Ey, I2(k, j, i + 1)), ld(Ey, I2(k, j, i))), d1s[i]);
          cz t2 = cdivr(csub(ld(Ex, I1(k, j + 1, i)), ld(Ex, I1(k, j, i))), d2s[j]);
          st(Hz, IZ(k, j, i), cmul(csub(t1, t2), iwmu));
        }
      }
  if (D->airbc) {
    orc_airbc_apply(c, Hz, c->hxkm1, c->hykm1);
    const double *Hxk = c->hxkm1, *Hyk = c->hykm1;
    int k = 0;
    for (int j = 0; j < n2; j++)
      for (int i = 0; i < n1; i++) {
        if (j > 0) {
          cz t1 = cdivr(csub(ld(Hz, IZ(k, j, i)), ld(Hz, IZ(k, j - 1, i))), d2[j]);
          cz t2 = cdivr(csub(ld(Hy, IY(k, j, i)), ld(Hyk, i + (long)n1 * j)), d3[k]);
          cz r = csub(csub(t1, t2), rmul(s11[I1(k, j, i)], ld(Ex, I1(k, j, i))));
          if (D->fvm) r = cmul(r, rmul(d1s[i] * d2[j] * d3[k], c->iom));
          st(bx, I1(k, j, i), r);
        }
        if (i > 0) {
          cz t1 = cdivr(csub(ld(Hx, IX(k, j, i)), ld(Hxk, i + (long)(n1 + 1) * j)), d3[k]);
          cz t2 = cdivr(csub(ld(Hz, IZ(k, j, i)), ld(Hz, IZ(k, j, i - 1))), d1[i]);
          cz r = csub(csub(t1, t2), rmul(s22[I2(k, j, i)], ld(Ey, I2(k, j, i))));
          if (D->fvm) r = cmul(r, rmul(d1[i] * d2s[j] * d3[k], c->iom));
          st(by, I2(k, j, i), r);
        }
      }
  }
  for (int k = 0; k < n3; k++)
    for (int j = 0; j < n2; j++)
      for (int i = 0; i < n1; i++) {
        if (j > 0 && k > 0) {
          cz t1 = cdivr(csub(ld(Hz, IZ(k, j, i)), ld(Hz, IZ(k, j - 1, i))), d2[j]);
          cz t2 = cdivr(csub(ld(Hy, IY(k, j, i)), ld(Hy, IY(k - 1, j, i))), d3[k]);
          cz r = csub(csub(t1, t2), rmul(s11[I1(k, j, i)], ld(Ex, I1(k, j, i))));
          if (D->fvm) r = cmul(r, rmul(d1s[i] * d2[j] * d3[k], c->iom));
          st(bx, I1(k, j, i), r);
        }
        if (i > 0 && k > 0) {
          cz t1 = cdivr(csub(ld(Hx, IX(k, j, i)), ld(Hx, IX(k - 1, j, i))), d3[k]);
          cz t2 = cdivr(csub(ld(Hz, IZ(k, j, i)), ld(Hz, IZ(k, j, i - 1))), d1[i]);
          cz r = csub(csub(t1, t2), rmul(s22[I2(k, j, i)], ld(Ey, I2(k, j, i))));
          if (D->fvm) r = cmul(r, rmul(d1[i] * d2s[j] * d3[k], c->iom));
          st(by, I2(k, j, i), r);
        }
        if (i > 0 && j > 0) {
          cz t1 = cdivr(csub(ld(Hy, IY(k, j, i)), ld(Hy, IY(k, j, i - 1))), d1[i]);
          cz t2 = cdivr(csub(ld(Hx, IX(k, j, i)), ld(Hx, IX(k, j - 1, i))), d2[j]);
          cz r = csub(csub(t1, t2), rmul(s33[I3(k, j, i)], ld(Ez, I3(k, j, i))));
          if (D->fvm) r = cmul(r, rmul(d1[i] * d2[j] * d3s[k], c->iom));
          st(bz, I3(k, j, i), r);
        }
      }
}

void orc_fdfd_apply_old(orc_ctx_t *c, const double *x, double *y)
{
  /* fdfd.c:212-284 (full grid arrays, no kstart shift, Dirichlet everywhere) */
  const orc_desc_t *D = &c->d;
  int n1 = c->n1, n2 = c->n2, n3 = c->n3;
  const double *d1 = D->d1, *d2 = D->d2, *d3 = D->d3, *d1s = D->d1s, *d2s = D->d2s, *d3s = D->d3s;
  const double *s11 = D->sigma11, *s22 = D->sigma22, *s33 = D->sigma33;
  const double *Ex = x, *Ey = x + 2 * c->lEx, *Ez = x + 2 * (c->lEx + c->lEy);
  double *bx = y, *by = y + 2 * c->lEx, *bz = y + 2 * (c->lEx + c->lEy);
  cz iwmu = iwmu_of(c);
  memset(y, 0, sizeof(double) * 2 * (size_t)c->lE);
  for (int k = 0; k < n3; k++) {
    int kp1 = k + 1 < n3 ? k + 1 : n3, km1 = k - 1 > 0 ? k - 1 : 0;
    for (int j = 0; j < n2; j++) {
      int jp1 = j + 1 < n2 ? j + 1 : n2, jm1 = j - 1 > 0 ? j - 1 : 0;
      for (int i = 0; i < n1; i++) {
        int ip1 = i + 1 < n1 ? i + 1 : n1, im1 = i - 1 > 0 ? i - 1 : 0;
        if (j > 0 && k > 0) {
          cz t1 = csub(cdivr(csub(ld(Ey, I2(k, j, ip1)), ld(Ey, I2(k, j, i))), d1s[i]),
                       cdivr(csub(ld(Ex, I1(k, jp1, i)), ld(Ex, I1(k, j, i))), d2s[j]));
          cz t2 = csub(cdivr(csub(ld(Ey, I2(k, jm1, ip1)), ld(Ey, I2(k, jm1, i))), d1s[i]),
                       cdivr(csub(ld(Ex, I1(k, j, i)), ld(Ex, I1(k, jm1, i))), d2s[jm1]));
          cz t3 = csub(cdivr(csub(ld(Ex, I1(kp1, j, i)), ld(Ex, I1(k, j, i))), d3s[k]),
                       cdivr(csub(ld(Ez, I3(k, j, ip1)), ld(Ez, I3(k, j, i))), d1s[i]));
          cz t4 = csub(cdivr(csub(ld(Ex, I1(k, j, i)), ld(Ex, I1(km1, j, i))), d3s[km1]),
                       cdivr(csub(ld(Ez, I3(km1, j, ip1)), ld(Ez, I3(km1, j, i))), d1s[i]));
          cz r = csub(cmul(csub(cdivr(csub(t1, t2), d2[j]), cdivr(csub(t3, t4), d3[k])), iwmu),
                      rmul(s11[I1(k, j, i)], ld(Ex, I1(k, j, i))));
          if (D->fvm) r = cmul(r, rmul(d1s[i] * d2[j] * d3[k], c->iom));
          st(bx, I1(k, j, i), r);
        }
        if (i > 0 && k > 0) {
          cz t1 = csub(cdivr(csub(ld(Ez, I3(k, jp1, i)), ld(Ez, I3(k, j, i))), d2s[j]),
                       cdivr(csub(ld(Ey, I2(kp1, j, i)), ld(Ey, I2(k, j, i))), d3s[k]));
          cz t2 = csub(cdivr(csub(ld(Ez, I3(km1, jp1, i)), ld(Ez, I3(km1, j, i))), d2s[j]),
                       cdivr(csub(ld(Ey, I2(k, j, i)), ld(Ey, I2(km1, j, i))), d3s[km1]));
          cz t3 = csub(cdivr(csub(ld(Ey, I2(k, j, ip1)), ld(Ey, I2(k, j, i))), d1s[i]),
                       cdivr(csub(ld(Ex, I1(k, jp1, i)), ld(Ex, I1(k, j, i))), d2s[j]));
          cz t4 = csub(cdivr(csub(ld(Ey, I2(k, j, i)), ld(Ey, I2(k, j, im1))), d1s[im1]),
                       cdivr(csub(ld(Ex, I1(k, jp1, im1)), ld(Ex, I1(k, j, im1))), d2s[j]));
          cz r = csub(cmul(csub(cdivr(csub(t1, t2), d3[k]), cdivr(csub(t3, t4), d1[i])), iwmu),
                      rmul(s22[I2(k, j, i)], ld(Ey, I2(k, j, i))));
          if (D->fvm) r = cmul(r, rmul(d1[i] * d2s[j] * d3[k], c->iom));
          st(by, I2(k, j, i), r);
        }
        if (i > 0 && j > 0) {
          cz t1 = csub(cdivr(csub(ld(Ex, I1(kp1, j, i)), ld(Ex, I1(k, j, i))), d3s[k]),
                       cdivr(csub(ld(Ez, I3(k, j, ip1)), ld(Ez, I3(k, j, i))), d1s[i]));
          cz t2 = csub(cdivr(csub(ld(Ex, I1(kp1, j, im1)), ld(Ex, I1(k, j, im1))), d3s[k]),
                       cdivr(csub(ld(Ez, I3(k, j, i)), ld(Ez, I3(k, j, im1))), d1s[im1]));
          cz t3 = csub(cdivr(csub(ld(Ez, I3(k, jp1, i)), ld(Ez, I3(k, j, i))), d2s[j]),
                       cdivr(csub(ld(Ey, I2(kp1, j, i)), ld(Ey, I2(k, j, i))), d3s[k]));
          cz t4 = csub(cdivr(csub(ld(Ez, I3(k, j, i)), ld(Ez, I3(k, jm1, i))), d2s[jm1]),
                       cdivr(csub(ld(Ey, I2(kp1, jm1, i)), ld(Ey, I2(k, jm1, i))), d3s[k]));
          cz r = csub(cmul(csub(cdivr(csub(t1, t2), d1[i]), cdivr(csub(t3, t4), d2[j])), iwmu),
                      rmul(s33[I3(k, j, i)], ld(Ez, I3(k, j, i))));
          if (D->fvm) r = cmul(r, rmul(d1[i] * d2[j] * d3s[k], c->iom));
          st(bz, I3(k, j, i), r);
        }
      }
    }
  }
}

/* ------------------------------------------------------------ LU-SGS rows */
typedef struct {
  int n1, n2, n3;
  const double *d1, *d2, *d3, *d1s, *d2s, *d3s, *s11, *s22, *s33;
  double *Ex, *Ey, *Ez;
  const double *bx, *by, *bz;
  cz iwmu, iom;
  int fvm;
  const double *v;   /* A-phi potential (NULL for LU-SGS) */
} rows_t;

#define RI1(k, j, i) ((i) + (long)R->n1 * ((j) + (long)(R->n2 + 1) * (k)))
#define RI2(k, j, i) ((i) + (long)(R->n1 + 1) * ((j) + (long)R->n2 * (k)))
#define RI3(k, j, i) ((i) + (long)(R->n1 + 1) * ((j) + (long)(R->n2 + 1) * (k)))

/* Ex row update (fdfd.c:357-369; A-phi variant fdfd.c:586-598 with the v term) */
static void row_ex(const rows_t *R, int k, int j, int i)
{
  const double *d1s = R->d1s, *d2s = R->d2s, *d3s = R->d3s, *d2 = R->d2, *d3 = R->d3;
  long p = RI1(k, j, i);
  st(R->Ex, p, mk(0., 0.));
  const double *Ex = R->Ex, *Ey = R->Ey, *Ez = R->Ez;
  cz t1 = csub(cdivr(csub(ld(Ey, RI2(k, j, i + 1)), ld(Ey, RI2(k, j, i))), d1s[i]),
               cdivr(csub(ld(Ex, RI1(k, j + 1, i)), ld(Ex, RI1(k, j, i))), d2s[j]));
  cz t2 = csub(cdivr(csub(ld(Ey, RI2(k, j - 1, i + 1)), ld(Ey, RI2(k, j - 1, i))), d1s[i]),
               cdivr(csub(ld(Ex, RI1(k, j, i)), ld(Ex, RI1(k, j - 1, i))), d2s[j - 1]));
  cz t3 = csub(cdivr(csub(ld(Ex, RI1(k + 1, j, i)), ld(Ex, RI1(k, j, i))), d3s[k]),
               cdivr(csub(ld(Ez, RI3(k, j, i + 1)), ld(Ez, RI3(k, j, i))), d1s[i]));
  cz t4 = csub(cdivr(csub(ld(Ex, RI1(k, j, i)), ld(Ex, RI1(k - 1, j, i))), d3s[k - 1]),
               cdivr(csub(ld(Ez, RI3(k - 1, j, i + 1)), ld(Ez, RI3(k - 1, j, i))), d1s[i]));
  double sg = R->s11[p];
  cz own = ld(Ex, p);
  if (R->v) own = cadd(own, cdivr(csub(ld(R->v, RI3(k, j, i + 1)), ld(R->v, RI3(k, j, i))), d1s[i]));
  cz aij = csub(cmul(csub(cdivr(csub(t1, t2), d2[j]), cdivr(csub(t3, t4), d3[k])), R->iwmu), rmul(sg, own));
  double g = (1. / d2s[j] + 1. / d2s[j - 1]) / d2[j] + (1. / d3s[k] + 1. / d3s[k - 1]) / d3[k];
  cz aii = rmul(g, R->iwmu);
  aii = mk(aii.re - sg, aii.im);
  if (R->fvm) {
    double vol = R->d1s[i] * d2[j] * d3[k];
    aij = cmul(aij, rmul(vol, R->iom));
    aii = cmul(aii, rmul(vol, R->iom));
  }
  st(R->Ex, p, cdiv(csub(ld(R->bx, p), aij), aii));
}

/* Ey row update (fdfd.c:383-395; A-phi fdfd.c:612-624) */
static void row_ey(const rows_t *R, int k, int j, int i)
{
  const double *d1s = R->d1s, *d2s = R->d2s, *d3s = R->d3s, *d1 = R->d1, *d3 = R->d3;
  long p = RI2(k, j, i);
  st(R->Ey, p, mk(0., 0.));
  const double *Ex = R->Ex, *Ey = R->Ey, *Ez = R->Ez;
  cz t1 = csub(cdivr(csub(ld(Ez, RI3(k, j + 1, i)), ld(Ez, RI3(k, j, i))), d2s[j]),
               cdivr(csub(ld(Ey, RI2(k + 1, j, i)), ld(Ey, RI2(k, j, i))), d3s[k]));
  cz t2 = csub(cdivr(csub(ld(Ez, RI3(k - 1, j + 1, i)), ld(Ez, RI3(k - 1, j, i))), d2s[j]),
               cdivr(csub(ld(Ey, RI2(k, j, i)), ld(Ey, RI2(k - 1, j, i))), d3s[k - 1]));
  cz t3 = csub(cdivr(csub(ld(Ey, RI2(k, j, i + 1)), ld(Ey, RI2(k, j, i))), d1s[i]),
               cdivr(csub(ld(Ex, RI1(k, j + 1, i)), ld(Ex, RI1(k, j, i))), d2s[j]));
  cz t4 = csub(cdivr(csub(ld(Ey, RI2(k, j, i)), ld(Ey, RI2(k, j, i - 1))), d1s[i - 1]),
               cdivr(csub(ld(Ex, RI1(k, j + 1, i - 1)), ld(Ex, RI1(k, j, i - 1))), d2s[j]));
  double sg = R->s22[p];
  cz own = ld(Ey, p);
  if (R->v) own = cadd(own, cdivr(csub(ld(R->v, RI3(k, j + 1, i)), ld(R->v, RI3(k, j, i))), d2s[j]));
  cz aij = csub(cmul(csub(cdivr(csub(t1, t2), d3[k]), cdivr(csub(t3, t4), d1[i])), R->iwmu), rmul(sg, own));
  double g = (1. / d3s[k] + 1. / d3s[k - 1]) / d3[k] + (1. / d1s[i] + 1. / d1s[i - 1]) / d1[i];
  cz aii = rmul(g, R->iwmu);
  aii = mk(aii.re - sg, aii.im);
  if (R->fvm) {
    double vol = d1s[i] * R->d2[j] * d3[k]; /* sic: Ex's cell volume (fdfd.c:391) */
    aij = cmul(aij, rmul(vol, R->iom));
    aii = cmul(aii, rmul(vol, R->iom));
  }
  st(R->Ey, p, cdiv(csub(ld(R->by, p), aij), aii));
}

/* Ez row update (fdfd.c:409-421; A-phi fdfd.c:638-650) */
static void row_ez(const rows_t *R, int k, int j, int i)
{
  const double *d1s = R->d1s, *d2s = R->d2s, *d3s = R->d3s, *d1 = R->d1, *d2 = R->d2;
  long p = RI3(k, j, i);
  st(R->Ez, p, mk(0., 0.));
  const double *Ex = R->Ex, *Ey = R->Ey, *Ez = R->Ez;
  cz t1 = csub(cdivr(csub(ld(Ex, RI1(k + 1, j, i)), ld(Ex, RI1(k, j, i))), d3s[k]),
               cdivr(csub(ld(Ez, RI3(k, j, i + 1)), ld(Ez, RI3(k, j, i))), d1s[i]));
  cz t2 = csub(cdivr(csub(ld(Ex, RI1(k + 1, j, i - 1)), ld(Ex, RI1(k, j, i - 1))), d3s[k]),
               cdivr(csub(ld(Ez, RI3(k, j, i)), ld(Ez, RI3(k, j, i - 1))), d1s[i - 1]));
  cz t3 = csub(cdivr(csub(ld(Ez, RI3(k, j + 1, i)), ld(Ez, RI3(k, j, i))), d2s[j]),
               cdivr(csub(ld(Ey, RI2(k + 1, j, i)), ld(Ey, RI2(k, j, i))), d3s[k]));
  cz t4 = csub(cdivr(csub(ld(Ez, RI3(k, j, i)), ld(Ez, RI3(k, j - 1, i))), d2s[j - 1]),
               cdivr(csub(ld(Ey, RI2(k + 1, j - 1, i)), ld(Ey, RI2(k, j - 1, i))), d3s[k]));
  double sg = R->s33[p];
  cz own = ld(Ez, p);
  if (R->v) own = cadd(own, cdivr(csub(ld(R->v, RI3(k + 1, j, i)), ld(R->v, RI3(k, j, i))), d3s[k]));
  cz aij = csub(cmul(csub(cdivr(csub(t1, t2), d1[i]), cdivr(csub(t3, t4), d2[j])), R->iwmu), rmul(sg, own));
  double g = (1. / d1s[i] + 1. / d1s[i - 1]) / d1[i] + (1. / d2s[j] + 1. / d2s[j - 1]) / d2[j];
  cz aii = rmul(g, R->iwmu);
  aii = mk(aii.re - sg, aii.im);
  if (R->fvm) {
    double vol = d1s[i] * d2[j] * R->d3[k]; /* sic: Ex's cell volume (fdfd.c:417) */
    aij = cmul(aij, rmul(vol, R->iom));
    aii = cmul(aii, rmul(vol, R->iom));
  }
  st(R->Ez, p, cdiv(csub(ld(R->bz, p), aij), aii));
}

/* the six component sweeps, fdfd.c:347-503 (same loop bounds in A-phi) */
static void sweeps_forward(const rows_t *R)
{
  int n1 = R->n1, n2 = R->n2, n3 = R->n3;
  for (int k = 1; k < n3; k++)
    for (int j = 1; j < n2; j++)
      for (int i = 0; i < n1; i++) row_ex(R, k, j, i);
  for (int k = 1; k < n3; k++)
    for (int j = 0; j < n2; j++)
      for (int i = 1; i < n1; i++) row_ey(R, k, j, i);
  for (int k = 0; k < n3; k++)
    for (int j = 1; j < n2; j++)
      for (int i = 1; i < n1; i++) row_ez(R, k, j, i);
}

static void sweeps_backward_ez(const rows_t *R)
{
  int n1 = R->n1, n2 = R->n2, n3 = R->n3;
  for (int k = n3 - 1; k >= 0; k--)
    for (int j = n2 - 1; j > 0; j--)
      for (int i = n1 - 1; i > 0; i--) row_ez(R, k, j, i);
}

static void sweeps_backward_eyex(const rows_t *R)
{
  int n1 = R->n1, n2 = R->n2, n3 = R->n3;
  for (int k = n3 - 1; k > 0; k--)
    for (int j = n2 - 1; j >= 0; j--)
      for (int i = n1 - 1; i > 0; i--) row_ey(R, k, j, i);
  for (int k = n3 - 1; k > 0; k--)
    for (int j = n2 - 1; j > 0; j--)
      for (int i = n1 - 1; i >= 0; i--) row_ex(R, k, j, i);
}

void orc_lusgs_apply(orc_ctx_t *c, const double *x, double *y)
{
  /* fdfd.c:287-510: on the full grid (air included) when airbc */
  const orc_desc_t *D = &c->d;
  rows_t R;
  memset(&R, 0, sizeof(R));
  R.n1 = c->n1;
  R.n2 = c->n2;
  R.n3 = D->airbc ? c->n3 + D->nb : c->n3;
  R.d1 = D->d1; R.d2 = D->d2; R.d3 = D->d3; R.d1s = D->d1s; R.d2s = D->d2s; R.d3s = D->d3s;
  R.s11 = D->sigma11; R.s22 = D->sigma22; R.s33 = D->sigma33;
  R.iwmu = iwmu_of(c);
  R.iom = c->iom;
  R.fvm = D->fvm;
  int n1 = R.n1, n2 = R.n2, n3 = R.n3;
  long lEx = (long)n1 * (n2 + 1) * (n3 + 1), lEy = (long)(n1 + 1) * n2 * (n3 + 1),
       lEz = (long)(n1 + 1) * (n2 + 1) * n3;
  if (D->airbc) {
    int nb = D->nb;
    memset(c->xx, 0, sizeof(double) * 2 * (size_t)(lEx + lEy + lEz));
    memset(c->yy, 0, sizeof(double) * 2 * (size_t)(lEx + lEy + lEz));
    memcpy(c->xx + 2 * (long)n1 * (n2 + 1) * nb, x, sizeof(double) * 2 * (size_t)c->lEx);
    memcpy(c->xx + 2 * ((long)(n1 + 1) * n2 * nb + lEx), x + 2 * c->lEx, sizeof(double) * 2 * (size_t)c->lEy);
    memcpy(c->xx + 2 * ((long)(n1 + 1) * (n2 + 1) * nb + lEx + lEy), x + 2 * (c->lEx + c->lEy),
           sizeof(double) * 2 * (size_t)c->lEz);
    R.Ex = c->yy; R.Ey = c->yy + 2 * lEx; R.Ez = c->yy + 2 * (lEx + lEy);
    R.bx = c->xx; R.by = c->xx + 2 * lEx; R.bz = c->xx + 2 * (lEx + lEy);
  } else {
    memset(y, 0, sizeof(double) * 2 * (size_t)c->lE);
    R.Ex = y; R.Ey = y + 2 * c->lEx; R.Ez = y + 2 * (c->lEx + c->lEy);
    R.bx = x; R.by = x + 2 * c->lEx; R.bz = x + 2 * (c->lEx + c->lEy);
  }
  sweeps_forward(&R);
  sweeps_backward_ez(&R);
  sweeps_backward_eyex(&R);
  if (D->airbc) {
    int nb = D->nb;
    memcpy(y, c->yy + 2 * (long)n1 * (n2 + 1) * nb, sizeof(double) * 2 * (size_t)c->lEx);
    memcpy(y + 2 * c->lEx, c->yy + 2 * ((long)(n1 + 1) * n2 * nb + lEx), sizeof(double) * 2 * (size_t)c->lEy);
    memcpy(y + 2 * (c->lEx + c->lEy), c->yy + 2 * ((long)(n1 + 1) * (n2 + 1) * nb + lEx + lEy),
           sizeof(double) * 2 * (size_t)c->lEz);
  }
}

/* ------------------------------------------------------------ A-phi */
static void phi_row(const orc_ctx_t *c, const rows_t *R, const double *S11u, const double *S22u,
                    const double *S33u, const double *bv, double *v, int k, int j, int i)
{
  /* fdfd.c:664-678: shifted sigma at the edge's own index, UNshifted emf->sigma*
   * lookups for the -1 neighbours (sic), a purely geometric diagonal (sic) */
  const double *d1 = R->d1, *d2 = R->d2, *d3 = R->d3, *d1s = R->d1s, *d2s = R->d2s, *d3s = R->d3s;
  int n1 = R->n1, n2 = R->n2;
  long p = RI3(k, j, i);
  st(v, p, mk(0., 0.));
  cz vp = ld(v, p);
  cz t1 = rmul(R->s11[RI1(k, j, i)], cadd(ld(R->Ex, RI1(k, j, i)), cdivr(csub(ld(v, RI3(k, j, i + 1)), vp), d1s[i])));
  cz t2 = rmul(S11u[((long)k * (n2 + 1) + j) * n1 + (i - 1)],
               cadd(ld(R->Ex, RI1(k, j, i - 1)), cdivr(csub(vp, ld(v, RI3(k, j, i - 1))), d1s[i - 1])));
  cz t3 = rmul(R->s22[RI2(k, j, i)], cadd(ld(R->Ey, RI2(k, j, i)), cdivr(csub(ld(v, RI3(k, j + 1, i)), vp), d2s[j])));
  cz t4 = rmul(S22u[((long)k * n2 + (j - 1)) * (n1 + 1) + i],
               cadd(ld(R->Ey, RI2(k, j - 1, i)), cdivr(csub(vp, ld(v, RI3(k, j - 1, i))), d2s[j - 1])));
  cz t5 = rmul(R->s33[RI3(k, j, i)], cadd(ld(R->Ez, RI3(k, j, i)), cdivr(csub(ld(v, RI3(k + 1, j, i)), vp), d3s[k])));
  cz t6 = rmul(S33u[((long)(k - 1) * (n2 + 1) + j) * (n1 + 1) + i],
               cadd(ld(R->Ez, RI3(k - 1, j, i)), cdivr(csub(vp, ld(v, RI3(k - 1, j, i))), d3s[k - 1])));
  cz aij = cadd(cadd(cdivr(csub(t1, t2), d1[i]), cdivr(csub(t3, t4), d2[j])), cdivr(csub(t5, t6), d3[k]));
  double g = -((1. / d1s[i] + 1. / d1s[i - 1]) / d1[i] + (1. / d2s[j] + 1. / d2s[j - 1]) / d2[j] +
               (1. / d3s[k] + 1. / d3s[k - 1]) / d3[k]);
  cz aii = mk(g, 0.);
  if (R->fvm) {
    double vol = d1s[i] * d2[j] * d3[k];
    aij = cmul(aij, rmul(vol, c->iom));
    aii = cmul(aii, rmul(vol, c->iom));
  }
  st(v, p, cdiv(csub(ld(bv, p), aij), aii));
}

void orc_aphi_apply(orc_ctx_t *c, const double *x, double *y)
{
  /* fdfd.c:513-821 on the operator grid (kstart shift when airbc) */
  const orc_desc_t *D = &c->d;
  int n1 = c->n1, n2 = c->n2, n3 = c->n3, ks = c->kstart;
  rows_t R;
  memset(&R, 0, sizeof(R));
  R.n1 = n1; R.n2 = n2; R.n3 = n3;
  R.d1 = D->d1; R.d2 = D->d2; R.d3 = D->d3 + ks; R.d1s = D->d1s; R.d2s = D->d2s; R.d3s = D->d3s + ks;
  R.s11 = D->sigma11 + (long)ks * (n2 + 1) * n1;
  R.s22 = D->sigma22 + (long)ks * n2 * (n1 + 1);
  R.s33 = D->sigma33 + (long)ks * (n2 + 1) * (n1 + 1);
  R.iwmu = iwmu_of(c);
  R.iom = c->iom;
  R.fvm = D->fvm;
  R.Ex = y; R.Ey = y + 2 * c->lEx; R.Ez = y + 2 * (c->lEx + c->lEy);
  R.bx = x; R.by = x + 2 * c->lEx; R.bz = x + 2 * (c->lEx + c->lEy);
  double *v = c->v, *bv = c->bv;
  const double *d1 = R.d1, *d2 = R.d2, *d3 = R.d3, *d1s = R.d1s, *d2s = R.d2s, *d3s = R.d3s;
  memset(bv, 0, sizeof(double) * 2 * (size_t)c->lv);
  for (int k = 1; k < n3; k++)
    for (int j = 1; j < n2; j++)
      for (int i = 1; i < n1; i++) {
        long p = ((long)k * (n2 + 1) + j) * (n1 + 1) + i;
        cz s = mk(0., 0.);
        s = cadd(s, cdivr(cneg(csub(ld(R.bx, ((long)k * (n2 + 1) + j) * n1 + i), ld(R.bx, ((long)k * (n2 + 1) + j) * n1 + i - 1))), d1[i]));
        s = cadd(s, cdivr(cneg(csub(ld(R.by, ((long)k * n2 + j) * (n1 + 1) + i), ld(R.by, ((long)k * n2 + j - 1) * (n1 + 1) + i))), d2[j]));
        s = cadd(s, cdivr(cneg(csub(ld(R.bz, p), ld(R.bz, ((long)(k - 1) * (n2 + 1) + j) * (n1 + 1) + i))), d3[k]));
        st(bv, p, s);
      }
  memset(y, 0, sizeof(double) * 2 * (size_t)c->lE);
  memset(v, 0, sizeof(double) * 2 * (size_t)c->lv);
  /* forward: ax, ay, az with v = 0 (v terms vanish), then v */
  R.v = v;
  {
    const rows_t *Q = &R;
    for (int k = 1; k < n3; k++)
      for (int j = 1; j < n2; j++)
        for (int i = 0; i < n1; i++) row_ex(Q, k, j, i);
    for (int k = 1; k < n3; k++)
      for (int j = 0; j < n2; j++)
        for (int i = 1; i < n1; i++) row_ey(Q, k, j, i);
    for (int k = 0; k < n3; k++)
      for (int j = 1; j < n2; j++)
        for (int i = 1; i < n1; i++) row_ez(Q, k, j, i);
  }
  for (int k = 1; k < n3; k++)
    for (int j = 1; j < n2; j++)
      for (int i = 1; i < n1; i++) phi_row(c, &R, D->sigma11, D->sigma22, D->sigma33, bv, v, k, j, i);
  for (int k = n3 - 1; k >= 1; k--)
    for (int j = n2 - 1; j >= 1; j--)
      for (int i = n1 - 1; i >= 1; i--) phi_row(c, &R, D->sigma11, D->sigma22, D->sigma33, bv, v, k, j, i);
  sweeps_backward_ez(&R);
  sweeps_backward_eyex(&R);
  /* E = A + grad v (fdfd.c:796-819), in place */
  for (int k = 1; k < n3; k++)
    for (int j = 1; j < n2; j++)
      for (int i = 0; i < n1; i++) {
        long p = ((long)k * (n2 + 1) + j) * n1 + i;
        cz dv = cdivr(csub(ld(v, ((long)k * (n2 + 1) + j) * (n1 + 1) + i + 1), ld(v, ((long)k * (n2 + 1) + j) * (n1 + 1) + i)), d1s[i]);
        st(R.Ex, p, cadd(ld(R.Ex, p), dv));
      }
  for (int k = 1; k < n3; k++)
    for (int j = 0; j < n2; j++)
      for (int i = 1; i < n1; i++) {
        long p = ((long)k * n2 + j) * (n1 + 1) + i;
        cz dv = cdivr(csub(ld(v, ((long)k * (n2 + 1) + j + 1) * (n1 + 1) + i), ld(v, ((long)k * (n2 + 1) + j) * (n1 + 1) + i)), d2s[j]);
        st(R.Ey, p, cadd(ld(R.Ey, p), dv));
      }
  for (int k = 0; k < n3; k++)
    for (int j = 1; j < n2; j++)
      for (int i = 1; i < n1; i++) {
        long p = ((long)k * (n2 + 1) + j) * (n1 + 1) + i;
        cz dv = cdivr(csub(ld(v, ((long)(k + 1) * (n2 + 1) + j) * (n1 + 1) + i), ld(v, p)), d3s[k]);
        st(R.Ez, p, cadd(ld(R.Ez, p), dv));
      }
}

/* ------------------------------------------------------------ BLAS-1 */
void orc_cdot(long n, const double *a, const double *b, double *out)
{
  /* cdotprod.c:13-19 */
  cz s = mk(0., 0.);
  for (long i = 0; i < n; i++) s = cadd(s, cmul(ld(a, i), cconj(ld(b, i))));
  out[0] = s.re;
  out[1] = s.im;
}

static cz dot(long n, const double *a, const double *b)
{
  double o[2];
  orc_cdot(n, a, b, o);
  return mk(o[0], o[1]);
}

typedef void (*orc_op_t)(orc_ctx_t *, const double *, double *);

static void push(double *hist, int cap, int *nh, double v)
{
  if (hist && *nh < cap) hist[*nh] = v;
  (*nh)++;
}

/* ------------------------------------------------------------ GMRES preconditioner */
void orc_gmres_pre_apply(orc_ctx_t *c, int m, const double *b, double *x)
{
  /* gmres_init_free.c:58-137: mp GMRES steps on A from x = 0, no convergence test */
  long n = c->lE;
  if (!c->gw || c->gm != m) {
    free(c->gw);
    c->gw = (double *)calloc(2 * (size_t)n * (size_t)(m + 3), sizeof(double));
    c->gm = m;
  }
  double *w = c->gw, *r = w + 2 * n, *V = r + 2 * n;
  cz *h = (cz *)calloc((size_t)(m + 1) * m, sizeof(cz));
  cz *g = (cz *)calloc((size_t)m + 1, sizeof(cz));
  cz *yv = (cz *)calloc((size_t)m + 1, sizeof(cz));
  cz *cc = (cz *)calloc((size_t)m + 1, sizeof(cz));
  double *s = (double *)calloc((size_t)m + 1, sizeof(double));
#define H(i, j) h[(long)(i) * m + (j)]
  memset(x, 0, sizeof(double) * 2 * (size_t)n);
  memcpy(r, b, sizeof(double) * 2 * (size_t)n);
  double beta = sqrt(dot(n, r, r).re);
  if (beta == 0.0) goto done;
  for (long i = 0; i < n; i++) st(V, i, cdivr(ld(r, i), beta));
  g[0] = mk(beta, 0.);
  for (int j = 0; j < m; j++) {
    orc_fdfd_apply(c, V + 2 * n * j, w);
    for (int i = 0; i <= j; i++) {
      H(i, j) = dot(n, w, V + 2 * n * i);
      for (long k = 0; k < n; k++) st(w, k, csub(ld(w, k), cmul(H(i, j), ld(V + 2 * n * i, k))));
    }
    H(j + 1, j) = mk(sqrt(dot(n, w, w).re), 0.);
    for (long i = 0; i < n; i++) st(V + 2 * n * (j + 1), i, cdiv(ld(w, i), H(j + 1, j)));
    for (int i = 0; i < j; i++) {
      cz ss = cadd(cmul(cconj(cc[i]), H(i, j)), rmul(s[i], H(i + 1, j)));
      H(i + 1, j) = cadd(rmul(-s[i], H(i, j)), cmul(cc[i], H(i + 1, j)));
      H(i, j) = ss;
    }
    double tmp = sqrt(cadd(cmul(H(j, j), cconj(H(j, j))), cmul(H(j + 1, j), cconj(H(j + 1, j)))).re);
    s[j] = H(j + 1, j).re / tmp;
    cc[j] = cdivr(H(j, j), tmp);
    H(j, j) = cadd(cmul(cconj(cc[j]), H(j, j)), rmul(s[j], H(j + 1, j)));
    H(j + 1, j) = mk(0., 0.);
    g[j + 1] = rmul(-s[j], g[j]);
    g[j] = cmul(cconj(cc[j]), g[j]);
  }
  yv[m - 1] = cdiv(g[m - 1], H(m - 1, m - 1));
  for (int i = m - 2; i >= 0; i--) {
    yv[i] = g[i];
    for (int j = i + 1; j < m; j++) yv[i] = csub(yv[i], cmul(H(i, j), yv[j]));
    yv[i] = cdiv(yv[i], H(i, i));
  }
  for (int j = 0; j < m; j++)
    for (long i = 0; i < n; i++) st(x, i, cadd(ld(x, i), cmul(yv[j], ld(V + 2 * n * j, i))));
#undef H
done:
  free(h); free(g); free(yv); free(cc); free(s);
}

static int g_pre_mp = 30;
static void op_A(orc_ctx_t *c, const double *x, double *y) { orc_fdfd_apply(c, x, y); }
static void op_gmres_pre(orc_ctx_t *c, const double *x, double *y) { orc_gmres_pre_apply(c, g_pre_mp, x, y); }
static orc_op_t precond_op(int precond, int mp)
{
  g_pre_mp = mp;
  switch (precond) {
  case 1: return orc_lusgs_apply;
  case 2: return op_gmres_pre;
  case 3: return orc_aphi_apply;
  default: return NULL;
  }
}

/* ------------------------------------------------------------ Krylov */
int orc_bicgstab(orc_ctx_t *c, double *x, const double *b, int niter, double tol,
                 double *hist, int hist_cap, int *nhist)
{
  /* solver.c:16-87 */
  long n = c->lE;
  int nh = 0, iter;
  double *r = (double *)malloc(sizeof(double) * 2 * (size_t)n * 6);
  double *r0 = r + 2 * n, *p = r0 + 2 * n, *v = p + 2 * n, *s = v + 2 * n, *t = s + 2 * n;
  op_A(c, x, v);
  for (long i = 0; i < n; i++) {
    cz ri = csub(ld(b, i), ld(v, i));
    st(r, i, ri); st(p, i, ri); st(r0, i, ri);
  }
  cz rho_old = dot(n, r, r0);
  double rs = dot(n, r, r).re, rs0 = rs, relres;
  if (rs == 0.) { free(r); if (nhist) *nhist = 0; return 0; }
  relres = sqrt(rs / rs0);
  push(hist, hist_cap, &nh, relres);
  for (iter = 0; iter < niter; ++iter) {
    op_A(c, p, v);
    cz alpha = cdiv(rho_old, dot(n, v, r0));
    for (long i = 0; i < n; i++) st(s, i, csub(ld(r, i), cmul(alpha, ld(v, i))));
    op_A(c, s, t);
    cz omega = cdivr(dot(n, t, s), dot(n, t, t).re);
    for (long i = 0; i < n; i++) {
      st(x, i, cadd(ld(x, i), cadd(cmul(alpha, ld(p, i)), cmul(omega, ld(s, i)))));
      st(r, i, csub(ld(s, i), cmul(omega, ld(t, i))));
    }
    rs = dot(n, r, r).re;
    relres = sqrt(rs / rs0);
    push(hist, hist_cap, &nh, relres);
    if (relres < tol) break;
    cz rho_new = dot(n, r, r0);
    cz beta = cdiv(cmul(cdiv(rho_new, rho_old), alpha), omega);
    for (long i = 0; i < n; i++)
      st(p, i, cadd(ld(r, i), cmul(beta, csub(ld(p, i), cmul(omega, ld(v, i))))));
    rho_old = rho_new;
  }
  free(r);
  if (nhist) *nhist = nh;
  return iter;
}

int orc_fbicgstab(orc_ctx_t *c, int precond, int mp, double *x, const double *b, int niter,
                  double tol, double *hist, int hist_cap, int *nhist)
{
  /* solver.c:93-178 */
  orc_op_t M = precond_op(precond, mp);
  long n = c->lE;
  int nh = 0, iter;
  double *r = (double *)malloc(sizeof(double) * 2 * (size_t)n * 7);
  double *r0 = r + 2 * n, *p = r0 + 2 * n, *pp = p + 2 * n, *v = pp + 2 * n, *s = v + 2 * n, *t = s + 2 * n;
  op_A(c, x, v);
  for (long i = 0; i < n; i++) {
    cz ri = csub(ld(b, i), ld(v, i));
    st(r, i, ri); st(p, i, ri); st(r0, i, ri);
  }
  cz rho_old = dot(n, r, r0);
  double rs = dot(n, r, r).re, rs0 = rs, relres;
  if (rs == 0.) { free(r); if (nhist) *nhist = 0; return 0; }
  relres = sqrt(rs / rs0);
  push(hist, hist_cap, &nh, relres);
  for (iter = 0; iter < niter; ++iter) {
    M(c, p, pp);
    op_A(c, pp, v);
    cz alpha = dot(n, v, r0);
    alpha = cdiv(rho_old, alpha);
    for (long i = 0; i < n; i++) st(s, i, csub(ld(r, i), cmul(alpha, ld(v, i))));
    M(c, s, r);
    op_A(c, r, t);
    cz omega = cdivr(dot(n, s, t), dot(n, t, t).re);
    for (long i = 0; i < n; i++) {
      st(x, i, cadd(ld(x, i), cadd(cmul(alpha, ld(pp, i)), cmul(omega, ld(r, i)))));
      st(r, i, csub(ld(s, i), cmul(omega, ld(t, i))));
    }
    rs = dot(n, r, r).re;
    relres = sqrt(rs / rs0);
    push(hist, hist_cap, &nh, relres);
    if (relres < tol) break;
    cz rho_new = dot(n, r, r0);
    cz beta = cdiv(cmul(cdiv(rho_new, rho_old), alpha), omega);
    for (long i = 0; i < n; i++)
      st(p, i, cadd(ld(r, i), cmul(beta, csub(ld(p, i), cmul(omega, ld(v, i))))));
    rho_old = rho_new;
  }
  free(r);
  if (nhist) *nhist = nh;
  return iter;
}

int orc_gmres(orc_ctx_t *c, double *x, const double *b, int niter, double tol, int m,
              double *hist, int hist_cap, int *nhist)
{
  /* solver.c:181-285, including its early return without the last update (sic) */
  long n = c->lE;
  int nh = 0, iter;
  double r0 = 0;
  double *w = (double *)malloc(sizeof(double) * 2 * (size_t)n * (size_t)(m + 3));
  double *r = w + 2 * n, *V = r + 2 * n;
  cz *h = (cz *)calloc((size_t)(m + 1) * m, sizeof(cz));
  cz *g = (cz *)calloc((size_t)m + 1, sizeof(cz));
  cz *yv = (cz *)calloc((size_t)m + 1, sizeof(cz));
  cz *cc = (cz *)calloc((size_t)m + 1, sizeof(cz));
  double *s = (double *)calloc((size_t)m + 1, sizeof(double));
#define H(i, j) h[(long)(i) * m + (j)]
  for (iter = 0; iter < niter; iter++) {
    op_A(c, x, w);
    for (long i = 0; i < n; i++) st(r, i, csub(ld(b, i), ld(w, i)));
    double beta = sqrt(dot(n, r, r).re);
    if (beta == 0.0) goto out;
    for (long i = 0; i < n; i++) st(V, i, cdivr(ld(r, i), beta));
    memset(g, 0, sizeof(cz) * (size_t)(m + 1));
    g[0] = mk(beta, 0.);
    memset(h, 0, sizeof(cz) * (size_t)(m + 1) * m);
    if (iter == 0) {
      r0 = beta;
      push(hist, hist_cap, &nh, beta / r0);
    }
    for (int j = 0; j < m; j++) {
      op_A(c, V + 2 * n * j, w);
      for (int i = 0; i <= j; i++) {
        H(i, j) = dot(n, w, V + 2 * n * i);
        for (long k = 0; k < n; k++) st(w, k, csub(ld(w, k), cmul(H(i, j), ld(V + 2 * n * i, k))));
      }
      H(j + 1, j) = mk(sqrt(dot(n, w, w).re), 0.);
      if (cabs_(H(j + 1, j)) == 0.0) { m = j + 1; break; }
      for (long i = 0; i < n; i++) st(V + 2 * n * (j + 1), i, cdiv(ld(w, i), H(j + 1, j)));
      for (int i = 0; i < j; i++) {
        cz ss = cadd(cmul(cconj(cc[i]), H(i, j)), rmul(s[i], H(i + 1, j)));
        H(i + 1, j) = cadd(rmul(-s[i], H(i, j)), cmul(cc[i], H(i + 1, j)));
        H(i, j) = ss;
      }
      double tmp = sqrt(cadd(cmul(H(j, j), cconj(H(j, j))), cmul(H(j + 1, j), cconj(H(j + 1, j)))).re);
      s[j] = H(j + 1, j).re / tmp;
      cc[j] = cdivr(H(j, j), tmp);
      H(j, j) = cadd(cmul(cconj(cc[j]), H(j, j)), rmul(s[j], H(j + 1, j)));
      H(j + 1, j) = mk(0., 0.);
      g[j + 1] = rmul(-s[j], g[j]);
      g[j] = cmul(cconj(cc[j]), g[j]);
      double rel = cabs_(g[j + 1]) / r0;
      push(hist, hist_cap, &nh, rel);
      if (rel < tol) { m = j + 1; goto out; }
    }
    yv[m - 1] = cdiv(g[m - 1], H(m - 1, m - 1));
    for (int i = m - 2; i >= 0; i--) {
      yv[i] = g[i];
      for (int j = i + 1; j < m; j++) yv[i] = csub(yv[i], cmul(H(i, j), yv[j]));
      yv[i] = cdiv(yv[i], H(i, i));
    }
    for (int j = 0; j < m; j++)
      for (long i = 0; i < n; i++) st(x, i, cadd(ld(x, i), cmul(yv[j], ld(V + 2 * n * j, i))));
  }
#undef H
out:
  free(w); free(h); free(g); free(yv); free(cc); free(s);
  if (nhist) *nhist = nh;
  return iter;
}

int orc_fgmres(orc_ctx_t *c, int precond, int mp, double *x, const double *b, int niter,
               double tol, int m, double *hist, int hist_cap, int *nhist)
{
  /* solver.c:403-512 */
  orc_op_t M = precond_op(precond, mp);
  long n = c->lE;
  int nh = 0, iter, j = 0, mm, conv = 0;
  double r0 = 0, relres;
  double *w = (double *)malloc(sizeof(double) * 2 * (size_t)n * (size_t)(2 * m + 3));
  double *r = w + 2 * n, *V = r + 2 * n, *Z = V + 2 * n * (m + 1);
  cz *h = (cz *)calloc((size_t)(m + 1) * m, sizeof(cz));
  cz *g = (cz *)calloc((size_t)m + 1, sizeof(cz));
  cz *yv = (cz *)calloc((size_t)m + 1, sizeof(cz));
  cz *cc = (cz *)calloc((size_t)m + 1, sizeof(cz));
  double *s = (double *)calloc((size_t)m + 1, sizeof(double));
#define HT(j, i) h[(long)(j) * (m + 1) + (i)]
  for (iter = 0; iter < niter; iter++) {
    op_A(c, x, w);
    for (long i = 0; i < n; i++) st(r, i, csub(ld(b, i), ld(w, i)));
    double beta = sqrt(dot(n, r, r).re);
    if (beta == 0.) break;
    for (long i = 0; i < n; i++) st(V, i, cdivr(ld(r, i), beta));
    memset(g, 0, sizeof(cz) * (size_t)(m + 1));
    g[0] = mk(beta, 0.);
    memset(h, 0, sizeof(cz) * (size_t)(m + 1) * m);
    relres = (iter > 0) ? (beta / r0) : 1;
    if (iter == 0) {
      r0 = beta;
      push(hist, hist_cap, &nh, relres);
    }
    for (j = 0; j < m; j++) {
      M(c, V + 2 * n * j, Z + 2 * n * j);
      op_A(c, Z + 2 * n * j, w);
      for (int i = 0; i <= j; i++) {
        HT(j, i) = dot(n, w, V + 2 * n * i);
        for (long k = 0; k < n; k++) st(w, k, csub(ld(w, k), cmul(HT(j, i), ld(V + 2 * n * i, k))));
      }
      HT(j, j + 1) = mk(sqrt(dot(n, w, w).re), 0.);
      if (cabs_(HT(j, j + 1)) == 0.) { conv = 1; break; }
      for (long i = 0; i < n; i++) st(V + 2 * n * (j + 1), i, cdiv(ld(w, i), HT(j, j + 1)));
      for (int i = 0; i < j; i++) {
        cz ss = cadd(cmul(cconj(cc[i]), HT(j, i)), rmul(s[i], HT(j, i + 1)));
        HT(j, i + 1) = cadd(rmul(-s[i], HT(j, i)), cmul(cc[i], HT(j, i + 1)));
        HT(j, i) = ss;
      }
      double tmp = sqrt(cadd(cmul(HT(j, j), cconj(HT(j, j))), cmul(HT(j, j + 1), cconj(HT(j, j + 1)))).re);
      s[j] = HT(j, j + 1).re / tmp;
      cc[j] = cdivr(HT(j, j), tmp);
      g[j + 1] = rmul(-s[j], g[j]);
      g[j] = cmul(cconj(cc[j]), g[j]);
      HT(j, j) = cadd(cmul(cconj(cc[j]), HT(j, j)), rmul(s[j], HT(j, j + 1)));
      relres = cabs_(g[j + 1]) / r0;
      push(hist, hist_cap, &nh, relres);
      if (relres < tol) { conv = 1; break; }
    }
    mm = m < j + 1 ? m : j + 1;
    yv[mm - 1] = cdiv(g[mm - 1], HT(mm - 1, mm - 1));
    for (int i = mm - 2; i >= 0; i--) {
      yv[i] = g[i];
      for (int jj = i + 1; jj < mm; jj++) yv[i] = csub(yv[i], cmul(HT(jj, i), yv[jj]));
      yv[i] = cdiv(yv[i], HT(i, i));
    }
    for (int jj = 0; jj < mm; jj++)
      for (long i = 0; i < n; i++) st(x, i, cadd(ld(x, i), cmul(yv[jj], ld(Z + 2 * n * jj, i))));
    if (conv) break;
  }
#undef HT
  free(w); free(h); free(g); free(yv); free(cc); free(s);
  if (nhist) *nhist = nh;
  return iter;
}

/* ------------------------------------------------------------ inject / extract */
static int find_index(int n, const double *x, double val)
{
  /* find_index.c:9-30 */
  int low = 0, high = n - 1;
  while (low < high) {
    int i = (low + high) / 2;
    if (x[i] <= val) low = i;
    if (x[i] > val) high = i;
    if (low == high || low == high - 1) break;
  }
  return low;
}

void orc_inject(orc_ctx_t *c, int nch, const int *ch, const float *src, double *b)
{
  /* inject_extract.c:24-120, incl. the sigma lookup nb rows too high with airbc (sic) */
  const orc_desc_t *D = &c->d;
  int n1 = D->n1, n2 = D->n2, n3 = D->n3f, nb = D->nb;
  int N1 = c->n1, N2 = c->n2;
  double *bx = b, *by = b + 2 * c->lEx, *bz = b + 2 * (c->lEx + c->lEy);
  memset(b, 0, sizeof(double) * 2 * (size_t)c->lE);
  double sx = src[0], sy = src[1], sz = src[2];
  for (int ic = 0; ic < nch; ic++) {
    if (ch[ic] == 0) {
      int i = find_index(n1, D->x1s, sx), j = find_index(n2 + 1, D->x2, sy), k = find_index(n3 + 1, D->x3, sz);
      double w1 = (sx - D->x1s[i]) / (D->x1s[i + 1] - D->x1s[i]);
      double w2 = (sy - D->x2[j]) / (D->x2[j + 1] - D->x2[j]);
      double w3 = (sz - D->x3[k]) / (D->x3[k + 1] - D->x3[k]);
      double vol = (D->x1s[i + 1] - D->x1s[i]) * (D->x2[j + 1] - D->x2[j]) * (D->x3[k + 1] - D->x3[k]);
      cz sv = mk(1. / vol, 0.);
      if (D->fvm) sv = c->iom;
      sv = cdivr(sv, (double)(float)D->rho_water);
      if (D->airbc) k -= nb;
      int di[8] = {0, 1, 0, 1, 0, 1, 0, 1}, dj[8] = {0, 0, 1, 1, 0, 0, 1, 1}, dk[8] = {0, 0, 0, 0, 1, 1, 1, 1};
      for (int q = 0; q < 8; q++) {
        double a1 = di[q] ? w1 : 1. - w1, a2 = dj[q] ? w2 : 1. - w2, a3 = dk[q] ? w3 : 1. - w3;
        int kk = k + dk[q], jj = j + dj[q], ii = i + di[q];
        double sg = D->sigma11[((long)kk * (n2 + 1) + jj) * n1 + ii];
        cz val = rmul(a3, rmul(a2, rmul(a1, cdivr(sv, sg))));
        long p = ii + (long)N1 * (jj + (long)(N2 + 1) * kk);
        st(bx, p, cadd(ld(bx, p), val));
      }
    } else if (ch[ic] == 1) {
      int i = find_index(n1 + 1, D->x1, sx), j = find_index(n2, D->x2s, sy), k = find_index(n3 + 1, D->x3, sz);
      double w1 = (sx - D->x1[i]) / (D->x1[i + 1] - D->x1[i]);
      double w2 = (sy - D->x2s[j]) / (D->x2s[j + 1] - D->x2s[j]);
      double w3 = (sz - D->x3[k]) / (D->x3[k + 1] - D->x3[k]);
      double vol = (D->x1[i + 1] - D->x1[i]) * (D->x2s[j + 1] - D->x2s[j]) * (D->x3[k + 1] - D->x3[k]);
      cz sv = mk(1. / vol, 0.);
      if (D->fvm) sv = c->iom;
      sv = cdivr(sv, (double)(float)D->rho_water);
      if (D->airbc) k -= nb;
      int di[8] = {0, 1, 0, 1, 0, 1, 0, 1}, dj[8] = {0, 0, 1, 1, 0, 0, 1, 1}, dk[8] = {0, 0, 0, 0, 1, 1, 1, 1};
      for (int q = 0; q < 8; q++) {
        double a1 = di[q] ? w1 : 1. - w1, a2 = dj[q] ? w2 : 1. - w2, a3 = dk[q] ? w3 : 1. - w3;
        int kk = k + dk[q], jj = j + dj[q], ii = i + di[q];
        double sg = D->sigma22[((long)kk * n2 + jj) * (n1 + 1) + ii];
        cz val = rmul(a3, rmul(a2, rmul(a1, cdivr(sv, sg))));
        long p = ii + (long)(N1 + 1) * (jj + (long)N2 * kk);
        st(by, p, cadd(ld(by, p), val));
      }
    } else if (ch[ic] == 2) {
      int i = find_index(n1 + 1, D->x1, sx), j = find_index(n2 + 1, D->x2, sy), k = find_index(n3, D->x3s, sz);
      double w1 = (sx - D->x1[i]) / (D->x1[i + 1] - D->x1[i]);
      double w2 = (sy - D->x2[j]) / (D->x2[j + 1] - D->x2[j]);
      double w3 = (sz - D->x3s[k]) / (D->x3s[k + 1] - D->x3s[k]);
      double vol = (D->x1[i + 1] - D->x1[i]) * (D->x2[j + 1] - D->x2[j]) * (D->x3s[k + 1] - D->x3s[k]);
      cz sv = mk(1. / vol, 0.);
      if (D->fvm) sv = c->iom;
      if (D->airbc) k -= nb;
      int di[8] = {0, 1, 0, 1, 0, 1, 0, 1}, dj[8] = {0, 0, 1, 1, 0, 0, 1, 1}, dk[8] = {0, 0, 0, 0, 1, 1, 1, 1};
      for (int q = 0; q < 8; q++) {
        double a1 = di[q] ? w1 : 1. - w1, a2 = dj[q] ? w2 : 1. - w2, a3 = dk[q] ? w3 : 1. - w3;
        int kk = k + dk[q], jj = j + dj[q], ii = i + di[q];
        cz val = rmul(a3, rmul(a2, rmul(a1, sv)));
        long p = ii + (long)(N1 + 1) * (jj + (long)(N2 + 1) * kk);
        st(bz, p, cadd(ld(bz, p), val));
      }
    }
  }
}

void orc_extract(orc_ctx_t *c, int nch, const int *ch, int nrec, const float *rec,
                 const double *x, double *out)
{
  /* inject_extract.c:123-213 */
  const orc_desc_t *D = &c->d;
  int n1 = D->n1, n2 = D->n2, n3 = D->n3f, nb = D->nb;
  int N1 = c->n1, N2 = c->n2;
  const double *Ex = x, *Ey = x + 2 * c->lEx, *Ez = x + 2 * (c->lEx + c->lEy);
  int di[8] = {0, 1, 0, 1, 0, 1, 0, 1}, dj[8] = {0, 0, 1, 1, 0, 0, 1, 1}, dk[8] = {0, 0, 0, 0, 1, 1, 1, 1};
  for (int ic = 0; ic < nch; ic++)
    for (int r = 0; r < nrec; r++) {
      double rx = rec[5 * r], ry = rec[5 * r + 1], rz = rec[5 * r + 2];
      cz s = mk(0., 0.);
      if (ch[ic] == 0) {
        int i = find_index(n1, D->x1s, rx), j = find_index(n2 + 1, D->x2, ry), k = find_index(n3 + 1, D->x3, rz);
        double w1 = (rx - D->x1s[i]) / (D->x1s[i + 1] - D->x1s[i]);
        double w2 = (ry - D->x2[j]) / (D->x2[j + 1] - D->x2[j]);
        double w3 = (rz - D->x3[k]) / (D->x3[k + 1] - D->x3[k]);
        if (D->airbc) k -= nb;
        for (int q = 0; q < 8; q++) {
          double a1 = di[q] ? w1 : 1. - w1, a2 = dj[q] ? w2 : 1. - w2, a3 = dk[q] ? w3 : 1. - w3;
          long p = (i + di[q]) + (long)N1 * ((j + dj[q]) + (long)(N2 + 1) * (k + dk[q]));
          s = cadd(s, rmul(a3, rmul(a2, rmul(a1, ld(Ex, p)))));
        }
      } else if (ch[ic] == 1) {
        int i = find_index(n1 + 1, D->x1, rx), j = find_index(n2, D->x2s, ry), k = find_index(n3 + 1, D->x3, rz);
        double w1 = (rx - D->x1[i]) / (D->x1[i + 1] - D->x1[i]);
        double w2 = (ry - D->x2s[j]) / (D->x2s[j + 1] - D->x2s[j]);
        double w3 = (rz - D->x3[k]) / (D->x3[k + 1] - D->x3[k]);
        if (D->airbc) k -= nb;
        for (int q = 0; q < 8; q++) {
          double a1 = di[q] ? w1 : 1. - w1, a2 = dj[q] ? w2 : 1. - w2, a3 = dk[q] ? w3 : 1. - w3;
          long p = (i + di[q]) + (long)(N1 + 1) * ((j + dj[q]) + (long)N2 * (k + dk[q]));
          s = cadd(s, rmul(a3, rmul(a2, rmul(a1, ld(Ey, p)))));
        }
      } else if (ch[ic] == 2) {
        int i = find_index(n1 + 1, D->x1, rx), j = find_index(n2 + 1, D->x2, ry), k = find_index(n3, D->x3s, rz);
        double w1 = (rx - D->x1[i]) / (D->x1[i + 1] - D->x1[i]);
        double w2 = (ry - D->x2[j]) / (D->x2[j + 1] - D->x2[j]);
        double w3 = (rz - D->x3s[k]) / (D->x3s[k + 1] - D->x3s[k]);
        int kk = k;
        if (D->airbc) k -= nb;
        for (int q = 0; q < 8; q++) {
          double a1 = di[q] ? w1 : 1. - w1, a2 = dj[q] ? w2 : 1. - w2, a3 = dk[q] ? w3 : 1. - w3;
          long p = (i + di[q]) + (long)(N1 + 1) * ((j + dj[q]) + (long)(N2 + 1) * (k + dk[q]));
          double sg = D->sigma33[((long)(kk + dk[q]) * (n2 + 1) + (j + dj[q])) * (n1 + 1) + (i + di[q])];
          s = cadd(s, rmul(a3, rmul(a2, rmul(a1, rmul(sg, ld(Ez, p))))));
        }
        s = rmul((double)(float)D->rho_water, s);
      }
      out[2 * ((long)ic * nrec + r)] = s.re;
      out[2 * ((long)ic * nrec + r) + 1] = s.im;
    }
}
