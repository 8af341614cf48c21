/* Same-symbol drop-in for the reference's hot path (include/csem_refabi.h), built as
 * libcsem_refabi.so on top of libcsem_gpu.so. One model per process, as the reference
 * (its hot path keeps the model in globals, fdfd.c:23-24). */
#include <complex.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "csem_gpu.h"
#include "csem_refabi.h"

/* the reference's flag reader (cstd.c); weak so the library also loads without it */
int getparint(char *name, int *p) __attribute__((weak));

static emf_t *g_emf;
static csem_ctx *g_ctx;
static csem_grid_t g_grid;
static int g_mp = 30;

static void fail(const char *what)
{
  fflush(stdout);
  fprintf(stderr, "\ncsem_refabi: %s: %s\n", what, csem_last_error());
  exit(1);
}

static void need_ctx(const char *what)
{
  if (!g_ctx) {
    fprintf(stderr, "\ncsem_refabi: %s called before fdfd_init\n", what);
    exit(1);
  }
}

void fdfd_init(emf_t *emf)
{
  g_emf = emf;
  memset(&g_grid, 0, sizeof(g_grid));
  csem_grid_t *g = &g_grid;
  g->nx = emf->nx; g->ny = emf->ny; g->nz = emf->nz; g->nb = emf->nb;
  g->x1node = emf->x1node; g->x2node = emf->x2node; g->x3node = emf->x3node;
  g->rho_water = emf->rho_water; g->rho_air = emf->rho_air; g->lextend = emf->lextend;
  g->airbc = emf->airbc; g->fvm = emf->fvm;
  g->n1 = emf->n1; g->n2 = emf->n2; g->n3 = emf->n3; /* full padded grid at this point */
  g->x1 = emf->x1; g->x2 = emf->x2; g->x3 = emf->x3;
  g->x1s = emf->x1s; g->x2s = emf->x2s; g->x3s = emf->x3s;
  g->d1 = emf->d1; g->d2 = emf->d2; g->d3 = emf->d3;
  g->d1s = emf->d1s; g->d2s = emf->d2s; g->d3s = emf->d3s;
  g->sigma11 = &emf->sigma11[0][0][0];
  g->sigma22 = &emf->sigma22[0][0][0];
  g->sigma33 = &emf->sigma33[0][0][0];
  if (emf->airbc) {
    int n1fft = 1024, n2fft = 1024; /* airbc_init_free.c:30-31 */
    if (getparint) {
      getparint("n1fft", &n1fft);
      getparint("n2fft", &n2fft);
    }
    if (csem_grid_airbc(g, n1fft, n2fft)) fail("airwave tables");
    emf->n1fft = g->n1fft;
    emf->n2fft = g->n2fft;
    emf->d1fft = g->d1fft;
    emf->d2fft = g->d2fft;
    emf->d3fft = g->d3fft;
    emf->n3 = emf->nz + emf->nb; /* the air is not part of the operator (fdfd.c:49) */
  }
  /* lengths of fdfd.c:54-62, including the reference's n2 for the last factor of lHy */
  int n1 = emf->n1, n2 = emf->n2, n3 = emf->n3;
  emf->lEx = n1 * (n2 + 1) * (n3 + 1);
  emf->lEy = (n1 + 1) * n2 * (n3 + 1);
  emf->lEz = (n1 + 1) * (n2 + 1) * n3;
  emf->lE = emf->lEx + emf->lEy + emf->lEz;
  emf->lHx = (n1 + 1) * n2 * n3;
  emf->lHy = n1 * (n2 + 1) * n2;
  emf->lHz = n1 * n2 * (n3 + 1);
  emf->lH = emf->lHx + emf->lHy + emf->lHz;
  emf->lv = (n1 + 1) * (n2 + 1) * (n3 + 1);
  if (csem_ctx_create(g, emf->airbc, emf->fvm, &g_ctx)) fail("fdfd_init");
  /* dot products in the reference's sequential order on request (flag dot_order=1 of a
   * driver that links the reference's getpar, or CSEM_DOT_ORDER=1 in the environment) */
  int dot_order = 0;
  const char *env = getenv("CSEM_DOT_ORDER");
  if (env) dot_order = atoi(env);
  if (getparint) getparint("dot_order", &dot_order);
  if (dot_order && csem_ctx_set_option(g_ctx, "dot_order", dot_order)) fail("dot_order");
}

void fdfd_free(emf_t *emf)
{
  (void)emf;
  csem_ctx_destroy(g_ctx);
  g_ctx = NULL;
  free(g_grid.sH1); free(g_grid.sH2); free(g_grid.jx); free(g_grid.jy); free(g_grid.wx); free(g_grid.wy);
  memset(&g_grid, 0, sizeof(g_grid));
}

#define IOM creal(g_emf->I_omega_mu0), cimag(g_emf->I_omega_mu0)

void fdfd_apply(int n, csem_z *x, csem_z *y)
{
  (void)n;
  need_ctx("fdfd_apply");
  if (csem_fdfd_apply_host(g_ctx, IOM, (const double *)x, (double *)y)) fail("fdfd_apply");
}

void lusgs_apply(int n, csem_z *x, csem_z *y)
{
  (void)n;
  need_ctx("lusgs_apply");
  if (csem_lusgs_apply_host(g_ctx, IOM, (const double *)x, (double *)y)) fail("lusgs_apply");
}

void aphi_apply(int n, csem_z *x, csem_z *y)
{
  (void)n;
  need_ctx("aphi_apply");
  if (csem_aphi_apply_host(g_ctx, IOM, (const double *)x, (double *)y)) fail("aphi_apply");
}

void gmres_init(int n, int m, op_t Aop)
{
  (void)n;
  if (Aop != fdfd_apply) {
    fprintf(stderr, "\ncsem_refabi: gmres_init supports Aop = fdfd_apply only\n");
    exit(1);
  }
  g_mp = m;
}

void gmres_free(void) {}

void gmres_apply(int n, csem_z *x, csem_z *y)
{
  (void)n;
  need_ctx("gmres_apply");
  if (csem_gmres_pre_apply_host(g_ctx, IOM, g_mp, (const double *)x, (double *)y)) fail("gmres_apply");
}

csem_z cdotprod(int n, csem_z *a, csem_z *b)
{
  double o[2];
  if (csem_cdot_host(n, (const double *)a, (const double *)b, o)) fail("cdotprod");
  return o[0] + I * o[1];
}

static int precond_code(op_t M)
{
  if (M == lusgs_apply) return 1;
  if (M == gmres_apply) return 2;
  if (M == aphi_apply) return 3;
  fprintf(stderr, "\ncsem_refabi: unknown preconditioner callback (lusgs_apply, gmres_apply or aphi_apply)\n");
  exit(1);
}

static void run(int algopt, int preco, csem_z *x, csem_z *b, int niter_total, int m, double tol, int verb,
                const char *fname, const char *tag)
{
  need_ctx(tag);
  int cap = niter_total * 2 + 64, nh = 0, it = 0, st = 0;
  double *h = (double *)malloc(sizeof(double) * (size_t)cap);
  if (csem_solve_fp64_host(g_ctx, algopt, preco, niter_total, tol, m, g_mp, IOM, (const double *)b, (double *)x, h,
                           cap, &nh, &it, &st))
    fail(tag);
  if (verb && st != CSEM_ST_ZERO_RHS) {
    const int nprint = csem_history_logged(algopt, preco, st, nh < cap ? nh : cap);
    FILE *fp = fopen(fname, "w");
    if (fp) {
      fprintf(fp, algopt == 1 ? "iteration \t relres\n" : "iteration \t error\n");
      for (int q = 0; q < nprint; q++) fprintf(fp, "%d \t %e\n", q, h[q]);
      fclose(fp);
    }
    for (int q = 0; q < nprint; q++) printf("%s iter=%d relres=%e\n", tag, q, h[q]);
    if (st == CSEM_ST_CONVERGED && algopt == 1) printf("converged at iter=%d\n", it - 1);
  }
  free(h);
}

void bicgstab(int n, csem_z *x, csem_z *b, op_t Aop, int niter, double tol, int verb)
{
  (void)n;
  if (Aop != fdfd_apply) precond_code(NULL);
  run(1, 0, x, b, niter, 10, tol, verb, "iterate_bicgstab.txt", "bicgstab");
}

void fbicgstab(int n, csem_z *x, csem_z *b, op_t Aop, op_t invMop, int niter, double tol, int verb)
{
  (void)n;
  if (Aop != fdfd_apply) precond_code(NULL);
  run(1, precond_code(invMop), x, b, niter, 10, tol, verb, "iterate_fbicgstab.txt", "f-bicgstab");
}

/* the reference's gmres/fgmres take the number of restart cycles (main.c:106,109) */
void gmres(int n, csem_z *x, csem_z *b, op_t Aop, int niter, double tol, int m, int verb)
{
  (void)n;
  if (Aop != fdfd_apply) precond_code(NULL);
  run(2, 0, x, b, niter * m, m, tol, verb, "iterate_gmres.txt", "gmres");
}

void fgmres(int n, csem_z *x, csem_z *b, op_t Aop, op_t invMop, int niter, double tol, int m, int verb)
{
  (void)n;
  if (Aop != fdfd_apply) precond_code(NULL);
  run(2, precond_code(invMop), x, b, niter * m, m, tol, verb, "iterate_fgmres.txt", "f-gmres");
}

static int channel_code(const char *s)
{
  if (!strcmp(s, "Ex")) return 0;
  if (!strcmp(s, "Ey")) return 1;
  if (!strcmp(s, "Ez")) return 2;
  return 3; /* H channels: accepted by the reference's parser, inject/extract nothing */
}

void inject_source(acq_t *acq, emf_t *emf, csem_z *b)
{
  need_ctx("inject_source");
  int ch[8], nch = emf->nchsrc > 8 ? 8 : emf->nchsrc;
  for (int c = 0; c < nch; c++) ch[c] = channel_code(emf->chsrc[c]);
  csem_z *t = (csem_z *)malloc(sizeof(csem_z) * (size_t)emf->lE);
  for (int s = 0; s < acq->nsrc; s++) {
    float src[3] = {acq->src_x1[s], acq->src_x2[s], acq->src_x3[s]};
    if (csem_inject_host(g_ctx, IOM, nch, ch, src, (double *)t)) fail("inject_source");
    for (int q = 0; q < emf->lE; q++) b[q] += t[q]; /* the reference accumulates into b */
  }
  free(t);
}

void extract_emf(acq_t *acq, emf_t *emf, csem_z *x, int ifreq)
{
  need_ctx("extract_emf");
  int nrec = acq->nrec, nch = emf->nchrec;
  float *rec = (float *)malloc(sizeof(float) * 5 * (size_t)(nrec > 0 ? nrec : 1));
  for (int r = 0; r < nrec; r++) {
    rec[5 * r] = acq->rec_x1[r];
    rec[5 * r + 1] = acq->rec_x2[r];
    rec[5 * r + 2] = acq->rec_x3[r];
    rec[5 * r + 3] = acq->rec_azimuth ? acq->rec_azimuth[r] : 0.f;
    rec[5 * r + 4] = acq->rec_dip ? acq->rec_dip[r] : 0.f;
  }
  int *ch = (int *)calloc((size_t)(nch > 0 ? nch : 1), sizeof(int));
  for (int c = 0; c < nch; c++) ch[c] = channel_code(emf->chrec[c]);
  double *out = (double *)malloc(sizeof(double) * 2 * (size_t)nch * (nrec > 0 ? nrec : 1));
  if (csem_extract_host(g_ctx, nch, ch, nrec, rec, (const double *)x, out)) fail("extract_emf");
  for (int c = 0; c < nch; c++)
    for (int r = 0; r < nrec; r++) {
      if (ch[c] > 2) continue; /* H channels produce nothing (inject_extract.c:137-211) */
      emf->dcal_fd[c][ifreq][r] = (float)out[2 * ((size_t)c * nrec + r)] + I * (float)out[2 * ((size_t)c * nrec + r) + 1];
    }
  free(rec);
  free(ch);
  free(out);
}

/* sizeof(emf_t), sizeof(acq_t) and a few member offsets, for layout checks */
void csem_refabi_layout(long *out)
{
  out[0] = (long)sizeof(emf_t);
  out[1] = (long)sizeof(acq_t);
  out[2] = (long)__builtin_offsetof(emf_t, sigma11);
  out[3] = (long)__builtin_offsetof(emf_t, I_omega_mu0);
  out[4] = (long)__builtin_offsetof(emf_t, dcal_fd);
  out[5] = (long)__builtin_offsetof(emf_t, param_extended);
  out[6] = (long)__builtin_offsetof(acq_t, rec_x1);
  out[7] = (long)__builtin_offsetof(acq_t, shot_idx);
}
