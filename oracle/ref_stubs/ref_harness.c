/* ctypes-facing harness around the unmodified reference sources (CPU oracle build,
 * test infrastructure only). It is compiled against the reference's own headers
 * where they lie and linked with the reference objects into oracle/_ref/.
 *
 * ref_setup() performs the same set-up sequence as the reference driver
 * (main.c:54-92): initargs, the flag defaults of main.c:62-69, emf_init,
 * acq_init, extend_model_init, fdfd_init and the xe/xh/be/dcal_fd allocations.
 * The other entry points expose the reference's hot-path functions one by one so
 * tests can feed them the same inputs as the GPU library.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <complex.h>
#include "cstd.h"
#include "emf.h"
#include "acq.h"
#include "solver.h"
#include "mpi.h"

extern int iproc, nproc, ierr;
void emf_init(emf_t *emf);
void acq_init(acq_t *acq, emf_t *emf);
void extend_model_init(acq_t *acq, emf_t *emf);
void fdfd_init(emf_t *emf);
void fdfd_free(emf_t *emf);
void fdfd_apply(int n, complex *x, complex *y);
void fdfd_apply_old(int n, complex *x, complex *y);
void lusgs_apply(int n, complex *x, complex *y);
void aphi_apply(int n, complex *x, complex *y);
void airbc_apply(emf_t *emf, complex *H3k, complex *H1km1, complex *H2km1);
void inject_source(acq_t *acq, emf_t *emf, complex *b);
void extract_emf(acq_t *acq, emf_t *emf, complex *x, int ifreq);
complex cdotprod(int n, complex *a, complex *b);
void gmres_init(int n, int m, op_t Aop);
void gmres_free();
void gmres_apply(int n, complex *x, complex *y);
void bicgstab(int n, complex *x, complex *b, op_t Aop, int niter, double tol, int verb);
void gmres(int n, complex *x, complex *b, op_t Aop, int niter, double tol, int m, int verb);
void fbicgstab(int n, complex *x, complex *b, op_t Aop, op_t invMop, int niter, double tol, int verb);
void fgmres(int n, complex *x, complex *b, op_t Aop, op_t invMop, int niter, double tol, int m, int verb);
void Acsr_init(emf_t *emf, int ifreq);
void Acsr_free();
void Acsr_apply(int n, complex *x, complex *y);
void Acsr_lusgs_apply(int n, complex *x, complex *y);
int ref_main(int argc, char **argv);
extern emf_t *emf; /* fdfd.c:23 */

static emf_t *H_emf;
static acq_t *H_acq;
static char **H_argv;
static int H_argc;

static char **dup_args(int argc, char **argv)
{
  char **a = (char **)malloc(sizeof(char *) * (size_t)(argc + 1));
  for (int i = 0; i < argc; i++) a[i] = strdup(argv[i]);
  a[argc] = NULL;
  return a;
}

int ref_setup(int argc, char **argv)
{
  H_argc = argc;
  H_argv = dup_args(argc, argv);
  MPI_Init(&H_argc, &H_argv);
  MPI_Comm_rank(MPI_COMM_WORLD, &iproc);
  MPI_Comm_size(MPI_COMM_WORLD, &nproc);
  initargs(H_argc, H_argv);
  H_emf = (emf_t *)calloc(1, sizeof(emf_t));
  H_acq = (acq_t *)calloc(1, sizeof(acq_t));
  emf_t *e = H_emf;
  if (!getparint("mode", &e->mode)) e->mode = 0;
  if (!getparint("verb", &e->verb)) e->verb = 0;
  if (!getparint("niter", &e->niter)) e->niter = 1000;
  if (!getparint("preco", &e->preco)) e->preco = 1;
  if (!getparint("algopt", &e->algopt)) e->algopt = 1;
  if (!getparfloat("tol", &e->tol)) e->tol = 1e-8;
  if (!getparint("nrestart", &e->nrestart)) e->nrestart = 10;
  if (!getparint("mp", &e->mp)) e->mp = 30;
  emf_init(e);
  acq_init(H_acq, e);
  extend_model_init(H_acq, e);
  fdfd_init(e);
  e->ne = e->lE;
  e->nh = e->lH;
  e->xe = alloc1complex(e->ne);
  e->xh = alloc1complex(e->nh);
  e->be = alloc1complex(e->ne);
  memset(e->xe, 0, sizeof(complex) * (size_t)e->ne);
  memset(e->xh, 0, sizeof(complex) * (size_t)e->nh);
  memset(e->be, 0, sizeof(complex) * (size_t)e->ne);
  e->dcal_fd = alloc3complexf(H_acq->nrec, e->nfreq, e->nchrec);
  memset(&e->dcal_fd[0][0][0], 0, sizeof(float _Complex) * (size_t)H_acq->nrec * e->nfreq * e->nchrec);
  return 0;
}

/* integer facts about the set-up model */
void ref_info(int *o)
{
  emf_t *e = H_emf;
  o[0] = e->n1; o[1] = e->n2; o[2] = e->n3; o[3] = e->nb;
  o[4] = e->nx; o[5] = e->ny; o[6] = e->nz;
  o[7] = e->lE; o[8] = e->lEx; o[9] = e->lEy; o[10] = e->lEz; o[11] = e->lH; o[12] = e->lv;
  o[13] = H_acq->nrec; o[14] = e->nfreq; o[15] = e->nchrec; o[16] = e->airbc; o[17] = e->fvm;
  o[18] = e->preco; o[19] = e->algopt; o[20] = e->niter; o[21] = e->nrestart; o[22] = e->mp;
  o[23] = e->airbc ? e->n1fft : 0; o[24] = e->airbc ? e->n2fft : 0; o[25] = e->nchsrc;
}

/* float facts */
void ref_finfo(double *o)
{
  emf_t *e = H_emf;
  o[0] = e->rho_water; o[1] = e->rho_air; o[2] = e->lextend; o[3] = e->tol;
  o[4] = e->airbc ? e->d1fft : 0; o[5] = e->airbc ? e->d2fft : 0; o[6] = e->airbc ? e->d3fft : 0;
  o[7] = creal(e->I_omega_mu0); o[8] = cimag(e->I_omega_mu0);
}

void ref_freqs(float *o) { memcpy(o, H_emf->freqs, sizeof(float) * (size_t)H_emf->nfreq); }

/* 1-D grid arrays (length n+1 of the full padded grid) */
void ref_grid(int which, double *o)
{
  emf_t *e = H_emf;
  int n1 = e->nx + 2 * e->nb, n2 = e->ny + 2 * e->nb, n3 = e->nz + 2 * e->nb;
  double *src[12] = {e->x1, e->x2, e->x3, e->x1s, e->x2s, e->x3s,
                     e->d1, e->d2, e->d3, e->d1s, e->d2s, e->d3s};
  int len[12] = {n1 + 1, n2 + 1, n3 + 1, n1 + 1, n2 + 1, n3 + 1,
                 n1 + 1, n2 + 1, n3 + 1, n1 + 1, n2 + 1, n3 + 1};
  memcpy(o, src[which], sizeof(double) * (size_t)len[which]);
}

/* full-grid edge conductivities, flat in the reference's index order */
void ref_sigma(int which, double *o)
{
  emf_t *e = H_emf;
  int n1 = e->nx + 2 * e->nb, n2 = e->ny + 2 * e->nb, n3 = e->nz + 2 * e->nb;
  size_t len[3] = {(size_t)n1 * (n2 + 1) * (n3 + 1), (size_t)(n1 + 1) * n2 * (n3 + 1),
                   (size_t)(n1 + 1) * (n2 + 1) * n3};
  double ***s[3] = {e->sigma11, e->sigma22, e->sigma33};
  memcpy(o, &s[which][0][0][0], sizeof(double) * len[which]);
}

/* airwave filters sH1kxky / sH2kxky, flat [n2fft][n1fft] */
void ref_airfilter(int which, double complex *o)
{
  emf_t *e = H_emf;
  complex **s = which == 0 ? e->sH1kxky : e->sH2kxky;
  memcpy(o, &s[0][0], sizeof(complex) * (size_t)e->n1fft * e->n2fft);
}

void ref_set_freq(int ifreq)
{
  /* main.c:95 */
  H_emf->I_omega_mu0 = I * 2. * PI * H_emf->freqs[ifreq] * mu0;
}

void ref_set_iwmu(double re, double im) { H_emf->I_omega_mu0 = re + I * im; }

void ref_apply(int op, complex *x, complex *y)
{
  int n = H_emf->lE;
  switch (op) {
  case 0: fdfd_apply(n, x, y); break;
  case 1: lusgs_apply(n, x, y); break;
  case 2: aphi_apply(n, x, y); break;
  case 3: fdfd_apply_old(n, x, y); break;
  case 4: gmres_apply(n, x, y); break;
  case 5: Acsr_apply(n, x, y); break;
  case 6: Acsr_lusgs_apply(n, x, y); break;
  }
}

void ref_get_h(complex *o) { memcpy(o, H_emf->xh, sizeof(complex) * (size_t)H_emf->lH); }

void ref_airbc(complex *Hz0, complex *hx, complex *hy) { airbc_apply(H_emf, Hz0, hx, hy); }

void ref_inject(complex *b)
{
  memset(b, 0, sizeof(complex) * (size_t)H_emf->lE);
  inject_source(H_acq, H_emf, b);
}

void ref_extract(complex *x, int ifreq) { extract_emf(H_acq, H_emf, x, ifreq); }

void ref_dcal(float _Complex *o)
{
  memcpy(o, &H_emf->dcal_fd[0][0][0],
         sizeof(float _Complex) * (size_t)H_acq->nrec * H_emf->nfreq * H_emf->nchrec);
}

void ref_cdot(int n, complex *a, complex *b, complex *out) { *out = cdotprod(n, a, b); }

void ref_acsr_init(int ifreq) { Acsr_init(H_emf, ifreq); }
void ref_acsr_free(void) { Acsr_free(); }
void ref_gmres_init(int m) { gmres_init(H_emf->lE, m, fdfd_apply); }
void ref_gmres_free(void) { gmres_free(); }

/* One frequency of the reference driver loop body (main.c:94-118): tolerance in
 * float, zeroed x/H/b, source injection, solver dispatch on preco/algopt. x and b
 * receive the solution and right-hand side. niter_override >= 0 replaces niter. */
double ref_solve(int ifreq, complex *x, complex *b, int niter_override, int verb)
{
  emf_t *e = H_emf;
  float tol = e->tol / e->freqs[ifreq];
  int niter = niter_override >= 0 ? niter_override : e->niter;
  e->verb = verb;
  ref_set_freq(ifreq);
  memset(e->xe, 0, e->ne * sizeof(complex));
  memset(e->xh, 0, e->nh * sizeof(complex));
  memset(e->be, 0, e->ne * sizeof(complex));
  inject_source(H_acq, e, e->be);
  double t0 = MPI_Wtime();
  if (e->preco == 0) {
    if (e->algopt == 1) bicgstab(e->ne, e->xe, e->be, fdfd_apply, niter, tol, e->verb);
    if (e->algopt == 2) gmres(e->ne, e->xe, e->be, fdfd_apply, niter / e->nrestart, tol, e->nrestart, e->verb);
  } else if (e->preco == 1) {
    if (e->algopt == 1) fbicgstab(e->ne, e->xe, e->be, fdfd_apply, lusgs_apply, niter, tol, e->verb);
    if (e->algopt == 2) fgmres(e->ne, e->xe, e->be, fdfd_apply, lusgs_apply, niter / e->nrestart, tol, e->nrestart, e->verb);
  } else if (e->preco == 2) {
    gmres_init(e->ne, e->mp, fdfd_apply);
    if (e->algopt == 1) fbicgstab(e->ne, e->xe, e->be, fdfd_apply, gmres_apply, niter, tol, e->verb);
    if (e->algopt == 2) fgmres(e->ne, e->xe, e->be, fdfd_apply, gmres_apply, niter / e->nrestart, tol, e->nrestart, e->verb);
    gmres_free();
  } else if (e->preco == 3) {
    if (e->algopt == 1) fbicgstab(e->ne, e->xe, e->be, fdfd_apply, aphi_apply, niter, tol, e->verb);
    if (e->algopt == 2) fgmres(e->ne, e->xe, e->be, fdfd_apply, aphi_apply, niter / e->nrestart, tol, e->nrestart, e->verb);
  }
  double t1 = MPI_Wtime();
  extract_emf(H_acq, e, e->xe, ifreq);
  if (x) memcpy(x, e->xe, sizeof(complex) * (size_t)e->ne);
  if (b) memcpy(b, e->be, sizeof(complex) * (size_t)e->ne);
  return t1 - t0;
}

/* the reference driver itself (main.c:46-145, built with -Dmain=ref_main) */
int ref_run_main(int argc, char **argv) { return ref_main(argc, dup_args(argc, argv)); }
