/* csem - key=value driver of the GB300 CSEM solver.
 *
 * Same command line, inputs and outputs as the reference driver (main.c:46-145):
 *   flags and defaults of main.c:62-69, emf_init_free.c:24-132, acq_init_free.c:26-32,
 *   extend_model.c:43,254 and airbc_init_free.c:30-31 (CWP getpar semantics);
 *   float32 fx1..3 / frho11..33 model files, text source/receiver files;
 *   emf_0001.txt (write_data.c:15-37) and iterate_<solver>.txt convergence histories.
 * Errors print "<prog>: <message>" and exit(1), as err() does (cstd.c:1539-1552).
 *
 * Keys added by this driver:
 *   precision=64  plain complex128 solve, one frequency after the other (default);
 *             32  all (frequency x source) systems in one batched mixed-precision solve;
 *   nsrc=1|all    solve the first source row only (the reference, acq_init_free.c:56,90)
 *                 or every row, writing emf_NNNN.txt per source (NNNN = row number);
 *   inner_tol, check_every, max_outer   options of the mixed-precision solver;
 *   fix_quirks=1  with airbc, inject the source with the conductivity of its own row
 *                 (the reference reads it nb rows higher, inject_extract.c:55-63);
 *   dot_order=1   complex128 dot products in the reference's sequential order (its
 *                 iterates bit for bit, slowly);
 *   graphs=0|1, autotune=0|1, lusgs_split, lusgs_vw, lusgs_pipelined, stencil_by,
 *   stencil_ctas   the context options of csem_ctx_set_option.
 */
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include "csem_gpu.h"

static const char *g_prog = "csem";

static void die(const char *fmt, ...)
{
  va_list ap;
  fflush(stdout);
  fprintf(stderr, "\n%s: ", g_prog);
  va_start(ap, fmt);
  vfprintf(stderr, fmt, ap);
  va_end(ap);
  fprintf(stderr, "\n");
  exit(1);
}

static void check(int rc)
{
  if (rc != CSEM_OK) die("%s", csem_last_error());
}

static double now(void)
{
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static int channel_code(const char *s)
{
  const char *names[6] = {"Ex", "Ey", "Ez", "Hx", "Hy", "Hz"};
  for (int c = 0; c < 6; c++)
    if (!strcmp(s, names[c])) return c;
  return -1;
}

static int read_channels(const char *key, int *codes, int max)
{
  int n = csem_countparval(key);
  if (!n) {
    codes[0] = 0; /* Ex (emf_init_free.c:33-37,43-47) */
    return 1;
  }
  if (n > max) die("too many %s channels", key);
  char *names[16];
  csem_getparstringarray(key, names);
  for (int c = 0; c < n; c++) {
    codes[c] = channel_code(names[c]);
    free(names[c]);
  }
  return n;
}

static const char *hist_name(int algopt, int preco)
{
  if (algopt == 1) return preco ? "iterate_fbicgstab.txt" : "iterate_bicgstab.txt";
  return preco ? "iterate_fgmres.txt" : "iterate_gmres.txt";
}

int main(int argc, char **argv)
{
  g_prog = argv[0];
  csem_initargs(argc, argv);
  int mode, verb, niter, preco, algopt, nrestart, mp;
  float tol;
  if (!csem_getparint("mode", &mode)) mode = 0;
  if (!csem_getparint("verb", &verb)) verb = 1;
  if (!csem_getparint("niter", &niter)) niter = 1000;
  if (!csem_getparint("preco", &preco)) preco = 1;
  if (!csem_getparint("algopt", &algopt)) algopt = 1;
  if (!csem_getparfloat("tol", &tol)) tol = 1e-8f;
  if (!csem_getparint("nrestart", &nrestart)) nrestart = 10;
  if (!csem_getparint("mp", &mp)) mp = 30;
  (void)mode;
  int precision = 64, fvm, nb, istretch, airbc, param_extended, n1fft, n2fft, check_every, max_outer;
  float rho_air, lextend;
  double inner_tol;
  csem_getparint("precision", &precision);
  if (!csem_getparint("fvm", &fvm)) fvm = 0;
  if (!csem_getparint("nb", &nb)) nb = 15;
  if (!csem_getparfloat("rho_air", &rho_air)) rho_air = 1e6f;
  if (!csem_getparint("istretch", &istretch)) istretch = 1;
  if (!csem_getparint("airbc", &airbc)) airbc = 0;
  if (airbc && nb == 0) die("airbc=1 assumes input model without air, you must ensure nb>0");
  if (!csem_getparfloat("lextend", &lextend)) lextend = -1.f;
  if (!csem_getparint("param_extended", &param_extended)) param_extended = 0;
  if (!csem_getparint("n1fft", &n1fft)) n1fft = 1024;
  if (!csem_getparint("n2fft", &n2fft)) n2fft = 1024;
  if (!csem_getpardouble("inner_tol", &inner_tol)) inner_tol = 0.2;
  if (!csem_getparint("check_every", &check_every)) check_every = 4;
  if (!csem_getparint("max_outer", &max_outer)) max_outer = 30;
  char *nsrc_s = NULL;
  int all_sources = csem_getparstring("nsrc", &nsrc_s) && !strcmp(nsrc_s, "all");
  if (verb) {
    printf("preco=%d (1=precondition; 0=unpreconditioned)\n", preco);
    printf("algopt=%d (1=BICGStab; 2=GMRES)\n", algopt);
    printf("niter=%d\n", niter);
    printf("nrestart=%d\n", nrestart);
    printf("mp=%d (GMRES(mp) preconditioner)\n", mp);
    printf("tol=%.2e\n", tol);
    printf("precision=%d (%s)\n", precision, precision == 32 ? "batched complex64 inner, complex128 outer" : "complex128");
  }

  int nfreq = csem_countparval("freqs");
  if (!nfreq) die("Need freqs= vector");
  float *freqs = (float *)malloc(sizeof(float) * (size_t)nfreq);
  csem_getparfloat("freqs", freqs);
  csem_sort_freqs(freqs, nfreq);
  int chsrc[8], chrec[8];
  int nchsrc = read_channels("chsrc", chsrc, 8);
  int nchrec = read_channels("chrec", chrec, 8);

  char *f[8];
  const char *keys[8] = {"fx1", "fx2", "fx3", "frho11", "frho22", "frho33", "fsrc", "frec"};
  for (int q = 0; q < 8; q++)
    if (!csem_getparstring(keys[q], &f[q])) die("Need %s= ", keys[q]);
  csem_grid_t g;
  check(csem_grid_read(&g, f[0], f[1], f[2], f[3], f[4], f[5]));
  csem_acq_t acq;
  check(csem_acq_read(&acq, f[6], f[7]));
  if (!all_sources) acq.nsrc = 1;
  check(csem_acq_check(&acq, &g));
  check(csem_grid_extend(&g, nb, lextend, rho_air, istretch));
  if (param_extended && verb) check(csem_grid_write_extended(&g, "."));
  if (airbc) check(csem_grid_airbc(&g, n1fft, n2fft));
  if (verb) {
    printf("nx=%d ny=%d nz=%d nb=%d lextend=%g rho_water=%g\n", g.nx, g.ny, g.nz, nb, g.lextend, g.rho_water);
    printf("n1=nx+2*nb=%d\nn2=ny+2*nb=%d\nn3=nz+2*nb=%d\n", g.n1, g.n2, g.n3);
  }
  csem_ctx *ctx;
  check(csem_ctx_create(&g, airbc, fvm, &ctx));
  {
    static const char *opt_keys[] = {"fix_quirks", "dot_order", "graphs", "autotune", "lusgs_split", "lusgs_vw",
                                     "lusgs_pipelined", "stencil_by", "stencil_ctas"};
    for (int q = 0; q < (int)(sizeof(opt_keys) / sizeof(opt_keys[0])); q++) {
      int v;
      if (csem_getparint(opt_keys[q], &v)) check(csem_ctx_set_option(ctx, opt_keys[q], v));
    }
  }
  long sz[10];
  csem_ctx_sizes(ctx, sz);
  const long lE = sz[0];
  if (verb) printf("dof=%ld\n", lE);

  const int nrec = acq.nrec, nsrc = acq.nsrc;
  /* dcal[isrc][ic][ifreq][irec] complex64 (emf.h:42) */
  float *dcal = (float *)calloc((size_t)2 * nsrc * nchrec * nfreq * (nrec > 0 ? nrec : 1), sizeof(float));
  double *tmp = (double *)malloc(sizeof(double) * 2 * (size_t)nchrec * (nrec > 0 ? nrec : 1) * nfreq * nsrc + 16);

  if (precision == 32) {
    int nsys = nsrc * nfreq;
    float *fs = (float *)malloc(sizeof(float) * (size_t)nsys), *ss = (float *)malloc(sizeof(float) * 3 * (size_t)nsys);
    for (int s = 0; s < nsrc; s++)
      for (int k = 0; k < nfreq; k++) {
        fs[s * nfreq + k] = freqs[k];
        memcpy(ss + 3 * (s * nfreq + k), acq.src + 5 * s, sizeof(float) * 3);
      }
    int *it = (int *)calloc((size_t)nsys, sizeof(int)), *ou = (int *)calloc((size_t)nsys, sizeof(int));
    int *st = (int *)calloc((size_t)nsys, sizeof(int));
    double *rr = (double *)calloc((size_t)nsys, sizeof(double));
    csem_batch_opts o = {32, algopt, preco, niter, tol, inner_tol, check_every, max_outer, nrestart, mp};
    double t0 = now();
    check(csem_solve_batch_host(ctx, nsys, fs, ss, nchsrc, chsrc, nchrec, chrec, nrec, acq.rec, &o, tmp, it, ou, st, rr));
    double t1 = now();
    for (int s = 0; s < nsrc; s++)
      for (int k = 0; k < nfreq; k++) {
        int q = s * nfreq + k;
        if (verb)
          printf("source %d freq=%g Hz: status %d, %d complex64 iterations, %d defect corrections, relres=%e\n",
                 s + 1, freqs[k], st[q], it[q], ou[q], rr[q]);
        for (int c = 0; c < nchrec; c++)
          for (int r = 0; r < nrec; r++) {
            size_t from = 2 * (((size_t)q * nchrec + c) * nrec + r);
            size_t to = 2 * ((((size_t)s * nchrec + c) * nfreq + k) * nrec + r);
            dcal[to] = (float)tmp[from];
            dcal[to + 1] = (float)tmp[from + 1];
          }
      }
    if (verb) printf("elapsed time: %g sec (%d systems in one batch)\n", t1 - t0, nsys);
    free(fs); free(ss); free(it); free(ou); free(st); free(rr);
  } else {
    double *b = (double *)malloc(sizeof(double) * 2 * (size_t)lE);
    double *x = (double *)malloc(sizeof(double) * 2 * (size_t)lE);
    const int hcap = niter + 16 + 2 * niter;
    double *hist = (double *)malloc(sizeof(double) * (size_t)hcap);
    for (int s = 0; s < nsrc; s++)
      for (int k = 0; k < nfreq; k++) {
        float tolf = tol / freqs[k]; /* main.c:94, in float */
        double iom_im = ((2. * 3.14159265358979323846264) * (double)freqs[k]) * (4. * 3.14159265358979323846264 * 1e-7);
        if (verb) printf("------freq=%g Hz, tol=%e--------\n", freqs[k], tolf);
        check(csem_inject_host(ctx, 0.0, iom_im, nchsrc, chsrc, acq.src + 5 * s, b));
        memset(x, 0, sizeof(double) * 2 * (size_t)lE);
        int nh = 0, iters = 0, status = 0;
        double t0 = now();
        check(csem_solve_fp64_host(ctx, algopt, preco, niter, tolf, nrestart, mp, 0.0, iom_im, b, x, hist, hcap, &nh,
                                   &iters, &status));
        double t1 = now();
        if (verb && status != CSEM_ST_ZERO_RHS) {
          FILE *fp = fopen(hist_name(algopt, preco), "w");
          if (fp) {
            fprintf(fp, algopt == 1 ? "iteration \t relres\n" : "iteration \t error\n");
            const int nprint = csem_history_logged(algopt, preco, status, nh < hcap ? nh : hcap);
            for (int q = 0; q < nprint; q++) fprintf(fp, "%d \t %e\n", q, hist[q]);
            fclose(fp);
          }
          if (status == CSEM_ST_CONVERGED) printf("converged at iter=%d\n", iters);
          printf("elapsed time: %g sec\n", t1 - t0);
        }
        check(csem_extract_host(ctx, nchrec, chrec, nrec, acq.rec, x, tmp));
        for (int c = 0; c < nchrec; c++)
          for (int r = 0; r < nrec; r++) {
            size_t from = 2 * ((size_t)c * nrec + r);
            size_t to = 2 * ((((size_t)s * nchrec + c) * nfreq + k) * nrec + r);
            dcal[to] = (float)tmp[from];
            dcal[to + 1] = (float)tmp[from + 1];
          }
      }
    free(b); free(x); free(hist);
  }
  for (int s = 0; s < nsrc; s++) {
    char fname[64];
    snprintf(fname, sizeof(fname), "emf_%04d.txt", s + 1);
    check(csem_write_emf(fname, s + 1, nchrec, nfreq, nrec, dcal + 2 * (size_t)s * nchrec * nfreq * nrec));
  }
  csem_ctx_destroy(ctx);
  csem_acq_free(&acq);
  csem_grid_free(&g);
  free(dcal);
  free(tmp);
  free(freqs);
  return 0;
}
