/* CPU oracle for the GB300 CSEM solver - TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's hot path (fdfd.c, airbc_init_free.c:130-209,
 * inject_extract.c, cdotprod.c, solver.c, gmres_init_free.c), used only by tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg as the checker. Nothing in
 * the product links or calls it.
 *
 * Every operation is written in the reference's order with complex arithmetic spelled
 * out on real/imaginary doubles: a*b = (ar*br - ai*bi, ar*bi + ai*br); complex/real and
 * real*complex act componentwise; complex/complex uses Smith's method (R. L. Smith,
 * "Algorithm 116: Complex division", CACM 5(8), 1962), which is what GCC's runtime
 * computes for operands in the normal range. Built with -ffp-contract=off, the
 * oracle reproduces the compiled reference bit for bit on x86-64 and aarch64; this is
 * pinned by tests against the reference built from its sources and by the golden
 * fixtures in tests/golden (generated from that build).
 *
 * Vectors are complex128 stored as interleaved doubles in the reference's layout:
 * E = [Ex | Ey | Ez] with Ex(k,j,i) at i + n1*(j + (n2+1)*k), Ey at
 * i + (n1+1)*(j + n2*k), Ez at i + (n1+1)*(j + (n2+1)*k)   (fdfd.c:13-15).
 */
#ifndef CSEM_ORACLE_H
#define CSEM_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

/* Model description; all arrays are borrowed and must outlive the context.
 * 1-D arrays cover the FULL padded grid (length n+1); conductivities are the
 * full-grid flat arrays of extend_model.c:180-252. */
typedef struct orc_desc {
  int n1, n2, n3f;        /* full padded grid */
  int nb, nz;             /* padding depth, core cells in z */
  int airbc, fvm;
  const double *x1, *x2, *x3, *x1s, *x2s, *x3s;
  const double *d1, *d2, *d3, *d1s, *d2s, *d3s;
  const double *sigma11, *sigma22, *sigma33;
  double rho_water;
  /* airwave (airbc=1) */
  int n1fft, n2fft;
  double d1fft, d2fft;
  const double *sH1, *sH2;   /* complex [n2fft][n1fft] */
  const int *jx, *jy;
  const double *wx, *wy;
} orc_desc_t;

typedef struct orc_ctx orc_ctx_t;

orc_ctx_t *orc_create(const orc_desc_t *d);
void orc_destroy(orc_ctx_t *c);
/* I*omega*mu0 as the driver sets it (main.c:95). */
void orc_set_iom(orc_ctx_t *c, double re, double im);
void orc_set_freq(orc_ctx_t *c, float freq);
/* sizes: [lE, lEx, lEy, lEz, lH, lv, n3 (operator grid)] */
void orc_sizes(const orc_ctx_t *c, long *out);

/* y = A x (fdfd.c:86-205); H is left in the context (orc_get_h). */
void orc_fdfd_apply(orc_ctx_t *c, const double *x, double *y);
/* legacy one-pass Dirichlet operator (fdfd.c:212-284), a cross-check of the above */
void orc_fdfd_apply_old(orc_ctx_t *c, const double *x, double *y);
/* Hy scratch length: sic != 0 (the default) as fdfd.c:59 (n1*(n2+1)*n2: Hy and Hz overlap
   when n2 < n3, and fdfd_apply then mixes the two), 0 for n1*(n2+1)*n3. */
void orc_set_hy_length(orc_ctx_t *c, int sic);
void orc_get_h(const orc_ctx_t *c, double *h);
/* y = M^-1 x, LU-SGS (fdfd.c:287-510) */
void orc_lusgs_apply(orc_ctx_t *c, const double *x, double *y);
/* y = M^-1 x, A-phi (fdfd.c:513-821) */
void orc_aphi_apply(orc_ctx_t *c, const double *x, double *y);
/* y = M^-1 x, fixed mp-step GMRES on A (gmres_init_free.c:58-137) */
void orc_gmres_pre_apply(orc_ctx_t *c, int mp, const double *x, double *y);
/* Hz(z=0) plane [n2][n1] -> ghosts Hx [(n2)][(n1+1)], Hy [(n2+1)][n1] (airbc_init_free.c:130-209) */
void orc_airbc_apply(orc_ctx_t *c, const double *hz0, double *hx, double *hy);

/* s = sum a_i conj(b_i), sequential (cdotprod.c:13-19) */
void orc_cdot(long n, const double *a, const double *b, double *out);

/* Krylov solvers (solver.c). precond: 0 none, 1 LU-SGS, 2 inner GMRES(mp), 3 A-phi.
 * hist (optional, capacity hist_cap) receives every relative residual the solver
 * computes, in order; *nhist its count. Return value: iterations performed
 * (BiCGStab: loop index at exit; GMRES: restart cycles). */
int orc_bicgstab(orc_ctx_t *c, double *x, const double *b, int niter, double tol,
                 double *hist, int hist_cap, int *nhist);
int orc_fbicgstab(orc_ctx_t *c, int precond, int mp, double *x, const double *b, int niter,
                  double tol, double *hist, int hist_cap, int *nhist);
int orc_gmres(orc_ctx_t *c, double *x, const double *b, int niter, double tol, int m,
              double *hist, int hist_cap, int *nhist);
int orc_fgmres(orc_ctx_t *c, int precond, int mp, double *x, const double *b, int niter,
               double tol, int m, double *hist, int hist_cap, int *nhist);

/* Source injection into b (inject_source, inject_extract.c:24-120). b is zeroed
 * first. ch: 0=Ex, 1=Ey, 2=Ez; other codes inject nothing. src = x1,x2,x3 (float). */
void orc_inject(orc_ctx_t *c, int nch, const int *ch, const float *src, double *b);
/* Receiver extraction (extract_emf, inject_extract.c:123-213). rec: [nrec][5] rows;
 * out: complex128 [nch][nrec] (the value before the complex64 store). */
void orc_extract(orc_ctx_t *c, int nch, const int *ch, int nrec, const float *rec,
                 const double *x, double *out);

#ifdef __cplusplus
}
#endif
#endif
