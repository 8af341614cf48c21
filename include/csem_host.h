/* csem_host.h - host-side C layer of the GB300 CSEM solver (libcsem_gpu.so).
 *
 * These functions keep the reference driver's inputs and outputs: the CWP-style
 * key=value flag table, the float32 fx1..3 and frho11..33 model files, the text source/receiver
 * files, the padded stretched grid with edge-averaged conductivities, and the
 * emf_NNNN.txt receiver table. They run once per model on the CPU; the per-iteration
 * work runs on the GPU through csem_gpu.h.
 *
 * Errors are returned as negative CSEM_E* codes with a message in csem_last_error();
 * the key=value driver turns them into the reference's print-and-exit(1) behaviour
 * (cstd.c:1539-1552).
 */
#ifndef CSEM_HOST_H
#define CSEM_HOST_H
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CSEM_OK 0
#define CSEM_EINVAL (-1)   /* bad argument or flag value */
#define CSEM_EIO (-2)      /* missing, short or unreadable file */
#define CSEM_ENOMEM (-3)   /* host or device allocation failed */
#define CSEM_EDOMAIN (-4)  /* acquisition outside the model (acq_init_free.c:133-138) */
#define CSEM_ECUDA (-5)    /* CUDA runtime or cuFFT error */
#define CSEM_ENODEV (-6)   /* no CUDA device available */
#define CSEM_ETOOBIG (-7)  /* size beyond a fixed capacity */

/* Message describing the most recent error on this thread ("" if none). */
const char *csem_last_error(void);

/* ---------------------------------------------------------------- flags ----
 * Same semantics as the reference's getpar (cstd.c:936-1436): "name=value" tokens;
 * the LAST occurrence of a name wins; comma-separated vectors; an optional
 * "par=file" whose whitespace-separated name=value tokens come before the command
 * line; tokens without '=' are ignored. Replaces initargs/getpar* (cstd.h:131-156). */
void csem_initargs(int argc, char **argv);
int csem_countparval(const char *name);             /* values in last occurrence, 0 if absent */
int csem_getparint(const char *name, int *p);       /* fills up to count values, returns count */
int csem_getparfloat(const char *name, float *p);   /* strtod then rounded to float (eatof) */
int csem_getpardouble(const char *name, double *p);
int csem_getparstring(const char *name, char **p);  /* whole value, commas kept */
int csem_getparstringarray(const char *name, char **p); /* comma fields, newly allocated */

/* ---------------------------------------------------------------- model ----
 * Replaces the model half of emf_t (emf.h:4-57) as filled by emf_init
 * (emf_init_free.c:14-172), extend_model_init (extend_model.c:24-252) and
 * airbc_init (airbc_init_free.c:24-109). All 1-D arrays have length n+1 of the
 * FULL padded grid (n1 = nx+2nb etc.). Conductivities are stored flat in the
 * reference's index order on the full grid:
 *   sigma11[(k*(n2+1) + j)*n1 + i]        k<=n3, j<=n2, i<n1
 *   sigma22[(k*n2 + j)*(n1+1) + i]         k<=n3, j<n2,  i<=n1
 *   sigma33[(k*(n2+1) + j)*(n1+1) + i]     k<n3,  j<=n2, i<=n1                 */
typedef struct csem_grid {
  /* input model (float32 files) */
  int nx, ny, nz;
  float *x1node, *x2node, *x3node;
  float *rho11, *rho22, *rho33;      /* [nz][ny][nx] */
  float rhomin, rhomax, rho_water, rho_air, lextend;
  int nb, istretch, airbc, fvm;
  /* padded grid */
  int n1, n2, n3;                    /* nx+2nb, ny+2nb, nz+2nb */
  double *x1, *x2, *x3, *x1s, *x2s, *x3s;
  double *d1, *d2, *d3, *d1s, *d2s, *d3s;
  double *sigma11, *sigma22, *sigma33;
  double rstretch[6];                /* left, right, front, rear, top, bottom */
  double d1min, d2min, d3min;
  /* airwave tables (only when airbc) */
  int n1fft, n2fft;
  double d1fft, d2fft, d3fft;
  double *sH1, *sH2;                 /* complex, interleaved re/im, [n2fft][n1fft] */
  int *jx, *jy;
  double *wx, *wy;
} csem_grid_t;

/* Read fx1..3 and frho11..33 (emf_init_free.c:77-166): cell counts from the file
 * sizes, rho_water = min over all three resistivity arrays. */
int csem_grid_read(csem_grid_t *g, const char *fx1, const char *fx2, const char *fx3,
                   const char *frho11, const char *frho22, const char *frho33);
/* Use caller-provided float32 arrays instead of files (copied). */
int csem_grid_set(csem_grid_t *g, int nx, int ny, int nz, const float *x1node,
                  const float *x2node, const float *x3node, const float *rho11,
                  const float *rho22, const float *rho33);
/* Pad, stretch and average (extend_model.c:24-252 incl. create_nugrid.c:16-40).
 * lextend < 0 selects the reference default (40e3 when nb>0, else 0). */
int csem_grid_extend(csem_grid_t *g, int nb, float lextend, float rho_air, int istretch);
/* Airwave tables (airbc_init_free.c:24-105); n1fft, n2fft <= 0 select 1024. */
int csem_grid_airbc(csem_grid_t *g, int n1fft, int n2fft);
void csem_grid_free(csem_grid_t *g);
/* Write the padded model as float64 (extend_model.c:254-289, param_extended=1). */
int csem_grid_write_extended(const csem_grid_t *g, const char *dir);

/* ----------------------------------------------------------- acquisition ---
 * Replaces acq_init (acq_init_free.c:14-148). Reads every row (up to 5000) of the
 * source and receiver files; unlike the reference, all source rows are kept
 * (nsrc_total); the reference solves only the first (nsrc=1). */
#define CSEM_MAX_ACQ_ROWS 5000
typedef struct csem_acq {
  int nsrc, nrec;
  float *src;   /* [nsrc][5]: x1 x2 x3 azimuth dip */
  float *rec;   /* [nrec][5] */
} csem_acq_t;
int csem_acq_read(csem_acq_t *a, const char *fsrc, const char *frec);
/* Check every source and receiver lies inside the input model (acq_init_free.c:133-138). */
int csem_acq_check(const csem_acq_t *a, const csem_grid_t *g);
void csem_acq_free(csem_acq_t *a);

/* ---------------------------------------------------------------- output ---
 * How many entries of a residual history (nh values: the initial one, then one per
 * BiCGStab step or GMRES inner step) the reference writes to iterate_*.txt:
 *  - bicgstab / fbicgstab log the previous step's residual at the top of each step
 *    (solver.c:49-54,136-141), so the last one computed is never logged;
 *  - gmres (no preconditioner) stops on convergence before logging that residual
 *    (solver.c:251-255); fgmres logs it first (solver.c:474-481);
 *  - a zero right-hand side logs nothing: the solvers return before opening the file.
 * algopt 1 BiCGStab, 2 GMRES; preco 0 none; status a CSEM_ST_* value (csem_gpu.h). */
int csem_history_logged(int algopt, int preco, int status, int nh);

/* emf_NNNN.txt as write_data (write_data.c:15-37): header line, then
 * "iTx iRx ichrec ifreq re im" in ichrec > ifreq > irec order, values printed %e
 * from complex64. dcal is complex64 interleaved [nchrec][nfreq][nrec][2]. */
int csem_write_emf(const char *fname, int isrc, int nchrec, int nfreq, int nrec,
                   const float *dcal);

/* Sort frequencies ascending the way the reference does (qsort with an int
 * comparator on the float bit patterns, emf_init_free.c:12,27). */
void csem_sort_freqs(float *freqs, int n);

/* ---------------------------------------------------------------- systems over GPUs ---
 * Split nsys independent systems over ndev devices so that the expected work per device
 * is balanced. No counterpart in the reference, which solves one system per process
 * (main.c:93-123; its acquisition keeps only the first source, acq_init_free.c:56,90).
 * The work of system s is cost[s] when cost is given; otherwise unknowns * freq[s]^(-2/3):
 * BiCGStab + LU-SGS iteration counts fall with frequency about as f^(-2/3) on the bench
 * model (the complex128 solver needs 1521, 987, 633, 423, 338 and 327 iterations at
 * 0.125, 0.25, 0.5, 0.75, 1.0 and 1.25 Hz for its first source). Longest work first:
 * systems in decreasing work (ties: lower index first) each go to the device with the
 * least work so far (ties: lower slot), so the split is deterministic. owner[s] receives
 * the slot 0..ndev-1 of system s; load (may be NULL) the summed work per slot.
 * CSEM_EINVAL for ndev < 1, nsys < 0, missing arrays or non-positive work. */
int csem_partition_systems(int nsys, const float *freq, const double *cost, double unknowns, int ndev, int *owner,
                           double *load);

#ifdef __cplusplus
}
#endif
#endif
