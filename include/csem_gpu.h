/* csem_gpu.h - C ABI of the GB300 CSEM solver (libcsem_gpu.so).
 *
 * The reference's hot path is a set of C callbacks over a global model
 * (op_t = void (*)(int, complex*, complex*), solver.h:4; emf set by fdfd_init,
 * fdfd.c:23,30-63). This library replaces it with a handle (csem_ctx) that owns one
 * padded model resident in GPU memory, a CUDA stream and workspaces, plus entry points
 * that take plain pointers and sizes.
 *
 * Conventions
 *  - complex128 vectors are interleaved doubles (re, im), complex64 interleaved floats,
 *    in the reference's layout E = [Ex | Ey | Ez] with Ex(k,j,i) at i + n1*(j+(n2+1)*k),
 *    Ey at i + (n1+1)*(j+n2*k), Ez at i + (n1+1)*(j+(n2+1)*k) (fdfd.c:13-15), on the
 *    operator grid (n3 = nz+nb with airbc=1, else nz+2nb);
 *  - "_host" buffers live in host memory (copied in and out inside the call); "_dev"
 *    buffers are device pointers and `stream` is a cudaStream_t (NULL: the context's);
 *  - every function returns CSEM_OK (0) or a negative CSEM_E* code (csem_host.h) and
 *    leaves a message in csem_last_error(); nothing exits the process;
 *  - iom = I*omega*mu0 = (0, 2*pi*f*mu0) as the reference's driver sets it (main.c:95).
 * The FP64 entry points reproduce the reference's arithmetic bit for bit except for the
 * summation order inside dot products (deterministic, fixed tree).
 */
#ifndef CSEM_GPU_H
#define CSEM_GPU_H
#include "csem_host.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct csem_ctx csem_ctx;

const char *csem_version(void);
/* number of visible CUDA devices (0 without a GPU; never fails) */
int csem_device_count(void);

/* Upload a padded model (csem_grid_extend / csem_grid_airbc done) for the operator
 * with airbc/fvm. Replaces fdfd_init (fdfd.c:30-63) and airbc_init
 * (airbc_init_free.c:24-109) state. */
int csem_ctx_create(const csem_grid_t *g, int airbc, int fvm, csem_ctx **out);
/* Replaces fdfd_free (fdfd.c:65-80) / airbc_free (airbc_init_free.c:111-124). */
void csem_ctx_destroy(csem_ctx *c);
/* [lE, lEx, lEy, lEz, lv, n1, n2, n3(operator), n3 full, nb] */
int csem_ctx_sizes(const csem_ctx *c, long *out10);

/* ------------------------------------------------------------ operators (FP64)
 * y = A x. Replaces fdfd_apply (fdfd.c:86-205). */
int csem_fdfd_apply_host(csem_ctx *c, double iom_re, double iom_im, const double *x, double *y);
/* y = M^-1 x, LU-SGS. Replaces lusgs_apply (fdfd.c:287-510). */
int csem_lusgs_apply_host(csem_ctx *c, double iom_re, double iom_im, const double *x, double *y);
/* y = M^-1 x, A-phi. Replaces aphi_apply (fdfd.c:513-821). */
int csem_aphi_apply_host(csem_ctx *c, double iom_re, double iom_im, const double *x, double *y);
/* y = M^-1 x, mp steps of GMRES on A. Replaces gmres_apply (gmres_init_free.c:58-137). */
int csem_gmres_pre_apply_host(csem_ctx *c, double iom_re, double iom_im, int mp, const double *x, double *y);
/* Airwave ghosts from Hz(z=0) [n2][n1] -> Hx [n2][n1+1], Hy [n2+1][n1].
 * Replaces airbc_apply (airbc_init_free.c:130-209). */
int csem_airbc_apply_host(csem_ctx *c, const double *hz0, double *hx, double *hy);

/* ------------------------------------------------------------ operators (complex64)
 * The same operators in complex64, as the mixed-precision inner solver runs them. */
int csem_fdfd_apply_c64_host(csem_ctx *c, double iom_re, double iom_im, const float *x, float *y);
int csem_lusgs_apply_c64_host(csem_ctx *c, double iom_re, double iom_im, const float *x, float *y);
int csem_aphi_apply_c64_host(csem_ctx *c, double iom_re, double iom_im, const float *x, float *y);

/* ------------------------------------------------------------ dot products
 * out = sum a_i conj(b_i). Replaces cdotprod (cdotprod.c:13-19). */
int csem_cdot_host(long n, const double *a, const double *b, double *out2);
int csem_cdot_c64_host(long n, const float *a, const float *b, double *out2);

/* ------------------------------------------------------------ source / receivers
 * b = unit dipole(s) at src = (x1,x2,x3) for channels ch[] (0 Ex, 1 Ey, 2 Ez); b is
 * zeroed first. Replaces inject_source (inject_extract.c:24-120). */
int csem_inject_host(csem_ctx *c, double iom_re, double iom_im, int nch, const int *ch, const float *src3,
                     double *b);
/* out[ic][r] (complex128) = receiver r of channel ch[ic]; rec is [nrec][5] rows
 * (x1 x2 x3 azimuth dip). Replaces extract_emf (inject_extract.c:123-213); the caller
 * stores complex64 where the reference does (emf.h:42). */
int csem_extract_host(csem_ctx *c, int nch, const int *ch, int nrec, const float *rec, const double *x,
                      double *out);

/* ------------------------------------------------------------ FP64 solve of one system
 * The dispatch of main.c:104-118 on a device-resident system: algopt 1 = BiCGStab,
 * 2 = GMRES(nrestart); preco 0 none, 1 LU-SGS, 2 inner GMRES(mp), 3 A-phi. niter is
 * the reference's iteration limit (GMRES runs niter/nrestart restart cycles, as
 * main.c:106,109). Replaces bicgstab/fbicgstab/gmres/fgmres (solver.c:16-512).
 * x: initial guess in, solution out. hist receives the relative residuals in order
 * (*nhist of them, at most hist_cap copied); *iters the iterations (BiCGStab) or cycles
 * (GMRES); *status a CSEM_ST_* value. */
#define CSEM_ST_RUNNING 0
#define CSEM_ST_CONVERGED 1
#define CSEM_ST_MAXITER 2
#define CSEM_ST_BREAKDOWN 3
#define CSEM_ST_NONFINITE 4
#define CSEM_ST_ZERO_RHS 5
int csem_solve_fp64_host(csem_ctx *c, int algopt, int preco, int niter, double tol, int nrestart, int mp,
                         double iom_re, double iom_im, const double *b, double *x, double *hist, int hist_cap,
                         int *nhist, int *iters, int *status);

/* ------------------------------------------------------------ many systems at once
 * Solve nsys independent systems (frequency freq[s], unit dipole at src3[s] on the
 * channels chsrc) on the context's model and extract the receivers. This replaces the
 * reference driver's per-frequency loop (main.c:93-123: injection, timed solve,
 * extraction) for every (frequency, source) pair at once; the reference itself solves
 * only the first source row (acq_init_free.c:56,90).
 *   precision 32: batched mixed precision - complex64 flexible BiCGStab (algopt 1) or
 *                 flexible GMRES(nrestart) (algopt 2) with complex64 LU-SGS (preco 1)
 *                 or A-phi (preco 3) inside complex128 defect correction; a system
 *                 stops when |b - A x| / |b| < tol/f (complex128, true residual);
 *   precision 64: the plain complex128 solver of csem_solve_fp64_host, one system after
 *                 the other (algopt/preco/nrestart/mp as the reference).
 * Outputs per system: dcal [nsys][nchrec][nrec] complex128 receivers, iters (inner
 * complex64 iterations, or complex128 iterations / GMRES cycles), outer (defect-
 * correction cycles), status (CSEM_ST_*), relres (final relative residual). */
typedef struct csem_batch_opts {
  int precision;     /* 32 or 64 */
  int algopt;        /* 1 BiCGStab, 2 GMRES */
  int preco;         /* 0 none, 1 LU-SGS, 2 inner GMRES (64 only), 3 A-phi */
  int niter;         /* the reference's niter */
  float tol;         /* the reference's tol; system s stops at tol/freq[s] in float (main.c:94) */
  double inner_tol;  /* precision 32: relative reduction of one inner solve (<= 0: 0.2) */
  int check_every;   /* precision 32: inner iterations between status reads (<= 0: 4) */
  int max_outer;     /* precision 32: defect-correction cycles (<= 0: 30) */
  int nrestart, mp;  /* GMRES(nrestart); precision 64: GMRES(mp) preconditioner */
} csem_batch_opts;
int csem_solve_batch_host(csem_ctx *c, int nsys, const float *freq, const float *src3, int nchsrc,
                          const int *chsrc, int nchrec, const int *chrec, int nrec, const float *rec,
                          const csem_batch_opts *opt, double *dcal, int *iters, int *outer, int *status,
                          double *relres);

/* ------------------------------------------------------------ several models at once
 * Solve independent batches on different contexts (different models, grid sizes or
 * padding) at the same time: one host thread per job drives that context's
 * csem_solve_batch_host on the context's own stream, so the GPU overlaps the contexts'
 * kernels. This is the uneven-size batch of several models (e.g. one context per model
 * and per padding); the reference solves one system of one model at a time (main.c:93-123).
 * Each job names a distinct context; rc receives that job's return code. Returns CSEM_OK
 * when every job succeeded, else the first failing job's code. */
typedef struct csem_batch_job {
  csem_ctx *ctx;
  int nsys;
  const float *freq, *src3;
  int nchsrc;
  const int *chsrc;
  int nchrec;
  const int *chrec;
  int nrec;
  const float *rec;
  const csem_batch_opts *opt;
  double *dcal;
  int *iters, *outer, *status;
  double *relres;
  int rc;
} csem_batch_job;
int csem_solve_batches_host(int njobs, csem_batch_job *jobs);

/* ------------------------------------------------------------ systems over several GPUs
 * Solve nsys systems of one model on ndev devices: csem_partition_systems splits them
 * (work = unknowns x freq^(-2/3)), every slot d gets its own context on CUDA device
 * devices[d] (model upload, stream, workspaces) driven by its own host thread through
 * csem_solve_batch_host, and each slot writes its systems' outputs at their original
 * positions in the caller's arrays: the only gather is these host writes, with no
 * communication between the GPUs. owner (may be NULL) receives each system's slot.
 * The same device may be named by several slots (independent contexts share it).
 * The reference solves one system per process (main.c:93-123). Returns CSEM_OK, or the
 * code of the first slot that failed (with that slot's message). */
int csem_solve_batch_multi(int ndev, const int *devices, const csem_grid_t *g, int airbc, int fvm, int nsys,
                           const float *freq, const float *src3, int nchsrc, const int *chsrc, int nchrec,
                           const int *chrec, int nrec, const float *rec, const csem_batch_opts *opt, double *dcal,
                           int *iters, int *outer, int *status, double *relres, int *owner);

/* The same-frequency groups the batched complex64 LU-SGS of a set of slots uses (no device
 * work; for callers planning batches, and for tests): slots with equal iom (re, im pairs
 * per slot) form groups of at most ns, the slots of one frequency in order, the
 * frequencies in order of first appearance. halves != 0 and nslot >= 8: built separately
 * for slots [0, nslot/2) and [nslot/2, nslot), each half numbering its slots from 0, as
 * the split sweeps on two streams use them; *nA and *ngA are then the first half's slots
 * and groups (0 otherwise). groups receives *ngroups x ns entries, -1 where a group has
 * fewer members, and must hold nslot x ns. */
int csem_sweep_groups(int nslot, const double *iom, int ns, int halves, int *groups, int *ngroups, int *nA,
                      int *ngA);

/* Capacity planning for large sets of systems (no counterpart in the reference, which
 * solves one system at a time). csem_batch_bytes: device bytes csem_solve_batch_host
 * needs for nsys systems with this precision and preconditioner, beyond the model and
 * cuFFT's work areas. csem_batch_capacity: the largest nsys whose batch fits in
 * budget_bytes (precision 64 solves one system at a time: any count if one fits, else 0).
 * Callers with more systems solve them in waves of that size. Both count the mixed path's
 * BiCGStab inner solver (algopt 1); its GMRES inner solver (algopt 2) needs
 * (2 nrestart + 4) x 8 bytes more per unknown and system, for its basis. */
int csem_batch_bytes(csem_ctx *c, int precision, int preco, int nsys, double *bytes);
int csem_batch_capacity(csem_ctx *c, int precision, int preco, double budget_bytes, int *nsys);

/* ------------------------------------------------------------ device-pointer entry points
 * For callers that keep vectors in GPU memory. nsys systems are stored back to back
 * (stride lE); iom is a host array of nsys (re, im) pairs. prec: 64 = complex128,
 * 32 = complex64. */
int csem_fdfd_apply_dev(csem_ctx *c, int prec, int nsys, const double *iom, const void *x, void *y, void *stream);
int csem_lusgs_apply_dev(csem_ctx *c, int prec, int nsys, const double *iom, const void *x, void *y, void *stream);
int csem_aphi_apply_dev(csem_ctx *c, int prec, int nsys, const double *iom, const void *x, void *y, void *stream);
/* out[s] (complex128, device) = <a_s, b_s> for nsys vectors of length n (stride n).
 * The per-block partial sums live in a buffer the library allocates on first use, one
 * per host thread and device, and grows on demand. Calls from one host thread on one
 * device share that buffer: two such calls on different streams that overlap in time
 * race on it, so order them (one stream, or an event between them). */
int csem_cdot_dev(int prec, long n, int nsys, const void *a, const void *b, double *out_dev, void *stream);
/* The same dot products, identical bits, without any device allocation by the library.
 * No counterpart in the reference (its cdotprod, cdotprod.c:13-19, is a host loop).
 * For callers that cannot let a library allocate: one that has handed all free device
 * memory to its own pool, or a loop that cannot absorb the device-wide synchronisation
 * cudaMalloc/cudaFree may bring. csem_cdot_dev allocates its partial-sum buffer on first
 * use; this variant keeps the partials in a fixed 1 MiB array inside the library's
 * device image instead.
 *  - nsys <= CSEM_NOALLOC_DOT_MAX_SYSTEMS, else CSEM_ETOOBIG with a message;
 *  - the first call on a device (made with that device current) looks the array up with
 *    cudaGetSymbolAddress and caches it: make that call before any stream capture starts;
 *  - the array is shared by all calls on a device: calls that overlap in time (other
 *    streams, other host threads) race on it; serialise them;
 *  - nothing needs clearing beforehand: each call writes every partial it reads;
 *  - the cached address is not refreshed: calling cudaDeviceReset on a device between
 *    two calls is not supported (the module, and with it the array, is reloaded). */
#define CSEM_NOALLOC_DOT_MAX_SYSTEMS 64
int csem_cdot_dev_noalloc(int prec, long n, int nsys, const void *a, const void *b, double *out_dev, void *stream);
/* The assembled operator as a comparison point (Acsr_init / Acsr_apply, Acsr.c:704-716,
 * which the reference uses only as a check): A is assembled in CSR on the device by
 * probing the matrix-free operator with 81 indicator vectors (13 stored entries per
 * row, 32-bit indices), then cuSPARSE's SpMV and the stencil are each timed nrep times on
 * one random vector. out[0] ms per SpMV, out[1] ms per stencil application, out[2] max
 * relative difference of the two products, out[3] stored entries, out[4] bytes one SpMV
 * must move (values, indices, row pointers, x, y). prec 64 or 32. airbc=0 only, as the
 * reference's assembly: the airwave couples the top plane through an FFT. */
int csem_csr_compare(csem_ctx *c, int prec, double iom_re, double iom_im, int nrep, double *out);
/* synchronise the context's stream */
int csem_ctx_sync(csem_ctx *c);
/* the context's CUDA stream (a cudaStream_t), for callers that record events on it */
void *csem_ctx_stream(csem_ctx *c);
/* Kernel-schedule and solver options. complex128 results do not depend on the schedule
 * options; complex64 results may differ in the last bits between schedules:
 *   "lusgs_pipelined" 1 (default): one launch per LU-SGS component sweep, rows as a
 *                     lockstep pipeline; 0: one launch per wavefront diagonal;
 *   "lusgs_vw"        points per thread and step of the pipelined (and split) sweeps: 1,
 *                     2, 4, or 0 for the default (2 complex64, 1 complex128).
 *   "lusgs_lines"     complex64 with lusgs_split 0 only: lines one CTA of the pipelined
 *                     sweeps carries one after the other (1..64), so the row pipeline fills
 *                     and drains once per CTA instead of once per line; 1 (default): one
 *                     line per CTA;
 *   "lusgs_split"     complex64 only. 1 (default): each LU-SGS component sweep runs as
 *                     a coalesced pass that forms every point's b/aii + w (known - cross)
 *                     and w = iwmu/aii (once per point for all the systems of a frequency)
 *                     and a row pipeline that reads them and runs only the dependent chain;
 *                     0: the one-pass pipelined sweeps. Same values to rounding;
 *   "quick_residual"  1 (default): the batched mixed-precision solve forms its complex128
 *                     residuals r = b - A x with a complex128 stencil that multiplies by
 *                     reciprocal spacings and lets the compiler contract multiply-adds
 *                     (complex128 accuracy, not the reference's rounding: the defect
 *                     correction needs no more); 0: the bit-faithful complex128 stencil.
 *                     The complex128 solver (precision 64) and the operator entry points
 *                     always use the bit-faithful one;
 *   "fused_dots"      1: the batched complex64 BiCGStab forms v.r0 after v = A p and s.t,
 *                     t.t after t = A s inside the operator's stencil (one deterministic
 *                     partial per CTA); 0 (default): separate dot-product passes, which
 *                     measured faster (the compensated sums double the stencil's
 *                     instructions). The two partition the sums differently;
 *   "lusgs_overlap"   with lusgs_split 1: 1 (default) runs batches of 8 or more systems
 *                     as two halves on two streams, so that one half's passes overlap the
 *                     other half's pipelines; 0: one stream. Same bits either way;
 *   "lusgs_cap"       on two streams, the split pipelines run this many CTAs per SM,
 *                     each taking lines in turn, to leave the other half's passes room on
 *                     the SMs (1..16); 0 (default): one CTA per line. Same bits either way;
 *   "lusgs_systems"   complex64 only: systems of one frequency one CTA of the pipelined
 *                     sweeps carries, 1 (default), 2 or 4. The members share the loads of
 *                     the grid and the frequency-only part of each point's update, and
 *                     each warp runs one dependent chain per member. With 2, lusgs_vw 2
 *                     gives 2 points per thread and step, any other value 1; 4 takes 1.
 *                     Sweeps of more than 256 rows run one system per CTA. Applies with
 *                     lusgs_split 0;
 *   "lusgs_tiled"     complex64 only. 1: line-tiled sweeps - 32 independent lines per CTA
 *                     (one lane each), the rows cut into one block per warp; 0: the
 *                     schedule chosen by lusgs_pipelined. Same values as the pipelined
 *                     complex64 sweeps;
 *   "aphi_fix"        1: the A-phi preconditioner's node-potential sweeps use the
 *                     diagonal of div(sigma grad v), the face conductivities on it as on
 *                     the couplings, all read from the operator grid; 0 (default): the
 *                     reference's sweeps (fdfd.c:655-710), whose diagonal omits the
 *                     conductivities and whose lower-face lookups skip the air-layer shift,
 *                     so a sweep through seawater (sigma > 1 S/m) amplifies its input
 *                     geometrically (about 1e44 for a unit input on a 125 x 125 x 100 cell
 *                     bathymetry model). This option changes results;
 *   "lusgs_tile_rows" rows per warp block of the tiled sweeps: 4, 8 (default) or 16;
 *   "lusgs_tile_vw"   march positions per step of the tiled Ey and Ez sweeps: 1, 2 or 4
 *                     (default);
 *   "autotune"        1: the batched mixed-precision solve times the complex64 kernel
 *                     shapes on its first running systems and keeps the fastest for that
 *                     batch: split or one-pass LU-SGS sweeps, their points per thread
 *                     (1, 2, 4), lines per CTA (1, 2, 4) and systems per CTA (1, 2, 4), the
 *                     stencil's rows per CTA (4, 8, 16) and plane-chunk
 *                     depth (CTAs per SM 2, 4, 8); 0 (default): the fixed defaults.
 *                     complex64 results may then differ in the last bits from run to run,
 *                     so it is off by default;
 *   "stencil_by"      stencil tile height, output rows per CTA: 4, 8 (default) or 16;
 *   "stencil_ctas"    CTAs per SM the stencil's plane chunks aim for (1..16, default 4),
 *                     which sets the z-block depth. Neither stencil option changes results;
 *   "graphs"          1 (default): the batched BiCGStab replays the iterations between
 *                     two status reads as a captured CUDA graph (from the second time a
 *                     given number of systems is running; not while csem_profile is on);
 *                     0: direct launches;
 *   "dot_order"       complex128 solver only: 0 (default) dot products as a fixed
 *                     parallel tree; 1 in the reference's sequential order (cdotprod.c:13-19),
 *                     bit-identical to it, one dependent chain of additions per product,
 *                     so the solve reproduces the reference's iterates bit for bit
 *                     (without airbc; with airbc the FFT still differs in rounding) at
 *                     a large cost in time;
 *   "fix_quirks"      1: with airbc, source injection reads the conductivity at the
 *                     source's own row of the air-included model; 0 (default): the
 *                     reference's lookup after its -nb row shift (inject_extract.c:55-63,
 *                     81-89), which reads nb rows higher and can land in the air. This
 *                     option changes results (b, hence x and the receivers).
 */
int csem_ctx_set_option(csem_ctx *c, const char *name, int value);

/* ------------------------------------------------------------ timing
 * Per-operator device time from CUDA events recorded on the operator's stream around
 * every application (no counterpart in the reference, which times only whole solves,
 * main.c:103,119). Categories: 0/1 A (complex128/complex64, airwave included),
 * 2/3 LU-SGS, 4/5 A-phi, 6/7 airwave only, 8/9 stencil kernel only.
 * csem_profile(1) clears and starts recording, csem_profile(0) stops. */
int csem_profile(int enable);
/* ms: summed device milliseconds, count: applications, units (may be NULL): systems
 * processed summed over the applications */
int csem_profile_read(int ncat, double *ms, long *count, long *units);
/* kernel launches issued by this library since it was loaded (cuFFT's excluded) */
long long csem_launch_count(void);

#ifdef __cplusplus
}
#endif
#endif
