/* csem_refabi.h - same-symbol drop-in for the reference's hot path (libcsem_refabi.so).
 *
 * The reference driver (main.c) and its set-up and I/O files (emf_init_free.c,
 * acq_init_free.c, extend_model.c, create_nugrid.c, find_index.c, write_data.c, cstd.c)
 * can be linked against libcsem_refabi.so in place of fdfd.c, airbc_init_free.c,
 * inject_extract.c, cdotprod.c, solver.c and gmres_init_free.c. The functions below
 * keep the reference's names and signatures (main.c:17-43, solver.h:4); they read the
 * same emf_t / acq_t state and run on the GPU through csem_gpu.h.
 *
 * The two structs must have exactly the reference's member order and types
 * (emf.h:4-57, acq.h:4-19) because the reference's own objects fill them; the
 * declarations here restate that layout.
 *
 * Behaviour:
 *  - fdfd_init uploads the padded model once and fills the same emf_t lengths as
 *    fdfd.c:30-63 (n3 = nz+nb with airbc, lEx..lE, lHx..lH, lv);
 *  - fdfd_apply / lusgs_apply / aphi_apply / gmres_apply take host vectors (copy in,
 *    apply on the GPU, copy out);
 *  - bicgstab / fbicgstab / gmres / fgmres recognise this library's operators
 *    (Aop == fdfd_apply; invMop in {lusgs_apply, aphi_apply, gmres_apply}) and then run
 *    the whole solve on the GPU with x and b copied once each way; the history files
 *    (iterate_*.txt) and progress lines keep the reference's format. Other operator
 *    pointers are refused (message and exit(1), as err()).
 *  - the solvers' dot products use the library's fixed parallel tree; with the flag
 *    dot_order=1 (read through the reference's getparint when the driver links cstd.c)
 *    or CSEM_DOT_ORDER=1 in the environment they use the reference's sequential order
 *    (cdotprod.c:13-19), and a solve without airwave repeats the reference's iterates
 *    bit for bit;
 *  - errors print "csem_refabi: <message>" and exit(1), as the reference's err() does.
 */
#ifndef CSEM_REFABI_H
#define CSEM_REFABI_H
#include <complex.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef double _Complex csem_z;   /* the reference's `complex` (cstd.h includes complex.h) */
typedef float _Complex csem_zf;

typedef struct {
  int mode, verb, reciprocity, fvm, airbc;
  int nfreq;
  float *freqs;
  float rho_air, lextend, rho_water;
  float rhomin, rhomax;
  int nchsrc, nchrec;
  char **chsrc, **chrec;
  int istretch;
  float rstretch;
  int nx, ny, nz, nb;
  int n1, n2, n3;
  int lv, lE, lH, lEx, lEy, lEz, lHx, lHy, lHz;
  float *x1node, *x2node, *x3node;
  double *x1, *x2, *x3;
  double *x1s, *x2s, *x3s;
  double *d1, *d2, *d3;
  double *d1s, *d2s, *d3s;
  double d1min, d2min, d3min;
  double x1min, x2min, x3min;
  double x1max, x2max, x3max;
  int n1fft, n2fft;
  double d1fft, d2fft, d3fft;
  csem_z **sH1kxky, **sH2kxky;
  float ***rho11, ***rho22, ***rho33;
  double ***sigma11, ***sigma22, ***sigma33;
  csem_zf ****E1, ****E2, ****E3;
  csem_zf ***dcal_fd;
  int ne, nh;
  csem_z *xe, *xh, *be;
  csem_z *v, *bv;
  csem_z *xx, *yy;
  csem_z I_omega_mu0;
  int preco, algopt, niter, nrestart, mp;
  float tol;
  int param_extended;
} emf_t;

typedef struct {
  int nsrc, nrec, nsubsrc, nsubrec;
  float lensrc, lenrec;
  float *src_x1, *src_x2, *src_x3, *src_azimuth, *src_dip;
  float *rec_x1, *rec_x2, *rec_x3, *rec_azimuth, *rec_dip;
  float x1min, x1max, x2min, x2max, x3min, x3max;
  int nsrc_total, nrec_total;
  int *shot_idx;
} acq_t;

typedef void (*op_t)(int, csem_z *, csem_z *);

/* fdfd.c:30 / fdfd.c:65 */
void fdfd_init(emf_t *emf);
void fdfd_free(emf_t *emf);
/* fdfd.c:86, fdfd.c:287, fdfd.c:513 */
void fdfd_apply(int n, csem_z *x, csem_z *y);
void lusgs_apply(int n, csem_z *x, csem_z *y);
void aphi_apply(int n, csem_z *x, csem_z *y);
/* gmres_init_free.c:29, :45, :58 */
void gmres_init(int n, int m, op_t Aop);
void gmres_free(void);
void gmres_apply(int n, csem_z *x, csem_z *y);
/* cdotprod.c:13 */
csem_z cdotprod(int n, csem_z *a, csem_z *b);
/* solver.c:16, :93, :181, :403 */
void bicgstab(int n, csem_z *x, csem_z *b, op_t Aop, int niter, double tol, int verb);
void fbicgstab(int n, csem_z *x, csem_z *b, op_t Aop, op_t invMop, int niter, double tol, int verb);
void gmres(int n, csem_z *x, csem_z *b, op_t Aop, int niter, double tol, int m, int verb);
void fgmres(int n, csem_z *x, csem_z *b, op_t Aop, op_t invMop, int niter, double tol, int m, int verb);
/* inject_extract.c:24, :123 */
void inject_source(acq_t *acq, emf_t *emf, csem_z *b);
void extract_emf(acq_t *acq, emf_t *emf, csem_z *x, int ifreq);

/* Layout probe (no counterpart in the reference): out[0..7] = sizeof(emf_t),
 * sizeof(acq_t), offsets of emf_t.sigma11, .I_omega_mu0, .dcal_fd, .param_extended,
 * acq_t.rec_x1, .shot_idx - compared against the reference's emf.h/acq.h in tests. */
void csem_refabi_layout(long *out);

#ifdef __cplusplus
}
#endif
#endif
