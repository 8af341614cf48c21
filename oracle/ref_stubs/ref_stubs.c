/* Link stubs that let the unmodified reference C sources build as a CPU oracle
 * (test infrastructure only; nothing here is part of the GPU product).
 *  - MPI: one rank, MPI_Wtime from CLOCK_MONOTONIC (main.c:54-56,103,119,142).
 *  - FFTW: fftw_plan_dft_2d / fftw_execute / fftw_malloc / fftw_free /
 *    fftw_destroy_plan over the self-written DFT in oracle/fft2d.c.
 *  - MUMPS path: Acoo_* are reached only from the dead main3 (main.c:226-280) and
 *    need MUMPS, which is absent; they abort if ever called.
 */
#include <stdio.h>
#include <stdlib.h>
#include <time.h>
#include <complex.h>
#include "mpi.h"
#include "fftw3.h"
#include "../fft2d.h"

int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return 0; }
int MPI_Comm_rank(MPI_Comm comm, int *rank) { (void)comm; *rank = 0; return 0; }
int MPI_Comm_size(MPI_Comm comm, int *size) { (void)comm; *size = 1; return 0; }
int MPI_Finalize(void) { return 0; }
double MPI_Wtime(void)
{
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

struct csem_fft_plan_s {
  int n0, n1, sign;
  fftw_complex *in, *out;
};

void *fftw_malloc(size_t n) { return malloc(n); }
void fftw_free(void *p) { free(p); }

fftw_plan fftw_plan_dft_2d(int n0, int n1, fftw_complex *in, fftw_complex *out,
                           int sign, unsigned flags)
{
  (void)flags;
  fftw_plan p = (fftw_plan)malloc(sizeof(*p));
  p->n0 = n0;
  p->n1 = n1;
  p->sign = sign;
  p->in = in;
  p->out = out;
  return p;
}

void fftw_execute(const fftw_plan p)
{
  if (p->in != p->out) {
    for (long i = 0; i < (long)p->n0 * p->n1; i++) p->out[i] = p->in[i];
  }
  csem_fft2d(p->n0, p->n1, (double *)p->out, p->sign);
}

void fftw_destroy_plan(fftw_plan p) { free(p); }

struct emf_s;
void Acoo_init(void *emf, int ifreq)
{
  (void)emf; (void)ifreq;
  fprintf(stderr, "Acoo_init: MUMPS direct solver is not available in the oracle build\n");
  abort();
}
void Acoo_free(void) {}
void Acoo_solve(void *emf)
{
  (void)emf;
  fprintf(stderr, "Acoo_solve: MUMPS direct solver is not available in the oracle build\n");
  abort();
}
