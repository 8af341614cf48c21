// Per-system Krylov state kept on the device, so an iteration needs no host round trip.
#pragma once
#include <cuda_runtime.h>
#include "csem_cuda.cuh"

namespace csem {

enum SysStatus {
  ST_RUNNING = 0,
  ST_CONVERGED = 1,   // relative residual below tolerance
  ST_MAXITER = 2,     // iteration limit reached
  ST_BREAKDOWN = 3,   // a Krylov denominator vanished (rho, omega, <v,r0> or <t,t> = 0)
  ST_NONFINITE = 4,   // a residual norm became NaN or Inf
  ST_ZERO_RHS = 5,    // ||b - A x0|| = 0: nothing to solve (solver.c:116-125)
};

struct KrylovScalars {
  double2 rho_old, alpha, omega, beta;
  double rs0, relres, tol;
  int status, iter;
};

enum VecOp { VEC_INIT = 0, VEC_S = 1, VEC_XR = 2, VEC_P = 3, VEC_XR_PLAIN = 4, VEC_SUB = 5 };

template <class P>
void launch_vec(int op, long n, int nslot, const int* sys_list, const KrylovScalars* ks, typename P::C* a,
                typename P::C* b, typename P::C* c, typename P::C* d, typename P::C* e, cudaStream_t st);
template <class P>  // x += alpha pp + omega ss; r = s - omega t (ss apart from r); r.r, r.r0
void launch_xr_dot2(long n, int nslot, const int* sys_list, const KrylovScalars* ks, typename P::C* x,
                    const typename P::C* pp, const typename P::C* ss, typename P::C* r, const typename P::C* s,
                    const typename P::C* t, const typename P::C* r0, double2* partial, int nblk, double2* out_rr,
                    double2* out_rr0, cudaStream_t st);
template <class P>
void launch_axpy(long n, int nslot, const int* sys_list, const double2* coef, int coef_stride, int neg,
                 const typename P::C* x, typename P::C* y, cudaStream_t st);
template <class P>
void launch_cdivv(long n, int nslot, const int* sys_list, const double2* d, int dstride, int real_only,
                  const typename P::C* x, typename P::C* y, cudaStream_t st);

// scalar steps of (F)BiCGStab (solver.c:113-126,145-146,151,157-165), one thread per slot
void launch_sc_init(int nslot, const int* sys_list, KrylovScalars* ks, const double2* d_rr0, const double2* d_rr,
                    double* hist, int hist_cap, cudaStream_t st);
void launch_sc_alpha(int nslot, const int* sys_list, KrylovScalars* ks, const double2* d_vr0, cudaStream_t st);
void launch_sc_omega(int nslot, const int* sys_list, KrylovScalars* ks, const double2* d_st, const double2* d_tt,
                     cudaStream_t st);
void launch_sc_rs_beta(int nslot, const int* sys_list, KrylovScalars* ks, const double2* d_rr, const double2* d_rr0,
                       double* hist, int hist_cap, int maxiter, cudaStream_t st);

}  // namespace csem
