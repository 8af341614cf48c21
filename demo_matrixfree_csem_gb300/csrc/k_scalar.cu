// Scalar steps of BiCGStab / flexible BiCGStab, evaluated on the device in the
// reference's order (solver.c:113-126,145-146,151,157-168) so the FP64 path keeps its
// rounding. Each thread owns one system slot.
#include "solver_state.h"

namespace csem {

__device__ __forceinline__ bool finite2(double2 v) { return isfinite(v.x) && isfinite(v.y); }

__global__ void k_sc_init(int nslot, const int* sys_list, KrylovScalars* ks, const double2* d_rr0,
                          const double2* d_rr, double* hist, int hist_cap)
{
  const int slot = blockIdx.x * blockDim.x + threadIdx.x;
  if (slot >= nslot) return;
  const int sys = sys_list ? sys_list[slot] : slot;
  KrylovScalars s = ks[sys];
  s.rho_old = d_rr0[slot];
  double rs = d_rr[slot].x;
  s.rs0 = rs;
  s.iter = 0;
  if (rs == 0.) {
    s.status = ST_ZERO_RHS;
    s.relres = 0.;
  } else {
    s.relres = __dsqrt_rn(__ddiv_rn(rs, s.rs0));
    s.status = isfinite(rs) ? ST_RUNNING : ST_NONFINITE;
  }
  if (hist && hist_cap > 0) hist[(size_t)sys * hist_cap] = s.relres;
  ks[sys] = s;
}

__global__ void k_sc_alpha(int nslot, const int* sys_list, KrylovScalars* ks, const double2* d_vr0)
{
  const int slot = blockIdx.x * blockDim.x + threadIdx.x;
  if (slot >= nslot) return;
  const int sys = sys_list ? sys_list[slot] : slot;
  KrylovScalars s = ks[sys];
  if (s.status != ST_RUNNING) return;
  double2 d = d_vr0[slot];
  if (d.x == 0. && d.y == 0.) { s.status = ST_BREAKDOWN; ks[sys] = s; return; }
  s.alpha = cdiv<F64>(s.rho_old, d);
  ks[sys] = s;
}

__global__ void k_sc_omega(int nslot, const int* sys_list, KrylovScalars* ks, const double2* d_st,
                           const double2* d_tt)
{
  const int slot = blockIdx.x * blockDim.x + threadIdx.x;
  if (slot >= nslot) return;
  const int sys = sys_list ? sys_list[slot] : slot;
  KrylovScalars s = ks[sys];
  if (s.status != ST_RUNNING) return;
  double tt = d_tt[slot].x;
  if (tt == 0.) { s.status = ST_BREAKDOWN; ks[sys] = s; return; }
  s.omega = cdivr<F64>(d_st[slot], tt);
  ks[sys] = s;
}

__global__ void k_sc_rs_beta(int nslot, const int* sys_list, KrylovScalars* ks, const double2* d_rr,
                             const double2* d_rr0, double* hist, int hist_cap, int maxiter)
{
  const int slot = blockIdx.x * blockDim.x + threadIdx.x;
  if (slot >= nslot) return;
  const int sys = sys_list ? sys_list[slot] : slot;
  KrylovScalars s = ks[sys];
  if (s.status != ST_RUNNING) return;
  double rs = d_rr[slot].x;
  s.relres = __dsqrt_rn(__ddiv_rn(rs, s.rs0));
  if (hist && s.iter + 1 < hist_cap) hist[(size_t)sys * hist_cap + s.iter + 1] = s.relres;
  if (!isfinite(s.relres)) {
    s.status = ST_NONFINITE;
  } else if (s.relres < s.tol) {
    s.status = ST_CONVERGED;
  } else {
    double2 rho_new = d_rr0[slot];
    if ((s.rho_old.x == 0. && s.rho_old.y == 0.) || (s.omega.x == 0. && s.omega.y == 0.)) {
      s.status = ST_BREAKDOWN;
    } else {
      s.beta = cdiv<F64>(cmul<F64>(cdiv<F64>(rho_new, s.rho_old), s.alpha), s.omega);
      s.rho_old = rho_new;
      if (!finite2(s.beta)) s.status = ST_NONFINITE;
    }
  }
  s.iter += 1;
  if (s.status == ST_RUNNING && s.iter >= maxiter) s.status = ST_MAXITER;
  ks[sys] = s;
}

static inline dim3 nb32(int n) { return dim3((n + 31) / 32); }

void launch_sc_init(int nslot, const int* sys_list, KrylovScalars* ks, const double2* d_rr0, const double2* d_rr,
                    double* hist, int hist_cap, cudaStream_t st)
{
  count_launch(), k_sc_init<<<nb32(nslot), 32, 0, st>>>(nslot, sys_list, ks, d_rr0, d_rr, hist, hist_cap);
}
void launch_sc_alpha(int nslot, const int* sys_list, KrylovScalars* ks, const double2* d_vr0, cudaStream_t st)
{
  count_launch(), k_sc_alpha<<<nb32(nslot), 32, 0, st>>>(nslot, sys_list, ks, d_vr0);
}
void launch_sc_omega(int nslot, const int* sys_list, KrylovScalars* ks, const double2* d_st, const double2* d_tt,
                     cudaStream_t st)
{
  count_launch(), k_sc_omega<<<nb32(nslot), 32, 0, st>>>(nslot, sys_list, ks, d_st, d_tt);
}
void launch_sc_rs_beta(int nslot, const int* sys_list, KrylovScalars* ks, const double2* d_rr, const double2* d_rr0,
                       double* hist, int hist_cap, int maxiter, cudaStream_t st)
{
  count_launch(), k_sc_rs_beta<<<nb32(nslot), 32, 0, st>>>(nslot, sys_list, ks, d_rr, d_rr0, hist, hist_cap, maxiter);
}

}  // namespace csem
