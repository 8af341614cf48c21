// Plain complex128 Krylov solvers, device-resident (solver.c, gmres_init_free.c).
#pragma once
#include <vector>
#include "engine_model.h"

namespace csem {

class Solver64 {
 public:
  Solver64(Model* m, cudaStream_t st);
  Model* m;
  cudaStream_t st;
  Ops<F64> ops;
  long n;
  int nblk;
  DevBuf scal, ks, dots, partial, coef, hist, work, prework;
  int nwork = 0, pre_mp = 0;
  // dot products in the reference's sequential order (bit-identical to cdotprod.c)
  // instead of the parallel tree; the context option "dot_order"
  bool seq_dots = false;
  void set_iom(double re, double im);
  double2* W(int i);
  void ensure_work(int count);
  void A(const double2* x, double2* y);
  void M(int precond, int mp, const double2* x, double2* y);
  double2 dot(const double2* a, const double2* b);
  void dot_async(const double2* a, const double2* b, int slot_out);
  // every solver returns iterations (BiCGStab) or restart cycles (GMRES) and fills
  // hist with the relative residuals it computed, status with a SysStatus
  int fbicgstab(int precond, int mp, double2* x, const double2* b, int niter, double tol, std::vector<double>& hist,
                int& status, bool flexible);
  int gmres(int precond, int mp, double2* x, const double2* b, int ncycle, double tol, int mrestart,
            std::vector<double>& hist, int& status);
  void gmres_pre(int mp, const double2* b, double2* x);
  double2 iom_h;
};

}  // namespace csem
