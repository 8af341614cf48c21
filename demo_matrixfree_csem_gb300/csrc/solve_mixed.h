// Batched mixed-precision solver: complex64 inner flexible BiCGStab (LU-SGS or A-phi
// preconditioned) inside a complex128 defect-correction loop, many systems at once.
#pragma once
#include <vector>
#include "engine_model.h"

namespace csem {

struct MixedOptions {
  int niter = 1000;         // iteration budget of one inner solve (the reference's niter)
  int max_inner_total = 3000;
  int max_outer = 30;
  int preco = 1;            // 1 LU-SGS, 3 A-phi
  double inner_tol = 0.1;   // relative reduction asked of one inner solve
  int check_every = 4;      // inner iterations between host status reads
  bool autotune = false;    // time the LU-SGS sweep variants on the batch, keep the fastest
};

struct MixedResult {
  int status = 0;           // SysStatus
  int inner_iters = 0;      // complex64 iterations, all cycles
  int outer = 0;            // defect-correction cycles (complex128 residuals)
  double relres = 0;        // final ||b - A x|| / ||b|| in complex128
};

class MixedBatch {
 public:
  MixedBatch(Model* m, int nsys, cudaStream_t st);
  Model* m;
  int nsys;
  cudaStream_t st;
  long n;
  int nblk;
  Ops<F64> o64;
  Ops<F32> o32;
  DevBuf x64, b64, r64, w64, vec32, ks, sc64, sc32, dots, partial, list, rn, srcbuf, chbuf, recbuf, outbuf;
  float2* V(int i) { return vec32.as<float2>() + (size_t)i * nsys * n; }
  // b64 := injected sources (src [nsys][3], iom [nsys] on the host)
  void inject(const float* src, const double* iom, int nch, const int* ch);
  // solve all systems; tol[s] is each system's relative tolerance
  void solve(const double* iom, const double* tol, const MixedOptions& o, std::vector<MixedResult>& res);
  // out [nsys][nch][nrec] complex128 from x64
  void extract(int nch, const int* ch, int nrec, const float* rec, double* out_host);
  double inner_seconds = 0, outer_seconds = 0;
  int tuned_vw = 0;  // sweep width chosen by autotune_lusgs (0: not tuned)
  long inner_launch_iters = 0;  // sum over launched iterations of active systems
 private:
  void inner_iteration(int nact, const int* dlist, int preco, int maxiter);
  void start_inner(const std::vector<int>& g, const std::vector<double>& tol_inner);
  int autotune_lusgs(int nact, const int* dlist);  // returns the chosen points per thread
  void outer_update(const std::vector<int>& g, std::vector<double>& rnorm, bool first);
};

}  // namespace csem
