// Batched mixed-precision solver: complex64 inner flexible BiCGStab (LU-SGS or A-phi
// preconditioned) inside a complex128 defect-correction loop, many systems at once.
#pragma once
#include <functional>
#include <map>
#include <tuple>
#include <vector>
#include "engine_model.h"

namespace csem {

struct MixedOptions {
  int niter = 1000;         // iteration budget of one inner solve (the reference's niter)
  int max_inner_total = 3000;
  int max_outer = 30;
  int preco = 1;            // 1 LU-SGS, 3 A-phi
  double inner_tol = 0.2;   // relative reduction asked of one inner solve
  int check_every = 4;      // inner iterations between host status reads
  bool autotune = false;    // time the LU-SGS sweep variants on the batch, keep the fastest
  int algopt = 1;           // inner solver: 1 flexible BiCGStab, 2 flexible GMRES(nrestart)
  bool graphs = true;       // replay the BiCGStab iterations between status reads as CUDA graphs
  int nrestart = 10;        // GMRES basis size
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
  ~MixedBatch();
  MixedBatch(const MixedBatch&) = delete;
  MixedBatch& operator=(const MixedBatch&) = delete;
  Model* m;
  int nsys;
  cudaStream_t st;
  long n;
  int nblk;
  Ops<F64> o64;
  Ops<F32> o32;
  DevBuf x64, b64, r64, w64, vec32, ks, sc64, sc32, dots, partial, list, rn, srcbuf, chbuf, recbuf, outbuf;
  DevBuf gm, gstate;  // GMRES basis (V, Z, w, d, r0) and per-system Hessenberg state
  // complex64 FBiCGStab vectors r, r0, p, pp, v, s, t, d (the correction), sh (preconditioned s)
  static constexpr int NVEC32 = 9;
  float2* V(int i) { return vec32.as<float2>() + (size_t)i * nsys * n; }
  // b64 := injected sources (src [nsys][3], iom [nsys] on the host)
  void inject(const float* src, const double* iom, int nch, const int* ch);
  // solve all systems; tol[s] is each system's relative tolerance
  void solve(const double* iom, const double* tol, const MixedOptions& o, std::vector<MixedResult>& res);
  // out [nsys][nch][nrec] complex128 from x64
  void extract(int nch, const int* ch, int nrec, const float* rec, double* out_host);
  double inner_seconds = 0, outer_seconds = 0;
  int tuned_vw = 0;  // shapes chosen by autotune_lusgs (0: not tuned): sweep width,
  int tuned_lines = 0, tuned_by = 0, tuned_ctas = 0;  // lines per CTA, stencil rows, stencil CTAs per SM
  int tuned_systems = 0;  // systems of one frequency per CTA
  int tuned_split = -1;   // 1: split sweeps chosen
  long inner_launch_iters = 0;  // sum over launched iterations of active systems
 private:
  void inner_iteration(int nact, const int* dlist, int preco, int maxiter);
  // check_every inner iterations: launched directly the first time a (systems, options)
  // combination occurs, as a captured CUDA graph from the second time on
  void inner_iterations(int nact, const MixedOptions& o);
  struct Graph {
    cudaGraphExec_t exec = nullptr;
    int launches = 0;   // kernels in it (they count as launches at every replay)
    int seen = 0;       // times the combination occurred
    bool failed = false;
  };
  // keyed by (systems, options..., preconditioner groups): the groups set the sweeps' grids
  std::map<std::tuple<int, int, int, int, int, int, int>, Graph> graphs_, gm_graphs_;
  // body() launched directly the first time g's combination occurs, as a captured CUDA
  // graph from the second time on (never while per-operator profiling records events)
  void run_captured(Graph& g, bool use_graphs, const std::function<void()>& body);
  void drop_gmres_graphs();  // before the GMRES buffers move
  void start_inner(const std::vector<int>& g, const std::vector<double>& tol_inner);
  // the active systems into list and, for grouped complex64 sweeps (o32.sweep_systems >
  // 1), their same-frequency groups into grp_
  void set_list(const std::vector<int>& l);
  std::vector<double> h_iom_;  // iom per system (re, im) of the current solve
  std::vector<int> grph_;
  DevBuf grpbuf;
  SweepGroups grp_;
  int autotune_lusgs(const std::vector<int>& running);  // LU-SGS and stencil shapes; returns the points per thread
  void outer_update(const std::vector<int>& g, std::vector<double>& rnorm, bool first, const float2* d = nullptr);
  void solve_gmres(const std::vector<double>& bn, const double* tol, const MixedOptions& o,
                   std::vector<MixedResult>& res, std::vector<double>& rnorm, std::vector<int> running);
  // one complex64 flexible GMRES(m) inner solve of A d = r/|r| for the systems g
  void gmres_inner(const std::vector<int>& g, const std::vector<double>& tol_inner, const MixedOptions& o,
                   std::vector<int>& iters);
};

}  // namespace csem
