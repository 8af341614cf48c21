// Batched mixed-precision solve.
//
// For every system (frequency x source) the solution x and the true residual
// r = b - A x are kept in complex128. Each defect-correction cycle scales r to unit
// norm, solves A d = r/|r| approximately with a complex64 flexible BiCGStab
// (preconditioner LU-SGS or A-phi in complex64, dot products with FP64-class
// accumulation), then updates x += |r| d and recomputes r with the complex128 operator
// (complex128 airwave included). A system is converged when |b - A x| / |b| < tol,
// the reference's relative-residual criterion (solver.c:157-159) evaluated on the true
// residual instead of the recursive one.
//
// All systems share one model and advance together: every kernel takes the list of
// systems still iterating, so a converged system costs nothing once the host has seen
// its status (read every `check_every` inner iterations).
#include <algorithm>
#include <complex>
#include <cmath>
#include <cstring>
#include <functional>
#include "solve_mixed.h"
#include "../../include/csem_gpu.h"

namespace csem {

// (r and r0 may be the same vector: the GMRES start writes r0 through both)
__global__ void k_start_inner(long n, const int* __restrict__ list, const double* __restrict__ rn,
                              const double2* __restrict__ r64, float2* r, float2* r0, float2* __restrict__ p,
                              float2* __restrict__ d)
{
  const int sys = list[blockIdx.y];
  const long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const size_t o = (size_t)sys * n + q;
  const double s = 1.0 / rn[sys];
  const double2 v = r64[o];
  const float2 f = make_float2((float)(v.x * s), (float)(v.y * s));
  r[o] = f;
  r0[o] = f;
  p[o] = f;
  d[o] = make_float2(0.f, 0.f);
}

__global__ void k_outer_accum(long n, const int* __restrict__ list, const double* __restrict__ rn,
                              double2* __restrict__ x, const float2* __restrict__ d)
{
  const int sys = list[blockIdx.y];
  const long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const size_t o = (size_t)sys * n + q;
  const double s = rn[sys];
  const float2 dv = d[o];
  double2 xv = x[o];
  xv.x = fma(s, (double)dv.x, xv.x);
  xv.y = fma(s, (double)dv.y, xv.y);
  x[o] = xv;
}

MixedBatch::MixedBatch(Model* m_, int nsys_, cudaStream_t st_)
    : m(m_), nsys(nsys_), st(st_), n(m_->lE), nblk(dot_blocks(m_->lE)), o64(m_, nsys_, st_), o32(m_, nsys_, st_)
{
  const size_t N = (size_t)nsys * n;
  x64.alloc(sizeof(double2) * N);
  b64.alloc(sizeof(double2) * N);
  r64.alloc(sizeof(double2) * N);
  w64.alloc(sizeof(double2) * N);
  vec32.alloc(sizeof(float2) * N * NVEC32);
  ks.alloc(sizeof(KrylovScalars) * nsys);
  sc64.alloc(sizeof(SysScal<F64>) * nsys);
  sc32.alloc(sizeof(SysScal<F32>) * nsys);
  dots.alloc(sizeof(double2) * 8 * nsys);
  partial.alloc(sizeof(double2) * (size_t)nblk * nsys * 2);
  list.alloc(sizeof(int) * nsys);
  rn.alloc(sizeof(double) * nsys);
}

void MixedBatch::drop_gmres_graphs()
{
  for (auto& kv : gm_graphs_)
    if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
  gm_graphs_.clear();
}

MixedBatch::~MixedBatch()
{
  for (auto* m : {&graphs_, &gm_graphs_})
    for (auto& kv : *m)
      if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
}

// The iterations between two status reads are the same launch sequence every time for a
// given number of running systems (their indices live in the device list the kernels
// read), so from the second occurrence on they are captured once and replayed as a CUDA
// graph. The first occurrence runs directly, which also creates everything created on
// first use (FFT plans, A-phi work arrays) before any capture. Per-operator profiling
// records events per application, so it keeps the direct launches.
void MixedBatch::run_captured(Graph& g, bool use_graphs, const std::function<void()>& body)
{
  if (!use_graphs || prof_on() || g.failed || g.seen++ == 0) {
    body();
    return;
  }
  if (!g.exec) {
    cudaGraph_t graph = nullptr;
    const long long l0 = csem_launch_count();
    CSEM_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    try {
      body();
    } catch (...) {
      cudaStreamEndCapture(st, &graph);
      if (graph) cudaGraphDestroy(graph);
      throw;
    }
    const cudaError_t e = cudaStreamEndCapture(st, &graph);
    g.launches = (int)(csem_launch_count() - l0);
    count_launch(-g.launches);  // captured, not launched yet
    if (e != cudaSuccess || !graph || cudaGraphInstantiate(&g.exec, graph, 0) != cudaSuccess) {
      if (graph) cudaGraphDestroy(graph);
      (void)cudaGetLastError();
      g.exec = nullptr;
      g.failed = true;
      body();
      return;
    }
    cudaGraphDestroy(graph);
  }
  CSEM_CUDA_TRY(cudaGraphLaunch(g.exec, st));
  count_launch(g.launches);
}

void MixedBatch::inner_iterations(int nact, const MixedOptions& o)
{
  const int* dl = list.as<int>();
  run_captured(graphs_[std::make_tuple(nact, o.preco, o.check_every, o.niter, grp_.n * 32 + grp_.ns, grp_.nA, grp_.ngA)],
               o.graphs, [&]() {
    for (int q = 0; q < o.check_every; q++) inner_iteration(nact, dl, o.preco, o.niter);
  });
}

void MixedBatch::inject(const float* src, const double* iom, int nch, const int* ch)
{
  srcbuf.alloc(sizeof(float) * 3 * nsys + sizeof(double2) * nsys + 64);
  chbuf.alloc(sizeof(int) * (nch > 0 ? nch : 1));
  char* d = srcbuf.as<char>();
  const size_t off = ((sizeof(float) * 3 * nsys + 15) / 16) * 16;
  CSEM_CUDA_TRY(cudaMemcpyAsync(d, src, sizeof(float) * 3 * nsys, cudaMemcpyHostToDevice, st));
  CSEM_CUDA_TRY(cudaMemcpyAsync(d + off, iom, sizeof(double2) * nsys, cudaMemcpyHostToDevice, st));
  CSEM_CUDA_TRY(cudaMemcpyAsync(chbuf.p, ch, sizeof(int) * nch, cudaMemcpyHostToDevice, st));
  CSEM_CUDA_TRY(cudaMemsetAsync(b64.p, 0, sizeof(double2) * (size_t)nsys * n, st));
  launch_inject(m->acq, nsys, (const float*)d, (const double2*)(d + off), chbuf.as<int>(), nch, b64.as<double2>(), st);
  CSEM_CUDA_TRY(cudaGetLastError());
}

void MixedBatch::inner_iteration(int nact, const int* dl, int preco, int maxiter)
{
  float2 *r = V(0), *r0 = V(1), *p = V(2), *pp = V(3), *v = V(4), *s = V(5), *t = V(6), *d = V(7), *sh = V(8);
  KrylovScalars* K = ks.as<KrylovScalars>();
  double2* D = dots.as<double2>();
  double2* part = partial.as<double2>();
  const SysScal<F32>* sc = sc32.as<SysScal<F32>>();
  // pp and sh are written only by the preconditioner, whose sweeps never write the
  // boundary entries: zeroed once per solve, those stay zero, so the LU-SGS output is
  // not cleared before each application
  auto M = [&](const float2* in, float2* out) {
    if (preco == PRE_APHI) o32.apply_aphi(in, out, nact, dl, sc);
    else o32.apply_lusgs(in, out, nact, dl, sc, true, &grp_);
  };
  DotEpi<F32> ep;  // v.r0 and s.t, t.t formed by the operator's stencil where it can
  ep.partial = part;
  ep.cap = nblk;
  ep.n = n;
  ep.nblk = nblk;
  M(p, pp);
  ep.kind = 1;
  ep.e = r0;
  ep.out1 = D + 0 * nsys;
  if (!o32.apply_A(pp, v, nact, dl, sc, &ep))  // v = A pp, <v, r0>
    launch_dot<F32>(v, r0, n, n, nact, dl, part, nblk, D + 0 * nsys, st);
  launch_sc_alpha(nact, dl, K, D + 0 * nsys, st);
  launch_vec<F32>(VEC_S, n, nact, dl, K, r, v, s, nullptr, nullptr, st);
  M(s, sh);
  ep.kind = 2;
  ep.e = s;
  ep.out1 = D + 1 * nsys;
  ep.out2 = D + 2 * nsys;
  if (!o32.apply_A(sh, t, nact, dl, sc, &ep))  // t = A sh, <s, t> and <t, t>
    launch_dot2<F32>(s, t, t, t, n, n, nact, dl, part, nblk, D + 1 * nsys, D + 2 * nsys, st);
  launch_sc_omega(nact, dl, K, D + 1 * nsys, D + 2 * nsys, st);
  launch_xr_dot2<F32>(n, nact, dl, K, d, pp, sh, r, s, t, r0, part, nblk, D + 3 * nsys, D + 4 * nsys, st);
  launch_sc_rs_beta(nact, dl, K, D + 3 * nsys, D + 4 * nsys, nullptr, 0, maxiter, st);
  launch_vec<F32>(VEC_P, n, nact, dl, K, r, p, v, nullptr, nullptr, st);
}

void MixedBatch::set_list(const std::vector<int>& l)
{
  CSEM_CUDA_TRY(cudaMemcpyAsync(list.p, l.data(), sizeof(int) * l.size(), cudaMemcpyHostToDevice, st));
  grp_ = SweepGroups();
  const int ns = o32.group_size();
  if (ns <= 1 || l.empty() || h_iom_.size() < 2 * (size_t)nsys) return;
  std::vector<double> iom_slot(2 * l.size());
  for (size_t q = 0; q < l.size(); q++) {
    iom_slot[2 * q] = h_iom_[2 * (size_t)l[q]];
    iom_slot[2 * q + 1] = h_iom_[2 * (size_t)l[q] + 1];
  }
  int nA = 0, ngA = 0;
  const int ng = ns == SPLIT_GROUP && o32.split_overlap
                     ? build_sweep_groups_halves((int)l.size(), iom_slot.data(), ns, 4, grph_, &nA, &ngA)
                     : build_sweep_groups((int)l.size(), iom_slot.data(), ns, grph_);
  // at most nsys groups of SPLIT_GROUP: allocated once, so the address captured graphs use stays
  if (!grpbuf.p) grpbuf.alloc(sizeof(int) * SPLIT_GROUP * (size_t)nsys);
  CSEM_CUDA_TRY(cudaMemcpyAsync(grpbuf.p, grph_.data(), sizeof(int) * grph_.size(), cudaMemcpyHostToDevice, st));
  grp_.dev = grpbuf.as<int>();
  grp_.n = ng;
  grp_.ns = ns;
  grp_.nA = nA;
  grp_.ngA = ngA;
}

void MixedBatch::start_inner(const std::vector<int>& g, const std::vector<double>& tol_inner)
{
  if (g.empty()) return;
  // per-system tolerance and a fresh state word
  std::vector<KrylovScalars> kh(nsys);
  CSEM_CUDA_TRY(cudaMemcpyAsync(kh.data(), ks.p, sizeof(KrylovScalars) * nsys, cudaMemcpyDeviceToHost, st));
  CSEM_CUDA_TRY(cudaStreamSynchronize(st));
  for (size_t q = 0; q < g.size(); q++) {
    KrylovScalars& k = kh[g[q]];
    memset(&k, 0, sizeof(k));
    k.tol = tol_inner[q];
    k.status = ST_RUNNING;
  }
  CSEM_CUDA_TRY(cudaMemcpyAsync(ks.p, kh.data(), sizeof(KrylovScalars) * nsys, cudaMemcpyHostToDevice, st));
  CSEM_CUDA_TRY(cudaMemcpyAsync(list.p, g.data(), sizeof(int) * g.size(), cudaMemcpyHostToDevice, st));
  const int ng = (int)g.size();
  const int* dl = list.as<int>();
  dim3 grd((unsigned)((n + 255) / 256), ng);
  count_launch(), k_start_inner<<<grd, 256, 0, st>>>(n, dl, rn.as<double>(), r64.as<double2>(), V(0), V(1), V(2), V(7));
  double2* D = dots.as<double2>();
  launch_dot2<F32>(V(0), V(1), V(0), V(0), n, n, ng, dl, partial.as<double2>(), nblk, D + 5 * nsys, D + 6 * nsys,
                   st);
  launch_sc_init(ng, dl, ks.as<KrylovScalars>(), D + 5 * nsys, D + 6 * nsys, nullptr, 0, st);
  CSEM_CUDA_TRY(cudaGetLastError());
}

void MixedBatch::outer_update(const std::vector<int>& g, std::vector<double>& rnorm, bool first, const float2* d)
{
  const int ng = (int)g.size();
  CSEM_CUDA_TRY(cudaMemcpyAsync(list.p, g.data(), sizeof(int) * ng, cudaMemcpyHostToDevice, st));
  const int* dl = list.as<int>();
  dim3 grd((unsigned)((n + 255) / 256), ng);
  if (!first) {
    count_launch(), k_outer_accum<<<grd, 256, 0, st>>>(n, dl, rn.as<double>(), x64.as<double2>(), d ? d : V(7));
    o64.apply_A(x64.as<double2>(), w64.as<double2>(), ng, dl, sc64.as<SysScal<F64>>());
    launch_vec<F64>(VEC_SUB, n, ng, dl, nullptr, b64.as<double2>(), w64.as<double2>(), r64.as<double2>(), nullptr,
                    nullptr, st);
  }
  double2* D = dots.as<double2>();
  launch_dot<F64>(r64.as<double2>(), r64.as<double2>(), n, n, ng, dl, partial.as<double2>(), nblk, D + 7 * nsys, st);
  std::vector<double2> h(ng);
  CSEM_CUDA_TRY(cudaMemcpyAsync(h.data(), D + 7 * nsys, sizeof(double2) * ng, cudaMemcpyDeviceToHost, st));
  CSEM_CUDA_TRY(cudaStreamSynchronize(st));
  for (int q = 0; q < ng; q++) rnorm[g[q]] = std::sqrt(h[q].x);
  CSEM_CUDA_TRY(cudaMemcpyAsync(rn.p, rnorm.data(), sizeof(double) * nsys, cudaMemcpyHostToDevice, st));
}

// Autotuner of the complex64 kernel shapes, on the batch's current vectors: each
// candidate is applied once untimed and once timed with CUDA events on the solver's
// stream, and the fastest is kept for the rest of this batch.
//  - LU-SGS: the split sweeps (a coalesced pass and a light row pipeline) at 1, 2, 4
//    points per thread and step; the one-pass pipelined sweeps at points per thread
//    (1, 2, 4) x lines per CTA (1, 2, 4), or with 2 (1 or 2 points) or 4 (1 point)
//    systems of one frequency per CTA;
//  - stencil: output rows per CTA (4, 8, 16) x CTAs per SM of the plane chunks, i.e. the
//    z-block depth (2, 4, 8).
// The scratch vectors it writes are overwritten before use by the solve. The stencil
// shape does not change results; the LU-SGS shape can change the last bits of complex64.
int MixedBatch::autotune_lusgs(const std::vector<int>& running)
{
  const int nact = (int)running.size();
  const int* dlist = list.as<int>();
  const SysScal<F32>* sc = sc32.as<SysScal<F32>>();
  cudaEvent_t e0, e1;
  CSEM_CUDA_TRY(cudaEventCreate(&e0));
  CSEM_CUDA_TRY(cudaEventCreate(&e1));
  auto time = [&](const std::function<void()>& f) {
    f();
    CSEM_CUDA_TRY(cudaEventRecord(e0, st));
    f();
    CSEM_CUDA_TRY(cudaEventRecord(e1, st));
    CSEM_CUDA_TRY(cudaEventSynchronize(e1));
    float ms = 0.f;
    CSEM_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
    return ms;
  };
  const bool saved = o32.pipelined_sweeps, saved_tiled = o32.tiled_sweeps;
  o32.pipelined_sweeps = true;
  o32.tiled_sweeps = false;
  float best_ms = 1e30f;
  int best_vw = 2, best_lines = 1, best_ns = 1;
  bool best_split = true;
  for (int split : {1, 0})
    for (int ns : {1, 2, 4}) {
      if (split && ns > 1) continue;
      o32.split_sweeps = split != 0;
      o32.sweep_systems = ns;
      set_list(running);  // the groups for this candidate (the split pass's, or ns per CTA)
      for (int vw : {1, 2, 4})
        for (int lines : {1, 2, 4}) {
          if ((split && lines > 1) || (ns > 1 && lines > 1) || (ns == 2 && vw == 4) || (ns == 4 && vw > 1)) continue;
          o32.sweep_vw = vw;
          o32.sweep_lines = lines;
          const float ms = time([&]() { o32.apply_lusgs(V(0), V(3), nact, dlist, sc, false, &grp_); });
          if (ms < best_ms) {
            best_ms = ms;
            best_vw = vw;
            best_lines = lines;
            best_ns = ns;
            best_split = split != 0;
          }
        }
    }
  o32.split_sweeps = best_split;
  o32.sweep_systems = best_ns;
  set_list(running);
  o32.pipelined_sweeps = saved;
  o32.tiled_sweeps = saved_tiled;
  o32.sweep_vw = best_vw;
  o32.sweep_lines = best_lines;
  best_ms = 1e30f;
  int best_by = 8, best_ctas = 4;
  for (int by : {4, 8, 16})
    for (int ctas : {2, 4, 8}) {
      o32.stencil_by = by;
      o32.stencil_ctas = ctas;
      const float ms = time([&]() { o32.apply_A(V(0), V(4), nact, dlist, sc); });
      if (ms < best_ms) {
        best_ms = ms;
        best_by = by;
        best_ctas = ctas;
      }
    }
  o32.stencil_by = best_by;
  o32.stencil_ctas = best_ctas;
  tuned_lines = best_lines;
  tuned_systems = best_ns;
  tuned_split = best_split ? 1 : 0;
  tuned_by = best_by;
  tuned_ctas = best_ctas;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return best_vw;
}

void MixedBatch::solve(const double* iom, const double* tol, const MixedOptions& o, std::vector<MixedResult>& res)
{
  res.assign(nsys, MixedResult());
  std::vector<SysScal<F64>> s64(nsys);
  std::vector<SysScal<F32>> s32(nsys);
  for (int q = 0; q < nsys; q++) {
    s64[q] = sys_scal64(iom[2 * q], iom[2 * q + 1]);
    s32[q] = sys_scal32(s64[q]);
  }
  CSEM_CUDA_TRY(cudaMemcpyAsync(sc64.p, s64.data(), sizeof(SysScal<F64>) * nsys, cudaMemcpyHostToDevice, st));
  CSEM_CUDA_TRY(cudaMemcpyAsync(sc32.p, s32.data(), sizeof(SysScal<F32>) * nsys, cudaMemcpyHostToDevice, st));
  h_iom_.assign(iom, iom + 2 * (size_t)nsys);
  CSEM_CUDA_TRY(cudaMemsetAsync(x64.p, 0, sizeof(double2) * (size_t)nsys * n, st));
  CSEM_CUDA_TRY(cudaMemcpyAsync(r64.p, b64.p, sizeof(double2) * (size_t)nsys * n, cudaMemcpyDeviceToDevice, st));
  CSEM_CUDA_TRY(cudaMemsetAsync(ks.p, 0, sizeof(KrylovScalars) * nsys, st));
  CSEM_CUDA_TRY(cudaMemsetAsync(vec32.p, 0, vec32.bytes, st));  // zero boundaries (inner_iteration)
  std::vector<int> all(nsys);
  for (int q = 0; q < nsys; q++) all[q] = q;
  std::vector<double> rnorm(nsys, 0.0), bn(nsys, 0.0);
  outer_update(all, rnorm, true);
  bn = rnorm;
  std::vector<int> running;
  std::vector<double> ti;
  for (int q = 0; q < nsys; q++) {
    if (!(bn[q] > 0.0)) {
      res[q].status = bn[q] == 0.0 ? ST_ZERO_RHS : ST_NONFINITE;
      continue;
    }
    res[q].status = ST_RUNNING;
    res[q].relres = 1.0;
    running.push_back(q);
    ti.push_back(std::min(0.5, std::max(o.inner_tol, 0.5 * tol[q])));
  }
  if (o.algopt == 2) {
    solve_gmres(bn, tol, o, res, rnorm, running);
    CSEM_CUDA_TRY(cudaStreamSynchronize(st));
    return;
  }
  if (o.autotune && o.preco != PRE_APHI && !running.empty()) {
    tuned_vw = autotune_lusgs(running);
  }
  start_inner(running, ti);
  std::vector<KrylovScalars> kh(nsys);
  inner_launch_iters = 0;
  while (!running.empty()) {
    set_list(running);
    inner_iterations((int)running.size(), o);
    inner_launch_iters += (long)running.size() * o.check_every;
    CSEM_CUDA_TRY(cudaGetLastError());
    CSEM_CUDA_TRY(cudaMemcpyAsync(kh.data(), ks.p, sizeof(KrylovScalars) * nsys, cudaMemcpyDeviceToHost, st));
    CSEM_CUDA_TRY(cudaStreamSynchronize(st));
    std::vector<int> done, still;
    for (int s : running) (kh[s].status != ST_RUNNING ? done : still).push_back(s);
    if (done.empty()) continue;
    for (int s : done) res[s].inner_iters += kh[s].iter;
    outer_update(done, rnorm, false);
    std::vector<int> restart;
    std::vector<double> rti;
    for (int s : done) {
      res[s].outer += 1;
      const double rel = rnorm[s] / bn[s];
      res[s].relres = rel;
      if (rel < tol[s]) res[s].status = ST_CONVERGED;
      else if (!std::isfinite(rel)) res[s].status = ST_NONFINITE;
      else if (res[s].inner_iters >= o.max_inner_total || res[s].outer >= o.max_outer) res[s].status = ST_MAXITER;
      else {
        restart.push_back(s);
        rti.push_back(std::min(0.5, std::max(o.inner_tol, 0.5 * tol[s] / rel)));
      }
    }
    start_inner(restart, rti);
    running = still;
    running.insert(running.end(), restart.begin(), restart.end());
    std::sort(running.begin(), running.end());
  }
  CSEM_CUDA_TRY(cudaStreamSynchronize(st));
}

// ------------------------------------------------------------------ flexible GMRES inner
// The same defect correction with a complex64 flexible GMRES(m) as the inner solver, the
// structure of fgmres (solver.c:403-512): z_j = M v_j, w = A z_j, modified Gram-Schmidt
// against v_0..v_j, Givens rotations of the Hessenberg column, restart after m steps.
// Everything runs on the device over the systems of the cycle: the vectors, the
// preconditioner, the operator and the dot products batched, and each system's
// (m+1) x m Hessenberg algebra in complex128 by one thread per system (k_gm_*), reading
// the dot products where the reduction left them. A system whose estimated residual
// reaches the inner reduction stops stepping (its later steps are skipped by these
// kernels and its update uses only the steps it took); the host reads the systems' state
// once per cycle to choose the next cycle's systems. The m steps of a cycle are one
// fixed launch sequence for a given number of systems, replayed as a CUDA graph from the
// second time it occurs.
namespace {

struct GmState {
  double beta0;  // |r0| of the solve's first cycle: the residual estimates refer to it
  double tol;    // relative reduction asked of this inner solve
  int steps;     // Arnoldi steps taken in the current cycle
  int iters;     // steps taken in this inner solve
  int niter;     // step budget (the reference's niter)
  int stop;      // 1: no more steps in this cycle
  int done;      // 1: the reduction is reached (or the Krylov space is exhausted)
  int pad;
};

__device__ __forceinline__ double2 zmul(double2 a, double2 b)
{
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 zconj(double2 a) { return make_double2(a.x, -a.y); }
__device__ __forceinline__ double2 zadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 zsub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 zscl(double s, double2 a) { return make_double2(s * a.x, s * a.y); }
__device__ __forceinline__ double2 zdiv(double2 a, double2 b)  // Smith's quotient
{
  if (fabs(b.x) < fabs(b.y)) {
    const double r = b.x / b.y, den = b.x * r + b.y;
    return make_double2((a.x * r + a.y) / den, (a.y * r - a.x) / den);
  }
  const double r = b.y / b.x, den = b.y * r + b.x;
  return make_double2((a.y * r + a.x) / den, (a.y - a.x * r) / den);
}

// cycle start: beta = |r| from its dot product, g = (beta, 0, ..), the divisor of v_0
__global__ void k_gm_begin(int nact, const int* __restrict__ list, GmState* __restrict__ st,
                           const double2* __restrict__ drr, double2* __restrict__ g, double2* __restrict__ coef, int m,
                           int first)
{
  const int slot = blockIdx.x * blockDim.x + threadIdx.x;
  if (slot >= nact) return;
  const int sys = list[slot];
  GmState& S = st[sys];
  const double beta = sqrt(drr[slot].x);
  if (first) S.beta0 = beta > 0 ? beta : 1.0;
  double2* gs = g + (size_t)sys * (m + 1);
  gs[0] = make_double2(beta, 0.0);
  for (int i = 1; i <= m; i++) gs[i] = make_double2(0.0, 0.0);
  coef[slot] = make_double2(beta > 0 ? beta : 1.0, 0.0);
  S.steps = 0;
  S.stop = 0;
}

// step j: Hessenberg column j from the Gram-Schmidt dots (slot-indexed rows i = 0..j of
// dots, the norm in row m), earlier rotations, the new rotation, the residual estimate
// (as the host algebra of fgmres, solver.c:448-481) and the divisor of v_{j+1}
__global__ void k_gm_step(int nact, const int* __restrict__ list, GmState* __restrict__ st,
                          const double2* __restrict__ dots, int dstride, double2* __restrict__ H,
                          double2* __restrict__ cs, double* __restrict__ sn, double2* __restrict__ g,
                          double2* __restrict__ coef, int m, int j)
{
  const int slot = blockIdx.x * blockDim.x + threadIdx.x;
  if (slot >= nact) return;
  const int sys = list[slot];
  GmState& S = st[sys];
  const double nn = dots[(size_t)m * dstride + slot].x;
  const double hn = sqrt(nn);
  coef[slot] = make_double2(hn > 0 ? hn : 1.0, 0.0);
  if (S.stop) return;
  double2* col = H + ((size_t)sys * m + j) * (m + 1);
  double2* c = cs + (size_t)sys * m;
  double* s = sn + (size_t)sys * m;
  double2* gs = g + (size_t)sys * (m + 1);
  for (int i = 0; i <= j; i++) col[i] = dots[(size_t)i * dstride + slot];
  col[j + 1] = make_double2(hn, 0.0);
  for (int i = 0; i < j; i++) {  // earlier rotations
    const double2 t = zadd(zmul(zconj(c[i]), col[i]), zscl(s[i], col[i + 1]));
    col[i + 1] = zadd(zscl(-s[i], col[i]), zmul(c[i], col[i + 1]));
    col[i] = t;
  }
  const double tmp = sqrt((col[j].x * col[j].x + col[j].y * col[j].y) +
                          (col[j + 1].x * col[j + 1].x + col[j + 1].y * col[j + 1].y));
  if (tmp == 0.0) {
    S.stop = 1;
    return;
  }
  s[j] = col[j + 1].x / tmp;
  c[j] = make_double2(col[j].x / tmp, col[j].y / tmp);
  gs[j + 1] = zscl(-s[j], gs[j]);
  gs[j] = zmul(zconj(c[j]), gs[j]);
  col[j] = zadd(zmul(zconj(c[j]), col[j]), zscl(s[j], col[j + 1]));
  S.steps = j + 1;
  S.iters += 1;
  const double rel = hypot(gs[j + 1].x, gs[j + 1].y) / S.beta0;
  if (rel < S.tol || !(nn > 0.0)) {
    S.stop = 1;
    S.done = 1;
  } else if (S.iters >= S.niter) {
    S.stop = 1;
  }
}

// y from the triangular system of the steps each system took (solver.c:489-495);
// y[i][slot] = 0 past them
__global__ void k_gm_solve(int nact, const int* __restrict__ list, const GmState* __restrict__ st,
                           const double2* __restrict__ H, const double2* __restrict__ g, double2* __restrict__ y,
                           int ystride, int m)
{
  const int slot = blockIdx.x * blockDim.x + threadIdx.x;
  if (slot >= nact) return;
  const int sys = list[slot];
  const int mm = st[sys].steps;
  const double2* Hs = H + (size_t)sys * m * (m + 1);  // column k at Hs[k * (m + 1)]
  const double2* gs = g + (size_t)sys * (m + 1);
  double2 yv[64];
  for (int i = mm - 1; i >= 0; i--) {
    double2 acc = gs[i];
    for (int k2 = i + 1; k2 < mm; k2++) acc = zsub(acc, zmul(Hs[(size_t)k2 * (m + 1) + i], yv[k2]));
    yv[i] = zdiv(acc, Hs[(size_t)i * (m + 1) + i]);
  }
  for (int i = 0; i < m; i++) y[(size_t)i * ystride + slot] = i < mm ? yv[i] : make_double2(0.0, 0.0);
}

// d += sum_{i < steps} y_i z_i (solver.c:496-500), the systems' own step counts
__global__ void k_gm_update(long n, const int* __restrict__ list, const GmState* __restrict__ st,
                            const double2* __restrict__ y, int ystride, const float2* __restrict__ Z, size_t zstride,
                            float2* __restrict__ d)
{
  const int slot = blockIdx.y;
  const int sys = list[slot];
  const long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const size_t o = (size_t)sys * n + q;
  const int mm = st[sys].steps;
  float2 acc = d[o];
  for (int i = 0; i < mm; i++) {
    const double2 a2 = y[(size_t)i * ystride + slot];
    const float2 a = make_float2((float)a2.x, (float)a2.y);
    const float2 z = Z[(size_t)i * zstride + o];
    acc = make_float2(acc.x + (a.x * z.x - a.y * z.y), acc.y + (a.x * z.y + a.y * z.x));
  }
  d[o] = acc;
}

}  // namespace

void MixedBatch::gmres_inner(const std::vector<int>& g, const std::vector<double>& tol_inner, const MixedOptions& o,
                             std::vector<int>& iters)
{
  const int m = std::max(1, o.nrestart);
  const size_t N = (size_t)nsys * n;
  float2* base = gm.as<float2>();
  auto GV = [&](int i) { return base + (size_t)i * N; };
  auto GZ = [&](int i) { return base + (size_t)(m + 1 + i) * N; };
  float2* GW = base + (size_t)(2 * m + 1) * N;
  float2* GD = base + (size_t)(2 * m + 2) * N;
  float2* GR0 = base + (size_t)(2 * m + 3) * N;
  const SysScal<F32>* sc = sc32.as<SysScal<F32>>();
  // device state: GmState[nsys] | H [nsys][m][m+1] | cs [nsys][m] | g [nsys][m+1] |
  // dots [m+2][nsys] | y [m][nsys] | coef [nsys] (double2), then sn [nsys][m] (double)
  const size_t nst = ((sizeof(GmState) * nsys + 15) / 16) * 16;
  const size_t nz = (size_t)nsys * ((size_t)m * (m + 1) + m + (m + 1) + (m + 2) + m + 1);
  const size_t need = nst + sizeof(double2) * nz + sizeof(double) * (size_t)nsys * m;
  if (gstate.bytes < need) {
    drop_gmres_graphs();  // they hold the old buffer's addresses
    gstate.alloc(need);
  }
  char* gb = gstate.as<char>();
  GmState* st = reinterpret_cast<GmState*>(gb);
  double2* zb = reinterpret_cast<double2*>(gb + nst);
  double2* H = zb;
  double2* cs = H + (size_t)nsys * m * (m + 1);
  double2* gg = cs + (size_t)nsys * m;
  double2* dots = gg + (size_t)nsys * (m + 1);
  double2* ycoef = dots + (size_t)(m + 2) * nsys;
  double2* coef = ycoef + (size_t)m * nsys;
  double* sn = reinterpret_cast<double*>(coef + nsys);
  const int ns = (int)g.size();
  std::vector<GmState> sh(nsys);
  memset(sh.data(), 0, sizeof(GmState) * nsys);
  for (int q = 0; q < ns; q++) {
    sh[g[q]].tol = tol_inner[q];
    sh[g[q]].niter = o.niter;
  }
  CSEM_CUDA_TRY(cudaMemcpyAsync(st, sh.data(), sizeof(GmState) * nsys, cudaMemcpyHostToDevice, this->st));
  auto M = [&](const float2* in, float2* out, int na, const int* dl) {  // Z_j: only written here
    if (o.preco == PRE_APHI) o32.apply_aphi(in, out, na, dl, sc);
    else o32.apply_lusgs(in, out, na, dl, sc, true, &grp_);
  };
  // r0 = r64 / |r64|, d = 0 (k_start_inner writes r, r0, p, d: here r0 twice and d)
  {
    CSEM_CUDA_TRY(cudaMemcpyAsync(list.p, g.data(), sizeof(int) * g.size(), cudaMemcpyHostToDevice, this->st));
    dim3 grd((unsigned)((n + 255) / 256), (unsigned)g.size());
    count_launch(), k_start_inner<<<grd, 256, 0, this->st>>>(n, list.as<int>(), rn.as<double>(), r64.as<double2>(),
                                                             GR0, GR0, GW, GD);
  }
  const int* dl = list.as<int>();
  for (int cycle = 0;; cycle++) {
    std::vector<int> act;
    for (int q = 0; q < ns; q++)
      if (!sh[g[q]].done && sh[g[q]].iters < o.niter) act.push_back(g[q]);
    if (act.empty()) break;
    const int na = (int)act.size();
    const unsigned nb32 = (unsigned)((na + 31) / 32);
    set_list(act);
    // r = r0 - A d  (d = 0 on the first cycle), v_0 = r / |r|
    if (cycle == 0) {
      CSEM_CUDA_TRY(cudaMemcpyAsync(GW, GR0, sizeof(float2) * N, cudaMemcpyDeviceToDevice, this->st));
    } else {
      o32.apply_A(GD, GV(0), na, dl, sc);
      launch_vec<F32>(VEC_SUB, n, na, dl, nullptr, GR0, GV(0), GW, nullptr, nullptr, this->st);
    }
    launch_dot<F32>(GW, GW, n, n, na, dl, partial.as<double2>(), nblk, dots + (size_t)(m + 1) * nsys, this->st);
    count_launch(), k_gm_begin<<<nb32, 32, 0, this->st>>>(na, dl, st, dots + (size_t)(m + 1) * nsys, gg, coef, m,
                                                          cycle == 0);
    launch_cdivv<F32>(n, na, dl, coef, 1, 1, GW, GV(0), this->st);
    // the m Arnoldi steps and the update of d: one fixed launch sequence for na systems
    auto steps = [&]() {
      for (int j = 0; j < m; j++) {
        M(GV(j), GZ(j), na, dl);
        o32.apply_A(GZ(j), GW, na, dl, sc);
        for (int i = 0; i <= j; i++) {  // modified Gram-Schmidt
          launch_dot<F32>(GW, GV(i), n, n, na, dl, partial.as<double2>(), nblk, dots + (size_t)i * nsys, this->st);
          launch_axpy<F32>(n, na, dl, dots + (size_t)i * nsys, 1, 1, GV(i), GW, this->st);
        }
        launch_dot<F32>(GW, GW, n, n, na, dl, partial.as<double2>(), nblk, dots + (size_t)m * nsys, this->st);
        count_launch(), k_gm_step<<<nb32, 32, 0, this->st>>>(na, dl, st, dots, nsys, H, cs, sn, gg, coef, m, j);
        launch_cdivv<F32>(n, na, dl, coef, 1, 1, GW, GV(j + 1), this->st);
      }
      count_launch(), k_gm_solve<<<nb32, 32, 0, this->st>>>(na, dl, st, H, gg, ycoef, nsys, m);
      dim3 grd((unsigned)((n + 255) / 256), (unsigned)na);
      count_launch(), k_gm_update<<<grd, 256, 0, this->st>>>(n, dl, st, ycoef, nsys, GZ(0), N, GD);
    };
    run_captured(gm_graphs_[std::make_tuple(na, m, o.preco, 0, grp_.n * 32 + grp_.ns, grp_.nA, grp_.ngA)], o.graphs,
                 steps);
    CSEM_CUDA_TRY(cudaGetLastError());
    CSEM_CUDA_TRY(cudaMemcpyAsync(sh.data(), st, sizeof(GmState) * nsys, cudaMemcpyDeviceToHost, this->st));
    CSEM_CUDA_TRY(cudaStreamSynchronize(this->st));
  }
  iters.assign(ns, 0);
  for (int q = 0; q < ns; q++) iters[q] = sh[g[q]].iters;
}

void MixedBatch::solve_gmres(const std::vector<double>& bn, const double* tol, const MixedOptions& o,
                             std::vector<MixedResult>& res, std::vector<double>& rnorm, std::vector<int> running)
{
  const int m = std::max(1, o.nrestart);
  const size_t need = sizeof(float2) * (size_t)(2 * m + 4) * nsys * n;
  if (gm.bytes < need) {
    drop_gmres_graphs();  // they hold the old buffer's addresses
    gm.alloc(need);
  }
  // the Z_j are written only by the preconditioner, which leaves boundary entries as
  // they are: they start at zero for this solve (the layout depends on m)
  CSEM_CUDA_TRY(cudaMemsetAsync(gm.p, 0, need, st));
  const float2* GD = gm.as<float2>() + (size_t)(2 * m + 2) * nsys * n;
  while (!running.empty()) {
    std::vector<double> ti;
    for (int s : running) {
      const double rel = res[s].outer == 0 ? 1.0 : rnorm[s] / bn[s];
      ti.push_back(std::min(0.5, std::max(o.inner_tol, 0.5 * tol[s] / rel)));
    }
    std::vector<int> it;
    gmres_inner(running, ti, o, it);
    for (size_t q = 0; q < running.size(); q++) res[running[q]].inner_iters += it[q];
    outer_update(running, rnorm, false, GD);
    std::vector<int> next;
    for (int s : running) {
      res[s].outer += 1;
      const double rel = rnorm[s] / bn[s];
      res[s].relres = rel;
      if (rel < tol[s]) res[s].status = ST_CONVERGED;
      else if (!std::isfinite(rel)) res[s].status = ST_NONFINITE;
      else if (res[s].inner_iters >= o.max_inner_total || res[s].outer >= o.max_outer) res[s].status = ST_MAXITER;
      else next.push_back(s);
    }
    running = next;
  }
}

void MixedBatch::extract(int nch, const int* ch, int nrec, const float* rec, double* out_host)
{
  const size_t rb = sizeof(float) * 5 * (size_t)nrec;
  recbuf.alloc(rb + sizeof(int) * nch + 16);
  outbuf.alloc(sizeof(double2) * (size_t)nsys * nch * (nrec > 0 ? nrec : 1));
  char* d = recbuf.as<char>();
  CSEM_CUDA_TRY(cudaMemcpyAsync(d, rec, rb, cudaMemcpyHostToDevice, st));
  CSEM_CUDA_TRY(cudaMemcpyAsync(d + rb, ch, sizeof(int) * nch, cudaMemcpyHostToDevice, st));
  launch_extract<double2>(m->acq, nsys, nch, (const int*)(d + rb), nrec, (const float*)d, x64.as<double2>(), n,
                          nullptr, outbuf.as<double2>(), st);
  CSEM_CUDA_TRY(cudaGetLastError());
  CSEM_CUDA_TRY(cudaMemcpyAsync(out_host, outbuf.p, sizeof(double2) * (size_t)nsys * nch * nrec,
                                cudaMemcpyDeviceToHost, st));
  CSEM_CUDA_TRY(cudaStreamSynchronize(st));
}

}  // namespace csem
