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
#include "solve_mixed.h"
#include "../../include/csem_gpu.h"

namespace csem {

__global__ void k_start_inner(long n, const int* __restrict__ list, const double* __restrict__ rn,
                              const double2* __restrict__ r64, float2* __restrict__ r, float2* __restrict__ r0,
                              float2* __restrict__ p, float2* __restrict__ d)
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

MixedBatch::~MixedBatch()
{
  for (auto& kv : graphs_)
    if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
}

// The iterations between two status reads are the same launch sequence every time for a
// given number of running systems (their indices live in the device list the kernels
// read), so from the second occurrence on they are captured once and replayed as a CUDA
// graph. The first occurrence runs directly, which also creates everything created on
// first use (FFT plans, A-phi work arrays) before any capture. Per-operator profiling
// records events per application, so it keeps the direct launches.
void MixedBatch::inner_iterations(int nact, const MixedOptions& o)
{
  const int* dl = list.as<int>();
  auto direct = [&]() {
    for (int q = 0; q < o.check_every; q++) inner_iteration(nact, dl, o.preco, o.niter);
  };
  if (!o.graphs || prof_on()) {
    direct();
    return;
  }
  Graph& g = graphs_[std::make_tuple(nact, o.preco, o.check_every, o.niter)];
  if (g.failed || g.seen++ == 0) {
    direct();
    return;
  }
  if (!g.exec) {
    cudaGraph_t graph = nullptr;
    const long long l0 = csem_launch_count();
    CSEM_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    try {
      for (int q = 0; q < o.check_every; q++) inner_iteration(nact, dl, o.preco, o.niter);
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
      direct();
      return;
    }
    cudaGraphDestroy(graph);
  }
  CSEM_CUDA_TRY(cudaGraphLaunch(g.exec, st));
  count_launch(g.launches);
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
    else o32.apply_lusgs(in, out, nact, dl, sc, true);
  };
  M(p, pp);
  o32.apply_A(pp, v, nact, dl, sc);
  launch_dot<F32>(v, r0, n, n, nact, dl, part, nblk, D + 0 * nsys, st);
  launch_sc_alpha(nact, dl, K, D + 0 * nsys, st);
  launch_vec<F32>(VEC_S, n, nact, dl, K, r, v, s, nullptr, nullptr, st);
  M(s, sh);
  o32.apply_A(sh, t, nact, dl, sc);
  launch_dot2<F32>(s, t, t, t, n, n, nact, dl, part, nblk, D + 1 * nsys, D + 2 * nsys, st);
  launch_sc_omega(nact, dl, K, D + 1 * nsys, D + 2 * nsys, st);
  launch_xr_dot2<F32>(n, nact, dl, K, d, pp, sh, r, s, t, r0, part, nblk, D + 3 * nsys, D + 4 * nsys, st);
  launch_sc_rs_beta(nact, dl, K, D + 3 * nsys, D + 4 * nsys, nullptr, 0, maxiter, st);
  launch_vec<F32>(VEC_P, n, nact, dl, K, r, p, v, nullptr, nullptr, st);
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

// Autotuner of the complex64 LU-SGS schedule: applies the preconditioner to the batch's
// current vectors once per candidate (points per thread 1, 2, 4 of the lockstep sweeps)
// after one untimed application each, times it with CUDA events on the solver's stream,
// and keeps the fastest for the rest of this batch. The scratch vector it writes is
// overwritten before use by the solve.
int MixedBatch::autotune_lusgs(int nact, const int* dlist)
{
  const SysScal<F32>* sc = sc32.as<SysScal<F32>>();
  const int cand[3] = {1, 2, 4};
  cudaEvent_t e0, e1;
  CSEM_CUDA_TRY(cudaEventCreate(&e0));
  CSEM_CUDA_TRY(cudaEventCreate(&e1));
  float best_ms = 1e30f;
  int best = 0;
  const bool saved = o32.pipelined_sweeps;
  o32.pipelined_sweeps = true;
  for (int vw : cand) {
    o32.sweep_vw = vw;
    o32.apply_lusgs(V(0), V(3), nact, dlist, sc);
    CSEM_CUDA_TRY(cudaEventRecord(e0, st));
    o32.apply_lusgs(V(0), V(3), nact, dlist, sc);
    CSEM_CUDA_TRY(cudaEventRecord(e1, st));
    CSEM_CUDA_TRY(cudaEventSynchronize(e1));
    float ms = 0.f;
    CSEM_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
    if (ms < best_ms) {
      best_ms = ms;
      best = vw;
    }
  }
  o32.pipelined_sweeps = saved;
  o32.sweep_vw = best;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return best;
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
    CSEM_CUDA_TRY(cudaMemcpyAsync(list.p, running.data(), sizeof(int) * running.size(), cudaMemcpyHostToDevice, st));
    tuned_vw = autotune_lusgs((int)running.size(), list.as<int>());
  }
  start_inner(running, ti);
  std::vector<KrylovScalars> kh(nsys);
  inner_launch_iters = 0;
  while (!running.empty()) {
    CSEM_CUDA_TRY(cudaMemcpyAsync(list.p, running.data(), sizeof(int) * running.size(), cudaMemcpyHostToDevice, st));
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
// Vectors, preconditioner, operator and dot products run batched on the device over the
// systems still iterating; the (m+1) x m Hessenberg algebra of every system runs in
// complex128 on the host (one read of the batched dot products per Gram-Schmidt step).
// A system leaves the step loop of a cycle when its estimated residual reaches the inner
// reduction.
namespace {
typedef std::complex<double> zc;
inline zc Z(double2 v) { return zc(v.x, v.y); }
inline double2 D2(zc v) { return make_double2(v.real(), v.imag()); }
}  // namespace

std::vector<double2> MixedBatch::batch_dot(const float2* a, const float2* b, int ng, const int* dl)
{
  double2* Dd = dots.as<double2>();
  launch_dot<F32>(a, b, n, n, ng, dl, partial.as<double2>(), nblk, Dd, st);
  std::vector<double2> h(ng);
  CSEM_CUDA_TRY(cudaMemcpyAsync(h.data(), Dd, sizeof(double2) * ng, cudaMemcpyDeviceToHost, st));
  CSEM_CUDA_TRY(cudaStreamSynchronize(st));
  return h;
}

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
  double2* cf = gcoef.as<double2>();
  auto M = [&](const float2* in, float2* out, int ng, const int* dl) {  // Z_j: only written here
    if (o.preco == PRE_APHI) o32.apply_aphi(in, out, ng, dl, sc);
    else o32.apply_lusgs(in, out, ng, dl, sc, true);
  };
  // r0 = r64 / |r64|, d = 0 (k_start_inner writes r, r0, p, d: here r0 twice and d)
  {
    CSEM_CUDA_TRY(cudaMemcpyAsync(list.p, g.data(), sizeof(int) * g.size(), cudaMemcpyHostToDevice, st));
    dim3 grd((unsigned)((n + 255) / 256), (unsigned)g.size());
    count_launch(), k_start_inner<<<grd, 256, 0, st>>>(n, list.as<int>(), rn.as<double>(), r64.as<double2>(), GR0, GR0,
                                                       GW, GD);
  }
  const int ns = (int)g.size();
  std::vector<double> beta0(ns, 1.0);
  std::vector<char> done(ns, 0);
  iters.assign(ns, 0);
  std::vector<int> lists(nsys);
  for (int cycle = 0;; cycle++) {
    std::vector<int> act;  // positions in g of systems still solving
    for (int q = 0; q < ns; q++)
      if (!done[q] && iters[q] < o.niter) act.push_back(q);
    if (act.empty()) break;
    int na = (int)act.size();
    std::vector<int> sl(na);
    for (int a = 0; a < na; a++) sl[a] = g[act[a]];
    CSEM_CUDA_TRY(cudaMemcpyAsync(list.p, sl.data(), sizeof(int) * na, cudaMemcpyHostToDevice, st));
    const int* dl = list.as<int>();
    // r = r0 - A d  (d = 0 on the first cycle)
    if (cycle == 0) {
      CSEM_CUDA_TRY(cudaMemcpyAsync(GW, GR0, sizeof(float2) * N, cudaMemcpyDeviceToDevice, st));
    } else {
      o32.apply_A(GD, GV(0), na, dl, sc);
      launch_vec<F32>(VEC_SUB, n, na, dl, nullptr, GR0, GV(0), GW, nullptr, nullptr, st);
    }
    std::vector<double2> bb = batch_dot(GW, GW, na, dl);
    std::vector<double> beta(na);
    std::vector<double2> cdiv(na);
    for (int a = 0; a < na; a++) {
      beta[a] = std::sqrt(bb[a].x);
      if (cycle == 0) beta0[act[a]] = beta[a] > 0 ? beta[a] : 1.0;
      cdiv[a] = make_double2(beta[a] > 0 ? beta[a] : 1.0, 0.0);
    }
    CSEM_CUDA_TRY(cudaMemcpyAsync(cf, cdiv.data(), sizeof(double2) * na, cudaMemcpyHostToDevice, st));
    launch_cdivv<F32>(n, na, dl, cf, 1, 1, GW, GV(0), st);
    // per-system Hessenberg (column j in H[j][0..j+1]), Givens and right-hand side
    std::vector<std::vector<zc>> H(na, std::vector<zc>((size_t)m * (m + 1))), gg(na, std::vector<zc>(m + 1));
    std::vector<std::vector<zc>> cs(na, std::vector<zc>(m));
    std::vector<std::vector<double>> sn(na, std::vector<double>(m));
    std::vector<int> steps(na, 0);
    std::vector<char> stop(na, 0);
    for (int a = 0; a < na; a++) gg[a][0] = zc(beta[a], 0.0);
    for (int j = 0; j < m; j++) {
      std::vector<int> live;  // positions in act of systems stepping
      for (int a = 0; a < na; a++)
        if (!stop[a]) live.push_back(a);
      if (live.empty()) break;
      const int nl = (int)live.size();
      std::vector<int> ll(nl);
      for (int b = 0; b < nl; b++) ll[b] = sl[live[b]];
      CSEM_CUDA_TRY(cudaMemcpyAsync(list.p, ll.data(), sizeof(int) * nl, cudaMemcpyHostToDevice, st));
      M(GV(j), GZ(j), nl, dl);
      o32.apply_A(GZ(j), GW, nl, dl, sc);
      for (int i = 0; i <= j; i++) {
        std::vector<double2> h = batch_dot(GW, GV(i), nl, dl);
        for (int b = 0; b < nl; b++) H[live[b]][(size_t)j * (m + 1) + i] = Z(h[b]);
        CSEM_CUDA_TRY(cudaMemcpyAsync(cf, h.data(), sizeof(double2) * nl, cudaMemcpyHostToDevice, st));
        launch_axpy<F32>(n, nl, dl, cf, 1, 1, GV(i), GW, st);
      }
      std::vector<double2> hn = batch_dot(GW, GW, nl, dl);
      std::vector<double2> dv(nl);
      for (int b = 0; b < nl; b++) {
        const double hv = std::sqrt(hn[b].x);
        H[live[b]][(size_t)j * (m + 1) + j + 1] = zc(hv, 0.0);
        dv[b] = make_double2(hv > 0 ? hv : 1.0, 0.0);
      }
      CSEM_CUDA_TRY(cudaMemcpyAsync(cf, dv.data(), sizeof(double2) * nl, cudaMemcpyHostToDevice, st));
      launch_cdivv<F32>(n, nl, dl, cf, 1, 1, GW, GV(j + 1), st);
      for (int b = 0; b < nl; b++) {
        const int a = live[b];
        zc* col = &H[a][(size_t)j * (m + 1)];
        for (int i = 0; i < j; i++) {  // earlier rotations
          const zc t = std::conj(cs[a][i]) * col[i] + sn[a][i] * col[i + 1];
          col[i + 1] = -sn[a][i] * col[i] + cs[a][i] * col[i + 1];
          col[i] = t;
        }
        const double tmp = std::sqrt(std::norm(col[j]) + std::norm(col[j + 1]));
        if (tmp == 0.0) {
          stop[a] = 1;
          continue;
        }
        sn[a][j] = col[j + 1].real() / tmp;
        cs[a][j] = col[j] / tmp;
        gg[a][j + 1] = -sn[a][j] * gg[a][j];
        gg[a][j] = std::conj(cs[a][j]) * gg[a][j];
        col[j] = std::conj(cs[a][j]) * col[j] + sn[a][j] * col[j + 1];
        steps[a] = j + 1;
        iters[act[a]] += 1;
        const double rel = std::abs(gg[a][j + 1]) / beta0[act[a]];
        if (rel < tol_inner[act[a]] || !(hn[b].x > 0.0)) {
          stop[a] = 1;
          done[act[a]] = 1;
        } else if (iters[act[a]] >= o.niter) {
          stop[a] = 1;
        }
      }
    }
    // d += sum_i y_i z_i, y from the triangular system, per system with its own size
    int mmax = 0;
    for (int a = 0; a < na; a++) mmax = std::max(mmax, steps[a]);
    std::vector<double2> y((size_t)mmax * na, make_double2(0, 0));
    for (int a = 0; a < na; a++) {
      const int mm = steps[a];
      std::vector<zc> yv(mm);
      for (int i = mm - 1; i >= 0; i--) {
        zc acc = gg[a][i];
        for (int k2 = i + 1; k2 < mm; k2++) acc -= H[a][(size_t)k2 * (m + 1) + i] * yv[k2];
        yv[i] = acc / H[a][(size_t)i * (m + 1) + i];
      }
      for (int i = 0; i < mm; i++) y[(size_t)i * na + a] = D2(yv[i]);
    }
    CSEM_CUDA_TRY(cudaMemcpyAsync(list.p, sl.data(), sizeof(int) * na, cudaMemcpyHostToDevice, st));
    if (mmax > 0)
      CSEM_CUDA_TRY(cudaMemcpyAsync(cf, y.data(), sizeof(double2) * y.size(), cudaMemcpyHostToDevice, st));
    for (int i = 0; i < mmax; i++) launch_axpy<F32>(n, na, dl, cf + (size_t)i * na, 1, 0, GZ(i), GD, st);
    CSEM_CUDA_TRY(cudaGetLastError());
  }
}

void MixedBatch::solve_gmres(const std::vector<double>& bn, const double* tol, const MixedOptions& o,
                             std::vector<MixedResult>& res, std::vector<double>& rnorm, std::vector<int> running)
{
  const int m = std::max(1, o.nrestart);
  const size_t need = sizeof(float2) * (size_t)(2 * m + 4) * nsys * n;
  if (gm.bytes < need) gm.alloc(need);
  // the Z_j are written only by the preconditioner, which leaves boundary entries as
  // they are: they start at zero for this solve (the layout depends on m)
  CSEM_CUDA_TRY(cudaMemsetAsync(gm.p, 0, need, st));
  const size_t needc = sizeof(double2) * (size_t)(m + 2) * nsys;
  if (gcoef.bytes < needc) gcoef.alloc(needc);
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
