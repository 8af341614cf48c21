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
#include <cmath>
#include <cstring>
#include "solve_mixed.h"

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
  vec32.alloc(sizeof(float2) * N * 8);
  ks.alloc(sizeof(KrylovScalars) * nsys);
  sc64.alloc(sizeof(SysScal<F64>) * nsys);
  sc32.alloc(sizeof(SysScal<F32>) * nsys);
  dots.alloc(sizeof(double2) * 8 * nsys);
  partial.alloc(sizeof(double2) * (size_t)nblk * nsys);
  list.alloc(sizeof(int) * nsys);
  rn.alloc(sizeof(double) * nsys);
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
  float2 *r = V(0), *r0 = V(1), *p = V(2), *pp = V(3), *v = V(4), *s = V(5), *t = V(6), *d = V(7);
  KrylovScalars* K = ks.as<KrylovScalars>();
  double2* D = dots.as<double2>();
  double2* part = partial.as<double2>();
  const SysScal<F32>* sc = sc32.as<SysScal<F32>>();
  auto M = [&](const float2* in, float2* out) {
    if (preco == PRE_APHI) o32.apply_aphi(in, out, nact, dl, sc);
    else o32.apply_lusgs(in, out, nact, dl, sc);
  };
  M(p, pp);
  o32.apply_A(pp, v, nact, dl, sc);
  launch_dot<F32>(v, r0, n, n, nact, dl, part, nblk, D + 0 * nsys, st);
  launch_sc_alpha(nact, dl, K, D + 0 * nsys, st);
  launch_vec<F32>(VEC_S, n, nact, dl, K, r, v, s, nullptr, nullptr, st);
  M(s, r);
  o32.apply_A(r, t, nact, dl, sc);
  launch_dot<F32>(s, t, n, n, nact, dl, part, nblk, D + 1 * nsys, st);
  launch_dot<F32>(t, t, n, n, nact, dl, part, nblk, D + 2 * nsys, st);
  launch_sc_omega(nact, dl, K, D + 1 * nsys, D + 2 * nsys, st);
  launch_vec<F32>(VEC_XR, n, nact, dl, K, d, pp, r, s, t, st);
  launch_dot<F32>(r, r, n, n, nact, dl, part, nblk, D + 3 * nsys, st);
  launch_dot<F32>(r, r0, n, n, nact, dl, part, nblk, D + 4 * nsys, st);
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
  launch_dot<F32>(V(0), V(1), n, n, ng, dl, partial.as<double2>(), nblk, D + 5 * nsys, st);
  launch_dot<F32>(V(0), V(0), n, n, ng, dl, partial.as<double2>(), nblk, D + 6 * nsys, st);
  launch_sc_init(ng, dl, ks.as<KrylovScalars>(), D + 5 * nsys, D + 6 * nsys, nullptr, 0, st);
  CSEM_CUDA_TRY(cudaGetLastError());
}

void MixedBatch::outer_update(const std::vector<int>& g, std::vector<double>& rnorm, bool first)
{
  const int ng = (int)g.size();
  CSEM_CUDA_TRY(cudaMemcpyAsync(list.p, g.data(), sizeof(int) * ng, cudaMemcpyHostToDevice, st));
  const int* dl = list.as<int>();
  dim3 grd((unsigned)((n + 255) / 256), ng);
  if (!first) {
    count_launch(), k_outer_accum<<<grd, 256, 0, st>>>(n, dl, rn.as<double>(), x64.as<double2>(), V(7));
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
  if (o.autotune && o.preco != PRE_APHI && !running.empty()) {
    CSEM_CUDA_TRY(cudaMemcpyAsync(list.p, running.data(), sizeof(int) * running.size(), cudaMemcpyHostToDevice, st));
    tuned_vw = autotune_lusgs((int)running.size(), list.as<int>());
  }
  start_inner(running, ti);
  std::vector<KrylovScalars> kh(nsys);
  inner_launch_iters = 0;
  while (!running.empty()) {
    CSEM_CUDA_TRY(cudaMemcpyAsync(list.p, running.data(), sizeof(int) * running.size(), cudaMemcpyHostToDevice, st));
    for (int q = 0; q < o.check_every; q++) {
      inner_iteration((int)running.size(), list.as<int>(), o.preco, o.niter);
      inner_launch_iters += (long)running.size();
    }
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
