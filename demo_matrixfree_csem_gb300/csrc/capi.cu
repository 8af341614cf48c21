// extern "C" entry points of libcsem_gpu.so (declared in include/csem_gpu.h).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <string>
#include <system_error>
#include <thread>
#include <cstring>
#include <memory>
#include <new>
#include <vector>
#include "../../include/csem_gpu.h"
#include "engine_model.h"
#include "solve_fp64.h"
#include "solve_mixed.h"

extern "C" int csem_set_error(int code, const char* fmt, ...);

using namespace csem;

struct csem_ctx {
  Model* model = nullptr;
  cudaStream_t st = nullptr;
  Ops<F64>* ops64 = nullptr;
  Ops<F32>* ops32 = nullptr;
  Solver64* solver = nullptr;
  MixedBatch* batch = nullptr;
  DevBuf io[4], sc64, sc32, dotp, groups;
  int nmax64 = 0, nmax32 = 0;
  bool lusgs_pipelined = true;
  int lusgs_vw = 0;
  int lusgs_lines = 1;
  int lusgs_systems = 1;
  bool lusgs_split = true;
  bool lusgs_overlap = true;
  bool fused_dots = false;
  bool quick_residual = true;
  int lusgs_cap = 0;
  int stencil_by = 8, stencil_ctas = 4;
  bool lusgs_tiled = false;
  bool aphi_fix = false;
  int tile_rows = 8, tile_vw = 4;
  bool autotune = false;
  bool graphs = true;
  bool seq_dots = false;
};

// the context's kernel-schedule options on one operator set
template <class P> static void configure(const csem_ctx* c, Ops<P>& o)
{
  o.pipelined_sweeps = c->lusgs_pipelined;
  o.sweep_vw = c->lusgs_vw;
  o.sweep_lines = c->lusgs_lines;
  o.sweep_systems = c->lusgs_systems;
  o.split_sweeps = c->lusgs_split;
  o.split_overlap = c->lusgs_overlap;
  o.fused_dots = c->fused_dots;
  o.split_cap = c->lusgs_cap;
  o.stencil_by = c->stencil_by;
  o.stencil_ctas = c->stencil_ctas;
  o.tiled_sweeps = c->lusgs_tiled;
  o.aphi_fix = c->aphi_fix;
  o.tile_rows = c->tile_rows;
  o.tile_vw = c->tile_vw;
}

#define API_BEGIN try {
#define API_END                                                                                          \
  }                                                                                                      \
  catch (const CudaError& e) {                                                                           \
    return csem_set_error(CSEM_ECUDA, "CUDA error %d (%s) in %s at %s:%d", (int)e.err,                  \
                          cudaGetErrorString(e.err), e.expr, e.file, e.line);                            \
  }                                                                                                      \
  catch (const std::bad_alloc&) {                                                                        \
    return csem_set_error(CSEM_ENOMEM, "host allocation failed");                                        \
  }                                                                                                      \
  return CSEM_OK;

static Ops<F64>* ops64_for(csem_ctx* c, int nsys)
{
  if (!c->ops64 || c->nmax64 < nsys) {
    delete c->ops64;
    c->ops64 = new Ops<F64>(c->model, nsys, c->st);
    configure(c, *c->ops64);
    c->nmax64 = nsys;
  }
  return c->ops64;
}

static Ops<F32>* ops32_for(csem_ctx* c, int nsys)
{
  if (!c->ops32 || c->nmax32 < nsys) {
    delete c->ops32;
    c->ops32 = new Ops<F32>(c->model, nsys, c->st);
    configure(c, *c->ops32);
    c->nmax32 = nsys;
  }
  return c->ops32;
}

static void ensure(DevBuf& b, size_t bytes)
{
  if (b.bytes < bytes) b.alloc(bytes);
}

// per-system scalars from host (re,im) pairs
static void upload_scal(csem_ctx* c, int nsys, const double* iom)
{
  std::vector<SysScal<F64>> s64(nsys);
  std::vector<SysScal<F32>> s32(nsys);
  for (int q = 0; q < nsys; q++) {
    s64[q] = sys_scal64(iom[2 * q], iom[2 * q + 1]);
    s32[q] = sys_scal32(s64[q]);
  }
  ensure(c->sc64, sizeof(SysScal<F64>) * nsys);
  ensure(c->sc32, sizeof(SysScal<F32>) * nsys);
  CSEM_CUDA_TRY(cudaMemcpyAsync(c->sc64.p, s64.data(), sizeof(SysScal<F64>) * nsys, cudaMemcpyHostToDevice, c->st));
  CSEM_CUDA_TRY(cudaMemcpyAsync(c->sc32.p, s32.data(), sizeof(SysScal<F32>) * nsys, cudaMemcpyHostToDevice, c->st));
  CSEM_CUDA_TRY(cudaStreamSynchronize(c->st));
}

extern "C" {

const char* csem_version(void) { return "csem-gb300 0.1 (sm_103a)"; }

int csem_device_count(void)
{
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

int csem_ctx_create(const csem_grid_t* g, int airbc, int fvm, csem_ctx** out)
{
  *out = nullptr;
  if (csem_device_count() < 1) return csem_set_error(CSEM_ENODEV, "no CUDA device available");
  if (!g || !g->sigma11) return csem_set_error(CSEM_EINVAL, "grid is not extended (csem_grid_extend)");
  if (airbc && (g->nb <= 0 || !g->sH1))
    return csem_set_error(CSEM_EINVAL, "airbc=1 needs nb>0 and the airwave tables (csem_grid_airbc)");
  API_BEGIN
  std::unique_ptr<csem_ctx> c(new csem_ctx());
  CSEM_CUDA_TRY(cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking));
  c->model = new Model((const csem_grid*)g, airbc, fvm);
  *out = c.release();
  API_END
}

void csem_ctx_destroy(csem_ctx* c)
{
  if (!c) return;
  cudaStreamSynchronize(c->st);
  delete c->batch;
  delete c->solver;
  delete c->ops64;
  delete c->ops32;
  delete c->model;
  for (auto& b : c->io) b.free_();
  c->sc64.free_();
  c->sc32.free_();
  c->dotp.free_();
  cudaStreamDestroy(c->st);
  delete c;
}

int csem_ctx_sizes(const csem_ctx* c, long* o)
{
  const Model* m = c->model;
  o[0] = m->lE; o[1] = m->lEx; o[2] = m->lEy; o[3] = m->lEz; o[4] = m->lv;
  o[5] = m->n1; o[6] = m->n2; o[7] = m->n3; o[8] = m->n3f; o[9] = m->nb;
  return CSEM_OK;
}

void* csem_ctx_stream(csem_ctx* c) { return (void*)c->st; }

int csem_ctx_set_option(csem_ctx* c, const char* name, int value)
{
  if (!strcmp(name, "lusgs_pipelined")) {
    c->lusgs_pipelined = value != 0;
  } else if (!strcmp(name, "lusgs_vw")) {
    if (value != 0 && value != 1 && value != 2 && value != 4)
      return csem_set_error(CSEM_EINVAL, "lusgs_vw must be 0, 1, 2 or 4");
    c->lusgs_vw = value;
  } else if (!strcmp(name, "stencil_by")) {
    if (value != 4 && value != 8 && value != 16) return csem_set_error(CSEM_EINVAL, "stencil_by must be 4, 8 or 16");
    c->stencil_by = value;
  } else if (!strcmp(name, "stencil_ctas")) {
    if (value < 1 || value > 16) return csem_set_error(CSEM_EINVAL, "stencil_ctas must be in 1..16");
    c->stencil_ctas = value;
  } else if (!strcmp(name, "lusgs_lines")) {
    if (value < 1 || value > 64) return csem_set_error(CSEM_EINVAL, "lusgs_lines must be in 1..64");
    c->lusgs_lines = value;
  } else if (!strcmp(name, "lusgs_systems")) {
    if (value != 1 && value != 2 && value != 4) return csem_set_error(CSEM_EINVAL, "lusgs_systems must be 1, 2 or 4");
    c->lusgs_systems = value;
  } else if (!strcmp(name, "lusgs_split")) {
    c->lusgs_split = value != 0;
  } else if (!strcmp(name, "quick_residual")) {
    c->quick_residual = value != 0;
  } else if (!strcmp(name, "fused_dots")) {
    c->fused_dots = value != 0;
  } else if (!strcmp(name, "lusgs_overlap")) {
    c->lusgs_overlap = value != 0;
  } else if (!strcmp(name, "lusgs_cap")) {
    if (value < 0 || value > 16) return csem_set_error(CSEM_EINVAL, "lusgs_cap must be in 0..16");
    c->lusgs_cap = value;
  } else if (!strcmp(name, "aphi_fix")) {
    c->aphi_fix = value != 0;
  } else if (!strcmp(name, "lusgs_tiled")) {
    c->lusgs_tiled = value != 0;
  } else if (!strcmp(name, "lusgs_tile_rows")) {
    if (value != 4 && value != 8 && value != 16) return csem_set_error(CSEM_EINVAL, "lusgs_tile_rows must be 4, 8 or 16");
    c->tile_rows = value;
  } else if (!strcmp(name, "lusgs_tile_vw")) {
    if (value != 1 && value != 2 && value != 4) return csem_set_error(CSEM_EINVAL, "lusgs_tile_vw must be 1, 2 or 4");
    c->tile_vw = value;
  } else if (!strcmp(name, "autotune")) {
    c->autotune = value != 0;
  } else if (!strcmp(name, "graphs")) {
    c->graphs = value != 0;
  } else if (!strcmp(name, "dot_order")) {
    if (value != 0 && value != 1) return csem_set_error(CSEM_EINVAL, "dot_order must be 0 (tree) or 1 (reference)");
    c->seq_dots = value == 1;
  } else if (!strcmp(name, "fix_quirks")) {
    c->model->acq.fix_src_sigma = value != 0;
  } else {
    return csem_set_error(CSEM_EINVAL, "unknown option %s", name);
  }
  if (c->ops64) configure(c, *c->ops64);
  if (c->ops32) configure(c, *c->ops32);
  if (c->solver) {
    configure(c, c->solver->ops);
    c->solver->seq_dots = c->seq_dots;
  }
  if (c->batch) {
    configure(c, c->batch->o64);
    configure(c, c->batch->o32);
    c->batch->o64.quick_stencil = c->quick_residual;  // the defect correction's residual only
  }
  return CSEM_OK;
}

// Device bytes a batch of nsys systems needs on this context (MixedBatch and its two
// operator sets, or the complex128 solver), excluding the model itself and cuFFT's work
// areas.
static double batch_bytes(const Model* m, int precision, int preco, int nsys)
{
  const double lE = (double)m->lE, lv = (double)m->lv;
  auto ops = [&](double cs) {
    double b = 0;
    if (m->airbc) {
      const double capE = (double)m->nb * ((double)m->n1 * (m->n2 + 1) + (double)(m->n1 + 1) * m->n2 +
                                           (double)(m->n1 + 1) * (m->n2 + 1));
      b += cs * ((double)m->n1 * m->n2 + 3.0 * m->N1 * m->N2 + (double)(m->n1 + 1) * m->n2 +
                 (double)m->n1 * (m->n2 + 1) + capE);
    }
    if (preco == PRE_APHI) b += 2.0 * cs * lv;
    return b;
  };
  if (precision == 32) {
    // x, b, r, w in complex128; 9 complex64 Krylov vectors; per-system scalars; the split
    // LU-SGS sweeps' (B, w) of the largest component on the sweep grid
    const double split = preco == PRE_LUSGS
                             ? 16.0 * (double)sweep_split_scratch(m->n1, m->n2, m->airbc ? m->n3f : m->n3)
                             : 0.0;
    return nsys * (4.0 * 16 * lE + 9.0 * 8 * lE + ops(16) + ops(8) + split + 4096.0);
  }
  // the complex128 solver runs one system at a time: 7 BiCGStab vectors or GMRES(m) bases
  return 16.0 * lE * 40 + ops(16);
}

int csem_batch_bytes(csem_ctx* c, int precision, int preco, int nsys, double* bytes)
{
  if (!c || !bytes || nsys < 1 || (precision != 32 && precision != 64))
    return csem_set_error(CSEM_EINVAL, "csem_batch_bytes: bad argument");
  *bytes = batch_bytes(c->model, precision, preco, nsys);
  return CSEM_OK;
}

int csem_sweep_groups(int nslot, const double* iom, int ns, int halves, int* groups, int* ngroups, int* nA, int* ngA)
{
  if (nslot < 1 || ns < 1 || !iom || !groups || !ngroups || !nA || !ngA)
    return csem_set_error(CSEM_EINVAL, "csem_sweep_groups: bad argument");
  try {
    std::vector<int> out;
    *ngroups = halves ? build_sweep_groups_halves(nslot, iom, ns, 4, out, nA, ngA)
                      : (*nA = *ngA = 0, build_sweep_groups(nslot, iom, ns, out));
    memcpy(groups, out.data(), sizeof(int) * out.size());
  } catch (const std::bad_alloc&) {
    return csem_set_error(CSEM_ENOMEM, "host allocation failed");
  }
  return CSEM_OK;
}

int csem_batch_capacity(csem_ctx* c, int precision, int preco, double budget_bytes, int* nsys)
{
  if (!c || !nsys || (precision != 32 && precision != 64))
    return csem_set_error(CSEM_EINVAL, "csem_batch_capacity: bad argument");
  if (precision == 64) {
    *nsys = budget_bytes >= batch_bytes(c->model, 64, preco, 1) ? 1 << 30 : 0;
    return CSEM_OK;
  }
  const double one = batch_bytes(c->model, 32, preco, 1);
  *nsys = one > 0 ? (int)std::min(1.0e9, std::floor(budget_bytes / one)) : 0;
  return CSEM_OK;
}

int csem_solve_batches_host(int njobs, csem_batch_job* jobs)
{
  if (njobs < 0 || (njobs > 0 && !jobs)) return csem_set_error(CSEM_EINVAL, "csem_solve_batches_host: bad arguments");
  for (int a = 0; a < njobs; a++) {
    if (!jobs[a].ctx) return csem_set_error(CSEM_EINVAL, "csem_solve_batches_host: job %d has no context", a);
    for (int b = 0; b < a; b++)
      if (jobs[a].ctx == jobs[b].ctx)
        return csem_set_error(CSEM_EINVAL, "csem_solve_batches_host: jobs %d and %d share a context", b, a);
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return csem_set_error(CSEM_ENODEV, "no CUDA device available");
  std::vector<std::string> msgs(njobs);
  auto run = [&](int a) {
    cudaSetDevice(dev);
    csem_batch_job& j = jobs[a];
    j.rc = csem_solve_batch_host(j.ctx, j.nsys, j.freq, j.src3, j.nchsrc, j.chsrc, j.nchrec, j.chrec, j.nrec, j.rec,
                                 j.opt, j.dcal, j.iters, j.outer, j.status, j.relres);
    if (j.rc) msgs[a] = csem_last_error();  // the message lives in this thread
  };
  std::vector<std::thread> th;
  try {
    for (int a = 1; a < njobs; a++) th.emplace_back(run, a);
  } catch (const std::system_error&) {
    for (auto& t : th) t.join();
    return csem_set_error(CSEM_ENOMEM, "csem_solve_batches_host: cannot start threads");
  }
  if (njobs > 0) run(0);
  for (auto& t : th) t.join();
  for (int a = 0; a < njobs; a++)
    if (jobs[a].rc) return csem_set_error(jobs[a].rc, "job %d: %s", a, msgs[a].c_str());
  return CSEM_OK;
}

int csem_solve_batch_multi(int ndev, const int* devices, const csem_grid_t* g, int airbc, int fvm, int nsys,
                           const float* freq, const float* src3, int nchsrc, const int* chsrc, int nchrec,
                           const int* chrec, int nrec, const float* rec, const csem_batch_opts* opt, double* dcal,
                           int* iters, int* outer, int* status, double* relres, int* owner)
{
  if (ndev < 1 || !devices || !g || nsys < 1 || !freq || !src3 || !opt || !dcal)
    return csem_set_error(CSEM_EINVAL, "csem_solve_batch_multi: bad arguments");
  const int ndevs = csem_device_count();
  if (ndevs < 1) return csem_set_error(CSEM_ENODEV, "no CUDA device available");
  for (int d = 0; d < ndev; d++)
    if (devices[d] < 0 || devices[d] >= ndevs)
      return csem_set_error(CSEM_EINVAL, "csem_solve_batch_multi: device %d does not exist", devices[d]);
  // work per system: unknowns of the operator grid (the same model on every slot)
  const long n3 = airbc ? (long)g->nz + g->nb : (long)g->n3;
  const double unknowns = (double)g->n1 * (g->n2 + 1) * (n3 + 1) + (double)(g->n1 + 1) * g->n2 * (n3 + 1) +
                          (double)(g->n1 + 1) * (g->n2 + 1) * n3;
  std::vector<int> own(nsys);
  int rc = csem_partition_systems(nsys, freq, nullptr, unknowns, ndev, own.data(), nullptr);
  if (rc) return rc;
  if (owner)
    for (int s = 0; s < nsys; s++) owner[s] = own[s];
  const size_t per = (size_t)nchrec * (nrec > 0 ? nrec : 0) * 2;
  std::vector<int> rcs(ndev, CSEM_OK);
  std::vector<std::string> msgs(ndev);
  auto run = [&](int d) {
    std::vector<int> mine;
    for (int s = 0; s < nsys; s++)
      if (own[s] == d) mine.push_back(s);
    if (mine.empty()) return;
    const int m = (int)mine.size();
    std::vector<float> f(m), xyz(3 * (size_t)m);
    for (int q = 0; q < m; q++) {
      f[q] = freq[mine[q]];
      for (int c = 0; c < 3; c++) xyz[3 * (size_t)q + c] = src3[3 * (size_t)mine[q] + c];
    }
    std::vector<double> dc(per * m + 1), rr(m);
    std::vector<int> it(m), ou(m), st(m);
    csem_ctx* ctx = nullptr;
    int r = cudaSetDevice(devices[d]) == cudaSuccess ? CSEM_OK
                                                      : csem_set_error(CSEM_ECUDA, "cudaSetDevice(%d) failed", devices[d]);
    if (!r) r = csem_ctx_create(g, airbc, fvm, &ctx);
    if (!r)
      r = csem_solve_batch_host(ctx, m, f.data(), xyz.data(), nchsrc, chsrc, nchrec, chrec, nrec, rec, opt,
                                dc.data(), it.data(), ou.data(), st.data(), rr.data());
    if (ctx) csem_ctx_destroy(ctx);
    if (r) {
      rcs[d] = r;
      msgs[d] = csem_last_error();  // the message lives in this thread
      return;
    }
    for (int q = 0; q < m; q++) {  // the gather: this slot's systems at their positions
      const int s = mine[q];
      for (size_t k = 0; k < per; k++) dcal[per * (size_t)s + k] = dc[per * (size_t)q + k];
      if (iters) iters[s] = it[q];
      if (outer) outer[s] = ou[q];
      if (status) status[s] = st[q];
      if (relres) relres[s] = rr[q];
    }
  };
  int caller_dev = 0;
  cudaGetDevice(&caller_dev);
  std::vector<std::thread> th;
  try {
    for (int d = 1; d < ndev; d++) th.emplace_back(run, d);
  } catch (const std::system_error&) {
    for (auto& t : th) t.join();
    return csem_set_error(CSEM_ENOMEM, "csem_solve_batch_multi: cannot start threads");
  }
  run(0);
  for (auto& t : th) t.join();
  cudaSetDevice(caller_dev);  // slot 0 ran on this thread
  for (int d = 0; d < ndev; d++)
    if (rcs[d]) return csem_set_error(rcs[d], "slot %d (device %d): %s", d, devices[d], msgs[d].c_str());
  return CSEM_OK;
}

int csem_ctx_sync(csem_ctx* c)
{
  API_BEGIN
  CSEM_CUDA_TRY(cudaStreamSynchronize(c->st));
  API_END
}

}  // extern "C"

// ---------------------------------------------------------------- host-buffer operators
enum { OP_A = 0, OP_LUSGS = 1, OP_APHI = 2 };

template <class P>
static int op_host(csem_ctx* c, int op, double re, double im, const void* x, void* y)
{
  typedef typename P::C C;
  const long n = c->model->lE;
  const size_t bytes = sizeof(C) * (size_t)n;
  ensure(c->io[0], bytes);
  ensure(c->io[1], bytes);
  double iom[2] = {re, im};
  upload_scal(c, 1, iom);
  CSEM_CUDA_TRY(cudaMemcpyAsync(c->io[0].p, x, bytes, cudaMemcpyHostToDevice, c->st));
  C* X = c->io[0].as<C>();
  C* Y = c->io[1].as<C>();
  if (P::exact) {
    Ops<F64>* o = ops64_for(c, 1);
    const SysScal<F64>* s = c->sc64.as<SysScal<F64>>();
    if (op == OP_A) o->apply_A((double2*)X, (double2*)Y, 1, nullptr, s);
    else if (op == OP_LUSGS) o->apply_lusgs((double2*)X, (double2*)Y, 1, nullptr, s);
    else o->apply_aphi((double2*)X, (double2*)Y, 1, nullptr, s);
  } else {
    Ops<F32>* o = ops32_for(c, 1);
    const SysScal<F32>* s = c->sc32.as<SysScal<F32>>();
    if (op == OP_A) o->apply_A((float2*)X, (float2*)Y, 1, nullptr, s);
    else if (op == OP_LUSGS) o->apply_lusgs((float2*)X, (float2*)Y, 1, nullptr, s);
    else o->apply_aphi((float2*)X, (float2*)Y, 1, nullptr, s);
  }
  CSEM_CUDA_TRY(cudaGetLastError());
  CSEM_CUDA_TRY(cudaMemcpyAsync(y, Y, bytes, cudaMemcpyDeviceToHost, c->st));
  CSEM_CUDA_TRY(cudaStreamSynchronize(c->st));
  return CSEM_OK;
}

template <class P>
static int cdot_host(long n, const void* a, const void* b, double* out)
{
  if (csem_device_count() < 1) return csem_set_error(CSEM_ENODEV, "no CUDA device available");
  typedef typename P::C C;
  DevBuf A, B, part, res;
  const int nblk = dot_blocks(n);
  A.alloc(sizeof(C) * (size_t)(n > 0 ? n : 1));
  B.alloc(sizeof(C) * (size_t)(n > 0 ? n : 1));
  part.alloc(sizeof(double2) * nblk);
  res.alloc(sizeof(double2));
  CSEM_CUDA_TRY(cudaMemcpy(A.p, a, sizeof(C) * (size_t)n, cudaMemcpyHostToDevice));
  CSEM_CUDA_TRY(cudaMemcpy(B.p, b, sizeof(C) * (size_t)n, cudaMemcpyHostToDevice));
  launch_dot<P>(A.as<C>(), B.as<C>(), n, n, 1, nullptr, part.as<double2>(), nblk, res.as<double2>(), 0);
  CSEM_CUDA_TRY(cudaGetLastError());
  CSEM_CUDA_TRY(cudaMemcpy(out, res.p, sizeof(double2), cudaMemcpyDeviceToHost));
  return CSEM_OK;
}

extern "C" {

int csem_fdfd_apply_host(csem_ctx* c, double re, double im, const double* x, double* y)
{
  API_BEGIN return op_host<F64>(c, OP_A, re, im, x, y); API_END
}
int csem_lusgs_apply_host(csem_ctx* c, double re, double im, const double* x, double* y)
{
  API_BEGIN return op_host<F64>(c, OP_LUSGS, re, im, x, y); API_END
}
int csem_aphi_apply_host(csem_ctx* c, double re, double im, const double* x, double* y)
{
  API_BEGIN return op_host<F64>(c, OP_APHI, re, im, x, y); API_END
}
int csem_fdfd_apply_c64_host(csem_ctx* c, double re, double im, const float* x, float* y)
{
  API_BEGIN return op_host<F32>(c, OP_A, re, im, x, y); API_END
}
int csem_lusgs_apply_c64_host(csem_ctx* c, double re, double im, const float* x, float* y)
{
  API_BEGIN return op_host<F32>(c, OP_LUSGS, re, im, x, y); API_END
}
int csem_aphi_apply_c64_host(csem_ctx* c, double re, double im, const float* x, float* y)
{
  API_BEGIN return op_host<F32>(c, OP_APHI, re, im, x, y); API_END
}

static Solver64* solver_for(csem_ctx* c)
{
  if (!c->solver) {
    c->solver = new Solver64(c->model, c->st);
    configure(c, c->solver->ops);
    c->solver->seq_dots = c->seq_dots;
  }
  return c->solver;
}

int csem_gmres_pre_apply_host(csem_ctx* c, double re, double im, int mp, const double* x, double* y)
{
  if (mp < 1) return csem_set_error(CSEM_EINVAL, "mp must be >= 1");
  API_BEGIN
  Solver64* s = solver_for(c);
  const size_t bytes = sizeof(double2) * (size_t)c->model->lE;
  ensure(c->io[0], bytes);
  ensure(c->io[1], bytes);
  s->set_iom(re, im);
  CSEM_CUDA_TRY(cudaMemcpyAsync(c->io[0].p, x, bytes, cudaMemcpyHostToDevice, c->st));
  s->gmres_pre(mp, c->io[0].as<double2>(), c->io[1].as<double2>());
  CSEM_CUDA_TRY(cudaMemcpyAsync(y, c->io[1].p, bytes, cudaMemcpyDeviceToHost, c->st));
  CSEM_CUDA_TRY(cudaStreamSynchronize(c->st));
  API_END
}

int csem_airbc_apply_host(csem_ctx* c, const double* hz0, double* hx, double* hy)
{
  Model* m = c->model;
  if (!m->airbc) return csem_set_error(CSEM_EINVAL, "context was created with airbc=0");
  API_BEGIN
  Ops<F64>* o = ops64_for(c, 1);
  const size_t nz = sizeof(double2) * (size_t)m->n1 * m->n2;
  CSEM_CUDA_TRY(cudaMemcpyAsync(o->hz0.p, hz0, nz, cudaMemcpyHostToDevice, c->st));
  const AirP<F64>& a = m->a64;
  launch_air_gather<F64>(a, o->hz0.as<double2>(), o->K.as<double2>(), 1, c->st);
  o->fft->exec(true, o->K.p, 1, CUFFT_FORWARD, c->st);
  launch_air_filter<F64>(a, o->K.as<double2>(), o->K2.as<double2>(), 1, c->st);
  o->fft->exec(true, o->K2.p, 2, CUFFT_INVERSE, c->st);
  launch_air_scatter<F64>(a, o->K2.as<double2>(), o->ghx.as<double2>(), o->ghy.as<double2>(), 1, c->st);
  CSEM_CUDA_TRY(cudaGetLastError());
  CSEM_CUDA_TRY(cudaMemcpyAsync(hx, o->ghx.p, sizeof(double2) * (size_t)(m->n1 + 1) * m->n2, cudaMemcpyDeviceToHost, c->st));
  CSEM_CUDA_TRY(cudaMemcpyAsync(hy, o->ghy.p, sizeof(double2) * (size_t)m->n1 * (m->n2 + 1), cudaMemcpyDeviceToHost, c->st));
  CSEM_CUDA_TRY(cudaStreamSynchronize(c->st));
  API_END
}

// ---------------------------------------------------------------- dots
int csem_cdot_host(long n, const double* a, const double* b, double* out)
{
  API_BEGIN return cdot_host<F64>(n, a, b, out); API_END
}
int csem_cdot_c64_host(long n, const float* a, const float* b, double* out)
{
  API_BEGIN return cdot_host<F32>(n, a, b, out); API_END
}

// ---------------------------------------------------------------- inject / extract
int csem_inject_host(csem_ctx* c, double re, double im, int nch, const int* ch, const float* src3, double* b)
{
  API_BEGIN
  Model* m = c->model;
  const size_t bytes = sizeof(double2) * (size_t)m->lE;
  ensure(c->io[0], bytes);
  ensure(c->io[2], 64 + sizeof(int) * 8);
  double2 iom = make_double2(re, im);
  char stage[64 + sizeof(int) * 8];
  memcpy(stage, src3, sizeof(float) * 3);
  memcpy(stage + 16, &iom, sizeof(iom));
  int nc = nch > 8 ? 8 : nch;
  memcpy(stage + 64, ch, sizeof(int) * nc);
  CSEM_CUDA_TRY(cudaMemcpyAsync(c->io[2].p, stage, sizeof(stage), cudaMemcpyHostToDevice, c->st));
  CSEM_CUDA_TRY(cudaMemsetAsync(c->io[0].p, 0, bytes, c->st));
  char* d = c->io[2].as<char>();
  launch_inject(m->acq, 1, (const float*)d, (const double2*)(d + 16), (const int*)(d + 64), nc, c->io[0].as<double2>(), c->st);
  CSEM_CUDA_TRY(cudaGetLastError());
  CSEM_CUDA_TRY(cudaMemcpyAsync(b, c->io[0].p, bytes, cudaMemcpyDeviceToHost, c->st));
  CSEM_CUDA_TRY(cudaStreamSynchronize(c->st));
  API_END
}

int csem_extract_host(csem_ctx* c, int nch, const int* ch, int nrec, const float* rec, const double* x, double* out)
{
  API_BEGIN
  Model* m = c->model;
  const size_t bytes = sizeof(double2) * (size_t)m->lE;
  ensure(c->io[0], bytes);
  const size_t rb = sizeof(float) * 5 * (size_t)nrec, cb = sizeof(int) * nch, ob = sizeof(double2) * (size_t)nch * nrec;
  ensure(c->io[2], rb + cb + 16);
  ensure(c->io[3], ob + 16);
  CSEM_CUDA_TRY(cudaMemcpyAsync(c->io[0].p, x, bytes, cudaMemcpyHostToDevice, c->st));
  char* d = c->io[2].as<char>();
  CSEM_CUDA_TRY(cudaMemcpyAsync(d, rec, rb, cudaMemcpyHostToDevice, c->st));
  CSEM_CUDA_TRY(cudaMemcpyAsync(d + rb, ch, cb, cudaMemcpyHostToDevice, c->st));
  launch_extract<double2>(m->acq, 1, nch, (const int*)(d + rb), nrec, (const float*)d, c->io[0].as<double2>(), m->lE,
                          nullptr, c->io[3].as<double2>(), c->st);
  CSEM_CUDA_TRY(cudaGetLastError());
  CSEM_CUDA_TRY(cudaMemcpyAsync(out, c->io[3].p, ob, cudaMemcpyDeviceToHost, c->st));
  CSEM_CUDA_TRY(cudaStreamSynchronize(c->st));
  API_END
}

// ---------------------------------------------------------------- FP64 solve
int csem_solve_fp64_host(csem_ctx* c, int algopt, int preco, int niter, double tol, int nrestart, int mp,
                         double re, double im, const double* b, double* x, double* hist, int hist_cap, int* nhist,
                         int* iters, int* status)
{
  if (algopt != 1 && algopt != 2) return csem_set_error(CSEM_EINVAL, "algopt must be 1 (BiCGStab) or 2 (GMRES)");
  if (preco < 0 || preco > 3) return csem_set_error(CSEM_EINVAL, "preco must be 0..3");
  if (algopt == 2 && nrestart < 1) return csem_set_error(CSEM_EINVAL, "nrestart must be >= 1");
  if (preco == 2 && mp < 1) return csem_set_error(CSEM_EINVAL, "mp must be >= 1");
  API_BEGIN
  Solver64* s = solver_for(c);
  const size_t bytes = sizeof(double2) * (size_t)c->model->lE;
  ensure(c->io[0], bytes);
  ensure(c->io[1], bytes);
  s->set_iom(re, im);
  CSEM_CUDA_TRY(cudaMemcpyAsync(c->io[0].p, b, bytes, cudaMemcpyHostToDevice, c->st));
  CSEM_CUDA_TRY(cudaMemcpyAsync(c->io[1].p, x, bytes, cudaMemcpyHostToDevice, c->st));
  std::vector<double> h;
  int st = ST_RUNNING, it;
  if (algopt == 1)
    it = s->fbicgstab(preco, mp, c->io[1].as<double2>(), c->io[0].as<double2>(), niter, tol, h, st, preco != 0);
  else
    it = s->gmres(preco, mp, c->io[1].as<double2>(), c->io[0].as<double2>(), niter / nrestart, tol, nrestart, h, st);
  CSEM_CUDA_TRY(cudaGetLastError());
  CSEM_CUDA_TRY(cudaMemcpyAsync(x, c->io[1].p, bytes, cudaMemcpyDeviceToHost, c->st));
  CSEM_CUDA_TRY(cudaStreamSynchronize(c->st));
  if (hist)
    for (int q = 0; q < (int)h.size() && q < hist_cap; q++) hist[q] = h[q];
  if (nhist) *nhist = (int)h.size();
  if (iters) *iters = it;
  if (status) *status = st;
  API_END
}

// ---------------------------------------------------------------- many systems
static MixedBatch* batch_for(csem_ctx* c, int nsys)
{
  if (!c->batch || c->batch->nsys != nsys) {
    delete c->batch;
    c->batch = nullptr;
    c->batch = new MixedBatch(c->model, nsys, c->st);
    configure(c, c->batch->o64);
    configure(c, c->batch->o32);
    c->batch->o64.quick_stencil = c->quick_residual;  // the defect correction's residual only
  }
  return c->batch;
}

int csem_solve_batch_host(csem_ctx* c, int nsys, const float* freq, const float* src3, int nchsrc, const int* chsrc,
                          int nchrec, const int* chrec, int nrec, const float* rec, const csem_batch_opts* opt,
                          double* dcal, int* iters, int* outer, int* status, double* relres)
{
  if (nsys < 1) return csem_set_error(CSEM_EINVAL, "nsys must be >= 1");
  if (!opt || (opt->precision != 32 && opt->precision != 64))
    return csem_set_error(CSEM_EINVAL, "precision must be 32 or 64");
  if (opt->precision == 32 && !(opt->preco == 1 || opt->preco == 3))
    return csem_set_error(CSEM_EINVAL, "the mixed-precision solver takes preco 1 (LU-SGS) or 3 (A-phi)");
  if (opt->precision == 32 && opt->algopt != 1 && opt->algopt != 2)
    return csem_set_error(CSEM_EINVAL, "algopt must be 1 (BiCGStab) or 2 (GMRES)");
  if (opt->precision == 32 && opt->algopt == 2 && (opt->nrestart < 1 || opt->nrestart > 64))
    return csem_set_error(CSEM_EINVAL, "nrestart must be in 1..64");
  if (opt->precision == 64) {  // the reference's dispatch (main.c:104-118) on one system at a time
    if (opt->algopt != 1 && opt->algopt != 2) return csem_set_error(CSEM_EINVAL, "algopt must be 1 (BiCGStab) or 2 (GMRES)");
    if (opt->preco < 0 || opt->preco > 3) return csem_set_error(CSEM_EINVAL, "preco must be 0..3");
    if (opt->algopt == 2 && opt->nrestart < 1) return csem_set_error(CSEM_EINVAL, "nrestart must be >= 1");
    if (opt->preco == 2 && opt->mp < 1) return csem_set_error(CSEM_EINVAL, "mp must be >= 1");
  }
  if (nchsrc < 1 || nchsrc > 8) return csem_set_error(CSEM_EINVAL, "1..8 source channels");
  if (!c) return csem_set_error(CSEM_EINVAL, "csem_solve_batch_host: no context");
  API_BEGIN
  std::vector<double> iom(2 * nsys), tol(nsys);
  for (int s = 0; s < nsys; s++) {
    const double pi = 3.14159265358979323846264, mu0 = 4. * pi * 1e-7;
    iom[2 * s] = 0.0;
    iom[2 * s + 1] = ((2. * pi) * (double)freq[s]) * mu0;  // main.c:95
    const float tf = opt->tol / freq[s];                        // main.c:94, in float
    tol[s] = (double)tf;
  }
  if (opt->precision == 32) {
    MixedBatch* B = batch_for(c, nsys);
    B->inject(src3, iom.data(), nchsrc, chsrc);
    MixedOptions mo;
    mo.niter = opt->niter > 0 ? opt->niter : 1000;
    mo.max_inner_total = 3 * mo.niter;
    mo.max_outer = opt->max_outer > 0 ? opt->max_outer : 30;
    mo.preco = opt->preco;
    mo.inner_tol = opt->inner_tol > 0 ? opt->inner_tol : 0.2;
    mo.check_every = opt->check_every > 0 ? opt->check_every : 4;
    mo.autotune = c->autotune;
    mo.algopt = opt->algopt;
    mo.graphs = c->graphs;
    mo.nrestart = opt->nrestart;
    std::vector<MixedResult> res;
    B->solve(iom.data(), tol.data(), mo, res);
    B->extract(nchrec, chrec, nrec, rec, dcal);
    for (int s = 0; s < nsys; s++) {
      if (iters) iters[s] = res[s].inner_iters;
      if (outer) outer[s] = res[s].outer;
      if (status) status[s] = res[s].status;
      if (relres) relres[s] = res[s].relres;
    }
  } else {
    Solver64* S = solver_for(c);
    Model* m = c->model;
    const size_t bytes = sizeof(double2) * (size_t)m->lE;
    ensure(c->io[0], bytes);
    ensure(c->io[1], bytes);
    ensure(c->io[2], 256);
    ensure(c->io[3], sizeof(double2) * (size_t)nchrec * (nrec > 0 ? nrec : 1) + sizeof(float) * 5 * (size_t)nrec +
                         sizeof(int) * (nchrec + nchsrc) + 64);
    for (int s = 0; s < nsys; s++) {
      S->set_iom(iom[2 * s], iom[2 * s + 1]);
      double2 io = make_double2(iom[2 * s], iom[2 * s + 1]);
      char stage[64 + 8 * sizeof(int)];
      memcpy(stage, src3 + 3 * s, sizeof(float) * 3);
      memcpy(stage + 16, &io, sizeof(io));
      memcpy(stage + 64, chsrc, sizeof(int) * nchsrc);
      CSEM_CUDA_TRY(cudaMemcpyAsync(c->io[2].p, stage, sizeof(stage), cudaMemcpyHostToDevice, c->st));
      CSEM_CUDA_TRY(cudaMemsetAsync(c->io[0].p, 0, bytes, c->st));
      char* d2 = c->io[2].as<char>();
      launch_inject(m->acq, 1, (const float*)d2, (const double2*)(d2 + 16), (const int*)(d2 + 64), nchsrc,
                    c->io[0].as<double2>(), c->st);
      CSEM_CUDA_TRY(cudaMemsetAsync(c->io[1].p, 0, bytes, c->st));
      std::vector<double> h;
      int st = ST_RUNNING, it;
      const int niter = opt->niter > 0 ? opt->niter : 1000;
      if (opt->algopt == 2)
        it = S->gmres(opt->preco, opt->mp, c->io[1].as<double2>(), c->io[0].as<double2>(), niter / opt->nrestart,
                      tol[s], opt->nrestart, h, st);
      else
        it = S->fbicgstab(opt->preco, opt->mp, c->io[1].as<double2>(), c->io[0].as<double2>(), niter, tol[s], h, st,
                          opt->preco != 0);
      char* d3 = c->io[3].as<char>();
      const size_t ob = sizeof(double2) * (size_t)nchrec * nrec, rb = sizeof(float) * 5 * (size_t)nrec;
      CSEM_CUDA_TRY(cudaMemcpyAsync(d3 + ob, rec, rb, cudaMemcpyHostToDevice, c->st));
      CSEM_CUDA_TRY(cudaMemcpyAsync(d3 + ob + rb, chrec, sizeof(int) * nchrec, cudaMemcpyHostToDevice, c->st));
      launch_extract<double2>(m->acq, 1, nchrec, (const int*)(d3 + ob + rb), nrec, (const float*)(d3 + ob),
                              c->io[1].as<double2>(), m->lE, nullptr, (double2*)d3, c->st);
      CSEM_CUDA_TRY(cudaGetLastError());
      CSEM_CUDA_TRY(cudaMemcpyAsync(dcal + 2 * (size_t)s * nchrec * nrec, d3, ob, cudaMemcpyDeviceToHost, c->st));
      CSEM_CUDA_TRY(cudaStreamSynchronize(c->st));
      if (iters) iters[s] = it;
      if (outer) outer[s] = 0;
      if (status) status[s] = st;
      if (relres) relres[s] = h.empty() ? 0.0 : h.back();
    }
  }
  API_END
}

// ---------------------------------------------------------------- device pointers
static int op_dev(csem_ctx* c, int which, int prec, int nsys, const double* iom, const void* x, void* y, void* stream)
{
  if (prec != 64 && prec != 32) return csem_set_error(CSEM_EINVAL, "prec must be 64 or 32");
  if (nsys < 1) return csem_set_error(CSEM_EINVAL, "nsys must be >= 1");
  upload_scal(c, nsys, iom);
  cudaStream_t user = (cudaStream_t)stream;
  if (user) {  // order after the caller's work
    cudaEvent_t ev;
    CSEM_CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    CSEM_CUDA_TRY(cudaEventRecord(ev, user));
    CSEM_CUDA_TRY(cudaStreamWaitEvent(c->st, ev, 0));
    cudaEventDestroy(ev);
  }
  if (prec == 64) {
    Ops<F64>* o = ops64_for(c, nsys);
    const SysScal<F64>* s = c->sc64.as<SysScal<F64>>();
    if (which == OP_A) o->apply_A((const double2*)x, (double2*)y, nsys, nullptr, s);
    else if (which == OP_LUSGS) o->apply_lusgs((const double2*)x, (double2*)y, nsys, nullptr, s);
    else o->apply_aphi((const double2*)x, (double2*)y, nsys, nullptr, s);
  } else {
    Ops<F32>* o = ops32_for(c, nsys);
    const SysScal<F32>* s = c->sc32.as<SysScal<F32>>();
    if (which == OP_A) o->apply_A((const float2*)x, (float2*)y, nsys, nullptr, s);
    else if (which == OP_LUSGS) {
      SweepGroups grp;
      if (o->group_size() > 1) {  // the systems of one frequency, grouped
        std::vector<int> h;
        grp.ns = o->group_size();
        grp.n = grp.ns == SPLIT_GROUP && o->split_overlap
                    ? build_sweep_groups_halves(nsys, iom, grp.ns, 4, h, &grp.nA, &grp.ngA)
                    : build_sweep_groups(nsys, iom, grp.ns, h);
        ensure(c->groups, sizeof(int) * h.size());
        // from pageable memory: staged before the call returns, so h may go
        CSEM_CUDA_TRY(cudaMemcpyAsync(c->groups.p, h.data(), sizeof(int) * h.size(), cudaMemcpyHostToDevice, c->st));
        grp.dev = c->groups.as<int>();
      }
      o->apply_lusgs((const float2*)x, (float2*)y, nsys, nullptr, s, false, &grp);
    } else o->apply_aphi((const float2*)x, (float2*)y, nsys, nullptr, s);
  }
  CSEM_CUDA_TRY(cudaGetLastError());
  if (user) {
    cudaEvent_t ev;
    CSEM_CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    CSEM_CUDA_TRY(cudaEventRecord(ev, c->st));
    CSEM_CUDA_TRY(cudaStreamWaitEvent(user, ev, 0));
    cudaEventDestroy(ev);
  }
  return CSEM_OK;
}

int csem_fdfd_apply_dev(csem_ctx* c, int prec, int nsys, const double* iom, const void* x, void* y, void* stream)
{
  API_BEGIN return op_dev(c, OP_A, prec, nsys, iom, x, y, stream); API_END
}
int csem_lusgs_apply_dev(csem_ctx* c, int prec, int nsys, const double* iom, const void* x, void* y, void* stream)
{
  API_BEGIN return op_dev(c, OP_LUSGS, prec, nsys, iom, x, y, stream); API_END
}
int csem_aphi_apply_dev(csem_ctx* c, int prec, int nsys, const double* iom, const void* x, void* y, void* stream)
{
  API_BEGIN return op_dev(c, OP_APHI, prec, nsys, iom, x, y, stream); API_END
}

int csem_csr_compare(csem_ctx* c, int prec, double iom_re, double iom_im, int nrep, double* out)
{
  if (prec != 64 && prec != 32) return csem_set_error(CSEM_EINVAL, "prec must be 64 or 32");
  if (nrep < 1) return csem_set_error(CSEM_EINVAL, "nrep must be >= 1");
  if (c->model->airbc)
    return csem_set_error(CSEM_EINVAL, "the assembled operator has no airwave coupling: airbc=0 only (as Acsr.c)");
  if ((double)c->model->lE * 13 > 2147483647.0)
    return csem_set_error(CSEM_ETOOBIG, "more than 2^31 stored entries: 32-bit CSR indices do not reach");
  API_BEGIN
  csr_compare(c->model, c->st, prec, iom_re, iom_im, nrep, out);
  API_END
}

static constexpr int kMaxDotDevices = 64;

int csem_cdot_dev(int prec, long n, int nsys, const void* a, const void* b, double* out_dev, void* stream)
{
  if (prec != 64 && prec != 32) return csem_set_error(CSEM_EINVAL, "prec must be 64 or 32");
  if (n < 1 || nsys < 1) return csem_set_error(CSEM_EINVAL, "csem_cdot_dev: n and nsys must be positive");
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return csem_set_error(CSEM_ENODEV, "no CUDA device available");
  if (dev >= kMaxDotDevices) return csem_set_error(CSEM_EINVAL, "csem_cdot_dev: device %d beyond the %d supported", dev,
                                                   kMaxDotDevices);
  API_BEGIN
  const int nblk = dot_blocks(n);
  // one partial-sum buffer per host thread and device: a buffer is only ever handed to
  // kernels on the device it was allocated on
  static thread_local DevBuf part[kMaxDotDevices];
  ensure(part[dev], sizeof(double2) * (size_t)nblk * nsys);
  if (prec == 64)
    launch_dot<F64>((const double2*)a, (const double2*)b, n, n, nsys, nullptr, part[dev].as<double2>(), nblk,
                    (double2*)out_dev, (cudaStream_t)stream);
  else
    launch_dot<F32>((const float2*)a, (const float2*)b, n, n, nsys, nullptr, part[dev].as<double2>(), nblk,
                    (double2*)out_dev, (cudaStream_t)stream);
  CSEM_CUDA_TRY(cudaGetLastError());
  API_END
}

}  // extern "C"
