// Model upload, airwave FFT plans, and the operator / preconditioner pipelines.
#include <cmath>
#include <cstring>
#include <map>
#include <utility>
#include <vector>
#include "engine_model.h"
#include "prof.h"
#include "../../include/csem_host.h"

namespace csem {

void DevBuf::alloc(size_t b)
{
  free_();
  if (b == 0) b = 16;
  CSEM_CUDA_TRY(cudaMalloc(&p, b));
  bytes = b;
}
void DevBuf::free_()
{
  if (p) cudaFree(p);
  p = nullptr;
  bytes = 0;
}

template <class T> static void upload(DevBuf& buf, const std::vector<T>& v)
{
  buf.alloc(sizeof(T) * v.size());
  CSEM_CUDA_TRY(cudaMemcpy(buf.p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice));
}

Model::Model(const csem_grid* gp, int airbc_, int fvm_)
{
  const csem_grid_t& G = *(const csem_grid_t*)gp;
  n1 = G.n1;
  n2 = G.n2;
  n3f = G.n3;
  nb = G.nb;
  nz = G.nz;
  airbc = airbc_;
  fvm = fvm_;
  n3 = airbc ? nz + nb : n3f;
  lEx = (long)n1 * (n2 + 1) * (n3 + 1);
  lEy = (long)(n1 + 1) * n2 * (n3 + 1);
  lEz = (long)(n1 + 1) * (n2 + 1) * n3;
  lE = lEx + lEy + lEz;
  lv = (long)(n1 + 1) * (n2 + 1) * (n3 + 1);
  rho_water = G.rho_water;

  // 1-D spacings and their reciprocals: 12 arrays, each padded to a common length
  const int L = std::max(n1, std::max(n2, n3f)) + 1;
  const double* src[6] = {G.d1, G.d2, G.d3, G.d1s, G.d2s, G.d3s};
  const int len[6] = {n1 + 1, n2 + 1, n3f + 1, n1 + 1, n2 + 1, n3f + 1};
  std::vector<double> h64((size_t)12 * L, 0.0);
  std::vector<float> h32((size_t)12 * L, 0.f);
  for (int a = 0; a < 6; a++)
    for (int q = 0; q < len[a]; q++) {
      h64[(size_t)a * L + q] = src[a][q];
      h64[(size_t)(a + 6) * L + q] = 1.0 / src[a][q];
      h32[(size_t)a * L + q] = (float)src[a][q];
      h32[(size_t)(a + 6) * L + q] = (float)(1.0 / src[a][q]);
    }
  upload(d64, h64);
  upload(d32, h32);
  const long ls[3] = {(long)n1 * (n2 + 1) * (n3f + 1), (long)(n1 + 1) * n2 * (n3f + 1), (long)(n1 + 1) * (n2 + 1) * n3f};
  const double* sg[3] = {G.sigma11, G.sigma22, G.sigma33};
  std::vector<double> s64h;
  std::vector<float> s32h;
  for (int c = 0; c < 3; c++)
    for (long q = 0; q < ls[c]; q++) {
      s64h.push_back(sg[c][q]);
      s32h.push_back((float)sg[c][q]);
    }
  upload(s64, s64h);
  upload(s32, s32h);
  std::vector<double> xh((size_t)6 * L, 0.0);
  const double* xs[6] = {G.x1, G.x2, G.x3, G.x1s, G.x2s, G.x3s};
  for (int a = 0; a < 6; a++)
    for (int q = 0; q < len[a % 3]; q++) xh[(size_t)a * L + q] = xs[a][q];
  upload(x64, xh);

  auto fill = [&](auto& g, auto* dbase, auto* sbase) {
    g.n1 = n1; g.n2 = n2; g.n3 = n3; g.n3f = n3f; g.nb = nb; g.airbc = airbc; g.fvm = fvm;
    g.kstart = airbc ? nb : 0;
    g.lEx = lEx; g.lEy = lEy; g.lEz = lEz; g.lE = lE;
    g.d1 = dbase; g.d2 = dbase + L; g.d3 = dbase + 2 * L;
    g.d1s = dbase + 3 * L; g.d2s = dbase + 4 * L; g.d3s = dbase + 5 * L;
    g.r1 = dbase + 6 * L; g.r2 = dbase + 7 * L; g.r3 = dbase + 8 * L;
    g.r1s = dbase + 9 * L; g.r2s = dbase + 10 * L; g.r3s = dbase + 11 * L;
    g.s11 = sbase; g.s22 = sbase + ls[0]; g.s33 = sbase + ls[0] + ls[1];
  };
  fill(g64, d64.as<double>(), s64.as<double>());
  fill(g32, d32.as<float>(), s32.as<float>());

  acq.n1 = n1; acq.n2 = n2; acq.n3f = n3f; acq.nb = nb; acq.airbc = airbc; acq.fvm = fvm;
  acq.lEx = lEx; acq.lEy = lEy; acq.lE = lE;
  const double* xd = x64.as<double>();
  acq.x1 = xd; acq.x2 = xd + L; acq.x3 = xd + 2 * L; acq.x1s = xd + 3 * L; acq.x2s = xd + 4 * L; acq.x3s = xd + 5 * L;
  acq.s11 = g64.s11; acq.s22 = g64.s22; acq.s33 = g64.s33;
  acq.rho_water = rho_water;
  acq.fix_src_sigma = 0;

  memset(&a64, 0, sizeof(a64));
  memset(&a32, 0, sizeof(a32));
  if (airbc) {
    N1 = G.n1fft;
    N2 = G.n2fft;
    fft_plans.N1 = N1;
    fft_plans.N2 = N2;
    // gather tables (airbc_init_free.c:90-105), -1 where the reference writes zero
    std::vector<int> ih;  // jx[N1], jy[N2], hx_j1[n1+1], hx_j2[n2], hy_j1[n1], hy_j2[n2+1]
    std::vector<double> wh;
    for (int i1 = 0; i1 < N1; i1++) {
      double x1 = G.x1s[0] + i1 * G.d1fft;
      bool in = x1 < G.x1s[n1 - 1];
      ih.push_back(in ? G.jx[i1] : -1);
      wh.push_back(in ? G.wx[i1] : 0.0);
    }
    for (int i2 = 0; i2 < N2; i2++) {
      double x2 = G.x2s[0] + i2 * G.d2fft;
      bool in = x2 < G.x2s[n2 - 1];
      ih.push_back(in ? G.jy[i2] : -1);
      wh.push_back(in ? G.wy[i2] : 0.0);
    }
    // back-interpolation (airbc_init_free.c:168-207)
    auto back = [&](const double* x, int n, double dfft) {
      for (int q = 0; q < n; q++) {
        double s = x[q] - x[0];
        int j = (int)(s / dfft);
        double w = s / dfft - j;
        ih.push_back(j);
        wh.push_back(w);
      }
    };
    back(G.x1, n1 + 1, G.d1fft);
    back(G.x2s, n2, G.d2fft);
    back(G.x1s, n1, G.d1fft);
    back(G.x2, n2 + 1, G.d2fft);
    upload(air_i, ih);
    upload(air_w64, wh);
    std::vector<float> wf(wh.begin(), wh.end());
    upload(air_w32, wf);
    const long NN = (long)N1 * N2;
    std::vector<double2> f64((size_t)2 * NN);
    std::vector<float2> f32((size_t)2 * NN);
    for (long q = 0; q < NN; q++) {
      f64[q] = make_double2(G.sH1[2 * q], G.sH1[2 * q + 1]);
      f64[NN + q] = make_double2(G.sH2[2 * q], G.sH2[2 * q + 1]);
      f32[q] = make_float2((float)G.sH1[2 * q], (float)G.sH1[2 * q + 1]);
      f32[NN + q] = make_float2((float)G.sH2[2 * q], (float)G.sH2[2 * q + 1]);
    }
    upload(sH64, f64);
    upload(sH32, f32);
    auto afill = [&](auto& a, auto* w, auto* sh) {
      const int* iv = air_i.as<int>();
      a.n1 = n1; a.n2 = n2; a.N1 = N1; a.N2 = N2;
      a.jx = iv; a.jy = iv + N1;
      a.hx_j1 = iv + N1 + N2; a.hx_j2 = a.hx_j1 + n1 + 1;
      a.hy_j1 = a.hx_j2 + n2; a.hy_j2 = a.hy_j1 + n1;
      a.wx = w; a.wy = w + N1;
      a.hx_w1 = w + N1 + N2; a.hx_w2 = a.hx_w1 + n1 + 1;
      a.hy_w1 = a.hx_w2 + n2; a.hy_w2 = a.hy_w1 + n1;
      a.sH1 = sh; a.sH2 = sh + NN;
    };
    afill(a64, air_w64.as<double>(), sH64.as<double2>());
    afill(a32, air_w32.as<float>(), sH32.as<float2>());
  }
}

Model::~Model() {}

template <> const GridP<F64>& Model::grid<F64>() const { return g64; }
template <> const GridP<F32>& Model::grid<F32>() const { return g32; }
template <> const AirP<F64>& Model::air<F64>() const { return a64; }
template <> const AirP<F32>& Model::air<F32>() const { return a32; }

template <class P> GridP<P> Model::grid_shifted() const
{
  GridP<P> g = grid<P>();
  const int ks = g.kstart;
  g.d3 += ks; g.d3s += ks; g.r3 += ks; g.r3s += ks;
  g.s11 += (long)ks * n1 * (n2 + 1);
  g.s22 += (long)ks * (n1 + 1) * n2;
  g.s33 += (long)ks * (n1 + 1) * (n2 + 1);
  g.kstart = 0;
  return g;
}
template GridP<F64> Model::grid_shifted<F64>() const;
template GridP<F32> Model::grid_shifted<F32>() const;

// ------------------------------------------------------------------ FFT plans
FftPlans::~FftPlans()
{
  for (auto h : z) if (h) cufftDestroy(h);
  for (auto h : c) if (h) cufftDestroy(h);
}

void FftPlans::exec(bool dbl, void* data, int count, int dir, cudaStream_t st)
{
  const size_t NN = (size_t)N1 * N2;
  size_t off = 0;
  while (count > 0) {
    int lg = 0;
    while ((2 << lg) <= count && lg < 7) lg++;
    const int b = 1 << lg;
    std::vector<cufftHandle>& v = dbl ? z : c;
    if ((int)v.size() <= lg) v.resize(lg + 1, 0);
    if (!v[lg]) {
      int n[2] = {N1, N2};
      cufftHandle h;
      if (cufftPlanMany(&h, 2, n, nullptr, 1, (int)NN, nullptr, 1, (int)NN, dbl ? CUFFT_Z2Z : CUFFT_C2C, b) !=
          CUFFT_SUCCESS)
        throw CudaError(cudaErrorMemoryAllocation, "cufftPlanMany", __FILE__, __LINE__);
      v[lg] = h;
    }
    cufftSetStream(v[lg], st);
    cufftResult r;
    if (dbl) {
      cufftDoubleComplex* p = (cufftDoubleComplex*)data + off;
      r = cufftExecZ2Z(v[lg], p, p, dir);
    } else {
      cufftComplex* p = (cufftComplex*)data + off;
      r = cufftExecC2C(v[lg], p, p, dir);
    }
    if (r != CUFFT_SUCCESS) throw CudaError(cudaErrorLaunchFailure, "cufftExec", __FILE__, __LINE__);
    off += (size_t)b * NN;
    count -= b;
  }
}

SysScal<F64> sys_scal64(double iom_re, double iom_im)
{
  // 1/(I omega mu0) as the reference computes it (fdfd.c:100): real over complex,
  // i.e. (1+0i)/z by Smith's method on the host
  SysScal<F64> s;
  s.iom = make_double2(iom_re, iom_im);
  double a = 1.0, b = 0.0, c = iom_re, d = iom_im, x, y;
  if (std::fabs(c) < std::fabs(d)) {
    double r = c / d, den = c * r + d;
    x = (a * r + b) / den;
    y = (b * r - a) / den;
  } else {
    double r = d / c, den = d * r + c;
    x = (b * r + a) / den;
    y = (b - a * r) / den;
  }
  s.iwmu = make_double2(x, y);
  return s;
}

SysScal<F32> sys_scal32(const SysScal<F64>& s)
{
  SysScal<F32> f;
  f.iom = make_float2((float)s.iom.x, (float)s.iom.y);
  f.iwmu = make_float2((float)s.iwmu.x, (float)s.iwmu.y);
  return f;
}

// ------------------------------------------------------------------ Ops
template <class C>
__global__ void k_zero_slots(C* Y, long n, const int* sys_list)
{
  const int slot = blockIdx.y;
  const int sys = sys_list ? sys_list[slot] : slot;
  const long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n) {
    C z;
    z.x = 0;
    z.y = 0;
    Y[(size_t)sys * n + q] = z;
  }
}

template <class P>
Ops<P>::Ops(Model* m_, int nslot_max, cudaStream_t st_) : m(m_), nmax(nslot_max), st(st_), fft(nullptr)
{
  const size_t cs = sizeof(C);
  if (m->airbc) {
    hz0.alloc(cs * (size_t)m->n1 * m->n2 * nmax);
    K.alloc(cs * (size_t)m->N1 * m->N2 * nmax);
    K2.alloc(cs * (size_t)m->N1 * m->N2 * nmax * 2);
    ghx.alloc(cs * (size_t)(m->n1 + 1) * m->n2 * nmax);
    ghy.alloc(cs * (size_t)m->n1 * (m->n2 + 1) * nmax);
    const long capE = (long)m->nb * ((long)m->n1 * (m->n2 + 1) + (long)(m->n1 + 1) * m->n2 + (long)(m->n1 + 1) * (m->n2 + 1));
    cap.alloc(cs * (size_t)capE * nmax);
    CSEM_CUDA_TRY(cudaMemsetAsync(cap.p, 0, cap.bytes, st));  // its boundary planes stay zero
    fft = &m->fft_plans;
  }
  if (!P::exact) {  // the second stream of the overlapped split sweeps (created outside any capture)
    CSEM_CUDA_TRY(cudaStreamCreateWithFlags(&aux, cudaStreamNonBlocking));
    CSEM_CUDA_TRY(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
    CSEM_CUDA_TRY(cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming));
  }
}

template <class P> Ops<P>::~Ops()
{
  if (ev_fork) cudaEventDestroy(ev_fork);
  if (ev_join) cudaEventDestroy(ev_join);
  if (aux) cudaStreamDestroy(aux);
}

template <class P> int Ops<P>::split_ctas() const { return split_cap > 0 ? split_cap * sm_count() : 0; }

template <class P>
void Ops<P>::zero(C* Y, long n, int nslot, const int* sys_list)
{
  dim3 grd((unsigned)((n + 255) / 256), nslot);
  count_launch(), k_zero_slots<C><<<grd, 256, 0, st>>>(Y, n, sys_list);
}

template <class P>
bool Ops<P>::apply_A(const C* X, C* Y, int nslot, const int* sys_list, const SysScal<P>* sc, const DotEpi<P>* epi)
{
  ProfScope whole(P::exact ? PROF_A64 : PROF_A32, st, nslot);
  const GridP<P>& g = m->grid<P>();
  const C* ghxp = nullptr;
  const C* ghyp = nullptr;
  if (m->airbc) {
    const AirP<P>& a = m->air<P>();
    ProfScope air(P::exact ? PROF_AIR64 : PROF_AIR32, st, nslot);
    launch_hz0<P>(g, sc, X, hz0.as<C>(), nslot, sys_list, st);
    launch_air_gather<P>(a, hz0.as<C>(), K.as<C>(), nslot, st);
    fft->exec(P::exact, K.p, nslot, CUFFT_FORWARD, st);
    launch_air_filter<P>(a, K.as<C>(), K2.as<C>(), nslot, st);
    fft->exec(P::exact, K2.p, 2 * nslot, CUFFT_INVERSE, st);
    launch_air_scatter<P>(a, K2.as<C>(), ghx.as<C>(), ghy.as<C>(), nslot, st);
    ghxp = ghx.as<C>();
    ghyp = ghy.as<C>();
  }
  ProfScope sten(P::exact ? PROF_STENCIL64 : PROF_STENCIL32, st, nslot);
  if constexpr (!P::exact) {
    // the dot products folded into the stencil where its partials fit the caller's buffer
    if (epi && epi->kind && fused_dots &&
        fdfd_partials(g.n1, g.n2, g.n3, nslot, stencil_by, stencil_ctas) <= epi->cap) {
      const int np = fdfd_partials(g.n1, g.n2, g.n3, nslot, stencil_by, stencil_ctas);
      launch_fdfd_dot(g, sc, X, Y, ghxp, ghyp, nslot, sys_list, st, stencil_by, stencil_ctas, epi->kind, epi->e,
                      epi->partial);
      launch_dot_finish(epi->partial, np, nslot, epi->out1, epi->kind == 2 ? epi->out2 : nullptr, st);
      return true;
    }
  }
  if constexpr (P::exact) {
    if (quick_stencil) {
      launch_fdfd<F64Q>(grid_as<F64Q>(g), reinterpret_cast<const SysScal<F64Q>*>(sc), X, Y, ghxp, ghyp, nslot,
                        sys_list, st, stencil_by, stencil_ctas);
      return false;
    }
  }
  launch_fdfd<P>(g, sc, X, Y, ghxp, ghyp, nslot, sys_list, st, stencil_by, stencil_ctas);
  return false;
}

int build_sweep_groups(int nslot, const double* iom_of_slot, int ns, std::vector<int>& out)
{
  out.clear();
  if (ns < 1) ns = 1;
  std::vector<char> taken((size_t)nslot, 0);
  int ng = 0;
  for (int a = 0; a < nslot; a++) {
    if (taken[a]) continue;
    int q = 0;
    for (int b = a; b < nslot; b++) {
      if (taken[b] || iom_of_slot[2 * b] != iom_of_slot[2 * a] || iom_of_slot[2 * b + 1] != iom_of_slot[2 * a + 1])
        continue;
      if (q == 0) {
        out.resize(out.size() + ns, -1);
        ng++;
      }
      out[(size_t)(ng - 1) * ns + q] = b;
      taken[b] = 1;
      if (++q == ns) q = 0;
    }
  }
  return ng;
}

int build_sweep_groups_halves(int nslot, const double* iom_of_slot, int ns, int min_half, std::vector<int>& out,
                              int* nA, int* ngA)
{
  *nA = *ngA = 0;
  if (min_half < 1 || nslot < 2 * min_half) return build_sweep_groups(nslot, iom_of_slot, ns, out);
  const int a = nslot / 2;
  std::vector<int> g2;
  const int na = build_sweep_groups(a, iom_of_slot, ns, out);
  const int nb = build_sweep_groups(nslot - a, iom_of_slot + 2 * (size_t)a, ns, g2);
  out.insert(out.end(), g2.begin(), g2.end());
  *nA = a;
  *ngA = na;
  return na + nb;
}

template <class P>
void Ops<P>::apply_lusgs(const C* X, C* Y, int nslot, const int* sys_list, const SysScal<P>* sc, bool bounds_zero,
                         const SweepGroups* grp)
{
  ProfScope prof(P::exact ? PROF_LUSGS64 : PROF_LUSGS32, st, nslot);
  SweepP<P> s;
  memset(&s, 0, sizeof(s));
  s.g = m->grid<P>();
  s.nK = m->airbc ? m->n3f : m->n3;
  s.vshift = m->airbc ? m->nb : 0;
  s.X = X;
  s.Y = Y;
  s.scal = sc;
  s.sys_list = sys_list;
  const int n1 = m->n1, n2 = m->n2, nb = m->nb;
  if (m->airbc) {
    s.CAP = cap.as<C>();
    s.capEx = (long)nb * n1 * (n2 + 1);
    s.capEy = (long)nb * (n1 + 1) * n2;
    s.capE = s.capEx + s.capEy + (long)nb * (n1 + 1) * (n2 + 1);
    if (!bounds_zero) CSEM_CUDA_TRY(cudaMemsetAsync(cap.p, 0, sizeof(C) * (size_t)s.capE * nslot, st));
  }
  if (!bounds_zero) zero(Y, m->lE, nslot, sys_list);
  if constexpr (!P::exact) {
    // split sweeps on two halves of the slots, one per stream, the second starting once the
    // first half's first pass is queued: a half's passes (HBM-bound) then run while the
    // other half's pipelines (hand-over-bound) do
    const bool all_fit = sweep_pipelined_fits(0, n1, n2, s.nK) && sweep_pipelined_fits(1, n1, n2, s.nK) &&
                         sweep_pipelined_fits(2, n1, n2, s.nK);
    if (split_sweeps && split_overlap && pipelined_sweeps && !tiled_sweeps && all_fit && aux && grp &&
        grp->ns == SPLIT_GROUP && grp->nA > 0 && grp->nA < nslot && grp->ngA > 0 && grp->ngA < grp->n) {
      const long sbs = sweep_split_scratch(n1, n2, s.nK);
      if (sb.bytes < sizeof(float4) * (size_t)sbs * nmax) sb.alloc(sizeof(float4) * (size_t)sbs * nmax);
      const int nA = grp->nA, nB = nslot - nA, vw = sweep_vw == 1 || sweep_vw == 4 ? sweep_vw : 2;
      SweepP<P> sB = s;
      if (s.sys_list) {
        sB.sys_list = s.sys_list + nA;
      } else {  // slot = system: the second half's systems start nA systems in
        sB.X = s.X + (size_t)nA * m->lE;
        sB.Y = s.Y + (size_t)nA * m->lE;
        sB.scal = s.scal + nA;
      }
      if (s.CAP) sB.CAP = s.CAP + (size_t)nA * s.capE;
      float4* SA = sb.as<float4>();
      float4* SBh = SA + (size_t)nA * sbs;
      const int* gA = grp->dev;
      const int* gB = grp->dev + (size_t)grp->ngA * grp->ns;
      const int cap = split_ctas();
      static const int order[6][2] = {{0, 1}, {1, 1}, {2, 1}, {2, 0}, {1, 0}, {0, 0}};
      for (int q = 0; q < 6; q++) {
        const int comp = order[q][0];
        const bool fwd = order[q][1] != 0;
        launch_split_prep(s, comp, fwd, nA, SA, sbs, gA, grp->ngA, grp->ns, st);
        if (q == 0) {
          CSEM_CUDA_TRY(cudaEventRecord(ev_fork, st));
          CSEM_CUDA_TRY(cudaStreamWaitEvent(aux, ev_fork, 0));
        }
        launch_split_sweep(s, comp, fwd, nA, SA, sbs, vw, cap, st);
        launch_split_prep(sB, comp, fwd, nB, SBh, sbs, gB, grp->n - grp->ngA, grp->ns, aux);
        launch_split_sweep(sB, comp, fwd, nB, SBh, sbs, vw, cap, aux);
      }
      CSEM_CUDA_TRY(cudaEventRecord(ev_join, aux));
      CSEM_CUDA_TRY(cudaStreamWaitEvent(st, ev_join, 0));
      return;
    }
  }
  // both schedules visit the points of a sweep in an order that respects every
  // dependency of the lexicographic sweep, so they may be mixed sweep by sweep
  auto sweep = [&](int comp, bool fwd) {
    if constexpr (!P::exact) {
      if (tiled_sweeps && sweep_tiled_fits(comp, n1, n2, s.nK, tile_rows, tile_vw)) {
        launch_sweep_tiled(s, comp, fwd, nslot, st, tile_rows, tile_vw);
        return;
      }
      if (split_sweeps && pipelined_sweeps && sweep_pipelined_fits(comp, n1, n2, s.nK)) {
        const long sbs = sweep_split_scratch(n1, n2, s.nK);
        if (sb.bytes < sizeof(float4) * (size_t)sbs * nmax) sb.alloc(sizeof(float4) * (size_t)sbs * nmax);
        // groups built as two halves number their slots within each half: here, on one
        // stream, the pass then takes the slots one by one
        const bool g16 = grp && grp->ns == SPLIT_GROUP && grp->n > 0 && grp->nA == 0;
        launch_sweep_split(s, comp, fwd, nslot, sb.as<float4>(), sbs, sweep_vw == 1 || sweep_vw == 4 ? sweep_vw : 2,
                           g16 ? grp->dev : nullptr, g16 ? grp->n : 0, g16 ? grp->ns : 1, st);
        return;
      }
      if (grp && (grp->ns == 2 || grp->ns == 4) && grp->n > 0 && pipelined_sweeps &&
          sweep_grouped_fits(comp, n1, n2, s.nK)) {
        launch_sweep_grouped(s, comp, fwd, grp->dev, grp->n, grp->ns, sweep_vw == 2 && grp->ns == 2 ? 2 : 1, st);
        return;
      }
    }
    if (pipelined_sweeps && sweep_pipelined_fits(comp, n1, n2, s.nK)) {
      launch_sweep_pipelined<P>(s, comp, fwd, nslot, st, sweep_vw, sweep_lines);
      return;
    }
    const int nd = sweep_diagonals(comp, n1, n2, s.nK);
    if (fwd)
      for (int t = 2; t < 2 + nd; t++) launch_sweep<P>(s, comp, true, false, t, nslot, st);
    else
      for (int t = 1 + nd; t >= 2; t--) launch_sweep<P>(s, comp, false, false, t, nslot, st);
  };
  for (int comp = 0; comp < 3; comp++) sweep(comp, true);
  for (int comp = 2; comp >= 0; comp--) sweep(comp, false);
}

template <class P>
void Ops<P>::apply_aphi(const C* X, C* Y, int nslot, const int* sys_list, const SysScal<P>* sc)
{
  ProfScope prof(P::exact ? PROF_APHI64 : PROF_APHI32, st, nslot);
  if (!V.p) {
    V.alloc(sizeof(C) * (size_t)m->lv * nmax);
    BV.alloc(sizeof(C) * (size_t)m->lv * nmax);
  }
  SweepP<P> s;
  memset(&s, 0, sizeof(s));
  s.g = m->grid_shifted<P>();
  s.nK = m->n3;
  s.vshift = 0;
  s.X = X;
  s.Y = Y;
  s.scal = sc;
  s.sys_list = sys_list;
  s.V = V.as<C>();
  s.BV = BV.as<C>();
  s.lv = m->lv;
  const GridP<P>& gu = m->grid<P>();
  s.s11u = gu.s11;
  s.s22u = gu.s22;
  s.s33u = gu.s33;
  s.aphi_fix = aphi_fix ? 1 : 0;
  const int n1 = m->n1, n2 = m->n2, n3 = m->n3;
  zero(Y, m->lE, nslot, sys_list);
  launch_aphi_div<P>(s, BV.as<C>(), nslot, st);
  CSEM_CUDA_TRY(cudaMemsetAsync(V.p, 0, sizeof(C) * (size_t)m->lv * nslot, st));
  for (int comp = 0; comp < 3; comp++) {
    const int nd = sweep_diagonals(comp, n1, n2, n3);
    for (int t = 2; t < 2 + nd; t++) launch_sweep<P>(s, comp, true, true, t, nslot, st);
  }
  const int np = phi_diagonals(n1, n2, n3);
  for (int t = 3; t < 3 + np; t++) launch_aphi_phi<P>(s, V.as<C>(), t, nslot, st);
  for (int t = 2 + np; t >= 3; t--) launch_aphi_phi<P>(s, V.as<C>(), -t, nslot, st);
  for (int comp = 2; comp >= 0; comp--) {
    const int nd = sweep_diagonals(comp, n1, n2, n3);
    for (int t = 1 + nd; t >= 2; t--) launch_sweep<P>(s, comp, false, true, t, nslot, st);
  }
  launch_aphi_grad<P>(s, V.as<C>(), nslot, st);
}

template class Ops<F64>;
template class Ops<F32>;

}  // namespace csem
