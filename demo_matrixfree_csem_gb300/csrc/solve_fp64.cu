// Plain complex128 Krylov solvers with every vector resident on the GPU.
//
//  fbicgstab (solver.c:93-178) / bicgstab (solver.c:16-87): the vector work, dot
//  products and scalar recurrences all run on the device; the host only reads the
//  status word once per iteration.
//  gmres (solver.c:181-285) / fgmres (solver.c:403-512) / the inner GMRES(mp)
//  preconditioner (gmres_init_free.c:58-137): vectors and dots on the device, the
//  (m+1) x m Hessenberg/Givens algebra on the host in the reference's order.
// Scalar arithmetic follows the reference's C complex semantics exactly (products
// (ac-bd, ad+bc), Smith quotients), so the only departure from the reference's rounding
// is the summation order inside the dot products.
#include <cmath>
#include <cstring>
#include "solve_fp64.h"

namespace csem {

namespace {
struct hz {
  double re, im;
};
inline hz H(double a, double b) { return hz{a, b}; }
inline hz hadd(hz a, hz b) { return H(a.re + b.re, a.im + b.im); }
inline hz hsub(hz a, hz b) { return H(a.re - b.re, a.im - b.im); }
inline hz hmul(hz a, hz b) { return H(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re); }
inline hz hrmul(double s, hz a) { return H(s * a.re, s * a.im); }
inline hz hdivr(hz a, double d) { return H(a.re / d, a.im / d); }
inline hz hconj(hz a) { return H(a.re, -a.im); }
inline hz hdiv(hz a, hz b)
{
  if (std::fabs(b.re) < std::fabs(b.im)) {
    double r = b.re / b.im, den = b.re * r + b.im;
    return H((a.re * r + a.im) / den, (a.im * r - a.re) / den);
  }
  double r = b.im / b.re, den = b.im * r + b.re;
  return H((a.im * r + a.re) / den, (a.im - a.re * r) / den);
}
inline double habs(hz a) { return std::hypot(a.re, a.im); }
inline double2 D(hz a) { return make_double2(a.re, a.im); }
inline hz Hd(double2 a) { return H(a.x, a.y); }
}  // namespace

Solver64::Solver64(Model* m_, cudaStream_t st_) : m(m_), st(st_), ops(m_, 1, st_)
{
  n = m->lE;
  nblk = dot_blocks(n);
  scal.alloc(sizeof(SysScal<F64>));
  ks.alloc(sizeof(KrylovScalars));
  dots.alloc(sizeof(double2) * 16);
  partial.alloc(sizeof(double2) * nblk * 16);
  coef.alloc(sizeof(double2) * 128);
  hist.alloc(sizeof(double) * 8);
}

void Solver64::set_iom(double re, double im)
{
  SysScal<F64> s = sys_scal64(re, im);
  iom_h = s.iom;
  CSEM_CUDA_TRY(cudaMemcpyAsync(scal.p, &s, sizeof(s), cudaMemcpyHostToDevice, st));
}

void Solver64::ensure_work(int count)
{
  if (count <= nwork) return;
  work.alloc(sizeof(double2) * (size_t)n * count);
  nwork = count;
}

double2* Solver64::W(int i) { return work.as<double2>() + (size_t)i * n; }

void Solver64::A(const double2* x, double2* y) { ops.apply_A(x, y, 1, nullptr, scal.as<SysScal<F64>>()); }

void Solver64::M(int precond, int mp, const double2* x, double2* y)
{
  if (precond == PRE_LUSGS) ops.apply_lusgs(x, y, 1, nullptr, scal.as<SysScal<F64>>());
  else if (precond == PRE_APHI) ops.apply_aphi(x, y, 1, nullptr, scal.as<SysScal<F64>>());
  else if (precond == PRE_GMRES) gmres_pre(mp, x, y);
  else CSEM_CUDA_TRY(cudaMemcpyAsync(y, x, sizeof(double2) * n, cudaMemcpyDeviceToDevice, st));
}

void Solver64::dot_async(const double2* a, const double2* b, int slot_out)
{
  if (seq_dots) {
    launch_dot_seq(a, b, n, dots.as<double2>() + slot_out, st);
    return;
  }
  launch_dot<F64>(a, b, n, n, 1, nullptr, partial.as<double2>() + (size_t)slot_out * nblk, nblk,
                  dots.as<double2>() + slot_out, st);
}

double2 Solver64::dot(const double2* a, const double2* b)
{
  dot_async(a, b, 15);
  double2 r;
  CSEM_CUDA_TRY(cudaMemcpyAsync(&r, dots.as<double2>() + 15, sizeof(r), cudaMemcpyDeviceToHost, st));
  CSEM_CUDA_TRY(cudaStreamSynchronize(st));
  return r;
}

int Solver64::fbicgstab(int precond, int mp, double2* x, const double2* b, int niter, double tol,
                        std::vector<double>& hh, int& status, bool flexible)
{
  ensure_work(7);
  double2 *r = W(0), *r0 = W(1), *p = W(2), *pp = W(3), *v = W(4), *s = W(5), *t = W(6);
  KrylovScalars* K = ks.as<KrylovScalars>();
  double2* d = dots.as<double2>();
  const int hcap = niter + 2;
  if ((size_t)hcap * sizeof(double) > hist.bytes) hist.alloc(sizeof(double) * hcap);
  KrylovScalars k0;
  memset(&k0, 0, sizeof(k0));
  k0.tol = tol;
  CSEM_CUDA_TRY(cudaMemcpyAsync(K, &k0, sizeof(k0), cudaMemcpyHostToDevice, st));
  A(x, v);
  launch_vec<F64>(VEC_INIT, n, 1, nullptr, K, (double2*)b, v, r, p, r0, st);
  dot_async(r, r0, 0);
  dot_async(r, r, 1);
  launch_sc_init(1, nullptr, K, d + 0, d + 1, hist.as<double>(), hcap, st);
  KrylovScalars kh;
  CSEM_CUDA_TRY(cudaMemcpyAsync(&kh, K, sizeof(kh), cudaMemcpyDeviceToHost, st));
  CSEM_CUDA_TRY(cudaStreamSynchronize(st));
  if (kh.status == ST_RUNNING && niter <= 0) kh.status = ST_MAXITER;
  while (kh.status == ST_RUNNING) {
    if (flexible) {
      M(precond, mp, p, pp);
      A(pp, v);
    } else {
      A(p, v);
    }
    dot_async(v, r0, 2);
    launch_sc_alpha(1, nullptr, K, d + 2, st);
    launch_vec<F64>(VEC_S, n, 1, nullptr, K, r, v, s, nullptr, nullptr, st);
    if (flexible) {
      M(precond, mp, s, r);  // r holds M^-1 s
      A(r, t);
      dot_async(s, t, 3);    // <s,t> (solver.c:151)
    } else {
      A(s, t);
      dot_async(t, s, 3);    // <t,s> (solver.c:61)
    }
    dot_async(t, t, 4);
    launch_sc_omega(1, nullptr, K, d + 3, d + 4, st);
    if (flexible) launch_vec<F64>(VEC_XR, n, 1, nullptr, K, x, pp, r, s, t, st);
    else launch_vec<F64>(VEC_XR_PLAIN, n, 1, nullptr, K, x, p, r, s, t, st);
    dot_async(r, r, 5);
    dot_async(r, r0, 6);
    launch_sc_rs_beta(1, nullptr, K, d + 5, d + 6, hist.as<double>(), hcap, niter, st);
    CSEM_CUDA_TRY(cudaMemcpyAsync(&kh, K, sizeof(kh), cudaMemcpyDeviceToHost, st));
    CSEM_CUDA_TRY(cudaStreamSynchronize(st));
    if (kh.status != ST_RUNNING) break;
    launch_vec<F64>(VEC_P, n, 1, nullptr, K, r, p, v, nullptr, nullptr, st);
  }
  const int nh = std::min(hcap, kh.status == ST_ZERO_RHS ? 0 : kh.iter + 1);
  hh.resize(nh);
  if (nh) CSEM_CUDA_TRY(cudaMemcpy(hh.data(), hist.p, sizeof(double) * nh, cudaMemcpyDeviceToHost));
  status = kh.status;
  // the reference's loop index at exit: the converged iteration, or niter
  return kh.status == ST_CONVERGED ? kh.iter - 1 : kh.iter;
}

void Solver64::gmres_pre(int mp, const double2* b, double2* x)
{
  // fixed mp-step GMRES on A from x = 0 (gmres_init_free.c:58-137); its vectors
  // w, r, V[0..mp] live in a buffer of their own, so growing it never moves the outer
  // solver's vectors
  if (pre_mp < mp) {
    prework.alloc(sizeof(double2) * (size_t)n * (mp + 3));
    pre_mp = mp;
  }
  double2* pw = prework.as<double2>();
  double2 *w = pw, *r = pw + n;
  auto V = [&](int i) { return pw + (size_t)(2 + i) * n; };
  std::vector<hz> h((size_t)(mp + 1) * mp, H(0, 0)), g(mp + 1, H(0, 0)), yv(mp + 1), c(mp + 1);
  std::vector<double> sn(mp + 1, 0.0);
  auto Hm = [&](int i, int j) -> hz& { return h[(size_t)i * mp + j]; };
  double2* cf = coef.as<double2>();
  CSEM_CUDA_TRY(cudaMemsetAsync(x, 0, sizeof(double2) * n, st));
  CSEM_CUDA_TRY(cudaMemcpyAsync(r, b, sizeof(double2) * n, cudaMemcpyDeviceToDevice, st));
  double beta = std::sqrt(dot(r, r).x);
  if (beta == 0.0) return;
  double2 bd = make_double2(beta, 0.);
  CSEM_CUDA_TRY(cudaMemcpyAsync(cf, &bd, sizeof(bd), cudaMemcpyHostToDevice, st));
  launch_cdivv<F64>(n, 1, nullptr, cf, 0, 1, r, V(0), st);
  g[0] = H(beta, 0);
  for (int j = 0; j < mp; j++) {
    A(V(j), w);
    for (int i = 0; i <= j; i++) {
      Hm(i, j) = Hd(dot(w, V(i)));
      double2 hv = D(Hm(i, j));
      CSEM_CUDA_TRY(cudaMemcpyAsync(cf + 1, &hv, sizeof(hv), cudaMemcpyHostToDevice, st));
      launch_axpy<F64>(n, 1, nullptr, cf + 1, 0, 1, V(i), w, st);
    }
    Hm(j + 1, j) = H(std::sqrt(dot(w, w).x), 0);
    double2 hv = D(Hm(j + 1, j));
    CSEM_CUDA_TRY(cudaMemcpyAsync(cf + 2, &hv, sizeof(hv), cudaMemcpyHostToDevice, st));
    launch_cdivv<F64>(n, 1, nullptr, cf + 2, 0, 0, w, V(j + 1), st);
    for (int i = 0; i < j; i++) {
      hz ss = hadd(hmul(hconj(c[i]), Hm(i, j)), hrmul(sn[i], Hm(i + 1, j)));
      Hm(i + 1, j) = hadd(hrmul(-sn[i], Hm(i, j)), hmul(c[i], Hm(i + 1, j)));
      Hm(i, j) = ss;
    }
    double tmp = std::sqrt(hadd(hmul(Hm(j, j), hconj(Hm(j, j))), hmul(Hm(j + 1, j), hconj(Hm(j + 1, j)))).re);
    sn[j] = Hm(j + 1, j).re / tmp;
    c[j] = hdivr(Hm(j, j), tmp);
    Hm(j, j) = hadd(hmul(hconj(c[j]), Hm(j, j)), hrmul(sn[j], Hm(j + 1, j)));
    Hm(j + 1, j) = H(0, 0);
    g[j + 1] = hrmul(-sn[j], g[j]);
    g[j] = hmul(hconj(c[j]), g[j]);
  }
  yv[mp - 1] = hdiv(g[mp - 1], Hm(mp - 1, mp - 1));
  for (int i = mp - 2; i >= 0; i--) {
    yv[i] = g[i];
    for (int j = i + 1; j < mp; j++) yv[i] = hsub(yv[i], hmul(Hm(i, j), yv[j]));
    yv[i] = hdiv(yv[i], Hm(i, i));
  }
  std::vector<double2> yd(mp);
  for (int j = 0; j < mp; j++) yd[j] = D(yv[j]);
  CSEM_CUDA_TRY(cudaMemcpyAsync(cf + 8, yd.data(), sizeof(double2) * mp, cudaMemcpyHostToDevice, st));
  for (int j = 0; j < mp; j++) launch_axpy<F64>(n, 1, nullptr, cf + 8 + j, 0, 0, V(j), x, st);
}

int Solver64::gmres(int precond, int mp, double2* x, const double2* b, int ncycle, double tol, int m0,
                    std::vector<double>& hh, int& status)
{
  // precond == PRE_NONE: gmres (solver.c:181-285, h[i][j] layout, early return without
  // the last update on convergence); otherwise fgmres (solver.c:403-512)
  int mr = m0;
  const bool flex = precond != PRE_NONE;
  ensure_work(2 + (mr + 1) + (flex ? mr : 0));
  double2 *w = W(0), *r = W(1);
  auto V = [&](int i) { return W(2 + i); };
  auto Z = [&](int i) { return W(2 + (mr + 1) + i); };
  const int m_alloc = mr;
  std::vector<hz> h((size_t)(m_alloc + 1) * (m_alloc + 1), H(0, 0)), g(m_alloc + 1), yv(m_alloc + 1), c(m_alloc + 1);
  std::vector<double> sn(m_alloc + 1, 0.0);
  // unpreconditioned: H(i,j) = h[i][j]; flexible: H(j,i) = h[j][i] (transposed storage)
  auto Hm = [&](int i, int j) -> hz& { return h[(size_t)i * (m_alloc + 1) + j]; };
  double2* cf = coef.as<double2>();
  double r0 = 0;
  int iter, conv = 0, j = 0;
  hh.clear();
  status = ST_MAXITER;
  for (iter = 0; iter < ncycle; iter++) {
    A(x, w);
    launch_vec<F64>(VEC_SUB, n, 1, nullptr, nullptr, (double2*)b, w, r, nullptr, nullptr, st);
    double beta = std::sqrt(dot(r, r).x);
    if (beta == 0.0) {
      status = iter == 0 ? ST_ZERO_RHS : ST_CONVERGED;
      return iter;
    }
    double2 bd = make_double2(beta, 0.);
    CSEM_CUDA_TRY(cudaMemcpyAsync(cf, &bd, sizeof(bd), cudaMemcpyHostToDevice, st));
    launch_cdivv<F64>(n, 1, nullptr, cf, 0, 1, r, V(0), st);
    std::fill(g.begin(), g.end(), H(0, 0));
    g[0] = H(beta, 0);
    std::fill(h.begin(), h.end(), H(0, 0));
    if (iter == 0) {
      r0 = beta;
      hh.push_back(flex ? 1.0 : beta / r0);
    }
    for (j = 0; j < mr; j++) {
      if (flex) {
        M(precond, mp, V(j), Z(j));
        A(Z(j), w);
      } else {
        A(V(j), w);
      }
      for (int i = 0; i <= j; i++) {
        hz hij = Hd(dot(w, V(i)));
        if (flex) Hm(j, i) = hij; else Hm(i, j) = hij;
        double2 hv = D(hij);
        CSEM_CUDA_TRY(cudaMemcpyAsync(cf + 1, &hv, sizeof(hv), cudaMemcpyHostToDevice, st));
        launch_axpy<F64>(n, 1, nullptr, cf + 1, 0, 1, V(i), w, st);
      }
      hz hn = H(std::sqrt(dot(w, w).x), 0);
      if (flex) Hm(j, j + 1) = hn; else Hm(j + 1, j) = hn;
      if (habs(hn) == 0.0) {
        if (flex) { conv = 1; break; }
        mr = j + 1;
        break;
      }
      double2 hv = D(hn);
      CSEM_CUDA_TRY(cudaMemcpyAsync(cf + 2, &hv, sizeof(hv), cudaMemcpyHostToDevice, st));
      launch_cdivv<F64>(n, 1, nullptr, cf + 2, 0, 0, w, V(j + 1), st);
      if (flex) {
        for (int i = 0; i < j; i++) {
          hz ss = hadd(hmul(hconj(c[i]), Hm(j, i)), hrmul(sn[i], Hm(j, i + 1)));
          Hm(j, i + 1) = hadd(hrmul(-sn[i], Hm(j, i)), hmul(c[i], Hm(j, i + 1)));
          Hm(j, i) = ss;
        }
        double tmp = std::sqrt(hadd(hmul(Hm(j, j), hconj(Hm(j, j))), hmul(Hm(j, j + 1), hconj(Hm(j, j + 1)))).re);
        sn[j] = Hm(j, j + 1).re / tmp;
        c[j] = hdivr(Hm(j, j), tmp);
        g[j + 1] = hrmul(-sn[j], g[j]);
        g[j] = hmul(hconj(c[j]), g[j]);
        Hm(j, j) = hadd(hmul(hconj(c[j]), Hm(j, j)), hrmul(sn[j], Hm(j, j + 1)));
        double rel = habs(g[j + 1]) / r0;
        hh.push_back(rel);
        if (rel < tol) { conv = 1; break; }
      } else {
        for (int i = 0; i < j; i++) {
          hz ss = hadd(hmul(hconj(c[i]), Hm(i, j)), hrmul(sn[i], Hm(i + 1, j)));
          Hm(i + 1, j) = hadd(hrmul(-sn[i], Hm(i, j)), hmul(c[i], Hm(i + 1, j)));
          Hm(i, j) = ss;
        }
        double tmp = std::sqrt(hadd(hmul(Hm(j, j), hconj(Hm(j, j))), hmul(Hm(j + 1, j), hconj(Hm(j + 1, j)))).re);
        sn[j] = Hm(j + 1, j).re / tmp;
        c[j] = hdivr(Hm(j, j), tmp);
        Hm(j, j) = hadd(hmul(hconj(c[j]), Hm(j, j)), hrmul(sn[j], Hm(j + 1, j)));
        Hm(j + 1, j) = H(0, 0);
        g[j + 1] = hrmul(-sn[j], g[j]);
        g[j] = hmul(hconj(c[j]), g[j]);
        double rel = habs(g[j + 1]) / r0;
        hh.push_back(rel);
        if (rel < tol) {  // returns without applying this cycle's update (solver.c:250-251)
          status = ST_CONVERGED;
          return iter;
        }
      }
    }
    const int mm = flex ? std::min(mr, j + 1) : mr;
    yv[mm - 1] = hdiv(g[mm - 1], flex ? Hm(mm - 1, mm - 1) : Hm(mm - 1, mm - 1));
    for (int i = mm - 2; i >= 0; i--) {
      yv[i] = g[i];
      for (int jj = i + 1; jj < mm; jj++) yv[i] = hsub(yv[i], hmul(flex ? Hm(jj, i) : Hm(i, jj), yv[jj]));
      yv[i] = hdiv(yv[i], Hm(i, i));
    }
    std::vector<double2> yd(mm);
    for (int q = 0; q < mm; q++) yd[q] = D(yv[q]);
    CSEM_CUDA_TRY(cudaMemcpyAsync(cf + 8, yd.data(), sizeof(double2) * mm, cudaMemcpyHostToDevice, st));
    for (int q = 0; q < mm; q++) launch_axpy<F64>(n, 1, nullptr, cf + 8 + q, 0, 0, flex ? Z(q) : V(q), x, st);
    CSEM_CUDA_TRY(cudaStreamSynchronize(st));
    if (conv) {
      status = ST_CONVERGED;
      return iter;
    }
  }
  return iter;
}

}  // namespace csem
