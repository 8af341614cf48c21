// Internal C++ interface between the kernel files and the solver engine.
#pragma once
#include <cuda_runtime.h>
#include <cufft.h>
#include "csem_cuda.cuh"

namespace csem {

// ---------------------------------------------------------------- operator
template <class P>
void launch_fdfd(const GridP<P>& g, const SysScal<P>* scal, const typename P::C* X, typename P::C* Y,
                 const typename P::C* ghx, const typename P::C* ghy, int nsys, const int* sys_list,
                 cudaStream_t st, int by = 8, int ctas_per_sm = 4);
// complex64 y = A x with the Krylov dot products of y folded in (k_fdfd EPI): kind 1 sums
// y conj(E), kind 2 e conj(y) and y conj(y); part gets fdfd_partials(...) partials per slot
// (kind 2: two sets of nsys), for launch_dot_finish
void launch_fdfd_dot(const GridP<F32>& g, const SysScal<F32>* scal, const float2* X, float2* Y, const float2* ghx,
                     const float2* ghy, int nsys, const int* sys_list, cudaStream_t st, int by, int ctas_per_sm,
                     int kind, const float2* E, double2* part);
int fdfd_partials(int n1, int n2, int n3, int nsys, int by, int ctas_per_sm);  // CTAs per system of the stencil
template <class P>
void launch_hz0(const GridP<P>& g, const SysScal<P>* scal, const typename P::C* X, typename P::C* out,
                int nsys, const int* sys_list, cudaStream_t st);

// ---------------------------------------------------------------- airwave
// Tables of airbc_init_free.c:86-105 and of the back-interpolation
// (airbc_init_free.c:168-207), precomputed on the host in double.
template <class P> struct AirP {
  typedef typename P::R R;
  int n1, n2, N1, N2;
  const int *jx, *jy;      // gather cell per uniform node, -1 outside x1s[n1-1] / x2s[n2-1]
  const R *wx, *wy;
  const int *hx_j1, *hx_j2;  // Hx ghost: per i1 <= n1 (from x1), per i2 < n2 (from x2s)
  const R *hx_w1, *hx_w2;
  const int *hy_j1, *hy_j2;  // Hy ghost: per i1 < n1 (from x1s), per i2 <= n2 (from x2)
  const R *hy_w1, *hy_w2;
  const typename P::C *sH1, *sH2;  // [N2][N1]
};

template <class P>
void launch_air_gather(const AirP<P>& a, const typename P::C* hz0, typename P::C* K, int nslot, cudaStream_t st);
template <class P>
void launch_air_filter(const AirP<P>& a, const typename P::C* K, typename P::C* K2, int nslot, cudaStream_t st);
template <class P>
void launch_air_scatter(const AirP<P>& a, const typename P::C* K2, typename P::C* ghx, typename P::C* ghy,
                        int nslot, cudaStream_t st);

// ---------------------------------------------------------------- LU-SGS / A-phi
// A component sweep over one wavefront diagonal. The sweep grid has nK planes
// (full grid for LU-SGS with airbc); stored vector plane = sweep plane - vshift,
// planes below vshift live in the cap scratch (air layers).
template <class P> struct SweepP {
  GridP<P> g;          // d3/sigma pointers already shifted by dshift
  int nK;              // sweep grid depth
  int vshift;          // planes below vshift are air (cap)
  const typename P::C* X;   // right-hand side (operator grid), [sys][lE]
  typename P::C* Y;         // solution (operator grid), [sys][lE]
  typename P::C* CAP;       // [slot][capE] air planes, full-grid plane layout
  long capEx, capEy, capE;  // cap component offsets
  const SysScal<P>* scal;
  const int* sys_list;
  // A-phi only
  const typename P::C* V;   // node potential [slot][lv]
  const typename P::R *s11u, *s22u, *s33u;  // unshifted full-grid sigma (the Q2 lookups)
  const typename P::C* BV;  // divergence right-hand side [slot][lv]
  long lv;
  int aphi_fix;             // 1: node sweeps with the conductivity-weighted diagonal (not the reference's)
};

// one launch per component sweep (pipelined warps, k_lusgs2.cu)
template <class P>
void launch_sweep_pipelined(const SweepP<P>& s, int comp, bool fwd, int nslot, cudaStream_t st, int vw,
                            int lines_per_cta = 1);
bool sweep_pipelined_fits(int comp, int n1, int n2, int nK);  // the sweep's rows fit one CTA
// complex64 line-tiled sweeps (k_lusgs3.cu): 32 lines per CTA, rows in warp blocks of at
// most rows_per_warp (4, 8, 16), vw march positions per step for Ey/Ez (1, 2, 4)
void launch_sweep_tiled(const SweepP<F32>& s, int comp, bool fwd, int nslot, cudaStream_t st, int rows_per_warp,
                        int vw);
bool sweep_tiled_fits(int comp, int n1, int n2, int nK, int rows_per_warp, int vw);  // the rows fit one CTA
// complex64 pipelined sweeps with ns systems of one frequency per CTA (k_lusgs4.cu):
// groups[g * ns + q] is the slot of member q of group g (-1: absent, member 0 present);
// ns 2 (vw 1 or 2) or 4 (vw 1)
void launch_sweep_grouped(const SweepP<F32>& s, int comp, bool fwd, const int* groups, int ngroups, int ns, int vw,
                          cudaStream_t st);
bool sweep_grouped_fits(int comp, int n1, int n2, int nK);  // at most 256 rows
// complex64 split sweeps (k_lusgs5.cu): a coalesced pass stores (B, w) of every point in
// SB (sbs float4 per slot, at least sweep_split_scratch), then the row pipeline runs the
// chain; vw 1, 2 or 4 points per thread and step. With groups (ns == SPLIT_GROUP: the
// slots of one frequency, SPLIT_GROUP per group, -1 padded) the pass forms each point's
// frequency-only coefficients once per group.
constexpr int SPLIT_GROUP = 16;
void launch_sweep_split(const SweepP<F32>& s, int comp, bool fwd, int nslot, float4* SB, long sbs, int vw,
                        const int* groups, int ngroups, int ns, cudaStream_t st);
// the two halves of launch_sweep_split; max_ctas > 0 caps the pipeline's grid (each CTA
// then takes several lines in turn), which leaves room on the SMs for the passes of
// another stream
void launch_split_prep(const SweepP<F32>& s, int comp, bool fwd, int nslot, float4* SB, long sbs, const int* groups,
                       int ngroups, int ns, cudaStream_t st);
void launch_split_sweep(const SweepP<F32>& s, int comp, bool fwd, int nslot, const float4* SB, long sbs, int vw,
                        int max_ctas, cudaStream_t st);
int sm_count();  // multiprocessors of the current device
long sweep_split_scratch(int n1, int n2, int nK);  // largest component on the sweep grid
template <class P>
void launch_sweep(const SweepP<P>& s, int comp, bool fwd, bool aphi, int t, int nslot, cudaStream_t st);
int sweep_diagonals(int comp, int n1, int n2, int nK);  // number of diagonals t (2..)

template <class P>
void launch_aphi_div(const SweepP<P>& s, typename P::C* BV, int nslot, cudaStream_t st);
template <class P>
void launch_aphi_phi(const SweepP<P>& s, typename P::C* V, int t, int nslot, cudaStream_t st);
int phi_diagonals(int n1, int n2, int n3);
template <class P>
void launch_aphi_grad(const SweepP<P>& s, const typename P::C* V, int nslot, cudaStream_t st);

// ---------------------------------------------------------------- BLAS-1
template <class P>
void launch_dot(const typename P::C* a, const typename P::C* b, long n, long stride, int nslot,
                const int* sys_list, double2* partial, int nblk, double2* out, cudaStream_t st);
// out1 = a1.conj(b1), out2 = a2.conj(b2) in one pass, each bit-identical to launch_dot;
// partial holds 2 * nslot * nblk entries
template <class P>
void launch_dot2(const typename P::C* a1, const typename P::C* b1, const typename P::C* a2,
                 const typename P::C* b2, long n, long stride, int nslot, const int* sys_list, double2* partial,
                 int nblk, double2* out1, double2* out2, cudaStream_t st);
// complex128 <a, b> of one system in the reference's sequential order (bit-identical to
// cdotprod.c), into out[0]; one CTA, a dependent chain of n additions
void launch_dot_seq(const double2* a, const double2* b, long n, double2* out, cudaStream_t st);
int dot_blocks(long n);
// out1[slot] (and out2[slot]) = fixed-order sums of partial[slot][0..nblk) (and of
// partial[nslot + slot][...]), as launch_dot / launch_dot2 finish
void launch_dot_finish(const double2* partial, int nblk, int nslot, double2* out1, double2* out2, cudaStream_t st);

}  // namespace csem
