// Device-resident model and the operator / preconditioner applications built on it.
#pragma once
#include <cuda_runtime.h>
#include <cufft.h>
#include <vector>
#include "csem_cuda.cuh"
#include "engine.h"
#include "engine_acq.h"
#include "solver_state.h"

struct csem_grid;

namespace csem {

#define CSEM_CUDA_TRY(x)                                                     \
  do {                                                                       \
    cudaError_t e_ = (x);                                                    \
    if (e_ != cudaSuccess) throw CudaError(e_, #x, __FILE__, __LINE__);      \
  } while (0)

struct CudaError {
  cudaError_t err;
  const char *expr, *file;
  int line;
  CudaError(cudaError_t e, const char* x, const char* f, int l) : err(e), expr(x), file(f), line(l) {}
};
struct CsemError {
  int code;
  char msg[256];
};

// device allocation owned by a Model / workspace
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  void alloc(size_t b);
  void free_();
  ~DevBuf() { free_(); }
  template <class T> T* as() const { return (T*)p; }
};

enum Precond { PRE_NONE = 0, PRE_LUSGS = 1, PRE_GMRES = 2, PRE_APHI = 3 };

// FFT plans for batches of 1,2,4,..,2^k uniform airwave grids
struct FftPlans {
  int N1 = 0, N2 = 0;
  std::vector<cufftHandle> z, c;  // index = log2(batch)
  ~FftPlans();
  void exec(bool dbl, void* data, int count, int dir, cudaStream_t st);
};

class Model {
 public:
  Model(const csem_grid* g, int airbc, int fvm);
  ~Model();
  // geometry
  int n1, n2, n3, n3f, nb, nz, airbc, fvm;
  long lEx, lEy, lEz, lE, lv;
  float rho_water;
  int N1 = 0, N2 = 0;  // airwave grid
  // device data
  DevBuf d64, d32, s64, s32, x64, air_i, air_w64, air_w32, sH64, sH32;
  GridP<F64> g64;  // operator view (kstart shift applied inside kernels)
  GridP<F32> g32;
  AirP<F64> a64;
  AirP<F32> a32;
  AcqGrid acq;
  // cuFFT plans of this model's airwave grid (one set per model: a plan is bound to one
  // stream at a time, and contexts may run on different host threads)
  FftPlans fft_plans;
  template <class P> const GridP<P>& grid() const;
  template <class P> const AirP<P>& air() const;
  template <class P> GridP<P> grid_shifted() const;  // d3/sigma advanced by kstart planes
};

// Groups of slots at one frequency for the grouped complex64 sweeps (k_lusgs4.cu):
// dev[g * ns + q] is the slot of member q of group g (-1: absent)
struct SweepGroups {
  const int* dev = nullptr;
  int n = 0;   // groups
  int ns = 1;  // members per group
  // split sweeps run as two halves on two streams when nA > 0: slots [0, nA) and
  // [nA, nslot); the first ngA groups hold slots of the first half, the others slots of
  // the second, each numbered from the start of its half
  int nA = 0, ngA = 0;
};

// Groups of at most ns slots with equal iom (iom_of_slot[2 slot], [2 slot + 1]), the
// slots of one frequency in their order, the frequencies in order of first appearance;
// out gets ngroups * ns entries. Returns the number of groups.
int build_sweep_groups(int nslot, const double* iom_of_slot, int ns, std::vector<int>& out);
// The same for the two halves of the slots when nslot >= 2 * min_half (*nA = nslot / 2,
// *ngA the first half's groups, slot numbers local to each half); otherwise one set and
// *nA = *ngA = 0. Returns the number of groups.
int build_sweep_groups_halves(int nslot, const double* iom_of_slot, int ns, int min_half, std::vector<int>& out,
                              int* nA, int* ngA);

// Krylov dot products of A's result y to form with it: kind 1 out1 = <y, e>, kind 2
// out1 = <e, y> and out2 = <y, y> (<a, b> = sum a conj(b)), per slot; partial holds
// 2 * nslot * cap doubles2 (cap >= nblk, the blocks of the separate dot products over n)
template <class P> struct DotEpi {
  int kind = 0;
  const typename P::C* e = nullptr;
  double2* partial = nullptr;
  int cap = 0;
  double2* out1 = nullptr;
  double2* out2 = nullptr;
  long n = 0;
  int nblk = 0;
};

// Per-precision workspace for nslot systems on one model.
template <class P>
class Ops {
 public:
  typedef typename P::C C;
  Ops(Model* m, int nslot_max, cudaStream_t st);
  Model* m;
  int nmax;
  cudaStream_t st;
  DevBuf hz0, K, K2, ghx, ghy, cap, V, BV, scal, sb;
  FftPlans* fft;
  // LU-SGS sweeps: true = one pipelined-warp launch per component sweep (k_lusgs2.cu),
  // false = one launch per wavefront diagonal (k_lusgs.cu); both give identical results
  bool pipelined_sweeps = true;
  int sweep_vw = 0;  // points per thread and step of the pipelined sweeps (0: default)
  int sweep_lines = 1;  // complex64: lines one CTA of the pipelined sweeps carries as a conveyor
  // complex64: systems of one frequency one CTA of the pipelined sweeps carries (1, 2, 4);
  // used where the caller passes groups of 2 or 4 to apply_lusgs
  int sweep_systems = 1;
  // members per group of same-frequency slots the caller should pass to apply_lusgs: 2 or
  // 4 for the grouped sweeps, SPLIT_GROUP for the split sweeps' pass, 1 for none
  int group_size() const { return split_sweeps ? SPLIT_GROUP : (sweep_systems >= 4 ? 4 : sweep_systems); }
  // complex64: each component sweep as a coalesced pass storing every point's (B, w) and a
  // row pipeline that reads them (k_lusgs5.cu); scratch sb holds the pass's output
  bool split_sweeps = true;
  // split sweeps on two halves of the slots, one on `aux`, so that one half's passes can
  // run while the other half's pipelines do; split_cap > 0 runs the pipelines as that many
  // CTAs per SM, each taking lines in turn (0: one CTA per line)
  bool split_overlap = true;
  int split_cap = 0;
  cudaStream_t aux = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  int stencil_by = 8;    // stencil tile: output rows per CTA (4, 8, 16)
  int stencil_ctas = 4;  // stencil z-blocks: CTAs per SM the plane chunks aim for
  // complex64 only: line-tiled sweeps (k_lusgs3.cu) instead of the pipelined ones, with
  // at most tile_rows rows per warp and tile_vw march positions per step (Ey, Ez)
  bool tiled_sweeps = false;
  // A-phi node sweeps with the conductivity-weighted diagonal and consistently shifted
  // conductivities instead of the reference's (an option; off reproduces the reference)
  bool aphi_fix = false;
  int tile_rows = 8;
  int tile_vw = 4;
  // y = A x for nslot slots (sys_list maps slot -> system index in X/Y/scal). With epi,
  // the complex64 stencil also forms the dot products epi asks for where fused_dots is on
  // and its partials fit; returns whether it did (otherwise the caller runs the separate
  // dot-product kernels, the default: they measured faster)
  bool apply_A(const C* X, C* Y, int nslot, const int* sys_list, const SysScal<P>* sc,
               const DotEpi<P>* epi = nullptr);
  bool fused_dots = false;
  // complex128 only: the stencil in F64Q (reciprocal spacings, contraction allowed), for
  // residuals that need complex128 accuracy but not the reference's bits
  bool quick_stencil = false;
  // bounds_zero: the caller guarantees that Y's entries outside the swept interior are
  // zero (they are never written by the sweeps, so a buffer only ever written by
  // apply_lusgs, or by operations that keep them zero, stays so); then Y is not cleared
  // first. The sweeps overwrite every interior point before reading it.
  // grp: same-frequency groups of the slots (complex64; sweep_systems > 1 only), or null
  void apply_lusgs(const C* X, C* Y, int nslot, const int* sys_list, const SysScal<P>* sc,
                   bool bounds_zero = false, const SweepGroups* grp = nullptr);
  void apply_aphi(const C* X, C* Y, int nslot, const int* sys_list, const SysScal<P>* sc);
  void zero(C* Y, long n, int nslot, const int* sys_list);
  int split_ctas() const;  // the split pipelines' grid cap on two streams: split_cap CTAs per SM (0: none)
  ~Ops();
};


SysScal<F64> sys_scal64(double iom_re, double iom_im);
SysScal<F32> sys_scal32(const SysScal<F64>& s);

// The operator assembled in CSR by probing the stencil, timed against it with cuSPARSE's
// SpMV (csr_compare.cu); out: ms per SpMV, ms per stencil, max relative difference, nnz,
// bytes one SpMV moves. Model without airwave coupling only.
void csr_compare(Model* m, cudaStream_t st, int prec, double iom_re, double iom_im, int nrep, double* out);

}  // namespace csem
