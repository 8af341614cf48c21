// Vector kernels of the Krylov loops (solver.c) and the complex dot product
// s = sum a_i conj(b_i) (cdotprod.c:13-19).
//
// Dot products are deterministic: a fixed partition of the vector into `nblk` blocks
// (a function of the length only), a fixed per-thread order, a fixed shuffle tree and
// a fixed-order sum of block partials. Complex128 inputs accumulate in FP64. For
// complex64 inputs each product term is split exactly (p = a*b, e = fma(a,b,-p)) and
// summed per thread with a compensated (TwoSum) float pair, so the per-thread partials
// carry ~48 significant bits; partials are combined in FP64.
#include "csem_cuda.cuh"
#include "engine.h"
#include "solver_state.h"

namespace csem {

static constexpr int DOT_THREADS = 256;

int dot_blocks(long n)
{
  long b = (n + DOT_THREADS * 8 - 1) / (DOT_THREADS * 8);
  if (b < 1) b = 1;
  if (b > 1024) b = 1024;
  return (int)b;
}

struct Acc2 {  // compensated float accumulator for one real component
  float hi, lo;
  __device__ __forceinline__ void add(float x)
  {
    float s = hi + x;
    float bb = s - hi;
    float err = (hi - (s - bb)) + (x - bb);
    hi = s;
    lo += err;
  }
  __device__ __forceinline__ void addprod(float a, float b)
  {
    float p = a * b;
    float e = fmaf(a, b, -p);
    add(p);
    lo += e;
  }
  __device__ __forceinline__ void subprod(float a, float b)
  {
    float p = a * b;
    float e = fmaf(a, b, -p);
    add(-p);
    lo -= e;
  }
  __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

__device__ __forceinline__ double2 warp_sum(double2 v)
{
  for (int o = 16; o > 0; o >>= 1) {
    v.x = __dadd_rn(v.x, __shfl_down_sync(0xffffffffu, v.x, o));
    v.y = __dadd_rn(v.y, __shfl_down_sync(0xffffffffu, v.y, o));
  }
  return v;
}

__device__ __forceinline__ double2 block_sum(double2 v)
{
  __shared__ double2 red[DOT_THREADS / 32];
  v = warp_sum(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) red[w] = v;
  __syncthreads();
  if (w == 0) {
    v = l < DOT_THREADS / 32 ? red[l] : make_double2(0, 0);
    v = warp_sum(v);
  }
  __syncthreads();
  return v;
}

// partial[slot][blk] = sum over the block's chunk of a*conj(b)
template <class P>
__global__ void __launch_bounds__(DOT_THREADS)
k_dot_partial(const typename P::C* __restrict__ A, const typename P::C* __restrict__ B, long n, long stride,
              const int* __restrict__ sys_list, double2* __restrict__ partial, int nblk)
{
  const int slot = blockIdx.y;
  const int sys = sys_list ? sys_list[slot] : slot;
  const typename P::C* a = A + (size_t)sys * stride;
  const typename P::C* b = B + (size_t)sys * stride;
  const long chunk = (n + nblk - 1) / nblk;
  const long beg = (long)blockIdx.x * chunk, end = min(n, beg + chunk);
  double2 acc;
  if (P::exact) {
    acc = make_double2(0, 0);
    for (long q = beg + threadIdx.x; q < end; q += DOT_THREADS) {
      double2 x = make_double2((double)a[q].x, (double)a[q].y), y = make_double2((double)b[q].x, -(double)b[q].y);
      double2 pr = cmul<F64>(x, y);
      acc.x = __dadd_rn(acc.x, pr.x);
      acc.y = __dadd_rn(acc.y, pr.y);
    }
  } else {
    Acc2 re = {0.f, 0.f}, im = {0.f, 0.f};
    for (long q = beg + threadIdx.x; q < end; q += DOT_THREADS) {
      const float ar = (float)a[q].x, ai = (float)a[q].y, br = (float)b[q].x, bi = (float)b[q].y;
      re.addprod(ar, br);
      re.addprod(ai, bi);
      im.addprod(ai, br);
      im.subprod(ar, bi);
    }
    acc = make_double2(re.value(), im.value());
  }
  acc = block_sum(acc);
  if (threadIdx.x == 0) partial[(size_t)slot * nblk + blockIdx.x] = acc;
}

__global__ void k_dot_final(const double2* __restrict__ partial, int nblk, double2* __restrict__ out)
{
  const int slot = blockIdx.x;
  double2 acc = make_double2(0, 0);
  for (int q = threadIdx.x; q < nblk; q += DOT_THREADS) {
    double2 v = partial[(size_t)slot * nblk + q];
    acc.x = __dadd_rn(acc.x, v.x);
    acc.y = __dadd_rn(acc.y, v.y);
  }
  acc = block_sum(acc);
  if (threadIdx.x == 0) out[slot] = acc;
}

template <class P>
void launch_dot(const typename P::C* a, const typename P::C* b, long n, long stride, int nslot,
                const int* sys_list, double2* partial, int nblk, double2* out, cudaStream_t st)
{
  dim3 grd(nblk, nslot);
  count_launch(), k_dot_partial<P><<<grd, DOT_THREADS, 0, st>>>(a, b, n, stride, sys_list, partial, nblk);
  count_launch(), k_dot_final<<<nslot, DOT_THREADS, 0, st>>>(partial, nblk, out);
}

template void launch_dot<F64>(const double2*, const double2*, long, long, int, const int*, double2*, int,
                              double2*, cudaStream_t);
template void launch_dot<F32>(const float2*, const float2*, long, long, int, const int*, double2*, int,
                              double2*, cudaStream_t);

// ------------------------------------------------------------------ vector updates
template <class P> __device__ __forceinline__ typename P::C cast_c(double2 v);
template <> __device__ __forceinline__ double2 cast_c<F64>(double2 v) { return v; }
template <> __device__ __forceinline__ float2 cast_c<F32>(double2 v) { return make_float2((float)v.x, (float)v.y); }

#define CSEM_VEC_PROLOGUE                                                  \
  const int slot = blockIdx.y;                                             \
  const int sys = sys_list ? sys_list[slot] : slot;                        \
  const long q = (long)blockIdx.x * blockDim.x + threadIdx.x;              \
  if (q >= n) return;                                                      \
  const size_t o = (size_t)sys * n + q;

// r = b - v; p = r; r0 = r   (solver.c:108-112)
template <class P>
__global__ void k_vec_init(long n, const int* __restrict__ sys_list, const typename P::C* __restrict__ b,
                           const typename P::C* __restrict__ v, typename P::C* __restrict__ r,
                           typename P::C* __restrict__ p, typename P::C* __restrict__ r0)
{
  CSEM_VEC_PROLOGUE
  typename P::C x = csub<P>(b[o], v[o]);
  r[o] = x;
  p[o] = x;
  r0[o] = x;
}

// r = b - w   (solver.c:198,423)
template <class P>
__global__ void k_vec_sub(long n, const int* __restrict__ sys_list, const typename P::C* __restrict__ b,
                          const typename P::C* __restrict__ w, typename P::C* __restrict__ r)
{
  CSEM_VEC_PROLOGUE
  r[o] = csub<P>(b[o], w[o]);
}

// s = r - alpha v   (solver.c:147)
template <class P>
__global__ void k_vec_s(long n, const int* __restrict__ sys_list, const KrylovScalars* __restrict__ ks,
                        const typename P::C* __restrict__ r, const typename P::C* __restrict__ v,
                        typename P::C* __restrict__ s)
{
  CSEM_VEC_PROLOGUE
  if (ks[sys].status != ST_RUNNING) return;  // finished systems keep their vectors
  const typename P::C alpha = cast_c<P>(ks[sys].alpha);
  s[o] = csub<P>(r[o], cmul<P>(alpha, v[o]));
}

// x += alpha pp + omega ss; r = s - omega t   (solver.c:153-156, flexible: ss lives in r;
// solver.c:63-66, plain: pp = p and ss = s)
template <class P, bool SS_IS_S>
__global__ void k_vec_xr(long n, const int* __restrict__ sys_list, const KrylovScalars* __restrict__ ks,
                         typename P::C* __restrict__ x, const typename P::C* __restrict__ pp,
                         typename P::C* __restrict__ r, const typename P::C* __restrict__ s,
                         const typename P::C* __restrict__ t)
{
  CSEM_VEC_PROLOGUE
  if (ks[sys].status != ST_RUNNING) return;
  const typename P::C alpha = cast_c<P>(ks[sys].alpha), omega = cast_c<P>(ks[sys].omega);
  const typename P::C ss = SS_IS_S ? s[o] : r[o];
  x[o] = cadd<P>(x[o], cadd<P>(cmul<P>(alpha, pp[o]), cmul<P>(omega, ss)));
  r[o] = csub<P>(s[o], cmul<P>(omega, t[o]));
}

// p = r + beta (p - omega v)   (solver.c:166)
template <class P>
__global__ void k_vec_p(long n, const int* __restrict__ sys_list, const KrylovScalars* __restrict__ ks,
                        const typename P::C* __restrict__ r, typename P::C* __restrict__ p,
                        const typename P::C* __restrict__ v)
{
  CSEM_VEC_PROLOGUE
  if (ks[sys].status != ST_RUNNING) return;
  const typename P::C beta = cast_c<P>(ks[sys].beta), omega = cast_c<P>(ks[sys].omega);
  p[o] = cadd<P>(r[o], cmul<P>(beta, csub<P>(p[o], cmul<P>(omega, v[o]))));
}

// y = a*x + y with a per-system scalar taken from a double2 array (GMRES updates)
template <class P>
__global__ void k_vec_axpy(long n, const int* __restrict__ sys_list, const double2* __restrict__ coef,
                           int coef_stride, int neg, const typename P::C* __restrict__ x,
                           typename P::C* __restrict__ y)
{
  CSEM_VEC_PROLOGUE
  const typename P::C a = cast_c<P>(coef[(size_t)slot * coef_stride]);
  if (neg) y[o] = csub<P>(y[o], cmul<P>(a, x[o]));   // w -= h*v   (solver.c:221)
  else y[o] = cadd<P>(y[o], cmul<P>(a, x[o]));       // x += y*v   (solver.c:272)
}

// y = x / d with a per-system complex divisor (GMRES v_{j+1} = w / h, beta scaling)
template <class P>
__global__ void k_vec_cdiv(long n, const int* __restrict__ sys_list, const double2* __restrict__ d, int dstride,
                           int real_only, const typename P::C* __restrict__ x, typename P::C* __restrict__ y)
{
  CSEM_VEC_PROLOGUE
  const typename P::C dv = cast_c<P>(d[(size_t)slot * dstride]);
  if (real_only) y[o] = cdivr<P>(x[o], dv.x);
  else y[o] = cdiv<P>(x[o], dv);
}

template <class P>
void launch_vec(int op, long n, int nslot, const int* sys_list, const KrylovScalars* ks, typename P::C* a,
                typename P::C* b, typename P::C* c, typename P::C* d, typename P::C* e, cudaStream_t st)
{
  dim3 grd((unsigned)((n + 255) / 256), nslot);
  switch (op) {
  case VEC_INIT: count_launch(), k_vec_init<P><<<grd, 256, 0, st>>>(n, sys_list, a, b, c, d, e); break;
  case VEC_S: count_launch(), k_vec_s<P><<<grd, 256, 0, st>>>(n, sys_list, ks, a, b, c); break;
  case VEC_XR: count_launch(), k_vec_xr<P, false><<<grd, 256, 0, st>>>(n, sys_list, ks, a, b, c, d, e); break;
  case VEC_SUB: count_launch(), k_vec_sub<P><<<grd, 256, 0, st>>>(n, sys_list, a, b, c); break;
  case VEC_XR_PLAIN: count_launch(), k_vec_xr<P, true><<<grd, 256, 0, st>>>(n, sys_list, ks, a, b, c, d, e); break;
  case VEC_P: count_launch(), k_vec_p<P><<<grd, 256, 0, st>>>(n, sys_list, ks, a, b, c); break;
  }
}

template <class P>
void launch_axpy(long n, int nslot, const int* sys_list, const double2* coef, int coef_stride, int neg,
                 const typename P::C* x, typename P::C* y, cudaStream_t st)
{
  dim3 grd((unsigned)((n + 255) / 256), nslot);
  count_launch(), k_vec_axpy<P><<<grd, 256, 0, st>>>(n, sys_list, coef, coef_stride, neg, x, y);
}

template <class P>
void launch_cdivv(long n, int nslot, const int* sys_list, const double2* d, int dstride, int real_only,
                  const typename P::C* x, typename P::C* y, cudaStream_t st)
{
  dim3 grd((unsigned)((n + 255) / 256), nslot);
  count_launch(), k_vec_cdiv<P><<<grd, 256, 0, st>>>(n, sys_list, d, dstride, real_only, x, y);
}

#define CSEM_INST(P)                                                                                        \
  template void launch_vec<P>(int, long, int, const int*, const KrylovScalars*, P::C*, P::C*, P::C*, P::C*, \
                              P::C*, cudaStream_t);                                                         \
  template void launch_axpy<P>(long, int, const int*, const double2*, int, int, const P::C*, P::C*,         \
                               cudaStream_t);                                                               \
  template void launch_cdivv<P>(long, int, const int*, const double2*, int, int, const P::C*, P::C*,        \
                                cudaStream_t);
CSEM_INST(F64)
CSEM_INST(F32)
#undef CSEM_INST

}  // namespace csem
