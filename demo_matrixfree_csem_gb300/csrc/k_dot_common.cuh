// Deterministic dot-product accumulation shared by the vector kernels (k_blas.cu) and the
// stencil's fused dot products (k_fdfd.cu): per-thread accumulators of a*conj(b) and a
// fixed shuffle tree.
#pragma once
#include "csem_cuda.cuh"

namespace csem {
namespace {

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

// A thread's running sum of a*conj(b) (FP64 for complex128, compensated float pairs for
// complex64).
template <class P> struct DotAcc;
template <> struct DotAcc<F64> {
  double2 acc = make_double2(0, 0);
  __device__ __forceinline__ void add(double2 a, double2 b)
  {
    double2 x = make_double2(a.x, a.y), y = make_double2(b.x, -b.y);
    double2 pr = cmul<F64>(x, y);
    acc.x = __dadd_rn(acc.x, pr.x);
    acc.y = __dadd_rn(acc.y, pr.y);
  }
  __device__ __forceinline__ double2 value() const { return acc; }
};
template <> struct DotAcc<F32> {
  Acc2 re = {0.f, 0.f}, im = {0.f, 0.f};
  __device__ __forceinline__ void add(float2 a, float2 b)
  {
    re.addprod(a.x, b.x);
    re.addprod(a.y, b.y);
    im.addprod(a.y, b.x);
    im.subprod(a.x, b.y);
  }
  __device__ __forceinline__ double2 value() const { return make_double2(re.value(), im.value()); }
};

template <> struct DotAcc<F64Q> : DotAcc<F64> {};  // the complex128 accumulation

}  // namespace
}  // namespace csem
