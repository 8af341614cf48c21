// Airwave top boundary (airbc_init_free.c:130-209): Hz(z=0) on the stretched grid is
// interpolated onto a uniform n1fft x n2fft grid, Fourier transformed (cuFFT, batched
// over systems), multiplied by the two upward-continuation filters sH1/sH2, inverse
// transformed, normalised and interpolated back onto the staggered ghost nodes
// Hx(z=-dz/2) [(n2) x (n1+1)] and Hy(z=-dz/2) [(n2+1) x n1].
//
// The back-interpolation may address one node past the uniform grid (the last
// stretched node maps exactly onto the last uniform node, airbc_init_free.c:173-205);
// flat indices past n1fft*n2fft read zero here.
#include "csem_cuda.cuh"
#include "engine.h"

namespace csem {

template <class P>
__global__ void k_air_gather(AirP<P> a, const typename P::C* __restrict__ hz0, typename P::C* __restrict__ K)
{
  typedef typename P::C C;
  typedef typename P::R R;
  const int i1 = blockIdx.x * blockDim.x + threadIdx.x, i2 = blockIdx.y;
  const int slot = blockIdx.z;
  if (i1 >= a.N1) return;
  C val = czero<P>();
  const int j1 = a.jx[i1], j2 = a.jy[i2];
  if (j1 >= 0 && j2 >= 0) {
    const C* H = hz0 + (size_t)slot * a.n1 * a.n2;
    const R w1 = a.wx[i1], w2 = a.wy[i2];
    const R one = 1;
    C t0 = rmul<P>(P::mul(P::sub(one, w1), P::sub(one, w2)), H[j1 + (long)a.n1 * j2]);
    C t1 = rmul<P>(P::mul(w1, P::sub(one, w2)), H[j1 + 1 + (long)a.n1 * j2]);
    C t2 = rmul<P>(P::mul(P::sub(one, w1), w2), H[j1 + (long)a.n1 * (j2 + 1)]);
    C t3 = rmul<P>(P::mul(w1, w2), H[j1 + 1 + (long)a.n1 * (j2 + 1)]);
    val = cadd<P>(cadd<P>(cadd<P>(t0, t1), t2), t3);
  }
  K[(size_t)slot * a.N1 * a.N2 + i1 + (long)a.N1 * i2] = val;
}

template <class P>
__global__ void k_air_filter(AirP<P> a, const typename P::C* __restrict__ K, typename P::C* __restrict__ K2)
{
  const long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long NN = (long)a.N1 * a.N2;
  const int slot = blockIdx.y;
  if (q >= NN) return;
  typename P::C k0 = K[(size_t)slot * NN + q];
  K2[((size_t)2 * slot) * NN + q] = cmul<P>(k0, a.sH1[q]);
  K2[((size_t)2 * slot + 1) * NN + q] = cmul<P>(k0, a.sH2[q]);
}

template <class P>
__device__ __forceinline__ typename P::C tap(const typename P::C* K, long NN, long q, typename P::R nn)
{
  if (q >= NN) return czero<P>();
  if (P::exact) return cdivr<P>(K[q], nn);  // reference: divide by n1fft*n2fft, then interpolate
  return rmul<P>((typename P::R)1 / nn, K[q]);
}

template <class P>
__global__ void k_air_scatter(AirP<P> a, const typename P::C* __restrict__ K2, typename P::C* __restrict__ ghx,
                              typename P::C* __restrict__ ghy)
{
  typedef typename P::C C;
  typedef typename P::R R;
  const int i1 = blockIdx.x * blockDim.x + threadIdx.x, i2 = blockIdx.y;
  const int slot = blockIdx.z;
  const long NN = (long)a.N1 * a.N2;
  const R nn = (R)((double)a.N1 * (double)a.N2);
  const R one = 1;
  const int N1 = a.N1;
  if (i2 < a.n2 && i1 <= a.n1) {  // Hx ghost from filter 1
    const C* K = K2 + (size_t)2 * slot * NN;
    const int j1 = a.hx_j1[i1], j2 = a.hx_j2[i2];
    const R w1 = a.hx_w1[i1], w2 = a.hx_w2[i2];
    C t0 = rmul<P>(P::mul(P::sub(one, w1), P::sub(one, w2)), tap<P>(K, NN, j1 + (long)N1 * j2, nn));
    C t1 = rmul<P>(P::mul(w1, P::sub(one, w2)), tap<P>(K, NN, j1 + 1 + (long)N1 * j2, nn));
    C t2 = rmul<P>(P::mul(P::sub(one, w1), w2), tap<P>(K, NN, j1 + (long)N1 * (j2 + 1), nn));
    C t3 = rmul<P>(P::mul(w1, w2), tap<P>(K, NN, j1 + 1 + (long)N1 * (j2 + 1), nn));
    ghx[(size_t)slot * (a.n1 + 1) * a.n2 + i1 + (long)(a.n1 + 1) * i2] = cadd<P>(cadd<P>(cadd<P>(t0, t1), t2), t3);
  }
  if (i2 <= a.n2 && i1 < a.n1) {  // Hy ghost from filter 2
    const C* K = K2 + ((size_t)2 * slot + 1) * NN;
    const int j1 = a.hy_j1[i1], j2 = a.hy_j2[i2];
    const R w1 = a.hy_w1[i1], w2 = a.hy_w2[i2];
    C t0 = rmul<P>(P::mul(P::sub(one, w1), P::sub(one, w2)), tap<P>(K, NN, j1 + (long)N1 * j2, nn));
    C t1 = rmul<P>(P::mul(w1, P::sub(one, w2)), tap<P>(K, NN, j1 + 1 + (long)N1 * j2, nn));
    C t2 = rmul<P>(P::mul(P::sub(one, w1), w2), tap<P>(K, NN, j1 + (long)N1 * (j2 + 1), nn));
    C t3 = rmul<P>(P::mul(w1, w2), tap<P>(K, NN, j1 + 1 + (long)N1 * (j2 + 1), nn));
    ghy[(size_t)slot * a.n1 * (a.n2 + 1) + i1 + (long)a.n1 * i2] = cadd<P>(cadd<P>(cadd<P>(t0, t1), t2), t3);
  }
}

template <class P>
void launch_air_gather(const AirP<P>& a, const typename P::C* hz0, typename P::C* K, int nslot, cudaStream_t st)
{
  dim3 grd((a.N1 + 127) / 128, a.N2, nslot);
  count_launch(), k_air_gather<P><<<grd, 128, 0, st>>>(a, hz0, K);
}

template <class P>
void launch_air_filter(const AirP<P>& a, const typename P::C* K, typename P::C* K2, int nslot, cudaStream_t st)
{
  long NN = (long)a.N1 * a.N2;
  dim3 grd((unsigned)((NN + 255) / 256), nslot);
  count_launch(), k_air_filter<P><<<grd, 256, 0, st>>>(a, K, K2);
}

template <class P>
void launch_air_scatter(const AirP<P>& a, const typename P::C* K2, typename P::C* ghx, typename P::C* ghy,
                        int nslot, cudaStream_t st)
{
  dim3 grd((a.n1 + 1 + 127) / 128, a.n2 + 1, nslot);
  count_launch(), k_air_scatter<P><<<grd, 128, 0, st>>>(a, K2, ghx, ghy);
}

template void launch_air_gather<F64>(const AirP<F64>&, const double2*, double2*, int, cudaStream_t);
template void launch_air_gather<F32>(const AirP<F32>&, const float2*, float2*, int, cudaStream_t);
template void launch_air_filter<F64>(const AirP<F64>&, const double2*, double2*, int, cudaStream_t);
template void launch_air_filter<F32>(const AirP<F32>&, const float2*, float2*, int, cudaStream_t);
template void launch_air_scatter<F64>(const AirP<F64>&, const double2*, double2*, double2*, int, cudaStream_t);
template void launch_air_scatter<F32>(const AirP<F32>&, const float2*, float2*, float2*, int, cudaStream_t);

}  // namespace csem
