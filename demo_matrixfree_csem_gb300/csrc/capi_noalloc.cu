// csem_cdot_dev_noalloc: the batched dot product of csem_cdot_dev without any device
// allocation by the library.
//
// Who needs it: a caller that has already given all free device memory to its own pool
// (a framework's caching allocator, or a batch of Krylov vectors sized to fill HBM)
// cannot let a library take more, and a caller inside a tight loop may not accept the
// device-wide synchronisation that cudaMalloc/cudaFree can imply. csem_cdot_dev keeps its
// per-block partial sums in a buffer it allocates on first use and grows on demand; this
// variant keeps them in a fixed array that is part of the library's own device image.
//
// Rules of use (also stated in include/csem_gpu.h):
//  - at most CSEM_NOALLOC_DOT_MAX_SYSTEMS systems per call (1 MiB of partials: 64
//    systems x the at most 1024 blocks one dot product is split into);
//  - the array's device address is looked up with cudaGetSymbolAddress once per device,
//    on the first call made with that device current, and cached; make that first call
//    before any stream capture starts. The cache is never refreshed, so a
//    cudaDeviceReset of that device between two calls is not supported;
//  - the array is one per device for the whole process: calls on the same device that
//    overlap in time (other streams, other host threads) race on it and return wrong
//    results, so serialise them, e.g. on one stream;
//  - nothing in the array has to start at zero: the first kernel of a call writes every
//    partial the second kernel reads.
// The arithmetic is the same kernels as csem_cdot_dev, so both give identical bits.
#include <mutex>
#include "../../include/csem_gpu.h"
#include "engine.h"

extern "C" int csem_set_error(int code, const char* fmt, ...);

namespace {

constexpr int NOALLOC_MAX_BLOCKS = 1024;  // the largest block count dot_blocks() returns
constexpr int NOALLOC_MAX_DEVICES = 64;

__device__ __align__(256) double2 g_noalloc_partial[CSEM_NOALLOC_DOT_MAX_SYSTEMS * NOALLOC_MAX_BLOCKS];

std::mutex g_noalloc_mu;
double2* g_noalloc_addr[NOALLOC_MAX_DEVICES];

}  // namespace

extern "C" int csem_cdot_dev_noalloc(int prec, long n, int nsys, const void* a, const void* b, double* out_dev,
                                     void* stream)
{
  if (prec != 64 && prec != 32) return csem_set_error(CSEM_EINVAL, "csem_cdot_dev_noalloc: prec must be 64 or 32");
  if (n < 1 || nsys < 1) return csem_set_error(CSEM_EINVAL, "csem_cdot_dev_noalloc: n and nsys must be positive");
  if (nsys > CSEM_NOALLOC_DOT_MAX_SYSTEMS)
    return csem_set_error(CSEM_ETOOBIG,
                          "csem_cdot_dev_noalloc: nsys=%d is more than the %d systems its fixed scratch holds; "
                          "split the call or use csem_cdot_dev",
                          nsys, CSEM_NOALLOC_DOT_MAX_SYSTEMS);
  const int nblk = csem::dot_blocks(n);
  if (nblk > NOALLOC_MAX_BLOCKS)
    return csem_set_error(CSEM_ETOOBIG, "csem_cdot_dev_noalloc: %d partial blocks exceed the scratch", nblk);
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess)
    return csem_set_error(CSEM_ECUDA, "csem_cdot_dev_noalloc: cudaGetDevice: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= NOALLOC_MAX_DEVICES)
    return csem_set_error(CSEM_EINVAL, "csem_cdot_dev_noalloc: device %d is beyond the %d supported", dev,
                          NOALLOC_MAX_DEVICES);
  double2* part = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    part = g_noalloc_addr[dev];
    if (!part) {
      e = cudaGetSymbolAddress((void**)&part, g_noalloc_partial);
      if (e != cudaSuccess)
        return csem_set_error(CSEM_ECUDA, "csem_cdot_dev_noalloc: cudaGetSymbolAddress on device %d: %s", dev,
                              cudaGetErrorString(e));
      g_noalloc_addr[dev] = part;
    }
  }
  cudaStream_t st = (cudaStream_t)stream;
  if (prec == 64)
    csem::launch_dot<csem::F64>((const double2*)a, (const double2*)b, n, n, nsys, nullptr, part, nblk,
                                (double2*)out_dev, st);
  else
    csem::launch_dot<csem::F32>((const float2*)a, (const float2*)b, n, n, nsys, nullptr, part, nblk,
                                (double2*)out_dev, st);
  e = cudaGetLastError();
  if (e != cudaSuccess)
    return csem_set_error(CSEM_ECUDA, "csem_cdot_dev_noalloc: launch: %s", cudaGetErrorString(e));
  return CSEM_OK;
}
