// noalloc.cu -- cappgpu_spmv_noalloc: the product zk = A pk and the dot
// pk.zk of cappgpu_spmv (pcg-sip.f90:143-155) with its reduction scratch in
// a fixed device array instead of memory obtained from the allocator.
//
// Some callers cannot allocate device memory at the point where they need
// this product: a time-step loop whose process has handed the whole device
// pool to another allocator (a framework's caching allocator sharing the GPU
// with the solver), or one that must not take the implicit device-wide
// synchronisation of cudaMalloc/cudaFree between two steps.  This entry point
// touches only the context's field arrays, which cappgpu_init allocated, and
// the file-scope array below.
//
// Scratch: one partial sum per chunk of kNaChunk interior cells, at most
// kNaMaxParts chunks, plus one result word -- 32 KB.  Larger grids are
// rejected with CAPPGPU_E_ARG.  Nothing in the scratch has to start at zero:
// every partial is written before it is read and the result word is written
// by the finishing kernel.  All calls share the one array, so calls that
// overlap (from several host threads, or while an earlier call's kernels are
// still running on another stream) race on it.
//
// The first call on a device looks up the array's device address with
// cudaGetSymbolAddress and keeps it; that first call should come before any
// stream capture is started.  Calls must be made with the context's device
// (the one current at cappgpu_init) current: the kernels run on the
// context's stream, so another device's address of the array would be
// wrong for them, and such calls are refused.
#include <math.h>

#include <atomic>

#include "common.cuh"
#include "kernels.cuh"

namespace cap {

namespace {

constexpr int kNaThreads = 256;
constexpr int kNaPerThread = 8;
constexpr int kNaChunk = kNaThreads * kNaPerThread;   // interior cells per partial
constexpr int kNaMaxParts = 4096;                     // => at most 8,388,608 interior cells
constexpr int kNaMaxDevices = 64;

__device__ __align__(256) double g_na_scratch[kNaMaxParts + 1];   // partials, then the result

// device address of g_na_scratch per device ordinal; atomic because two host
// threads may make their first call at once (both look up the same address)
std::atomic<double*> g_na_ptr[kNaMaxDevices] = {};

int na_scratch(int ctx_dev, double** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice", __FILE__, __LINE__);
  if (dev != ctx_dev) {
    set_error("spmv_noalloc: device %d is current, the context lives on device %d", dev, ctx_dev);
    return CAPPGPU_E_ARG;
  }
  if (dev < 0 || dev >= kNaMaxDevices) {
    set_error("spmv_noalloc: device ordinal %d beyond %d", dev, kNaMaxDevices);
    return CAPPGPU_E_ARG;
  }
  double* ptr = g_na_ptr[dev].load(std::memory_order_acquire);
  if (!ptr) {   // set-up, once per device, with that device current
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_na_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress", __FILE__, __LINE__);
    ptr = static_cast<double*>(p);
    g_na_ptr[dev].store(ptr, std::memory_order_release);
  }
  *out = ptr;
  return CAPPGPU_OK;
}

// Block b covers interior cells [b*kNaChunk, (b+1)*kNaChunk) of the box
// (j fastest, as Box::at); per cell the arithmetic of k_spmv.  The block's
// partial of pk.zk is summed in a fixed order: per thread over its cells,
// then a fixed tree.
__global__ void k_na_spmv(Dims d, Box b, const double* __restrict__ ae, const double* __restrict__ aw,
                          const double* __restrict__ an, const double* __restrict__ as,
                          const double* __restrict__ at, const double* __restrict__ ab,
                          const double* __restrict__ ap, const double* __restrict__ p, double* z, double* parts) {
  __shared__ double sh[kNaThreads];
  const long long n = b.count();
  const long long base = (long long)blockIdx.x * kNaChunk;
  double v = 0.0;
#pragma unroll
  for (int m = 0; m < kNaPerThread; ++m) {
    const long long t = base + threadIdx.x + (long long)m * kNaThreads;
    if (t < n) {
      int i, j, k;
      b.at(t, i, j, k);
      const int ijk = ixk(d, i, j, k);
      const double r = ap[ijk] * p[ijk] - ae[ijk] * p[ijk + d.nj] - aw[ijk] * p[ijk - d.nj] - an[ijk] * p[ijk + 1] -
                       as[ijk] * p[ijk - 1] - at[ijk] * p[ijk + d.nij] - ab[ijk] * p[ijk - d.nij];
      z[ijk] = r;
      v += p[ijk] * r;
    }
  }
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int s = kNaThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) parts[blockIdx.x] = sh[0];
}

// result = sum of the n partials, fixed order
__global__ void k_na_finish(const double* __restrict__ parts, int n, double* out) {
  __shared__ double sh[kNaThreads];
  double v = 0.0;
  for (int q = threadIdx.x; q < n; q += kNaThreads) v += parts[q];
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int s = kNaThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sh[0];
}

}  // namespace
}  // namespace cap

using namespace cap;

extern "C" {

int cappgpu_spmv_noalloc(int pk, int zk, double* dot) {
  CAP_REQUIRE_INIT();
  if (pk < 0 || pk >= CAP_NFIELDS || zk < 0 || zk >= CAP_NFIELDS || pk == zk || !spmv_output_ok(zk)) {
    set_error("spmv_noalloc: bad fields %d %d (zk may not be a matrix coefficient or a geometry field)", pk, zk);
    return CAPPGPU_E_ARG;
  }
  Ctx& c = ctx();
  const Dims& d = c.d;
  const Box b{3, d.nimm, 3, d.njmm, 3, d.nkmm};
  const long long cells = b.count();
  const long long nparts = (cells + kNaChunk - 1) / kNaChunk;
  if (nparts > kNaMaxParts) {
    set_error("spmv_noalloc: %lld interior cells exceed the fixed scratch (at most %lld)", cells,
              (long long)kNaMaxParts * kNaChunk);
    return CAPPGPU_E_ARG;
  }
  double* scratch = nullptr;
  int rc = na_scratch(c.device, &scratch);
  if (rc) return rc;
  if (nparts > 0) {
    double** F = c.f;
    launch(k_na_spmv, (int)nparts, kNaThreads, c.st, d, b, (const double*)F[CAP_AE], (const double*)F[CAP_AW],
           (const double*)F[CAP_AN], (const double*)F[CAP_AS], (const double*)F[CAP_AT], (const double*)F[CAP_AB],
           (const double*)F[CAP_AP], (const double*)F[pk], F[zk], scratch);
    CAP_CHECK_LAUNCH();
  }
  launch(k_na_finish, 1, kNaThreads, c.st, (const double*)scratch, (int)nparts, scratch + kNaMaxParts);
  CAP_CHECK_LAUNCH();
  if (dot) CAP_CUDA(cudaMemcpyAsync(dot, scratch + kNaMaxParts, sizeof(double), cudaMemcpyDeviceToHost, c.st));
  CAP_CUDA(cudaStreamSynchronize(c.st));
  return CAPPGPU_OK;
}

}  // extern "C"
