// dlayout.cuh -- the hyperplane-major ("diagonal") layout used inside the
// fast SIP-based solvers, plus the memory-ordering helpers of the
// persistent wavefront.
//
// Interior cell (i,j,k), i=3..nimm etc., has local coordinates a=i-3,
// b=j-3, c=k-3 and hyperplane s=a+b+c.  Its diagonal-layout index is
//     D(a,b,c) = (s*Nk + c)*Ni + a
// so that all cells of one hyperplane are contiguous, ordered by (c, a).
// A thread that owns the line (a,c) and walks j meets hyperplane s at
// step s: the threads of a warp (consecutive a) then touch consecutive
// addresses, which the natural j-fastest layout cannot give along a
// diagonal.  The layout holds S*Nk*Ni slots (S = Ni+Nj+Nk-2); only the
// Ni*Nj*Nk slots with 0 <= b < Nj are used.
#pragma once
#include "common.cuh"

namespace cap {

struct DG {
  int Ni, Nj, Nk, S;   // interior extents and hyperplane count
  int nj, nij;         // natural strides
  long long plane;     // Nk*Ni
  __host__ __device__ long long d(int a, int b, int c) const {
    return (long long)(a + b + c) * plane + (long long)c * Ni + a;
  }
  // 0-based natural index of interior-local (a,b,c); valid for a,b,c >= -1
  __host__ __device__ int nat(int a, int b, int c) const { return (c + 2) * nij + (a + 2) * nj + (b + 2); }
  __host__ __device__ long long size() const { return (long long)S * plane; }
};

inline DG make_dg(const Dims& d) {
  DG g;
  g.Ni = d.nimm - 2;
  g.Nj = d.njmm - 2;
  g.Nk = d.nkmm - 2;
  g.S = g.Ni + g.Nj + g.Nk - 2;
  g.nj = d.nj;
  g.nij = d.nij;
  g.plane = (long long)g.Nk * g.Ni;
  return g;
}

// ------------------------------------------------------- memory ordering
__device__ __forceinline__ void st_release_u64(unsigned long long* p, unsigned long long v) {
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void fence_acq_rel_gpu() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }
__device__ __forceinline__ void st_release_cta_shared(unsigned long long* p, unsigned long long v) {
  unsigned a = (unsigned)__cvta_generic_to_shared(p);
  asm volatile("st.release.cta.shared.u64 [%0], %1;" ::"r"(a), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_acquire_cta_shared(const unsigned long long* p) {
  unsigned a = (unsigned)__cvta_generic_to_shared(p);
  unsigned long long v;
  asm volatile("ld.acquire.cta.shared.u64 %0, [%1];" : "=l"(v) : "r"(a) : "memory");
  return v;
}
__device__ __forceinline__ void named_bar_sync(int id, int nthreads) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}
__device__ __forceinline__ int ld_relaxed_i32(const int* p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// ---------------------------------------------------- layout conversion
// natural -> diagonal for the interior box (one thread per interior cell,
// reads coalesced along j)
template <typename T>
__global__ void k_nat_to_d(DG g, const double* __restrict__ src, T* __restrict__ dst) {
  long long n = (long long)g.Ni * g.Nj * g.Nk;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    int b = (int)(t % g.Nj);
    long long r = t / g.Nj;
    int a = (int)(r % g.Ni);
    int c = (int)(r / g.Ni);
    dst[g.d(a, b, c)] = (T)src[g.nat(a, b, c)];
  }
}

// diagonal -> natural for the interior box
template <typename T>
__global__ void k_d_to_nat(DG g, const T* __restrict__ src, double* __restrict__ dst) {
  long long n = (long long)g.Ni * g.Nj * g.Nk;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    int b = (int)(t % g.Nj);
    long long r = t / g.Nj;
    int a = (int)(r % g.Ni);
    int c = (int)(r / g.Ni);
    dst[g.nat(a, b, c)] = (double)src[g.d(a, b, c)];
  }
}

}  // namespace cap
