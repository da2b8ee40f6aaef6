// dlayout.cuh -- the hyperplane-major ("diagonal") layout used inside the
// fast SIP-based solvers, plus the memory-ordering, mbarrier and TMA helpers
// of the persistent wavefront.
//
// Interior cell (i,j,k), i=3..nimm etc., has local coordinates a=i-3,
// b=j-3, c=k-3 and hyperplane s=a+b+c.  Its diagonal-layout index is
//     D(a,b,c) = (s*Nk + c)*P + a          (P = pitch >= Ni, multiple of 4)
// so that all cells of one hyperplane are contiguous rows ordered by c.
// A thread that owns the line (a,c) and walks j meets hyperplane s at
// step s: the threads of a warp (consecutive a) then touch consecutive
// addresses, which the natural j-fastest layout cannot give along a
// diagonal.  The layout holds S*Nk*P slots (S = Ni+Nj+Nk-2); only the
// Ni*Nj*Nk slots with a < Ni and 0 <= b < Nj are used.  The pitch makes every
// row of doubles or floats start on a 16-byte boundary, which the
// tensor-memory-access (TMA) copies of the wavefront require.
//
// In row order -- rows (s,c) by s, then c; cells of a row by a -- the cells
// form one compact sequence; chunk q of 32 consecutive cells starts at the
// cell recorded in chunk[q] (the vector kernels walk it).
//
// Factors with several components per cell use the component-major variant
//     Dc(a,b,c,q) = ((s*Nk + c)*NQ + q)*P + a
// so that one component of a row of cells is contiguous.
#pragma once
#include "common.cuh"

namespace cap {

struct DG {
  int Ni, Nj, Nk, S;   // interior extents and hyperplane count
  int P;               // row pitch (Ni rounded up to a multiple of 4)
  int nj, nij;         // natural strides
  int kb;              // natural k-plane index (0-based) of c = 0: 2 (k = 3) for the interior box,
                       // 1 (k = 2) for the box that also holds the k ghost layers
  long long plane;     // Nk*P
  long long ncell;     // Ni*Nj*Nk
  int nchunk;          // ceil(ncell / 32)
  const int4* chunk;   // (s, c, a) of the first cell of each 32-cell chunk
  __host__ __device__ long long d(int a, int b, int c) const {
    return (long long)(a + b + c) * plane + (long long)c * P + a;
  }
  // component q of NQ at (a,b,c)
  __host__ __device__ long long dq(int a, int b, int c, int q, int NQ) const {
    return dqs(a + b + c, c, a, q, NQ);
  }
  // the same from the cell's hyperplane s = a+b+c
  __host__ __device__ long long dqs(int s, int c, int a, int q, int NQ) const {
    return ((long long)s * Nk * NQ + (long long)c * NQ + q) * P + a;
  }
  // 0-based natural index of box-local (a,b,c); valid for a,b,c >= -1
  __host__ __device__ int nat(int a, int b, int c) const { return (c + kb) * nij + (a + 2) * nj + (b + 2); }
  __host__ __device__ long long size() const { return (long long)S * plane; }
};

// the box i = 3..nimm, j = 3..njmm and k = 3..nkmm (the interior), or with
// ghost_k k = 2..nkm (the loops of iccg.f90 and cgstab*.f90)
inline DG make_dg(const Dims& d, bool ghost_k = false) {
  DG g;
  g.Ni = d.nimm - 2;
  g.Nj = d.njmm - 2;
  g.Nk = d.nkmm - 2 + (ghost_k ? 2 : 0);
  g.kb = ghost_k ? 1 : 2;
  g.S = g.Ni + g.Nj + g.Nk - 2;
  g.P = (g.Ni + 3) & ~3;
  g.nj = d.nj;
  g.nij = d.nij;
  g.plane = (long long)g.Nk * g.P;
  g.ncell = (long long)g.Ni * g.Nj * g.Nk;
  g.nchunk = (int)((g.ncell + 31) / 32);
  g.chunk = nullptr;
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
// named barrier that also returns the OR of a predicate over its participants
__device__ __forceinline__ bool named_bar_red_or(int id, int nthreads, bool v) {
  unsigned r;
  asm volatile(
      "{\n .reg .pred p, q;\n setp.ne.u32 p, %1, 0;\n bar.red.or.pred q, %2, %3, p;\n selp.u32 %0, 1, 0, q;\n}"
      : "=r"(r)
      : "r"((unsigned)v), "r"(id), "r"(nthreads)
      : "memory");
  return r != 0;
}
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ unsigned long long ld_relaxed_b64(const void* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed_b64(void* p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ int ld_relaxed_i32(const int* p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// ------------------------------------------------------- mbarrier / TMA
__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long* b, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive(unsigned long long* b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(b)) : "memory");
}
__device__ __forceinline__ void mbar_arrive_tx(unsigned long long* b, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_test(unsigned long long* b, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
// 3-D / 4-D tiled tensor loads into shared memory, completion on an mbarrier
__device__ __forceinline__ void tma_load3(void* dst, const void* map, int x, int y, int z, unsigned long long* b) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
      ::"r"(smem_u32(dst)), "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(b))
      : "memory");
}
__device__ __forceinline__ void tma_load4(void* dst, const void* map, int x, int q, int y, int z, unsigned long long* b) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], [%6];"
      ::"r"(smem_u32(dst)), "l"(map), "r"(x), "r"(q), "r"(y), "r"(z), "r"(smem_u32(b))
      : "memory");
}

// L2 prefetch of a tiled box (no shared memory, no completion to wait for):
// a later copy of the same box then reads from L2 instead of HBM
__device__ __forceinline__ void tma_prefetch3(const void* map, int x, int y, int z) {
  asm volatile("cp.async.bulk.prefetch.tensor.3d.L2.global.tile [%0, {%1, %2, %3}];" ::"l"(map), "r"(x), "r"(y), "r"(z)
               : "memory");
}
__device__ __forceinline__ void tma_prefetch4(const void* map, int x, int q, int y, int z) {
  asm volatile("cp.async.bulk.prefetch.tensor.4d.L2.global.tile [%0, {%1, %2, %3, %4}];" ::"l"(map), "r"(x), "r"(q),
               "r"(y), "r"(z)
               : "memory");
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

// natural -> diagonal copies of up to kConvMax fields in one launch, and
// FP32 copies of those with a non-null dst32.  A block transposes a 32 x 32
// (a, b) tile of one c-plane through shared memory: it reads the tile along
// b (contiguous in the natural layout) and writes it by anti-diagonals
// a + b = const, each a contiguous run of one hyperplane row -- the
// one-thread-per-cell copy above reads coalesced but writes every element
// one hyperplane apart.  Grid: (ceil(Ni/32), ceil(Nj/32), Nk), 256 threads.
constexpr int kConvMax = 9;
struct ConvList {
  const double* src[kConvMax];
  double* dst[kConvMax];    // null: no FP64 copy
  float* dst32[kConvMax];   // null: no FP32 copy
  int n;
};

static __global__ void __launch_bounds__(256) k_nat_to_d_tiles(DG g, ConvList L) {
  __shared__ double tile[32][34];   // row pitch 34: the anti-diagonal reads fall in distinct banks
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int a0 = blockIdx.x * 32, b0 = blockIdx.y * 32, c = blockIdx.z;
  for (int q = 0; q < L.n; ++q) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int i = ty + 8 * k, a = a0 + i, b = b0 + tx;
      if (a < g.Ni && b < g.Nj) tile[i][tx] = L.src[q][g.nat(a, b, c)];
    }
    __syncthreads();
    for (int m = ty; m < 63; m += 8) {   // anti-diagonal i + j = m of the tile
      const int i = (m > 31 ? m - 31 : 0) + tx, j = m - i;
      const int a = a0 + i, b = b0 + j;
      if (i <= (m < 31 ? m : 31) && a < g.Ni && b < g.Nj) {
        const double v = tile[i][j];
        const long long d = g.d(a, b, c);
        if (L.dst[q]) L.dst[q][d] = v;
        if (L.dst32[q]) L.dst32[q][d] = (float)v;
      }
    }
    __syncthreads();
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
