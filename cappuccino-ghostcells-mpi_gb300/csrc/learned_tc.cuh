// learned_tc.cuh -- the learned guess's 3x3x3 convolution as an implicit
// GEMM on the 5th-generation tensor cores (tcgen05, sm_103a).
//
// One CTA of 128 threads owns a tile of M = 128 consecutive voxels; thread
// i gathers voxel i's row.  For each of the 27 taps the CTA stages in shared
// memory the A tile (128 voxels x CI channels of the tap-shifted input, zero
// outside the grid, optionally masked by a ReLU output) and the B tile (the
// tap's CO x CI weights), both K-major in the no-swizzle canonical layout
// (8-row x 16-byte core matrices; leading-dimension offset = 128 B between
// the two 8-element K halves of a 16-element step, stride-dimension offset
// between 8-row groups = CI/8 x 128 B).  One elected thread issues CI/16
// tcgen05.mma (kind::f16, BF16 in, FP32 accumulate, M=128, N=CO, K=16) into
// a TMEM accumulator of CO columns and commits them to the stage's mbarrier;
// two stages let the gather of tap t+1 overlap the MMAs of tap t.  The
// epilogue reads the accumulator with tcgen05.ld (warp w: lanes 32w..32w+31,
// the tile's rows), adds the bias, applies ReLU and stores BF16.
//
// Every mbarrier wait is bounded; a wait that runs out records an error in
// *err and the CTA leaves at the end of the tile (TMEM is always freed).
#pragma once
#include <cuda_bf16.h>

#include "dlayout.cuh"

namespace cap {
namespace tc {

typedef __nv_bfloat16 bf16;

__host__ __device__ constexpr int pow2_cols(int n) { return n <= 32 ? 32 : (n <= 64 ? 64 : (n <= 128 ? 128 : 256)); }

// instruction descriptor of tcgen05.mma kind::f16: D F32 (bits 4-5 = 1),
// A and B BF16 (bits 7-9, 10-12 = 1), both K-major (bits 15, 16 = 0),
// N >> 3 at bits 17-22, M >> 4 at bits 24-28
__host__ __device__ constexpr unsigned idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned)(N >> 3) << 17) | ((unsigned)(M >> 4) << 24);
}

// shared-memory matrix descriptor, no swizzle: start address >> 4 (bits
// 0-13), leading-dimension byte offset >> 4 (16-29), stride-dimension byte
// offset >> 4 (32-45), descriptor version 1 (bits 46-47), layout 0 (61-63)
__device__ __forceinline__ unsigned long long smem_desc(unsigned addr, unsigned lbo, unsigned sbo) {
  return (unsigned long long)((addr >> 4) & 0x3FFFu) | ((unsigned long long)((lbo >> 4) & 0x3FFFu) << 16) |
         ((unsigned long long)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

__device__ __forceinline__ void tmem_alloc(unsigned* slot, unsigned ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(unsigned taddr, unsigned ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void mma_bf16(unsigned d_tmem, unsigned long long adesc, unsigned long long bdesc,
                                         unsigned idesc, int accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(unsigned long long* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// 16 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld16(unsigned taddr, float (&v)[16]) {
  unsigned r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int q = 0; q < 16; ++q) v[q] = __uint_as_float(r[q]);
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// bounded wait on an mbarrier phase; false if it ran out
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, unsigned parity) {
  for (int it = 0; it < (1 << 20); ++it)
    if (mbar_test(bar, parity)) return true;
  return false;
}

// 8 BF16 channels with the ReLU mask: a channel counts where the mask is > 0
__device__ __forceinline__ uint4 mask8(uint4 u, uint4 m) {
  unsigned* pu = reinterpret_cast<unsigned*>(&u);
  const unsigned* pm = reinterpret_cast<const unsigned*>(&m);
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const unsigned lo = pm[q] & 0xffffu, hi = pm[q] >> 16;
    if (!(lo != 0u && (lo & 0x8000u) == 0u)) pu[q] &= 0xffff0000u;
    if (!(hi != 0u && (hi & 0x8000u) == 0u)) pu[q] &= 0x0000ffffu;
  }
  return u;
}

template <int CI, int CO>
struct ConvTC {
  static constexpr int kA = 128 * CI * 2;               // A tile bytes
  static constexpr int kB = CO * CI * 2;                // B tile bytes
  static constexpr int kStage = (kA + kB + 1023) & ~1023;
  static constexpr int kSboA = CI / 8 * 128;            // 8-row group stride (A and B)
  static constexpr int kCols = pow2_cols(CO);
  // 2 stages, alignment slack, barriers + TMEM slot; at least kCols/512 of
  // the SM's 228 KB so that the CTAs an SM holds never ask for more than its
  // 512 TMEM columns together
  static constexpr int kSmemUse = 2 * kStage + 1024 + 64;
  static constexpr int kSmemTmem = kCols * (228 * 1024 / 512);
  static constexpr int kSmem = kSmemUse > kSmemTmem ? kSmemUse : kSmemTmem;
  static_assert(CI % 16 == 0 && CO % 16 == 0 && CO <= 256, "tile shape");
};

// y = act(conv3x3x3(x * [mask > 0], w) + bias): x has CI channels at pitch
// ldx, w is [CO][27][CI], y gets CO channels at pitch ldy.
template <int CI, int CO, bool MASK>
__global__ void __launch_bounds__(128) k_conv3_tc(const bf16* __restrict__ x, int ldx, const bf16* __restrict__ w,
                                                  const float* __restrict__ bias, const bf16* __restrict__ mask,
                                                  int ldm, bf16* __restrict__ y, int ldy, int D, int H, int W,
                                                  int relu, int* err) {
  typedef ConvTC<CI, CO> T;
  extern __shared__ unsigned char smem_raw[];
  unsigned char* smem = (unsigned char*)(((unsigned long long)smem_raw + 1023) & ~1023ull);
  unsigned long long* bar = (unsigned long long*)(smem + 2 * T::kStage);
  unsigned* tslot = (unsigned*)(bar + 2);
  const int tid = threadIdx.x, warp = tid >> 5;
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_fence_init();
  }
  if (warp == 0) tmem_alloc(tslot, T::kCols);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const unsigned tmem = *tslot;
  constexpr unsigned idesc = idesc_bf16(128, CO);
  const int V = D * H * W;
  const int ntiles = (V + 127) / 128;
  unsigned phase[2] = {0u, 0u};
  bool pending[2] = {false, false};
  bool bad = false;
  int it = 0;   // tap iterations issued by this CTA (selects the stage)
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int v = tile * 128 + tid;
    const bool valid = v < V;
    const int x0 = valid ? v % W : 0, r0 = valid ? v / W : 0;
    const int y0 = r0 % H, z0 = r0 / H;
    // operand rows of one tap in registers: the A row of this thread's voxel
    // (masked) and this thread's share of the tap's weights
    constexpr int NB = (CO * CI / 8 + 127) / 128;
    uint4 an[CI / 8], bn[NB];
    auto fetch = [&](int tap) {
      const int dz = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
      const int zz = z0 + dz, yy = y0 + dy, xx = x0 + dx;
      const bool in = valid && (unsigned)zz < (unsigned)D && (unsigned)yy < (unsigned)H && (unsigned)xx < (unsigned)W;
      const long long n = in ? (long long)v + (dz * H + dy) * W + dx : 0;
#pragma unroll
      for (int kc = 0; kc < CI / 8; ++kc) {
        uint4 u = make_uint4(0u, 0u, 0u, 0u);
        if (in) {
          u = *reinterpret_cast<const uint4*>(x + n * ldx + kc * 8);
          if (MASK) u = mask8(u, *reinterpret_cast<const uint4*>(mask + n * ldm + kc * 8));
        }
        an[kc] = u;
      }
#pragma unroll
      for (int j = 0; j < NB; ++j) {
        const int q = tid + 128 * j;
        if (q < CO * CI / 8) {
          const int co = q / (CI / 8), kc = q - co * (CI / 8);
          bn[j] = *reinterpret_cast<const uint4*>(w + ((size_t)co * 27 + tap) * CI + kc * 8);
        }
      }
    };
    fetch(0);
    for (int tap = 0; tap < 27; ++tap, ++it) {
      uint4 ac[CI / 8], bc[NB];
#pragma unroll
      for (int kc = 0; kc < CI / 8; ++kc) ac[kc] = an[kc];
#pragma unroll
      for (int j = 0; j < NB; ++j) bc[j] = bn[j];
      if (tap + 1 < 27) fetch(tap + 1);   // in flight while this tap is staged and multiplied
      const int s = it & 1;
      if (pending[s]) {   // the MMAs that last read this stage are done
        if (!bad && !mbar_wait_bounded(&bar[s], phase[s])) bad = true;
        phase[s] ^= 1u;
        pending[s] = false;
      }
      unsigned char* A = smem + s * T::kStage;
      unsigned char* B = A + T::kA;
      unsigned char* arow = A + (tid >> 3) * T::kSboA + (tid & 7) * 16;
#pragma unroll
      for (int kc = 0; kc < CI / 8; ++kc) *reinterpret_cast<uint4*>(arow + kc * 128) = ac[kc];
#pragma unroll
      for (int j = 0; j < NB; ++j) {
        const int q = tid + 128 * j;
        if (q < CO * CI / 8) {
          const int co = q / (CI / 8), kc = q - co * (CI / 8);
          *reinterpret_cast<uint4*>(B + (co >> 3) * T::kSboA + kc * 128 + (co & 7) * 16) = bc[j];
        }
      }
      fence_proxy_async_smem();
      __syncthreads();
      if (tid == 0) {
        tc_fence_after();
        const unsigned a0 = smem_u32(A), b0 = smem_u32(B);
#pragma unroll
        for (int ks = 0; ks < CI / 16; ++ks)
          mma_bf16(tmem, smem_desc(a0 + ks * 256, 128, T::kSboA), smem_desc(b0 + ks * 256, 128, T::kSboA), idesc,
                   (tap | ks) != 0);
        mma_commit(&bar[s]);
      }
      pending[s] = true;
    }
    // the last commit tracks every MMA of the tile
    const int sl = (it - 1) & 1;
    if (!bad && !mbar_wait_bounded(&bar[sl], phase[sl])) bad = true;
    phase[sl] ^= 1u;
    pending[sl] = false;
    tc_fence_after();
    const unsigned trow = tmem + ((unsigned)(warp * 32) << 16);
#pragma unroll
    for (int c0 = 0; c0 < CO; c0 += 16) {
      float acc[16];
      tmem_ld16(trow + c0, acc);
      tmem_wait_ld();
      if (valid) {
        unsigned pk[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          float a = acc[2 * q], b = acc[2 * q + 1];
          if (bias) {
            a += bias[c0 + 2 * q];
            b += bias[c0 + 2 * q + 1];
          }
          if (relu) {
            a = fmaxf(a, 0.f);
            b = fmaxf(b, 0.f);
          }
          const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
          pk[q] = *reinterpret_cast<const unsigned*>(&h);
        }
        uint4* dst = reinterpret_cast<uint4*>(y + (long long)v * ldy + c0);
        dst[0] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
        dst[1] = make_uint4(pk[4], pk[5], pk[6], pk[7]);
      }
    }
    tc_fence_before();
    if (__syncthreads_or(bad)) break;
  }
  // drain the other stage's last commit, then free TMEM
  for (int s = 0; s < 2; ++s)
    if (pending[s] && !bad && !mbar_wait_bounded(&bar[s], phase[s])) bad = true;
  if (bad && tid == 0) atomicExch(err, 1);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) tmem_dealloc(tmem, T::kCols);
}

}  // namespace tc
}  // namespace cap

namespace cap {
namespace tc {

// Halo-tile form.  An output tile is 8 (x) x 16 (y) voxels of one z-plane
// (M = 128 rows, row r = (x = r % 8, y = r / 8)).  The CTA stages the tile's
// input halo, 10 x 18 x 3 voxels, once: each 8-channel group is a plane of
// 540 rows of 16 bytes, row (hz*18 + hy)*10 + hx.  For tap (dz, dy, dx) the
// A operand is that plane read from row ((1+dz)*18 + 1+dy)*10 + 1+dx on:
// 8 consecutive rows (x) form a core matrix, row groups (y) are 10 rows =
// 160 B apart (stride-dimension offset) and the two 8-channel halves of a
// 16-channel K step are one plane apart (leading-dimension offset), so a tap
// costs only a descriptor.  All 27 taps' weights stay in shared memory for
// the CTA's life.  One elected thread issues the tile's 27 x CI/16 MMAs.
template <int CI, int CO>
struct HaloTC {
  static constexpr int HX = 10, HY = 18, HZ = 3, HV = HX * HY * HZ;
  static constexpr int NC = CI / 8;                      // 8-channel groups
  static constexpr int kPlane = HV * 16;                 // bytes of one group's plane
  static constexpr int kA = (NC * kPlane + 1023) & ~1023;
  static constexpr int kB = (27 * CO * CI * 2 + 1023) & ~1023;
  static constexpr int kSboB = CI / 8 * 128;
  static constexpr int kCols = pow2_cols(CO);
  static constexpr int kSmemUse = kA + kB + 1024 + 64;
  static constexpr int kSmemTmem = kCols * (228 * 1024 / 512);
  static constexpr int kSmem = kSmemUse > kSmemTmem ? kSmemUse : kSmemTmem;
  static constexpr bool kFits = kSmem <= 220 * 1024;
  static_assert(CI % 16 == 0 && CO % 16 == 0 && CO <= 256, "tile shape");
};

template <int CI, int CO, bool MASK>
__global__ void __launch_bounds__(128) k_conv3_halo(const bf16* __restrict__ x, int ldx, const bf16* __restrict__ w,
                                                    const float* __restrict__ bias, const bf16* __restrict__ mask,
                                                    int ldm, bf16* __restrict__ y, int ldy, int D, int H, int W,
                                                    int relu, int* err) {
  typedef HaloTC<CI, CO> T;
  extern __shared__ unsigned char smem_raw[];
  unsigned char* smem = (unsigned char*)(((unsigned long long)smem_raw + 1023) & ~1023ull);
  unsigned char* A = smem;
  unsigned char* B = smem + T::kA;
  unsigned long long* bar = (unsigned long long*)(B + T::kB);
  unsigned* tslot = (unsigned*)(bar + 1);
  const int tid = threadIdx.x, warp = tid >> 5;
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_fence_init();
  }
  if (warp == 0) tmem_alloc(tslot, T::kCols);
  // the weights of all taps, K-major per tap
  for (int q = tid; q < 27 * CO * T::NC; q += 128) {
    const int tap = q / (CO * T::NC), r = q - tap * (CO * T::NC);
    const int co = r / T::NC, kc = r - co * T::NC;
    const uint4 u = *reinterpret_cast<const uint4*>(w + ((size_t)co * 27 + tap) * CI + kc * 8);
    *reinterpret_cast<uint4*>(B + tap * (CO * CI * 2) + (co >> 3) * T::kSboB + kc * 128 + (co & 7) * 16) = u;
  }
  fence_proxy_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const unsigned tmem = *tslot;
  constexpr unsigned idesc = idesc_bf16(128, CO);
  const int ntx = (W + 7) / 8, nty = (H + 15) / 16;
  const int ntiles = ntx * nty * D;
  unsigned phase = 0u;
  bool bad = false;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int tx = tile % ntx, ty = (tile / ntx) % nty, z0 = tile / (ntx * nty);
    const int x0 = tx * 8, y0 = ty * 16;
    // input halo, zero outside the grid
    for (int q = tid; q < T::HV * T::NC; q += 128) {
      const int hv = q / T::NC, kc = q - hv * T::NC;
      const int hx = hv % T::HX, hy = (hv / T::HX) % T::HY, hz = hv / (T::HX * T::HY);
      const int gx = x0 - 1 + hx, gy = y0 - 1 + hy, gz = z0 - 1 + hz;
      uint4 u = make_uint4(0u, 0u, 0u, 0u);
      if ((unsigned)gx < (unsigned)W && (unsigned)gy < (unsigned)H && (unsigned)gz < (unsigned)D) {
        const long long n = ((long long)gz * H + gy) * W + gx;
        u = *reinterpret_cast<const uint4*>(x + n * ldx + kc * 8);
        if (MASK) u = mask8(u, *reinterpret_cast<const uint4*>(mask + n * ldm + kc * 8));
      }
      *reinterpret_cast<uint4*>(A + kc * T::kPlane + hv * 16) = u;
    }
    fence_proxy_async_smem();
    __syncthreads();
    if (tid == 0) {
      tc_fence_after();
      const unsigned a0 = smem_u32(A), b0 = smem_u32(B);
      for (int tap = 0; tap < 27; ++tap) {
        const int dz = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
        const unsigned row = (unsigned)(((1 + dz) * T::HY + 1 + dy) * T::HX + 1 + dx);
#pragma unroll
        for (int ks = 0; ks < CI / 16; ++ks)
          mma_bf16(tmem, smem_desc(a0 + 2 * ks * T::kPlane + row * 16, T::kPlane, T::HX * 16),
                   smem_desc(b0 + tap * (CO * CI * 2) + ks * 256, 128, T::kSboB), idesc, (tap | ks) != 0);
      }
      mma_commit(&bar[0]);
    }
    if (!bad && !mbar_wait_bounded(&bar[0], phase)) bad = true;
    phase ^= 1u;
    tc_fence_after();
    const int ox = x0 + (tid & 7), oy = y0 + (tid >> 3);
    const bool valid = ox < W && oy < H;
    const long long v = ((long long)z0 * H + oy) * W + ox;
    const unsigned trow = tmem + ((unsigned)(warp * 32) << 16);
#pragma unroll
    for (int c0 = 0; c0 < CO; c0 += 16) {
      float acc[16];
      tmem_ld16(trow + c0, acc);
      tmem_wait_ld();
      if (valid) {
        unsigned pk[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          float a = acc[2 * q], b = acc[2 * q + 1];
          if (bias) {
            a += bias[c0 + 2 * q];
            b += bias[c0 + 2 * q + 1];
          }
          if (relu) {
            a = fmaxf(a, 0.f);
            b = fmaxf(b, 0.f);
          }
          const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
          pk[q] = *reinterpret_cast<const unsigned*>(&h);
        }
        uint4* dst = reinterpret_cast<uint4*>(y + v * ldy + c0);
        dst[0] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
        dst[1] = make_uint4(pk[4], pk[5], pk[6], pk[7]);
      }
    }
    tc_fence_before();
    if (__syncthreads_or(bad)) break;
  }
  if (bad && tid == 0) atomicExch(err, 1);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) tmem_dealloc(tmem, T::kCols);
}

}  // namespace tc
}  // namespace cap

namespace cap {
namespace tc {

// Weight gradient on the halo tile: for the taps t of a group and the
// tiles of a chunk, G_t[co][ci] += sum over the tile's voxels v of
// gm[v][co] x[v + off(t)][ci], gm = gy masked by the layer's ReLU output.
// Both operands are MN-major in shared memory (the 16-byte rows run along
// the channels, consecutive rows along the voxels = K).  Without swizzling
// the leading-dimension offset is the step between core matrices along K
// and the stride-dimension offset the step along M/N, for either major: A
// is the tile's 128 rows of gm, one 2 KB plane per 8 output channels,
// padded with zero planes to M = 128 (leading offset 128 B between 8-voxel
// groups, stride offset 2 KB between channel groups); B is the input halo of
// the forward kernel read from the tap's shifted row (leading offset 160 B
// = one tile row, stride offset one plane).  The group's taps accumulate side by side
// in TMEM (CI columns each); the CTA writes its partial sums for the
// chunk, summed over chunks in a fixed order afterwards.
template <int CI, int CO>
struct WgradTC {
  static constexpr int NC = CI / 8, NG = CO / 8;
  static constexpr int kPlaneB = HaloTC<CI, 16>::kPlane;   // 540 rows of 16 B
  static constexpr int kB = (NC * kPlaneB + 1023) & ~1023;
  static constexpr int kPlaneA = 128 * 16;
  static constexpr int kA = 16 * kPlaneA;                  // M = 128
  static constexpr int kTG = (256 / CI) < 27 ? (256 / CI) : 27;   // taps per group
  static constexpr int kCols = pow2_cols(kTG * CI);
  static constexpr int kSmemUse = kB + kA + 1024 + 64;
  static constexpr int kSmemTmem = kCols * (228 * 1024 / 512);
  static constexpr int kSmem = kSmemUse > kSmemTmem ? kSmemUse : kSmemTmem;
  static_assert(CI % 16 == 0 && CO % 8 == 0 && CO <= 128, "tile shape");
};

// instruction descriptor, both operands MN-major (bits 15, 16 = 1)
__host__ __device__ constexpr unsigned idesc_bf16_mn(int M, int N) { return idesc_bf16(M, N) | (1u << 15) | (1u << 16); }

template <int CI, int CO>
__global__ void __launch_bounds__(128) k_wgrad_halo(const bf16* __restrict__ x, int ldx, const bf16* __restrict__ gy,
                                                    int ldg, const bf16* __restrict__ y, int ldy,
                                                    float* __restrict__ part, int D, int H, int W, int tiles_per_chunk,
                                                    int* err) {
  typedef WgradTC<CI, CO> T;
  typedef HaloTC<CI, 16> Hl;
  extern __shared__ unsigned char smem_raw[];
  unsigned char* smem = (unsigned char*)(((unsigned long long)smem_raw + 1023) & ~1023ull);
  unsigned char* B = smem;              // halo planes (B first: an overrun lands in A)
  unsigned char* A = smem + T::kB;      // gm planes
  unsigned long long* bar = (unsigned long long*)(A + T::kA);
  unsigned* tslot = (unsigned*)(bar + 1);
  const int tid = threadIdx.x, warp = tid >> 5;
  const int tap0 = blockIdx.x * T::kTG;
  const int ntap = 27 - tap0 < T::kTG ? 27 - tap0 : T::kTG;
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_fence_init();
  }
  if (warp == 0) tmem_alloc(tslot, T::kCols);
  // the padding planes of A (output channels CO..127) stay zero
  for (int q = tid; q < (16 - T::NG) * T::kPlaneA / 16; q += 128)
    reinterpret_cast<uint4*>(A + T::NG * T::kPlaneA)[q] = make_uint4(0u, 0u, 0u, 0u);
  fence_proxy_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const unsigned tmem = *tslot;
  constexpr unsigned idesc = idesc_bf16_mn(128, CI);
  const int ntx = (W + 7) / 8, nty = (H + 15) / 16;
  const int ntiles = ntx * nty * D;
  const int t_begin = blockIdx.y * tiles_per_chunk;
  const int t_end = t_begin + tiles_per_chunk < ntiles ? t_begin + tiles_per_chunk : ntiles;
  unsigned phase = 0u;
  bool bad = false, first = true;
  for (int tile = t_begin; tile < t_end; ++tile) {
    const int tx = tile % ntx, ty = (tile / ntx) % nty, z0 = tile / (ntx * nty);
    const int x0 = tx * 8, y0 = ty * 16;
    for (int q = tid; q < Hl::HV * T::NC; q += 128) {   // input halo, zero outside the grid
      const int hv = q / T::NC, kc = q - hv * T::NC;
      const int hx = hv % Hl::HX, hy = (hv / Hl::HX) % Hl::HY, hz = hv / (Hl::HX * Hl::HY);
      const int gx = x0 - 1 + hx, gyy = y0 - 1 + hy, gz = z0 - 1 + hz;
      uint4 u = make_uint4(0u, 0u, 0u, 0u);
      if ((unsigned)gx < (unsigned)W && (unsigned)gyy < (unsigned)H && (unsigned)gz < (unsigned)D)
        u = *reinterpret_cast<const uint4*>(x + (((long long)gz * H + gyy) * W + gx) * ldx + kc * 8);
      *reinterpret_cast<uint4*>(B + kc * T::kPlaneB + hv * 16) = u;
    }
    {   // the tile's masked output gradient, row = tid (x = tid % 8, y = tid / 8)
      const int ox = x0 + (tid & 7), oy = y0 + (tid >> 3);
      const bool valid = ox < W && oy < H;
      const long long v = ((long long)z0 * H + oy) * W + ox;
#pragma unroll
      for (int kc = 0; kc < T::NG; ++kc) {
        uint4 u = make_uint4(0u, 0u, 0u, 0u);
        if (valid)
          u = mask8(*reinterpret_cast<const uint4*>(gy + v * ldg + kc * 8),
                    *reinterpret_cast<const uint4*>(y + v * ldy + kc * 8));
        *reinterpret_cast<uint4*>(A + kc * T::kPlaneA + tid * 16) = u;
      }
    }
    fence_proxy_async_smem();
    __syncthreads();
    if (tid == 0) {
      tc_fence_after();
      const unsigned a0 = smem_u32(A), b0 = smem_u32(B);
      for (int j = 0; j < ntap; ++j) {
        const int tap = tap0 + j;
        const int dz = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
        const unsigned row = (unsigned)(((1 + dz) * Hl::HY + 1 + dy) * Hl::HX + 1 + dx);
#pragma unroll
        for (int ks = 0; ks < 8; ++ks)
          mma_bf16(tmem + (unsigned)(j * CI), smem_desc(a0 + ks * 256, 128, T::kPlaneA),
                   smem_desc(b0 + row * 16 + ks * 320, Hl::HX * 16, T::kPlaneB), idesc, (!first || ks) ? 1 : 0);
      }
      mma_commit(&bar[0]);
    }
    if (!bad && !mbar_wait_bounded(&bar[0], phase)) bad = true;
    phase ^= 1u;
    first = false;
    tc_fence_before();
    if (__syncthreads_or(bad)) break;
    tc_fence_after();
  }
  // partial sums of the chunk: lane co, CI columns per tap
  if (t_begin < t_end && !bad && warp * 32 < CO) {
    const int co = warp * 32 + (tid & 31);
    const unsigned trow = tmem + ((unsigned)(warp * 32) << 16);
    for (int j = 0; j < ntap; ++j) {
#pragma unroll
      for (int c0 = 0; c0 < CI; c0 += 16) {
        float acc[16];
        tmem_ld16(trow + (unsigned)(j * CI + c0), acc);
        tmem_wait_ld();
        if (co < CO) {
          float* dst = part + (((size_t)blockIdx.y * 27 + tap0 + j) * CO + co) * CI + c0;
#pragma unroll
          for (int q = 0; q < 16; ++q) dst[q] = acc[q];
        }
      }
    }
  } else if (t_begin >= t_end && warp * 32 < CO) {   // an empty chunk adds nothing
    const int co = warp * 32 + (tid & 31);
    if (co < CO)
      for (int j = 0; j < ntap; ++j)
        for (int c = 0; c < CI; ++c) part[(((size_t)blockIdx.y * 27 + tap0 + j) * CO + co) * CI + c] = 0.f;
  }
  if (bad && tid == 0) atomicExch(err, 1);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) tmem_dealloc(tmem, T::kCols);
}

}  // namespace tc
}  // namespace cap
