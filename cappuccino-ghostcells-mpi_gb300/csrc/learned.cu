// learned.cu -- the learned initial guess of the pressure solve
// (cappgpu_precision(2); no counterpart in the reference).
//
// A 3-level 3-D convolutional U-Net predicts the correction d of a pressure
// solve, A d = r0, from the solve's initial residual r0.  Inputs are
// normalised by the RMS of r0 and the operator by the mean of its diagonal
// (r^ = r0/rms, A^ = A/mean(ap)); the net's output d^ is trained to make
// A^ d^ = r^ on the residual-norm loss |A^ d^ - r^|^2 / |r^|^2, with A^ the
// 7-point operator of the recorded solve restricted to the training window.
// At solve time the amplitude and the level of the guess, fi + alpha d +
// beta over the interior, come from a Galerkin projection onto span{d, 1}
// (two products with A): the energy-norm error of CG's start cannot grow.  The plain solve
// always continues from the guess to the same tolerance -- the exit test
// stays relative to the residual of the solve's own start -- so the solver
// is both judge and fallback: a guess that does not lower the FP64 residual
// is discarded.
//
// Net (channels 16/32/64, 3x3x3 kernels, ReLU, zero padding):
//   level 1  e1a 1->16, e1b 16->16 ............ d1a 48->16, d1b 16->16, 1x1x1 16->1
//   level 2  avg-pool 2, e2a 16->32, e2b 32->32 ... d2a 96->32, d2b 32->32, nearest-up 2
//   level 3  avg-pool 2, e3a 32->64, e3b 64->64, nearest-up 2
// The decoder's input at each level is the up-sampled coarser output
// followed by the encoder's output of that level (channel concatenation,
// written in place by the producing layer).  Grid extents are multiples of 4
// (the solve's interior is zero-padded up to that).
//
// Activations and weights are BF16, accumulation FP32, FP32 master weights,
// Adam.  Convolutions are implicit GEMMs on the tensor cores: forward and
// input gradient (the same kernel with flipped, transposed weights and the
// ReLU mask of the layer's output) as tcgen05 MMAs into TMEM, 128 voxels x
// all output channels per CTA and K = 27 taps x input channels
// (learned_tc.cuh); an mma.sync m16n8k16 form of the same convolution (16
// voxels x 16 output channels per warp) is kept for cross-checks
// (cappgpu_set_option("learn_conv", 0)).  The weight gradient is a GEMM
// over voxels per tap (mma.sync), split in chunks and summed in a fixed
// order.  Training pairs are recorded by the solver itself
// (cappgpu_learn_collect) and the net is trained on random cubic windows of
// them (cappgpu_learn_train).
#include <cuda_bf16.h>
#include <math.h>
#include <string.h>

#include <vector>

#include "common.cuh"
#include "kernels.cuh"
#include "learned_tc.cuh"

namespace cap {

namespace {

typedef __nv_bfloat16 bf16;

// ------------------------------------------------------------ the layers
constexpr int kNL = 10;   // 3x3x3 layers in execution order
constexpr int kCI[kNL] = {16, 16, 16, 32, 32, 64, 96, 32, 48, 16};   // layer 0: 1 used of 16
constexpr int kCO[kNL] = {16, 16, 32, 32, 64, 64, 32, 32, 16, 16};
constexpr int kC1 = 16;   // channels at the output of the last 3x3x3 layer
constexpr int wsize(int l) { return kCO[l] * 27 * kCI[l]; }
constexpr int woff(int l) { return l == 0 ? 0 : woff(l - 1) + wsize(l - 1); }                // BF16 weight arrays
constexpr int offW(int l) { return l == 0 ? 0 : offW(l - 1) + wsize(l - 1) + kCO[l - 1]; }   // parameters
constexpr int offB(int l) { return offW(l) + wsize(l); }
constexpr int kWAll = woff(kNL - 1) + wsize(kNL - 1);
constexpr int kOffLastW = offB(kNL - 1) + kCO[kNL - 1];
constexpr int kOffLastB = kOffLastW + kC1;
constexpr int kParams = kOffLastB + 1;
constexpr int kChunk = 8192;   // voxels per weight-gradient partial
constexpr int kPlanes = 9;     // planes of a recorded pair: r^, A^ (7), the converged correction t^

__constant__ int cCI[kNL] = {16, 16, 16, 32, 32, 64, 96, 32, 48, 16};
__constant__ int cCO[kNL] = {16, 16, 32, 32, 64, 64, 32, 32, 16, 16};
__constant__ int cWoff[kNL] = {woff(0), woff(1), woff(2), woff(3), woff(4),
                               woff(5), woff(6), woff(7), woff(8), woff(9)};
__constant__ int cOffW[kNL] = {offW(0), offW(1), offW(2), offW(3), offW(4),
                               offW(5), offW(6), offW(7), offW(8), offW(9)};

// activation and gradient buffers of one grid size (level 1: V1 voxels)
struct Acts {
  long long V1 = 0;
  bf16 *a0, *a1, *cat1, *p1, *a3, *cat2, *p2, *a5, *b3, *a7, *x2, *a9, *x1;
  bf16 *gx1, *ga9, *gcat1, *gx2, *ga7, *gcat2, *gb3, *ga5, *gp2, *ga3, *gp1, *ga1;
  float *out, *gout, *rhs, *coef, *res, *tgt;
  void* base = nullptr;
};

struct Net {
  bool ready = false, trained = false, collect = false;
  float *p = nullptr, *gp = nullptr, *m = nullptr, *v = nullptr;   // parameters, gradients, Adam moments
  bf16* wb = nullptr;    // BF16 conv weights, layer l at woff(l): [co][tap][ci]
  bf16* wt = nullptr;    // flipped, transposed, layer l at woff(l): [ci][tap][co] (input gradient)
  int adam_t = 0;
  Acts A;
  float* part = nullptr;         // partial sums
  size_t part_n = 0;
  double* dsum = nullptr;        // device scalars: loss
  int* err = nullptr;            // set by a tensor-core convolution whose wait ran out
  // recorded pairs: [sample][kPlanes][sV]: r^, then A^ as xp, xm, yp, ym, zp,
  // zm, diag, then the solve's converged correction t^ on the same scale
  // (A^ t^ = r^ to the solve's tolerance); a sample is the whole interior,
  // or (window mode, wper > 0) a random sD^3 window of it, wper windows per
  // recorded solve
  int max_samples = 0, nsamples = 0, next = 0;
  int sD = 0, sH = 0, sW = 0;
  int wper = 0;
  unsigned long long wrng = 0;   // window origins (xorshift64*)
  float* store = nullptr;
  // the solve being recorded: fi at its start, the start's scale sums
  // (|r0|^2, sum ap) and the samples whose t^ its end fills (slot, z0, y0, x0)
  double* fi0 = nullptr;
  long long fi0_n = 0;
  double* tsum = nullptr;
  std::vector<int4> pend;
  // training loss: 0 residual norm |A^ d - r^|^2/|r^|^2 (the learned-guess
  // configuration's), 1 supervised |d - t^|^2/|t^|^2, 2 energy norm
  // (d - t^)'A^(d - t^) / t^'A^t^
  int loss = 0;
  // statistics of the guesses
  int guesses = 0, fallbacks = 0;
  double last_ratio = 0.0, last_alpha = 0.0, last_beta = 0.0;
  unsigned long long seed = 0;
};

Net N;

void acts_free() {
  cudaFree(N.A.base);
  N.A = Acts();
}

void net_free() {
  cudaFree(N.p); cudaFree(N.gp); cudaFree(N.m); cudaFree(N.v);
  cudaFree(N.wb); cudaFree(N.wt);
  acts_free();
  cudaFree(N.part); cudaFree(N.dsum); cudaFree(N.err);
  cudaFree(N.store);
  cudaFree(N.fi0); cudaFree(N.tsum);
  N = Net();
}

// ------------------------------------------------------------ tensor core
__device__ __forceinline__ void mma16816(float (&d)[4], const unsigned (&a)[4], const unsigned (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ unsigned pack2(bf16 lo, bf16 hi) {
  return (unsigned)__bfloat16_as_ushort(lo) | ((unsigned)__bfloat16_as_ushort(hi) << 16);
}

__device__ __forceinline__ bool pos(bf16 x) {
  const unsigned short u = __bfloat16_as_ushort(x);
  return u != 0 && (u & 0x8000u) == 0;
}

// a voxel's coordinates in a D x H x W grid (x fastest)
struct Vox {
  int x, y, z;
  __device__ Vox(int v, int H, int W) {
    x = v % W;
    const int r = v / W;
    y = r % H;
    z = r / H;
  }
  __device__ int nbr(int v, int dz, int dy, int dx, int D, int H, int W) const {
    const int zz = z + dz, yy = y + dy, xx = x + dx;
    if ((unsigned)zz >= (unsigned)D || (unsigned)yy >= (unsigned)H || (unsigned)xx >= (unsigned)W) return -1;
    return v + (dz * H + dy) * W + dx;
  }
};

// two channels (c, c+1) of voxel n (row pitch ld); with a mask, a channel
// counts only where the mask (a ReLU output) is positive
__device__ __forceinline__ unsigned load_pair(const bf16* __restrict__ x, int ld, const bf16* __restrict__ mask,
                                              int ldm, int n, int c) {
  if (n < 0) return 0u;
  unsigned u = *reinterpret_cast<const unsigned*>(x + (long long)n * ld + c);
  if (mask) {
    const unsigned mk = *reinterpret_cast<const unsigned*>(mask + (long long)n * ldm + c);
    const unsigned lo = mk & 0xffffu, hi = mk >> 16;
    if (!(lo != 0u && (lo & 0x8000u) == 0u)) u &= 0xffff0000u;
    if (!(hi != 0u && (hi & 0x8000u) == 0u)) u &= 0x0000ffffu;
  }
  return u;
}

// row pitch (32-bit words) of one output channel's weights in shared memory:
// 27*CI/2 rounded so that the 8 rows a warp reads fall in distinct banks
__host__ __device__ constexpr int wrow(int CI) { return 27 * CI / 2 + ((4 - (27 * CI / 2) % 32) + 32) % 32; }

// y[:, co0..co0+15] = act(conv3x3x3(x * [mask > 0], w) + bias) for the
// output-channel slice co0 = 16*blockIdx.y.  x: CI channels at pitch ldx;
// w: [CO][27][CI]; y at pitch ldy.  One warp: 16 voxels x 16 channels per
// tile, tiles grid-strided.
template <int CI>
__global__ void __launch_bounds__(256) k_conv3(const bf16* __restrict__ x, int ldx, const bf16* __restrict__ w,
                                               const float* __restrict__ bias, const bf16* __restrict__ mask, int ldm,
                                               bf16* __restrict__ y, int ldy, int D, int H, int W, int relu) {
  extern __shared__ unsigned ws[];   // [16][wrow(CI)]
  constexpr int R = wrow(CI);
  const int co0 = blockIdx.y * 16;
  for (int q = threadIdx.x; q < 16 * 27 * CI / 2; q += blockDim.x) {
    const int co = q / (27 * CI / 2), r = q - co * (27 * CI / 2);
    ws[co * R + r] = reinterpret_cast<const unsigned*>(w + (size_t)(co0 + co) * 27 * CI)[r];
  }
  __syncthreads();
  const int V = D * H * W;
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const int ntiles = (V + 15) / 16;
  for (int tile = blockIdx.x * 8 + (threadIdx.x >> 5); tile < ntiles; tile += gridDim.x * 8) {
    const int v0 = tile * 16 + g, v1 = v0 + 8;
    const Vox P0(v0 < V ? v0 : 0, H, W), P1(v1 < V ? v1 : 0, H, W);
    float acc[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
    for (int tap = 0; tap < 27; ++tap) {
      const int dz = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
      const int n0 = v0 < V ? P0.nbr(v0, dz, dy, dx, D, H, W) : -1;
      const int n1 = v1 < V ? P1.nbr(v1, dz, dy, dx, D, H, W) : -1;
#pragma unroll
      for (int ks = 0; ks < CI / 16; ++ks) {
        unsigned a[4];
        a[0] = load_pair(x, ldx, mask, ldm, n0, ks * 16 + t * 2);
        a[1] = load_pair(x, ldx, mask, ldm, n1, ks * 16 + t * 2);
        a[2] = load_pair(x, ldx, mask, ldm, n0, ks * 16 + 8 + t * 2);
        a[3] = load_pair(x, ldx, mask, ldm, n1, ks * 16 + 8 + t * 2);
#pragma unroll
        for (int nt = 0; nt < 2; ++nt) {
          const unsigned* wr = ws + (nt * 8 + g) * R + tap * (CI / 2) + ks * 8 + t;
          const unsigned b[2] = {wr[0], wr[4]};
          mma16816(acc[nt], a, b);
        }
      }
    }
#pragma unroll
    for (int nt = 0; nt < 2; ++nt) {
      const int co = co0 + nt * 8 + t * 2;
      const float b0 = bias ? bias[co] : 0.f, b1 = bias ? bias[co + 1] : 0.f;
      float r[4] = {acc[nt][0] + b0, acc[nt][1] + b1, acc[nt][2] + b0, acc[nt][3] + b1};
      if (relu)
        for (int q = 0; q < 4; ++q) r[q] = fmaxf(r[q], 0.f);
      if (v0 < V)
        *reinterpret_cast<unsigned*>(y + (long long)v0 * ldy + co) = pack2(__float2bfloat16(r[0]), __float2bfloat16(r[1]));
      if (v1 < V)
        *reinterpret_cast<unsigned*>(y + (long long)v1 * ldy + co) = pack2(__float2bfloat16(r[2]), __float2bfloat16(r[3]));
    }
  }
}

// partial weight gradients of a 3x3x3 layer: for one tap, one chunk of
// voxels and the output-channel slice co0 = 16*blockIdx.z,
// G[co][ci] = sum_v gy[v][co] [y[v][co] > 0] x[v + off(tap)][ci]
template <int CI>
__global__ void __launch_bounds__(128) k_wgrad3(const bf16* __restrict__ x, int ldx, const bf16* __restrict__ gy,
                                                int ldg, const bf16* __restrict__ y, int ldy, float* __restrict__ part,
                                                int CO, int D, int H, int W) {
  __shared__ float red[4][16 * CI];
  const int V = D * H * W;
  const int tap = blockIdx.x, ch = blockIdx.y, co0 = blockIdx.z * 16;
  const int vs = ch * kChunk, ve = min(V, vs + kChunk);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const int dz = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
  auto gm = [&](int v, int co) -> bf16 {   // masked output gradient
    if (v >= ve) return __float2bfloat16(0.f);
    return pos(y[(long long)v * ldy + co0 + co]) ? gy[(long long)v * ldg + co0 + co] : __float2bfloat16(0.f);
  };
  auto xs = [&](int n, int ci) -> bf16 {   // shifted input
    return n < 0 ? __float2bfloat16(0.f) : x[(long long)n * ldx + ci];
  };
  float acc[CI / 8][4];
#pragma unroll
  for (int q = 0; q < CI / 8; ++q) acc[q][0] = acc[q][1] = acc[q][2] = acc[q][3] = 0.f;
  for (int vb = vs + warp * 16; vb < ve; vb += 64) {
    unsigned a[4];   // A[co][v] (16 x 16)
    a[0] = pack2(gm(vb + t * 2, g), gm(vb + t * 2 + 1, g));
    a[1] = pack2(gm(vb + t * 2, g + 8), gm(vb + t * 2 + 1, g + 8));
    a[2] = pack2(gm(vb + 8 + t * 2, g), gm(vb + 9 + t * 2, g));
    a[3] = pack2(gm(vb + 8 + t * 2, g + 8), gm(vb + 9 + t * 2, g + 8));
    int n[4];   // shifted voxels of rows 2t, 2t+1, 2t+8, 2t+9 of B
    const int vv[4] = {vb + t * 2, vb + t * 2 + 1, vb + 8 + t * 2, vb + 9 + t * 2};
#pragma unroll
    for (int q = 0; q < 4; ++q) n[q] = vv[q] < ve ? Vox(vv[q], H, W).nbr(vv[q], dz, dy, dx, D, H, W) : -1;
#pragma unroll
    for (int nt = 0; nt < CI / 8; ++nt) {   // B[v][ci] (16 x 8)
      const int ci = nt * 8 + g;
      unsigned b[2];
      b[0] = pack2(xs(n[0], ci), xs(n[1], ci));
      b[1] = pack2(xs(n[2], ci), xs(n[3], ci));
      mma16816(acc[nt], a, b);
    }
  }
#pragma unroll
  for (int nt = 0; nt < CI / 8; ++nt) {
    const int ci = nt * 8 + t * 2;
    red[warp][g * CI + ci] = acc[nt][0];
    red[warp][g * CI + ci + 1] = acc[nt][1];
    red[warp][(g + 8) * CI + ci] = acc[nt][2];
    red[warp][(g + 8) * CI + ci + 1] = acc[nt][3];
  }
  __syncthreads();
  for (int q = threadIdx.x; q < 16 * CI; q += blockDim.x)
    part[(((size_t)ch * 27 + tap) * CO + co0) * CI + q] = ((red[0][q] + red[1][q]) + red[2][q]) + red[3][q];
}

// gradient of one layer: W[co][tap][ci] = sum over chunks (fixed order)
__global__ void k_wgrad_sum(const float* __restrict__ part, int nch, int CO, int CI, float* __restrict__ gw) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;   // (tap, co, ci)
  if (q >= 27 * CO * CI) return;
  const int tap = q / (CO * CI), co = (q / CI) % CO, ci = q % CI;
  float s = 0.f;
  for (int c = 0; c < nch; ++c) s += part[(((size_t)c * 27 + tap) * CO + co) * CI + ci];
  gw[(co * 27 + tap) * CI + ci] = s;
}

// bias gradient partials of a layer with C outputs: sum_v gy[v][co] [y > 0]
__global__ void k_bgrad(const bf16* __restrict__ gy, int ldg, const bf16* __restrict__ y, int ldy, int C, int V,
                        float* part) {
  __shared__ float sh[256];
  const int co = threadIdx.x % C, row = threadIdx.x / C, rows = 256 / C;
  float s = 0.f;
  for (int v = blockIdx.x * rows + row; v < V; v += rows * gridDim.x)
    if (pos(y[(long long)v * ldy + co])) s += __bfloat162float(gy[(long long)v * ldg + co]);
  sh[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x < C) {
    float r = 0.f;
    for (int q = 0; q < rows; ++q) r += sh[q * C + threadIdx.x];
    part[blockIdx.x * C + threadIdx.x] = r;
  }
}

__global__ void k_sum_cols(const float* __restrict__ part, int rows, int cols, float* __restrict__ out) {
  const int c = threadIdx.x;
  if (c >= cols) return;
  float s = 0.f;
  for (int r = 0; r < rows; ++r) s += part[r * cols + c];
  out[c] = s;
}

// ---------------------------------------------------- pooling, up-sampling
// child k (0..7) of coarse voxel P on the fine grid H x W (x fastest)
__device__ __forceinline__ int child(const Vox& P, int k, int H, int W) {
  return ((2 * P.z + (k >> 2)) * H + 2 * P.y + ((k >> 1) & 1)) * W + 2 * P.x + (k & 1);
}

// out[v] = mean of the 8 children of v (coarse grid Dc x Hc x Wc), C channels
__global__ void k_pool(const bf16* __restrict__ in, int ldi, bf16* __restrict__ out, int ldo, int C, int Dc, int Hc,
                       int Wc) {
  const int Vc = Dc * Hc * Wc, np = C / 2;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < (long long)Vc * np;
       q += (long long)gridDim.x * blockDim.x) {
    const int v = (int)(q / np), c = (int)(q % np) * 2;
    const Vox P(v, Hc, Wc);
    float s0 = 0.f, s1 = 0.f;
    for (int k = 0; k < 8; ++k) {
      const __nv_bfloat162 u =
          *reinterpret_cast<const __nv_bfloat162*>(in + (long long)child(P, k, 2 * Hc, 2 * Wc) * ldi + c);
      s0 += __low2float(u);
      s1 += __high2float(u);
    }
    *reinterpret_cast<unsigned*>(out + (long long)v * ldo + c) =
        pack2(__float2bfloat16(s0 * 0.125f), __float2bfloat16(s1 * 0.125f));
  }
}

// gin[child] += gout[parent] / 8 (fine grid 2Dc x 2Hc x 2Wc)
__global__ void k_pool_bwd_add(const bf16* __restrict__ gout, int ldo, bf16* __restrict__ gin, int ldi, int C, int Dc,
                               int Hc, int Wc) {
  const int H = 2 * Hc, W = 2 * Wc, V = 8 * Dc * Hc * Wc, np = C / 2;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < (long long)V * np;
       q += (long long)gridDim.x * blockDim.x) {
    const int f = (int)(q / np), c = (int)(q % np) * 2;
    const Vox P(f, H, W);
    const int v = ((P.z >> 1) * Hc + (P.y >> 1)) * Wc + (P.x >> 1);
    const __nv_bfloat162 go = *reinterpret_cast<const __nv_bfloat162*>(gout + (long long)v * ldo + c);
    unsigned* gi = reinterpret_cast<unsigned*>(gin + (long long)f * ldi + c);
    const unsigned cur = *gi;
    const float lo = __bfloat162float(__ushort_as_bfloat16((unsigned short)(cur & 0xffffu)));
    const float hi = __bfloat162float(__ushort_as_bfloat16((unsigned short)(cur >> 16)));
    *gi = pack2(__float2bfloat16(lo + 0.125f * __low2float(go)), __float2bfloat16(hi + 0.125f * __high2float(go)));
  }
}

// out[child] = in[parent] (nearest), C channels; coarse grid Dc x Hc x Wc
__global__ void k_up(const bf16* __restrict__ in, int ldi, bf16* __restrict__ out, int ldo, int C, int Dc, int Hc,
                     int Wc) {
  const int H = 2 * Hc, W = 2 * Wc, V = 8 * Dc * Hc * Wc, np = C / 2;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < (long long)V * np;
       q += (long long)gridDim.x * blockDim.x) {
    const int f = (int)(q / np), c = (int)(q % np) * 2;
    const Vox P(f, H, W);
    const int v = ((P.z >> 1) * Hc + (P.y >> 1)) * Wc + (P.x >> 1);
    *reinterpret_cast<unsigned*>(out + (long long)f * ldo + c) =
        *reinterpret_cast<const unsigned*>(in + (long long)v * ldi + c);
  }
}

// gin[parent] = sum of gout over the 8 children
__global__ void k_up_bwd(const bf16* __restrict__ gout, int ldo, bf16* __restrict__ gin, int ldi, int C, int Dc, int Hc,
                         int Wc) {
  const int Vc = Dc * Hc * Wc, np = C / 2;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < (long long)Vc * np;
       q += (long long)gridDim.x * blockDim.x) {
    const int v = (int)(q / np), c = (int)(q % np) * 2;
    const Vox P(v, Hc, Wc);
    float s0 = 0.f, s1 = 0.f;
    for (int k = 0; k < 8; ++k) {
      const __nv_bfloat162 u =
          *reinterpret_cast<const __nv_bfloat162*>(gout + (long long)child(P, k, 2 * Hc, 2 * Wc) * ldo + c);
      s0 += __low2float(u);
      s1 += __high2float(u);
    }
    *reinterpret_cast<unsigned*>(gin + (long long)v * ldi + c) = pack2(__float2bfloat16(s0), __float2bfloat16(s1));
  }
}

// ------------------------------------------------------- output and loss
// out = b + sum_ci w[ci] x[v][ci] (1x1x1 convolution to one channel)
__global__ void k_last_fwd(const bf16* __restrict__ x, const float* __restrict__ p, float* __restrict__ out, int V) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
    float s = p[kOffLastB];
#pragma unroll
    for (int c = 0; c < kC1; ++c) s += p[kOffLastW + c] * __bfloat162float(x[(long long)v * kC1 + c]);
    out[v] = s;
  }
}

// backward of the 1x1x1 layer: dx[v][ci] = w[ci] gout[v]; partials of
// dw[ci] = sum gout x and db = sum gout (17 values per block)
__global__ void k_last_bwd(const bf16* __restrict__ x, const float* __restrict__ gout, const float* __restrict__ p,
                           bf16* __restrict__ gx, int V, float* part) {
  __shared__ float sh[kC1 + 1][256 / 32];
  float acc[kC1 + 1];
  for (int c = 0; c <= kC1; ++c) acc[c] = 0.f;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
    const float go = gout[v];
#pragma unroll
    for (int c = 0; c < kC1; ++c) {
      acc[c] += go * __bfloat162float(x[(long long)v * kC1 + c]);
      gx[(long long)v * kC1 + c] = __float2bfloat16(p[kOffLastW + c] * go);
    }
    acc[kC1] += go;
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int c = 0; c <= kC1; ++c) {
    float y = acc[c];
    for (int o = 16; o > 0; o >>= 1) y += __shfl_down_sync(0xffffffffu, y, o);
    if (lane == 0) sh[c][wid] = y;
  }
  __syncthreads();
  if (threadIdx.x <= kC1) {
    float s = 0.f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += sh[threadIdx.x][w];
    part[blockIdx.x * (kC1 + 1) + threadIdx.x] = s;
  }
}

// res = A^ out - rhs with the window operator (coef planes xp, xm, yp, ym,
// zp, zm, diag of V each; (A d)_v = diag d_v - sum_nb coef_nb d_nb,
// neighbours outside the window 0); partials of |res|^2 and |rhs|^2
__global__ void k_resloss(const float* __restrict__ out, const float* __restrict__ rhs, const float* __restrict__ cf,
                          float* __restrict__ res, int D, int H, int W, double* part) {
  const int V = D * H * W;
  double a[2] = {0.0, 0.0};
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
    const Vox P(v, H, W);
    float s = cf[6 * (long long)V + v] * out[v];
    if (P.x + 1 < W) s -= cf[v] * out[v + 1];
    if (P.x > 0) s -= cf[(long long)V + v] * out[v - 1];
    if (P.y + 1 < H) s -= cf[2 * (long long)V + v] * out[v + W];
    if (P.y > 0) s -= cf[3 * (long long)V + v] * out[v - W];
    if (P.z + 1 < D) s -= cf[4 * (long long)V + v] * out[v + H * W];
    if (P.z > 0) s -= cf[5 * (long long)V + v] * out[v - H * W];
    const float r = s - rhs[v];
    res[v] = r;
    a[0] += (double)r * r;
    a[1] += (double)rhs[v] * rhs[v];
  }
  block_reduce_store<2>(a, part);
}

// gout = 2 A^T res / |rhs|^2 (sums[0..1] = |res|^2, |rhs|^2); loss[0] = ratio
__global__ void k_resloss_grad(const float* __restrict__ res, const float* __restrict__ cf,
                               const double* __restrict__ sums, float* __restrict__ gout, double* loss, int D, int H,
                               int W) {
  const int V = D * H * W;
  const float sc = sums[1] > 0.0 ? (float)(2.0 / sums[1]) : 0.f;
  if (blockIdx.x == 0 && threadIdx.x == 0) loss[0] = sums[1] > 0.0 ? sums[0] / sums[1] : 0.0;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
    const Vox P(v, H, W);
    float s = cf[6 * (long long)V + v] * res[v];
    if (P.x + 1 < W) s -= cf[(long long)V + v + 1] * res[v + 1];              // xm of the +x neighbour
    if (P.x > 0) s -= cf[v - 1] * res[v - 1];                                  // xp of the -x neighbour
    if (P.y + 1 < H) s -= cf[3 * (long long)V + v + W] * res[v + W];
    if (P.y > 0) s -= cf[2 * (long long)V + v - W] * res[v - W];
    if (P.z + 1 < D) s -= cf[5 * (long long)V + v + H * W] * res[v + H * W];
    if (P.z > 0) s -= cf[4 * (long long)V + v - H * W] * res[v - H * W];
    gout[v] = sc * s;
  }
}

// supervised loss: partials of |out - tgt|^2 and |tgt|^2
__global__ void k_suploss(const float* __restrict__ out, const float* __restrict__ tgt, int V, double* part) {
  double a[2] = {0.0, 0.0};
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
    const float e = out[v] - tgt[v];
    a[0] += (double)e * e;
    a[1] += (double)tgt[v] * tgt[v];
  }
  block_reduce_store<2>(a, part);
}

// gout = 2 (out - tgt) / |tgt|^2; loss[0] = ratio
__global__ void k_suploss_grad(const float* __restrict__ out, const float* __restrict__ tgt,
                               const double* __restrict__ sums, float* __restrict__ gout, double* loss, int V) {
  const float sc = sums[1] > 0.0 ? (float)(2.0 / sums[1]) : 0.f;
  if (blockIdx.x == 0 && threadIdx.x == 0) loss[0] = sums[1] > 0.0 ? sums[0] / sums[1] : 0.0;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x)
    gout[v] = sc * (out[v] - tgt[v]);
}

// (A^ q)_v of the window operator for q = a - b (b may be null)
__device__ __forceinline__ float apply_w(const float* __restrict__ cf, const float* __restrict__ a,
                                         const float* __restrict__ b, int v, const Vox& P, int D, int H, int W, int V) {
  auto q = [&](int u) { return b ? a[u] - b[u] : a[u]; };
  float s = cf[6 * (long long)V + v] * q(v);
  if (P.x + 1 < W) s -= cf[v] * q(v + 1);
  if (P.x > 0) s -= cf[(long long)V + v] * q(v - 1);
  if (P.y + 1 < H) s -= cf[2 * (long long)V + v] * q(v + W);
  if (P.y > 0) s -= cf[3 * (long long)V + v] * q(v - W);
  if (P.z + 1 < D) s -= cf[4 * (long long)V + v] * q(v + H * W);
  if (P.z > 0) s -= cf[5 * (long long)V + v] * q(v - H * W);
  return s;
}

// energy-norm loss: res = A^ e with e = out - tgt; partials of e'A^e and
// tgt'A^tgt
__global__ void k_enloss(const float* __restrict__ out, const float* __restrict__ tgt, const float* __restrict__ cf,
                         float* __restrict__ res, int D, int H, int W, double* part) {
  const int V = D * H * W;
  double a[2] = {0.0, 0.0};
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
    const Vox P(v, H, W);
    const float r = apply_w(cf, out, tgt, v, P, D, H, W, V);
    res[v] = r;
    a[0] += (double)(out[v] - tgt[v]) * r;
    a[1] += (double)tgt[v] * apply_w(cf, tgt, nullptr, v, P, D, H, W, V);
  }
  block_reduce_store<2>(a, part);
}

// gout = (A^ e + A^' e) / tgt'A^tgt (the gradient of e'A^e for an A^ that
// need not be exactly symmetric in FP32); loss[0] = ratio
__global__ void k_enloss_grad(const float* __restrict__ out, const float* __restrict__ tgt,
                              const float* __restrict__ res, const float* __restrict__ cf,
                              const double* __restrict__ sums, float* __restrict__ gout, double* loss, int D, int H,
                              int W) {
  const int V = D * H * W;
  const float sc = sums[1] > 0.0 ? (float)(1.0 / sums[1]) : 0.f;
  if (blockIdx.x == 0 && threadIdx.x == 0) loss[0] = sums[1] > 0.0 ? sums[0] / sums[1] : 0.0;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
    const Vox P(v, H, W);
    auto e = [&](int u) { return out[u] - tgt[u]; };
    float s = cf[6 * (long long)V + v] * e(v);
    if (P.x + 1 < W) s -= cf[(long long)V + v + 1] * e(v + 1);
    if (P.x > 0) s -= cf[v - 1] * e(v - 1);
    if (P.y + 1 < H) s -= cf[3 * (long long)V + v + W] * e(v + W);
    if (P.y > 0) s -= cf[2 * (long long)V + v - W] * e(v - W);
    if (P.z + 1 < D) s -= cf[5 * (long long)V + v + H * W] * e(v + H * W);
    if (P.z > 0) s -= cf[4 * (long long)V + v - H * W] * e(v - H * W);
    gout[v] = sc * (res[v] + s);
  }
}

// Adam (lr, 0.9, 0.999, 1e-8) on the FP32 parameters
__global__ void k_adam(float* __restrict__ p, const float* __restrict__ gp, float* __restrict__ m, float* __restrict__ v,
                       int n, float lr, float c1, float c2) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const float gq = gp[q];
  const float mq = 0.9f * m[q] + 0.1f * gq;
  const float vq = 0.999f * v[q] + 0.001f * gq * gq;
  m[q] = mq;
  v[q] = vq;
  p[q] -= lr * (mq / c1) / (sqrtf(vq / c2) + 1e-8f);
}

// BF16 weights for the forward pass and, flipped and transposed, for the
// input gradient
__global__ void k_cast_w(const float* __restrict__ p, bf16* __restrict__ wb, bf16* __restrict__ wt) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= kWAll) return;
  int l = 0;
  while (l + 1 < kNL && q >= cWoff[l + 1]) ++l;
  const int CI = cCI[l], CO = cCO[l], r = q - cWoff[l];
  const int co = r / (27 * CI), tap = (r / CI) % 27, ci = r % CI;
  const bf16 w = __float2bfloat16(p[cOffW[l] + r]);
  wb[q] = w;
  wt[cWoff[l] + (ci * 27 + (26 - tap)) * CO + co] = w;
}

// training window from a recorded pair: input (channel 0 = r^), r^, A^, t^
__global__ void k_window(const float* __restrict__ smp, int sD, int sH, int sW, int z0, int y0, int x0, int B,
                         bf16* __restrict__ in, float* __restrict__ rhs, float* __restrict__ cf,
                         float* __restrict__ tgt) {
  const int V = B * B * B;
  const long long sV = (long long)sD * sH * sW;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
    const int x = v % B, y = (v / B) % B, z = v / (B * B);
    const long long s = ((long long)(z + z0) * sH + (y + y0)) * sW + (x + x0);
    const float r = smp[s];
    in[(long long)v * 16] = __float2bfloat16(r);
#pragma unroll
    for (int c = 1; c < 16; ++c) in[(long long)v * 16 + c] = __float2bfloat16(0.f);
    rhs[v] = r;
#pragma unroll
    for (int q = 0; q < 7; ++q) cf[(long long)q * V + v] = smp[(1 + q) * sV + s];
    tgt[v] = smp[8 * sV + s];
  }
}

// interior of a natural-layout field (k, i, j order: z = k, y = i, x = j)
__device__ __forceinline__ int nat_of(const Dims& d, int x, int y, int z) { return ixk(d, y + 3, x + 3, z + 3); }

// sums over the interior of r^2 and ap (the scales of a recorded pair and of
// the net's input)
__global__ void k_scales(Dims d, const double* __restrict__ r, const double* __restrict__ ap, int Ni, int Nj, int Nk,
                         double* part) {
  const int V = Ni * Nj * Nk;
  double a[2] = {0.0, 0.0};
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
    const int x = v % Nj, y = (v / Nj) % Ni, z = v / (Nj * Ni);
    const int n = nat_of(d, x, y, z);
    a[0] += r[n] * r[n];
    a[1] += ap[n];
  }
  block_reduce_store<2>(a, part);
}

// a recorded pair: r^ = r0/rms(r0), A^ = A/mean(ap) (both scales over the
// whole interior) in window axes (x = j: an, as; y = i: ae, aw; z = k: at,
// ab), on the window of wz x wy x wx cells at (z0, y0, x0) of the interior
__global__ void k_record(Dims d, const double* __restrict__ r, const double* __restrict__ ae,
                         const double* __restrict__ aw, const double* __restrict__ an, const double* __restrict__ as,
                         const double* __restrict__ at, const double* __restrict__ ab, const double* __restrict__ ap,
                         const double* __restrict__ sums, int Ni, int Nj, int Nk, int z0, int y0, int x0, int wz, int wy,
                         int wx, float* __restrict__ smp) {
  const long long Vi = (long long)Ni * Nj * Nk;
  const int V = wz * wy * wx;
  const double rinv = sums[0] > 0.0 ? 1.0 / sqrt(sums[0] / Vi) : 0.0;
  const double ainv = sums[1] != 0.0 ? (double)Vi / sums[1] : 0.0;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
    const int x = x0 + v % wx, y = y0 + (v / wx) % wy, z = z0 + v / (wx * wy);
    const int n = nat_of(d, x, y, z);
    smp[v] = (float)(r[n] * rinv);
    smp[1LL * V + v] = (float)(an[n] * ainv);
    smp[2LL * V + v] = (float)(as[n] * ainv);
    smp[3LL * V + v] = (float)(ae[n] * ainv);
    smp[4LL * V + v] = (float)(aw[n] * ainv);
    smp[5LL * V + v] = (float)(at[n] * ainv);
    smp[6LL * V + v] = (float)(ab[n] * ainv);
    smp[7LL * V + v] = (float)(ap[n] * ainv);
    smp[8LL * V + v] = 0.f;   // t^, filled at the end of the solve
  }
}

// t^ of a recorded window at the end of its solve: (fi - fi0) scaled as the
// pair, t^ = (fi - fi0) mean(ap) / rms(r0), so that A^ t^ = r^ when the solve
// has converged (sums = the start's |r0|^2 and sum of ap)
__global__ void k_record_target(Dims d, const double* __restrict__ fi, const double* __restrict__ fi0,
                                const double* __restrict__ sums, int Ni, int Nj, int Nk, int z0, int y0, int x0,
                                int wz, int wy, int wx, float* __restrict__ tgt) {
  const long long Vi = (long long)Ni * Nj * Nk;
  const int V = wz * wy * wx;
  const double sc = sums[0] > 0.0 ? (sums[1] / (double)Vi) / sqrt(sums[0] / Vi) : 0.0;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
    const int x = x0 + v % wx, y = y0 + (v / wx) % wy, z = z0 + v / (wx * wy);
    const int n = nat_of(d, x, y, z);
    tgt[v] = (float)((fi[n] - fi0[n]) * sc);
  }
}

// the net's input on the padded grid D x H x W (interior Nk x Ni x Nj at the
// origin, zero elsewhere): channel 0 = r0/rms(r0)
__global__ void k_rhs_in(Dims d, const double* __restrict__ r, const double* __restrict__ sums, int Ni, int Nj, int Nk,
                         bf16* __restrict__ in, int D, int H, int W) {
  const int V = D * H * W;
  const int Vi = Ni * Nj * Nk;
  const double rinv = sums[0] > 0.0 ? 1.0 / sqrt(sums[0] / Vi) : 0.0;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
    const int x = v % W, y = (v / W) % H, z = v / (W * H);
    const float q = (x < Nj && y < Ni && z < Nk) ? (float)(r[nat_of(d, x, y, z)] * rinv) : 0.f;
    in[(long long)v * 16] = __float2bfloat16(q);
#pragma unroll
    for (int c = 1; c < 16; ++c) in[(long long)v * 16 + c] = __float2bfloat16(0.f);
  }
}

// the predicted shape on the interior of a natural field (zero elsewhere)
__global__ void k_shape_nat(Dims d, double* __restrict__ z, const float* __restrict__ out, int Ni, int Nj, int Nk, int H,
                            int W) {
  const int Vi = Ni * Nj * Nk;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < Vi; v += gridDim.x * blockDim.x) {
    const int x = v % Nj, y = (v / Nj) % Ni, zz = v / (Nj * Ni);
    z[nat_of(d, x, y, zz)] = (double)out[((long long)zz * H + y) * W + x];
  }
}

// 1 on the interior of a natural field (the rest left as it is)
__global__ void k_ones_nat(Dims d, double* __restrict__ z, int Ni, int Nj, int Nk) {
  const int Vi = Ni * Nj * Nk;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < Vi; v += gridDim.x * blockDim.x) {
    const int x = v % Nj, y = (v / Nj) % Ni, zz = v / (Nj * Ni);
    z[nat_of(d, x, y, zz)] = 1.0;
  }
}

__global__ void k_axpy_nat(int n, double alpha, const double* __restrict__ x, double* __restrict__ y) {
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) y[q] = y[q] + alpha * x[q];
}

// ------------------------------------------------------------ host side
int round4(int n) { return (n + 3) & ~3; }

// voxel count of the grid layer l runs on, for level-1 count V1
long long layer_voxels(int l, long long V1) {
  const int lev[kNL] = {0, 0, 1, 1, 2, 2, 1, 1, 0, 0};
  return lev[l] == 0 ? V1 : (lev[l] == 1 ? V1 / 8 : V1 / 64);
}

int ensure_acts(long long V1) {
  if (V1 <= N.A.V1) return CAPPGPU_OK;
  acts_free();
  const long long V2 = V1 / 8, V3 = V1 / 64;
  struct Item { void** p; long long bytes; };
  Acts& A = N.A;
  const long long b = sizeof(bf16);
  Item items[] = {
      {(void**)&A.a0, V1 * 16 * b},    {(void**)&A.a1, V1 * 16 * b},   {(void**)&A.cat1, V1 * 48 * b},
      {(void**)&A.p1, V2 * 16 * b},    {(void**)&A.a3, V2 * 32 * b},   {(void**)&A.cat2, V2 * 96 * b},
      {(void**)&A.p2, V3 * 32 * b},    {(void**)&A.a5, V3 * 64 * b},   {(void**)&A.b3, V3 * 64 * b},
      {(void**)&A.a7, V2 * 32 * b},    {(void**)&A.x2, V2 * 32 * b},   {(void**)&A.a9, V1 * 16 * b},
      {(void**)&A.x1, V1 * 16 * b},    {(void**)&A.gx1, V1 * 16 * b},  {(void**)&A.ga9, V1 * 16 * b},
      {(void**)&A.gcat1, V1 * 48 * b}, {(void**)&A.gx2, V2 * 32 * b},  {(void**)&A.ga7, V2 * 32 * b},
      {(void**)&A.gcat2, V2 * 96 * b}, {(void**)&A.gb3, V3 * 64 * b},  {(void**)&A.ga5, V3 * 64 * b},
      {(void**)&A.gp2, V3 * 32 * b},   {(void**)&A.ga3, V2 * 32 * b},  {(void**)&A.gp1, V2 * 16 * b},
      {(void**)&A.ga1, V1 * 16 * b},   {(void**)&A.out, V1 * 4},       {(void**)&A.gout, V1 * 4},
      {(void**)&A.rhs, V1 * 4},        {(void**)&A.coef, 7 * V1 * 4},  {(void**)&A.res, V1 * 4},
      {(void**)&A.tgt, V1 * 4},
  };
  long long total = 0;
  for (auto& it : items) total += (it.bytes + 255) & ~255LL;
  char* base = nullptr;
  if (cudaMalloc(&base, total) != cudaSuccess) {
    set_error("learned guess: out of device memory for %lld voxels", V1);
    return CAPPGPU_E_NOMEM;
  }
  long long o = 0;
  for (auto& it : items) {
    *it.p = base + o;
    o += (it.bytes + 255) & ~255LL;
  }
  A.base = base;
  A.V1 = V1;
  // partial sums: weight gradients of the largest layer at this size, then
  // the bias and last-layer partials
  size_t need = 0;
  for (int l = 0; l < kNL; ++l) {
    const size_t n = (size_t)((layer_voxels(l, V1) + kChunk - 1) / kChunk) * 27 * kCO[l] * kCI[l];
    if (n > need) need = n;
  }
  need += 512 * (kC1 + 1) + 256 * 64;
  if (need > N.part_n) {
    cudaFree(N.part);
    N.part = nullptr;
    if (cudaMalloc(&N.part, need * sizeof(float)) != cudaSuccess) {
      N.part_n = 0;
      set_error("learned guess: out of device memory for partial sums");
      return CAPPGPU_E_NOMEM;
    }
    N.part_n = need;
  }
  return CAPPGPU_OK;
}

int cast_weights() {
  launch(k_cast_w, (kWAll + 255) / 256, 256, ctx().st, (const float*)N.p, N.wb, N.wt);
  CAP_CHECK_LAUNCH();
  return CAPPGPU_OK;
}

int init_params(unsigned long long seed) {
  std::vector<float> h(kParams, 0.f);
  unsigned long long s = seed * 6364136223846793005ULL + 1442695040888963407ULL;
  auto uni = [&]() {   // splitmix64 -> [-1, 1)
    s += 0x9e3779b97f4a7c15ULL;
    unsigned long long z = s;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    z ^= z >> 31;
    return (float)((double)(z >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0);
  };
  for (int l = 0; l < kNL; ++l) {
    const int fan_in = 27 * (l == 0 ? 1 : kCI[l]);
    const float a = sqrtf(6.f / (float)fan_in);   // He-uniform
    for (int q = 0; q < wsize(l); ++q) {
      const int ci = q % kCI[l];
      h[offW(l) + q] = (l == 0 && ci > 0) ? 0.f : a * uni();
    }
  }
  for (int c = 0; c < kC1; ++c) h[kOffLastW + c] = sqrtf(3.f / kC1) * uni();
  Ctx& c = ctx();
  CAP_CUDA(cudaMemcpyAsync(N.p, h.data(), sizeof(float) * kParams, cudaMemcpyHostToDevice, c.st));
  CAP_CUDA(cudaMemsetAsync(N.m, 0, sizeof(float) * kParams, c.st));
  CAP_CUDA(cudaMemsetAsync(N.v, 0, sizeof(float) * kParams, c.st));
  CAP_CUDA(cudaStreamSynchronize(c.st));   // h is released on return
  N.adam_t = 0;
  return cast_weights();
}

constexpr int kConvGrid = 152 * 4;

template <int CI>
int conv_ci(const bf16* x, int ldx, const bf16* w, int CO, const float* bias, const bf16* mask, int ldm, bf16* y,
            int ldy, int D, int H, int W, int relu) {
  const size_t smem = (size_t)16 * wrow(CI) * sizeof(unsigned);
  CAP_CUDA(cudaFuncSetAttribute(k_conv3<CI>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int ntiles = (D * H * W + 15) / 16;
  int gx = (ntiles + 7) / 8;
  if (gx > kConvGrid) gx = kConvGrid;
  ++ctx().launches;
  k_conv3<CI><<<dim3(gx, CO / 16), 256, smem, ctx().st>>>(x, ldx, w, bias, mask, ldm, y, ldy, D, H, W, relu);
  return CAPPGPU_OK;
}

// the convolution kernels: 1 = tcgen05, halo tiles where they fit (default),
// 2 = tcgen05 per-tap gathers only, 0 = mma.sync
int g_conv_impl = 1;

template <int CI, int CO, bool MASK>
int conv_tc(const bf16* x, int ldx, const bf16* w, const float* bias, const bf16* mask, int ldm, bf16* y, int ldy,
            int D, int H, int W, int relu) {
  typedef tc::ConvTC<CI, CO> T;
  CAP_CUDA(cudaFuncSetAttribute(tc::k_conv3_tc<CI, CO, MASK>, cudaFuncAttributeMaxDynamicSharedMemorySize, T::kSmem));
  const int ntiles = (D * H * W + 127) / 128;
  // CTAs one SM holds: shared memory, 512 TMEM columns, 16 x 128 threads
  int per_sm = (228 * 1024) / (T::kSmem + 1024);
  if (per_sm > 512 / T::kCols) per_sm = 512 / T::kCols;
  if (per_sm > 16) per_sm = 16;
  if (per_sm < 1) per_sm = 1;
  int grid = 152 * per_sm;
  if (grid > ntiles) grid = ntiles;
  ++ctx().launches;
  tc::k_conv3_tc<CI, CO, MASK><<<grid, 128, T::kSmem, ctx().st>>>(x, ldx, w, bias, mask, ldm, y, ldy, D, H, W, relu,
                                                                   N.err);
  return CAPPGPU_OK;
}

template <int CI, int CO, bool MASK>
int conv_halo(const bf16* x, int ldx, const bf16* w, const float* bias, const bf16* mask, int ldm, bf16* y, int ldy,
              int D, int H, int W, int relu) {
  typedef tc::HaloTC<CI, CO> T;
  CAP_CUDA(cudaFuncSetAttribute(tc::k_conv3_halo<CI, CO, MASK>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                T::kSmem));
  const int ntiles = ((W + 7) / 8) * ((H + 15) / 16) * D;
  int per_sm = (228 * 1024) / (T::kSmem + 1024);
  if (per_sm > 512 / T::kCols) per_sm = 512 / T::kCols;
  if (per_sm > 16) per_sm = 16;
  if (per_sm < 1) per_sm = 1;
  int grid = 152 * per_sm;
  if (grid > ntiles) grid = ntiles;
  ++ctx().launches;
  tc::k_conv3_halo<CI, CO, MASK><<<grid, 128, T::kSmem, ctx().st>>>(x, ldx, w, bias, mask, ldm, y, ldy, D, H, W,
                                                                     relu, N.err);
  return CAPPGPU_OK;
}

// the tensor-core form for the net's (CI, CO) pairs: the halo-tile kernel
// where all 27 taps' weights fit in shared memory beside the halo (unless
// impl 2 asks for the per-tap kernel), else the per-tap kernel (d2a 96->32
// and e3b 64->64: two half-width halo launches of one CTA per SM each were
// slower); -1 if there is none
int conv_tc_any(int CI, const bf16* x, int ldx, const bf16* w, int CO, const float* bias, const bf16* mask, int ldm,
                bf16* y, int ldy, int D, int H, int W, int relu) {
  const bool halo = g_conv_impl == 1;
#define CAP_TC(ci, co)                                                                                  \
  if (CI == ci && CO == co) {                                                                           \
    if (tc::HaloTC<ci, co>::kFits && halo)                                                              \
      return mask ? conv_halo<ci, co, true>(x, ldx, w, bias, mask, ldm, y, ldy, D, H, W, relu)          \
                  : conv_halo<ci, co, false>(x, ldx, w, bias, mask, ldm, y, ldy, D, H, W, relu);        \
    return mask ? conv_tc<ci, co, true>(x, ldx, w, bias, mask, ldm, y, ldy, D, H, W, relu)              \
                : conv_tc<ci, co, false>(x, ldx, w, bias, mask, ldm, y, ldy, D, H, W, relu);            \
  }
  CAP_TC(16, 16) CAP_TC(16, 32) CAP_TC(32, 32) CAP_TC(32, 64) CAP_TC(64, 64) CAP_TC(96, 32) CAP_TC(48, 16)
  CAP_TC(32, 16) CAP_TC(64, 32) CAP_TC(32, 96) CAP_TC(16, 48)
#undef CAP_TC
  return -1;
}

// y = relu(conv(x) + b) (forward, mask == null) or the input gradient
// (mask = the layer's output, w = flipped transposed weights)
int conv(int CI, const bf16* x, int ldx, const bf16* w, int CO, const float* bias, const bf16* mask, int ldm, bf16* y,
         int ldy, int D, int H, int W, int relu) {
  if (g_conv_impl >= 1) {
    const int rc = conv_tc_any(CI, x, ldx, w, CO, bias, mask, ldm, y, ldy, D, H, W, relu);
    if (rc >= 0) return rc;
  }
  switch (CI) {
    case 16: return conv_ci<16>(x, ldx, w, CO, bias, mask, ldm, y, ldy, D, H, W, relu);
    case 32: return conv_ci<32>(x, ldx, w, CO, bias, mask, ldm, y, ldy, D, H, W, relu);
    case 48: return conv_ci<48>(x, ldx, w, CO, bias, mask, ldm, y, ldy, D, H, W, relu);
    case 64: return conv_ci<64>(x, ldx, w, CO, bias, mask, ldm, y, ldy, D, H, W, relu);
    case 96: return conv_ci<96>(x, ldx, w, CO, bias, mask, ldm, y, ldy, D, H, W, relu);
  }
  set_error("learned guess: no convolution for %d input channels", CI);
  return CAPPGPU_E_ARG;
}

int fwd_layer(int l, const bf16* x, int ldx, bf16* y, int ldy, int D, int H, int W) {
  return conv(kCI[l], x, ldx, N.wb + woff(l), kCO[l], N.p + offB(l), nullptr, 0, y, ldy, D, H, W, 1);
}

template <int CI>
void wgrad_ci(const bf16* x, int ldx, const bf16* gy, int ldg, const bf16* y, int ldy, int CO, int D, int H, int W) {
  const int nch = (D * H * W + kChunk - 1) / kChunk;
  launch(k_wgrad3<CI>, dim3(27, nch, CO / 16), 128, ctx().st, x, ldx, gy, ldg, y, ldy, N.part, CO, D, H, W);
}

// tcgen05 weight gradient on halo tiles; returns the number of chunks
template <int CI, int CO>
int wgrad_halo(const bf16* x, int ldx, const bf16* gy, int ldg, const bf16* y, int ldy, int D, int H, int W) {
  typedef tc::WgradTC<CI, CO> T;
  CAP_CUDA(cudaFuncSetAttribute(tc::k_wgrad_halo<CI, CO>, cudaFuncAttributeMaxDynamicSharedMemorySize, T::kSmem));
  const int ntiles = ((W + 7) / 8) * ((H + 15) / 16) * D;
  // 16 tiles per chunk, fewer chunks if the partial sums would not fit
  const long long cap = (long long)(N.part_n / ((size_t)27 * CO * CI));
  int per = 16;
  while ((ntiles + per - 1) / per > cap) per *= 2;
  const int nch = (ntiles + per - 1) / per;
  const int ngroups = (27 + T::kTG - 1) / T::kTG;
  ++ctx().launches;
  tc::k_wgrad_halo<CI, CO><<<dim3(ngroups, nch), 128, T::kSmem, ctx().st>>>(x, ldx, gy, ldg, y, ldy, N.part, D, H,
                                                                             W, per, N.err);
  return nch;
}

int wgrad_any_halo(int CI, int CO, const bf16* x, int ldx, const bf16* gy, int ldg, const bf16* y, int ldy, int D,
                   int H, int W) {
#define CAP_WG(ci, co) \
  if (CI == ci && CO == co) return wgrad_halo<ci, co>(x, ldx, gy, ldg, y, ldy, D, H, W);
  CAP_WG(16, 16) CAP_WG(16, 32) CAP_WG(32, 32) CAP_WG(32, 64) CAP_WG(64, 64) CAP_WG(96, 32) CAP_WG(48, 16)
#undef CAP_WG
  return -1;
}

// weight and bias gradients of layer l (input x, output y, output gradient
// gy), then (dx != null) the gradient with respect to its input
int bwd_layer(int l, const bf16* x, int ldx, const bf16* gy, int ldg, const bf16* y, int ldy, bf16* dx, int lddx,
              int D, int H, int W) {
  Ctx& c = ctx();
  const int CI = kCI[l], CO = kCO[l];
  const int V = D * H * W;
  int nch = -1;
  if (g_conv_impl == 1) nch = wgrad_any_halo(CI, CO, x, ldx, gy, ldg, y, ldy, D, H, W);
  if (nch < 0) {
    switch (CI) {
      case 16: wgrad_ci<16>(x, ldx, gy, ldg, y, ldy, CO, D, H, W); break;
      case 32: wgrad_ci<32>(x, ldx, gy, ldg, y, ldy, CO, D, H, W); break;
      case 48: wgrad_ci<48>(x, ldx, gy, ldg, y, ldy, CO, D, H, W); break;
      case 64: wgrad_ci<64>(x, ldx, gy, ldg, y, ldy, CO, D, H, W); break;
      case 96: wgrad_ci<96>(x, ldx, gy, ldg, y, ldy, CO, D, H, W); break;
      default: set_error("learned guess: bad layer"); return CAPPGPU_E_ARG;
    }
    nch = (V + kChunk - 1) / kChunk;
  }
  launch(k_wgrad_sum, (27 * CO * CI + 255) / 256, 256, c.st, (const float*)N.part, nch, CO, CI, N.gp + offW(l));
  launch(k_bgrad, 256, 256, c.st, gy, ldg, y, ldy, CO, V, N.part);
  launch(k_sum_cols, 1, 64, c.st, (const float*)N.part, 256, CO, N.gp + offB(l));
  CAP_CHECK_LAUNCH();
  if (dx) return conv(CO, gy, ldg, N.wt + woff(l), CI, nullptr, y, ldy, dx, lddx, D, H, W, 0);
  return CAPPGPU_OK;
}

// forward pass on A.a0 (D x H x W, multiples of 4) into A.out
int forward(int D, int H, int W) {
  Ctx& c = ctx();
  Acts& A = N.A;
  const int D2 = D / 2, H2 = H / 2, W2 = W / 2, D3 = D / 4, H3 = H / 4, W3 = W / 4;
  const long long V = (long long)D * H * W, V2 = V / 8, V3 = V / 64;
  int rc;
  if ((rc = fwd_layer(0, A.a0, 16, A.a1, 16, D, H, W))) return rc;
  if ((rc = fwd_layer(1, A.a1, 16, A.cat1 + 32, 48, D, H, W))) return rc;
  launch(k_pool, grid_for(V2 * 8), kThreads, c.st, (const bf16*)(A.cat1 + 32), 48, A.p1, 16, 16, D2, H2, W2);
  if ((rc = fwd_layer(2, A.p1, 16, A.a3, 32, D2, H2, W2))) return rc;
  if ((rc = fwd_layer(3, A.a3, 32, A.cat2 + 64, 96, D2, H2, W2))) return rc;
  launch(k_pool, grid_for(V3 * 16), kThreads, c.st, (const bf16*)(A.cat2 + 64), 96, A.p2, 32, 32, D3, H3, W3);
  if ((rc = fwd_layer(4, A.p2, 32, A.a5, 64, D3, H3, W3))) return rc;
  if ((rc = fwd_layer(5, A.a5, 64, A.b3, 64, D3, H3, W3))) return rc;
  launch(k_up, grid_for(V2 * 32), kThreads, c.st, (const bf16*)A.b3, 64, A.cat2, 96, 64, D3, H3, W3);
  if ((rc = fwd_layer(6, A.cat2, 96, A.a7, 32, D2, H2, W2))) return rc;
  if ((rc = fwd_layer(7, A.a7, 32, A.x2, 32, D2, H2, W2))) return rc;
  launch(k_up, grid_for(V * 16), kThreads, c.st, (const bf16*)A.x2, 32, A.cat1, 48, 32, D2, H2, W2);
  if ((rc = fwd_layer(8, A.cat1, 48, A.a9, 16, D, H, W))) return rc;
  if ((rc = fwd_layer(9, A.a9, 16, A.x1, 16, D, H, W))) return rc;
  launch(k_last_fwd, grid_for(V), kThreads, c.st, (const bf16*)A.x1, (const float*)N.p, A.out, (int)V);
  CAP_CHECK_LAUNCH();
  return CAPPGPU_OK;
}

// the training loss of A.out (N.loss: residual norm against A.rhs / A.coef,
// supervised or energy norm against A.tgt; loss in N.dsum[0]), then the
// backward pass into N.gp
int backward(int D, int H, int W) {
  Ctx& c = ctx();
  Acts& A = N.A;
  const int V = D * H * W;
  const int D2 = D / 2, H2 = H / 2, W2 = W / 2, D3 = D / 4, H3 = H / 4, W3 = W / 4;
  const long long V2 = V / 8, V3 = V / 64;
  const float *out = A.out, *tgt = A.tgt, *cf = A.coef;
  if (N.loss == 1)
    launch(k_suploss, kRedBlocks, kThreads, c.st, out, tgt, V, c.partials);
  else if (N.loss == 2)
    launch(k_enloss, kRedBlocks, kThreads, c.st, out, tgt, cf, A.res, D, H, W, c.partials);
  else
    launch(k_resloss, kRedBlocks, kThreads, c.st, out, (const float*)A.rhs, cf, A.res, D, H, W, c.partials);
  CAP_CHECK_LAUNCH();
  int rc = finish_reduce(2);
  if (rc) return rc;
  const double* sums = c.redout;
  if (N.loss == 1)
    launch(k_suploss_grad, grid_for(V), kThreads, c.st, out, tgt, sums, A.gout, N.dsum, V);
  else if (N.loss == 2)
    launch(k_enloss_grad, grid_for(V), kThreads, c.st, out, tgt, (const float*)A.res, cf, sums, A.gout, N.dsum, D, H,
           W);
  else
    launch(k_resloss_grad, grid_for(V), kThreads, c.st, (const float*)A.res, cf, sums, A.gout, N.dsum, D, H, W);
  const int lb = 512;
  launch(k_last_bwd, lb, 256, c.st, (const bf16*)A.x1, (const float*)A.gout, (const float*)N.p, A.gx1, V, N.part);
  launch(k_sum_cols, 1, 32, c.st, (const float*)N.part, lb, kC1 + 1, N.gp + kOffLastW);
  CAP_CHECK_LAUNCH();
  if ((rc = bwd_layer(9, A.a9, 16, A.gx1, 16, A.x1, 16, A.ga9, 16, D, H, W))) return rc;
  if ((rc = bwd_layer(8, A.cat1, 48, A.ga9, 16, A.a9, 16, A.gcat1, 48, D, H, W))) return rc;
  launch(k_up_bwd, grid_for(V2 * 16), kThreads, c.st, (const bf16*)A.gcat1, 48, A.gx2, 32, 32, D2, H2, W2);
  if ((rc = bwd_layer(7, A.a7, 32, A.gx2, 32, A.x2, 32, A.ga7, 32, D2, H2, W2))) return rc;
  if ((rc = bwd_layer(6, A.cat2, 96, A.ga7, 32, A.a7, 32, A.gcat2, 96, D2, H2, W2))) return rc;
  launch(k_up_bwd, grid_for(V3 * 32), kThreads, c.st, (const bf16*)A.gcat2, 96, A.gb3, 64, 64, D3, H3, W3);
  if ((rc = bwd_layer(5, A.a5, 64, A.gb3, 64, A.b3, 64, A.ga5, 64, D3, H3, W3))) return rc;
  if ((rc = bwd_layer(4, A.p2, 32, A.ga5, 64, A.a5, 64, A.gp2, 32, D3, H3, W3))) return rc;
  launch(k_pool_bwd_add, grid_for(V2 * 16), kThreads, c.st, (const bf16*)A.gp2, 32, A.gcat2 + 64, 96, 32, D3, H3, W3);
  if ((rc = bwd_layer(3, A.a3, 32, A.gcat2 + 64, 96, A.cat2 + 64, 96, A.ga3, 32, D2, H2, W2))) return rc;
  if ((rc = bwd_layer(2, A.p1, 16, A.ga3, 32, A.a3, 32, A.gp1, 16, D2, H2, W2))) return rc;
  launch(k_pool_bwd_add, grid_for((long long)V * 8), kThreads, c.st, (const bf16*)A.gp1, 16, A.gcat1 + 32, 48, 16, D2,
         H2, W2);
  if ((rc = bwd_layer(1, A.a1, 16, A.gcat1 + 32, 48, A.cat1 + 32, 48, A.ga1, 16, D, H, W))) return rc;
  if ((rc = bwd_layer(0, A.a0, 16, A.ga1, 16, A.a1, 16, nullptr, 0, D, H, W))) return rc;
  CAP_CHECK_LAUNCH();
  return CAPPGPU_OK;
}

// a tensor-core convolution whose bounded wait ran out (synchronises)
int check_err() {
  int h = 0;
  CAP_CUDA(cudaMemcpyAsync(&h, N.err, sizeof(int), cudaMemcpyDeviceToHost, ctx().st));
  CAP_CUDA(cudaStreamSynchronize(ctx().st));
  if (h) {
    cudaMemsetAsync(N.err, 0, sizeof(int), ctx().st);
    set_error("learned guess: a tensor-core convolution waited beyond its limit");
    return CAPPGPU_E_SPIN;
  }
  return CAPPGPU_OK;
}

int adam_step(float lr) {
  ++N.adam_t;
  const float c1 = 1.f - powf(0.9f, (float)N.adam_t), c2 = 1.f - powf(0.999f, (float)N.adam_t);
  launch(k_adam, (kParams + 255) / 256, 256, ctx().st, N.p, (const float*)N.gp, N.m, N.v, kParams, lr, c1, c2);
  CAP_CHECK_LAUNCH();
  return cast_weights();
}

// algorithmic FLOPs of one forward pass per level-1 voxel (layer 0 has one
// input channel) and of the weight and input gradients
double fwd_flops_per_voxel() {
  double f = 0.0;
  for (int l = 0; l < kNL; ++l) {
    const double vl = (double)layer_voxels(l, 64) / 64.0;
    f += 2.0 * 27.0 * (l == 0 ? 1 : kCI[l]) * kCO[l] * vl;
  }
  return f + 2.0 * kC1;
}

double bwd_flops_per_voxel() {
  double f = 0.0;
  for (int l = 0; l < kNL; ++l) {
    const double vl = (double)layer_voxels(l, 64) / 64.0;
    const double ci = l == 0 ? 1 : kCI[l];
    f += 2.0 * 27.0 * ci * kCO[l] * vl;                 // weight gradient
    if (l > 0) f += 2.0 * 27.0 * ci * kCO[l] * vl;      // input gradient
  }
  return f + 4.0 * kC1;
}

}  // namespace

void learned_free() { net_free(); }

int learned_set_conv(int impl) {
  if (impl < 0 || impl > 2) return CAPPGPU_E_ARG;
  g_conv_impl = impl;
  return CAPPGPU_OK;
}

// Unit timing (cappgpu_profile_kernel): 9 = one forward pass of the net on
// this grid (interior padded to multiples of 4) from the module residual;
// 10 = one forward and backward pass on a 64^3 window (or the grid, if
// smaller) of the first recorded pair.  *flops = algorithmic FLOPs.
int learned_profile_unit(int which, double* flops) {
  if (!N.ready) { set_error("profile unit %d: call cappgpu_learn_reset first", which); return CAPPGPU_E_NOINIT; }
  Ctx& c = ctx();
  const Dims& d = c.d;
  const int Ni = d.nimm - 2, Nj = d.njmm - 2, Nk = d.nkmm - 2;
  int rc;
  if (which == 9) {
    const int D = round4(Nk), H = round4(Ni), W = round4(Nj);
    if ((rc = ensure_acts((long long)D * H * W))) return rc;
    launch(k_scales, kRedBlocks, kThreads, c.st, d, (const double*)c.f[CAP_RES], (const double*)c.f[CAP_AP], Ni, Nj,
           Nk, c.partials);
    CAP_CHECK_LAUNCH();
    if ((rc = finish_reduce(2))) return rc;
    launch(k_rhs_in, grid_for((long long)D * H * W), kThreads, c.st, d, (const double*)c.f[CAP_RES],
           (const double*)c.redout, Ni, Nj, Nk, N.A.a0, D, H, W);
    CAP_CHECK_LAUNCH();
    *flops = fwd_flops_per_voxel() * (double)D * H * W;
    return forward(D, H, W);
  }
  if (N.nsamples == 0) { set_error("profile unit 10: no recorded pairs"); return CAPPGPU_E_NOINIT; }
  const int B = min(64, min(N.sD, min(N.sH, N.sW))) & ~3;
  if (B < 4) { set_error("profile unit 10: the grid is smaller than 4 cells"); return CAPPGPU_E_ARG; }
  const int V = B * B * B;
  if ((rc = ensure_acts(V))) return rc;
  launch(k_window, grid_for(V), kThreads, c.st, (const float*)N.store, N.sD, N.sH, N.sW, 0, 0, 0, B, N.A.a0, N.A.rhs,
         N.A.coef, N.A.tgt);
  CAP_CHECK_LAUNCH();
  *flops = (fwd_flops_per_voxel() + bwd_flops_per_voxel()) * (double)V;
  if ((rc = forward(B, B, B))) return rc;
  return backward(B, B, B);
}

// Record hook and the guess, called by the refinement form of pcgsip at the
// start of a solve: r0 (module res) and res0 are known.
int learned_solve_start(int fif, double res0) {
  if (!N.ready) return CAPPGPU_OK;
  N.pend.clear();
  Ctx& c = ctx();
  const Dims& d = c.d;
  const int Ni = d.nimm - 2, Nj = d.njmm - 2, Nk = d.nkmm - 2;
  const long long Vi = (long long)Ni * Nj * Nk;
  if (!(res0 > 0.0) || !isfinite(res0)) return CAPPGPU_OK;
  const bool rec = N.collect && N.max_samples > 0 &&
                   (N.wper > 0 ? N.sD <= Nk && N.sD <= Ni && N.sD <= Nj : N.sD == Nk && N.sH == Ni && N.sW == Nj);
  const bool guess = c.precision == 2 && N.trained;
  if (!rec && !guess) return CAPPGPU_OK;
  launch(k_scales, kRedBlocks, kThreads, c.st, d, (const double*)c.f[CAP_RES], (const double*)c.f[CAP_AP], Ni, Nj, Nk,
         c.partials);
  CAP_CHECK_LAUNCH();
  int rc = finish_reduce(2);
  if (rc) return rc;
  if (rec) {
    // fi and the scale sums at the start: the end of the solve forms t^ from them
    if (N.fi0_n < d.nijk) {
      cudaFree(N.fi0);
      N.fi0 = nullptr;
      N.fi0_n = 0;
      if (cudaMalloc(&N.fi0, sizeof(double) * d.nijk) != cudaSuccess) {
        set_error("learned guess: out of device memory for the recorded solve's start");
        return CAPPGPU_E_NOMEM;
      }
      N.fi0_n = d.nijk;
    }
    if (!N.tsum) CAP_CUDA(cudaMalloc(&N.tsum, sizeof(double) * 2));
    CAP_CUDA(cudaMemcpyAsync(N.fi0, c.f[fif], sizeof(double) * d.nijk, cudaMemcpyDeviceToDevice, c.st));
    CAP_CUDA(cudaMemcpyAsync(N.tsum, c.redout, sizeof(double) * 2, cudaMemcpyDeviceToDevice, c.st));
    const long long sV = (long long)N.sD * N.sH * N.sW;
    auto rnd = [&](unsigned m) {   // xorshift64*
      unsigned long long& q = N.wrng;
      q ^= q >> 12; q ^= q << 25; q ^= q >> 27;
      return (unsigned)((q * 0x2545f4914f6cdd1dULL) >> 33) % m;
    };
    for (int k = 0; k < (N.wper > 0 ? N.wper : 1); ++k) {
      int z0 = 0, y0 = 0, x0 = 0;
      if (N.wper > 0) {
        z0 = (int)rnd((unsigned)(Nk - N.sD + 1));
        y0 = (int)rnd((unsigned)(Ni - N.sH + 1));
        x0 = (int)rnd((unsigned)(Nj - N.sW + 1));
      }
      float* smp = N.store + (size_t)N.next * kPlanes * sV;
      launch(k_record, grid_for(sV), kThreads, c.st, d, (const double*)c.f[CAP_RES], (const double*)c.f[CAP_AE],
             (const double*)c.f[CAP_AW], (const double*)c.f[CAP_AN], (const double*)c.f[CAP_AS],
             (const double*)c.f[CAP_AT], (const double*)c.f[CAP_AB], (const double*)c.f[CAP_AP],
             (const double*)c.redout, Ni, Nj, Nk, z0, y0, x0, N.sD, N.sH, N.sW, smp);
      CAP_CHECK_LAUNCH();
      N.pend.push_back(make_int4(N.next, z0, y0, x0));
      N.next = (N.next + 1) % N.max_samples;
      if (N.nsamples < N.max_samples) ++N.nsamples;
    }
  }
  if (!guess) return CAPPGPU_OK;
  // the guess: fi + alpha * net(r0 / rms(r0)), kept only if it lowers the
  // FP64 residual
  const int D = round4(Nk), H = round4(Ni), W = round4(Nj);
  if ((rc = ensure_acts((long long)D * H * W))) return rc;
  launch(k_rhs_in, grid_for((long long)D * H * W), kThreads, c.st, d, (const double*)c.f[CAP_RES],
         (const double*)c.redout, Ni, Nj, Nk, N.A.a0, D, H, W);
  CAP_CHECK_LAUNCH();
  if ((rc = forward(D, H, W))) return rc;
  if ((rc = check_err())) return rc;
  // amplitude and level of the guess, fi + alpha d + beta (beta on the
  // interior), by Galerkin projection onto span{d, 1}: the pair that
  // minimises the error in the energy norm of A, the norm CG minimises, so
  // the guess cannot start CG from a larger energy error (a residual
  // least-squares fit can: it weights the high frequencies, and on a
  // Neumann system pinned at one cell it left smooth error that cost CG
  // 2.4x the iterations of the plain solve).  A is symmetric apart from the
  // pinned row.
  double* shape = c.work[4];
  double* ashape = c.work[5];
  double* one = c.work[6];
  double* aone = c.work[7];
  double* cand = c.work[2];
  double* rcand = c.work[3];
  CAP_CUDA(cudaMemsetAsync(shape, 0, sizeof(double) * d.nijk, c.st));
  CAP_CUDA(cudaMemsetAsync(one, 0, sizeof(double) * d.nijk, c.st));
  launch(k_shape_nat, grid_for(Vi), kThreads, c.st, d, shape, (const float*)N.A.out, Ni, Nj, Nk, H, W);
  launch(k_ones_nat, grid_for(Vi), kThreads, c.st, d, one, Ni, Nj, Nk);
  CAP_CHECK_LAUNCH();
  double t[2], g1[2], g2[2], rr[2];
  if ((rc = spmv_dot2_natural(shape, ashape, c.f[CAP_RES], t))) return rc;   // Ad
  if ((rc = spmv_dot2_natural(one, aone, c.f[CAP_RES], t))) return rc;       // A1
  if ((rc = dot2_natural(shape, ashape, shape, aone, g1))) return rc;         // d.Ad, d.A1
  if ((rc = dot2_natural(one, ashape, one, aone, g2))) return rc;             // 1.Ad, 1.A1
  if ((rc = dot2_natural(shape, c.f[CAP_RES], one, c.f[CAP_RES], rr))) return rc;   // d.r0, 1.r0
  double alpha = 0.0, beta = 0.0;
  const double det = g1[0] * g2[1] - g1[1] * g2[0];
  if (g2[1] > 0.0 && fabs(det) > 1e-12 * fabs(g1[0] * g2[1])) {
    alpha = (rr[0] * g2[1] - g1[1] * rr[1]) / det;
    beta = (g1[0] * rr[1] - g2[0] * rr[0]) / det;
  } else if (g1[0] > 0.0) {
    alpha = rr[0] / g1[0];
  }
  N.last_alpha = alpha;
  N.last_beta = beta;
  if (!isfinite(alpha) || !isfinite(beta) || (alpha == 0.0 && beta == 0.0)) {
    ++N.fallbacks;
    return CAPPGPU_OK;
  }
  CAP_CUDA(cudaMemcpyAsync(cand, c.f[fif], sizeof(double) * d.nijk, cudaMemcpyDeviceToDevice, c.st));
  launch(k_axpy_nat, grid_for(d.nijk), kThreads, c.st, d.nijk, alpha, (const double*)shape, cand);
  launch(k_axpy_nat, grid_for(d.nijk), kThreads, c.st, d.nijk, beta, (const double*)one, cand);
  CAP_CHECK_LAUNCH();
  double res1 = 0.0;
  if ((rc = resid_into(cand, rcand, &res1))) return rc;
  N.last_ratio = res1 / res0;
  if (isfinite(res1) && res1 < res0) {
    CAP_CUDA(cudaMemcpyAsync(c.f[fif], cand, sizeof(double) * d.nijk, cudaMemcpyDeviceToDevice, c.st));
    CAP_CUDA(cudaMemcpyAsync(c.f[CAP_RES], rcand, sizeof(double) * d.nijk, cudaMemcpyDeviceToDevice, c.st));
    ++N.guesses;
  } else {
    ++N.fallbacks;
  }
  return CAPPGPU_OK;
}

// At the end of a solve: the converged correction t^ of the windows its
// start recorded.
int learned_solve_end(int fif) {
  if (N.pend.empty()) return CAPPGPU_OK;
  Ctx& c = ctx();
  const Dims& d = c.d;
  const int Ni = d.nimm - 2, Nj = d.njmm - 2, Nk = d.nkmm - 2;
  const long long sV = (long long)N.sD * N.sH * N.sW;
  for (const int4& q : N.pend) {
    launch(k_record_target, grid_for(sV), kThreads, c.st, d, (const double*)c.f[fif], (const double*)N.fi0,
           (const double*)N.tsum, Ni, Nj, Nk, q.y, q.z, q.w, N.sD, N.sH, N.sW,
           N.store + ((size_t)q.x * kPlanes + 8) * sV);
    CAP_CHECK_LAUNCH();
  }
  N.pend.clear();
  return CAPPGPU_OK;
}

int learned_set_loss(int kind) {
  if (kind < 0 || kind > 2) return CAPPGPU_E_ARG;
  N.loss = kind;
  return CAPPGPU_OK;
}

}  // namespace cap

using namespace cap;

extern "C" {

int cappgpu_learn_reset(int max_samples, unsigned long long seed) {
  CAP_REQUIRE_INIT();
  if (max_samples < 0) { set_error("learn_reset: max_samples < 0"); return CAPPGPU_E_ARG; }
  net_free();
  const Dims& d = ctx().d;
  N.sD = d.nkmm - 2;
  N.sH = d.nimm - 2;
  N.sW = d.njmm - 2;
  const long long V = (long long)N.sD * N.sH * N.sW;
  CAP_CUDA(cudaMalloc(&N.p, sizeof(float) * kParams));
  CAP_CUDA(cudaMalloc(&N.gp, sizeof(float) * kParams));
  CAP_CUDA(cudaMalloc(&N.m, sizeof(float) * kParams));
  CAP_CUDA(cudaMalloc(&N.v, sizeof(float) * kParams));
  CAP_CUDA(cudaMalloc(&N.wb, sizeof(bf16) * kWAll));
  CAP_CUDA(cudaMalloc(&N.wt, sizeof(bf16) * kWAll));
  CAP_CUDA(cudaMalloc(&N.dsum, sizeof(double) * 4));
  CAP_CUDA(cudaMalloc(&N.err, sizeof(int)));
  CAP_CUDA(cudaMemset(N.err, 0, sizeof(int)));
  CAP_CUDA(cudaMemset(N.gp, 0, sizeof(float) * kParams));
  CAP_CUDA(cudaMemset(N.dsum, 0, sizeof(double) * 4));
  if (max_samples > 0 && cudaMalloc(&N.store, sizeof(float) * kPlanes * (size_t)max_samples * V) != cudaSuccess) {
    net_free();
    set_error("learn_reset: out of device memory for %d samples", max_samples);
    return CAPPGPU_E_NOMEM;
  }
  N.max_samples = max_samples;
  N.seed = seed;
  int rc = init_params(seed);
  if (rc) return rc;
  N.ready = true;
  CAP_CUDA(cudaStreamSynchronize(ctx().st));
  return CAPPGPU_OK;
}

int cappgpu_learn_windows(int block, int per_solve) {
  CAP_REQUIRE_INIT();
  if (!N.ready) { set_error("learn_windows: call cappgpu_learn_reset first"); return CAPPGPU_E_NOINIT; }
  const Dims& d = ctx().d;
  const int Ni = d.nimm - 2, Nj = d.njmm - 2, Nk = d.nkmm - 2;
  if (per_solve < 1 || block < 4 || block % 4 != 0 || block > Ni || block > Nj || block > Nk) {
    set_error("learn_windows: block %d (a multiple of 4 within the interior %d x %d x %d), %d windows per solve",
              block, Ni, Nj, Nk, per_solve);
    return CAPPGPU_E_ARG;
  }
  cudaFree(N.store);
  N.store = nullptr;
  const long long V = (long long)block * block * block;
  if (N.max_samples > 0 && cudaMalloc(&N.store, sizeof(float) * kPlanes * (size_t)N.max_samples * V) != cudaSuccess) {
    N.max_samples = 0;
    set_error("learn_windows: out of device memory for the windows");
    return CAPPGPU_E_NOMEM;
  }
  N.sD = N.sH = N.sW = block;
  N.wper = per_solve;
  N.wrng = N.seed * 0x9e3779b97f4a7c15ULL + 777;
  N.nsamples = N.next = 0;
  return CAPPGPU_OK;
}

int cappgpu_learn_collect(int on) {
  CAP_REQUIRE_INIT();
  if (!N.ready) { set_error("learn_collect: call cappgpu_learn_reset first"); return CAPPGPU_E_NOINIT; }
  N.collect = on != 0;
  return CAPPGPU_OK;
}

int cappgpu_learn_train(int epochs, int block, double lr, double* loss) {
  CAP_REQUIRE_INIT();
  if (!N.ready || N.nsamples == 0) { set_error("learn_train: no recorded pairs"); return CAPPGPU_E_NOINIT; }
  if (epochs < 1 || block < 4 || !(lr > 0.0)) { set_error("learn_train: bad arguments"); return CAPPGPU_E_ARG; }
  const int B = min(block, min(N.sD, min(N.sH, N.sW))) & ~3;
  if (B < 4) { set_error("learn_train: the grid is smaller than 4 cells"); return CAPPGPU_E_ARG; }
  Ctx& c = ctx();
  const int V = B * B * B;
  int rc = ensure_acts(V);
  if (rc) return rc;
  const long long sV = (long long)N.sD * N.sH * N.sW;
  unsigned long long s = N.seed * 0x9e3779b97f4a7c15ULL + 12345;
  auto rnd = [&](unsigned m) {   // xorshift64*
    s ^= s >> 12; s ^= s << 25; s ^= s >> 27;
    return (unsigned)((s * 0x2545f4914f6cdd1dULL) >> 33) % m;
  };
  double last = 0.0;
  for (int e = 0; e < epochs; ++e) {
    double sum = 0.0;
    for (int k = 0; k < N.nsamples; ++k) {
      const int sidx = (int)rnd((unsigned)N.nsamples);
      const int z0 = (int)rnd((unsigned)(N.sD - B + 1)), y0 = (int)rnd((unsigned)(N.sH - B + 1)),
                x0 = (int)rnd((unsigned)(N.sW - B + 1));
      launch(k_window, grid_for(V), kThreads, c.st, (const float*)(N.store + (size_t)sidx * kPlanes * sV), N.sD, N.sH,
             N.sW, z0, y0, x0, B, N.A.a0, N.A.rhs, N.A.coef, N.A.tgt);
      CAP_CHECK_LAUNCH();
      if ((rc = forward(B, B, B))) return rc;
      if ((rc = backward(B, B, B))) return rc;
      if ((rc = adam_step((float)lr))) return rc;
      double h = 0.0;
      CAP_CUDA(cudaMemcpyAsync(&h, N.dsum, sizeof(double), cudaMemcpyDeviceToHost, c.st));
      if ((rc = check_err())) return rc;
      sum += h;
    }
    last = sum / N.nsamples;
  }
  N.trained = true;
  if (loss) *loss = last;
  return CAPPGPU_OK;
}

int cappgpu_learn_params(float* host, int n, int direction) {
  CAP_REQUIRE_INIT();
  if (!N.ready) { set_error("learn_params: call cappgpu_learn_reset first"); return CAPPGPU_E_NOINIT; }
  if (!host) return kParams;
  if (n != kParams) { set_error("learn_params: %d values, the net has %d", n, kParams); return CAPPGPU_E_ARG; }
  if (direction == 0) {
    CAP_CUDA(cudaMemcpy(host, N.p, sizeof(float) * kParams, cudaMemcpyDeviceToHost));
  } else {
    CAP_CUDA(cudaMemcpy(N.p, host, sizeof(float) * kParams, cudaMemcpyHostToDevice));
    // new parameters: Adam starts afresh
    CAP_CUDA(cudaMemsetAsync(N.m, 0, sizeof(float) * kParams, ctx().st));
    CAP_CUDA(cudaMemsetAsync(N.v, 0, sizeof(float) * kParams, ctx().st));
    N.adam_t = 0;
    int rc = cast_weights();
    if (rc) return rc;
    N.trained = true;
    CAP_CUDA(cudaStreamSynchronize(ctx().st));
  }
  return kParams;
}

int cappgpu_learn_stats(int* samples, int* guesses, int* fallbacks, double* last_ratio) {
  CAP_REQUIRE_INIT();
  if (samples) *samples = N.nsamples;
  if (guesses) *guesses = N.guesses;
  if (fallbacks) *fallbacks = N.fallbacks;
  if (last_ratio) *last_ratio = N.last_ratio;
  return CAPPGPU_OK;
}

int cappgpu_learn_fit(double* alpha, double* beta) {
  CAP_REQUIRE_INIT();
  if (alpha) *alpha = N.last_alpha;
  if (beta) *beta = N.last_beta;
  return CAPPGPU_OK;
}

int cappgpu_learn_check_loss(int kind, const float* rhs, const float* coef, const float* target, int D, int H, int W,
                             float* output, float* grad, double* loss) {
  CAP_REQUIRE_INIT();
  if (!N.ready) { set_error("learn_check: call cappgpu_learn_reset first"); return CAPPGPU_E_NOINIT; }
  if (!rhs || !coef || D < 4 || H < 4 || W < 4 || ((D | H | W) & 3)) {
    set_error("learn_check: extents must be multiples of 4");
    return CAPPGPU_E_ARG;
  }
  if (kind < 0 || kind > 2 || (kind > 0 && !target)) {
    set_error("learn_check: loss kind %d (0 residual, 1 supervised, 2 energy; 1-2 need the target)", kind);
    return CAPPGPU_E_ARG;
  }
  Ctx& c = ctx();
  const long long V = (long long)D * H * W;
  int rc = ensure_acts(V);
  if (rc) return rc;
  std::vector<bf16> in((size_t)V * 16, __float2bfloat16(0.f));
  for (long long v = 0; v < V; ++v) in[v * 16] = __float2bfloat16(rhs[v]);
  CAP_CUDA(cudaMemcpy(N.A.a0, in.data(), sizeof(bf16) * in.size(), cudaMemcpyHostToDevice));
  CAP_CUDA(cudaMemcpy(N.A.rhs, rhs, sizeof(float) * V, cudaMemcpyHostToDevice));
  CAP_CUDA(cudaMemcpy(N.A.coef, coef, sizeof(float) * 7 * V, cudaMemcpyHostToDevice));
  if (target) CAP_CUDA(cudaMemcpy(N.A.tgt, target, sizeof(float) * V, cudaMemcpyHostToDevice));
  const int keep = N.loss;
  N.loss = kind;
  if (!(rc = forward(D, H, W))) rc = backward(D, H, W);
  N.loss = keep;
  if (rc) return rc;
  if ((rc = check_err())) return rc;
  if (output) CAP_CUDA(cudaMemcpy(output, N.A.out, sizeof(float) * V, cudaMemcpyDeviceToHost));
  if (grad) CAP_CUDA(cudaMemcpy(grad, N.gp, sizeof(float) * kParams, cudaMemcpyDeviceToHost));
  if (loss) CAP_CUDA(cudaMemcpy(loss, N.dsum, sizeof(double), cudaMemcpyDeviceToHost));
  return CAPPGPU_OK;
}

int cappgpu_learn_check(const float* rhs, const float* coef, int D, int H, int W, float* output, float* grad,
                        double* loss) {
  return cappgpu_learn_check_loss(0, rhs, coef, nullptr, D, H, W, output, grad, loss);
}

int cappgpu_learn_sample(int index, float* host, long long n) {
  CAP_REQUIRE_INIT();
  if (!N.ready) { set_error("learn_sample: call cappgpu_learn_reset first"); return CAPPGPU_E_NOINIT; }
  const long long sV = (long long)N.sD * N.sH * N.sW, need = kPlanes * sV;
  if (index < 0 || index >= N.nsamples) {
    set_error("learn_sample: pair %d of %d recorded", index, N.nsamples);
    return CAPPGPU_E_ARG;
  }
  if (!host || n != need) {
    set_error("learn_sample: %lld values for %d planes of %d x %d x %d", need, kPlanes, N.sD, N.sH, N.sW);
    return CAPPGPU_E_ARG;
  }
  CAP_CUDA(cudaStreamSynchronize(ctx().st));
  CAP_CUDA(cudaMemcpy(host, N.store + (size_t)index * need, sizeof(float) * need, cudaMemcpyDeviceToHost));
  return CAPPGPU_OK;
}

}  // extern "C"
