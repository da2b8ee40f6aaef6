// learned.cu -- the learned initial guess of the pressure solve
// (cappgpu_precision(2); no counterpart in the reference).
//
// A small 3-D convolutional net predicts the shape of the correction
// d = A^-1 r0 of a pressure solve from its initial residual r0 (input
// normalised by the mean |r0|, target by the mean |d|); the amplitude is
// fitted at solve time by least squares, alpha = (r0.Ad)/(Ad.Ad), which
// costs one product with A.  The plain solve always continues from the guess
// to the same tolerance -- the exit test stays relative to the residual of
// the solve's own start -- so the solver is both judge and fallback: a guess
// that does not lower the FP64 residual is discarded.
//
// Net: four 3x3x3 convolutions of 16 channels with dilations 1, 2, 4, 8 and
// ReLU, then a 1x1x1 convolution to one channel (receptive field 31 cells).
// Activations and weights are BF16, accumulation FP32, FP32 master weights,
// Adam.  Convolutions are implicit GEMMs on the tensor cores (mma.sync
// m16n8k16): forward and input gradient (the same kernel with flipped,
// transposed weights) take 16 output voxels x 16 channels per warp and K = 27
// taps x 16 channels; the weight gradient is a GEMM over voxels per tap,
// split in chunks and summed in a fixed order.  Training pairs are recorded by
// the solver itself (cappgpu_learn_collect) and the net is trained on random
// cubic windows of them (cappgpu_learn_train).
#include <cuda_bf16.h>
#include <math.h>
#include <string.h>

#include <vector>

#include "common.cuh"
#include "kernels.cuh"

namespace cap {

namespace {

typedef __nv_bfloat16 bf16;
constexpr int kC = 16;                 // channels of the hidden layers
constexpr int kLayers = 4;             // 3x3x3 layers
constexpr int kWConv = kC * 27 * kC;   // weights of one 3x3x3 layer, [co][tap][ci]
constexpr int kParams = kLayers * (kWConv + kC) + kC + 1;
__host__ __device__ constexpr int offW(int l) { return l * (kWConv + kC); }
__host__ __device__ constexpr int offB(int l) { return l * (kWConv + kC) + kWConv; }
constexpr int kOffLastW = kLayers * (kWConv + kC);
constexpr int kOffLastB = kOffLastW + kC;
constexpr int kDil[kLayers] = {1, 2, 4, 8};
constexpr int kChunk = 4096;           // voxels per weight-gradient partial

struct Net {
  bool ready = false, trained = false, collect = false;
  float *p = nullptr, *gp = nullptr, *m = nullptr, *v = nullptr;   // parameters, gradients, Adam moments
  bf16* wb = nullptr;    // BF16 conv weights [layer][co][tap][ci]
  bf16* wt = nullptr;    // flipped, transposed [layer][ci][tap][co] (input gradient)
  int adam_t = 0;
  long long maxV = 0;
  bf16* act[kLayers + 1] = {};   // act[0] input (16 channels, channel 0 used); act[l+1] output of layer l
  float* out = nullptr;          // output (1 channel)
  float* tgt = nullptr;          // training target
  float* gout = nullptr;         // dL/dout
  bf16* g[2] = {};               // gradients w.r.t. activations
  float* part = nullptr;         // partial sums
  size_t part_n = 0;
  double* dsum = nullptr;        // device scalars
  // recorded pairs
  int max_samples = 0, nsamples = 0, next = 0;
  int sD = 0, sH = 0, sW = 0;
  bf16* srhs = nullptr;          // [max_samples][sV] normalised initial residual
  float* sdel = nullptr;         // [max_samples][sV] normalised correction
  double* fi0 = nullptr;         // interior of fi at the start of the solve being recorded
  int pending = -1;              // slot of the sample whose correction is still to come
  // statistics of the guesses
  int guesses = 0, fallbacks = 0;
  double last_ratio = 0.0;
  unsigned long long seed = 0;
};

Net N;

void net_free() {
  cudaFree(N.p); cudaFree(N.gp); cudaFree(N.m); cudaFree(N.v);
  cudaFree(N.wb); cudaFree(N.wt);
  for (auto& a : N.act) cudaFree(a);
  cudaFree(N.out); cudaFree(N.tgt); cudaFree(N.gout);
  cudaFree(N.g[0]); cudaFree(N.g[1]);
  cudaFree(N.part); cudaFree(N.dsum);
  cudaFree(N.srhs); cudaFree(N.sdel); cudaFree(N.fi0);
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

// voxel v of a D x H x W grid (x fastest); neighbour at (dz,dy,dx) or -1
__device__ __forceinline__ long long nbr(long long v, int dz, int dy, int dx, int D, int H, int W) {
  const int x = (int)(v % W);
  const long long r = v / W;
  const int y = (int)(r % H), z = (int)(r / H);
  const int zz = z + dz, yy = y + dy, xx = x + dx;
  if (zz < 0 || zz >= D || yy < 0 || yy >= H || xx < 0 || xx >= W) return -1;
  return ((long long)zz * H + yy) * W + xx;
}

__device__ __forceinline__ void tap_off(int tap, int dil, int& dz, int& dy, int& dx) {
  dz = (tap / 9 - 1) * dil;
  dy = ((tap / 3) % 3 - 1) * dil;
  dx = (tap % 3 - 1) * dil;
}

// two channels (c, c+1) of voxel n; with a mask, a channel counts only where
// the mask activation is positive (ReLU derivative)
__device__ __forceinline__ unsigned load_pair(const bf16* __restrict__ x, const bf16* __restrict__ mask, long long n,
                                              int c) {
  if (n < 0) return 0u;
  unsigned u = *reinterpret_cast<const unsigned*>(x + n * kC + c);
  if (mask) {
    const unsigned mk = *reinterpret_cast<const unsigned*>(mask + n * kC + c);
    const unsigned lo = mk & 0xffffu, hi = mk >> 16;
    if (!(lo != 0u && (lo & 0x8000u) == 0u)) u &= 0xffff0000u;
    if (!(hi != 0u && (hi & 0x8000u) == 0u)) u &= 0x0000ffffu;
  }
  return u;
}

// y = act(conv3x3x3(x * [mask > 0], w) + bias): 16 -> 16 channels, dilation
// dil, zero padding.  One warp: 16 voxels x 16 output channels.
__global__ void __launch_bounds__(256) k_conv3(const bf16* __restrict__ x, const bf16* __restrict__ w,
                                               const float* __restrict__ bias, const bf16* __restrict__ mask,
                                               bf16* __restrict__ y, int D, int H, int W, int dil, int relu) {
  __shared__ unsigned ws[kWConv / 2];
  for (int q = threadIdx.x; q < kWConv / 2; q += blockDim.x) ws[q] = reinterpret_cast<const unsigned*>(w)[q];
  __syncthreads();
  const long long V = (long long)D * H * W;
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const long long vb = ((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5) * 16;
  if (vb >= V) return;
  const long long v0 = vb + g, v1 = vb + g + 8;
  float acc[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
  for (int tap = 0; tap < 27; ++tap) {
    int dz, dy, dx;
    tap_off(tap, dil, dz, dy, dx);
    const long long n0 = v0 < V ? nbr(v0, dz, dy, dx, D, H, W) : -1;
    const long long n1 = v1 < V ? nbr(v1, dz, dy, dx, D, H, W) : -1;
    unsigned a[4];
    a[0] = load_pair(x, mask, n0, t * 2);
    a[1] = load_pair(x, mask, n1, t * 2);
    a[2] = load_pair(x, mask, n0, 8 + t * 2);
    a[3] = load_pair(x, mask, n1, 8 + t * 2);
#pragma unroll
    for (int nt = 0; nt < 2; ++nt) {
      const int co = nt * 8 + g;
      unsigned b[2];
      b[0] = ws[((co * 27 + tap) * kC + t * 2) / 2];
      b[1] = ws[((co * 27 + tap) * kC + 8 + t * 2) / 2];
      mma16816(acc[nt], a, b);
    }
  }
#pragma unroll
  for (int nt = 0; nt < 2; ++nt) {
    const int co = nt * 8 + t * 2;
    const float b0 = bias ? bias[co] : 0.f, b1 = bias ? bias[co + 1] : 0.f;
    float r[4] = {acc[nt][0] + b0, acc[nt][1] + b1, acc[nt][2] + b0, acc[nt][3] + b1};
    if (relu)
      for (int q = 0; q < 4; ++q) r[q] = fmaxf(r[q], 0.f);
    if (v0 < V) *reinterpret_cast<unsigned*>(y + v0 * kC + co) = pack2(__float2bfloat16(r[0]), __float2bfloat16(r[1]));
    if (v1 < V) *reinterpret_cast<unsigned*>(y + v1 * kC + co) = pack2(__float2bfloat16(r[2]), __float2bfloat16(r[3]));
  }
}

// partial weight gradients of a 3x3x3 layer: for one tap and one chunk of
// voxels, G[co][ci] = sum_v gy[v][co] [y[v][co] > 0] x[v + off(tap)][ci]
__global__ void __launch_bounds__(128) k_wgrad3(const bf16* __restrict__ x, const bf16* __restrict__ gy,
                                                const bf16* __restrict__ y, float* __restrict__ part, int D, int H,
                                                int W, int dil) {
  __shared__ float red[4][kC * kC];
  const long long V = (long long)D * H * W;
  const int tap = blockIdx.x, ch = blockIdx.y;
  const long long vs = (long long)ch * kChunk, ve = min(V, vs + kChunk);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  int dz, dy, dx;
  tap_off(tap, dil, dz, dy, dx);
  auto gm = [&](long long v, int co) -> bf16 {   // masked output gradient
    if (v >= ve) return __float2bfloat16(0.f);
    const bf16 yy = y[v * kC + co];
    return __bfloat162float(yy) > 0.f ? gy[v * kC + co] : __float2bfloat16(0.f);
  };
  auto xs = [&](long long v, int ci) -> bf16 {   // shifted input
    if (v >= ve) return __float2bfloat16(0.f);
    const long long n = nbr(v, dz, dy, dx, D, H, W);
    return n < 0 ? __float2bfloat16(0.f) : x[n * kC + ci];
  };
  float acc[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
  for (long long vb = vs + warp * 16; vb < ve; vb += 64) {
    unsigned a[4];   // A[co][v] (16 x 16)
    a[0] = pack2(gm(vb + t * 2, g), gm(vb + t * 2 + 1, g));
    a[1] = pack2(gm(vb + t * 2, g + 8), gm(vb + t * 2 + 1, g + 8));
    a[2] = pack2(gm(vb + 8 + t * 2, g), gm(vb + 9 + t * 2, g));
    a[3] = pack2(gm(vb + 8 + t * 2, g + 8), gm(vb + 9 + t * 2, g + 8));
#pragma unroll
    for (int nt = 0; nt < 2; ++nt) {   // B[v][ci] (16 x 8)
      const int ci = nt * 8 + g;
      unsigned b[2];
      b[0] = pack2(xs(vb + t * 2, ci), xs(vb + t * 2 + 1, ci));
      b[1] = pack2(xs(vb + 8 + t * 2, ci), xs(vb + 9 + t * 2, ci));
      mma16816(acc[nt], a, b);
    }
  }
#pragma unroll
  for (int nt = 0; nt < 2; ++nt) {
    const int ci = nt * 8 + t * 2;
    red[warp][g * kC + ci] = acc[nt][0];
    red[warp][g * kC + ci + 1] = acc[nt][1];
    red[warp][(g + 8) * kC + ci] = acc[nt][2];
    red[warp][(g + 8) * kC + ci + 1] = acc[nt][3];
  }
  __syncthreads();
  for (int q = threadIdx.x; q < kC * kC; q += blockDim.x)
    part[((size_t)ch * 27 + tap) * kC * kC + q] = ((red[0][q] + red[1][q]) + red[2][q]) + red[3][q];
}

// gradient of layer l: W[co][tap][ci] = sum over chunks (fixed order)
__global__ void k_wgrad_sum(const float* __restrict__ part, int nch, float* __restrict__ gw) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;   // (tap, co, ci)
  if (q >= 27 * kC * kC) return;
  const int tap = q / (kC * kC), co = (q / kC) % kC, ci = q % kC;
  float s = 0.f;
  for (int c = 0; c < nch; ++c) s += part[((size_t)c * 27 + tap) * kC * kC + co * kC + ci];
  gw[(co * 27 + tap) * kC + ci] = s;
}

// bias gradient partials of a 3x3x3 layer: sum_v gy[v][co] [y > 0]
__global__ void k_bgrad(const bf16* __restrict__ gy, const bf16* __restrict__ y, long long V, float* part) {
  __shared__ float sh[256];
  const int co = threadIdx.x & (kC - 1), row = threadIdx.x >> 4;   // 16 rows x 16 channels
  float s = 0.f;
  for (long long v = blockIdx.x * 16LL + row; v < V; v += 16LL * gridDim.x) {
    const float yy = __bfloat162float(y[v * kC + co]);
    if (yy > 0.f) s += __bfloat162float(gy[v * kC + co]);
  }
  sh[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x < kC) {
    float r = 0.f;
    for (int q = 0; q < 16; ++q) r += sh[q * kC + threadIdx.x];
    part[blockIdx.x * kC + threadIdx.x] = r;
  }
}

__global__ void k_sum_cols(const float* __restrict__ part, int rows, int cols, float* __restrict__ out) {
  const int c = threadIdx.x;
  if (c >= cols) return;
  float s = 0.f;
  for (int r = 0; r < rows; ++r) s += part[r * cols + c];
  out[c] = s;
}

// out = b + sum_ci w[ci] x[v][ci] (1x1x1 convolution to one channel)
__global__ void k_last_fwd(const bf16* __restrict__ x, const float* __restrict__ p, float* __restrict__ out, long long V) {
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x) {
    float s = p[kOffLastB];
#pragma unroll
    for (int c = 0; c < kC; ++c) s += p[kOffLastW + c] * __bfloat162float(x[v * kC + c]);
    out[v] = s;
  }
}

// dL/dout of the mean squared error and partial sums of the squared error
__global__ void k_mse(const float* __restrict__ out, const float* __restrict__ tgt, float* __restrict__ gout, long long V,
                      double* part) {
  double v[1] = {0.0};
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < V; q += (long long)gridDim.x * blockDim.x) {
    const float d = out[q] - tgt[q];
    gout[q] = 2.f * d / (float)V;
    v[0] += (double)d * d;
  }
  block_reduce_store<1>(v, part);
}

// backward of the 1x1x1 layer: dx[v][ci] = w[ci] gout[v]; partials of
// dw[ci] = sum gout x and db = sum gout (17 values per block)
__global__ void k_last_bwd(const bf16* __restrict__ x, const float* __restrict__ gout, const float* __restrict__ p,
                           bf16* __restrict__ gx, long long V, float* part) {
  __shared__ float sh[kC + 1][256 / 32];
  float acc[kC + 1];
  for (int c = 0; c <= kC; ++c) acc[c] = 0.f;
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x) {
    const float go = gout[v];
#pragma unroll
    for (int c = 0; c < kC; ++c) {
      acc[c] += go * __bfloat162float(x[v * kC + c]);
      gx[v * kC + c] = __float2bfloat16(p[kOffLastW + c] * go);
    }
    acc[kC] += go;
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int c = 0; c <= kC; ++c) {
    float y = acc[c];
    for (int o = 16; o > 0; o >>= 1) y += __shfl_down_sync(0xffffffffu, y, o);
    if (lane == 0) sh[c][wid] = y;
  }
  __syncthreads();
  if (threadIdx.x <= kC) {
    float s = 0.f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += sh[threadIdx.x][w];
    part[blockIdx.x * (kC + 1) + threadIdx.x] = s;
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
  const int q = blockIdx.x * blockDim.x + threadIdx.x;   // (l, co, tap, ci)
  if (q >= kLayers * kWConv) return;
  const int l = q / kWConv, r = q % kWConv;
  const int co = r / (27 * kC), tap = (r / kC) % 27, ci = r % kC;
  const bf16 w = __float2bfloat16(p[offW(l) + r]);
  wb[q] = w;
  wt[(size_t)l * kWConv + (ci * 27 + (26 - tap)) * kC + co] = w;
}

// training window: input (channel 0 = normalised residual) and target
__global__ void k_window(const bf16* __restrict__ srhs, const float* __restrict__ sdel, int sD, int sH, int sW, int z0,
                         int y0, int x0, int B, bf16* __restrict__ in, float* __restrict__ tgt) {
  const long long V = (long long)B * B * B;
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(v % B), y = (int)((v / B) % B), z = (int)(v / ((long long)B * B));
    const long long s = ((long long)(z + z0) * sH + (y + y0)) * sW + (x + x0);
    in[v * kC] = srhs[s];
#pragma unroll
    for (int c = 1; c < kC; ++c) in[v * kC + c] = __float2bfloat16(0.f);
    tgt[v] = sdel[s];
  }
}

// interior of a natural-layout field (k, i, j order: z = k, y = i, x = j)
__device__ __forceinline__ int nat_of(const Dims& d, long long v, int Ni, int Nj) {
  const int x = (int)(v % Nj);
  const long long r = v / Nj;
  const int y = (int)(r % Ni), z = (int)(r / Ni);
  return ixk(d, y + 3, x + 3, z + 3);
}

__global__ void k_rhs_in(Dims d, const double* __restrict__ r, double inv_scale, bf16* __restrict__ in,
                         bf16* __restrict__ rec, long long V, int Ni, int Nj) {
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x) {
    const bf16 q = __float2bfloat16((float)(r[nat_of(d, v, Ni, Nj)] * inv_scale));
    if (in) {
      in[v * kC] = q;
#pragma unroll
      for (int c = 1; c < kC; ++c) in[v * kC + c] = __float2bfloat16(0.f);
    }
    if (rec) rec[v] = q;
  }
}

__global__ void k_save_interior(Dims d, const double* __restrict__ fi, double* __restrict__ dst, long long V, int Ni, int Nj) {
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x)
    dst[v] = fi[nat_of(d, v, Ni, Nj)];
}

// the correction of a recorded solve and partial sums of its |.|
__global__ void k_record_delta(Dims d, const double* __restrict__ fi, const double* __restrict__ fi0,
                               float* __restrict__ del, long long V, int Ni, int Nj, double* part) {
  double a[1] = {0.0};
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x) {
    const double x = fi[nat_of(d, v, Ni, Nj)] - fi0[v];
    del[v] = (float)x;
    a[0] += fabs(x);
  }
  block_reduce_store<1>(a, part);
}

__global__ void k_scale_f(float* __restrict__ x, long long V, const double* __restrict__ sum) {
  const float inv = sum[0] > 0.0 ? (float)((double)V / sum[0]) : 0.f;   // 1 / mean |x|
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x)
    x[v] *= inv;
}

// the predicted shape on the interior of a natural field, zero elsewhere
__global__ void k_shape_nat(Dims d, double* __restrict__ z, const float* __restrict__ out, long long V, int Ni, int Nj) {
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x)
    z[nat_of(d, v, Ni, Nj)] = (double)out[v];
}

__global__ void k_axpy_nat(int n, double alpha, const double* __restrict__ x, double* __restrict__ y) {
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) y[q] = y[q] + alpha * x[q];
}

// ------------------------------------------------------------ host side
int ensure_act(long long V) {
  if (V <= N.maxV) return CAPPGPU_OK;
  for (auto& a : N.act) { cudaFree(a); a = nullptr; }
  cudaFree(N.out); cudaFree(N.tgt); cudaFree(N.gout); cudaFree(N.g[0]); cudaFree(N.g[1]); cudaFree(N.part);
  N.out = N.tgt = N.gout = nullptr; N.g[0] = N.g[1] = nullptr; N.part = nullptr;
  N.maxV = 0;
  const size_t na = (size_t)V * kC * sizeof(bf16);
  for (auto& a : N.act) CAP_CUDA(cudaMalloc(&a, na));
  CAP_CUDA(cudaMalloc(&N.g[0], na));
  CAP_CUDA(cudaMalloc(&N.g[1], na));
  CAP_CUDA(cudaMalloc(&N.out, V * sizeof(float)));
  CAP_CUDA(cudaMalloc(&N.tgt, V * sizeof(float)));
  CAP_CUDA(cudaMalloc(&N.gout, V * sizeof(float)));
  const long long nch = (V + kChunk - 1) / kChunk;
  N.part_n = (size_t)nch * 27 * kC * kC + 4096 * (kC + 1);
  CAP_CUDA(cudaMalloc(&N.part, N.part_n * sizeof(float)));
  N.maxV = V;
  return CAPPGPU_OK;
}

int cast_weights() {
  launch(k_cast_w, (kLayers * kWConv + 255) / 256, 256, ctx().st, (const float*)N.p, N.wb, N.wt);
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
  const float a3 = sqrtf(6.f / (27.f * kC)), a1 = sqrtf(3.f / kC);   // He-uniform
  for (int l = 0; l < kLayers; ++l)
    for (int q = 0; q < kWConv; ++q) h[offW(l) + q] = a3 * uni();
  for (int c = 0; c < kC; ++c) h[kOffLastW + c] = a1 * uni() * 0.1f;
  Ctx& c = ctx();
  CAP_CUDA(cudaMemcpyAsync(N.p, h.data(), sizeof(float) * kParams, cudaMemcpyHostToDevice, c.st));
  CAP_CUDA(cudaMemsetAsync(N.m, 0, sizeof(float) * kParams, c.st));
  CAP_CUDA(cudaMemsetAsync(N.v, 0, sizeof(float) * kParams, c.st));
  N.adam_t = 0;
  return cast_weights();
}

// forward pass on act[0] (V voxels, D x H x W)
int forward(int D, int H, int W) {
  Ctx& c = ctx();
  const long long V = (long long)D * H * W;
  const int blocks = (int)((V + 127) / 128);   // 8 warps x 16 voxels
  for (int l = 0; l < kLayers; ++l) {
    launch(k_conv3, blocks, 256, c.st, (const bf16*)N.act[l], (const bf16*)(N.wb + (size_t)l * kWConv),
           (const float*)(N.p + offB(l)), (const bf16*)nullptr, N.act[l + 1], D, H, W, kDil[l], 1);
  }
  launch(k_last_fwd, grid_for(V), kThreads, c.st, (const bf16*)N.act[kLayers], (const float*)N.p, N.out, V);
  CAP_CHECK_LAUNCH();
  return CAPPGPU_OK;
}

// loss, backward pass into N.gp; loss returned on the device in dsum[0]
int backward(int D, int H, int W) {
  Ctx& c = ctx();
  const long long V = (long long)D * H * W;
  launch(k_mse, kRedBlocks, kThreads, c.st, (const float*)N.out, (const float*)N.tgt, N.gout, V, c.partials);
  CAP_CHECK_LAUNCH();
  int rc = finish_reduce(1);
  if (rc) return rc;
  CAP_CUDA(cudaMemcpyAsync(N.dsum, c.redout, sizeof(double), cudaMemcpyDeviceToDevice, c.st));
  const int lb = 512;
  launch(k_last_bwd, lb, 256, c.st, (const bf16*)N.act[kLayers], (const float*)N.gout, (const float*)N.p, N.g[0], V,
         N.part);
  launch(k_sum_cols, 1, 32, c.st, (const float*)N.part, lb, kC + 1, N.gp + kOffLastW);
  int cur = 0;
  const int nch = (int)((V + kChunk - 1) / kChunk);
  const int blocks = (int)((V + 127) / 128);
  for (int l = kLayers - 1; l >= 0; --l) {
    // weight and bias gradients of layer l (input act[l], output act[l+1])
    launch(k_wgrad3, dim3(27, nch), 128, c.st, (const bf16*)N.act[l], (const bf16*)N.g[cur], (const bf16*)N.act[l + 1],
           N.part, D, H, W, kDil[l]);
    launch(k_wgrad_sum, (27 * kC * kC + 255) / 256, 256, c.st, (const float*)N.part, nch, N.gp + offW(l));
    launch(k_bgrad, 256, 256, c.st, (const bf16*)N.g[cur], (const bf16*)N.act[l + 1], V, N.part);
    launch(k_sum_cols, 1, 32, c.st, (const float*)N.part, 256, kC, N.gp + offB(l));
    if (l > 0) {   // gradient with respect to act[l]
      launch(k_conv3, blocks, 256, c.st, (const bf16*)N.g[cur], (const bf16*)(N.wt + (size_t)l * kWConv),
             (const float*)nullptr, (const bf16*)N.act[l + 1], N.g[cur ^ 1], D, H, W, kDil[l], 0);
      cur ^= 1;
    }
  }
  CAP_CHECK_LAUNCH();
  return CAPPGPU_OK;
}

int adam_step(float lr) {
  ++N.adam_t;
  const float c1 = 1.f - powf(0.9f, (float)N.adam_t), c2 = 1.f - powf(0.999f, (float)N.adam_t);
  launch(k_adam, (kParams + 255) / 256, 256, ctx().st, N.p, (const float*)N.gp, N.m, N.v, kParams, lr, c1, c2);
  CAP_CHECK_LAUNCH();
  return cast_weights();
}

}  // namespace

void learned_free() { net_free(); }

// Record hooks and the guess, called by the refinement form of pcgsip.
// At the start of a solve: r0 (module res) and res0 are known.
int learned_solve_start(int fif, double res0) {
  if (!N.ready) return CAPPGPU_OK;
  Ctx& c = ctx();
  const Dims& d = c.d;
  const int Ni = d.nimm - 2, Nj = d.njmm - 2, Nk = d.nkmm - 2;
  const long long V = (long long)Ni * Nj * Nk;
  const double scale = res0 / (double)V;   // mean |r0|
  if (!(scale > 0.0) || !isfinite(scale)) return CAPPGPU_OK;
  N.pending = -1;
  if (N.collect && N.max_samples > 0 && N.sD == Nk && N.sH == Ni && N.sW == Nj) {
    const int slot = N.next;
    launch(k_rhs_in, grid_for(V), kThreads, c.st, d, (const double*)c.f[CAP_RES], 1.0 / scale, (bf16*)nullptr,
           N.srhs + (size_t)slot * V, V, Ni, Nj);
    launch(k_save_interior, grid_for(V), kThreads, c.st, d, (const double*)c.f[fif], N.fi0, V, Ni, Nj);
    CAP_CHECK_LAUNCH();
    N.pending = slot;
  }
  if (c.precision != 2 || !N.trained) return CAPPGPU_OK;
  // the guess: fi + scale * net(r0 / scale), kept only if it lowers the FP64 residual
  int rc = ensure_act(V);
  if (rc) return rc;
  launch(k_rhs_in, grid_for(V), kThreads, c.st, d, (const double*)c.f[CAP_RES], 1.0 / scale, N.act[0], (bf16*)nullptr,
         V, Ni, Nj);
  CAP_CHECK_LAUNCH();
  if ((rc = forward(Nk, Ni, Nj))) return rc;
  // amplitude by least squares: alpha = (r0.Ad)/(Ad.Ad)
  double* shape = c.work[4];
  double* ashape = c.work[5];
  double* cand = c.work[2];
  double* rcand = c.work[3];
  CAP_CUDA(cudaMemsetAsync(shape, 0, sizeof(double) * d.nijk, c.st));
  launch(k_shape_nat, grid_for(V), kThreads, c.st, d, shape, (const float*)N.out, V, Ni, Nj);
  CAP_CHECK_LAUNCH();
  double dots[2] = {0.0, 0.0};
  if ((rc = spmv_dot2_natural(shape, ashape, c.f[CAP_RES], dots))) return rc;
  if (!(dots[1] > 0.0) || !isfinite(dots[0] / dots[1])) {
    ++N.fallbacks;
    return CAPPGPU_OK;
  }
  const double alpha = dots[0] / dots[1];
  CAP_CUDA(cudaMemcpyAsync(cand, c.f[fif], sizeof(double) * d.nijk, cudaMemcpyDeviceToDevice, c.st));
  launch(k_axpy_nat, grid_for(d.nijk), kThreads, c.st, d.nijk, alpha, (const double*)shape, cand);
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

// At the end of a solve: the correction of a recorded pair
int learned_solve_end(int fif) {
  if (N.pending < 0) return CAPPGPU_OK;
  Ctx& c = ctx();
  const Dims& d = c.d;
  const int Ni = d.nimm - 2, Nj = d.njmm - 2, Nk = d.nkmm - 2;
  const long long V = (long long)Ni * Nj * Nk;
  float* del = N.sdel + (size_t)N.pending * V;
  launch(k_record_delta, kRedBlocks, kThreads, c.st, d, (const double*)c.f[fif], (const double*)N.fi0, del, V, Ni, Nj,
         c.partials);
  CAP_CHECK_LAUNCH();
  int rc = finish_reduce(1);
  if (rc) return rc;
  launch(k_scale_f, grid_for(V), kThreads, c.st, del, V, (const double*)c.redout);   // target: the shape
  CAP_CHECK_LAUNCH();
  N.next = (N.pending + 1) % N.max_samples;
  if (N.nsamples < N.max_samples) ++N.nsamples;
  N.pending = -1;
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
  CAP_CUDA(cudaMalloc(&N.wb, sizeof(bf16) * kLayers * kWConv));
  CAP_CUDA(cudaMalloc(&N.wt, sizeof(bf16) * kLayers * kWConv));
  CAP_CUDA(cudaMalloc(&N.dsum, sizeof(double) * 4));
  CAP_CUDA(cudaMemset(N.gp, 0, sizeof(float) * kParams));
  if (max_samples > 0) {
    if (cudaMalloc(&N.srhs, sizeof(bf16) * (size_t)max_samples * V) != cudaSuccess ||
        cudaMalloc(&N.sdel, sizeof(float) * (size_t)max_samples * V) != cudaSuccess ||
        cudaMalloc(&N.fi0, sizeof(double) * (size_t)V) != cudaSuccess) {
      net_free();
      set_error("learn_reset: out of device memory for %d samples", max_samples);
      return CAPPGPU_E_NOMEM;
    }
  }
  N.max_samples = max_samples;
  N.seed = seed;
  int rc = init_params(seed);
  if (rc) return rc;
  N.ready = true;
  CAP_CUDA(cudaStreamSynchronize(ctx().st));
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
  Ctx& c = ctx();
  const int B = min(block, min(N.sD, min(N.sH, N.sW)));
  const long long V = (long long)B * B * B;
  int rc = ensure_act(V);
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
      launch(k_window, grid_for(V), kThreads, c.st, (const bf16*)(N.srhs + (size_t)sidx * sV),
             (const float*)(N.sdel + (size_t)sidx * sV), N.sD, N.sH, N.sW, z0, y0, x0, B, N.act[0], N.tgt);
      CAP_CHECK_LAUNCH();
      if ((rc = forward(B, B, B))) return rc;
      if ((rc = backward(B, B, B))) return rc;
      if ((rc = adam_step((float)lr))) return rc;
      double h = 0.0;
      CAP_CUDA(cudaMemcpyAsync(&h, N.dsum, sizeof(double), cudaMemcpyDeviceToHost, c.st));
      CAP_CUDA(cudaStreamSynchronize(c.st));
      sum += h / (double)V;
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
    int rc = cast_weights();
    if (rc) return rc;
    N.trained = true;
    CAP_CUDA(cudaStreamSynchronize(ctx().st));
    return kParams;
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

int cappgpu_learn_check(const float* input, const float* target, int D, int H, int W, float* output, float* grad,
                        double* loss) {
  CAP_REQUIRE_INIT();
  if (!N.ready) { set_error("learn_check: call cappgpu_learn_reset first"); return CAPPGPU_E_NOINIT; }
  if (!input || !target || D < 1 || H < 1 || W < 1) { set_error("learn_check: bad arguments"); return CAPPGPU_E_ARG; }
  Ctx& c = ctx();
  const long long V = (long long)D * H * W;
  int rc = ensure_act(V);
  if (rc) return rc;
  std::vector<bf16> in((size_t)V * kC, __float2bfloat16(0.f));
  for (long long v = 0; v < V; ++v) in[v * kC] = __float2bfloat16(input[v]);
  CAP_CUDA(cudaMemcpy(N.act[0], in.data(), sizeof(bf16) * in.size(), cudaMemcpyHostToDevice));
  CAP_CUDA(cudaMemcpy(N.tgt, target, sizeof(float) * V, cudaMemcpyHostToDevice));
  if ((rc = forward(D, H, W))) return rc;
  if ((rc = backward(D, H, W))) return rc;
  CAP_CUDA(cudaStreamSynchronize(c.st));
  if (output) CAP_CUDA(cudaMemcpy(output, N.out, sizeof(float) * V, cudaMemcpyDeviceToHost));
  if (grad) CAP_CUDA(cudaMemcpy(grad, N.gp, sizeof(float) * kParams, cudaMemcpyDeviceToHost));
  if (loss) {
    double h;
    CAP_CUDA(cudaMemcpy(&h, N.dsum, sizeof(double), cudaMemcpyDeviceToHost));
    *loss = h / (double)V;
  }
  return CAPPGPU_OK;
}

}  // extern "C"
