// common.cuh -- shared device/host definitions of the GB300 library.
//
// Storage: every module array of the reference is a device double array of
// nijk elements; element ijk-1 holds the reference's element ijk with
// ijk = lk(k)+li(i)+j (setind.f90:34-40), i.e. j fastest, then i, then k.
// Kernels iterate the reference's loop boxes with 1-based i,j,k.
//
// Floating point: the library is compiled with --fmad=false so that every
// a*b+c is a rounded multiply followed by a rounded add, the arithmetic of
// the reference (gfortran -O2, x86-64, no FMA).  Division and sqrt of
// doubles are IEEE round-to-nearest on both sides.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include "../../include/cappgpu.h"

namespace cap {

// modules_allocatable.f90:39 -- small is a default-real (single precision)
// literal stored in a real(dp) parameter.
#define CAP_SMALL ((double)1e-30f)

struct Dims {
  int ni, nj, nk, nim, njm, nkm, nimm, njmm, nkmm, nij, nik, njk, nijk;
};

// 0-based storage index of the reference's ijk
__host__ __device__ inline int ixk(const Dims& d, int i, int j, int k) {
  return (k - 1) * d.nij + (i - 1) * d.nj + (j - 1);
}

// An inclusive loop box of the reference, iterated j fastest.
struct Box {
  int i0, i1, j0, j1, k0, k1;
  __host__ __device__ long long count() const {
    if (i1 < i0 || j1 < j0 || k1 < k0) return 0;
    return (long long)(i1 - i0 + 1) * (j1 - j0 + 1) * (k1 - k0 + 1);
  }
  __host__ __device__ void at(long long t, int& i, int& j, int& k) const {
    int nj_ = j1 - j0 + 1, ni_ = i1 - i0 + 1;
    j = j0 + (int)(t % nj_);
    long long r = t / nj_;
    i = i0 + (int)(r % ni_);
    k = k0 + (int)(r / ni_);
  }
};

constexpr int kThreads = 256;
// Reductions use a fixed grid so that per-block partials are summed in a
// fixed order (deterministic results, run to run).
constexpr int kRedBlocks = 608;   // 152 SMs x 4
constexpr int kMaxRed = 4;        // values reduced by one kernel

// Polls of the exit wait for the block's own TMA copies in flight.  A copy
// from valid memory always lands, so this bound is independent of the
// spin limit on predecessors (which a caller may set very low): the block
// never leaves while a copy into its shared memory is still running.
constexpr long long kDrainPolls = 1LL << 27;

constexpr int kStageSlots = 8;   // staging arrays for unregistered host-pointer arguments

struct Ctx {
  bool init = false;
  Dims d{};
  // fields, then kStageSlots staging arrays of the host-pointer entry points
  // (allocated on first use; ids CAP_NFIELDS + k)
  double* f[CAP_NFIELDS + kStageSlots] = {};
  int* bc[CAP_NBC] = {};
  int* li = nullptr;   // device li[1..ni]
  int* lk = nullptr;   // device lk[1..nk]
  cappgpu_params prm{};
  cudaStream_t st = nullptr;
  double* partials = nullptr;   // kMaxRed * kRedBlocks
  double* redout = nullptr;     // kMaxRed results (device)
  double* hred = nullptr;       // pinned host mirror of redout
  double* dscal = nullptr;      // device scalars shared by kernels (16)
  double* work[8] = {};         // solver work vectors (nijk each)
  int* wf_flags = nullptr;      // wavefront tile flags / counters
  double* host_reg[CAP_NFIELDS] = {};  // registered host arrays
  double* host_vec3[CAP_NFIELDS] = {}; // registered interleaved (3, nijk) host arrays, by x-component field
  double* vec3buf = nullptr;           // device staging of one interleaved array (3 nijk doubles)
  cappgpu_solve_report last_rep{};     // the last linear solve: report, solver and ifi
  int last_solver = 0, last_ifi = 0;
  // instrumentation (cappgpu_get_stats)
  unsigned long long launches = 0;     // kernels launched since init
  double p_solve_ms = 0.0;             // last PISO/SIMPLE pressure solve
  cappgpu_solve_report p_rep{};        // its report
  cudaEvent_t ev[4] = {};
  // option sweep_timing: CUDA events around the FP64 pcgsip forward sweeps
  // (one pair per iteration of a batch), their durations summed at the
  // batch's host read (cappgpu_sweep_stats)
  int sweep_timing = 0;
  cudaEvent_t sw_ev[2 * 64] = {};
  double sw_ms = 0.0;
  long long sw_n = 0;
  int wave_impl = 1;                   // 1 persistent wavefront, 0 one launch per hyperplane
  int fused_dot = 1;                   // FP32 CG (wavefront 0): sk = r.z in the backward substitution
  int lane_wave = 0;                   // FP32 substitutions: 0 the wavefront of wave.cuh, 1 the warp-tile engine
  int sip_slabs = 4096;                // FP32 SIP of the refinement form (wavefront 0): block-local per slab
                                       // (as the reference's SIP per MPI rank), at most this many slabs
  int sip_slab_axis = 0;               // the slabs' axis: 0 = i, 1 = k
  int face_geo = 1;                    // 1: FP64 face kernels read the per-face geometry cache
  int tight_correctors = 0;            // 1: every PISO corrector solves p to reltol, not only the last
  int cg_batch = 4;                    // CG iterations launched between two host reads of the exit test
  int inner_drop = 4;                  // FP32 inner CG stops at 10^-inner_drop of the outer residual
  long long spin_limit = 1LL << 21;    // polls of a wavefront wait on a predecessor before CAPPGPU_E_SPIN
  int device = 0;                      // CUDA device ordinal current at cappgpu_init
  int fp32_parts = 11;                 // parts in FP32 in precision modes 1-2: 1 p solve, 2 sipsol,
                                       // 4 momentum assembly (fluxuvw, LES viscosity), 8 velocity
                                       // gradients, 16 pressure-equation assembly
  bool fp32(int part) const { return precision >= 1 && (fp32_parts & part) != 0; }
  int precision = 0;                   // pcgsip: 0 FP64 plain, 1 FP32 preconditioned CG in FP64 refinement
  unsigned long long geo_gen = 1;      // bumped whenever a grid-geometry field may have changed
};

Ctx& ctx();
void set_error(const char* fmt, ...);
// record a write into field q: a write into a grid-geometry field (nodes,
// centres, face areas, interpolation factors) invalidates the per-face
// geometry derived from it
void note_write(int q);
bool spmv_output_ok(int q);
int cuda_fail(cudaError_t e, const char* what, const char* file, int line);

#define CAP_CUDA(call)                                                     \
  do {                                                                     \
    cudaError_t e_ = (call);                                               \
    if (e_ != cudaSuccess) return cap::cuda_fail(e_, #call, __FILE__, __LINE__); \
  } while (0)

#define CAP_CHECK_LAUNCH()                                                 \
  do {                                                                     \
    cudaError_t e_ = cudaGetLastError();                                   \
    if (e_ != cudaSuccess) return cap::cuda_fail(e_, "kernel launch", __FILE__, __LINE__); \
  } while (0)

#define CAP_REQUIRE_INIT()                                                 \
  do {                                                                     \
    if (!cap::ctx().init) { cap::set_error("cappgpu_init not called"); return CAPPGPU_E_NOINIT; } \
  } while (0)

// Every kernel launch of the library goes through launch(), which counts it
// (cappgpu_get_stats reports the count).
template <typename... KArgs, typename... Args>
inline void launch(void (*k)(KArgs...), int grid, int block, cudaStream_t s, Args... args) {
  ++ctx().launches;
  k<<<grid, block, 0, s>>>(args...);
}

// launch() with a 2-D or 3-D grid
template <typename... KArgs, typename... Args>
inline void launch(void (*k)(KArgs...), dim3 grid, int block, cudaStream_t s, Args... args) {
  ++ctx().launches;
  k<<<grid, block, 0, s>>>(args...);
}

// launch() with dynamic shared memory
template <typename... KArgs, typename... Args>
inline void launch_smem(void (*k)(KArgs...), int grid, int block, size_t smem, cudaStream_t s, Args... args) {
  ++ctx().launches;
  k<<<grid, block, smem, s>>>(args...);
}

inline int grid_for(long long n, int threads = kThreads) {
  long long b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > 152 * 32) b = 152 * 32;
  return (int)b;
}

// Deterministic reductions --------------------------------------------------
// Block-level sum of NV values; thread 0 of each block writes its partials
// to part[v*kRedBlocks + blockIdx.x].
template <int NV>
__device__ inline void block_reduce_store(double (&v)[NV], double* part) {
  __shared__ double sh[NV][kThreads / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < NV; ++q) {
    double x = v[q];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) sh[q][wid] = x;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int q = 0; q < NV; ++q) {
      double s = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += sh[q][w];
      part[q * kRedBlocks + blockIdx.x] = s;
    }
  }
}

// Block-level max of one non-negative value.
__device__ inline void block_max_store(double v, double* part) {
  __shared__ double sh[kThreads / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = sh[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) s = fmax(s, sh[w]);
    part[blockIdx.x] = s;
  }
}

// Final combine (one block): out[v] = sum (or max) of the partial slots
// first..first+nv-1 in block order.
int finish_reduce(int nv, bool is_max = false, int first = 0);
// Copy the reduced values to the host (synchronises the stream).
int fetch_reduce(int nv, double* out);

}  // namespace cap
