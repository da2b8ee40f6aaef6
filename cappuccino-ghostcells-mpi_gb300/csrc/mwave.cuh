// mwave.cuh -- multi-line persistent wavefront for the FP32 SIP
// substitutions of the refinement form (precision modes 1-2).
//
// The engine of wave.cuh gives every compute thread one line (a, c) and
// releases each hyperplane step through a reduction barrier that a pacing
// warp joins; in FP32 its step costs about 470 cycles, of which the
// arithmetic is a few dozen.  Here a compute thread owns R consecutive
// a-lines of one c-row, so per step it computes R cells of hyperplane s
// that do not depend on one another:
//   cell m = (a0+m, s-a0-m-c, c): its W neighbour (a-1) is the thread's own
//   cell m-1 of the previous step (a register), S (b-1) its own cell m of
//   the previous step, B (c-1) cell m of the thread one row down (four
//   consecutive floats of shared memory, one 16-byte load);
// the inputs of the R cells are consecutive in the TMA-staged boxes (16-byte
// loads).  A block of GA x BC threads covers R*GA x BC lines, so there are
// four times fewer blocks than with one line per thread and fewer block
// hand-overs on the critical path (10 instead of 22 at 128^3).
//
// The compute threads step with a plain barrier; every kMG steps (one TMA
// copy group) a reduction barrier carries the stop decision instead, thread
// 0 refills the slot the group before used, and each thread checks that
// the next copy has landed.  Edge states from predecessor blocks arrive
// through the same mailboxes and communication warp as in wave.cuh
// (value-as-flag entries, staged into shared-memory rings); the threads on
// the block's first column and first row check the staged plane counters
// themselves.  Every wait is bounded by the spin limit and ends in the
// device-wide abort flag and CAPPGPU_E_SPIN; a thread that gives up keeps
// stepping (in bounds, results discarded) to the next group boundary,
// where all threads leave together.
//
// The cell arithmetic and its operand order are those of SipFwdF / SipBwdF
// (wave.cuh), so both engines give the same bits.
#pragma once
#include <cuda.h>

#include "common.cuh"
#include "dlayout.cuh"
#include "wave.cuh"

namespace cap {

#ifndef CAP_MWAVE_G
#define CAP_MWAVE_G 4
#endif
#ifndef CAP_MWAVE_SLOTS
#define CAP_MWAVE_SLOTS 3
#endif
#ifndef CAP_MWAVE_PREFETCH
#define CAP_MWAVE_PREFETCH 4
#endif
constexpr int kMG = CAP_MWAVE_G;              // hyperplanes per TMA copy
constexpr int kMSlots = CAP_MWAVE_SLOTS;      // copies in flight
constexpr int kMPrefetch = CAP_MWAVE_PREFETCH;   // groups between the L2 prefetch of a box and its copy
constexpr int kMR = 4;       // lines per compute thread (along a)
constexpr int kMGA = 8;      // compute threads along a
constexpr int kMBC = 16;     // lines (and compute threads) along c
constexpr int kMBA = kMR * kMGA;   // lines along a per block

template <class Op>
struct MWaveLayout {
  static constexpr int bw = kMBA + 4;   // box columns: the block's lines plus 16 bytes of alignment slack
  __host__ __device__ static constexpr size_t map_bytes(int m) { return (size_t)bw * kMBC * kMG * Op::nq(m) * 4; }
  __host__ __device__ static constexpr size_t map_off(int m) {
    size_t o = 0;
    for (int q = 0; q < m; ++q) o += map_bytes(q);
    return o;
  }
  static constexpr size_t tx_bytes = map_off(Op::kMaps);
  static constexpr size_t slot_bytes = (tx_bytes + 127) / 128 * 128;
  static constexpr size_t in_bytes = kMSlots * slot_bytes;
};

struct MWaveSmem {
  float sbuf[2][kMBC + 1][kMBA + 4];   // the two latest planes; line x of row r at [r+1][4+x]
  float ringW[kRing][kMBC];            // W edge states by plane
  float ringB[kRing][kMBA];            // B edge states by plane
  unsigned long long full[kMSlots];
  unsigned long long stagedW, stagedB; // edge planes <= value-2 are staged
  int done;                            // compute steps < done finished (updated per copy group)
  int blk[2];
  int start_ok;
  int bail;
};

constexpr int mwave_threads() { return kMGA * kMBC + 32; }

template <class Op>
constexpr size_t mwave_smem_bytes() {
  return 128 + MWaveLayout<Op>::in_bytes + sizeof(MWaveSmem);
}

template <class Op, bool BWD>
__global__ void __launch_bounds__(mwave_threads(), 1) k_mwave(const __grid_constant__ Op op, const DG g, const WaveCtl w) {
  using L = MWaveLayout<Op>;
  constexpr int R = kMR, GA = kMGA, BC = kMBC, BA = kMBA;
  constexpr int NC = GA * BC;
  static_assert(NC % 32 == 0 && R == 4, "block shape");
  extern __shared__ unsigned char smem_raw[];
  unsigned char* base = (unsigned char*)(((size_t)smem_raw + 127) & ~(size_t)127);
  unsigned char* inbuf = base;
  MWaveSmem& sm = *reinterpret_cast<MWaveSmem*>(base + L::in_bytes);
  volatile int* bail = &sm.bail;
  const int tid = threadIdx.x;
  if (tid == 0) {
    sm.stagedW = 0;
    sm.stagedB = 0;
    sm.done = 0;
    sm.bail = 0;
    for (int k = 0; k < kMSlots; ++k) mbar_init(&sm.full[k], 1);
    mbar_fence_init();
    const unsigned t = atomicAdd(w.ticket, 1u);
    if (t == (unsigned)w.nblk - 1) atomicExch(w.ticket, 0u);   // every ticket of this launch is taken
    if (t < (unsigned)w.nblk) {
      int2 blk = w.order[t];
      sm.blk[0] = blk.x;
      sm.blk[1] = blk.y;
      sm.start_ok = (w.skip && *(volatile const int*)w.skip) ? 0 : 1;
    } else {   // ticket counter out of step with the host: refuse to run
      sm.blk[0] = sm.blk[1] = 0;
      sm.start_ok = 0;
      atomicExch(w.abort, 1);
      atomicCAS(w.err, 0, 2);
    }
  }
  // zero states before the lines start (the FP32 ghost state is zero)
  for (int q = tid; q < 2 * (BC + 1) * (BA + 4); q += blockDim.x) (&sm.sbuf[0][0][0])[q] = 0.f;
  __syncthreads();
  if (!sm.start_ok) return;
  const int ba = sm.blk[0], bc = sm.blk[1];
  const int s0 = ba * BA + bc * BC;
  const int s1 = min(g.S - 1, s0 + (BA - 1) + (BC - 1) + (g.Nj - 1));
  const int s1W = min(g.S - 1, s0 - 1 + (BC - 1) + (g.Nj - 1));   // last plane of the W / B predecessor lines
  const int s1B = min(g.S - 1, s0 - 1 + (BA - 1) + (g.Nj - 1));
  const int blk_id = bc * w.nBA + ba;
  const int ngroups = (s1 - s0 + kMG) / kMG;
  const int alo = BWD ? g.Ni - (ba + 1) * BA : ba * BA;   // first real column of the block's lines
  const int x0 = alo & ~3;                                 // 16-byte aligned box start (may be negative)

  const int y0 = BWD ? g.Nk - (bc + 1) * BC : bc * BC;
  auto zof = [&](int gq) { const int sg = s0 + gq * kMG; return BWD ? g.S - sg - kMG : sg; };
  auto prefetch = [&](int gq) {   // group gq into L2, kMPrefetch groups before its copy
    if (kMPrefetch <= 0 || gq >= ngroups) return;
    const int z0 = zof(gq);
#pragma unroll
    for (int m = 0; m < Op::kMaps; ++m) {
      if (Op::nq(m) == 1) tma_prefetch3(&op.map[m], x0, y0, z0);
      else tma_prefetch4(&op.map[m], x0, 0, y0, z0);
    }
  };
  auto issue = [&](int gq) {   // TMA copy of group gq (planes s0 + gq*kMG ...) into its slot
    const int slot = gq % kMSlots;
    const int z0 = zof(gq);
    unsigned char* dst = inbuf + slot * L::slot_bytes;
    mbar_arrive_tx(&sm.full[slot], (unsigned)L::tx_bytes);
#pragma unroll
    for (int m = 0; m < Op::kMaps; ++m) {
      if (Op::nq(m) == 1) tma_load3(dst + L::map_off(m), &op.map[m], x0, y0, z0, &sm.full[slot]);
      else tma_load4(dst + L::map_off(m), &op.map[m], x0, 0, y0, z0, &sm.full[slot]);
    }
    prefetch(gq + kMPrefetch);
  };

  if (tid >= NC) {
    // --------------------------------------------- communication warp
    const int lane = tid - NC;
    double* srcW = ba > 0 ? w.mailW + (size_t)(blk_id - 1) * BC * g.Nj : nullptr;
    double* srcB = bc > 0 ? w.mailB + (size_t)(blk_id - w.nBA) * BA * g.Nj : nullptr;
    auto lineW = [&](int e, int& av, int& cv, int& pa, int& pc) {
      av = ba * BA; cv = bc * BC + e; pa = av - 1; pc = cv;
    };
    auto lineB = [&](int e, int& av, int& cv, int& pa, int& pc) {
      av = ba * BA + e; cv = bc * BC; pa = av; pc = cv - 1;
    };
    EdgeProbe<float, Op::kPW * BC / 32> PW;
    EdgeProbe<float, Op::kPW * BA / 32> PB;
    int loadedW = s0 - 2, loadedB = s0 - 2;   // last staged plane
    long long idle = 0;
    while (loadedW < s1W || loadedB < s1B) {
      if (__any_sync(0xffffffffu, *bail)) break;
      const int cur = __shfl_sync(0xffffffffu, *(volatile int*)&sm.done, 0);
      const int limit = max(cur, s0) + kRing - 2;   // ring capacity
      const int hiW = min(s1W, limit), hiB = min(s1B, limit);
      probe_edge<Op, BC, BWD>(PW, op, g, lane, loadedW, hiW, srcW, lineW, make_int2(0, g.Ni), g.Ni);
      probe_edge<Op, BA, BWD>(PB, op, g, lane, loadedB, hiB, srcB, lineB, make_int2(0, g.Ni), g.Ni);
      const int nW = commit_edge<float, BC, Op::kPW>(PW, g, lane, loadedW, srcW, sm.ringW, lineW);
      const int nB = commit_edge<float, BA, Op::kPW>(PB, g, lane, loadedB, srcB, sm.ringB, lineB);
      if (nW + nB > 0) {
        __syncwarp();
        if (lane == 0) {
          if (nW) st_release_cta_shared(&sm.stagedW, (unsigned long long)(unsigned)(loadedW + nW + 2));
          if (nB) st_release_cta_shared(&sm.stagedB, (unsigned long long)(unsigned)(loadedB + nB + 2));
        }
        free_edge<float, BC, Op::kPW>(PW, g, lane, loadedW, nW, srcW, lineW);
        free_edge<float, BA, Op::kPW>(PB, g, lane, loadedB, nB, srcB, lineB);
        loadedW += nW;
        loadedB += nB;
        idle = 0;
      } else {
        int stop = 0;
        if (lane == 0) {
          if (++idle > w.spin_limit) { wave_fail(w, bail, 1); stop = 1; }
          else if ((idle & 31) == 31 && ld_relaxed_i32(w.abort)) { *bail = 1; stop = 1; }
        }
        if (__shfl_sync(0xffffffffu, stop, 0)) break;
      }
    }
    return;
  }

  // ------------------------------------------------------ compute threads
  const int gt = tid % GA, cl = tid / GA;
  const int av0 = ba * BA + gt * R;            // virtual (mirrored when BWD) a of cell m = 0
  const int cv = bc * BC + cl;
  const int c = BWD ? g.Nk - 1 - cv : cv;
  const bool row_ok = cv < g.Nk;
  // box coordinates: row, and the column of cell m (forward: xb + m; mirrored: xb - m)
  const int yb = BWD ? BC - 1 - cl : cl;
  const int xb = BWD ? (alo - x0) + BA - 1 - gt * R : gt * R;
  const bool vec_in = !BWD || ((xb - (R - 1)) & 3) == 0;   // the R inputs form one aligned 16-byte row
  const bool edgeE = gt == GA - 1 && ba + 1 < w.nBA;   // feeds the next block along a
  const bool edgeT = cl == BC - 1 && bc + 1 < w.nBC;   // feeds the next block along c
  double* const mW = w.mailW + ((size_t)blk_id * BC + cl) * g.Nj;
  double* const mB = w.mailB + ((size_t)blk_id * BA + gt * R) * g.Nj;
  // W of cell 0 and B of the R cells, for the two buffer parities
  const float* const rdW = gt > 0 ? &sm.sbuf[0][cl + 1][4 + gt * R - 1] : nullptr;
  const float* const rdB = cl > 0 ? &sm.sbuf[0][cl][4 + gt * R] : nullptr;
  float* const wr = &sm.sbuf[0][cl + 1][4 + gt * R];
  constexpr int kPar = (BC + 1) * (BA + 4);   // floats between the two buffers
  long long di[R];                            // hyperplane-layout index of cell m at plane s0 (sr for BWD)
  bool line_ok[R];
#pragma unroll
  for (int m = 0; m < R; ++m) {
    const int av = av0 + m;
    line_ok[m] = row_ok && av < g.Ni;
    const int a = BWD ? g.Ni - 1 - av : av;
    const int sr = BWD ? g.S - 1 - s0 : s0;
    di[m] = (long long)sr * g.plane + (long long)c * g.P + a;
  }
  const long long dstep = BWD ? -g.plane : g.plane;
  float prev[R];
#pragma unroll
  for (int m = 0; m < R; ++m) prev[m] = 0.f;
  unsigned long long knownW = 0, knownB = 0;
  bool gave_up = false;

  if (tid == 0) {
    for (int gq = kMSlots; gq < kMSlots + kMPrefetch; ++gq) prefetch(gq);
    for (int gq = 0; gq < min(kMSlots, ngroups); ++gq) issue(gq);
  }
  int issued = min(kMSlots, ngroups);

  int ds = 0, gi = 0;
  for (int s = s0; s <= s1; ++s) {
    if (ds == 0) {
      if (named_bar_red_or(1, NC, gave_up)) break;   // plane s-1 done; everyone leaves together
      if (tid == 0 && gi > 0) {
        *(volatile int*)&sm.done = s;
        const int gq = gi - 1 + kMSlots;   // the slot of the previous group is free
        if (gq < ngroups) {
          fence_proxy_async_smem();
          issue(gq);
          issued = gq + 1;
        }
      }
      long long it = 0;   // this group's copy has landed
      while (!gave_up && !mbar_test(&sm.full[gi % kMSlots], (unsigned)((gi / kMSlots) & 1))) {
        if (++it > 64LL * w.spin_limit) { wave_fail(w, bail, 1); gave_up = true; }
        else if ((it & 1023) == 0 && (*bail || ld_relaxed_i32(w.abort))) gave_up = true;
      }
    } else {
      named_bar_sync(1, NC);   // plane s-1 done
    }
    // edge states of plane s-1 staged (first column / first row only)
    if (gt == 0) {
      const unsigned long long need = (unsigned long long)(unsigned)(min(s, s1W + 1) + 1);
      long long it = 0;
      while (!gave_up && knownW < need) {
        knownW = ld_acquire_cta_shared(&sm.stagedW);
        if (knownW >= need) break;
        if (++it > 64LL * w.spin_limit) { wave_fail(w, bail, 1); gave_up = true; }
        else if ((it & 1023) == 0 && (*bail || ld_relaxed_i32(w.abort))) gave_up = true;
      }
    }
    if (cl == 0) {
      const unsigned long long need = (unsigned long long)(unsigned)(min(s, s1B + 1) + 1);
      long long it = 0;
      while (!gave_up && knownB < need) {
        knownB = ld_acquire_cta_shared(&sm.stagedB);
        if (knownB >= need) break;
        if (++it > 64LL * w.spin_limit) { wave_fail(w, bail, 1); gave_up = true; }
        else if ((it & 1023) == 0 && (*bail || ld_relaxed_i32(w.abort))) gave_up = true;
      }
    }
    const int par = ((s & 1) ^ 1) * kPar;   // buffer of plane s-1
    const int rs = ring_slot(s - 1);
    const float W0 = gt > 0 ? rdW[par] : sm.ringW[rs][cl];
    const float4 B4 = *reinterpret_cast<const float4*>(cl > 0 ? rdB + par : &sm.ringB[rs][gt * R]);
    const float B[R] = {B4.x, B4.y, B4.z, B4.w};
    // inputs of the R cells: map m, component q
    const float* slot = reinterpret_cast<const float*>(inbuf + (gi % kMSlots) * L::slot_bytes);
    const int zb = BWD ? kMG - 1 - ds : ds;
    float in[Op::kMaps][4][R];
#pragma unroll
    for (int m = 0; m < Op::kMaps; ++m) {
#pragma unroll
      for (int q = 0; q < Op::nq(m); ++q) {
        const float* row = slot + L::map_off(m) / 4 + ((size_t)(zb * BC + yb) * Op::nq(m) + q) * L::bw;
        if (vec_in) {
          const float4 v = *reinterpret_cast<const float4*>(row + (BWD ? xb - (R - 1) : xb));
          if (BWD) { in[m][q][0] = v.w; in[m][q][1] = v.z; in[m][q][2] = v.y; in[m][q][3] = v.x; }
          else { in[m][q][0] = v.x; in[m][q][1] = v.y; in[m][q][2] = v.z; in[m][q][3] = v.w; }
        } else {
#pragma unroll
          for (int k = 0; k < R; ++k) in[m][q][k] = row[BWD ? xb - k : xb + k];
        }
      }
    }
    float v[R];
#pragma unroll
    for (int m = 0; m < R; ++m) v[m] = Op::cell(in, m, m == 0 ? W0 : prev[m - 1], prev[m], B[m]);
    const int b0 = s - av0 - cv;   // b of cell 0; cell m has b0 - m
#pragma unroll
    for (int m = 0; m < R; ++m) {
      const bool ok = line_ok[m] && (unsigned)(b0 - m) < (unsigned)g.Nj;
      if (ok) op.z[di[m]] = v[m];
      else v[m] = prev[m];   // zero before the line starts (the ghost state), unused after it ends
      di[m] += dstep;
    }
    *reinterpret_cast<float4*>(wr + (s & 1) * kPar) = make_float4(v[0], v[1], v[2], v[3]);
    if (edgeE && line_ok[R - 1] && (unsigned)(b0 - (R - 1)) < (unsigned)g.Nj)
      st_relaxed_b64(mW + (b0 - (R - 1)), (unsigned long long)__float_as_uint(v[R - 1]));
    if (edgeT) {
#pragma unroll
      for (int m = 0; m < R; ++m)
        if (line_ok[m] && (unsigned)(b0 - m) < (unsigned)g.Nj)
          st_relaxed_b64(mB + (size_t)m * g.Nj + (b0 - m), (unsigned long long)__float_as_uint(v[m]));
    }
#pragma unroll
    for (int m = 0; m < R; ++m) prev[m] = v[m];
    if (++ds == kMG) { ds = 0; ++gi; }
  }
  if (gave_up) *bail = 1;
  // the copies in flight land before the block exits
  // (the last use of each slot; a completed phase tests complete again)
  if (tid == 0) {
    for (int gq = max(0, issued - kMSlots); gq < issued; ++gq) {
      long long it = 0;
      while (!mbar_test(&sm.full[gq % kMSlots], (unsigned)((gq / kMSlots) & 1))) {
        if (++it > kDrainPolls) { wave_fail(w, bail, 1); break; }
      }
    }
  }
}

// ------------------------------------------------------------------ ops
// The FP32 substitutions of SipFwdF / SipBwdF (wave.cuh) on the R cells of
// a thread: in[m][q][k] is component q of map m at cell k.

struct MSipFwdF {
  using St = float;
  static constexpr int kMaps = 2;   // r, forward factors (bb, bw, bs, bp)
  static constexpr int kPW = 8;     // edge planes polled per communication pass
  __host__ __device__ static constexpr int nq(int m) { return m == 0 ? 1 : 4; }
  CUtensorMap map[kMaps];
  float* z;
  __device__ St ghost(int) const { return 0.0f; }
  template <class In>
  __device__ static float cell(const In& in, int k, float W, float S, float B) {
    return (in[0][0][k] - in[1][0][k] * B - in[1][1][k] * W - in[1][2][k] * S) * in[1][3][k];
  }
};

struct MSipBwdF {
  using St = float;
  static constexpr int kMaps = 2;   // z, backward factors (bn, be, bt)
  static constexpr int kPW = 8;
  __host__ __device__ static constexpr int nq(int m) { return m == 1 ? 3 : 1; }
  CUtensorMap map[kMaps];
  float* z;
  __device__ St ghost(int) const { return 0.0f; }
  template <class In>
  __device__ static float cell(const In& in, int k, float W, float S, float B) {
    return in[0][0][k] - in[1][0][k] * S - in[1][1][k] * W - in[1][2][k] * B;
  }
};

}  // namespace cap
