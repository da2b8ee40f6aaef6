// lanewave.cuh -- warp-synchronous hyperplane wavefront for the FP32 SIP
// substitutions of the refinement form.
//
// The persistent wavefront of wave.cuh gives every line (a,c) its own
// thread and closes each hyperplane step with a CTA barrier; in FP32 the
// arithmetic of a step is a few instructions, and the barrier, the
// shared-memory hand-over and the pacing warp's release set the step time
// (0.44 us per hyperplane at 128^3).  Here one warp owns a tile of 32
// a-lines x kCW c-lines and walks j.  Lane L holds the tile's kCW cells
// (a0+L, b, c0+m), m = 0..kCW-1, with b = tau - L - m at local step tau: all
// of them lie on hyperplane a0+c0+tau, and each predecessor was computed at
// step tau-1 --
//   (a, b-1, c):  the same lane, the same m       (a register)
//   (a, b, c-1):  the same lane, m-1              (a register)
//   (a-1, b, c):  lane L-1, the same m            (a warp shuffle)
// so a step needs no barrier at all.  Lane 0's a-predecessors and the m = 0
// c-predecessors come from the neighbouring tiles through global mailboxes
// whose data is its own flag (a signalling-NaN sentinel that no arithmetic
// result equals): the producer tile stores the value; a second warp of the
// consumer's CTA polls the mailboxes, stages the values into a
// shared-memory ring, puts the sentinel back for the next launch and
// publishes how many steps are staged.  The compute warp reads only shared
// memory: its per-step inputs arrive by TMA, kLG hyperplanes per copy,
// kLSlots copies in flight, and it checks the staged count before a step
// only when its last reading does not cover that step.
//
// The per-cell expressions are those of SipFwdF / SipBwdF (wave.cuh) with
// the same operand order, so both engines give the same bits.  Backward
// sweeps run in mirrored coordinates (virtual a = Ni-1-a etc.).
//
// Measured on GB300 (one forward sweep, FP32): 58-68 us on a single tile of
// 32 x 124 x 8 cells (0.36-0.42 us per step: the compute warp issues about
// 160 instructions per step at 4 cycles each, mostly fixed-latency
// dependency waits a lone warp cannot hide), 192 us at 124^3 and 439 us at
// 252^3, against 152 and 443 us for the wavefront of wave.cuh.  Tiles hand
// over with a lag of about 13 steps along c and 42 along a (the skew of 31
// lanes).  It is therefore an option (lane_wave), not the default.
//
// Tiles are taken by ticket in topological (diagonal) order, so a tile only
// waits on tiles started before it.  Every wait is bounded: on timeout the
// kernel raises the device-wide abort flag and error code 1, every warp
// leaves its loop, waits (bounded) for its copies in flight and returns.
#pragma once
#include <cuda.h>

#include "common.cuh"
#include "dlayout.cuh"

namespace cap {

constexpr int kLW = 32;        // a-lines per tile (one per lane)
constexpr int kCW = 8;         // c-lines per tile (per lane)
constexpr int kLG = 8;         // hyperplanes per TMA copy = edge prefetch distance
constexpr int kLSlots = 4;     // copies in flight
constexpr int kLR = 32;        // steps of staged edge values (a power of two)
constexpr int kLC = 2;         // steps staged per polling pass
constexpr unsigned kSentinelF = 0x7F80DEADu;   // signalling NaN (FP32)
static_assert(kLR >= kLG + kLC && (kLR & (kLR - 1)) == 0, "edge ring");

struct LaneCtl {
  unsigned* ticket;      // 0 between launches (the last tile to take one resets it)
  const int2* order;     // tiles (A, C) in topological order
  int nA, nC, ntile;
  int nt;                // local steps of a tile = mailbox rows per tile
  int* abort;
  int* err;
  float* mailW;          // per tile: nt x kCW values of its last a-line
  float* mailB;          // per tile: nt x kLW values of its last c-line
  long long spin_limit;
  const int* skip;       // when non-null and *skip != 0 at launch, every tile exits at once
};

// Relaxed gpu-scope accesses of the mailboxes.  The value is its own flag,
// so no other access has to be ordered around them and they carry no
// compiler barrier.
__device__ __forceinline__ unsigned ld_relaxed_u32(const float* p) {
  unsigned v;
  asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p));
  return v;
}
__device__ __forceinline__ void st_relaxed_u32(float* p, unsigned v) {
  asm volatile("st.relaxed.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v));
}
// predicated forms (no branch around the store)
__device__ __forceinline__ void st_relaxed_f32_if(float* p, float v, bool pred) {
  asm volatile("{\n .reg .pred q;\n setp.ne.u32 q, %2, 0;\n @q st.relaxed.gpu.global.b32 [%0], %1;\n}" ::"l"(p),
               "r"(__float_as_uint(v)), "r"((unsigned)pred));
}
__device__ __forceinline__ void st_relaxed_v4_if(float* p, float a, float b, float c, float d, bool pred) {
  asm volatile("{\n .reg .pred q;\n setp.ne.u32 q, %5, 0;\n @q st.relaxed.gpu.global.v4.b32 [%0], {%1, %2, %3, %4};\n}" ::"l"(p),
               "r"(__float_as_uint(a)), "r"(__float_as_uint(b)), "r"(__float_as_uint(c)), "r"(__float_as_uint(d)),
               "r"((unsigned)pred));
}

__device__ __forceinline__ void st_release_cta_shared_i32(int* p, int v) {
  asm volatile("st.release.cta.shared.b32 [%0], %1;" ::"r"(smem_u32(p)), "r"(v) : "memory");
}
__device__ __forceinline__ int ld_acquire_cta_shared_i32(const int* p) {
  int v;
  asm volatile("ld.acquire.cta.shared.b32 %0, [%1];" : "=r"(v) : "r"(smem_u32(p)) : "memory");
  return v;
}

__device__ __forceinline__ void st_global_f32_if(float* p, float v, bool pred) {
  asm volatile("{\n .reg .pred q;\n setp.ne.u32 q, %2, 0;\n @q st.global.f32 [%0], %1;\n}" ::"l"(p), "f"(v),
               "r"((unsigned)pred));
}

struct LaneSmem {
  float ringW[kLR][kCW];          // W edge values by step (read by lane 31)
  float ringB[kLR][kLW];          // B edge values by step
  unsigned long long staged;      // edge values of steps < staged are in the rings
  unsigned long long full[kLSlots];
  int done;                       // compute steps < done finished (updated per copy group)
  int bail;                       // a warp gave up
};

// Shared memory per slot: for each map a box of (kLW + 4) x nq x kCW x kLG
// floats (the four extra columns let a mirrored tile start its copy on a
// 16-byte aligned column).
template <class Op>
struct LaneLayout {
  static constexpr int bw = kLW + 4;
  __host__ __device__ static constexpr size_t map_bytes(int m) { return (size_t)bw * Op::nq(m) * kCW * kLG * 4; }
  __host__ __device__ static constexpr size_t map_off(int m) {
    size_t o = 0;
    for (int q = 0; q < m; ++q) o += map_bytes(q);
    return o;
  }
  static constexpr size_t tx_bytes = map_off(Op::kMaps);
  static constexpr size_t slot_bytes = (tx_bytes + 127) / 128 * 128;
  static constexpr size_t smem = 128 + kLSlots * slot_bytes + sizeof(LaneSmem);
};

// z = (r - bb zB - bw zW - bs zS) bp   (pcg-sip.f90:102-103; SipFwdF)
struct LaneFwdF {
  static constexpr int kMaps = 2;   // r, forward factors (bb, bw, bs, bp)
  __host__ __device__ static constexpr int nq(int m) { return m == 0 ? 1 : 4; }
  CUtensorMap map[kMaps];
  float* z;
  template <class In>
  __device__ __forceinline__ float compute(const In& in, float W, float S, float B) const {
    return (in(0, 0) - in(1, 0) * B - in(1, 1) * W - in(1, 2) * S) * in(1, 3);
  }
};

// z = z - bn zN - be zE - bt zT   (pcg-sip.f90:116-117; SipBwdF), the
// engine's S, W, B being the j+1, i+1, k+1 cells
struct LaneBwdF {
  static constexpr int kMaps = 2;   // z, backward factors (bn, be, bt)
  __host__ __device__ static constexpr int nq(int m) { return m == 1 ? 3 : 1; }
  CUtensorMap map[kMaps];
  float* z;
  template <class In>
  __device__ __forceinline__ float compute(const In& in, float W, float S, float B) const {
    return in(0, 0) - in(1, 0) * S - in(1, 1) * W - in(1, 2) * B;
  }
};

template <class Op, bool BWD>
__global__ void __launch_bounds__(64, 1) k_lane_wave(const __grid_constant__ Op op, const DG g, const LaneCtl w) {
  using L = LaneLayout<Op>;
  extern __shared__ unsigned char smem_raw[];
  unsigned char* base = (unsigned char*)(((size_t)smem_raw + 127) & ~(size_t)127);
  LaneSmem& sm = *reinterpret_cast<LaneSmem*>(base + kLSlots * L::slot_bytes);
  volatile int* bail = &sm.bail;
  const int tid = threadIdx.x, lane = tid & 31;
  const unsigned FULL = 0xffffffffu;
  __shared__ int tile_sh[3];
  if (tid == 0) {
    for (int k = 0; k < kLSlots; ++k) mbar_init(&sm.full[k], 1);
    mbar_fence_init();
    sm.staged = 0;
    sm.done = 0;
    sm.bail = 0;
    const unsigned t = atomicAdd(w.ticket, 1u);
    if (t == (unsigned)w.ntile - 1) atomicExch(w.ticket, 0u);   // every ticket of this launch is taken
    int start = 1;
    if (t >= (unsigned)w.ntile) {   // ticket counter out of step with the host: refuse to run
      atomicExch(w.abort, 1);
      atomicCAS(w.err, 0, 2);
      start = 0;
    } else if (w.skip && *(volatile const int*)w.skip) {
      start = 0;
    }
    const int2 tl = start ? w.order[t] : make_int2(0, 0);
    tile_sh[0] = start;
    tile_sh[1] = tl.x;
    tile_sh[2] = tl.y;
  }
  __syncthreads();
  if (!tile_sh[0]) return;
  const int A = tile_sh[1], C = tile_sh[2];
  const int a0v = A * kLW, c0v = C * kCW;
  const int nt = w.nt;
  const bool hasW = A > 0, hasB = C > 0;                  // edge inputs from neighbour tiles
  const int av = a0v + lane;
  const bool a_ok = av < g.Ni;

  if (tid >= 32) {
    // ------------------------------------------------ staging warp
    // step tau needs W entry (tau + kLW - 1, m) of tile (A-1, C) for lane 0's
    // cell m, and B entry (tau + kCW - 1, L) of tile (A, C-1) for lane L's
    // cell m = 0; an entry exists where that cell does.
    const float* mWin = hasW ? w.mailW + (size_t)(C * w.nA + A - 1) * nt * kCW : nullptr;
    const float* mBin = hasB ? w.mailB + (size_t)((C - 1) * w.nA + A) * nt * kLW : nullptr;
    const bool rowW = hasW && lane < kCW && c0v + lane < g.Nk;
    int st = 0;
    long long idle = 0;
    while (st < nt) {
      const int done = ld_acquire_cta_shared_i32(&sm.done);
      const int n = min(kLC, min(nt, done + kLR - kLC) - st);   // ring capacity
      if (n <= 0) {
        __nanosleep(64);   // leave the issue slots to the compute warp
        int stop = 0;
        if (lane == 0) {
          if (++idle > w.spin_limit) {
            atomicExch(w.abort, 1);
            atomicCAS(w.err, 0, 1);
            *bail = 1;
            stop = 1;
          } else if (*bail || ((idle & 255) == 0 && ld_relaxed_i32(w.abort))) {
            *bail = 1;
            stop = 1;
          }
        }
        if (__shfl_sync(FULL, stop, 0)) break;
        continue;
      }
      idle = 0;
      unsigned vB[kLC], vW[kLC];
      bool nB[kLC], nW[kLC];
#pragma unroll
      for (int j = 0; j < kLC; ++j) {
        const int tau = st + j, bv = tau - lane;
        nB[j] = j < n && hasB && a_ok && bv >= 0 && bv < g.Nj;
        nW[j] = j < n && rowW && bv >= 0 && bv < g.Nj;
        vB[j] = nB[j] ? ld_relaxed_u32(mBin + (size_t)(tau + kCW - 1) * kLW + lane) : 0u;
        vW[j] = nW[j] ? ld_relaxed_u32(mWin + (size_t)(tau + kLW - 1) * kCW + lane) : 0u;
      }
      bool stop = false;
#pragma unroll
      for (int j = 0; j < kLC; ++j) {
        const int tau = st + j;
        long long it = 0;
        while (nB[j] && vB[j] == kSentinelF) {
          if (++it > w.spin_limit) { atomicExch(w.abort, 1); atomicCAS(w.err, 0, 1); stop = true; break; }
          if ((it & 255) == 0 && (*bail || ld_relaxed_i32(w.abort))) { stop = true; break; }
          __nanosleep(32);
          vB[j] = ld_relaxed_u32(mBin + (size_t)(tau + kCW - 1) * kLW + lane);
        }
        it = 0;
        while (!stop && nW[j] && vW[j] == kSentinelF) {
          if (++it > w.spin_limit) { atomicExch(w.abort, 1); atomicCAS(w.err, 0, 1); stop = true; break; }
          if ((it & 255) == 0 && (*bail || ld_relaxed_i32(w.abort))) { stop = true; break; }
          __nanosleep(32);
          vW[j] = ld_relaxed_u32(mWin + (size_t)(tau + kLW - 1) * kCW + lane);
        }
      }
      if (__any_sync(FULL, stop)) { *bail = 1; break; }
#pragma unroll
      for (int j = 0; j < kLC; ++j) {
        const int tau = st + j, rs = tau & (kLR - 1);
        if (j < n) {
          sm.ringB[rs][lane] = __uint_as_float(vB[j]);
          if (lane < kCW) sm.ringW[rs][lane] = __uint_as_float(vW[j]);
        }
      }
      __syncwarp();
      if (lane == 0) st_release_cta_shared(&sm.staged, (unsigned long long)(st + n));
      // the consumed entries get the sentinel back, ready for the next launch
#pragma unroll
      for (int j = 0; j < kLC; ++j) {
        const int tau = st + j;
        if (nB[j]) st_relaxed_u32(const_cast<float*>(mBin) + (size_t)(tau + kCW - 1) * kLW + lane, kSentinelF);
        if (nW[j]) st_relaxed_u32(const_cast<float*>(mWin) + (size_t)(tau + kLW - 1) * kCW + lane, kSentinelF);
      }
      st += n;
    }
    return;
  }

  // ------------------------------------------------------ compute warp
  const int sv0 = a0v + c0v;                 // virtual hyperplane of local step 0
  const int ngroups = (nt + kLG - 1) / kLG;
  const int alo = BWD ? g.Ni - a0v - kLW : a0v;   // first real column of the tile
  const int x0 = alo & ~3;                         // 16-byte aligned start
  auto issue = [&](int gq) {   // TMA copy of group gq (virtual planes sv0 + gq*kLG ...)
    const int slot = gq % kLSlots, svg = sv0 + gq * kLG;
    const int y0 = BWD ? g.Nk - c0v - kCW : c0v;
    const int z0 = BWD ? g.S - svg - kLG : svg;
    unsigned char* dst = base + slot * L::slot_bytes;
    mbar_arrive_tx(&sm.full[slot], (unsigned)L::tx_bytes);
#pragma unroll
    for (int m = 0; m < Op::kMaps; ++m) {
      if (Op::nq(m) == 1) tma_load3(dst + L::map_off(m), &op.map[m], x0, y0, z0, &sm.full[slot]);
      else tma_load4(dst + L::map_off(m), &op.map[m], x0, 0, y0, z0, &sm.full[slot]);
    }
  };
  int issued = min(kLSlots, ngroups);
  if (lane == 0)
    for (int gq = 0; gq < issued; ++gq) issue(gq);

  const int a = BWD ? g.Ni - 1 - av : av;
  const int col = BWD ? (alo - x0) + kLW - 1 - lane : lane;
  int rowoff[kCW];   // c*P + a of the lane's cell m (the layout has fewer than 2^31 slots)
  bool c_ok[kCW];
#pragma unroll
  for (int m = 0; m < kCW; ++m) {
    const int cv = c0v + m;
    c_ok[m] = a_ok && cv < g.Nk;
    const int c = BWD ? g.Nk - 1 - cv : cv;
    rowoff[m] = c * g.P + a;
  }
  const bool outW = A + 1 < w.nA, outB = C + 1 < w.nC;    // edge outputs for the neighbour tiles
  float* const mWout = w.mailW + (size_t)(C * w.nA + A) * nt * kCW;
  float* const mBout = w.mailB + (size_t)(C * w.nA + A) * nt * kLW;
  const int src = (lane + kLW - 1) & (kLW - 1);   // lane L reads lane L-1; lane 0 reads lane 31
  const int pstep = BWD ? -(int)g.plane : (int)g.plane;
  float* const zbase = op.z + (long long)(BWD ? g.S - 1 - sv0 : sv0) * g.plane;

  float prev[kCW];
#pragma unroll
  for (int m = 0; m < kCW; ++m) prev[m] = 0.0f;
  bool failed = false;
  int waited = 0;
  unsigned long long staged = 0;   // last value read of sm.staged
  for (int gq = 0; gq < ngroups; ++gq) {
    const int t0 = gq * kLG;
    {   // the copy of this group has landed
      const int slot = gq % kLSlots;
      const unsigned par = (unsigned)((gq / kLSlots) & 1);
      long long it = 0;
      bool ok = false;
      for (;;) {
        ok = mbar_test(&sm.full[slot], par);
        if (ok) break;
        if (++it > 64LL * w.spin_limit) {
          atomicExch(w.abort, 1);
          atomicCAS(w.err, 0, 1);
          break;
        }
        if ((it & 1023) == 0 && (*bail || ld_relaxed_i32(w.abort))) break;
      }
      if (__any_sync(FULL, !ok)) { failed = true; *bail = 1; break; }
      waited = gq + 1;
    }
    const float* const sp = reinterpret_cast<const float*>(base + (gq % kLSlots) * L::slot_bytes) + col;
#pragma unroll
    for (int d = 0; d < kLG; ++d) {
      const int tau = t0 + d;
      if (tau >= nt) break;   // warp-uniform
      if (staged <= (unsigned long long)tau) {   // the edge values of this step are staged
        long long it = 0;
        for (;;) {
          staged = ld_acquire_cta_shared(&sm.staged);
          if (staged > (unsigned long long)tau) break;
          if (++it > 64LL * w.spin_limit) {
            atomicExch(w.abort, 1);
            atomicCAS(w.err, 0, 1);
            failed = true;
            break;
          }
          if ((it & 1023) == 0 && (*bail || ld_relaxed_i32(w.abort))) { failed = true; break; }
        }
        if (__any_sync(FULL, failed)) { failed = true; break; }
      }
      // Straight-line step without branches, in phases, so that the eight
      // cells' chains interleave: neighbours, inputs, arithmetic, stores.
      // The rings hold zero where a neighbour tile is missing (the ghost).
      const int rs = tau & (kLR - 1);
      const float eB = sm.ringB[rs][lane];
      const float4 w0 = *reinterpret_cast<const float4*>(&sm.ringW[rs][0]);   // broadcast
      const float4 w1 = *reinterpret_cast<const float4*>(&sm.ringW[rs][4]);
      const float eW[kCW] = {w0.x, w0.y, w0.z, w0.w, w1.x, w1.y, w1.z, w1.w};
      const int zb = BWD ? kLG - 1 - d : d;
      const int t1 = tau - lane;
      float Wn[kCW], Sn[kCW], Bn[kCW];
      bool ok[kCW];
#pragma unroll
      for (int m = 0; m < kCW; ++m)   // lane 31 passes the W edge to lane 0, every other lane its value on
        Wn[m] = __shfl_sync(FULL, lane == kLW - 1 ? eW[m] : prev[m], src);
#pragma unroll
      for (int m = 0; m < kCW; ++m) {
        const int bv = t1 - m;
        ok[m] = c_ok[m] && (unsigned)bv < (unsigned)g.Nj;
        Sn[m] = bv > 0 ? prev[m] : 0.0f;
        Bn[m] = m > 0 ? prev[m - 1] : eB;
      }
      float out[kCW];
#pragma unroll
      for (int m = 0; m < kCW; ++m) {
        const int row = BWD ? kCW - 1 - m : m;
        auto in = [&](int mp, int q) {
          return sp[L::map_off(mp) / 4 + ((zb * kCW + row) * Op::nq(mp) + q) * L::bw];
        };
        out[m] = op.compute(in, Wn[m], Sn[m], Bn[m]);
      }
      float* const zp = zbase + (long long)tau * pstep;
#pragma unroll
      for (int m = 0; m < kCW; ++m) {
        out[m] = ok[m] ? out[m] : 0.0f;
        st_global_f32_if(zp + rowoff[m], out[m], ok[m]);
      }
      if (outW) {
        float* const pw = mWout + (size_t)tau * kCW;
        st_relaxed_v4_if(pw, out[0], out[1], out[2], out[3], lane == kLW - 1);
        st_relaxed_v4_if(pw + 4, out[4], out[5], out[6], out[7], lane == kLW - 1);
      }
      if (outB) st_relaxed_f32_if(mBout + (size_t)tau * kLW + lane, out[kCW - 1], true);
#pragma unroll
      for (int m = 0; m < kCW; ++m) prev[m] = out[m];
    }
    if (failed) { *bail = 1; break; }
    // the slot and the ring entries of this group are free
    __syncwarp();
    if (lane == 0) {
      st_release_cta_shared_i32(&sm.done, t0 + kLG);
      if (gq + kLSlots < ngroups) {
        fence_proxy_async_smem();
        issue(gq + kLSlots);
        issued = gq + kLSlots + 1;
      }
    }
  }
  if (failed) *bail = 1;
  // the copies in flight land before the tile exits
  if (lane == 0) {
    for (int gq = waited; gq < issued; ++gq) {
      long long it = 0;
      while (!mbar_test(&sm.full[gq % kLSlots], (unsigned)((gq / kLSlots) & 1))) {
        if (++it > kDrainPolls) {
          atomicExch(w.abort, 1);
          atomicCAS(w.err, 0, 1);
          break;
        }
      }
    }
  }
  __syncwarp();
}

}  // namespace cap
