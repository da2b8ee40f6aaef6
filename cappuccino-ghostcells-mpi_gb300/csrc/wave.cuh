// wave.cuh -- persistent hyperplane wavefront for the SIP recurrences.
//
// The interior (Ni x Nj x Nk cells) is cut into lines along j; a CTA owns
// a BA x BC block of lines (a = i-3, c = k-3) with one compute thread per
// line.  Thread (a,c) computes cell (a, b, c) at hyperplane step s = a+b+c,
// so a whole CTA works on one hyperplane per step and every cell is computed
// after its three predecessors (a-1), (b-1), (c-1) -- the same per-cell
// arithmetic on the same final inputs as the reference's sequential k,i,j
// loop, hence bit-identical results.
//
// On GB300 a double-precision instruction occupies its SM sub-partition
// for 64 cycles whatever the number of active lanes, so a step costs at
// least the op's FP64 instruction count x 64 cycles.  The compute warps do
// nothing but that arithmetic and one barrier per hyperplane: a cell's
// inputs and its products with the own j-predecessor are formed before the
// step's barrier (Op::pre), only the W and B neighbours after it (Op::post).
// Two other roles run beside them:
//  * the pacing warp streams the block's inputs with tensor-memory-access
//    (TMA) copies, kG hyperplanes per copy, into kSlots shared-memory slots,
//    checks that a copy has landed (mbarrier) one step before the compute
//    warps read it and that the edge states are staged, and releases the
//    step through a named barrier: bar.red.or on barrier 1 at a copy
//    group's first step (it also carries the stop flag), bar.sync on
//    barrier 3 at the others;
//  * the communication warp moves edge states across blocks through global
//    mailboxes in which the data is its own flag: every entry holds a
//    signalling-NaN sentinel that no arithmetic result can equal, the
//    producing block stores the value, the successor's communication warp
//    polls it, stages it into a shared-memory ring indexed by plane and puts
//    the sentinel back for the next launch.  No progress counters, no
//    GPU-scope fences.
//
// Blocks are taken by ticket in topological (diagonal) order, so a block only
// waits on blocks started before it: no deadlock whatever the residency.
// Every wait is bounded: on timeout the kernel raises a device-wide abort flag
// and an error code, all warps leave their loops (the pacing warp after its
// copies in flight have landed), and the host reports CAPPGPU_E_SPIN.
//
// Backward recurrences (successors i+1, j+1, k+1) run the same engine in
// mirrored coordinates.
//
// Block-local recurrences (the FP32 preconditioner of the refinement form):
// WaveCtl::slabBA / slabBC restart the recurrence every so many blocks
// along a / c -- a slab's first line or row takes zero states, no block
// waits on or writes the mailbox across the boundary, and the slabs'
// wavefronts run side by side.  For slabs along a the mirrored blocks are
// mirrored about whole blocks (WaveCtl::mirrorA) so that they end where the
// forward blocks do; ops allow this only with zero ghost states
// (Op::kZeroGhost).  Ops may also reduce a per-cell quantity (Op::kReduce,
// accumulated per thread in Op::Part, one partial per block).
#pragma once
#include <cuda.h>

#include <type_traits>

#include "common.cuh"
#include "dlayout.cuh"

namespace cap {

struct WaveCtl {
  unsigned* ticket;               // block ticket counter: 0 between launches (the last block resets it)
  const int2* order;              // blocks in topological order
  int nBA, nBC, nblk;
  int* abort;                     // device-wide abort flag
  int* err;                       // first error (1 = spin limit, 2 = ticket)
  double* partials;               // per-block partial sums (reducing ops)
  double* mailW;                  // per block: BC x Nj states of its last a-line
  double* mailB;                  // per block: BA x Nj states of its last c-row
  long long spin_limit;
  const int* skip;                // when non-null and *skip != 0 at launch, every block exits at once
  int slabBA, slabBC;             // > 0: the recurrence restarts every slabBA blocks along a / slabBC blocks
                                  // along c (block-local SIP per slab); a slab's first line / row sees zero
                                  // states before it
  int mirrorA;                    // > 0 (mirrored blocks of an op with zero ghost states only): mirror a
                                  // about this extent, nBA x BA, instead of Ni, so that the blocks cover the
                                  // same a ranges as the forward ones; the first mirrored block then starts
                                  // with mirrorA - Ni lines outside the box
};

constexpr int kG = 4;        // hyperplanes per TMA copy
constexpr int kMaxSlots = 8; // copies in flight (per op: Op::kSlots)
constexpr int kRing = 32;    // planes of staged edge states (a power of two)
#ifndef CAP_WAVE_COMM_WARPS
#define CAP_WAVE_COMM_WARPS 1
#endif
constexpr int kComm = CAP_WAVE_COMM_WARPS;   // communication warps: 1 stages both edges, 2 one edge each
static_assert(kComm == 1 || kComm == 2, "communication warps");
// steps per barrier of the pacing warp in the FP32 substitutions and
// factorisation (a copy group: its edge-plane checks cover the whole group)
#ifndef CAP_FP32_SYNC_STEPS
#define CAP_FP32_SYNC_STEPS 4
#endif
constexpr int kFp32SyncSteps = CAP_FP32_SYNC_STEPS;
constexpr unsigned long long kSentinel = 0x7FF0DEAD5EA1F00DULL;   // signalling NaN
// a slot is refilled at the start of the next group, so two slots at least;
// the ring holds the planes between two updates of the consumed-plane count
static_assert(kRing >= kG + 3, "edge ring capacity");

__host__ __device__ constexpr int ring_slot(int q) { return q & (kRing - 1); }   // also for q < 0
static_assert((kRing & (kRing - 1)) == 0, "ring size");

// Shared-memory input slots: per map a box of (BA + 16/esize) x NQ x BC x kG
// elements (the extra columns let a mirrored block start its copy on a
// 16-byte aligned column).
template <class Op, int BA, int BC>
struct WaveLayout {
  __host__ __device__ static constexpr int align(int m) { return 16 / Op::esize(m); }   // elements per 16 bytes
  __host__ __device__ static constexpr int bw(int m) { return BA + align(m); }
  __host__ __device__ static constexpr size_t map_bytes(int m) {
    return (size_t)bw(m) * BC * kG * Op::nq(m) * Op::esize(m);
  }
  __host__ __device__ static constexpr size_t map_off(int m) {
    size_t o = 0;
    for (int q = 0; q < m; ++q) o += map_bytes(q);
    return o;
  }
  static constexpr size_t tx_bytes = map_off(Op::kMaps);
  static constexpr size_t slot_bytes = (tx_bytes + 127) / 128 * 128;
  static constexpr size_t in_bytes = Op::kSlots * slot_bytes;
  static_assert(Op::kSlots >= 2 && Op::kSlots <= kMaxSlots, "TMA slots");
};

// The compute thread's view of its inputs in one slot: element q of map m
// at box plane zb of its line.  off[m] is the byte offset of the line's
// element (q = 0, zb = 0) in a slot; with zb and q known at compile time the
// rest of the address is an immediate.
template <class Op, int BA, int BC>
struct InView {
  using L = WaveLayout<Op, BA, BC>;
  const unsigned char* slot;
  int zb;                  // plane in the box
  int off[Op::kMaps];
  // xb8 / xb4: the line's column for 8- and 4-byte maps, yb its row
  __device__ __forceinline__ void init(int xb8, int xb4, int yb) {
#pragma unroll
    for (int m = 0; m < Op::kMaps; ++m)
      off[m] = (int)L::map_off(m) + (yb * Op::nq(m) * L::bw(m) + (Op::esize(m) == 8 ? xb8 : xb4)) * Op::esize(m);
  }
  __device__ __forceinline__ int at(int m, int q) const {
    return off[m] + (zb * BC * Op::nq(m) + q) * L::bw(m) * Op::esize(m);
  }
  __device__ __forceinline__ double d(int m, int q) const { return *reinterpret_cast<const double*>(slot + at(m, q)); }
  __device__ __forceinline__ float f(int m, int q) const { return *reinterpret_cast<const float*>(slot + at(m, q)); }
};

// The cell a compute thread works on at the current step.
struct Cell {
  long long di;   // hyperplane-layout index
  int nat;        // 0-based natural index
  int sr;         // its hyperplane a+b+c
  int a, c;
};

template <class St, int BA, int BC>
struct WaveSmem {
  St sbuf[2][BC + 1][BA + 1];              // states of the two latest planes (row 0 and column 0 unused)
  St ringW[kRing][BC];                     // W edge states by plane
  St ringB[kRing][BA];                     // B edge states by plane
  unsigned long long full[kMaxSlots];
  unsigned long long stagedW, stagedB;     // edge planes <= value-2 are staged
  double red[BA * BC / 32];
  int done;                                // compute steps < done finished (updated per copy group)
  int blk[2];
  int start_ok;
  int bail;                                // any warp gave up
};

// compute warps (one thread per line) + communication warp(s) + pacing warp(s)
template <class Op, int BA, int BC>
constexpr int wave_threads() { return BA * BC + 32 * kComm + 32 * Op::kPacers; }

template <class Op, int BA, int BC>
constexpr size_t wave_smem_bytes() {
  return 128 + WaveLayout<Op, BA, BC>::in_bytes + sizeof(WaveSmem<typename Op::St, BA, BC>);
}

__device__ __forceinline__ void wave_fail(const WaveCtl& w, volatile int* bail, int code) {
  atomicExch(w.abort, 1);
  atomicCAS(w.err, 0, code);
  *bail = 1;
}

// Edge staging, split in two phases so that the loads of both edges are in
// flight together: probe_edge reads up to kPW planes of one edge (E entries
// per plane), commit_edge keeps the leading complete planes.  Entry e of
// plane q belongs to consumer line (av, cv) = line(e) whose predecessor line
// (pa, pc) is read either from the producer block's mailbox (mail[e][bv]) or,
// on the domain boundary, from the ghost layer.
template <class St>
__host__ __device__ constexpr int state_words() { return (int)((sizeof(St) + 7) / 8); }   // 8-byte mailbox words per state

template <class St, int R>
struct EdgeProbe {
  unsigned long long u[R][state_words<St>()];
  bool need[R];   // the consumer cell exists
  bool inwin[R];  // plane within the window this pass may stage
};

template <class Op, int E, bool BWD, class LineFn>
__device__ __forceinline__ void probe_edge(EdgeProbe<typename Op::St, Op::kPW * E / 32>& P, const Op& op, const DG& g,
                                           int lane, int loaded, int hi, const double* mail, LineFn line,
                                           int2 avr, int Mi, bool zero_ghost = false) {
  using St = typename Op::St;
  constexpr int NS = state_words<St>();
#pragma unroll
  for (int r = 0; r < Op::kPW * E / 32; ++r) {
    const int x = lane + 32 * r, j = x / E, e = x % E, q = loaded + 1 + j;
    int av, cv, pa, pc;
    line(e, av, cv, pa, pc);
    const int bv = q - pa - pc;   // the predecessor cell lies on plane q; the consumer has the same b
    P.inwin[r] = q <= hi;
    P.need[r] = q <= hi && av >= avr.x && av < avr.y && cv < g.Nk && bv >= 0 && bv < g.Nj;
    if (P.need[r]) {
      if (mail) {
        const double* m = mail + ((size_t)e * g.Nj + bv) * NS;
#pragma unroll
        for (int k = 0; k < NS; ++k) P.u[r][k] = ld_relaxed_b64(m + k);
      } else {
        const int a = BWD ? Mi - 1 - pa : pa;
        const int b = BWD ? g.Nj - 1 - bv : bv;
        const int c = BWD ? g.Nk - 1 - pc : pc;
        const St v = zero_ghost ? St{} : op.ghost(g.nat(a, b, c));
#pragma unroll
        for (int k = 0; k < NS; ++k) P.u[r][k] = 0;
        memcpy(P.u[r], &v, sizeof(St));
      }
    }
  }
}

template <class St, int E, int kPW, class LineFn>
__device__ __forceinline__ int commit_edge(EdgeProbe<St, kPW * E / 32>& P, const DG& g, int lane, int loaded,
                                           double* mail, St (*ring)[E], LineFn line) {
  constexpr int NS = state_words<St>();
  constexpr int R = kPW * E / 32;
  unsigned bal[R];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    bool ok = P.inwin[r];
    if (P.need[r] && mail) {
#pragma unroll
      for (int k = 0; k < NS; ++k) ok = ok && P.u[r][k] != kSentinel;
    }
    bal[r] = __ballot_sync(0xffffffffu, ok);
  }
  int n = 0;
#pragma unroll
  for (int j = 0; j < kPW; ++j) {
    const unsigned m = E >= 32 ? 0xffffffffu : ((1u << E) - 1u);
    if (((bal[(j * E) / 32] >> ((j * E) % 32)) & m) != m) break;
    ++n;
  }
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int x = lane + 32 * r, j = x / E, e = x % E, q = loaded + 1 + j;
    if (j < n && P.need[r]) memcpy(&ring[ring_slot(q)][e], P.u[r], sizeof(St));
  }
  return n;
}

// After the staged planes are published: the mailbox entries they came from
// get the sentinel back, ready for the next launch (kept out of the
// published planes' release, which would otherwise wait for these stores).
template <class St, int E, int kPW, class LineFn>
__device__ __forceinline__ void free_edge(const EdgeProbe<St, kPW * E / 32>& P, const DG& g, int lane, int loaded,
                                          int n, double* mail, LineFn line) {
  constexpr int NS = state_words<St>();
  constexpr int R = kPW * E / 32;
  if (!mail) return;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int x = lane + 32 * r, j = x / E, e = x % E, q = loaded + 1 + j;
    if (j < n && P.need[r]) {
      int av, cv, pa, pc;
      line(e, av, cv, pa, pc);
      double* m = mail + ((size_t)e * g.Nj + (q - pa - pc)) * NS;
#pragma unroll
      for (int k = 0; k < NS; ++k) st_relaxed_b64(m + k, kSentinel);
    }
  }
}

// ops whose ghost (boundary) state is zero declare kZeroGhost; only their
// mirrored launches may take a mirror extent (WaveCtl::mirrorA), and the
// others compile without its checks
template <class Op, class = void>
struct ZeroGhost : std::false_type {};
template <class Op>
struct ZeroGhost<Op, std::void_t<decltype(Op::kZeroGhost)>> : std::bool_constant<Op::kZeroGhost> {};

// the type a thread accumulates the op's reduction in: Op::Part where the op
// names one (FP32 ops: one FP64 conversion per thread, not per cell -- on
// GB300 each FP64 instruction, conversions included, holds its
// sub-partition for 64 cycles), double otherwise
template <class Op, class = void>
struct PartOf {
  using type = double;
};
template <class Op>
struct PartOf<Op, std::void_t<typename Op::Part>> {
  using type = typename Op::Part;
};

template <class Op, int BA, int BC, bool BWD>
__global__ void __launch_bounds__(wave_threads<Op, BA, BC>(), 1) k_wave(const __grid_constant__ Op op, const DG g, const WaveCtl w) {
  using St = typename Op::St;
  using L = WaveLayout<Op, BA, BC>;
  constexpr int NC = BA * BC;
  constexpr int NS = state_words<St>();
  constexpr int NSLOT = Op::kSlots;
  constexpr int NP = Op::kPacers;        // pacing warps; pacer p checks the steps with (s - s0) % NP == p
  constexpr int NB = NC + 32 * NP;       // threads in named barrier 1
  // The pacing warp takes part in the barrier of every Op::kSyncSteps-th
  // step of a copy group (every step when 1); before it, it checks the edge
  // planes of the steps up to the next such barrier and, at the group's
  // last one, the next group's copy.  The compute warps take the other
  // steps' barriers among themselves (named barrier 4).
  constexpr int E = Op::kSyncSteps;
  static_assert(E >= 1 && kG % E == 0 && (E == 1 || NP == 1), "pacing steps");
  static_assert(NC % 32 == 0, "block shape");
  constexpr int kPW = Op::kPW;           // edge planes examined per communication pass
  static_assert(32 % BC == 0 && (kPW * BC) % 32 == 0 && (kPW * BA) % 32 == 0, "edge staging shape");
  extern __shared__ unsigned char smem_raw[];
  unsigned char* base = (unsigned char*)(((size_t)smem_raw + 127) & ~(size_t)127);
  unsigned char* inbuf = base;
  WaveSmem<St, BA, BC>& sm = *reinterpret_cast<WaveSmem<St, BA, BC>*>(base + L::in_bytes);
  volatile int* bail = &sm.bail;
  const int tid = threadIdx.x;
  if (tid == 0) {
    sm.stagedW = 0;
    sm.stagedB = 0;
    sm.done = 0;
    sm.bail = 0;
    for (int k = 0; k < NSLOT; ++k) mbar_init(&sm.full[k], 1);
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
  __syncthreads();
  if (!sm.start_ok) return;
  const int ba = sm.blk[0], bc = sm.blk[1];
  // the extent a is mirrored about, the steps of the (virtual) box and the
  // range of virtual a inside the box
  constexpr bool kMirror = BWD && ZeroGhost<Op>::value;
  const int Mi = kMirror && w.mirrorA > 0 ? w.mirrorA : g.Ni;
  const int SV = Mi + g.Nj + g.Nk - 2;
  const int2 avr = make_int2(BWD ? Mi - g.Ni : 0, BWD ? Mi : g.Ni);
  const int s0 = ba * BA + bc * BC;
  const int s1 = min(SV - 1, s0 + (BA - 1) + (BC - 1) + (g.Nj - 1));
  // last plane of the W / B predecessor lines
  const int s1W = min(SV - 1, s0 - 1 + (BC - 1) + (g.Nj - 1));
  const int s1B = min(SV - 1, s0 - 1 + (BA - 1) + (g.Nj - 1));
  const int blk_id = bc * w.nBA + ba;
  const int ngroups = (s1 - s0 + kG) / kG;

  if (tid >= NC + 32 * kComm) {
    // ------------------------------------------------------- pacing warps
    const int lane = (tid - NC) & 31;
    const int pw = (tid - NC - 32 * kComm) >> 5;   // this pacer's index
    auto issue = [&](int gq) {   // TMA copy of group gq (planes s0 + gq*kG ...) into its slot
      const int slot = gq % NSLOT, sg = s0 + gq * kG;
      const int alo = BWD ? Mi - (ba + 1) * BA : ba * BA;   // first column of the block's lines
      const int y0 = BWD ? g.Nk - (bc + 1) * BC : bc * BC;
      const int z0 = BWD ? SV - sg - kG : sg;
      unsigned char* dst = inbuf + slot * L::slot_bytes;
      mbar_arrive_tx(&sm.full[slot], (unsigned)L::tx_bytes);
#pragma unroll
      for (int m = 0; m < Op::kMaps; ++m) {
        const int x0 = alo & ~(L::align(m) - 1);   // 16-byte aligned start
        if (Op::nq(m) == 1) tma_load3(dst + L::map_off(m), &op.map[m], x0, y0, z0, &sm.full[slot]);
        else tma_load4(dst + L::map_off(m), &op.map[m], x0, 0, y0, z0, &sm.full[slot]);
      }
    };
    // the copy of group gq has landed (bounded wait); false when the block gives up
    auto landed = [&](int gq) {
      long long it = 0;
      while (!mbar_test(&sm.full[gq % NSLOT], (unsigned)((gq / NSLOT) & 1))) {
        if (*bail) return false;
        if (++it > 64LL * w.spin_limit) { wave_fail(w, bail, 1); return false; }
      }
      return true;
    };
    // pacer 0 owns the copies (issue, refill, drain); group starts fall on
    // its steps because kG is a multiple of NP
    static_assert(kG % NP == 0, "group starts on pacer 0");
    int issued = min(NSLOT, ngroups);
    if (pw == 0 && lane == 0)
      for (int gq = 0; gq < issued; ++gq) issue(gq);
    // prologue: the first group's inputs are in shared memory before the
    // compute warps read them, ahead of their first step's barrier
    int pend = (pw == 0 && lane == 0 && !landed(0)) ? 1 : 0;   // a failed check, carried by the next group barrier
    bool stop = named_bar_red_or(1, NB, pend != 0);
    unsigned long long knownW = 0, knownB = 0;
    int gi = 0, ds = 0;
    for (int s = s0; s <= s1 && !stop; ++s) {
      if (ds % E != 0) {   // not part of this step's barrier
        if (++ds == kG) { ds = 0; ++gi; }
        continue;
      }
      if (lane == 0 && !pend && (s - s0) % NP == pw) {
        const int sl = min(s + E - 1, s1);   // the last step whose edge planes are checked now
        const unsigned long long needW = (unsigned long long)(unsigned)(min(sl, s1W + 1) + 1);
        const unsigned long long needB = (unsigned long long)(unsigned)(min(sl, s1B + 1) + 1);
        if (knownW < needW || knownB < needB) {   // the edge states of plane s-1 are staged
          long long it = 0;
          for (;;) {
            knownW = ld_acquire_cta_shared(&sm.stagedW);
            knownB = ld_acquire_cta_shared(&sm.stagedB);
            if (knownW >= needW && knownB >= needB) break;
            if (*bail) { pend = 1; break; }
            if (++it > 64LL * w.spin_limit) { wave_fail(w, bail, 1); pend = 1; break; }
          }
        }
        // the compute warps read the next group's inputs after the barrier
        // of this group's last step: checked before the pacing warp's last
        // barrier of the group
        if (!pend && ds == kG - E && gi + 1 < ngroups && !landed(gi + 1)) pend = 1;
      }
      // a group's first step: the barrier also carries the stop decision;
      // the other steps take a plain barrier (a failed check lets the
      // compute warps finish the group on inputs that are discarded)
      if (ds == 0) {
        if (named_bar_red_or(1, NB, pend != 0)) break;
      } else {
        named_bar_sync(3, NB);
      }
      if (pw == 0 && lane == 0 && ds == 0 && gi > 0) {
        // step s-1 is complete: the edge rings up to plane s-2 and the slot
        // of the previous group are free
        *(volatile int*)&sm.done = s;
        const int gq = gi - 1 + NSLOT;
        if (gq < ngroups) {
          fence_proxy_async_smem();
          issue(gq);
          issued = gq + 1;
        }
      }
      if (++ds == kG) { ds = 0; ++gi; }
    }
    // the copies in flight land before the block exits
    if (pw == 0 && lane == 0) {
      for (int gq = max(0, issued - NSLOT); gq < issued; ++gq) {
        long long it = 0;
        while (!mbar_test(&sm.full[gq % NSLOT], (unsigned)((gq / NSLOT) & 1))) {
          if (++it > kDrainPolls) { wave_fail(w, bail, 1); break; }
        }
      }
    }
    return;
  }

  if (tid >= NC) {
    // --------------------------------------------- communication warp(s)
    const int lane = (tid - NC) & 31;
    const int cw = (tid - NC) >> 5;   // with two warps: 0 stages the W edge, 1 the B edge
    const bool slabW = ba > 0 && w.slabBA > 0 && ba % w.slabBA == 0;   // first block column of an i-slab
    double* srcW = ba > 0 && !slabW ? w.mailW + (size_t)(blk_id - 1) * BC * g.Nj * NS : nullptr;
    const bool slab0 = bc > 0 && w.slabBC > 0 && bc % w.slabBC == 0;   // first block row of a k-slab
    double* srcB = bc > 0 && !slab0 ? w.mailB + (size_t)(blk_id - w.nBA) * BA * g.Nj * NS : nullptr;
    auto lineW = [&](int e, int& av, int& cv, int& pa, int& pc) {
      av = ba * BA; cv = bc * BC + e; pa = av - 1; pc = cv;
    };
    auto lineB = [&](int e, int& av, int& cv, int& pa, int& pc) {
      av = ba * BA + e; cv = bc * BC; pa = av; pc = cv - 1;
    };
    EdgeProbe<St, kPW * BC / 32> PW;
    EdgeProbe<St, kPW * BA / 32> PB;
    int loadedW = kComm == 2 && cw == 1 ? s1W : s0 - 2;   // last staged plane (an edge the warp
    int loadedB = kComm == 2 && cw == 0 ? s1B : s0 - 2;   // does not stage starts complete)
    long long idle = 0;
    while (loadedW < s1W || loadedB < s1B) {
      // warp-uniform decisions: the staging uses warp-wide ballots
      if (__any_sync(0xffffffffu, *bail)) break;
      const int cur = __shfl_sync(0xffffffffu, *(volatile int*)&sm.done, 0);
      const int limit = max(cur, s0) + kRing - 2;   // ring capacity
      const int hiW = min(s1W, limit), hiB = min(s1B, limit);
      probe_edge<Op, BC, BWD>(PW, op, g, lane, loadedW, hiW, srcW, lineW, avr, Mi, slabW);
      probe_edge<Op, BA, BWD>(PB, op, g, lane, loadedB, hiB, srcB, lineB, avr, Mi, slab0);
      const int nW = commit_edge<St, BC, kPW>(PW, g, lane, loadedW, srcW, sm.ringW, lineW);
      const int nB = commit_edge<St, BA, kPW>(PB, g, lane, loadedB, srcB, sm.ringB, lineB);
      if (nW + nB > 0) {
        __syncwarp();
        if (lane == 0) {
          if (nW) st_release_cta_shared(&sm.stagedW, (unsigned long long)(unsigned)(loadedW + nW + 2));
          if (nB) st_release_cta_shared(&sm.stagedB, (unsigned long long)(unsigned)(loadedB + nB + 2));
        }
        free_edge<St, BC, kPW>(PW, g, lane, loadedW, nW, srcW, lineW);
        free_edge<St, BA, kPW>(PB, g, lane, loadedB, nB, srcB, lineB);
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

  // ------------------------------------------------------ compute warps
  // Per step: the cell's inputs are read and the products with the own
  // j-predecessor formed (Op::pre) before the step's barrier, the W and B
  // neighbours after it (Op::post).  The steps of a copy group are unrolled,
  // so box offsets and buffer parities are constants and the running
  // indices advance by one addition per step.
  static_assert(BA % 2 == 0 && BC % 2 == 0 && kG % 2 == 0, "even group starts: a step's plane parity is static");
  const int al = tid % BA, cl = tid / BA;
  const int av = ba * BA + al, cv = bc * BC + cl;     // virtual (mirrored when BWD) line
  const bool line_ok = av >= avr.x && av < avr.y && cv < g.Nk;
  const int a = BWD ? Mi - 1 - av : av;
  const int c = BWD ? g.Nk - 1 - cv : cv;
  const int sfirst = av + cv;                         // step of this line's first cell
  InView<Op, BA, BC> in;                              // this line's column and row in an input box
  if (!BWD) {
    in.init(al, al, cl);
  } else {
    const int alo = Mi - (ba + 1) * BA;
    in.init((alo - (alo & ~1)) + BA - 1 - al, (alo - (alo & ~3)) + BA - 1 - al, BC - 1 - cl);
  }
  const bool edgeE = al == BA - 1 && ba + 1 < w.nBA &&   // feeds the next block along a
                     !(w.slabBA > 0 && (ba + 1) % w.slabBA == 0);   // (not across an i-slab boundary)
  const bool edgeT = cl == BC - 1 && bc + 1 < w.nBC &&   // feeds the next block along c
                     !(w.slabBC > 0 && (bc + 1) % w.slabBC == 0);   // (not across a k-slab boundary)
  double* mW = w.mailW + ((size_t)blk_id * BC + cl) * g.Nj * NS;
  double* mB = w.mailB + ((size_t)blk_id * BA + al) * g.Nj * NS;
  // W and B come from the previous plane's buffer inside the block and from
  // the staged edge rings on its first column / row
  const St* const rdW0 = al > 0 ? &sm.sbuf[0][cl + 1][al] : nullptr;
  const St* const rdW1 = al > 0 ? &sm.sbuf[1][cl + 1][al] : nullptr;
  const St* const rdB0 = cl > 0 ? &sm.sbuf[0][cl][al + 1] : nullptr;
  const St* const rdB1 = cl > 0 ? &sm.sbuf[1][cl][al + 1] : nullptr;
  St* const wr0 = &sm.sbuf[0][cl + 1][al + 1];
  St* const wr1 = &sm.sbuf[1][cl + 1][al + 1];
  // S: the j-predecessor, the ghost cell until the line's first cell
  St prevS = line_ok ? op.ghost(g.nat(a, BWD ? g.Nj : -1, c)) : St{};
  const int nat_first = g.nat(a, BWD ? g.Nj - 1 : 0, c);
  int bv = s0 - sfirst;                               // the line's j offset at the current step
  Cell x;                                             // running indices of the current step's cell
  x.a = a;
  x.c = c;
  x.sr = BWD ? SV - 1 - s0 : s0;
  x.di = (long long)x.sr * g.plane + (long long)c * g.P + a;
  x.nat = BWD ? nat_first - bv : nat_first + bv;
  const long long dstep = BWD ? -g.plane : g.plane;
  typename PartOf<Op>::type part = 0;                // this thread's share of the op's reduction
  bool stop = named_bar_red_or(1, NB, false);        // prologue: the first group has landed
  const unsigned char* slot = inbuf;
  const unsigned char* const slot_end = inbuf + NSLOT * L::slot_bytes;
  for (int sg = s0; sg <= s1 && !stop; sg += kG) {
    in.slot = slot;
#pragma unroll
    for (int ds = 0; ds < kG; ++ds) {
      if (sg + ds > s1) break;
      const bool act = line_ok && (unsigned)bv < (unsigned)g.Nj;
      in.zb = BWD ? kG - 1 - ds : ds;
      typename Op::Pre pv{};
      if (act) pv = op.pre(in, prevS);
      if (ds == 0) {
        if (named_bar_red_or(1, NB, false)) { stop = true; break; }   // plane s-1 computed; edge states staged
      } else if (ds % E == 0) {
        named_bar_sync(3, NB);
      } else {
        named_bar_sync(4, NC);
      }
      if (act) {
        const bool odd = (ds & 1) != 0;   // the plane's parity (group starts are even); previous plane in buffer !odd
        const int rs = ring_slot(sg + ds - 1);
        // (the first line inside a mirrored box that starts inside the block
        // has no neighbour line before it: the op's zero ghost state)
        const St W = kMirror && av == avr.x && al > 0 ? St{} : *(al > 0 ? (odd ? rdW0 : rdW1) : &sm.ringW[rs][cl]);
        const St B = *(cl > 0 ? (odd ? rdB0 : rdB1) : &sm.ringB[rs][al]);
        const St out = op.post(in, pv, g, x, W, B, part);
        *(odd ? wr1 : wr0) = out;
        prevS = out;
        if (edgeE || edgeT) {
          unsigned long long u[NS];
#pragma unroll
          for (int k = 0; k < NS; ++k) u[k] = 0;
          memcpy(u, &out, sizeof(St));
#pragma unroll
          for (int k = 0; k < NS; ++k) {
            if (edgeE) st_relaxed_b64(mW + (size_t)bv * NS + k, u[k]);
            if (edgeT) st_relaxed_b64(mB + (size_t)bv * NS + k, u[k]);
          }
        }
      }
      ++bv;
      x.di += dstep;
      x.sr += BWD ? -1 : 1;
      x.nat += BWD ? -1 : 1;
    }
    slot += L::slot_bytes;
    if (slot == slot_end) slot = inbuf;
  }
  if (Op::kReduce) {
    const int lane = tid & 31, wid = tid >> 5;
    double x = (double)part;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) sm.red[wid] = x;
    named_bar_sync(2, NC);
    if (tid == 0) {
      double sum = 0.0;
      for (int q = 0; q < NC / 32; ++q) sum += sm.red[q];
      w.partials[blk_id] = sum;
    }
  }
}

// ------------------------------------------------------------------ ops
// An op defines St (the state passed to successors), kMaps tensor maps of
// inputs with nq(m) components each (1 = scalar hyperplane layout, >1 =
// component-major layout), ghost (the state of a ghost cell, read from the
// module arrays) and compute (one cell: reads its inputs through in(m,q),
// writes its outputs, returns its state).

struct St3 { double bn, be, bt; };

// SIP forward substitution z = (r - bb zB - bw zW - bs zS) bp (pcg-sip.f90:102-103)
struct SipFwdD {
  using St = double;
  static constexpr int kMaps = 2;   // r, forward factors (bb, bw, bs, bp)
  static constexpr bool kReduce = false;
  static constexpr int kSlots = 3;
  static constexpr int kPacers = 1;
  static constexpr int kSyncSteps = 1;
  static constexpr int kPW = 4;   // edge planes polled per communication pass
  __host__ __device__ static constexpr int nq(int m) { return m == 0 ? 1 : 4; }
  __host__ __device__ static constexpr int esize(int) { return 8; }
  CUtensorMap map[kMaps];
  double* z;                  // hyperplane layout (output; may alias r)
  const double* ghost_src;    // natural array of ghost values, or null (zero)
  __device__ St ghost(int nat) const { return ghost_src ? ghost_src[nat] : 0.0; }
  struct Pre { double r, bb, bw, bp, tS; };   // tS = bs zS
  template <class In>
  __device__ Pre pre(const In& in, St S) const {
    return Pre{in.d(0, 0), in.d(1, 0), in.d(1, 1), in.d(1, 3), in.d(1, 2) * S};
  }
  template <class In>
  __device__ St post(const In&, const Pre& p, const DG&, const Cell& x, St W, St B, double&) const {
    const double v = (p.r - p.bb * B - p.bw * W - p.tS) * p.bp;
    z[x.di] = v;
    return v;
  }
};

// SIP backward substitution z = z - bn zN - be zE - bt zT (pcg-sip.f90:116-117)
// with the fused dot sk = sum res.z (pcg-sip.f90:118); the engine's S, W, B
// neighbours are the j+1, i+1, k+1 cells here.
struct SipBwdD {
  using St = double;
  static constexpr int kMaps = 3;   // z, backward factors (bn, be, bt), res
  static constexpr bool kReduce = true;
  static constexpr int kSlots = 3;
  static constexpr int kPacers = 1;
  static constexpr int kSyncSteps = 1;
  static constexpr int kPW = 4;   // edge planes polled per communication pass
  __host__ __device__ static constexpr int nq(int m) { return m == 1 ? 3 : 1; }
  __host__ __device__ static constexpr int esize(int) { return 8; }
  CUtensorMap map[kMaps];
  double* z;
  const double* ghost_src;
  __device__ St ghost(int nat) const { return ghost_src ? ghost_src[nat] : 0.0; }
  struct Pre { double t, be, bt, res; };   // t = z - bn zS
  template <class In>
  __device__ Pre pre(const In& in, St S) const {
    return Pre{in.d(0, 0) - in.d(1, 0) * S, in.d(1, 1), in.d(1, 2), in.d(2, 0)};
  }
  template <class In>
  __device__ St post(const In&, const Pre& p, const DG&, const Cell& x, St W, St B, double& part) const {
    const double v = p.t - p.be * W - p.bt * B;
    z[x.di] = v;
    part += p.res * v;
    return v;
  }
};

// SIP backward substitution with fi += z (sipsol.f90:86-88)
struct SipBwdFiD {
  using St = double;
  static constexpr int kMaps = 3;   // z, backward factors, fi
  static constexpr bool kReduce = false;
  static constexpr int kSlots = 3;
  static constexpr int kPacers = 1;
  static constexpr int kSyncSteps = 1;
  static constexpr int kPW = 4;   // edge planes polled per communication pass
  __host__ __device__ static constexpr int nq(int m) { return m == 1 ? 3 : 1; }
  __host__ __device__ static constexpr int esize(int) { return 8; }
  CUtensorMap map[kMaps];
  double* z;
  double* fi;                 // hyperplane layout
  const double* ghost_src;    // module res (stale ghost values, as the reference reads them)
  __device__ St ghost(int nat) const { return ghost_src[nat]; }
  struct Pre { double t, be, bt, fi; };   // t = z - bn zS
  template <class In>
  __device__ Pre pre(const In& in, St S) const {
    return Pre{in.d(0, 0) - in.d(1, 0) * S, in.d(1, 1), in.d(1, 2), in.d(2, 0)};
  }
  template <class In>
  __device__ St post(const In&, const Pre& p, const DG&, const Cell& x, St W, St B, double&) const {
    const double v = p.t - p.be * W - p.bt * B;
    z[x.di] = v;
    fi[x.di] = p.fi + v;
    return v;
  }
};

// SIP factorisation (pcg-sip.f90:68-87); state passed on = (bn, be, bt)
struct SipFactorD {
  using St = St3;
  static constexpr int kMaps = 7;   // ae, aw, an, as, at, ab, ap
  static constexpr bool kReduce = false;
  static constexpr int kSlots = 3;
  static constexpr int kPacers = 1;
  static constexpr int kSyncSteps = 1;
  static constexpr int kPW = 4;   // edge planes polled per communication pass
  __host__ __device__ static constexpr int nq(int) { return 1; }
  __host__ __device__ static constexpr int esize(int) { return 8; }
  CUtensorMap map[kMaps];
  double *bbn, *bwn, *bsn, *bpn, *bnn, *ben, *btn;  // natural layout outputs (module coefb)
  double* fq;                                       // forward factors, 4 components
  double* bq;                                       // backward factors, 3 components
  double alfa;
  __device__ St ghost(int nat) const { return St3{bnn[nat], ben[nat], btn[nat]}; }
  // pre: the terms of the j-predecessor S (bs and its products)
  struct Pre { double ab, aw, ap, an, ae, at, bsv, sbe, sbt, sbn; };
  template <class In>
  __device__ Pre pre(const In& in, St S) const {
    const double bsv = -in.d(3, 0) / (1.0 + alfa * (S.be + S.bt));
    return Pre{in.d(5, 0), in.d(1, 0), in.d(6, 0), in.d(2, 0), in.d(0, 0), in.d(4, 0),
               bsv, bsv * S.be, bsv * S.bt, bsv * S.bn};
  }
  template <class In>
  __device__ St post(const In&, const Pre& q, const DG& g, const Cell& x, St W, St B, double&) const {
    const double bbv = -q.ab / (1.0 + alfa * (B.bn + B.be));
    const double bwv = -q.aw / (1.0 + alfa * (W.bn + W.bt));
    const double bsv = q.bsv;
    const double p1 = alfa * (bbv * B.bn + bwv * W.bn);
    const double p2 = alfa * (bbv * B.be + q.sbe);
    const double p3 = alfa * (bwv * W.bt + q.sbt);
    const double bpv = 1.0 / (q.ap + p1 + p2 + p3 - bbv * B.bt - bwv * W.be - q.sbn + CAP_SMALL);
    const double bnv = (-q.an - p1) * bpv;
    const double bev = (-q.ae - p2) * bpv;
    const double btv = (-q.at - p3) * bpv;
    const int nat = x.nat;
    bbn[nat] = bbv; bwn[nat] = bwv; bsn[nat] = bsv; bpn[nat] = bpv;
    bnn[nat] = bnv; ben[nat] = bev; btn[nat] = btv;
    fq[g.dqs(x.sr, x.c, x.a, 0, 4)] = bbv;
    fq[g.dqs(x.sr, x.c, x.a, 1, 4)] = bwv;
    fq[g.dqs(x.sr, x.c, x.a, 2, 4)] = bsv;
    fq[g.dqs(x.sr, x.c, x.a, 3, 4)] = bpv;
    bq[g.dqs(x.sr, x.c, x.a, 0, 3)] = bnv;
    bq[g.dqs(x.sr, x.c, x.a, 1, 3)] = bev;
    bq[g.dqs(x.sr, x.c, x.a, 2, 3)] = btv;
    return St3{bnv, bev, btv};
  }
};

// ICCG (iccg.f90:3-197).  IC(0) diagonal d = 1/(ap - aw^2 dW - as^2 dS -
// ab^2 dB) (iccg.f90:73-80; its 1. is exactly 1); state passed on = d; written to the
// hyperplane layout only (the reference's d is a local work array).
struct IcDiagD {
  using St = double;
  static constexpr int kMaps = 4;   // ap, aw, as, ab
  static constexpr bool kReduce = false;
  static constexpr int kSlots = 3;
  static constexpr int kPacers = 1;
  static constexpr int kSyncSteps = 1;
  static constexpr int kPW = 4;
  __host__ __device__ static constexpr int nq(int) { return 1; }
  __host__ __device__ static constexpr int esize(int) { return 8; }
  CUtensorMap map[kMaps];
  double* dg;
  __device__ St ghost(int) const { return 0.0; }   // the work array is zero outside the loop box
  struct Pre { double ap, aww, abb, sS; };          // sS = as^2 dS
  template <class In>
  __device__ Pre pre(const In& in, St S) const {
    const double as = in.d(2, 0);
    return Pre{in.d(0, 0), in.d(1, 0) * in.d(1, 0), in.d(3, 0) * in.d(3, 0), as * as * S};
  }
  template <class In>
  __device__ St post(const In&, const Pre& p, const DG&, const Cell& x, St W, St B, double&) const {
    const double v = 1.0 / (p.ap - p.aww * W - p.sS - p.abb * B);
    dg[x.di] = v;
    return v;
  }
};

// ICCG forward substitution z = (r + aw zW + as zS + ab zB) d (iccg.f90:92-99)
struct IcFwdD {
  using St = double;
  static constexpr int kMaps = 5;   // r, aw, as, ab, d
  static constexpr bool kReduce = false;
  static constexpr int kSlots = 3;
  static constexpr int kPacers = 1;
  static constexpr int kSyncSteps = 1;
  static constexpr int kPW = 4;
  __host__ __device__ static constexpr int nq(int) { return 1; }
  __host__ __device__ static constexpr int esize(int) { return 8; }
  CUtensorMap map[kMaps];
  double* z;
  __device__ St ghost(int) const { return 0.0; }
  struct Pre { double r, aw, ab, dg, sS; };   // sS = as zS
  template <class In>
  __device__ Pre pre(const In& in, St S) const {
    return Pre{in.d(0, 0), in.d(1, 0), in.d(3, 0), in.d(4, 0), in.d(2, 0) * S};
  }
  template <class In>
  __device__ St post(const In&, const Pre& p, const DG&, const Cell& x, St W, St B, double&) const {
    const double v = (p.r + p.aw * W + p.sS + p.ab * B) * p.dg;
    z[x.di] = v;
    return v;
  }
};

// ICCG backward substitution z = (z + ae zE + an zN + at zT) d with the
// dot sk = sum res z in the same loop (iccg.f90:112-124); the
// engine's S, W, B neighbours are the j+1, i+1, k+1 cells here.
struct IcBwdD {
  using St = double;
  static constexpr int kMaps = 6;   // z (after the division by d), ae, an, at, d, res
  static constexpr bool kReduce = true;
  static constexpr int kSlots = 3;
  static constexpr int kPacers = 1;
  static constexpr int kSyncSteps = 1;
  static constexpr int kPW = 4;
  __host__ __device__ static constexpr int nq(int) { return 1; }
  __host__ __device__ static constexpr int esize(int) { return 8; }
  CUtensorMap map[kMaps];
  double* z;
  __device__ St ghost(int) const { return 0.0; }
  struct Pre { double z, ae, at, dg, res, sS; };   // sS = an zN
  template <class In>
  __device__ Pre pre(const In& in, St S) const {
    return Pre{in.d(0, 0), in.d(1, 0), in.d(3, 0), in.d(4, 0), in.d(5, 0), in.d(2, 0) * S};
  }
  template <class In>
  __device__ St post(const In&, const Pre& p, const DG&, const Cell& x, St W, St B, double& part) const {
    const double v = (p.z + p.ae * W + p.sS + p.at * B) * p.dg;
    z[x.di] = v;
    part += p.res * v;
    return v;
  }
};

// ------------------------------------------------- single-precision ops
// The preconditioner of the FP32 + FP64-refinement form of the pressure
// solve: the same SIP recurrences (pcg-sip.f90:68-121) on FP32 copies of
// the matrix, FP32 arithmetic, zero ghost states for the substitutions.
// These do not reproduce the reference's FP64 results bit for bit and are
// not meant to; the refinement loop around them restores the FP64 residual.

struct St3f { float bn, be, bt; };

struct SipFwdF {
  using St = float;
  static constexpr bool kZeroGhost = true;   // ghost() is zero: mirror extents allowed
  static constexpr int kMaps = 2;   // r, forward factors (bb, bw, bs, bp)
  static constexpr bool kReduce = false;
  static constexpr int kSlots = 6;
  static constexpr int kPacers = 1;
  static constexpr int kSyncSteps = kFp32SyncSteps;
  static constexpr int kPW = 8;
  __host__ __device__ static constexpr int nq(int m) { return m == 0 ? 1 : 4; }
  __host__ __device__ static constexpr int esize(int) { return 4; }
  CUtensorMap map[kMaps];
  float* z;
  __device__ St ghost(int) const { return 0.0f; }
  struct Pre { float r, bb, bw, bp, tS; };
  template <class In>
  __device__ Pre pre(const In& in, St S) const {
    return Pre{in.f(0, 0), in.f(1, 0), in.f(1, 1), in.f(1, 3), in.f(1, 2) * S};
  }
  template <class In>
  __device__ St post(const In&, const Pre& p, const DG&, const Cell& x, St W, St B, double&) const {
    const float v = (p.r - p.bb * B - p.bw * W - p.tS) * p.bp;
    z[x.di] = v;
    return v;
  }
};

struct SipBwdF {
  using St = float;
  static constexpr bool kZeroGhost = true;   // ghost() is zero: mirror extents allowed
  static constexpr int kMaps = 2;   // z, backward factors (bn, be, bt)
  static constexpr bool kReduce = false;
  static constexpr int kSlots = 6;
  static constexpr int kPacers = 1;
  static constexpr int kSyncSteps = kFp32SyncSteps;
  static constexpr int kPW = 8;
  __host__ __device__ static constexpr int nq(int m) { return m == 1 ? 3 : 1; }
  __host__ __device__ static constexpr int esize(int) { return 4; }
  CUtensorMap map[kMaps];
  float* z;
  __device__ St ghost(int) const { return 0.0f; }
  struct Pre { float t, be, bt; };
  template <class In>
  __device__ Pre pre(const In& in, St S) const {
    return Pre{in.f(0, 0) - in.f(1, 0) * S, in.f(1, 1), in.f(1, 2)};
  }
  template <class In>
  __device__ St post(const In&, const Pre& p, const DG&, const Cell& x, St W, St B, double&) const {
    const float v = p.t - p.be * W - p.bt * B;
    z[x.di] = v;
    return v;
  }
};

// the same with the dot sk = sum r.z fused (the FP32 CG of the refinement
// form; pcg-sip.f90:118), partials per block
struct SipBwdDotF {
  using St = float;
  static constexpr bool kZeroGhost = true;   // ghost() is zero: mirror extents allowed
  using Part = float;   // per-thread FP32 sum, as the vector pass forms it
  static constexpr int kMaps = 3;   // z, backward factors (bn, be, bt), r
  static constexpr bool kReduce = true;
  static constexpr int kSlots = 6;
  static constexpr int kPacers = 1;
  static constexpr int kSyncSteps = kFp32SyncSteps;
  static constexpr int kPW = 8;
  __host__ __device__ static constexpr int nq(int m) { return m == 1 ? 3 : 1; }
  __host__ __device__ static constexpr int esize(int) { return 4; }
  CUtensorMap map[kMaps];
  float* z;
  __device__ St ghost(int) const { return 0.0f; }
  struct Pre { float t, be, bt, r; };
  template <class In>
  __device__ Pre pre(const In& in, St S) const {
    return Pre{in.f(0, 0) - in.f(1, 0) * S, in.f(1, 1), in.f(1, 2), in.f(2, 0)};
  }
  template <class In>
  __device__ St post(const In&, const Pre& p, const DG&, const Cell& x, St W, St B, float& part) const {
    const float v = p.t - p.be * W - p.bt * B;
    z[x.di] = v;
    part += p.r * v;
    return v;
  }
};

struct SipFactorF {
  using St = St3f;
  static constexpr int kMaps = 7;   // ae, aw, an, as, at, ab, ap (FP32 copies)
  static constexpr bool kReduce = false;
  static constexpr int kSlots = 4;
  static constexpr int kPacers = 1;
  static constexpr int kSyncSteps = kFp32SyncSteps;
  static constexpr int kPW = 8;
  __host__ __device__ static constexpr int nq(int) { return 1; }
  __host__ __device__ static constexpr int esize(int) { return 4; }
  CUtensorMap map[kMaps];
  const double *bnn, *ben, *btn;   // module factors: the ghost-layer states the factorisation reads
  float* fq;                       // forward factors, 4 components
  float* bq;                       // backward factors, 3 components
  float alfa;
  __device__ St ghost(int nat) const { return St3f{(float)bnn[nat], (float)ben[nat], (float)btn[nat]}; }
  struct Pre { float ab, aw, ap, an, ae, at, bsv, sbe, sbt, sbn; };
  template <class In>
  __device__ Pre pre(const In& in, St S) const {
    const float bsv = -in.f(3, 0) / (1.0f + alfa * (S.be + S.bt));
    return Pre{in.f(5, 0), in.f(1, 0), in.f(6, 0), in.f(2, 0), in.f(0, 0), in.f(4, 0),
               bsv, bsv * S.be, bsv * S.bt, bsv * S.bn};
  }
  template <class In>
  __device__ St post(const In&, const Pre& q, const DG& g, const Cell& x, St W, St B, double&) const {
    const float bbv = -q.ab / (1.0f + alfa * (B.bn + B.be));
    const float bwv = -q.aw / (1.0f + alfa * (W.bn + W.bt));
    const float bsv = q.bsv;
    const float p1 = alfa * (bbv * B.bn + bwv * W.bn);
    const float p2 = alfa * (bbv * B.be + q.sbe);
    const float p3 = alfa * (bwv * W.bt + q.sbt);
    const float bpv = 1.0f / (q.ap + p1 + p2 + p3 - bbv * B.bt - bwv * W.be - q.sbn + 1e-30f);
    const float bnv = (-q.an - p1) * bpv;
    const float bev = (-q.ae - p2) * bpv;
    const float btv = (-q.at - p3) * bpv;
    fq[g.dqs(x.sr, x.c, x.a, 0, 4)] = bbv;
    fq[g.dqs(x.sr, x.c, x.a, 1, 4)] = bwv;
    fq[g.dqs(x.sr, x.c, x.a, 2, 4)] = bsv;
    fq[g.dqs(x.sr, x.c, x.a, 3, 4)] = bpv;
    bq[g.dqs(x.sr, x.c, x.a, 0, 3)] = bnv;
    bq[g.dqs(x.sr, x.c, x.a, 1, 3)] = bev;
    bq[g.dqs(x.sr, x.c, x.a, 2, 3)] = btv;
    return St3f{bnv, bev, btv};
  }
};

}  // namespace cap
