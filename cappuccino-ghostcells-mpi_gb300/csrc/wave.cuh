// wave.cuh -- persistent hyperplane wavefront for the SIP recurrences.
//
// The interior (Ni x Nj x Nk cells) is cut into lines along j; a CTA owns
// a BA x BC block of lines (a = i-3, c = k-3) with one thread per line.
// Thread (a,c) computes cell (a, b, c) at hyperplane step s = a+b+c, so a
// whole CTA works on one hyperplane per step and every cell is computed
// after its three predecessors (a-1), (b-1), (c-1) -- the same per-cell
// arithmetic on the same final inputs as the reference's sequential
// k,i,j loop, hence bit-identical results.
//
// Predecessor states: along j from the thread's own previous step; across
// the CTA's lines through shared memory; across CTA blocks from the
// neighbour block's published output in global memory.  Each block
// publishes "planes < s done" with st.release.gpu and its successors wait
// for it through their communication warp (see k_wave).  Blocks are
// taken by ticket in topological (diagonal) order, so a block only ever
// waits on blocks that were started before it: no deadlock whatever the
// residency.  Every wait is bounded: on timeout the kernel raises a
// device-wide abort flag and an error code, all blocks leave their loops,
// and the host reports CAPPGPU_E_SPIN.
//
// Backward recurrences (successors i+1, j+1, k+1) run the same engine in
// mirrored coordinates.
#pragma once
#include "common.cuh"
#include "dlayout.cuh"

namespace cap {

struct WaveCtl {
  unsigned* ticket;               // monotonically increasing ticket counter
  unsigned ticket_base;           // its value when this launch started
  const int2* order;              // blocks in topological order
  unsigned long long* prog;       // per-block progress: tag | planes done
  unsigned long long tag;         // launch epoch << 32
  int nBA, nBC, nblk;
  int* abort;                     // device-wide abort flag
  int* err;                       // first error (1 = spin limit)
  double* partials;               // per-block partial sums (reducing ops)
  long long spin_limit;
  int publish_every;
};

// Block structure: BA*BC compute threads (one per line) plus one
// communication warp.  Compute warps synchronise per hyperplane with named
// barrier 1 and never touch global synchronisation variables; lane 0 of the
// communication warp polls the two predecessor blocks' progress (relaxed
// loads + acquire fence) and mirrors it into shared memory, and publishes
// this block's progress (release store) whenever the compute warps finish
// planes.  Shared-memory handoffs use cta-scope release/acquire, so a compute
// thread that has seen the mirrored progress also sees the producer's data.
template <class Op, int BA, int BC, bool BWD>
__global__ void __launch_bounds__(BA * BC + 32) k_wave(Op op, DG g, WaveCtl w) {
  using St = typename Op::St;
  constexpr int NC = BA * BC;
  __shared__ St sbuf[2][BC][BA];
  __shared__ int s_blk[2];
  __shared__ volatile int s_bail;
  __shared__ unsigned long long s_seenW, s_seenB, s_done;
  const int tid = threadIdx.x;
  if (tid == 0) {
    s_seenW = 0;
    s_seenB = 0;
    s_done = 0;
    unsigned t = atomicAdd(w.ticket, 1u) - w.ticket_base;
    if (t < (unsigned)w.nblk) {
      int2 blk = w.order[t];
      s_blk[0] = blk.x;
      s_blk[1] = blk.y;
      s_bail = 0;
    } else {   // ticket counter out of step with the host: refuse to run
      s_blk[0] = s_blk[1] = 0;
      s_bail = 1;
      atomicExch(w.abort, 1);
      atomicCAS(w.err, 0, 2);
    }
  }
  __syncthreads();
  if (s_bail) return;
  const int ba = s_blk[0], bc = s_blk[1];
  const int s0 = ba * BA + bc * BC;
  const int s1 = min(g.S - 1, s0 + (BA - 1) + (BC - 1) + (g.Nj - 1));
  // a predecessor block publishes planes up to its own last plane only; its
  // lines have no cells beyond it, so waits are capped there
  const int s1W = min(g.S - 1, s0 - BA + (BA - 1) + (BC - 1) + (g.Nj - 1));
  const int s1B = min(g.S - 1, s0 - BC + (BA - 1) + (BC - 1) + (g.Nj - 1));
  const int blk_id = bc * w.nBA + ba;
  const bool hasW = ba > 0, hasB = bc > 0;

  if (tid >= NC) {
    // ------------------------------------------------ communication warp
    if (tid != NC) return;
    unsigned long long* myprog = w.prog + blk_id;
    const unsigned long long* pW = hasW ? w.prog + (blk_id - 1) : nullptr;
    const unsigned long long* pB = hasB ? w.prog + (blk_id - w.nBA) : nullptr;
    const unsigned long long lastW = w.tag | (unsigned long long)(unsigned)(s1W + 1);
    const unsigned long long lastB = w.tag | (unsigned long long)(unsigned)(s1B + 1);
    const unsigned long long fin = (unsigned long long)(unsigned)(s1 + 1);
    unsigned long long seenW = 0, seenB = 0, pub = 0;
    long long idle = 0;
    for (;;) {
      bool act = false;
      unsigned long long vW = (pW && seenW < lastW) ? ld_relaxed_u64(pW) : 0;
      unsigned long long vB = (pB && seenB < lastB) ? ld_relaxed_u64(pB) : 0;
      if (vW > seenW || vB > seenB) {
        fence_acq_rel_gpu();   // acquire: the producers' data is visible from here on
        if (vW > seenW) { seenW = vW; st_release_cta_shared(&s_seenW, vW); }
        if (vB > seenB) { seenB = vB; st_release_cta_shared(&s_seenB, vB); }
        act = true;
      }
      const unsigned long long dn = ld_acquire_cta_shared(&s_done);
      if (dn > pub) {
        st_release_u64(myprog, w.tag | dn);
        pub = dn;
        act = true;
        if (dn == fin) break;
      }
      if (s_bail) break;
      if (act) {
        idle = 0;
      } else {
        if (++idle > w.spin_limit) {
          atomicExch(w.abort, 1);
          atomicCAS(w.err, 0, 1);
          s_bail = 1;
          break;
        }
        if ((idle & 31) == 31 && ld_relaxed_i32(w.abort)) { s_bail = 1; break; }
        __nanosleep(20);
      }
    }
    return;
  }

  // ------------------------------------------------------ compute warps
  const int al = tid % BA, cl = tid / BA;
  const int av = ba * BA + al, cv = bc * BC + cl;     // virtual (mirrored when BWD) line
  const bool line_ok = av < g.Ni && cv < g.Nk;
  const int a = BWD ? g.Ni - 1 - av : av;
  const int c = BWD ? g.Nk - 1 - cv : cv;
  const int da = BWD ? 1 : -1;                         // real offset of a predecessor
  St prevS{};
  double part = 0.0;
  for (int s = s0; s <= s1; ++s) {
    if (tid == 0) {
      const unsigned long long needW = w.tag | (unsigned long long)(unsigned)min(s, s1W + 1);
      const unsigned long long needB = w.tag | (unsigned long long)(unsigned)min(s, s1B + 1);
      long long it = 0;
      while ((hasW && ld_acquire_cta_shared(&s_seenW) < needW) || (hasB && ld_acquire_cta_shared(&s_seenB) < needB)) {
        if (s_bail) break;
        if (++it > 64LL * w.spin_limit) {
          atomicExch(w.abort, 1);
          atomicCAS(w.err, 0, 1);
          s_bail = 1;
          break;
        }
      }
    }
    named_bar_sync(1, NC);   // plane s-1 done in this block; predecessors' planes <= s-1 visible
    if (s_bail) break;
    if (tid == 0 && s > s0) st_release_cta_shared(&s_done, (unsigned long long)(unsigned)s);
    const int bv = s - av - cv;
    if (line_ok && bv >= 0 && bv < g.Nj) {
      const int b = BWD ? g.Nj - 1 - bv : bv;
      St W, B, S;
      if (al > 0) W = sbuf[(s - 1) & 1][cl][al - 1];
      else if (av > 0) W = op.load(g.d(a + da, b, c));
      else W = op.ghost(g.nat(a + da, b, c));
      if (cl > 0) B = sbuf[(s - 1) & 1][cl - 1][al];
      else if (cv > 0) B = op.load(g.d(a, b, c + da));
      else B = op.ghost(g.nat(a, b, c + da));
      if (bv > 0) S = prevS;
      else S = op.ghost(g.nat(a, b + da, c));
      St out = op.compute(g.d(a, b, c), g.nat(a, b, c), W, S, B, part);
      sbuf[s & 1][cl][al] = out;
      prevS = out;
    }
  }
  named_bar_sync(1, NC);
  if (tid == 0 && !s_bail) st_release_cta_shared(&s_done, (unsigned long long)(unsigned)(s1 + 1));
  if (Op::kReduce) {
    __shared__ double sh[NC / 32];
    const int lane = tid & 31, wid = tid >> 5;
    double x = part;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) sh[wid] = x;
    named_bar_sync(1, NC);
    if (tid == 0) {
      double sum = 0.0;
      for (int q = 0; q < NC / 32; ++q) sum += sh[q];
      w.partials[blk_id] = sum;
    }
  }
}

// ------------------------------------------------------------------ ops

struct __align__(32) F4 { double bb, bw, bs, bp; };
struct __align__(32) B4 { double bn, be, bt, pad; };
struct St3 { double bn, be, bt; };

// SIP forward substitution z = (r - bb zB - bw zW - bs zS) bp (pcg-sip.f90:208-209)
struct SipFwdD {
  using St = double;
  static constexpr bool kReduce = false;
  const double* r;            // diagonal layout
  const F4* f;                // diagonal layout
  double* z;                  // diagonal layout (output)
  const double* ghost_src;    // natural array of ghost values, or null (zero)
  __device__ St ghost(int nat) const { return ghost_src ? ghost_src[nat] : 0.0; }
  __device__ St load(long long di) const { return __ldcg(z + di); }
  __device__ St compute(long long di, int, St W, St S, St B, double&) const {
    const F4 q = f[di];
    const double v = (r[di] - q.bb * B - q.bw * W - q.bs * S) * q.bp;
    z[di] = v;
    return v;
  }
};

// SIP backward substitution z = z - bn zN - be zE - bt zT (pcg-sip.f90:222-223)
// with the fused dot sk = sum res.z (pcg-sip.f90:224); the engine's S, W, B
// neighbours are the j+1, i+1, k+1 cells here.
struct SipBwdD {
  using St = double;
  static constexpr bool kReduce = true;
  const B4* f;
  double* z;
  const double* res;          // diagonal layout (dot), may be null
  const double* ghost_src;
  __device__ St ghost(int nat) const { return ghost_src ? ghost_src[nat] : 0.0; }
  __device__ St load(long long di) const { return __ldcg(z + di); }
  __device__ St compute(long long di, int, St W, St S, St B, double& part) const {
    const B4 q = f[di];
    const double v = z[di] - q.bn * S - q.be * W - q.bt * B;
    z[di] = v;
    if (res) part += res[di] * v;
    return v;
  }
};

// SIP factorisation (pcg-sip.f90:178-190); state passed on = (bn, be, bt)
struct SipFactorD {
  using St = St3;
  static constexpr bool kReduce = false;
  const double *ae, *aw, *an, *as, *at, *ab, *ap;   // diagonal layout
  double *bbn, *bwn, *bsn, *bpn, *bnn, *ben, *btn;  // natural layout outputs (module coefb)
  F4* f;                                            // diagonal layout outputs
  B4* g4;
  double alfa;
  __device__ St ghost(int nat) const { return St3{bnn[nat], ben[nat], btn[nat]}; }
  __device__ St load(long long di) const {
    const double* p = reinterpret_cast<const double*>(g4 + di);
    return St3{__ldcg(p), __ldcg(p + 1), __ldcg(p + 2)};
  }
  __device__ St compute(long long di, int nat, St W, St S, St B, double&) const {
    const double bbv = -ab[di] / (1.0 + alfa * (B.bn + B.be));
    const double bwv = -aw[di] / (1.0 + alfa * (W.bn + W.bt));
    const double bsv = -as[di] / (1.0 + alfa * (S.be + S.bt));
    const double p1 = alfa * (bbv * B.bn + bwv * W.bn);
    const double p2 = alfa * (bbv * B.be + bsv * S.be);
    const double p3 = alfa * (bwv * W.bt + bsv * S.bt);
    const double bpv = 1.0 / (ap[di] + p1 + p2 + p3 - bbv * B.bt - bwv * W.be - bsv * S.bn + CAP_SMALL);
    const double bnv = (-an[di] - p1) * bpv;
    const double bev = (-ae[di] - p2) * bpv;
    const double btv = (-at[di] - p3) * bpv;
    bbn[nat] = bbv; bwn[nat] = bwv; bsn[nat] = bsv; bpn[nat] = bpv;
    bnn[nat] = bnv; ben[nat] = bev; btn[nat] = btv;
    f[di] = F4{bbv, bwv, bsv, bpv};
    g4[di] = B4{bnv, bev, btv, 0.0};
    return St3{bnv, bev, btv};
  }
};

}  // namespace cap
