// wavefront.cuh -- the incomplete-factorisation recurrences of the
// reference (SIP factorisation, SIP forward/backward substitution, IC(0)
// and ILU(0) diagonals and substitutions) executed in i+j+k hyperplane
// order.
//
// Each recurrence computes cell (i,j,k) from already-final values at
// (i-1,j,k), (i,j-1,k), (i,j,k-1) (forward) or (i+1,j,k), (i,j+1,k),
// (i,j,k+1) (backward) with a fixed per-cell expression.  Every cell of
// hyperplane s = i+j+k depends only on hyperplane s-1 (s+1), so computing the
// planes in order reproduces the sequential k,i,j loop of the reference bit
// for bit: the per-cell arithmetic is identical and its inputs are the same
// final values.  Cells outside the loop box (ghost layers) are read as they
// are, exactly as the reference reads them.
#pragma once
#include "common.cuh"

namespace cap {

// SIP factorisation, sipsol.f90:34-46 (pcg-sip.f90:68-87, cgstab_sip.f90:64-76)
struct SipFactorOp {
  const double *ae, *aw, *an, *as, *at, *ab, *ap;
  double *bb, *bw, *bs, *bp, *bn, *be, *bt;
  double alfa;
  int nj, nij;
  __device__ void operator()(int ijk) const {
    double bbv = -ab[ijk] / (1.0 + alfa * (bn[ijk - nij] + be[ijk - nij]));
    double bwv = -aw[ijk] / (1.0 + alfa * (bn[ijk - nj] + bt[ijk - nj]));
    double bsv = -as[ijk] / (1.0 + alfa * (be[ijk - 1] + bt[ijk - 1]));
    double p1 = alfa * (bbv * bn[ijk - nij] + bwv * bn[ijk - nj]);
    double p2 = alfa * (bbv * be[ijk - nij] + bsv * be[ijk - 1]);
    double p3 = alfa * (bwv * bt[ijk - nj] + bsv * bt[ijk - 1]);
    double bpv = 1.0 / (ap[ijk] + p1 + p2 + p3 - bbv * bt[ijk - nij] - bwv * be[ijk - nj] -
                        bsv * bn[ijk - 1] + CAP_SMALL);
    bb[ijk] = bbv; bw[ijk] = bwv; bs[ijk] = bsv; bp[ijk] = bpv;
    bn[ijk] = (-an[ijk] - p1) * bpv;
    be[ijk] = (-ae[ijk] - p2) * bpv;
    bt[ijk] = (-at[ijk] - p3) * bpv;
  }
};

// SIP forward substitution z = (r - bb zB - bw zW - bs zS) bp
// (pcg-sip.f90:102-103; sipsol.f90:70-71 with r = z = res)
struct SipFwdOp {
  const double *r, *bb, *bw, *bs, *bp;
  double* z;
  int nj, nij;
  __device__ void operator()(int ijk) const {
    z[ijk] = (r[ijk] - bb[ijk] * z[ijk - nij] - bw[ijk] * z[ijk - nj] - bs[ijk] * z[ijk - 1]) * bp[ijk];
  }
};

// SIP backward substitution z = z - bn zN - be zE - bt zT (pcg-sip.f90:116-117);
// with fi != nullptr also fi += z (sipsol.f90:86-88).
struct SipBwdOp {
  const double *bn, *be, *bt;
  double* z;
  double* fi;
  int nj, nij;
  __device__ void operator()(int ijk) const {
    double v = z[ijk] - bn[ijk] * z[ijk + 1] - be[ijk] * z[ijk + nj] - bt[ijk] * z[ijk + nij];
    z[ijk] = v;
    if (fi) fi[ijk] = fi[ijk] + v;
  }
};

// IC(0) diagonal, iccg.f90:77-78
struct IccgDiagOp {
  const double *ap, *aw, *as, *ab;
  double* dg;
  int nj, nij;
  __device__ void operator()(int ijk) const {
    dg[ijk] = 1.0 / (ap[ijk] - aw[ijk] * aw[ijk] * dg[ijk - nj] - as[ijk] * as[ijk] * dg[ijk - 1] -
                     ab[ijk] * ab[ijk] * dg[ijk - nij]);
  }
};

// ILU(0) diagonal, cgstab.f90:62-64
struct IluDiagOp {
  const double *ap, *aw, *as, *ab, *ae, *an, *at;
  double* dg;
  int nj, nij;
  __device__ void operator()(int ijk) const {
    dg[ijk] = 1.0 / (ap[ijk] - aw[ijk] * dg[ijk - nj] * ae[ijk - nj] - as[ijk] * dg[ijk - 1] * an[ijk - 1] -
                     ab[ijk] * dg[ijk - nij] * at[ijk - nij]);
  }
};

// IC/ILU forward: z = (r + aw zW + as zS + ab zB) d  (iccg.f90:96-97, cgstab.f90:123-124)
struct DiagFwdOp {
  const double *r, *aw, *as, *ab, *dg;
  double* z;
  int nj, nij;
  __device__ void operator()(int ijk) const {
    z[ijk] = (r[ijk] + aw[ijk] * z[ijk - nj] + as[ijk] * z[ijk - 1] + ab[ijk] * z[ijk - nij]) * dg[ijk];
  }
};

// IC/ILU backward: z = (z + ae zE + an zN + at zT) d  (iccg.f90:118-119, cgstab.f90:144-145)
struct DiagBwdOp {
  const double *ae, *an, *at, *dg;
  double* z;
  int nj, nij;
  __device__ void operator()(int ijk) const {
    z[ijk] = (z[ijk] + ae[ijk] * z[ijk + nj] + an[ijk] * z[ijk + 1] + at[ijk] * z[ijk + nij]) * dg[ijk];
  }
};

template <class Op>
__global__ void k_plane(Op op, Dims d, Box b, int s) {
  int ni_ = b.i1 - b.i0 + 1;
  int nk_ = b.k1 - b.k0 + 1;
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ni_ * nk_) return;
  int i = b.i0 + t % ni_;
  int k = b.k0 + t / ni_;
  int j = s - i - k;
  if (j < b.j0 || j > b.j1) return;
  op(ixk(d, i, j, k));
}

// Run op over box b in hyperplane order (ascending for forward recurrences,
// descending for backward ones): one launch per plane.
template <class Op>
int wavefront(const Op& op, const Box& b, bool backward) {
  Ctx& c = ctx();
  int smin = b.i0 + b.j0 + b.k0, smax = b.i1 + b.j1 + b.k1;
  int n = (b.i1 - b.i0 + 1) * (b.k1 - b.k0 + 1);
  int grid = (n + 127) / 128;
  for (int q = 0; q <= smax - smin; ++q) {
    int s = backward ? smax - q : smin + q;
    launch(k_plane<Op>, grid, 128, c.st, op, c.d, b, s);
  }
  CAP_CHECK_LAUNCH();
  return CAPPGPU_OK;
}

}  // namespace cap
