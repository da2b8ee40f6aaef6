// solvers.cu -- the reference's 7-diagonal linear solvers on the device:
// sipsol (sipsol.f90), pcgsip (pcg-sip.f90), iccg (iccg.f90), cgstab
// (cgstab.f90), cgstab_sip (cgstab_sip.f90) and the Jacobi-preconditioned
// CG (pcg-jacobi.f90).  Recurrences run as hyperplane wavefronts
// (wavefront.cuh); streaming passes are box kernels with deterministic
// block reductions in place of the reference's serial sums and
// MPI_ALLREDUCE calls.
#include <math.h>

#include "common.cuh"
#include "kernels.cuh"
#include "wavefront.cuh"

namespace cap {

struct Coef {
  const double *ae, *aw, *an, *as, *at, *ab, *ap, *su;
};

static Coef coef() {
  double** F = ctx().f;
  return Coef{F[CAP_AE], F[CAP_AW], F[CAP_AN], F[CAP_AS], F[CAP_AT], F[CAP_AB], F[CAP_AP], F[CAP_SU]};
}

#define BOX_LOOP(b)                                                                              \
  for (long long t_ = blockIdx.x * (long long)blockDim.x + threadIdx.x, n_ = (b).count(); t_ < n_; \
       t_ += (long long)gridDim.x * blockDim.x)

// res = su + sum a_nb fi_nb - ap fi over box; partial sum |res|
// (pcg-sip.f90:48-59)
__global__ void k_resid(Dims d, Box b, Coef A, const double* __restrict__ fi, double* res, double* part) {
  double v[1] = {0.0};
  BOX_LOOP(b) {
    int i, j, k;
    b.at(t_, i, j, k);
    int ijk = ixk(d, i, j, k);
    double r = A.ae[ijk] * fi[ijk + d.nj] + A.aw[ijk] * fi[ijk - d.nj] + A.an[ijk] * fi[ijk + 1] +
               A.as[ijk] * fi[ijk - 1] + A.at[ijk] * fi[ijk + d.nij] + A.ab[ijk] * fi[ijk - d.nij] + A.su[ijk] -
               A.ap[ijk] * fi[ijk];
    res[ijk] = r;
    v[0] += fabs(r);
  }
  block_reduce_store<1>(v, part);
}

// z = A p (pcg-sip.f90:147-149); partial sum p.z
__global__ void k_spmv(Dims d, Box b, Coef A, const double* __restrict__ p, double* z, double* part) {
  double v[1] = {0.0};
  BOX_LOOP(b) {
    int i, j, k;
    b.at(t_, i, j, k);
    int ijk = ixk(d, i, j, k);
    double r = A.ap[ijk] * p[ijk] - A.ae[ijk] * p[ijk + d.nj] - A.aw[ijk] * p[ijk - d.nj] - A.an[ijk] * p[ijk + 1] -
               A.as[ijk] * p[ijk - 1] - A.at[ijk] * p[ijk + d.nij] - A.ab[ijk] * p[ijk - d.nij];
    z[ijk] = r;
    if (part) v[0] += p[ijk] * r;
  }
  if (part) block_reduce_store<1>(v, part);
}

// partial sums of a.b (and optionally c.e)
__global__ void k_dot(Dims d, Box b, const double* __restrict__ a, const double* __restrict__ bb,
                      const double* __restrict__ c2, const double* __restrict__ e2, double* part) {
  double v[2] = {0.0, 0.0};
  BOX_LOOP(b) {
    int i, j, k;
    b.at(t_, i, j, k);
    int ijk = ixk(d, i, j, k);
    v[0] += a[ijk] * bb[ijk];
    if (c2) v[1] += c2[ijk] * e2[ijk];
  }
  block_reduce_store<2>(v, part);
}

// pk = zk + bet pk (pcg-sip.f90:135)
__global__ void k_pk(Dims d, Box b, const double* __restrict__ zk, double* pk, double bet) {
  BOX_LOOP(b) {
    int i, j, k;
    b.at(t_, i, j, k);
    int ijk = ixk(d, i, j, k);
    pk[ijk] = zk[ijk] + bet * pk[ijk];
  }
}

// fi += alf pk; res -= alf zk; partial sum |res| (pcg-sip.f90:167-171)
__global__ void k_update(Dims d, Box b, double* fi, double* res, const double* __restrict__ pk,
                         const double* __restrict__ zk, double alf, double* part) {
  double v[1] = {0.0};
  BOX_LOOP(b) {
    int i, j, k;
    b.at(t_, i, j, k);
    int ijk = ixk(d, i, j, k);
    fi[ijk] = fi[ijk] + alf * pk[ijk];
    double r = res[ijk] - alf * zk[ijk];
    res[ijk] = r;
    v[0] += fabs(r);
  }
  if (part) block_reduce_store<1>(v, part);
}

// zk = zk / (d + small)  (iccg.f90:106)
__global__ void k_divd(Dims d, Box b, double* zk, const double* __restrict__ dg) {
  BOX_LOOP(b) {
    int i, j, k;
    b.at(t_, i, j, k);
    int ijk = ixk(d, i, j, k);
    zk[ijk] = zk[ijk] / (dg[ijk] + CAP_SMALL);
  }
}

// zk = res/(ap+small); partial sum res.zk  (pcg-jacobi.f90:84-85)
__global__ void k_jacobi(Dims d, Box b, const double* __restrict__ res, const double* __restrict__ ap, double* zk,
                         double* part) {
  double v[1] = {0.0};
  BOX_LOOP(b) {
    int i, j, k;
    b.at(t_, i, j, k);
    int ijk = ixk(d, i, j, k);
    double z = res[ijk] / (ap[ijk] + CAP_SMALL);
    zk[ijk] = z;
    v[0] += res[ijk] * z;
  }
  block_reduce_store<1>(v, part);
}

// BiCGStab init: reso = res; pk = uk = zk = vk = 0 (cgstab.f90:72-82)
__global__ void k_bicg_init(Dims d, Box b, const double* __restrict__ res, double* reso, double* pk, double* uk,
                            double* zk, double* vk) {
  BOX_LOOP(b) {
    int i, j, k;
    b.at(t_, i, j, k);
    int ijk = ixk(d, i, j, k);
    reso[ijk] = res[ijk];
    pk[ijk] = 0.0; uk[ijk] = 0.0; zk[ijk] = 0.0; vk[ijk] = 0.0;
  }
}

// pk = res + om (pk - alf uk)  (cgstab.f90:108)
__global__ void k_bicg_pk(Dims d, Box b, const double* __restrict__ res, double* pk, const double* __restrict__ uk,
                          double om, double alf) {
  BOX_LOOP(b) {
    int i, j, k;
    b.at(t_, i, j, k);
    int ijk = ixk(d, i, j, k);
    pk[ijk] = res[ijk] + om * (pk[ijk] - alf * uk[ijk]);
  }
}

static int launch_red_grid() { return kRedBlocks; }

static int reduce_fetch(int nv, double* out) {
  int rc = finish_reduce(nv);
  if (rc) return rc;
  return fetch_reduce(nv, out);
}

static void fill(cappgpu_solve_report* rep, double res0, double resl, int iters, int status) {
  if (!rep) return;
  rep->res0 = res0; rep->resl = resl; rep->iters = iters; rep->status = status;
}

static SipFactorOp sip_factor_op() {
  Ctx& c = ctx();
  double** F = c.f;
  return SipFactorOp{F[CAP_AE], F[CAP_AW], F[CAP_AN], F[CAP_AS], F[CAP_AT], F[CAP_AB], F[CAP_AP],
                     F[CAP_BB], F[CAP_BW], F[CAP_BS], F[CAP_BP], F[CAP_BN], F[CAP_BE], F[CAP_BT],
                     c.prm.alfa, c.d.nj, c.d.nij};
}

static int finish_status(double resl, bool done, cappgpu_solve_report* rep) {
  if (!isfinite(resl)) {
    set_error("linear solver residual is not finite");
    if (rep) rep->status = CAPPGPU_E_NONFINITE;
    return CAPPGPU_E_NONFINITE;
  }
  return done ? CAPPGPU_OK : CAPPGPU_NOT_CONVERGED;
}

// ------------------------------------------------------------------ SIPSOL
// sipsol.f90:3-106
int sipsol(int fif, int ifi, cappgpu_solve_report* rep) {
  Ctx& c = ctx();
  if (c.wave_impl == 1 && c.d.nimm >= 4 && c.d.njmm >= 4 && c.d.nkmm >= 4)
    return c.fp32(2) ? sipsol_mixed(fif, ifi, rep) : sipsol_fast(fif, ifi, rep);
  const Dims& d = c.d;
  double** F = c.f;
  cappgpu_params& P = c.prm;
  Box b{3, d.nimm, 3, d.njmm, 3, d.nkmm};
  int rc = wavefront(sip_factor_op(), b, false);
  if (rc) return rc;
  int ns = P.nsw[ifi - 1];
  double res1 = 0.0, rsm = 0.0;
  int n = 0;
  bool done = false;
  SipFwdOp fwd{F[CAP_RES], F[CAP_BB], F[CAP_BW], F[CAP_BS], F[CAP_BP], F[CAP_RES], d.nj, d.nij};
  SipBwdOp bwd{F[CAP_BN], F[CAP_BE], F[CAP_BT], F[CAP_RES], F[fif], d.nj, d.nij};
  for (n = 1; n <= ns; ++n) {
    // residual pass (its values feed the recurrence below through res)
    launch(k_resid, launch_red_grid(), kThreads, c.st, d, b, coef(), F[fif], F[CAP_RES], c.partials);
    CAP_CHECK_LAUNCH();
    if ((rc = reduce_fetch(1, &res1))) return rc;
    if ((rc = wavefront(fwd, b, false))) return rc;
    if (n == 1) P.resor[ifi - 1] = res1;
    rsm = res1 / (P.resor[ifi - 1] + CAP_SMALL);
    if ((rc = wavefront(bwd, b, true))) return rc;
    if (!isfinite(res1)) break;
    if (rsm < P.sor[ifi - 1]) { done = true; break; }
  }
  CAP_CUDA(cudaStreamSynchronize(c.st));
  fill(rep, P.resor[ifi - 1], res1, done ? n : ns, done ? CAPPGPU_OK : CAPPGPU_NOT_CONVERGED);
  return finish_status(res1, done, rep);
}

// ------------------------------------------------------------------ PCGSIP
// pcg-sip.f90:3-200
int resid_natural(int fif, double* res0) {
  Ctx& c = ctx();
  const Dims& d = c.d;
  Box b{3, d.nimm, 3, d.njmm, 3, d.nkmm};
  launch(k_resid, kRedBlocks, kThreads, c.st, d, b, coef(), (const double*)c.f[fif], c.f[CAP_RES], c.partials);
  CAP_CHECK_LAUNCH();
  return reduce_fetch(1, res0);
}

// the same over i = 3..nimm, j = 3..njmm and k = k0..k1 (cgstab_sip.f90:45-57 takes k = 2..nkm)
int resid_natural_k(int fif, int k0, int k1, double* res0) {
  Ctx& c = ctx();
  const Dims& d = c.d;
  Box b{3, d.nimm, 3, d.njmm, k0, k1};
  launch(k_resid, kRedBlocks, kThreads, c.st, d, b, coef(), (const double*)c.f[fif], c.f[CAP_RES], c.partials);
  CAP_CHECK_LAUNCH();
  return reduce_fetch(1, res0);
}

int spmv_dot2_natural(const double* p, double* z, const double* r, double* out2) {
  Ctx& c = ctx();
  const Dims& d = c.d;
  Box b{3, d.nimm, 3, d.njmm, 3, d.nkmm};
  launch(k_spmv, kRedBlocks, kThreads, c.st, d, b, coef(), p, z, (double*)nullptr);
  launch(k_dot, kRedBlocks, kThreads, c.st, d, b, r, (const double*)z, (const double*)z, (const double*)z, c.partials);
  CAP_CHECK_LAUNCH();
  return reduce_fetch(2, out2);
}

int dot2_natural(const double* a1, const double* b1, const double* a2, const double* b2, double* out2) {
  Ctx& c = ctx();
  const Dims& d = c.d;
  Box b{3, d.nimm, 3, d.njmm, 3, d.nkmm};
  launch(k_dot, kRedBlocks, kThreads, c.st, d, b, a1, b1, a2, b2, c.partials);
  CAP_CHECK_LAUNCH();
  return reduce_fetch(2, out2);
}

int resid_into(const double* fi, double* res, double* l1) {
  Ctx& c = ctx();
  const Dims& d = c.d;
  Box b{3, d.nimm, 3, d.njmm, 3, d.nkmm};
  launch(k_resid, kRedBlocks, kThreads, c.st, d, b, coef(), fi, res, c.partials);
  CAP_CHECK_LAUNCH();
  return reduce_fetch(1, l1);
}

int pcgsip(int fif, int ifi, cappgpu_solve_report* rep) {
  Ctx& c = ctx();
  if (c.wave_impl == 1 && c.d.nimm >= 4 && c.d.njmm >= 4 && c.d.nkmm >= 4)
    return c.fp32(1) ? pcgsip_mixed(fif, ifi, rep) : pcgsip_fast(fif, ifi, rep);
  const Dims& d = c.d;
  double** F = c.f;
  cappgpu_params& P = c.prm;
  size_t nb = sizeof(double) * d.nijk;
  double *pk = c.work[0], *zk = c.work[1], *res = F[CAP_RES], *fi = F[fif];
  double resmax = P.sor[ifi - 1];
  CAP_CUDA(cudaMemsetAsync(pk, 0, nb, c.st));
  CAP_CUDA(cudaMemsetAsync(zk, 0, nb, c.st));
  CAP_CUDA(cudaMemsetAsync(res, 0, nb, c.st));
  Box b{3, d.nimm, 3, d.njmm, 3, d.nkmm};
  int rc;
  launch(k_resid, launch_red_grid(), kThreads, c.st, d, b, coef(), fi, res, c.partials);
  CAP_CHECK_LAUNCH();
  double res0;
  if ((rc = reduce_fetch(1, &res0))) return rc;
  if ((rc = wavefront(sip_factor_op(), b, false))) return rc;
  double s0 = (double)1.e20f, sk, pkapk, alf, bet, resl = 0.0, rsm;
  int ns = P.nsw[ifi - 1], l;
  bool done = false;
  SipFwdOp fwd{res, F[CAP_BB], F[CAP_BW], F[CAP_BS], F[CAP_BP], zk, d.nj, d.nij};
  SipBwdOp bwd{F[CAP_BN], F[CAP_BE], F[CAP_BT], zk, nullptr, d.nj, d.nij};
  for (l = 1; l <= ns; ++l) {
    if ((rc = wavefront(fwd, b, false))) return rc;
    if ((rc = wavefront(bwd, b, true))) return rc;
    launch(k_dot, launch_red_grid(), kThreads, c.st, d, b, res, zk, nullptr, nullptr, c.partials);
    CAP_CHECK_LAUNCH();
    if ((rc = reduce_fetch(1, &sk))) return rc;
    bet = sk / s0;
    launch(k_pk, grid_for(b.count()), kThreads, c.st, d, b, zk, pk, bet);
    launch(k_spmv, launch_red_grid(), kThreads, c.st, d, b, coef(), pk, zk, c.partials);
    CAP_CHECK_LAUNCH();
    if ((rc = reduce_fetch(1, &pkapk))) return rc;
    alf = sk / pkapk;
    launch(k_update, launch_red_grid(), kThreads, c.st, d, b, fi, res, pk, zk, alf, c.partials);
    CAP_CHECK_LAUNCH();
    if ((rc = reduce_fetch(1, &resl))) return rc;
    s0 = sk;
    if (l == 1) P.resor[ifi - 1] = res0;
    rsm = resl / (P.resor[ifi - 1] + CAP_SMALL);
    if (!isfinite(resl)) break;
    if (rsm < resmax) { done = true; break; }
  }
  fill(rep, res0, resl, done ? l : ns, done ? CAPPGPU_OK : CAPPGPU_NOT_CONVERGED);
  return finish_status(resl, done, rep);
}

// -------------------------------------------------------------------- ICCG
// iccg.f90:3-197
int iccg(int fif, int ifi, cappgpu_solve_report* rep) {
  Ctx& c = ctx();
  if (c.wave_impl == 1 && c.d.nimm >= 4 && c.d.njmm >= 4 && c.d.nkmm >= 4) return iccg_fast(fif, ifi, rep);
  const Dims& d = c.d;
  double** F = c.f;
  cappgpu_params& P = c.prm;
  size_t nb = sizeof(double) * d.nijk;
  double *pk = c.work[0], *zk = c.work[1], *dg = c.work[2], *res = F[CAP_RES], *fi = F[fif];
  double resmax = P.sor[ifi - 1];
  CAP_CUDA(cudaMemsetAsync(pk, 0, nb, c.st));
  CAP_CUDA(cudaMemsetAsync(zk, 0, nb, c.st));
  CAP_CUDA(cudaMemsetAsync(dg, 0, nb, c.st));
  CAP_CUDA(cudaMemsetAsync(res, 0, nb, c.st));
  Box b{3, d.nimm, 3, d.njmm, 2, d.nkm};
  int rc;
  launch(k_resid, launch_red_grid(), kThreads, c.st, d, b, coef(), fi, res, c.partials);
  CAP_CHECK_LAUNCH();
  double res0;
  if ((rc = reduce_fetch(1, &res0))) return rc;
  IccgDiagOp dop{F[CAP_AP], F[CAP_AW], F[CAP_AS], F[CAP_AB], dg, d.nj, d.nij};
  if ((rc = wavefront(dop, b, false))) return rc;
  double s0 = (double)1.e20f, sk, pkapk, alf, bet, resl = 0.0, rsm;
  int ns = P.nsw[ifi - 1], l;
  bool done = false;
  DiagFwdOp fwd{res, F[CAP_AW], F[CAP_AS], F[CAP_AB], dg, zk, d.nj, d.nij};
  DiagBwdOp bwd{F[CAP_AE], F[CAP_AN], F[CAP_AT], dg, zk, d.nj, d.nij};
  for (l = 1; l <= ns; ++l) {
    if ((rc = wavefront(fwd, b, false))) return rc;
    launch(k_divd, grid_for(b.count()), kThreads, c.st, d, b, zk, dg);
    CAP_CHECK_LAUNCH();
    if ((rc = wavefront(bwd, b, true))) return rc;
    launch(k_dot, launch_red_grid(), kThreads, c.st, d, b, res, zk, nullptr, nullptr, c.partials);
    CAP_CHECK_LAUNCH();
    if ((rc = reduce_fetch(1, &sk))) return rc;
    bet = sk / s0;
    launch(k_pk, grid_for(b.count()), kThreads, c.st, d, b, zk, pk, bet);
    launch(k_spmv, launch_red_grid(), kThreads, c.st, d, b, coef(), pk, zk, c.partials);
    CAP_CHECK_LAUNCH();
    if ((rc = reduce_fetch(1, &pkapk))) return rc;
    alf = sk / pkapk;
    launch(k_update, launch_red_grid(), kThreads, c.st, d, b, fi, res, pk, zk, alf, c.partials);
    CAP_CHECK_LAUNCH();
    if ((rc = reduce_fetch(1, &resl))) return rc;
    s0 = sk;
    if (l == 1) P.resor[ifi - 1] = res0;
    rsm = resl / (P.resor[ifi - 1] + CAP_SMALL);
    if (!isfinite(resl)) break;
    if (rsm < resmax) { done = true; break; }
  }
  fill(rep, res0, resl, done ? l : ns, done ? CAPPGPU_OK : CAPPGPU_NOT_CONVERGED);
  return finish_status(resl, done, rep);
}

// ---------------------------------------------------------- BiCGStab family
// cgstab.f90:3-283 (sip=false) and cgstab_sip.f90:3-279 (sip=true).  The
// reference's automatic work arrays are undefined outside the loop box;
// here they are zero there (work vectors are cleared first).
int bicgstab(int fif, int ifi, bool sip, cappgpu_solve_report* rep) {
  Ctx& c = ctx();
  if (sip && c.wave_impl == 1 && c.d.nimm >= 4 && c.d.njmm >= 4 && c.d.nkmm >= 4)
    return cgstab_sip_fast(fif, ifi, rep);
  const Dims& d = c.d;
  double** F = c.f;
  cappgpu_params& P = c.prm;
  size_t nb = sizeof(double) * d.nijk;
  double *reso = c.work[0], *pk = c.work[1], *uk = c.work[2], *zk = c.work[3], *vk = c.work[4], *dg = c.work[5];
  double *res = F[CAP_RES], *fi = F[fif];
  for (double* w : {reso, pk, uk, zk, vk, dg}) CAP_CUDA(cudaMemsetAsync(w, 0, nb, c.st));
  double resmax = P.sor[ifi - 1];
  Box b{3, d.nimm, 3, d.njmm, 2, d.nkm};
  int rc;
  launch(k_resid, launch_red_grid(), kThreads, c.st, d, b, coef(), fi, res, c.partials);
  CAP_CHECK_LAUNCH();
  double res0;
  if ((rc = reduce_fetch(1, &res0))) return rc;
  if (sip) {
    if ((rc = wavefront(sip_factor_op(), b, false))) return rc;
  } else {
    IluDiagOp dop{F[CAP_AP], F[CAP_AW], F[CAP_AS], F[CAP_AB], F[CAP_AE], F[CAP_AN], F[CAP_AT], dg, d.nj, d.nij};
    if ((rc = wavefront(dop, b, false))) return rc;
  }
  launch(k_bicg_init, grid_for(b.count()), kThreads, c.st, d, b, res, reso, pk, uk, zk, vk);
  CAP_CHECK_LAUNCH();
  double alf = 1.0, beto = 1.0, gam = 1.0, bet, om, ukreso, vres, vv, resl = 0.0, rsm, red[2];
  int ns = P.nsw[ifi - 1], l;
  bool done = false;
  // second backward substitution box: cgstab.f90:212 uses k=nkmm..3,
  // cgstab_sip.f90:207 uses k=nkm..2
  Box b2 = b;
  if (!sip) { b2.k0 = 3; b2.k1 = d.nkmm; }
  auto precond = [&](const double* rhs, const Box& bb2) -> int {
    int r;
    if (sip) {
      SipFwdOp f{rhs, F[CAP_BB], F[CAP_BW], F[CAP_BS], F[CAP_BP], zk, d.nj, d.nij};
      SipBwdOp g{F[CAP_BN], F[CAP_BE], F[CAP_BT], zk, nullptr, d.nj, d.nij};
      if ((r = wavefront(f, b, false))) return r;
      return wavefront(g, bb2, true);
    }
    DiagFwdOp f{rhs, F[CAP_AW], F[CAP_AS], F[CAP_AB], dg, zk, d.nj, d.nij};
    DiagBwdOp g{F[CAP_AE], F[CAP_AN], F[CAP_AT], dg, zk, d.nj, d.nij};
    if ((r = wavefront(f, b, false))) return r;
    launch(k_divd, grid_for(b.count()), kThreads, c.st, d, b, zk, dg);
    CAP_CHECK_LAUNCH();
    return wavefront(g, bb2, true);
  };
  for (l = 1; l <= ns; ++l) {
    launch(k_dot, launch_red_grid(), kThreads, c.st, d, b, res, reso, nullptr, nullptr, c.partials);
    CAP_CHECK_LAUNCH();
    if ((rc = reduce_fetch(1, &bet))) return rc;
    om = bet * gam / (alf * beto + CAP_SMALL);
    beto = bet;
    launch(k_bicg_pk, grid_for(b.count()), kThreads, c.st, d, b, res, pk, uk, om, alf);
    CAP_CHECK_LAUNCH();
    if ((rc = precond(pk, b))) return rc;
    launch(k_spmv, launch_red_grid(), kThreads, c.st, d, b, coef(), zk, uk, nullptr);
    launch(k_dot, launch_red_grid(), kThreads, c.st, d, b, uk, reso, nullptr, nullptr, c.partials);
    CAP_CHECK_LAUNCH();
    if ((rc = reduce_fetch(1, &ukreso))) return rc;
    gam = bet / ukreso;
    launch(k_update, launch_red_grid(), kThreads, c.st, d, b, fi, res, zk, uk, gam, nullptr);
    CAP_CHECK_LAUNCH();
    if ((rc = precond(res, b2))) return rc;
    launch(k_spmv, launch_red_grid(), kThreads, c.st, d, b, coef(), zk, vk, nullptr);
    launch(k_dot, launch_red_grid(), kThreads, c.st, d, b, vk, res, vk, vk, c.partials);
    CAP_CHECK_LAUNCH();
    if ((rc = reduce_fetch(2, red))) return rc;
    vres = red[0];
    vv = red[1];
    alf = vres / (vv + CAP_SMALL);
    launch(k_update, launch_red_grid(), kThreads, c.st, d, b, fi, res, zk, vk, alf, c.partials);
    CAP_CHECK_LAUNCH();
    if ((rc = reduce_fetch(1, &resl))) return rc;
    if (l == 1) P.resor[ifi - 1] = res0;
    rsm = resl / (P.resor[ifi - 1] + CAP_SMALL);
    if (!isfinite(resl)) break;
    if (rsm < resmax) { done = true; break; }
  }
  fill(rep, res0, resl, done ? l : ns, done ? CAPPGPU_OK : CAPPGPU_NOT_CONVERGED);
  return finish_status(resl, done, rep);
}

// -------------------------------------------------------------------- DPCG
// pcg-jacobi.f90:3-155
int dpcg(int fif, int ifi, cappgpu_solve_report* rep) {
  Ctx& c = ctx();
  const Dims& d = c.d;
  double** F = c.f;
  cappgpu_params& P = c.prm;
  size_t nb = sizeof(double) * d.nijk;
  double *pk = c.work[0], *zk = c.work[1], *res = F[CAP_RES], *fi = F[fif];
  CAP_CUDA(cudaMemsetAsync(pk, 0, nb, c.st));
  CAP_CUDA(cudaMemsetAsync(zk, 0, nb, c.st));
  CAP_CUDA(cudaMemsetAsync(res, 0, nb, c.st));
  double resmax = P.sor[ifi - 1];
  Box b{3, d.nimm, 3, d.njmm, 3, d.nkmm};
  int rc;
  launch(k_resid, launch_red_grid(), kThreads, c.st, d, b, coef(), fi, res, c.partials);
  CAP_CHECK_LAUNCH();
  double res0;
  if ((rc = reduce_fetch(1, &res0))) return rc;
  double s0 = (double)1.e20f, sk, pkapk, alf, bet, resl = 0.0, rsm;
  int ns = P.nsw[ifi - 1], l;
  bool done = false;
  for (l = 1; l <= ns; ++l) {
    launch(k_jacobi, launch_red_grid(), kThreads, c.st, d, b, res, F[CAP_AP], zk, c.partials);
    CAP_CHECK_LAUNCH();
    if ((rc = reduce_fetch(1, &sk))) return rc;
    bet = sk / s0;
    launch(k_pk, grid_for(b.count()), kThreads, c.st, d, b, zk, pk, bet);
    launch(k_spmv, launch_red_grid(), kThreads, c.st, d, b, coef(), pk, zk, c.partials);
    CAP_CHECK_LAUNCH();
    if ((rc = reduce_fetch(1, &pkapk))) return rc;
    alf = sk / pkapk;
    launch(k_update, launch_red_grid(), kThreads, c.st, d, b, fi, res, pk, zk, alf, c.partials);
    CAP_CHECK_LAUNCH();
    if ((rc = reduce_fetch(1, &resl))) return rc;
    s0 = sk;
    if (l == 1) P.resor[ifi - 1] = res0;
    rsm = resl / (P.resor[ifi - 1] + CAP_SMALL);
    if (!isfinite(resl)) break;
    if (rsm < resmax) { done = true; break; }
  }
  fill(rep, res0, resl, done ? l : ns, done ? CAPPGPU_OK : CAPPGPU_NOT_CONVERGED);
  return finish_status(resl, done, rep);
}

static int solve_dispatch(int solver, int fi, int ifi, cappgpu_solve_report* rep) {
  switch (solver) {
    case CAPPGPU_SOLVER_SIPSOL: return sipsol(fi, ifi, rep);
    case CAPPGPU_SOLVER_CGSTAB: return bicgstab(fi, ifi, false, rep);
    case CAPPGPU_SOLVER_ICCG: return iccg(fi, ifi, rep);
    case CAPPGPU_SOLVER_PCGSIP: return pcgsip(fi, ifi, rep);
    case CAPPGPU_SOLVER_CGSTAB_SIP: return bicgstab(fi, ifi, true, rep);
    case CAPPGPU_SOLVER_DPCG: return dpcg(fi, ifi, rep);
    default: set_error("unknown solver %d", solver); return CAPPGPU_E_ARG;
  }
}

// every solve through the selector records its report (cappgpu_last_report)
int solve(int solver, int fi, int ifi, cappgpu_solve_report* rep) {
  cappgpu_solve_report r{};
  const int rc = solve_dispatch(solver, fi, ifi, &r);
  Ctx& c = ctx();
  c.last_rep = r;
  c.last_solver = solver;
  c.last_ifi = ifi;
  if (rep) *rep = r;
  return rc;
}

static int check_solver_args(int fi, int ifi) {
  CAP_REQUIRE_INIT();
  if (fi < 0 || fi >= CAP_NFIELDS || ifi < 1 || ifi > CAP_NPHI) {
    set_error("solver: bad field %d or ifi %d", fi, ifi);
    return CAPPGPU_E_ARG;
  }
  return CAPPGPU_OK;
}

// Host-pointer drop-in: fi must be registered; the registered host arrays
// of the matrix (ae..ap, su) and fi are copied in, fi and res copied back.
static int solve_h(int solver, double* fi, int ifi) {
  CAP_REQUIRE_INIT();
  Ctx& c = ctx();
  int fid = -1;
  for (int q = 0; q < CAP_NFIELDS; ++q)
    if (c.host_reg[q] && c.host_reg[q] == fi) fid = q;
  if (fid < 0) { set_error("solver_h: fi is not a registered host array"); return CAPPGPU_E_ARG; }
  const int ins[] = {CAP_AE, CAP_AW, CAP_AN, CAP_AS, CAP_AT, CAP_AB, CAP_AP, CAP_SU,
                     CAP_BB, CAP_BS, CAP_BW, CAP_BP, CAP_BN, CAP_BE, CAP_BT, CAP_RES};
  size_t nb = sizeof(double) * c.d.nijk;
  for (int q : ins)
    if (c.host_reg[q]) CAP_CUDA(cudaMemcpyAsync(c.f[q], c.host_reg[q], nb, cudaMemcpyHostToDevice, c.st));
  note_write(fid);
  CAP_CUDA(cudaMemcpyAsync(c.f[fid], fi, nb, cudaMemcpyHostToDevice, c.st));
  cappgpu_solve_report rep;
  int rc = solve(solver, fid, ifi, &rep);
  if (rc < 0) return rc;
  CAP_CUDA(cudaMemcpyAsync(fi, c.f[fid], nb, cudaMemcpyDeviceToHost, c.st));
  const int outs[] = {CAP_RES, CAP_BB, CAP_BS, CAP_BW, CAP_BP, CAP_BN, CAP_BE, CAP_BT};
  for (int q : outs)
    if (c.host_reg[q]) CAP_CUDA(cudaMemcpyAsync(c.host_reg[q], c.f[q], nb, cudaMemcpyDeviceToHost, c.st));
  CAP_CUDA(cudaStreamSynchronize(c.st));
  return rc;
}

}  // namespace cap

using namespace cap;

extern "C" {

#define SOLVER_ENTRY(name, id)                                                 \
  int cappgpu_##name(int fi, int ifi, cappgpu_solve_report* rep) {            \
    int rc = check_solver_args(fi, ifi);                                        \
    if (rc) return rc;                                                          \
    rc = solve(id, fi, ifi, rep);                                               \
    cudaError_t e = cudaStreamSynchronize(ctx().st);                            \
    if (e != cudaSuccess) return cuda_fail(e, #name, __FILE__, __LINE__);       \
    return rc;                                                                  \
  }                                                                             \
  int cappgpu_##name##_h(double* fi, int ifi) { return solve_h(id, fi, ifi); }

SOLVER_ENTRY(sipsol, CAPPGPU_SOLVER_SIPSOL)
SOLVER_ENTRY(pcgsip, CAPPGPU_SOLVER_PCGSIP)
SOLVER_ENTRY(iccg, CAPPGPU_SOLVER_ICCG)
SOLVER_ENTRY(cgstab, CAPPGPU_SOLVER_CGSTAB)
SOLVER_ENTRY(cgstab_sip, CAPPGPU_SOLVER_CGSTAB_SIP)
SOLVER_ENTRY(dpcg, CAPPGPU_SOLVER_DPCG)

int cappgpu_spmv(int pk, int zk, double* dot) {
  CAP_REQUIRE_INIT();
  if (pk < 0 || pk >= CAP_NFIELDS || zk < 0 || zk >= CAP_NFIELDS || pk == zk || !spmv_output_ok(zk)) {
    set_error("spmv: bad fields %d %d (zk may not be a matrix coefficient or a geometry field)", pk, zk);
    return CAPPGPU_E_ARG;
  }
  Ctx& c = ctx();
  const Dims& d = c.d;
  Box b{3, d.nimm, 3, d.njmm, 3, d.nkmm};
  launch(k_spmv, kRedBlocks, kThreads, c.st, d, b, coef(), c.f[pk], c.f[zk], c.partials);
  CAP_CHECK_LAUNCH();
  double v;
  int rc = reduce_fetch(1, &v);
  if (rc) return rc;
  if (dot) *dot = v;
  return CAPPGPU_OK;
}

}  // extern "C"

namespace cap {

// One hot-path unit for cappgpu_profile_kernel; *bytes = its algorithmic
// HBM traffic: words per interior cell x 8 bytes x interior cells
// (res,bb,bw,bs,bp -> z: 6 words; z,bn,be,bt -> z: 5; ap..ab,p -> z: 9;
// grad_gauss 17; fluxuvw one direction 35; piso assembly one direction 30;
// SIP factorisation 14).
int profile_unit(int which, double* bytes) {
  Ctx& c = ctx();
  const Dims& d = c.d;
  double** F = c.f;
  Box b{3, d.nimm, 3, d.njmm, 3, d.nkmm};
  double cells = (double)b.count();
  double* zk = c.work[1];
  double* pk = c.work[0];
  if (which == 9 || which == 10) return learned_profile_unit(which, bytes);
  if (which == 7 || which == 8) {
    if (d.nimm < 4 || d.njmm < 4 || d.nkmm < 4) { set_error("profile unit %d needs 2 interior cells per axis", which); return CAPPGPU_E_ARG; }
    return fast_profile_unit(which, bytes);
  }
  if (c.wave_impl == 1 && (which == 0 || which == 1 || which == 6)) return fast_profile_unit(which, bytes);
  switch (which) {
    case 0: {
      SipFwdOp fwd{F[CAP_RES], F[CAP_BB], F[CAP_BW], F[CAP_BS], F[CAP_BP], zk, d.nj, d.nij};
      *bytes = 6.0 * 8.0 * cells;
      return wavefront(fwd, b, false);
    }
    case 1: {
      SipBwdOp bwd{F[CAP_BN], F[CAP_BE], F[CAP_BT], zk, nullptr, d.nj, d.nij};
      *bytes = 5.0 * 8.0 * cells;
      return wavefront(bwd, b, true);
    }
    case 2:
      *bytes = 9.0 * 8.0 * cells;
      launch(k_spmv, kRedBlocks, kThreads, c.st, d, b, coef(), (const double*)pk, zk, c.partials);
      CAP_CHECK_LAUNCH();
      return finish_reduce(1);
    case 3:
      *bytes = 17.0 * 8.0 * cells;
      return grad_gauss(CAP_U, CAP_GRADU_X, CAP_GRADU_Y, CAP_GRADU_Z);
    case 4:
      *bytes = 35.0 * 8.0 * cells;
      return fluxuvw(d.nj, 1, d.nij, CAP_AR1X, CAP_AR1Y, CAP_AR1Z, CAP_FX, CAP_AE, CAP_AW, CAP_F1);
    case 5:
      *bytes = 30.0 * 8.0 * cells;
      return piso_assemble(d.nj, 1, d.nij, CAP_AR1X, CAP_AR1Y, CAP_AR1Z, CAP_FX, CAP_AE, CAP_AW, CAP_F1, 1, CAP_BE);
    default:
      *bytes = 14.0 * 8.0 * cells;
      return wavefront(sip_factor_op(), b, false);
  }
}

}  // namespace cap
