/*
 * oracle_solvers.c -- 7-diagonal linear solvers of the reference, restated
 * line by line (TEST INFRASTRUCTURE ONLY; pinned against the reference's
 * own routines, see oracle.h).
 *
 * Work arrays that the reference declares as automatic arrays of size
 * nxyza (e.g. pk,zk in pcg-sip.f90:33) are allocated here with nijk
 * elements.  Where the reference zeroes them (pk=0, zk=0) so does the
 * oracle; where it leaves parts of them undefined (cgstab.f90:69-92 sets
 * only k=2..nkm,i=3..nimm,j=3..njmm) the oracle zero-fills the rest, which
 * is the only defined reading of the reference.
 */
#include "oracle.h"
#include "oracle_internal.h"

#include <stdlib.h>
#include <string.h>
#include <math.h>

static double* zalloc(int n) { return (double*)calloc((size_t)n, sizeof(double)); }

/* residual res = su + sum(a_nb*fi_nb) - ap*fi, e.g. pcg-sip.f90:49-57 */
#define RESID(ijk)                                                                        \
  (ae[ijk] * fi[(ijk) + nj] + aw[ijk] * fi[(ijk) - nj] + an[ijk] * fi[(ijk) + 1] +          \
   as[ijk] * fi[(ijk) - 1] + at[ijk] * fi[(ijk) + nij] + ab[ijk] * fi[(ijk) - nij] + su[ijk] - \
   ap[ijk] * fi[ijk])

/* 7-point product z = A p, pcg-sip.f90:143-155 */
#define APROD(p, ijk)                                                                     \
  (ap[ijk] * p[ijk] - ae[ijk] * p[(ijk) + nj] - aw[ijk] * p[(ijk) - nj] - an[ijk] * p[(ijk) + 1] - \
   as[ijk] * p[(ijk) - 1] - at[ijk] * p[(ijk) + nij] - ab[ijk] * p[(ijk) - nij])

#define COEF_PTRS                                                                         \
  const double *ae = s->f[CAP_AE], *aw = s->f[CAP_AW], *an = s->f[CAP_AN];                  \
  const double *as = s->f[CAP_AS], *at = s->f[CAP_AT], *ab = s->f[CAP_AB];                  \
  const double *ap = s->f[CAP_AP], *su = s->f[CAP_SU];                                      \
  const int nj = s->nj, nij = s->nij;                                                       \
  (void)nj; (void)nij; (void)su

#define SIP_PTRS                                                                          \
  double *bb = s->f[CAP_BB], *bs = s->f[CAP_BS], *bw = s->f[CAP_BW], *bp = s->f[CAP_BP];    \
  double *bn = s->f[CAP_BN], *be = s->f[CAP_BE], *bt = s->f[CAP_BT]

/* SIP incomplete factorisation over k=k0..k1, i=3..nimm, j=3..njmm
   (sipsol.f90:28-50; pcg-sip.f90:68-87; cgstab_sip.f90:60-79). */
static void sip_factor(cap_state* s, int k0, int k1) {
  COEF_PTRS;
  SIP_PTRS;
  const double alfa = s->prm.alfa;
  for (int k = k0; k <= k1; ++k)
    for (int i = 3; i <= s->nimm; ++i)
      for (int j = 3; j <= s->njmm; ++j) {
        int ijk = IXK(i, j, k);
        bb[ijk] = -ab[ijk] / (1.0 + alfa * (bn[ijk - nij] + be[ijk - nij]));
        bw[ijk] = -aw[ijk] / (1.0 + alfa * (bn[ijk - nj] + bt[ijk - nj]));
        bs[ijk] = -as[ijk] / (1.0 + alfa * (be[ijk - 1] + bt[ijk - 1]));
        double p1 = alfa * (bb[ijk] * bn[ijk - nij] + bw[ijk] * bn[ijk - nj]);
        double p2 = alfa * (bb[ijk] * be[ijk - nij] + bs[ijk] * be[ijk - 1]);
        double p3 = alfa * (bw[ijk] * bt[ijk - nj] + bs[ijk] * bt[ijk - 1]);
        bp[ijk] = 1.0 / (ap[ijk] + p1 + p2 + p3 - bb[ijk] * bt[ijk - nij] - bw[ijk] * be[ijk - nj] -
                         bs[ijk] * bn[ijk - 1] + SMALL);
        bn[ijk] = (-an[ijk] - p1) * bp[ijk];
        be[ijk] = (-ae[ijk] - p2) * bp[ijk];
        bt[ijk] = (-at[ijk] - p3) * bp[ijk];
      }
}

static void fill_rep(cappgpu_solve_report* rep, double res0, double resl, int iters, int status) {
  if (!rep) return;
  rep->res0 = res0; rep->resl = resl; rep->iters = iters; rep->status = status;
}

/* ---------------------------------------------------------------- SIPSOL */
/* sipsol.f90:3-106 */
int cap_sipsol(cap_state* s, int fif, int ifi, cappgpu_solve_report* rep) {
  COEF_PTRS;
  SIP_PTRS;
  double* fi = s->f[fif];
  double* res = s->f[CAP_RES];
  cappgpu_params* P = &s->prm;
  sip_factor(s, 3, s->nkmm);
  int ns = P->nsw[ifi - 1];
  double res1 = 0.0, rsm = 0.0;
  int n, done = 0;
  for (n = 1; n <= ns; ++n) {
    res1 = 0.0;
    for (int k = 3; k <= s->nkmm; ++k)
      for (int i = 3; i <= s->nimm; ++i)
        for (int j = 3; j <= s->njmm; ++j) {
          int ijk = IXK(i, j, k);
          res[ijk] = RESID(ijk);
          res1 = res1 + fabs(res[ijk]);
          res[ijk] = (res[ijk] - bb[ijk] * res[ijk - nij] - bw[ijk] * res[ijk - nj] -
                      bs[ijk] * res[ijk - 1]) * bp[ijk];
        }
    if (n == 1) P->resor[ifi - 1] = res1;
    rsm = res1 / (P->resor[ifi - 1] + SMALL);
    for (int k = s->nkmm; k >= 3; --k)
      for (int i = s->nimm; i >= 3; --i)
        for (int j = s->njmm; j >= 3; --j) {
          int ijk = IXK(i, j, k);
          res[ijk] = res[ijk] - bn[ijk] * res[ijk + 1] - be[ijk] * res[ijk + nj] - bt[ijk] * res[ijk + nij];
          fi[ijk] = fi[ijk] + res[ijk];
        }
    if (rsm < P->sor[ifi - 1]) { done = 1; break; }
  }
  int iters = done ? n : ns;
  fill_rep(rep, P->resor[ifi - 1], res1, iters, done ? CAPPGPU_OK : CAPPGPU_NOT_CONVERGED);
  if (!isfinite(res1)) { if (rep) rep->status = CAPPGPU_E_NONFINITE; return CAPPGPU_E_NONFINITE; }
  return done ? CAPPGPU_OK : CAPPGPU_NOT_CONVERGED;
}

/* ---------------------------------------------------------------- PCGSIP */
/* pcg-sip.f90:3-200 */
int cap_pcgsip(cap_state* s, int fif, int ifi, cappgpu_solve_report* rep) {
  COEF_PTRS;
  SIP_PTRS;
  double* fi = s->f[fif];
  double* res = s->f[CAP_RES];
  cappgpu_params* P = &s->prm;
  const int n = s->nijk;
  double* pk = zalloc(n);
  double* zk = zalloc(n);
  double resmax = P->sor[ifi - 1];
  memset(res, 0, sizeof(double) * n);
  double res0 = 0.0;
  for (int k = 3; k <= s->nkmm; ++k)
    for (int i = 3; i <= s->nimm; ++i)
      for (int j = 3; j <= s->njmm; ++j) {
        int ijk = IXK(i, j, k);
        res[ijk] = RESID(ijk);
        res0 = res0 + fabs(res[ijk]);
      }
  /* global_sum(res0): identity on one rank */
  sip_factor(s, 3, s->nkmm);
  double s0 = (double)1.e20f, sk, pkapk, alf, bet, resl = 0.0, rsm;
  int ns = P->nsw[ifi - 1], l, done = 0;
  for (l = 1; l <= ns; ++l) {
    for (int k = 3; k <= s->nkmm; ++k)
      for (int i = 3; i <= s->nimm; ++i)
        for (int j = 3; j <= s->njmm; ++j) {
          int ijk = IXK(i, j, k);
          zk[ijk] = (res[ijk] - bb[ijk] * zk[ijk - nij] - bw[ijk] * zk[ijk - nj] - bs[ijk] * zk[ijk - 1]) * bp[ijk];
        }
    sk = 0.0;
    for (int k = s->nkmm; k >= 3; --k)
      for (int i = s->nimm; i >= 3; --i)
        for (int j = s->njmm; j >= 3; --j) {
          int ijk = IXK(i, j, k);
          zk[ijk] = zk[ijk] - bn[ijk] * zk[ijk + 1] - be[ijk] * zk[ijk + nj] - bt[ijk] * zk[ijk + nij];
          sk = sk + res[ijk] * zk[ijk];
        }
    bet = sk / s0;
    for (int k = 3; k <= s->nkmm; ++k)
      for (int i = 3; i <= s->nimm; ++i)
        for (int j = 3; j <= s->njmm; ++j) {
          int ijk = IXK(i, j, k);
          pk[ijk] = zk[ijk] + bet * pk[ijk];
        }
    pkapk = 0.0;
    for (int k = 3; k <= s->nkmm; ++k)
      for (int i = 3; i <= s->nimm; ++i)
        for (int j = 3; j <= s->njmm; ++j) {
          int ijk = IXK(i, j, k);
          zk[ijk] = APROD(pk, ijk);
          pkapk = pkapk + pk[ijk] * zk[ijk];
        }
    alf = sk / pkapk;
    resl = 0.0;
    for (int k = 3; k <= s->nkmm; ++k)
      for (int i = 3; i <= s->nimm; ++i)
        for (int j = 3; j <= s->njmm; ++j) {
          int ijk = IXK(i, j, k);
          fi[ijk] = fi[ijk] + alf * pk[ijk];
          res[ijk] = res[ijk] - alf * zk[ijk];
          resl = resl + fabs(res[ijk]);
        }
    /* global_sum(resl); exchange(fi); exchange(res): identity on one rank */
    s0 = sk;
    if (l == 1) P->resor[ifi - 1] = res0;
    rsm = resl / (P->resor[ifi - 1] + SMALL);
    if (rsm < resmax) { done = 1; break; }
  }
  free(pk); free(zk);
  int iters = done ? l : ns;
  fill_rep(rep, res0, resl, iters, done ? CAPPGPU_OK : CAPPGPU_NOT_CONVERGED);
  if (!isfinite(resl)) { if (rep) rep->status = CAPPGPU_E_NONFINITE; return CAPPGPU_E_NONFINITE; }
  return done ? CAPPGPU_OK : CAPPGPU_NOT_CONVERGED;
}

/* ------------------------------------------------------------------ ICCG */
/* iccg.f90:3-197 */
int cap_iccg(cap_state* s, int fif, int ifi, cappgpu_solve_report* rep) {
  COEF_PTRS;
  double* fi = s->f[fif];
  double* res = s->f[CAP_RES];
  cappgpu_params* P = &s->prm;
  const int n = s->nijk;
  double *pk = zalloc(n), *zk = zalloc(n), *d = zalloc(n);
  double resmax = P->sor[ifi - 1];
  memset(res, 0, sizeof(double) * n);
  double res0 = 0.0;
  for (int k = 2; k <= s->nkm; ++k)
    for (int i = 3; i <= s->nimm; ++i)
      for (int j = 3; j <= s->njmm; ++j) {
        int ijk = IXK(i, j, k);
        res[ijk] = RESID(ijk);
        res0 = res0 + fabs(res[ijk]);
      }
  for (int k = 2; k <= s->nkm; ++k)
    for (int i = 3; i <= s->nimm; ++i)
      for (int j = 3; j <= s->njmm; ++j) {
        int ijk = IXK(i, j, k);
        d[ijk] = 1.0 / (ap[ijk] - aw[ijk] * aw[ijk] * d[ijk - nj] - as[ijk] * as[ijk] * d[ijk - 1] -
                        ab[ijk] * ab[ijk] * d[ijk - nij]);
      }
  double s0 = (double)1.e20f, sk, pkapk, alf, bet, resl = 0.0, rsm;
  int ns = P->nsw[ifi - 1], l, done = 0;
  for (l = 1; l <= ns; ++l) {
    for (int k = 2; k <= s->nkm; ++k)
      for (int i = 3; i <= s->nimm; ++i)
        for (int j = 3; j <= s->njmm; ++j) {
          int ijk = IXK(i, j, k);
          zk[ijk] = (res[ijk] + aw[ijk] * zk[ijk - nj] + as[ijk] * zk[ijk - 1] + ab[ijk] * zk[ijk - nij]) * d[ijk];
        }
    for (int k = 2; k <= s->nkm; ++k)
      for (int i = 3; i <= s->nimm; ++i)
        for (int j = 3; j <= s->njmm; ++j) {
          int ijk = IXK(i, j, k);
          zk[ijk] = zk[ijk] / (d[ijk] + SMALL);
        }
    sk = 0.0;
    for (int k = s->nkm; k >= 2; --k)
      for (int i = s->nimm; i >= 3; --i)
        for (int j = s->njmm; j >= 3; --j) {
          int ijk = IXK(i, j, k);
          zk[ijk] = (zk[ijk] + ae[ijk] * zk[ijk + nj] + an[ijk] * zk[ijk + 1] + at[ijk] * zk[ijk + nij]) * d[ijk];
          sk = sk + res[ijk] * zk[ijk];
        }
    bet = sk / s0;
    for (int k = 2; k <= s->nkm; ++k)
      for (int i = 3; i <= s->nimm; ++i)
        for (int j = 3; j <= s->njmm; ++j) {
          int ijk = IXK(i, j, k);
          pk[ijk] = zk[ijk] + bet * pk[ijk];
        }
    pkapk = 0.0;
    for (int k = 2; k <= s->nkm; ++k)
      for (int i = 3; i <= s->nimm; ++i)
        for (int j = 3; j <= s->njmm; ++j) {
          int ijk = IXK(i, j, k);
          zk[ijk] = APROD(pk, ijk);
          pkapk = pkapk + pk[ijk] * zk[ijk];
        }
    alf = sk / pkapk;
    resl = 0.0;
    for (int k = 2; k <= s->nkm; ++k)
      for (int i = 3; i <= s->nimm; ++i)
        for (int j = 3; j <= s->njmm; ++j) {
          int ijk = IXK(i, j, k);
          fi[ijk] = fi[ijk] + alf * pk[ijk];
          res[ijk] = res[ijk] - alf * zk[ijk];
          resl = resl + fabs(res[ijk]);
        }
    s0 = sk;
    if (l == 1) P->resor[ifi - 1] = res0;
    rsm = resl / (P->resor[ifi - 1] + SMALL);
    if (rsm < resmax) { done = 1; break; }
  }
  free(pk); free(zk); free(d);
  int iters = done ? l : ns;
  fill_rep(rep, res0, resl, iters, done ? CAPPGPU_OK : CAPPGPU_NOT_CONVERGED);
  if (!isfinite(resl)) { if (rep) rep->status = CAPPGPU_E_NONFINITE; return CAPPGPU_E_NONFINITE; }
  return done ? CAPPGPU_OK : CAPPGPU_NOT_CONVERGED;
}

/* ------------------------------------------------------- BiCGStab family */
/* cgstab.f90:3-283 (sip=0, ILU(0) diagonal preconditioner) and
   cgstab_sip.f90:3-279 (sip=1, SIP preconditioner). */
static int bicgstab(cap_state* s, int fif, int ifi, int sip, cappgpu_solve_report* rep) {
  COEF_PTRS;
  SIP_PTRS;
  double* fi = s->f[fif];
  double* res = s->f[CAP_RES];
  cappgpu_params* P = &s->prm;
  const int n = s->nijk;
  double *reso = zalloc(n), *pk = zalloc(n), *uk = zalloc(n), *zk = zalloc(n), *vk = zalloc(n);
  double* d = sip ? 0 : zalloc(n);
  double resmax = P->sor[ifi - 1];
  double res0 = 0.0;
  for (int k = 2; k <= s->nkm; ++k)
    for (int i = 3; i <= s->nimm; ++i)
      for (int j = 3; j <= s->njmm; ++j) {
        int ijk = IXK(i, j, k);
        res[ijk] = RESID(ijk);
        res0 = res0 + fabs(res[ijk]);
      }
  if (sip) {
    sip_factor(s, 2, s->nkm);
  } else {
    for (int k = 2; k <= s->nkm; ++k)
      for (int i = 3; i <= s->nimm; ++i)
        for (int j = 3; j <= s->njmm; ++j) {
          int ijk = IXK(i, j, k);
          d[ijk] = 1.0 / (ap[ijk] - aw[ijk] * d[ijk - nj] * ae[ijk - nj] - as[ijk] * d[ijk - 1] * an[ijk - 1] -
                          ab[ijk] * d[ijk - nij] * at[ijk - nij]);
        }
  }
  for (int k = 2; k <= s->nkm; ++k)
    for (int i = 3; i <= s->nimm; ++i)
      for (int j = 3; j <= s->njmm; ++j) {
        int ijk = IXK(i, j, k);
        reso[ijk] = res[ijk];
        pk[ijk] = 0.0; uk[ijk] = 0.0; zk[ijk] = 0.0; vk[ijk] = 0.0;
      }
  double alf = 1.0, beto = 1.0, gam = 1.0, bet, om, ukreso, vres, vv, resl = 0.0, rsm;
  int ns = P->nsw[ifi - 1], l, done = 0;
  /* backward loop of the second preconditioner solve: cgstab.f90:212 runs
     k=nkmm..3, cgstab_sip.f90:207 runs k=nkm..2 */
  int kb2_hi = sip ? s->nkm : s->nkmm, kb2_lo = sip ? 2 : 3;
  for (l = 1; l <= ns; ++l) {
    bet = 0.0;
    for (int k = 2; k <= s->nkm; ++k)
      for (int i = 3; i <= s->nimm; ++i)
        for (int j = 3; j <= s->njmm; ++j) {
          int ijk = IXK(i, j, k);
          bet = bet + res[ijk] * reso[ijk];
        }
    om = bet * gam / (alf * beto + SMALL);
    beto = bet;
    for (int k = 2; k <= s->nkm; ++k)
      for (int i = 3; i <= s->nimm; ++i)
        for (int j = 3; j <= s->njmm; ++j) {
          int ijk = IXK(i, j, k);
          pk[ijk] = res[ijk] + om * (pk[ijk] - alf * uk[ijk]);
        }
    /* solve (M zk = pk) */
    for (int k = 2; k <= s->nkm; ++k)
      for (int i = 3; i <= s->nimm; ++i)
        for (int j = 3; j <= s->njmm; ++j) {
          int ijk = IXK(i, j, k);
          if (sip)
            zk[ijk] = (pk[ijk] - bb[ijk] * zk[ijk - nij] - bw[ijk] * zk[ijk - nj] - bs[ijk] * zk[ijk - 1]) * bp[ijk];
          else
            zk[ijk] = (pk[ijk] + aw[ijk] * zk[ijk - nj] + as[ijk] * zk[ijk - 1] + ab[ijk] * zk[ijk - nij]) * d[ijk];
        }
    if (!sip)
      for (int k = 2; k <= s->nkm; ++k)
        for (int i = 3; i <= s->nimm; ++i)
          for (int j = 3; j <= s->njmm; ++j) {
            int ijk = IXK(i, j, k);
            zk[ijk] = zk[ijk] / (d[ijk] + SMALL);
          }
    for (int k = s->nkm; k >= 2; --k)
      for (int i = s->nimm; i >= 3; --i)
        for (int j = s->njmm; j >= 3; --j) {
          int ijk = IXK(i, j, k);
          if (sip)
            zk[ijk] = zk[ijk] - bn[ijk] * zk[ijk + 1] - be[ijk] * zk[ijk + nj] - bt[ijk] * zk[ijk + nij];
          else
            zk[ijk] = (zk[ijk] + ae[ijk] * zk[ijk + nj] + an[ijk] * zk[ijk + 1] + at[ijk] * zk[ijk + nij]) * d[ijk];
        }
    for (int k = 2; k <= s->nkm; ++k)
      for (int i = 3; i <= s->nimm; ++i)
        for (int j = 3; j <= s->njmm; ++j) {
          int ijk = IXK(i, j, k);
          uk[ijk] = APROD(zk, ijk);
        }
    ukreso = 0.0;
    for (int k = 2; k <= s->nkm; ++k)
      for (int i = 3; i <= s->nimm; ++i)
        for (int j = 3; j <= s->njmm; ++j) {
          int ijk = IXK(i, j, k);
          ukreso = ukreso + uk[ijk] * reso[ijk];
        }
    gam = bet / ukreso;
    for (int k = 2; k <= s->nkm; ++k)
      for (int i = 3; i <= s->nimm; ++i)
        for (int j = 3; j <= s->njmm; ++j) {
          int ijk = IXK(i, j, k);
          fi[ijk] = fi[ijk] + gam * zk[ijk];
          res[ijk] = res[ijk] - gam * uk[ijk];
        }
    /* solve (M y = w); y overwrites zk */
    for (int k = 2; k <= s->nkm; ++k)
      for (int i = 3; i <= s->nimm; ++i)
        for (int j = 3; j <= s->njmm; ++j) {
          int ijk = IXK(i, j, k);
          if (sip)
            zk[ijk] = (res[ijk] - bb[ijk] * zk[ijk - nij] - bw[ijk] * zk[ijk - nj] - bs[ijk] * zk[ijk - 1]) * bp[ijk];
          else
            zk[ijk] = (res[ijk] + aw[ijk] * zk[ijk - nj] + as[ijk] * zk[ijk - 1] + ab[ijk] * zk[ijk - nij]) * d[ijk];
        }
    if (!sip)
      for (int k = 2; k <= s->nkm; ++k)
        for (int i = 3; i <= s->nimm; ++i)
          for (int j = 3; j <= s->njmm; ++j) {
            int ijk = IXK(i, j, k);
            zk[ijk] = zk[ijk] / (d[ijk] + SMALL);
          }
    for (int k = kb2_hi; k >= kb2_lo; --k)
      for (int i = s->nimm; i >= 3; --i)
        for (int j = s->njmm; j >= 3; --j) {
          int ijk = IXK(i, j, k);
          if (sip)
            zk[ijk] = zk[ijk] - bn[ijk] * zk[ijk + 1] - be[ijk] * zk[ijk + nj] - bt[ijk] * zk[ijk + nij];
          else
            zk[ijk] = (zk[ijk] + ae[ijk] * zk[ijk + nj] + an[ijk] * zk[ijk + 1] + at[ijk] * zk[ijk + nij]) * d[ijk];
        }
    for (int k = 2; k <= s->nkm; ++k)
      for (int i = 3; i <= s->nimm; ++i)
        for (int j = 3; j <= s->njmm; ++j) {
          int ijk = IXK(i, j, k);
          vk[ijk] = APROD(zk, ijk);
        }
    vres = 0.0; vv = 0.0;
    for (int k = 2; k <= s->nkm; ++k)
      for (int i = 3; i <= s->nimm; ++i)
        for (int j = 3; j <= s->njmm; ++j) {
          int ijk = IXK(i, j, k);
          vres = vres + vk[ijk] * res[ijk];
          vv = vv + vk[ijk] * vk[ijk];
        }
    alf = vres / (vv + SMALL);
    resl = 0.0;
    for (int k = 2; k <= s->nkm; ++k)
      for (int i = 3; i <= s->nimm; ++i)
        for (int j = 3; j <= s->njmm; ++j) {
          int ijk = IXK(i, j, k);
          fi[ijk] = fi[ijk] + alf * zk[ijk];
          res[ijk] = res[ijk] - alf * vk[ijk];
          resl = resl + fabs(res[ijk]);
        }
    if (l == 1) P->resor[ifi - 1] = res0;
    rsm = resl / (P->resor[ifi - 1] + SMALL);
    if (rsm < resmax) { done = 1; break; }
  }
  free(reso); free(pk); free(uk); free(zk); free(vk); free(d);
  int iters = done ? l : ns;
  fill_rep(rep, res0, resl, iters, done ? CAPPGPU_OK : CAPPGPU_NOT_CONVERGED);
  if (!isfinite(resl)) { if (rep) rep->status = CAPPGPU_E_NONFINITE; return CAPPGPU_E_NONFINITE; }
  return done ? CAPPGPU_OK : CAPPGPU_NOT_CONVERGED;
}

int cap_cgstab(cap_state* s, int fi, int ifi, cappgpu_solve_report* rep) { return bicgstab(s, fi, ifi, 0, rep); }
int cap_cgstab_sip(cap_state* s, int fi, int ifi, cappgpu_solve_report* rep) { return bicgstab(s, fi, ifi, 1, rep); }

/* ----------------------------------------------------------------- DPCG */
/* pcg-jacobi.f90:3-155 (Diagonally_Preconditioned_CG) */
int cap_dpcg(cap_state* s, int fif, int ifi, cappgpu_solve_report* rep) {
  COEF_PTRS;
  double* fi = s->f[fif];
  double* res = s->f[CAP_RES];
  cappgpu_params* P = &s->prm;
  const int n = s->nijk;
  double *pk = zalloc(n), *zk = zalloc(n);
  double resmax = P->sor[ifi - 1];
  memset(res, 0, sizeof(double) * n);
  double res0 = 0.0;
  for (int k = 3; k <= s->nkmm; ++k)
    for (int i = 3; i <= s->nimm; ++i)
      for (int j = 3; j <= s->njmm; ++j) {
        int ijk = IXK(i, j, k);
        res[ijk] = RESID(ijk);
        res0 = res0 + fabs(res[ijk]);
      }
  double s0 = (double)1.e20f, sk, pkapk, alf, bet, resl = 0.0, rsm;
  int ns = P->nsw[ifi - 1], l, done = 0;
  for (l = 1; l <= ns; ++l) {
    sk = 0.0;
    for (int k = 3; k <= s->nkmm; ++k)
      for (int i = 3; i <= s->nimm; ++i)
        for (int j = 3; j <= s->njmm; ++j) {
          int ijk = IXK(i, j, k);
          zk[ijk] = res[ijk] / (ap[ijk] + SMALL);
          sk = sk + res[ijk] * zk[ijk];
        }
    bet = sk / s0;
    for (int k = 3; k <= s->nkmm; ++k)
      for (int i = 3; i <= s->nimm; ++i)
        for (int j = 3; j <= s->njmm; ++j) {
          int ijk = IXK(i, j, k);
          pk[ijk] = zk[ijk] + bet * pk[ijk];
        }
    pkapk = 0.0;
    for (int k = 3; k <= s->nkmm; ++k)
      for (int i = 3; i <= s->nimm; ++i)
        for (int j = 3; j <= s->njmm; ++j) {
          int ijk = IXK(i, j, k);
          zk[ijk] = APROD(pk, ijk);
          pkapk = pkapk + pk[ijk] * zk[ijk];
        }
    alf = sk / pkapk;
    resl = 0.0;
    for (int k = 3; k <= s->nkmm; ++k)
      for (int i = 3; i <= s->nimm; ++i)
        for (int j = 3; j <= s->njmm; ++j) {
          int ijk = IXK(i, j, k);
          fi[ijk] = fi[ijk] + alf * pk[ijk];
          res[ijk] = res[ijk] - alf * zk[ijk];
          resl = resl + fabs(res[ijk]);
        }
    s0 = sk;
    if (l == 1) P->resor[ifi - 1] = res0;
    rsm = resl / (P->resor[ifi - 1] + SMALL);
    if (rsm < resmax) { done = 1; break; }
  }
  free(pk); free(zk);
  int iters = done ? l : ns;
  fill_rep(rep, res0, resl, iters, done ? CAPPGPU_OK : CAPPGPU_NOT_CONVERGED);
  if (!isfinite(resl)) { if (rep) rep->status = CAPPGPU_E_NONFINITE; return CAPPGPU_E_NONFINITE; }
  return done ? CAPPGPU_OK : CAPPGPU_NOT_CONVERGED;
}

/* The pcgsip SpMV pass alone (pcg-sip.f90:142-153): z = A p, returns p.z */
double cap_spmv(cap_state* s, int pkf, int zkf) {
  COEF_PTRS;
  const double* pk = s->f[pkf];
  double* zk = s->f[zkf];
  double pkapk = 0.0;
  for (int k = 3; k <= s->nkmm; ++k)
    for (int i = 3; i <= s->nimm; ++i)
      for (int j = 3; j <= s->njmm; ++j) {
        int ijk = IXK(i, j, k);
        zk[ijk] = APROD(pk, ijk);
        pkapk = pkapk + pk[ijk] * zk[ijk];
      }
  return pkapk;
}

int cap_solve_dispatch(cap_state* s, int solver, int fi, int ifi, cappgpu_solve_report* rep) {
  switch (solver) {
    case CAPPGPU_SOLVER_SIPSOL: return cap_sipsol(s, fi, ifi, rep);
    case CAPPGPU_SOLVER_CGSTAB: return cap_cgstab(s, fi, ifi, rep);
    case CAPPGPU_SOLVER_ICCG: return cap_iccg(s, fi, ifi, rep);
    case CAPPGPU_SOLVER_PCGSIP: return cap_pcgsip(s, fi, ifi, rep);
    case CAPPGPU_SOLVER_CGSTAB_SIP: return cap_cgstab_sip(s, fi, ifi, rep);
    case CAPPGPU_SOLVER_DPCG: return cap_dpcg(s, fi, ifi, rep);
    default: return CAPPGPU_E_ARG;
  }
}
