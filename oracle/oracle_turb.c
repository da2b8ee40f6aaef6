/* oracle_turb.c -- the two-equation turbulence path of the reference
 * restated in C (TEST INFRASTRUCTURE ONLY): Menter's k-omega SST as the
 * reference's built code runs it -- calcscm.f90 (sources, assembly and the
 * sipsol solve of te and ed), calculate_stuff_for_sst.f90 (blending),
 * fluxscm-overrelaxed-correction.f90 (face fluxes) and modvis.f90 (eddy
 * viscosity).  Only the branches the SST configuration takes are restated
 * (levm, gauss gradients, no buoyancy, no low-Re, no SAS); the rest of
 * those routines belongs to other turbulence models.
 *
 * Constants are init.f90:229-245 with the reference's literal kinds: the
 * default-real literals (0.075, 0.0828, 5./9., 0.44, 0.09) are single
 * precision there and are reproduced as (double)<float>.  MAX/MIN over
 * several arguments take the larger/smaller in argument order with a > b /
 * a < b tests, so a NaN argument loses to a number (modvis.f90:217-221 on
 * the wall ghost layers, where te is negative).
 */
#include <math.h>
#include <string.h>

#include "oracle.h"
#include "oracle_internal.h"

#define SIGMK1 (1.0 / 1.176)
#define SIGMK2 1.0
#define SIGMOM1 (1.0 / 2.0)
#define SIGMOM2 (1.0 / 1.168)
#define BETAI1 ((double)0.075f)
#define BETAI2 ((double)0.0828f)
#define A1SST 0.31
#define ALPHA1 ((double)(5.0f / 9.0f))
#define ALPHA2 ((double)0.44f)
#define BETTAST ((double)0.09f)

static inline double nmax(double a, double b) { return (b > a || a != a) ? b : a; }
static inline double nmin(double a, double b) { return (b < a || a != a) ? b : a; }

/* calculate_stuff_for_sst.f90:27-70 over the interior: blending function
   F from k, omega, the wall distance and the cross-diffusion term, then
   alphasst, bettasst, prtinv_te, prtinv_ed and domega. */
void cap_calculate_stuff_for_sst(cap_state* s) {
  const cappgpu_params* P = &s->prm;
  double** f = s->f;
  const double viscos = P->viscos;
  for (int k = 3; k <= s->nkmm; ++k)
    for (int i = 3; i <= s->nimm; ++i)
      for (int j = 3; j <= s->njmm; ++j) {
        const int inp = IXK(i, j, k);
        const double wldist = f[CAP_WALLDIST][inp];
        const double dtedx = f[CAP_GRADTE_X][inp], dtedy = f[CAP_GRADTE_Y][inp], dtedz = f[CAP_GRADTE_Z][inp];
        const double deddx = f[CAP_GRADED_X][inp], deddy = f[CAP_GRADED_Y][inp], deddz = f[CAP_GRADED_Z][inp];
        const double den = f[CAP_DEN][inp], te = f[CAP_TE][inp], ed = f[CAP_ED][inp];
        const double dot = dtedx * deddx + dtedy * deddy + dtedz * deddz;
        const double tmp1 = 2.0 * den / ((double)1.168f * ed) * dot;
        const double tmp2 = (double)1.e-10f;
        const double domegapl = nmax(tmp1, tmp2);
        const double ksi = nmin(nmax(sqrt(te) / ((double)0.09f * wldist * ed), (500.0 * viscos / den) / (wldist * wldist * ed)),
                                4.0 * den * te / ((double)1.168f * domegapl * (wldist * wldist)));
        const double k2 = ksi * ksi;
        const double F = tanh(k2 * k2);
        f[CAP_ALPHASST][inp] = F * ALPHA1 + (1.0 - F) * ALPHA2;
        f[CAP_BETTASST][inp] = F * BETAI1 + (1.0 - F) * BETAI2;
        f[CAP_PRTINV_TE][inp] = F * SIGMK1 + (1.0 - F) * SIGMK2;
        f[CAP_PRTINV_ED][inp] = F * SIGMOM1 + (1.0 - F) * SIGMOM2;
        const double dom = 2.0 * (1.0 - F) * den / ((double)1.168f * ed) * dot;
        f[CAP_DOMEGA][inp] = nmax(dom, 0.0);
      }
}

/* fluxscm-overrelaxed-correction.f90:40-230 for one face direction over
   k = 2..nkmm, i = 2..nimm, j = 2..njmm: face diffusion with the
   orthogonal correction (costn = 1), the SST diffusivity blend, upwind
   coefficients acfe/acfw, the deferred-correction and explicit-diffusion
   source into su (this cell) and, through bp, minus it into the east
   neighbour; bp is zero on return. */
void cap_fluxscm(cap_state* s, int idew, int idns, int idtb, int fi, int gx, int ifi, int arvx, int arvy, int arvz,
                 int fif, int acfe, int acfw, int fcf) {
  const cappgpu_params* P = &s->prm;
  double** f = s->f;
  const double viscos = P->viscos, gam = P->gds[ifi - 1], zero = P->zero;
  const double *x = f[CAP_X], *y = f[CAP_Y], *z = f[CAP_Z], *xc = f[CAP_XC], *yc = f[CAP_YC], *zc = f[CAP_ZC];
  const double *vis = f[CAP_VIS], *phi = f[fi], *g1 = f[gx], *g2 = f[gx + 1], *g3 = f[gx + 2];
  const double* prt = ifi == CAP_ITE ? f[CAP_PRTINV_TE] : f[CAP_PRTINV_ED];
  double *su = f[CAP_SU], *bp = f[CAP_BP];
  for (int k = 2; k <= s->nkmm; ++k)
    for (int i = 2; i <= s->nimm; ++i)
      for (int j = 2; j <= s->njmm; ++j) {
        const int inp = IXK(i, j, k);
        const int ine = inp + idew, ins = inp - idns, inb = inp - idtb, inbs = inb - idns;
        const double fxe = f[fif][inp], fxp = 1.0 - fxe;
        const double xpn = xc[ine] - xc[inp], ypn = yc[ine] - yc[inp], zpn = zc[ine] - zc[inp];
        const double dpn = sqrt(xpn * xpn + ypn * ypn + zpn * zpn);
        const double arx = f[arvx][inp], ary = f[arvy][inp], arz = f[arvz][inp];
        const double are = sqrt(arx * arx + ary * ary + arz * arz);
        const double costn = 1.0;
        const double vole = xpn * arx + ypn * ary + zpn * arz;
        const double d1x = costn, d1y = costn, d1z = costn;
        const double d2x = xpn * costn, d2y = ypn * costn, d2z = zpn * costn;
        const double prtr = prt[inp] * fxp + prt[ine] * fxe;   /* :102-105 (sst) */
        const double viste = (vis[inp] - viscos) * fxp + (vis[ine] - viscos) * fxe;
        const double game = viste * prtr + viscos;
        const double xf = 0.25 * (x[inp] + x[ins] + x[inb] + x[inbs]);
        const double yf = 0.25 * (y[inp] + y[ins] + y[inb] + y[inbs]);
        const double zf = 0.25 * (z[inp] + z[ins] + z[inb] + z[inbs]);
        const double xi = xc[inp] * fxp + xc[ine] * fxe;
        const double yi = yc[inp] * fxp + yc[ine] * fxe;
        const double zi = zc[inp] * fxp + zc[ine] * fxe;
        const double dfixi = g1[inp] * fxp + g1[ine] * fxe;
        const double dfiyi = g2[inp] * fxp + g2[ine] * fxe;
        const double dfizi = g3[inp] * fxp + g3[ine] * fxe;
        const double dfixii = dfixi * d1x + arx / vole * (phi[ine] - phi[inp] - dfixi * d2x - dfiyi * d2y - dfizi * d2z);
        const double dfiyii = dfiyi * d1y + ary / vole * (phi[ine] - phi[inp] - dfixi * d2x - dfiyi * d2y - dfizi * d2z);
        const double dfizii = dfizi * d1z + arz / vole * (phi[ine] - phi[inp] - dfixi * d2x - dfiyi * d2y - dfizi * d2z);
        const double fdfie = game * (dfixii * arx + dfiyii * ary + dfizii * arz);
        const double fdfii = game * are / dpn * (dfixi * xpn + dfiyi * ypn + dfizi * zpn);
        const double de = game * are / dpn;
        const double fm = f[fcf][inp];
        const double ce = dmin(fm, zero), cp = dmax(fm, zero);
        f[acfe][inp] = de - ce;
        f[acfw][ine] = de + cp;
        double fcfie;
        if (P->lcds) {
          const double fii = phi[inp] * fxp + phi[ine] * fxe + (dfixi * (xf - xi) + dfiyi * (yf - yi) + dfizi * (zf - zi));
          fcfie = fm * fii;
        } else {   /* :183-190, limited linear upwind */
          const double r1 = (2 * g1[inp] * xpn + 2 * g2[inp] * ypn + 2 * g3[inp] * zpn) / (phi[ine] - phi[inp]) - 1.0;
          const double r2 = (2 * g1[ine] * xpn + 2 * g2[ine] * ypn + 2 * g3[ine] * zpn) / (phi[inp] - phi[ine]) - 1.0;
          const double psiw = nmax(0.0, nmin(nmin(2.0 * r1, 0.5 * r1 + 0.5), 2.0));
          const double psie = nmax(0.0, nmin(nmin(2.0 * r2, 0.5 * r2 + 0.5), 2.0));
          fcfie = ce * (phi[ine] + fxe * psie * (phi[inp] - phi[ine])) + cp * (phi[inp] + fxp * psiw * (phi[ine] - phi[inp]));
        }
        const double fcfii = ce * phi[ine] + cp * phi[inp];
        const double ffic = gam * (fcfie - fcfii);
        const double suadd = -ffic + fdfie - fdfii;
        su[inp] = su[inp] + suadd;
        bp[ine] = suadd;
      }
  for (int k = 2; k <= s->nkmm; ++k)   /* :208-216 */
    for (int i = 2; i <= s->nimm; ++i)
      for (int j = 2; j <= s->njmm; ++j) {
        const int inp = IXK(i, j, k) + idew;
        su[inp] = su[inp] - bp[inp];
      }
  memset(bp, 0, sizeof(double) * s->nijk);   /* :218 */
}

/* calcscm.f90:3-602 for ifi = ite (k) or ied (omega) under SST: the
   gradient of fi, the volume sources (k: production limited to
   0.9 rho k omega, destruction bettast rho omega; omega: calculate_stuff_
   for_sst, then alphasst P / nu_t + cross diffusion, destruction
   bettasst rho omega), the implicit time term (bdf), the face fluxes in
   three directions, Crank-Nicolson terms (cn), ap, under-relaxation,
   sipsol, and fi >= small on the whole array. */
int cap_calcscm(cap_state* s, int ifi, cappgpu_solve_report* rep) {
  cappgpu_params* P = &s->prm;
  double** f = s->f;
  const int fi = ifi == CAP_ITE ? CAP_TE : CAP_ED;
  const int gx = ifi == CAP_ITE ? CAP_GRADTE_X : CAP_GRADED_X;
  const int fo = ifi == CAP_ITE ? CAP_TEO : CAP_EDO;
  const int foo = ifi == CAP_ITE ? CAP_TEOO : CAP_EDOO;
  const double viscos = P->viscos, zero = P->zero, densit = P->densit;
  cap_grad_gauss(s, fi, gx, gx + 1, gx + 2);   /* :53-55 */
  double *su = f[CAP_SU], *sp = f[CAP_SP];
  const double *vol = f[CAP_VOL], *den = f[CAP_DEN], *te = f[CAP_TE], *ed = f[CAP_ED], *vis = f[CAP_VIS];
  if (ifi == CAP_ITE) {
    cap_find_strain_rate(s);   /* :62 */
    for (int k = 3; k <= s->nkmm; ++k)
      for (int i = 3; i <= s->nimm; ++i)
        for (int j = 3; j <= s->njmm; ++j) {
          const int inp = IXK(i, j, k);
          const double ssq = f[CAP_STRAIN][inp] * f[CAP_STRAIN][inp];
          double gen = fabs(vis[inp] - viscos) * ssq;                        /* :73-74 */
          gen = dmin(gen, (double)0.9f * den[inp] * te[inp] * ed[inp]);      /* :80 */
          f[CAP_GEN][inp] = gen;
        }
    for (int k = 3; k <= s->nkmm; ++k)
      for (int i = 3; i <= s->nimm; ++i)
        for (int j = 3; j <= s->njmm; ++j) {
          const int inp = IXK(i, j, k);
          const double genp = dmax(f[CAP_GEN][inp], zero), genn = dmin(f[CAP_GEN][inp], zero);
          su[inp] = genp * vol[inp];                                          /* :147 */
          sp[inp] = BETTAST * ed[inp] * den[inp] * vol[inp];                  /* :195 */
          sp[inp] = sp[inp] - genn * vol[inp] / te[inp];                      /* :204 */
          if (P->bdf) {                                                       /* :213-220 */
            const double apotime = den[inp] * vol[inp] / P->timestep;
            const double sut = apotime * ((1 + P->btime) * f[fo][inp] - 0.5 * P->btime * f[foo][inp]);
            su[inp] = su[inp] + sut;
            sp[inp] = sp[inp] + apotime * (1 + 0.5 * P->btime);
          }
        }
  } else {
    cap_calculate_stuff_for_sst(s);   /* :267 */
    for (int k = 3; k <= s->nkmm; ++k)
      for (int i = 3; i <= s->nimm; ++i)
        for (int j = 3; j <= s->njmm; ++j) {
          const int inp = IXK(i, j, k);
          const double genp = dmax(f[CAP_GEN][inp], zero), genn = dmin(f[CAP_GEN][inp], zero);
          const double domegap = dmax(f[CAP_DOMEGA][inp], zero);
          f[CAP_SV][inp] = 0.0;                                               /* :320 */
          double vist = (vis[inp] - viscos) / densit;                         /* :425-438 */
          su[inp] = f[CAP_ALPHASST][inp] * genp * vol[inp] / vist;
          su[inp] = su[inp] + domegap * vol[inp];
          vist = (vis[inp] - viscos) / densit;
          sp[inp] = f[CAP_BETTASST][inp] * den[inp] * ed[inp] * vol[inp];
          sp[inp] = sp[inp] - f[CAP_ALPHASST][inp] * genn * vol[inp] / (vist * ed[inp]);
          if (P->bdf) {                                                       /* :478-486 */
            const double apotime = den[inp] * vol[inp] / P->timestep;
            const double sut = apotime * ((1 + P->btime) * f[fo][inp] - 0.5 * P->btime * f[foo][inp]);
            su[inp] = su[inp] + sut;
            sp[inp] = sp[inp] + apotime * (1 + 0.5 * P->btime);
          }
        }
  }
  /* :528-540 */
  cap_fluxscm(s, s->nj, 1, s->nij, fi, gx, ifi, CAP_AR1X, CAP_AR1Y, CAP_AR1Z, CAP_FX, CAP_AE, CAP_AW, CAP_F1);
  cap_fluxscm(s, 1, s->nij, s->nj, fi, gx, ifi, CAP_AR2X, CAP_AR2Y, CAP_AR2Z, CAP_FY, CAP_AN, CAP_AS, CAP_F2);
  cap_fluxscm(s, s->nij, s->nj, 1, fi, gx, ifi, CAP_AR3X, CAP_AR3Y, CAP_AR3Z, CAP_FZ, CAP_AT, CAP_AB, CAP_F3);
  const double urfrs = 1.0 / P->urf[ifi - 1], urfms = 1.0 - P->urf[ifi - 1];   /* init.f90:332-333 */
  double *ae = f[CAP_AE], *aw = f[CAP_AW], *an = f[CAP_AN], *as = f[CAP_AS], *at = f[CAP_AT], *ab = f[CAP_AB];
  double *ap = f[CAP_AP], *phi = f[fi];
  const int nj = s->nj, nij = s->nij;
  for (int k = 3; k <= s->nkmm; ++k)   /* :546-586 */
    for (int i = 3; i <= s->nimm; ++i)
      for (int j = 3; j <= s->njmm; ++j) {
        const int inp = IXK(i, j, k);
        if (P->cn) {
          ae[inp] = 0.5 * ae[inp];
          an[inp] = 0.5 * an[inp];
          at[inp] = 0.5 * at[inp];
          aw[inp] = 0.5 * aw[inp];
          as[inp] = 0.5 * as[inp];
          ab[inp] = 0.5 * ab[inp];
          const double apotime = den[inp] * vol[inp] / P->timestep;
          const double* o = f[fo];
          su[inp] = su[inp] + (ae[inp] * o[inp + nj] + aw[inp] * o[inp - nj] + an[inp] * o[inp + 1] +
                               as[inp] * o[inp - 1] + at[inp] * o[inp + nij] + ab[inp] * o[inp - nij]) +
                    (apotime - ae[inp] - aw[inp] - an[inp] - as[inp] - at[inp] - ab[inp]) * o[inp];
          sp[inp] = sp[inp] + apotime;
        }
        ap[inp] = ae[inp] + aw[inp] + an[inp] + as[inp] + at[inp] + ab[inp] + sp[inp];
        ap[inp] = ap[inp] * urfrs;
        su[inp] = su[inp] + urfms * ap[inp] * phi[inp];
      }
  const int rc = cap_solve_dispatch(s, CAPPGPU_SOLVER_SIPSOL, fi, ifi, rep);   /* :591 */
  for (int q = 0; q < s->nijk; ++q) phi[q] = dmax(phi[q], SMALL);              /* :595-599 */
  return rc;
}

/* modvis.f90:195-236, the SST branch (high-Re) over k = 2..nkm,
   i = 3..nimm, j = 3..njmm: F2 from the wall distance, the eddy viscosity
   viscos + rho a1 k / max(a1, omega, S F2) (the reference's three-argument
   MAX, :221) and under-relaxation with urf(ivis). */
void cap_modvis(cap_state* s) {
  const cappgpu_params* P = &s->prm;
  double** f = s->f;
  const double viscos = P->viscos, cmu = P->cmu, urf = P->urf[CAP_IVIS - 1];
  for (int k = 2; k <= s->nkm; ++k)
    for (int i = 3; i <= s->nimm; ++i)
      for (int j = 3; j <= s->njmm; ++j) {
        const int inp = IXK(i, j, k);
        const double visold = f[CAP_VIS][inp];
        const double wldist = f[CAP_WALLDIST][inp];
        const double te = f[CAP_TE][inp], ed = f[CAP_ED][inp], den = f[CAP_DEN][inp];
        const double etha = nmax(2 * sqrt(te) / (cmu * wldist * ed), (500 * viscos / den) / (wldist * wldist * ed));
        const double f2 = tanh(etha * etha);
        double v = viscos + den * A1SST * te / nmax(nmax(A1SST, ed), f[CAP_STRAIN][inp] * f2);
        v = urf * v + (1.0 - urf) * visold;
        f[CAP_VIS][inp] = v;
      }
}
