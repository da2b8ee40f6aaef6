/*
 * oracle_assembly.c -- momentum assembly (fluxuvw, calcuvw), PISO and
 * SIMPLE pressure-velocity coupling, Courant number, continuity errors and
 * the step drivers, restated line by line from the reference (TEST
 * INFRASTRUCTURE ONLY; pinned against the reference's own routines, see
 * oracle.h).
 */
#include "oracle.h"
#include "oracle_internal.h"

#include <stdlib.h>
#include <string.h>
#include <math.h>

/* --------------------------------------------------------------- fluxuvw */
/* fluxuvw-overrelaxed-correction.f90:3-659.  The deferred-correction
   source of the neighbour is staged in the SIP arrays bp,bt,bb exactly as
   the reference does (:631-656), so their final content (all zero) and the
   stale values picked up by the scatter loop (:639-650) match. */
void cap_fluxuvw(cap_state* s, int idew, int idns, int idtb, int arvxf, int arvyf, int arvzf,
                 int fiff, int acfef, int acfwf, int fcff) {
  const cappgpu_params* P = &s->prm;
  const double *arvx = s->f[arvxf], *arvy = s->f[arvyf], *arvz = s->f[arvzf], *fif = s->f[fiff];
  double *acfe = s->f[acfef], *acfw = s->f[acfwf];
  const double* fcf = s->f[fcff];
  const double *x = s->f[CAP_X], *y = s->f[CAP_Y], *z = s->f[CAP_Z];
  const double *xc = s->f[CAP_XC], *yc = s->f[CAP_YC], *zc = s->f[CAP_ZC];
  const double *u = s->f[CAP_U], *v = s->f[CAP_V], *w = s->f[CAP_W], *vis = s->f[CAP_VIS];
  const double *gux = s->f[CAP_GRADU_X], *guy = s->f[CAP_GRADU_Y], *guz = s->f[CAP_GRADU_Z];
  const double *gvx = s->f[CAP_GRADV_X], *gvy = s->f[CAP_GRADV_Y], *gvz = s->f[CAP_GRADV_Z];
  const double *gwx = s->f[CAP_GRADW_X], *gwy = s->f[CAP_GRADW_Y], *gwz = s->f[CAP_GRADW_Z];
  double *su = s->f[CAP_SU], *sv = s->f[CAP_SV], *sw = s->f[CAP_SW];
  double *bp = s->f[CAP_BP], *bt = s->f[CAP_BT], *bb = s->f[CAP_BB];
  const double gam = P->gds[CAP_IU - 1];
  const double zero = P->zero;
  int dir = 0;
  if (idew == s->nj) dir = 1;
  if (idew == 1) dir = 2;
  if (idew == s->nij) dir = 3;
  const double* gu_dir = dir == 1 ? gux : dir == 2 ? guy : guz;
  const double* gv_dir = dir == 1 ? gvx : dir == 2 ? gvy : gvz;
  const double* gw_dir = dir == 1 ? gwx : dir == 2 ? gwy : gwz;
  int kst = 2, kend = s->nkmm, ist = 2, iend = s->nimm, jst = 2, jend = s->njmm;
  if (dir == 1) { jst = 3; kst = 3; }
  else if (dir == 2) { ist = 3; kst = 3; }
  else if (dir == 3) { ist = 3; jst = 3; }
  /* :90-92 zero the high-order fluxes once, before the face loop: a face
     where no scheme assigns them (QUICK outside its box, :383-385) keeps
     the previous face's values */
  double fuhigh = 0.0, fvhigh = 0.0, fwhigh = 0.0;
  for (int k = kst; k <= kend; ++k)
    for (int i = ist; i <= iend; ++i)
      for (int j = jst; j <= jend; ++j) {
        int inp = IXK(i, j, k);
        int ine = inp + idew, inw = inp - idew, ins = inp - idns, inb = inp - idtb;
        int inee = inp + 2 * idew, inbs = inb - idns;
        double fxe = fif[inp], fxp = 1.0 - fxe;
        double fxpw = fif[inw], fxw = 1.0 - fxpw;
        double fxee = fif[ine], fxew = 1.0 - fxee;
        double xpn = xc[ine] - xc[inp], ypn = yc[ine] - yc[inp], zpn = zc[ine] - zc[inp];
        double dpn = sqrt(xpn * xpn + ypn * ypn + zpn * zpn);
        double arx = arvx[inp], ary = arvy[inp], arz = arvz[inp];
        double are = sqrt(arx * arx + ary * ary + arz * arz);
        /* costheta is computed by the reference (:155-172) but unused with
           costn = 1 (orthogonal correction, :178) */
        double costn = 1.0;
        double vole = xpn * arx + ypn * ary + zpn * arz;
        double d1x = costn, d1y = costn, d1z = costn;
        double d2x = xpn * costn, d2y = ypn * costn, d2z = zpn * costn;
        double game = (vis[inp] * fxp + vis[ine] * fxe);
        double xf = 0.25 * (x[inp] + x[ins] + x[inb] + x[inbs]);
        double yf = 0.25 * (y[inp] + y[ins] + y[inb] + y[inbs]);
        double zf = 0.25 * (z[inp] + z[ins] + z[inb] + z[inbs]);
        double xi = xc[inp] * fxp + xc[ine] * fxe;
        double yi = yc[inp] * fxp + yc[ine] * fxe;
        double zi = zc[inp] * fxp + zc[ine] * fxe;
        double duxi = gux[inp] * fxp + gux[ine] * fxe;
        double duyi = guy[inp] * fxp + guy[ine] * fxe;
        double duzi = guz[inp] * fxp + guz[ine] * fxe;
        double duxii = duxi * d1x + arx / vole * (u[ine] - u[inp] - duxi * d2x - duyi * d2y - duzi * d2z);
        double duyii = duyi * d1y + ary / vole * (u[ine] - u[inp] - duxi * d2x - duyi * d2y - duzi * d2z);
        double duzii = duzi * d1z + arz / vole * (u[ine] - u[inp] - duxi * d2x - duyi * d2y - duzi * d2z);
        double dvxi = gvx[inp] * fxp + gvx[ine] * fxe;
        double dvyi = gvy[inp] * fxp + gvy[ine] * fxe;
        double dvzi = gvz[inp] * fxp + gvz[ine] * fxe;
        double dvxii = dvxi * d1x + arx / vole * (v[ine] - v[inp] - dvxi * d2x - dvyi * d2y - dvzi * d2z);
        double dvyii = dvyi * d1y + ary / vole * (v[ine] - v[inp] - dvxi * d2x - dvyi * d2y - dvzi * d2z);
        double dvzii = dvzi * d1z + arz / vole * (v[ine] - v[inp] - dvxi * d2x - dvyi * d2y - dvzi * d2z);
        double dwxi = gwx[inp] * fxp + gwx[ine] * fxe;
        double dwyi = gwy[inp] * fxp + gwy[ine] * fxe;
        double dwzi = gwz[inp] * fxp + gwz[ine] * fxe;
        double dwxii = dwxi * d1x + arx / vole * (w[ine] - w[inp] - dwxi * d2x - dwyi * d2y - dwzi * d2z);
        double dwyii = dwyi * d1y + ary / vole * (w[ine] - w[inp] - dwxi * d2x - dwyi * d2y - dwzi * d2z);
        double dwzii = dwzi * d1z + arz / vole * (w[ine] - w[inp] - dwxi * d2x - dwyi * d2y - dwzi * d2z);
        double fdue = game * ((duxii + duxii) * arx + (duyii + dvxii) * ary + (duzii + dwxii) * arz);
        double fdve = game * ((duyii + dvxii) * arx + (dvyii + dvyii) * ary + (dvzii + dwyii) * arz);
        double fdwe = game * ((duzii + dwxii) * arx + (dwyii + dvzii) * ary + (dwzii + dwzii) * arz);
        double fdui = game * are / dpn * (duxi * xpn + duyi * ypn + duzi * zpn);
        double fdvi = game * are / dpn * (dvxi * xpn + dvyi * ypn + dvzi * zpn);
        double fdwi = game * are / dpn * (dwxi * xpn + dwyi * ypn + dwzi * zpn);
        double de = game * are / dpn;
        double flcf = fcf[inp];
        double ce = dmin(flcf, zero);
        double cp = dmax(flcf, zero);
        acfe[inp] = de - ce;
        acfw[ine] = de + cp;
        double fuuds = cp * u[inp] + ce * u[ine];
        double fvuds = cp * v[inp] + ce * v[ine];
        double fwuds = cp * w[inp] + ce * w[ine];
        double ue, ve, we;
        if (P->lcds) { /* :297-314 */
          ue = u[inp] * fxp + u[ine] * fxe + (duxi * (xf - xi) + duyi * (yf - yi) + duzi * (zf - zi));
          ve = v[inp] * fxp + v[ine] * fxe + (dvxi * (xf - xi) + dvyi * (yf - yi) + dvzi * (zf - zi));
          we = w[inp] * fxp + w[ine] * fxe + (dwxi * (xf - xi) + dwyi * (yf - yi) + dwzi * (zf - zi));
          fuhigh = flcf * ue; fvhigh = flcf * ve; fwhigh = flcf * we;
        }
        if (P->lcds4 && (idew == s->nj || idew == 1)) { /* :317-332 */
          ue = 1.0 / 48.0 * (27.0 * u[inp] + 27.0 * u[ine] - 3.0 * u[inw] - 3.0 * u[inee]);
          ve = 1.0 / 48.0 * (27.0 * v[inp] + 27.0 * v[ine] - 3.0 * v[inw] - 3.0 * v[inee]);
          we = 1.0 / 48.0 * (27.0 * w[inp] + 27.0 * w[ine] - 3.0 * w[inw] - 3.0 * w[inee]);
          fuhigh = flcf * ue; fvhigh = flcf * ve; fwhigh = flcf * we;
        }
        if (P->lluds) { /* :335-372 */
          double dxc = xf - xc[inp], dyc = yf - yc[inp], dzc = zf - zc[inp];
          double dxe = xc[ine] - xf, dye = yc[ine] - yf, dze = zc[ine] - zf;
          double dfidx_u = gu_dir[inw] * fxw + gu_dir[inp] * fxpw;
          double dfidy_u = gv_dir[inw] * fxw + gv_dir[inp] * fxpw;
          double dfidz_u = gw_dir[inw] * fxw + gw_dir[inp] * fxpw;
          double dfidx_u1 = gu_dir[inee] * fxee + gu_dir[ine] * fxew;
          double dfidy_u1 = gv_dir[inee] * fxee + gv_dir[ine] * fxew;
          double dfidz_u1 = gw_dir[inee] * fxee + gw_dir[ine] * fxew;
          fuhigh = ce * (u[ine] + dxe * dfidx_u1) + cp * (u[inp] + dxc * dfidx_u);
          fvhigh = ce * (v[ine] + dye * dfidy_u1) + cp * (v[inp] + dyc * dfidy_u);
          fwhigh = ce * (w[ine] + dze * dfidz_u1) + cp * (w[inp] + dzc * dfidz_u);
        }
        if (P->lquds) { /* :375-413 */
          if (k > 2 && k < s->nk - 1 && j > 2 && j < s->nj - 1 && i > 2 && i < s->ni - 1) {
            double fm = fif[inp - idew], f0 = fif[inp], fpl = fif[inp + idew];
            double g11 = ((2 - fm) * (f0 * f0)) / (1 + f0 - fm);
            double g12 = ((1 - f0) * ((1 - fm) * (1 - fm))) / (1 + f0 - fm);
            double g21 = ((1 + fpl) * ((1 - f0) * (1 - f0))) / (1 + fpl - f0);
            double g22 = ((fpl * fpl) * f0) / (1 + fpl - f0);
            fuhigh = ce * (g21 * u[inp] + (1 - g21 + g22) * u[ine] - g22 * u[inee]) +
                     cp * (g11 * u[ine] + (1 - g11 + g12) * u[inp] - g12 * u[inw]);
            fvhigh = ce * (g21 * v[inp] + (1 - g21 + g22) * v[ine] - g22 * v[inee]) +
                     cp * (g11 * v[ine] + (1 - g11 + g12) * v[inp] - g12 * v[inw]);
            fwhigh = ce * (g21 * w[inp] + (1 - g21 + g22) * w[ine] - g22 * w[inee]) +
                     cp * (g11 * w[ine] + (1 - g11 + g12) * w[inp] - g12 * w[inw]);
          }
        }
        if (P->flux_limiter) { /* :424-619 (patch-version 3, ver.3 flux) */
          double r1 = (2 * gux[inp] * xpn + 2 * guy[inp] * ypn + 2 * guz[inp] * zpn) / (u[ine] - u[inp]) - 1.0;
          double r2 = (2 * gvx[inp] * xpn + 2 * gvy[inp] * ypn + 2 * gvz[inp] * zpn) / (v[ine] - v[inp]) - 1.0;
          double r3 = (2 * gwx[inp] * xpn + 2 * gwy[inp] * ypn + 2 * gwz[inp] * zpn) / (w[ine] - w[inp]) - 1.0;
          double r4 = (2 * gux[ine] * xpn + 2 * guy[ine] * ypn + 2 * guz[ine] * zpn) / (u[inp] - u[ine]) - 1.0;
          double r5 = (2 * gvx[ine] * xpn + 2 * gvy[ine] * ypn + 2 * gvz[ine] * zpn) / (v[inp] - v[ine]) - 1.0;
          double r6 = (2 * gwx[ine] * xpn + 2 * gwy[ine] * ypn + 2 * gwz[ine] * zpn) / (w[inp] - w[ine]) - 1.0;
          double rr[6] = {r1, r2, r3, r4, r5, r6}, psi[6] = {0, 0, 0, 0, 0, 0};
          for (int q = 0; q < 6; ++q) {
            double r = rr[q];
            if (P->lsmart) psi[q] = dmax(0.0, dmin(dmin(2.0 * r, 0.75 * r + 0.25), 4.0));
            if (P->lavl) psi[q] = dmax(0.0, dmin(dmin(1.5 * r, 0.75 * r + 0.25), 2.5));
            if (P->lmuscl) psi[q] = dmax(0.0, dmin(dmin(2.0 * r, 0.5 * r + 0.5), 2.0));
            if (P->lumist) psi[q] = dmax(0.0, dmin(dmin(dmin(2.0 * r, 0.75 * r + 0.25), 0.25 * r + 0.75), 2.0));
            if (P->lgamma) psi[q] = dmax(0.0, dmin(r, 2.0 * r / (r + 1.0)));
          }
          /* psiw1..3 = psi[0..2], psie1..3 = psi[3..5] */
          fuhigh = ce * (u[ine] + fxe * psi[3] * (u[inp] - u[ine])) + cp * (u[inp] + fxp * psi[0] * (u[ine] - u[inp]));
          fvhigh = ce * (v[ine] + fxe * psi[4] * (v[inp] - v[ine])) + cp * (v[inp] + fxp * psi[1] * (v[ine] - v[inp]));
          fwhigh = ce * (w[ine] + fxe * psi[5] * (w[inp] - w[ine])) + cp * (w[inp] + fxp * psi[2] * (w[ine] - w[inp]));
        }
        su[inp] = su[inp] + gam * (fuuds - fuhigh) + fdue - fdui;
        sv[inp] = sv[inp] + gam * (fvuds - fvhigh) + fdve - fdvi;
        sw[inp] = sw[inp] + gam * (fwuds - fwhigh) + fdwe - fdwi;
        bp[ine] = -gam * (fuuds - fuhigh) - fdue + fdui;
        bt[ine] = -gam * (fvuds - fvhigh) - fdve + fdvi;
        bb[ine] = -gam * (fwuds - fwhigh) - fdwe + fdwi;
      }
  for (int k = 2; k <= s->nkmm; ++k)
    for (int i = 2; i <= s->nimm; ++i)
      for (int j = 2; j <= s->njmm; ++j) {
        int inp = IXK(i, j, k) + idew;
        su[inp] = su[inp] + bp[inp];
        sv[inp] = sv[inp] + bt[inp];
        sw[inp] = sw[inp] + bb[inp];
      }
  memset(bp, 0, sizeof(double) * s->nijk);
  memset(bt, 0, sizeof(double) * s->nijk);
  memset(bb, 0, sizeof(double) * s->nijk);
}

/* --------------------------------------------------------------- calcuvw */
/* wall shear source of one wall (calcuvw.f90:161-337, first-order model) */
static void calcuvw_wall(cap_state* s, int top) {
  const double *xc = s->f[CAP_XC], *yc = s->f[CAP_YC], *zc = s->f[CAP_ZC], *fz = s->f[CAP_FZ];
  const double *a3x = s->f[CAP_AR3X], *a3y = s->f[CAP_AR3Y], *a3z = s->f[CAP_AR3Z];
  const double *u = s->f[CAP_U], *v = s->f[CAP_V], *w = s->f[CAP_W], *vis = s->f[CAP_VIS];
  double *ap = s->f[CAP_AP], *spv = s->f[CAP_SPV], *sp = s->f[CAP_SP];
  double *su = s->f[CAP_SU], *sv = s->f[CAP_SV], *sw = s->f[CAP_SW];
  /* nx,ny,nz in the dnw dot product are the integer array extents of
     module parameters (set_parameters.f90:34-36: nx = nicv+2 = ni), used
     as the reference does (calcuvw.f90:187,277). */
  const double nxi = (double)s->ni, nyi = (double)s->nj, nzi = (double)s->nk;
  for (int i = 3; i <= s->nimm; ++i)
    for (int j = 3; j <= s->njmm; ++j) {
      int inbc, ingc, iface;
      double fxp, fxe;
      if (!top) {
        inbc = IXK(i, j, 3); ingc = inbc - s->nij; iface = ingc;
        fxp = fz[ingc]; fxe = 1.0 - fxp;
      } else {
        /* the reference takes lk(nimm) for the top wall (calcuvw.f90:254);
           params.top_plane = 1 takes lk(nkmm) */
        inbc = IXK(i, j, s->prm.top_plane ? s->nkmm : s->nimm); ingc = inbc + s->nij; iface = inbc;
        fxp = 1.0 - fz[inbc]; fxe = 1.0 - fxp;
      }
      double gzx = xc[inbc] * fxp + xc[ingc] * fxe;
      double gzy = yc[inbc] * fxp + yc[ingc] * fxe;
      double gzz = zc[inbc] * fxp + zc[ingc] * fxe;
      double are = sqrt(a3x[iface] * a3x[iface] + a3y[iface] * a3y[iface] + a3z[iface] * a3z[iface]);
      double nxf = a3x[iface] / are, nyf = a3y[iface] / are, nzf = a3z[iface] / are;
      double dnw = fabs((xc[inbc] - gzx) * nxi + (yc[inbc] - gzy) * nyi + (zc[inbc] - gzz) * nzi);
      double viss = vis[ingc];
      double cf = viss * are / dnw;
      double dx = xc[inbc] - xc[ingc], dy = yc[inbc] - yc[ingc], dz = zc[inbc] - zc[ingc];
      double dpb = 0.5 * sqrt(dx * dx + dy * dy + dz * dz);
      double vsol = viss * are / dpb;
      double upb = u[inbc], vpb = v[inbc], wpb = w[inbc];
      double vnp = upb * nxf + vpb * nyf + wpb * nzf;
      double utp = upb - vnp * nxf, vtp = vpb - vnp * nyf, wtp = wpb - vnp * nzf;
      ap[inbc] = ap[inbc] + vsol;
      spv[inbc] = spv[inbc] + vsol;
      sp[inbc] = sp[inbc] + vsol;
      su[inbc] = su[inbc] + vsol * u[inbc] - cf * utp;
      sv[inbc] = sv[inbc] + vsol * v[inbc] - cf * vtp;
      sw[inbc] = sw[inbc] + vsol * w[inbc] - cf * wtp;
    }
}

/* ap/su/apu assembly for one velocity component (calcuvw.f90:358-385,
   394-420, 431-457) */
static void calcuvw_assemble(cap_state* s, int comp) {
  const cappgpu_params* P = &s->prm;
  double *ae = s->f[CAP_AE], *aw = s->f[CAP_AW], *an = s->f[CAP_AN], *as = s->f[CAP_AS];
  double *at = s->f[CAP_AT], *ab = s->f[CAP_AB], *ap = s->f[CAP_AP], *su = s->f[CAP_SU];
  double* spx = comp == 0 ? 0 : comp == 1 ? s->f[CAP_SPV] : s->f[CAP_SP];
  double* srcx = comp == 0 ? s->f[CAP_SU] : comp == 1 ? s->f[CAP_SV] : s->f[CAP_SW];
  const double* fld = comp == 0 ? s->f[CAP_U] : comp == 1 ? s->f[CAP_V] : s->f[CAP_W];
  const double* old = comp == 0 ? s->f[CAP_UO] : comp == 1 ? s->f[CAP_VO] : s->f[CAP_WO];
  double* apx = comp == 0 ? s->f[CAP_APU] : comp == 1 ? s->f[CAP_APV] : s->f[CAP_APW];
  const double *den = s->f[CAP_DEN], *vol = s->f[CAP_VOL];
  int ifi = CAP_IU + comp;
  double urfrs = 1.0 / P->urf[ifi - 1];   /* urfr(i)=1./urf(i), init.f90:332 */
  double urfms = 1.0 - P->urf[ifi - 1];   /* urfm(i)=1.-urf(i), init.f90:333 */
  const int nj = s->nj, nij = s->nij;
  for (int k = 2; k <= s->nkm; ++k)
    for (int i = 3; i <= s->nimm; ++i)
      for (int j = 3; j <= s->njmm; ++j) {
        int inp = IXK(i, j, k);
        if (P->cn) {
          double apotime = den[inp] * vol[inp] / P->timestep;
          srcx[inp] = srcx[inp] + (ae[inp] * old[inp + nj] + aw[inp] * old[inp - nj] + an[inp] * old[inp + 1] +
                                   as[inp] * old[inp - 1] + at[inp] * old[inp + nij] + ab[inp] * old[inp - nij]) +
                      (apotime - ae[inp] - aw[inp] - an[inp] - as[inp] - at[inp] - ab[inp]) * old[inp];
          if (comp == 0) ap[inp] = ap[inp] + apotime;
          else spx[inp] = spx[inp] + apotime;
        }
        double diag = comp == 0 ? ap[inp] : spx[inp];
        ap[inp] = ae[inp] + aw[inp] + an[inp] + as[inp] + at[inp] + ab[inp] + diag;
        ap[inp] = ap[inp] * urfrs;
        su[inp] = srcx[inp] + urfms * ap[inp] * fld[inp];
        apx[inp] = 1.0 / (ap[inp] + SMALL);
      }
}

/* calcuvw.f90:3-464 with isol=1 (sipsol), gauss gradients */
int cap_calcuvw(cap_state* s, cappgpu_solve_report* rep3) {
  const cappgpu_params* P = &s->prm;
  /* the top-wall loop addresses lk(nimm) (calcuvw.f90:254); outside the
     array when nimm+1 > nk */
  if ((s->prm.top_plane ? s->nkmm : s->nimm) + 1 > s->nk) return CAPPGPU_E_ARG;
  cap_grad_gauss(s, CAP_U, CAP_GRADU_X, CAP_GRADU_Y, CAP_GRADU_Z);
  cap_grad_gauss(s, CAP_V, CAP_GRADV_X, CAP_GRADV_Y, CAP_GRADV_Z);
  cap_grad_gauss(s, CAP_W, CAP_GRADW_X, CAP_GRADW_Y, CAP_GRADW_Z);
  cap_grad_gauss(s, CAP_PP, CAP_GRADP_X, CAP_GRADP_Y, CAP_GRADP_Z);
  double *ap = s->f[CAP_AP], *spv = s->f[CAP_SPV], *sp = s->f[CAP_SP];
  double *su = s->f[CAP_SU], *sv = s->f[CAP_SV], *sw = s->f[CAP_SW];
  const double *gpx = s->f[CAP_GRADP_X], *gpy = s->f[CAP_GRADP_Y], *gpz = s->f[CAP_GRADP_Z];
  const double *vol = s->f[CAP_VOL], *den = s->f[CAP_DEN], *t = s->f[CAP_T];
  const double *uo = s->f[CAP_UO], *vo = s->f[CAP_VO], *wo = s->f[CAP_WO];
  const double *uoo = s->f[CAP_UOO], *voo = s->f[CAP_VOO], *woo = s->f[CAP_WOO];
  for (int k = 2; k <= s->nkm; ++k)
    for (int i = 3; i <= s->nimm; ++i)
      for (int j = 3; j <= s->njmm; ++j) {
        int inp = IXK(i, j, k);
        ap[inp] = 0.0; spv[inp] = 0.0; sp[inp] = 0.0;
        su[inp] = -gpx[inp] * vol[inp];
        sv[inp] = -gpy[inp] * vol[inp];
        sw[inp] = -gpz[inp] * vol[inp];
        if (P->const_mflux) su[inp] = su[inp] + P->gradpcmf * vol[inp];
        if (P->lcal[CAP_IEN - 1] && P->lbuoy) {
          double heat = 0.0;
          if (P->boussinesq) heat = P->beta * P->densit * (t[inp] - P->tref) * vol[inp];
          else heat = (P->densit - den[inp]) * vol[inp];
          su[inp] = su[inp] - P->gravx * heat;
          sv[inp] = sv[inp] - P->gravy * heat;
          sw[inp] = sw[inp] - P->gravz * heat;
        }
        if (P->bdf) {
          double apotime = den[inp] * vol[inp] / P->timestep;
          double sut = apotime * ((1 + P->btime) * uo[inp] - 0.5 * P->btime * uoo[inp]);
          double svt = apotime * ((1 + P->btime) * vo[inp] - 0.5 * P->btime * voo[inp]);
          double swt = apotime * ((1 + P->btime) * wo[inp] - 0.5 * P->btime * woo[inp]);
          su[inp] = su[inp] + sut;
          sv[inp] = sv[inp] + svt;
          sw[inp] = sw[inp] + swt;
          ap[inp] = ap[inp] + apotime * (1 + 0.5 * P->btime);
          spv[inp] = spv[inp] + apotime * (1 + 0.5 * P->btime);
          sp[inp] = sp[inp] + apotime * (1 + 0.5 * P->btime);
        }
      }
  /* calcstress (calcuvw.f90:129) only fills the Reynolds-stress arrays
     uu..vw, which the laminar/LES momentum assembly does not read. */
  cap_fluxuvw(s, s->nj, 1, s->nij, CAP_AR1X, CAP_AR1Y, CAP_AR1Z, CAP_FX, CAP_AE, CAP_AW, CAP_F1);
  cap_fluxuvw(s, 1, s->nij, s->nj, CAP_AR2X, CAP_AR2Y, CAP_AR2Z, CAP_FY, CAP_AN, CAP_AS, CAP_F2);
  cap_fluxuvw(s, s->nij, s->nj, 1, CAP_AR3X, CAP_AR3Y, CAP_AR3Z, CAP_FZ, CAP_AT, CAP_AB, CAP_F3);
  calcuvw_wall(s, 0);
  calcuvw_wall(s, 1);
  if (P->cn) {
    double* a[6] = {s->f[CAP_AE], s->f[CAP_AN], s->f[CAP_AT], s->f[CAP_AW], s->f[CAP_AS], s->f[CAP_AB]};
    for (int q = 0; q < 6; ++q)
      for (int c = 0; c < s->nijk; ++c) a[q][c] = 0.5 * a[q][c];
  }
  int rc = 0, r;
  calcuvw_assemble(s, 0);
  r = cap_sipsol(s, CAP_U, CAP_IU, rep3 ? &rep3[0] : 0); if (r < 0) return r; rc |= r;
  calcuvw_assemble(s, 1);
  r = cap_sipsol(s, CAP_V, CAP_IV, rep3 ? &rep3[1] : 0); if (r < 0) return r; rc |= r;
  calcuvw_assemble(s, 2);
  r = cap_sipsol(s, CAP_W, CAP_IW, rep3 ? &rep3[2] : 0); if (r < 0) return r; rc |= r;
  return rc;
}

/* ------------------------------------------------ pressure equation (PISO) */
/* PISO_assemble_pressure_eq.f90:3-257 */
void cap_piso_assemble_pressure_eq(cap_state* s, int idew, int idns, int idtb, int arvxf, int arvyf,
                                   int arvzf, int fiff, int acfef, int acfwf, int fcff, int ipc, int bpf) {
  const double *arvx = s->f[arvxf], *arvy = s->f[arvyf], *arvz = s->f[arvzf], *fif = s->f[fiff];
  double *acfe = s->f[acfef], *acfw = s->f[acfwf], *fcf = s->f[fcff], *bp = s->f[bpf];
  const double *x = s->f[CAP_X], *y = s->f[CAP_Y], *z = s->f[CAP_Z];
  const double *xc = s->f[CAP_XC], *yc = s->f[CAP_YC], *zc = s->f[CAP_ZC];
  const double *u = s->f[CAP_U], *v = s->f[CAP_V], *w = s->f[CAP_W], *p = s->f[CAP_P];
  const double *den = s->f[CAP_DEN], *vol = s->f[CAP_VOL], *apu = s->f[CAP_APU];
  const double *gux = s->f[CAP_GRADU_X], *guy = s->f[CAP_GRADU_Y], *guz = s->f[CAP_GRADU_Z];
  const double *gvx = s->f[CAP_GRADV_X], *gvy = s->f[CAP_GRADV_Y], *gvz = s->f[CAP_GRADV_Z];
  const double *gwx = s->f[CAP_GRADW_X], *gwy = s->f[CAP_GRADW_Y], *gwz = s->f[CAP_GRADW_Z];
  const double *gpx = s->f[CAP_GRADP_X], *gpy = s->f[CAP_GRADP_Y], *gpz = s->f[CAP_GRADP_Z];
  double* su = s->f[CAP_SU];
  memset(bp, 0, sizeof(double) * s->nijk);
  for (int k = 2; k <= s->nkmm; ++k)
    for (int i = 2; i <= s->nimm; ++i)
      for (int j = 2; j <= s->njmm; ++j) {
        int inp = IXK(i, j, k);
        int ine = inp + idew, ins = inp - idns, inb = inp - idtb, inbs = inb - idns;
        double fxe = fif[inp], fxp = 1.0 - fxe;
        double xf = 0.25 * (x[inp] + x[ins] + x[inb] + x[inbs]);
        double yf = 0.25 * (y[inp] + y[ins] + y[inb] + y[inbs]);
        double zf = 0.25 * (z[inp] + z[ins] + z[inb] + z[inbs]);
        double xi = xc[inp] * fxp + xc[ine] * fxe;
        double yi = yc[inp] * fxp + yc[ine] * fxe;
        double zi = zc[inp] * fxp + zc[ine] * fxe;
        double xpn = xc[ine] - xc[inp], ypn = yc[ine] - yc[inp], zpn = zc[ine] - zc[inp];
        double dpn = sqrt(xpn * xpn + ypn * ypn + zpn * zpn);
        double ixi1 = xpn / dpn, ixi2 = ypn / dpn, ixi3 = zpn / dpn;
        double arx = arvx[inp], ary = arvy[inp], arz = arvz[inp];
        double are = sqrt(arx * arx + ary * ary + arz * arz);
        double vole = xpn * arx + ypn * ary + zpn * arz;
        double nxx = arx / are, nyy = ary / are, nzz = arz / are;
        double costheta = nxx * ixi1 + nyy * ixi2 + nzz * ixi3;
        double costn = costheta;       /* minimal correction, :111 */
        double d1x = costn, d1y = costn, d1z = costn;
        double d2x = xpn * costn, d2y = ypn * costn, d2z = zpn * costn;
        double dene = den[inp] * fxp + den[ine] * fxe;
        double game = dene * (fxp * vol[inp] * apu[inp] + fxe * vol[ine] * apu[ine]);
        acfe[inp] = game * are / dpn;
        acfw[ine] = acfe[inp];
        if (ipc > 0) {
          double dfixi = gpx[inp] * fxp + gpx[ine] * fxe;
          double dfiyi = gpy[inp] * fxp + gpy[ine] * fxe;
          double dfizi = gpz[inp] * fxp + gpz[ine] * fxe;
          double dfixii = dfixi * d1x + arx / vole * (p[ine] - p[inp] - (dfixi * d2x + dfiyi * d2y + dfizi * d2z));
          double dfiyii = dfiyi * d1y + ary / vole * (p[ine] - p[inp] - (dfixi * d2x + dfiyi * d2y + dfizi * d2z));
          double dfizii = dfizi * d1z + arz / vole * (p[ine] - p[inp] - (dfixi * d2x + dfiyi * d2y + dfizi * d2z));
          double fdfie = game * (dfixii * arx + dfiyii * ary + dfizii * arz);
          double fdfii = game * are / dpn * (dfixi * xpn + dfiyi * ypn + dfizi * zpn);
          double suadd = fdfie - fdfii;
          su[inp] = su[inp] + suadd;
          bp[inp] = suadd;
          double duxi = gux[inp] * fxp + gux[ine] * fxe;
          double duyi = guy[inp] * fxp + guy[ine] * fxe;
          double duzi = guz[inp] * fxp + guz[ine] * fxe;
          double ui = u[inp] * fxp + u[ine] * fxe + duxi * (xf - xi) + duyi * (yf - yi) + duzi * (zf - zi);
          duxi = gvx[inp] * fxp + gvx[ine] * fxe;
          duyi = gvy[inp] * fxp + gvy[ine] * fxe;
          duzi = gvz[inp] * fxp + gvz[ine] * fxe;
          double vi = v[inp] * fxp + v[ine] * fxe + duxi * (xf - xi) + duyi * (yf - yi) + duzi * (zf - zi);
          duxi = gwx[inp] * fxp + gwx[ine] * fxe;
          duyi = gwy[inp] * fxp + gwy[ine] * fxe;
          duzi = gwz[inp] * fxp + gwz[ine] * fxe;
          double wi = w[inp] * fxp + w[ine] * fxe + duxi * (xf - xi) + duyi * (yf - yi) + duzi * (zf - zi);
          fcf[inp] = dene * (ui * arx + vi * ary + wi * arz);
        }
      }
  if (ipc > 0)
    for (int k = 3; k <= s->nkmm; ++k)
      for (int i = 3; i <= s->nimm; ++i)
        for (int j = 3; j <= s->njmm; ++j) {
          int inp = IXK(i, j, k) + idew;
          su[inp] = su[inp] - bp[inp];
        }
}

/* assemble_pressure_eq.f90:3-124 (not in the reference build) */
void cap_assemble_pressure_eq(cap_state* s, int idew, int idns, int idtb, int arvxf, int arvyf, int arvzf,
                              int fiff, int acfef, int acfwf, int fcff) {
  const double *arvx = s->f[arvxf], *arvy = s->f[arvyf], *arvz = s->f[arvzf], *fif = s->f[fiff];
  double *acfe = s->f[acfef], *acfw = s->f[acfwf], *fcf = s->f[fcff];
  const double *xc = s->f[CAP_XC], *yc = s->f[CAP_YC], *zc = s->f[CAP_ZC], *vol = s->f[CAP_VOL];
  const double *su = s->f[CAP_SU], *sv = s->f[CAP_SV], *sw = s->f[CAP_SW];
  for (int k = 2; k <= s->nkmm; ++k)
    for (int i = 2; i <= s->nimm; ++i)
      for (int j = 2; j <= s->njmm; ++j) {
        int inp = IXK(i, j, k), ine = inp + idew;
        double fxe = fif[inp], fxp = 1.0 - fxe;
        double xpn = xc[ine] - xc[inp], ypn = yc[ine] - yc[inp], zpn = zc[ine] - zc[inp];
        double arx = arvx[inp], ary = arvy[inp], arz = arvz[inp];
        double are = sqrt(arx * arx + ary * ary + arz * arz);
        double nxx = arx / are, nyy = ary / are, nzz = arz / are;
        double smdpn = (arx * arx + ary * ary + arz * arz) / (arx * xpn * nxx + ary * ypn * nyy + arz * zpn * nzz);
        acfe[inp] = (fxp * vol[inp] + fxe * vol[ine]) * smdpn;
        acfw[ine] = acfe[inp];
        double ui = su[inp] * fxp + su[ine] * fxe;
        double vi = sv[inp] * fxp + sv[ine] * fxe;
        double wi = sw[inp] * fxp + sw[ine] * fxe;
        fcf[inp] = ui * arx + vi * ary + wi * arz;
      }
}

/* ------------------------------------------------------------ PISO HbyA */
/* PISO_getHbyA.f90:3-233 */
void cap_piso_gethbya(cap_state* s) {
  const cappgpu_params* P = &s->prm;
  double *sp = s->f[CAP_SP], *su = s->f[CAP_SU], *sv = s->f[CAP_SV], *sw = s->f[CAP_SW];
  double *u = s->f[CAP_U], *v = s->f[CAP_V], *w = s->f[CAP_W];
  const double *he = s->f[CAP_HE], *hw = s->f[CAP_HW], *hn = s->f[CAP_HN], *hs = s->f[CAP_HS];
  const double *ht = s->f[CAP_HT], *hb = s->f[CAP_HB];
  const double *den = s->f[CAP_DEN], *vol = s->f[CAP_VOL], *t = s->f[CAP_T];
  const double *uo = s->f[CAP_UO], *vo = s->f[CAP_VO], *wo = s->f[CAP_WO];
  const double *uoo = s->f[CAP_UOO], *voo = s->f[CAP_VOO], *woo = s->f[CAP_WOO];
  const double *apu = s->f[CAP_APU], *apv = s->f[CAP_APV], *apw = s->f[CAP_APW];
  const int nj = s->nj, nij = s->nij;
  for (int k = 3; k <= s->nkmm; ++k)
    for (int i = 3; i <= s->nimm; ++i)
      for (int j = 3; j <= s->njmm; ++j) {
        int inp = IXK(i, j, k);
        sp[inp] = 0.0; su[inp] = 0.0; sv[inp] = 0.0; sw[inp] = 0.0;
        if (P->lcal[CAP_IEN - 1] && P->lbuoy) {
          double heat = 0.0;
          if (P->boussinesq) heat = P->beta * P->densit * (t[inp] - P->tref) * vol[inp];
          else heat = (P->densit - den[inp]) * vol[inp];
          su[inp] = su[inp] - P->gravx * heat;
          sv[inp] = sv[inp] - P->gravy * heat;
          sw[inp] = sw[inp] - P->gravz * heat;
        }
        if (P->bdf) {
          double apotime = den[inp] * vol[inp] / P->timestep;
          double sut = apotime * ((1 + P->btime) * uo[inp] - 0.5 * P->btime * uoo[inp]);
          double svt = apotime * ((1 + P->btime) * vo[inp] - 0.5 * P->btime * voo[inp]);
          double swt = apotime * ((1 + P->btime) * wo[inp] - 0.5 * P->btime * woo[inp]);
          su[inp] = su[inp] + sut;
          sv[inp] = sv[inp] + svt;
          sw[inp] = sw[inp] + swt;
        }
      }
  const double* fld[3] = {u, v, w};
  const double* old[3] = {uo, vo, wo};
  double* src[3] = {su, sv, sw};
  for (int c = 0; c < 3; ++c) {
    const double* f = fld[c];
    const double* o = old[c];
    double* q = src[c];
    for (int k = 3; k <= s->nkmm; ++k)
      for (int i = 3; i <= s->nimm; ++i)
        for (int j = 3; j <= s->njmm; ++j) {
          int inp = IXK(i, j, k);
          int ine = inp + nj, inw = inp - nj, inn = inp + 1, ins = inp - 1, int_ = inp + nij, inb = inp - nij;
          if (P->cn) {
            double apotime = den[inp] * vol[inp] / P->timestep;
            q[inp] = q[inp] + (he[inp] * o[ine] + hw[inp] * o[inw] + hn[inp] * o[inn] + hs[inp] * o[ins] +
                               ht[inp] * o[int_] + hb[inp] * o[inb]) +
                     (apotime - he[inp] - hw[inp] - hn[inp] - hs[inp] - ht[inp] - hb[inp]) * o[inp];
          }
          q[inp] = q[inp] + (he[inp] * f[ine] + hw[inp] * f[inw] + hn[inp] * f[inn] + hs[inp] * f[ins] +
                             ht[inp] * f[int_] + hb[inp] * f[inb]);
        }
  }
  for (int k = 3; k <= s->nkmm; ++k)
    for (int i = 3; i <= s->nimm; ++i)
      for (int j = 3; j <= s->njmm; ++j) {
        int inp = IXK(i, j, k);
        u[inp] = su[inp] * apu[inp];
        v[inp] = sv[inp] * apv[inp];
        w[inp] = sw[inp] * apw[inp];
      }
  cap_grad_gauss(s, CAP_U, CAP_GRADU_X, CAP_GRADU_Y, CAP_GRADU_Z);
  cap_grad_gauss(s, CAP_V, CAP_GRADV_X, CAP_GRADV_Y, CAP_GRADV_Z);
  cap_grad_gauss(s, CAP_W, CAP_GRADW_X, CAP_GRADW_Y, CAP_GRADW_Z);
}

/* --------------------------------------------------- continuity / Courant */
/* continuityErrors.h:55-83 */
void cap_continuity_errors(cap_state* s) {
  cappgpu_params* P = &s->prm;
  const double *f1 = s->f[CAP_F1], *f2 = s->f[CAP_F2], *f3 = s->f[CAP_F3];
  const int idew = s->nj, idns = 1, idtb = s->nij;
  double local = 0.0, glob = 0.0, sumloc = 0.0;
  for (int k = 2; k <= s->nkm; ++k)
    for (int i = 3; i <= s->nimm; ++i)
      for (int j = 3; j <= s->njmm; ++j) {
        int inp = IXK(i, j, k);
        local = -f1[inp] + f1[inp - idew] - f2[inp] + f2[inp - idns] - f3[inp] + f3[inp - idtb];
        glob = glob + local;
        sumloc = sumloc + fabs(local);
      }
  P->localconterr = local;
  P->globalconterr = glob;
  P->sumlocalconterr = sumloc;
  P->cumulativeconterr = P->cumulativeconterr + glob;
}

/* CourantNo.h:10-66 (su used as scratch, zeroed first, :32) */
void cap_courant(cap_state* s) {
  cappgpu_params* P = &s->prm;
  if (!P->ltransient) return;
  double* su = s->f[CAP_SU];
  const double *f1 = s->f[CAP_F1], *f2 = s->f[CAP_F2], *f3 = s->f[CAP_F3], *vol = s->f[CAP_VOL];
  double conum = 0.0, meanconum = 0.0, suma = 0.0;
  memset(su, 0, sizeof(double) * s->nijk);
  for (int k = 2; k <= s->nkm; ++k)
    for (int i = 3; i <= s->nimm; ++i)
      for (int j = 3; j <= s->njmm; ++j) {
        int inp = IXK(i, j, k);
        su[inp] = fabs(f1[inp]) + fabs(f1[inp - s->nj]) + fabs(f2[inp]) + fabs(f2[inp - 1]) + fabs(f3[inp]) +
                  fabs(f3[inp - s->nij]);
        conum = dmax(conum, su[inp] / vol[inp]);
        suma = suma + vol[inp];
        meanconum = meanconum + su[inp];
      }
  conum = 0.5 * conum * P->timestep;
  meanconum = 0.5 * meanconum / suma * P->timestep;
  /* global_max(CoNum): identity on one rank */
  if (P->conumfix) {
    double dt = P->timestep;
    P->timestep = P->conumfixvalue / conum * P->timestep;
    conum = conum * P->timestep / dt;
    meanconum = meanconum * P->timestep / dt;
  }
  P->time = P->time + P->timestep;
  P->conum = conum;
  P->meanconum = meanconum;
}

/* ------------------------------------------------------------ PISO loop */
/* PISO_multiple_correction.f90:3-296 (fluxmc/const_mflux paths commented
   out in the reference are not taken) */
int cap_piso_multiple_correction(cap_state* s, cappgpu_solve_report* reps) {
  cappgpu_params* P = &s->prm;
  double reltol = P->sor[CAP_IP - 1];
  const int n = s->nijk;
  memcpy(s->f[CAP_HE], s->f[CAP_AE], sizeof(double) * n);
  memcpy(s->f[CAP_HW], s->f[CAP_AW], sizeof(double) * n);
  memcpy(s->f[CAP_HN], s->f[CAP_AN], sizeof(double) * n);
  memcpy(s->f[CAP_HS], s->f[CAP_AS], sizeof(double) * n);
  memcpy(s->f[CAP_HT], s->f[CAP_AT], sizeof(double) * n);
  memcpy(s->f[CAP_HB], s->f[CAP_AB], sizeof(double) * n);
  memset(s->f[CAP_GRADP_X], 0, sizeof(double) * n);
  memset(s->f[CAP_GRADP_Y], 0, sizeof(double) * n);
  memset(s->f[CAP_GRADP_Z], 0, sizeof(double) * n);
  memset(s->f[CAP_P], 0, sizeof(double) * n);
  double *su = s->f[CAP_SU], *ap = s->f[CAP_AP], *p = s->f[CAP_P];
  double *ae = s->f[CAP_AE], *aw = s->f[CAP_AW], *an = s->f[CAP_AN], *as = s->f[CAP_AS];
  double *at = s->f[CAP_AT], *ab = s->f[CAP_AB];
  double *f1 = s->f[CAP_F1], *f2 = s->f[CAP_F2], *f3 = s->f[CAP_F3];
  double *u = s->f[CAP_U], *v = s->f[CAP_V], *w = s->f[CAP_W];
  const double *apu = s->f[CAP_APU], *apv = s->f[CAP_APV], *apw = s->f[CAP_APW], *vol = s->f[CAP_VOL];
  const double *gpx = s->f[CAP_GRADP_X], *gpy = s->f[CAP_GRADP_Y], *gpz = s->f[CAP_GRADP_Z];
  int rc = 0, nrep = 0;
  for (P->icorr = 1; P->icorr <= P->ncorr; ++P->icorr) {
    cap_piso_gethbya(s);
    for (P->ipcorr = 1; P->ipcorr <= P->npcor; ++P->ipcorr) {
      int ipc = P->ipcorr;
      cap_piso_assemble_pressure_eq(s, s->nj, 1, s->nij, CAP_AR1X, CAP_AR1Y, CAP_AR1Z, CAP_FX, CAP_AE, CAP_AW, CAP_F1, ipc, CAP_BE);
      cap_piso_assemble_pressure_eq(s, 1, s->nij, s->nj, CAP_AR2X, CAP_AR2Y, CAP_AR2Z, CAP_FY, CAP_AN, CAP_AS, CAP_F2, ipc, CAP_BN);
      cap_piso_assemble_pressure_eq(s, s->nij, s->nj, 1, CAP_AR3X, CAP_AR3Y, CAP_AR3Z, CAP_FZ, CAP_AT, CAP_AB, CAP_F3, ipc, CAP_BT);
      const int idew = s->nj, idns = 1, idtb = s->nij;
      if (P->ipcorr == 1) {
        if (!P->const_mflux) cap_outbc(s);
        for (int k = 3; k <= s->nkmm; ++k)
          for (int i = 3; i <= s->nimm; ++i)
            for (int j = 3; j <= s->njmm; ++j) {
              int inp = IXK(i, j, k);
              su[inp] = -f1[inp] + f1[inp - idew] - f2[inp] + f2[inp - idns] - f3[inp] + f3[inp - idtb];
            }
      }
      for (int k = 3; k <= s->nkmm; ++k)
        for (int i = 3; i <= s->nimm; ++i)
          for (int j = 3; j <= s->njmm; ++j) {
            int inp = IXK(i, j, k);
            ap[inp] = ae[inp] + aw[inp] + an[inp] + as[inp] + at[inp] + ab[inp];
          }
      int inpr = IXK(P->ipr, P->jpr, P->kpr);
      ap[inpr] = 1.0;
      ae[inpr] = 0.0; aw[inpr] = 0.0; an[inpr] = 0.0; as[inpr] = 0.0; at[inpr] = 0.0; ab[inpr] = 0.0;
      double ppref = p[inpr];
      su[inpr] = ppref;
      if (P->icorr != P->ncorr) P->sor[CAP_IP - 1] = (double)0.1f;  /* sor(ip) = 0.1, :132 */
      else P->sor[CAP_IP - 1] = reltol;
      int r = cap_solve_dispatch(s, P->piso_solver, CAP_P, CAP_IP, reps ? &reps[nrep] : 0);
      ++nrep;
      if (r < 0) return r;
      rc |= r;
      cap_bpres(s, CAP_P);
      cap_grad_gauss(s, CAP_P, CAP_GRADP_X, CAP_GRADP_Y, CAP_GRADP_Z);
      if (P->ipcorr == P->npcor) {
        for (int k = 2; k <= s->nkmm; ++k)
          for (int i = 2; i <= s->nimm; ++i)
            for (int j = 2; j <= s->njmm; ++j) {
              int inp = IXK(i, j, k);
              int ine = inp + idew, inn = inp + idns, int_ = inp + idtb;
              f1[inp] = f1[inp] - ae[inp] * (p[ine] - p[inp]);
              f2[inp] = f2[inp] - an[inp] * (p[inn] - p[inp]);
              f3[inp] = f3[inp] - at[inp] * (p[int_] - p[inp]);
            }
      }
    }
    P->ipcorr = P->npcor + 1;
    cap_continuity_errors(s);
    for (int k = 3; k <= s->nkmm; ++k)
      for (int i = 3; i <= s->nimm; ++i)
        for (int j = 3; j <= s->njmm; ++j) {
          int inp = IXK(i, j, k);
          u[inp] = u[inp] - apu[inp] * gpx[inp] * vol[inp];
          v[inp] = v[inp] - apv[inp] * gpy[inp] * vol[inp];
          w[inp] = w[inp] - apw[inp] * gpz[inp] * vol[inp];
        }
  }
  memcpy(s->f[CAP_PP], s->f[CAP_P], sizeof(double) * n);
  return rc;
}

/* ------------------------------------------------------------ SIMPLE */
/* fluxmass2.f90:3-195 */
void cap_fluxmass(cap_state* s, int idew, int idns, int idtb, int arvxf, int arvyf, int arvzf,
                  int fiff, int acfef, int acfwf, int fcff) {
  const double *arvx = s->f[arvxf], *arvy = s->f[arvyf], *arvz = s->f[arvzf], *fif = s->f[fiff];
  double *acfe = s->f[acfef], *acfw = s->f[acfwf], *fcf = s->f[fcff];
  const double *x = s->f[CAP_X], *y = s->f[CAP_Y], *z = s->f[CAP_Z];
  const double *xc = s->f[CAP_XC], *yc = s->f[CAP_YC], *zc = s->f[CAP_ZC];
  const double *u = s->f[CAP_U], *v = s->f[CAP_V], *w = s->f[CAP_W], *p = s->f[CAP_P];
  const double *den = s->f[CAP_DEN], *vol = s->f[CAP_VOL];
  const double *apu = s->f[CAP_APU], *apv = s->f[CAP_APV], *apw = s->f[CAP_APW];
  const double *gux = s->f[CAP_GRADU_X], *guy = s->f[CAP_GRADU_Y], *guz = s->f[CAP_GRADU_Z];
  const double *gvx = s->f[CAP_GRADV_X], *gvy = s->f[CAP_GRADV_Y], *gvz = s->f[CAP_GRADV_Z];
  const double *gwx = s->f[CAP_GRADW_X], *gwy = s->f[CAP_GRADW_Y], *gwz = s->f[CAP_GRADW_Z];
  const double *gpx = s->f[CAP_GRADP_X], *gpy = s->f[CAP_GRADP_Y], *gpz = s->f[CAP_GRADP_Z];
  for (int k = 2; k <= s->nkm; ++k)
    for (int i = 2; i <= s->nimm; ++i)
      for (int j = 2; j <= s->njmm; ++j) {
        int inp = IXK(i, j, k);
        int ine = inp + idew, ins = inp - idns, inb = inp - idtb, inbs = inb - idns;
        double fxe = fif[inp], fxp = 1.0 - fxe;
        double xf = 0.25 * (x[inp] + x[ins] + x[inb] + x[inbs]);
        double yf = 0.25 * (y[inp] + y[ins] + y[inb] + y[inbs]);
        double zf = 0.25 * (z[inp] + z[ins] + z[inb] + z[inbs]);
        double xi = xc[inp] * fxp + xc[ine] * fxe;
        double yi = yc[inp] * fxp + yc[ine] * fxe;
        double zi = zc[inp] * fxp + zc[ine] * fxe;
        double xpn = xc[ine] - xc[inp], ypn = yc[ine] - yc[inp], zpn = zc[ine] - zc[inp];
        double arx = arvx[inp], ary = arvy[inp], arz = arvz[inp];
        double are = sqrt(arx * arx + ary * ary + arz * arz);
        double nxx = arx / are, nyy = ary / are, nzz = arz / are;
        double sfdpnr = 1.0 / (arx * xpn * nxx + ary * ypn * nyy + arz * zpn * nzz);
        double dene = den[inp] * fxp + den[ine] * fxe;
        double smdpn = (arx * arx + ary * ary + arz * arz) * sfdpnr;
        acfe[inp] = dene * (fxp * vol[inp] * apu[inp] + fxe * vol[ine] * apu[ine]) * smdpn;
        acfw[ine] = acfe[inp];
        double duxi = gux[inp] * fxp + gux[ine] * fxe;
        double duyi = guy[inp] * fxp + guy[ine] * fxe;
        double duzi = guz[inp] * fxp + guz[ine] * fxe;
        double ui = u[inp] * fxp + u[ine] * fxe + (duxi * (xf - xi) + duyi * (yf - yi) + duzi * (zf - zi));
        duxi = gvx[inp] * fxp + gvx[ine] * fxe;
        duyi = gvy[inp] * fxp + gvy[ine] * fxe;
        duzi = gvz[inp] * fxp + gvz[ine] * fxe;
        double vi = v[inp] * fxp + v[ine] * fxe + (duxi * (xf - xi) + duyi * (yf - yi) + duzi * (zf - zi));
        duxi = gwx[inp] * fxp + gwx[ine] * fxe;
        duyi = gwy[inp] * fxp + gwy[ine] * fxe;
        duzi = gwz[inp] * fxp + gwz[ine] * fxe;
        double wi = w[inp] * fxp + w[ine] * fxe + (duxi * (xf - xi) + duyi * (yf - yi) + duzi * (zf - zi));
        double dpxi = (fxe * vol[ine] * apu[ine] + fxp * vol[inp] * apu[inp]) * (fxe * gpx[ine] + fxp * gpx[inp]) * xpn * nxx;
        double dpyi = (fxe * vol[ine] * apv[ine] + fxp * vol[inp] * apv[inp]) * (fxe * gpy[ine] + fxp * gpy[inp]) * ypn * nyy;
        double dpzi = (fxe * vol[ine] * apw[ine] + fxp * vol[inp] * apw[inp]) * (fxe * gpz[ine] + fxp * gpz[inp]) * zpn * nzz;
        double xpp = xf - (xf - xc[inp]) * nxx, ypp = yf - (yf - yc[inp]) * nyy, zpp = zf - (zf - zc[inp]) * nzz;
        double xep = xf - (xf - xc[ine]) * nxx, yep = yf - (yf - yc[ine]) * nyy, zep = zf - (zf - zc[ine]) * nzz;
        xpp = xpp - xc[inp]; ypp = ypp - yc[inp]; zpp = zpp - zc[inp];
        xep = xep - xc[ine]; yep = yep - yc[ine]; zep = zep - zc[ine];
        /* operator precedence of the reference kept (fluxmass2.f90:171-173):
           only the first inp term is subtracted */
        double dpe = (p[ine] - p[inp]) +
                     (gpx[ine] * xep + gpy[ine] * yep + gpz[ine] * zep - gpx[inp] * xpp + gpy[inp] * ypp + gpz[inp] * zpp);
        double dpex = (fxe * vol[ine] * apu[ine] + fxp * vol[inp] * apu[inp]) * (arx * sfdpnr) * dpe;
        double dpey = (fxe * vol[ine] * apv[ine] + fxp * vol[inp] * apv[inp]) * (ary * sfdpnr) * dpe;
        double dpez = (fxe * vol[ine] * apw[ine] + fxp * vol[inp] * apw[inp]) * (arz * sfdpnr) * dpe;
        double ue = ui - dpex + dpxi, ve = vi - dpey + dpyi, we = wi - dpez + dpzi;
        fcf[inp] = dene * (ue * arx + ve * ary + we * arz);
      }
}

/* fluxmc.f90:3-109; inp1 is the 0-based storage index of the reference inp */
double cap_fluxmc(cap_state* s, int inp, int idew, int idns, int idtb, int fiff) {
  const double* fif = s->f[fiff];
  const double *x = s->f[CAP_X], *y = s->f[CAP_Y], *z = s->f[CAP_Z];
  const double *xc = s->f[CAP_XC], *yc = s->f[CAP_YC], *zc = s->f[CAP_ZC];
  const double *apu = s->f[CAP_APU], *den = s->f[CAP_DEN], *vol = s->f[CAP_VOL];
  const double *gpx = s->f[CAP_GRADP_X], *gpy = s->f[CAP_GRADP_Y], *gpz = s->f[CAP_GRADP_Z];
  int ine = inp + idew, ins = inp - idns, inb = inp - idtb, inbs = inb - idns;
  double fxe = fif[inp], fxp = 1.0 - fxe;
  double arx, ary, arz;
  if (idew == s->nj) { arx = s->f[CAP_AR1X][inp]; ary = s->f[CAP_AR1Y][inp]; arz = s->f[CAP_AR1Z][inp]; }
  else if (idew == 1) { arx = s->f[CAP_AR2X][inp]; ary = s->f[CAP_AR2Y][inp]; arz = s->f[CAP_AR2Z][inp]; }
  else { arx = s->f[CAP_AR3X][inp]; ary = s->f[CAP_AR3Y][inp]; arz = s->f[CAP_AR3Z][inp]; }
  double xpn = xc[ine] - xc[inp], ypn = yc[ine] - yc[inp], zpn = zc[ine] - zc[inp];
  double are = sqrt(arx * arx + ary * ary + arz * arz);
  double nxx = arx / are, nyy = ary / are, nzz = arz / are;
  double dppnnr = 1.0 / ((xpn * nxx) + (ypn * nyy) + (zpn * nzz));
  double xf = 0.25 * (x[inp] + x[ins] + x[inb] + x[inbs]);
  double yf = 0.25 * (y[inp] + y[ins] + y[inb] + y[inbs]);
  double zf = 0.25 * (z[inp] + z[ins] + z[inb] + z[inbs]);
  double xpp = xf - (xf - xc[inp]) * nxx, ypp = yf - (yf - yc[inp]) * nyy, zpp = zf - (zf - zc[inp]) * nzz;
  double xep = xf - (xf - xc[ine]) * nxx, yep = yf - (yf - yc[ine]) * nyy, zep = zf - (zf - zc[ine]) * nzz;
  xpp = xpp - xc[inp]; ypp = ypp - yc[inp]; zpp = zpp - zc[inp];
  xep = xep - xc[ine]; yep = yep - yc[ine]; zep = zep - zc[ine];
  double rapr = (apu[inp] * den[inp] * vol[inp] * fxp + apu[ine] * den[ine] * vol[ine] * fxe);
  return rapr * are *
         ((gpx[ine] * xep - gpx[inp] * xpp) + (gpy[ine] * yep - gpy[inp] * ypp) + (gpz[ine] * zep - gpz[inp] * zpp)) *
         dppnnr;
}

/* outbc.f90:3-318: with an outlet (lout), the mass flux through the outlet
   faces (code 2) of every face set whose flag low..lot is set is formed --
   den(ghost) times u(interior) dotted with ar1x,ar1y,ar1z of the ghost for
   all six sets, as the reference writes it -- and summed in the routine's
   loop order (flow: minus on west/south/bottom, plus on east/north/top);
   then every outlet ghost takes the interior velocity times
   fac = flowin/(flow+small), its flux is scaled by fac, and te, ed, vis, t
   are copied from the interior (vart, con, utt, vtt, wtt have no field
   here).  Face sets: 0 W, 1 E, 2 S, 3 N, 4 B, 5 T. */
static void outbc_set(cap_state* s, int set, int pass, double fac, double* flow) {
  const cappgpu_params* P = &s->prm;
  const int on[6] = {P->low, P->loe, P->los, P->lon, P->lob, P->lot};
  if (!on[set]) return;
  static const int bcf[6] = {CAP_LBW, CAP_LBE, CAP_LBS, CAP_LBN, CAP_LBB, CAP_LBT};
  static const int ff[6] = {CAP_F1, CAP_F1, CAP_F2, CAP_F2, CAP_F3, CAP_F3};
  double *u = s->f[CAP_U], *v = s->f[CAP_V], *w = s->f[CAP_W], *f = s->f[ff[set]];
  double *te = s->f[CAP_TE], *ed = s->f[CAP_ED], *vis = s->f[CAP_VIS], *t = s->f[CAP_T];
  const double *den = s->f[CAP_DEN], *a1x = s->f[CAP_AR1X], *a1y = s->f[CAP_AR1Y], *a1z = s->f[CAP_AR1Z];
  /* outer x inner loop ranges: k,j (W/E); k,i (S/N); i,j (B/T) */
  const int o_hi = set < 4 ? s->nkm : s->nim;
  const int i_hi = (set == 2 || set == 3) ? s->nim : s->njm;
  for (int o = 2; o <= o_hi; ++o)
    for (int q = 2; q <= i_hi; ++q) {
      int inp, inbc, inh, at;
      switch (set) {
        case 0: inp = IXK(2, q, o); inbc = (q - 1) * s->nk + o; inh = inp + s->nj; at = inp; break;
        case 1: inp = IXK(s->nim, q, o); inbc = (q - 1) * s->nk + o; inh = inp - s->nj; at = inh; break;
        case 2: inp = IXK(q, 2, o); inbc = (q - 1) * s->nk + o; inh = inp + 1; at = inp; break;
        case 3: inp = IXK(q, s->njm, o); inbc = (q - 1) * s->nk + o; inh = inp - 1; at = inh; break;
        case 4: inp = IXK(o, q, 2); inbc = (o - 1) * s->nj + q; inh = inp + s->nij; at = inp; break;
        default: inp = IXK(o, q, s->nkm); inbc = (o - 1) * s->nj + q; inh = inp - s->nij; at = inh; break;
      }
      if (s->bc[bcf[set]][inbc - 1] != 2) continue;
      if (pass == 0) {
        f[at] = den[inp] * (a1x[inp] * u[inh] + a1y[inp] * v[inh] + a1z[inp] * w[inh]);
        *flow = (set & 1) ? *flow + f[at] : *flow - f[at];
      } else {
        u[inp] = u[inh] * fac;
        v[inp] = v[inh] * fac;
        w[inp] = w[inh] * fac;
        f[at] = f[at] * fac;
        te[inp] = te[inh];
        ed[inp] = ed[inh];
        vis[inp] = vis[inh];
        t[inp] = t[inh];
      }
    }
}

void cap_outbc(cap_state* s) {
  if (!s->prm.lout) return;   /* outbc.f90:31 */
  double flow = 0.0;
  for (int set = 0; set < 6; ++set) outbc_set(s, set, 0, 0.0, &flow);
  const double fac = s->prm.flowin / (flow + SMALL);   /* :147 */
  for (int set = 0; set < 6; ++set) outbc_set(s, set, 1, fac, &flow);
}

/* correctBoundaryConditions.f90:1-86 (periodic copies into the padding
   layers i=1,ni and j=1,nj) */
void cap_correct_boundary_conditions(cap_state* s) {
  double *u = s->f[CAP_U], *v = s->f[CAP_V], *w = s->f[CAP_W], *f1 = s->f[CAP_F1], *f2 = s->f[CAP_F2];
  for (int k = 2; k <= s->nkm; ++k)
    for (int j = 2; j <= s->njm; ++j) {
      int inp = IXK(s->ni, j, k), inh = IXK(2, j, k);
      u[inp] = u[inh]; v[inp] = v[inh]; w[inp] = w[inh];
    }
  for (int k = 2; k <= s->nkm; ++k)
    for (int j = 2; j <= s->njm; ++j) {
      /* li(njm) as in the reference (correctBoundaryConditions.f90:44) */
      int inp = IXK(1, j, k), inh = s->lk[k] + s->li[s->njm] + j - 1;
      u[inp] = u[inh]; v[inp] = v[inh]; w[inp] = w[inh];
      f1[inp] = f1[inh];
    }
  for (int k = 2; k <= s->nkm; ++k)
    for (int i = 2; i <= s->nim; ++i) {
      int inp = IXK(i, s->nj, k), inh = IXK(i, 2, k);
      u[inp] = u[inh]; v[inp] = v[inh]; w[inp] = w[inh];
    }
  for (int k = 2; k <= s->nkm; ++k)
    for (int i = 2; i <= s->nim; ++i) {
      int inp = IXK(i, 1, k), inh = IXK(i, s->njm, k);
      u[inp] = u[inh]; v[inp] = v[inh]; w[inp] = w[inh];
      f2[inp] = f2[inh];
    }
}

/* calcp-multiple_correction_SIMPLE.f90:3-238 */
int cap_calcp(cap_state* s, cappgpu_solve_report* reps) {
  cappgpu_params* P = &s->prm;
  const int idew = s->nj, idns = 1, idtb = s->nij;
  double *su = s->f[CAP_SU], *ap = s->f[CAP_AP], *pp = s->f[CAP_PP], *p = s->f[CAP_P];
  double *ae = s->f[CAP_AE], *aw = s->f[CAP_AW], *an = s->f[CAP_AN], *as = s->f[CAP_AS];
  double *at = s->f[CAP_AT], *ab = s->f[CAP_AB];
  double *f1 = s->f[CAP_F1], *f2 = s->f[CAP_F2], *f3 = s->f[CAP_F3];
  double *u = s->f[CAP_U], *v = s->f[CAP_V], *w = s->f[CAP_W];
  const double *apu = s->f[CAP_APU], *apv = s->f[CAP_APV], *apw = s->f[CAP_APW], *vol = s->f[CAP_VOL];
  const double *gpx = s->f[CAP_GRADP_X], *gpy = s->f[CAP_GRADP_Y], *gpz = s->f[CAP_GRADP_Z];
  int rc = 0, nrep = 0;
  for (P->icorr = 1; P->icorr <= P->ncorr; ++P->icorr) {
    cap_grad_gauss(s, CAP_U, CAP_GRADU_X, CAP_GRADU_Y, CAP_GRADU_Z);
    cap_grad_gauss(s, CAP_V, CAP_GRADV_X, CAP_GRADV_Y, CAP_GRADV_Z);
    cap_grad_gauss(s, CAP_W, CAP_GRADW_X, CAP_GRADW_Y, CAP_GRADW_Z);
    cap_fluxmass(s, s->nj, 1, s->nij, CAP_AR1X, CAP_AR1Y, CAP_AR1Z, CAP_FX, CAP_AE, CAP_AW, CAP_F1);
    cap_fluxmass(s, 1, s->nij, s->nj, CAP_AR2X, CAP_AR2Y, CAP_AR2Z, CAP_FY, CAP_AN, CAP_AS, CAP_F2);
    cap_fluxmass(s, s->nij, s->nj, 1, CAP_AR3X, CAP_AR3Y, CAP_AR3Z, CAP_FZ, CAP_AT, CAP_AB, CAP_F3);
    if (!P->const_mflux) cap_outbc(s);
    for (int k = 3; k <= s->nkmm; ++k)
      for (int i = 3; i <= s->nimm; ++i)
        for (int j = 3; j <= s->njmm; ++j) {
          int inp = IXK(i, j, k);
          su[inp] = -f1[inp] + f1[inp - idew] - f2[inp] + f2[inp - idns] - f3[inp] + f3[inp - idtb];
          ap[inp] = ae[inp] + aw[inp] + an[inp] + as[inp] + at[inp] + ab[inp];
        }
    for (P->ipcorr = 1; P->ipcorr <= P->npcor; ++P->ipcorr) {
      memset(pp, 0, sizeof(double) * s->nijk);
      int r = cap_solve_dispatch(s, P->isol_p, CAP_PP, CAP_IP, reps ? &reps[nrep] : 0);
      ++nrep;
      if (r < 0) return r;
      rc |= r;
      double ppref = pp[IXK(P->ipr, P->jpr, P->kpr)];
      cap_grad_gauss(s, CAP_PP, CAP_GRADP_X, CAP_GRADP_Y, CAP_GRADP_Z);
      if (P->ipcorr != P->npcor) {
        memset(su, 0, sizeof(double) * s->nijk);
        for (int k = 3; k <= s->nkmm; ++k)
          for (int i = 3; i <= s->nimm; ++i)
            for (int j = 3; j <= s->njmm; ++j) {
              int inp = IXK(i, j, k);
              int ine = inp + idew, inn = inp + idns, int_ = inp + idtb;
              double fmcor = cap_fluxmc(s, inp, s->nj, 1, s->nij, CAP_FX);
              f1[inp] = f1[inp] - fmcor; su[inp] = su[inp] + fmcor; su[ine] = su[ine] - fmcor;
              fmcor = cap_fluxmc(s, inp, 1, s->nij, s->nj, CAP_FY);
              f2[inp] = f2[inp] - fmcor; su[inp] = su[inp] + fmcor; su[inn] = su[inn] - fmcor;
              fmcor = cap_fluxmc(s, inp, s->nij, s->nj, 1, CAP_FZ);
              f3[inp] = f3[inp] - fmcor; su[inp] = su[inp] + fmcor; su[int_] = su[int_] - fmcor;
            }
      }
      for (int k = 3; k <= s->nkmm; ++k)
        for (int i = 3; i <= s->nimm; ++i)
          for (int j = 3; j <= s->njmm; ++j) {
            int inp = IXK(i, j, k);
            int ine = inp + idew, inn = inp + idns, int_ = inp + idtb;
            f1[inp] = f1[inp] - ae[inp] * (pp[ine] - pp[inp]);
            f2[inp] = f2[inp] - an[inp] * (pp[inn] - pp[inp]);
            f3[inp] = f3[inp] - at[inp] * (pp[int_] - pp[inp]);
          }
      for (int k = 3; k <= s->nkmm; ++k)
        for (int i = 3; i <= s->nimm; ++i)
          for (int j = 3; j <= s->njmm; ++j) {
            int inp = IXK(i, j, k);
            u[inp] = u[inp] - vol[inp] * apu[inp] * gpx[inp];
            v[inp] = v[inp] - vol[inp] * apv[inp] * gpy[inp];
            w[inp] = w[inp] - vol[inp] * apw[inp] * gpz[inp];
            p[inp] = p[inp] + P->urf[CAP_IP - 1] * (pp[inp] - ppref);
          }
    }
    P->ipcorr = P->npcor + 1;
    cap_continuity_errors(s);
    cap_correct_boundary_conditions(s);
  }
  cap_bpres(s, CAP_P);
  memcpy(pp, p, sizeof(double) * s->nijk);
  return rc;
}

/* ------------------------------------------------------------ drivers */
/* --------------------------------------------------- constant mass flux */
/* const_massflux_correction.f90:1-22 (included at main.f90:252 at the end
   of a transient step): volume-weighted averages of U and APU over
   k = 2..nkm, i = 3..nimm, j = 3..njmm (fieldManipulation.f90:10-44, summed
   in loop order), the pressure-gradient increment that restores the bulk
   velocity magUbar = uin (init.f90:356), applied to the whole U array. */
void cap_const_massflux_correction(cap_state* s) {
  cappgpu_params* P = &s->prm;
  const double *vol = s->f[CAP_VOL], *apu = s->f[CAP_APU];
  double* u = s->f[CAP_U];
  double su = 0.0, sa = 0.0, sv = 0.0;
  for (int k = 2; k <= s->nkm; ++k)
    for (int i = 3; i <= s->nimm; ++i)
      for (int j = 3; j <= s->njmm; ++j) {
        const int inp = IXK(i, j, k);
        sv = sv + vol[inp];
        su = su + vol[inp] * u[inp];
        sa = sa + vol[inp] * apu[inp];
      }
  const double mag_ubar_star = su / sv;
  const double rua = sa / sv;
  const double dgrad = (P->uin - mag_ubar_star) / rua;
  const double flow_direction = 1.0;
  for (int q = 0; q < s->nijk; ++q) u[q] = u[q] + flow_direction * apu[q] * dgrad;
  P->gradpcmf = P->gradpcmf + dgrad;
}

/* ------------------------------------------------------------------- LES */
/* find_strain_rate.f90:20-79, gauss branch: Green-Gauss gradients of u, v,
   w into the module gradients (:27-31), then |S| = sqrt(2 s_ij s_ij) over
   k = 2..nkm, i = 3..nimm, j = 3..njmm (:33-76).  The vorticity invariant
   of :77 is not kept (nothing on this path reads it). */
void cap_find_strain_rate(cap_state* s) {
  cap_grad_gauss(s, CAP_U, CAP_GRADU_X, CAP_GRADU_Y, CAP_GRADU_Z);
  cap_grad_gauss(s, CAP_V, CAP_GRADV_X, CAP_GRADV_Y, CAP_GRADV_Z);
  cap_grad_gauss(s, CAP_W, CAP_GRADW_X, CAP_GRADW_Y, CAP_GRADW_Z);
  const double *gux = s->f[CAP_GRADU_X], *guy = s->f[CAP_GRADU_Y], *guz = s->f[CAP_GRADU_Z];
  const double *gvx = s->f[CAP_GRADV_X], *gvy = s->f[CAP_GRADV_Y], *gvz = s->f[CAP_GRADV_Z];
  const double *gwx = s->f[CAP_GRADW_X], *gwy = s->f[CAP_GRADW_Y], *gwz = s->f[CAP_GRADW_Z];
  double* strain = s->f[CAP_STRAIN];
  for (int k = 2; k <= s->nkm; ++k)
    for (int i = 3; i <= s->nimm; ++i)
      for (int j = 3; j <= s->njmm; ++j) {
        const int inp = IXK(i, j, k);
        const double s11 = gux[inp];
        const double s12 = 0.5 * (guy[inp] + gvx[inp]);
        const double s13 = 0.5 * (guz[inp] + gwx[inp]);
        const double s22 = gvy[inp];
        const double s23 = 0.5 * (gvz[inp] + gwy[inp]);
        const double s33 = gwz[inp];
        strain[inp] = sqrt(2 * (s11 * s11 + s22 * s22 + s33 * s33 + 2 * (s12 * s12 + s13 * s13 + s23 * s23)));
      }
}

/* calc_vis_les.f90:38-249: Smagorinsky viscosity with the Van Driest and
   Schumann limits over k = 2..nkm, i = 3..nimm, j = 3..njmm (:42-73; the
   coefficient is the 0.17 assigned last at :66, C_delta the
   default-real 0.158, 1/3 the default-real 1./3.), under-relaxed by
   urf(ivis); then the wall-function viscosity of the bottom and top ghost
   layers (:80-246; dnw dotted with the integer extents nx,ny,nz and the
   top wall at lk(nimm), as calcuvw does). */
void cap_calc_vis_les(cap_state* s) {
  const cappgpu_params* P = &s->prm;
  const double *u = s->f[CAP_U], *v = s->f[CAP_V], *w = s->f[CAP_W];
  const double *wd = s->f[CAP_WALLDIST], *vol = s->f[CAP_VOL], *strain = s->f[CAP_STRAIN], *den = s->f[CAP_DEN];
  double* vis = s->f[CAP_VIS];
  const double viscos = P->viscos, cappa = P->cappa, urf = P->urf[CAP_IVIS - 1];
  const double c_delta = (double)0.158f, c_les = (double)0.17f, third = (double)(1.f / 3.f);
  for (int k = 2; k <= s->nkm; ++k)
    for (int i = 3; i <= s->nimm; ++i)
      for (int j = 3; j <= s->njmm; ++j) {
        const int inp = IXK(i, j, k);
        const double visold = vis[inp];
        const double wldist = wd[inp];
        const double uref = sqrt(u[inp] * u[inp] + v[inp] * v[inp] + w[inp] * w[inp]);
        const double utau = sqrt(viscos * uref / wldist);
        const double zplus = wldist * utau / viscos;
        const double l = dmin(c_les * pow(vol[inp], third), cappa / c_delta * wldist) * (1. - exp(-zplus / 26.0));
        const double vis_smag = l * l * strain[inp] * den[inp];
        double vnew = vis_smag + viscos;
        vnew = urf * vnew + (1. - urf) * visold;
        vis[inp] = vnew;
      }
  const double *xc = s->f[CAP_XC], *yc = s->f[CAP_YC], *zc = s->f[CAP_ZC], *fz = s->f[CAP_FZ];
  const double *a3x = s->f[CAP_AR3X], *a3y = s->f[CAP_AR3Y], *a3z = s->f[CAP_AR3Z];
  const double nxi = (double)s->ni, nyi = (double)s->nj, nzi = (double)s->nk;
  for (int top = 0; top < 2; ++top)
    for (int i = 3; i <= s->nimm; ++i)
      for (int j = 3; j <= s->njmm; ++j) {
        int inbc, ingc, iface;
        double fxp, fxe;
        if (!top) {
          inbc = IXK(i, j, 3); ingc = inbc - s->nij; iface = ingc;
          fxp = fz[ingc]; fxe = 1.0 - fxp;
        } else {
          inbc = IXK(i, j, s->prm.top_plane ? s->nkmm : s->nimm); ingc = inbc + s->nij; iface = inbc;
          fxp = 1.0 - fz[inbc]; fxe = 1.0 - fxp;
        }
        const double gzx = xc[inbc] * fxp + xc[ingc] * fxe;
        const double gzy = yc[inbc] * fxp + yc[ingc] * fxe;
        const double gzz = zc[inbc] * fxp + zc[ingc] * fxe;
        const double are = sqrt(a3x[iface] * a3x[iface] + a3y[iface] * a3y[iface] + a3z[iface] * a3z[iface]);
        const double nxf = a3x[iface] / are, nyf = a3y[iface] / are, nzf = a3z[iface] / are;
        const double vnp = u[inbc] * nxf + v[inbc] * nyf + w[inbc] * nzf;
        double xtp = u[inbc] - vnp * nxf, ytp = v[inbc] - vnp * nyf, ztp = w[inbc] - vnp * nzf;
        const double vtp = sqrt(xtp * xtp + ytp * ytp + ztp * ztp);
        xtp = xtp / vtp;
        ytp = ytp / vtp;
        ztp = ztp / vtp;
        const double ut2 = fabs(u[inbc] * xtp + v[inbc] * ytp + w[inbc] * ztp);
        const double dnw = fabs((xc[inbc] - gzx) * nxi + (yc[inbc] - gzy) * nyi + (zc[inbc] - gzz) * nzi);
        const double tau = viscos * ut2 / dnw;
        const double utau = sqrt(tau / P->densit);
        const double ypl = P->densit * utau * dnw / viscos;
        double viscw = P->zero;
        if (ypl > (double)11.61f) viscw = ypl * viscos * cappa / log(P->elog * ypl);
        vis[ingc] = dmax(viscos, viscw);
      }
}

/* main.f90:196-205 after the pressure-velocity coupling: the k and omega
   equations (calcscm) when lcal(ite) / lcal(ied), then the eddy viscosity
   (modvis) or, with lles, the sub-grid viscosity (calc_vis_les; its strain
   is formed here, as calcscm -- which forms it in the reference -- does not
   run on the LES path). */
static int turbulence(cap_state* s) {
  const cappgpu_params* P = &s->prm;
  int rc = 0;
  cappgpu_solve_report rep;
  if (P->sst && P->lcal[CAP_ITE - 1] && (rc = cap_calcscm(s, CAP_ITE, &rep)) < 0) return rc;
  if (P->sst && P->lcal[CAP_IED - 1] && (rc = cap_calcscm(s, CAP_IED, &rep)) < 0) return rc;
  if (P->lcal[CAP_IVIS - 1] && !P->lles && P->sst) cap_modvis(s);
  if (P->lcal[CAP_IVIS - 1] && P->lles) {
    cap_find_strain_rate(s);
    cap_calc_vis_les(s);
  }
  return 0;
}

/* main.f90:140-207 with maxit = 1 iteration per time step (transient PISO).
   The reference's residual-normalised convergence test (main.f90:218-237)
   uses snorin, which only bcin sets for inlet cases; the drivers here run
   the requested number of steps. */
int cap_piso_steps(cap_state* s, int nsteps, cappgpu_solve_report* last) {
  cappgpu_params* P = &s->prm;
  const size_t nb = sizeof(double) * s->nijk;
  int rc = 0;
  for (int st = 0; st < nsteps; ++st) {
    /* main.f90:140-157: te and ed shift whether or not their equations run */
    if (P->bdf) {
      memcpy(s->f[CAP_UOO], s->f[CAP_UO], nb);
      memcpy(s->f[CAP_VOO], s->f[CAP_VO], nb);
      memcpy(s->f[CAP_WOO], s->f[CAP_WO], nb);
      memcpy(s->f[CAP_TEOO], s->f[CAP_TEO], nb);
      memcpy(s->f[CAP_EDOO], s->f[CAP_EDO], nb);
    }
    memcpy(s->f[CAP_UO], s->f[CAP_U], nb);
    memcpy(s->f[CAP_VO], s->f[CAP_V], nb);
    memcpy(s->f[CAP_WO], s->f[CAP_W], nb);
    memcpy(s->f[CAP_TEO], s->f[CAP_TE], nb);
    memcpy(s->f[CAP_EDO], s->f[CAP_ED], nb);
    cap_courant(s);
    cap_update_values_at_ghostcells(s);
    cappgpu_solve_report r3[3];
    int r = cap_calcuvw(s, r3);
    if (r < 0) return r;
    if (!P->const_mflux) cap_outbc(s);
    cappgpu_solve_report reps[64];
    r = cap_piso_multiple_correction(s, reps);
    if (r < 0) return r;
    rc |= r;
    if (last) *last = reps[P->ncorr * P->npcor - 1];
    if ((r = turbulence(s)) < 0) return r;
    if (P->ltransient && P->const_mflux) cap_const_massflux_correction(s);   /* main.f90:252 */
  }
  return rc;
}

/* SIMPLE outer iterations (main.f90:185-192, steady) */
int cap_simple_iters(cap_state* s, int niters, cappgpu_solve_report* last) {
  cappgpu_params* P = &s->prm;
  int rc = 0;
  for (int it = 0; it < niters; ++it) {
    cap_update_values_at_ghostcells(s);
    cappgpu_solve_report r3[3];
    int r = cap_calcuvw(s, r3);
    if (r < 0) return r;
    if (!P->const_mflux) cap_outbc(s);
    cappgpu_solve_report reps[64];
    r = cap_calcp(s, reps);
    if (r < 0) return r;
    rc |= r;
    if (last) *last = reps[P->ncorr * P->npcor - 1];
    if ((r = turbulence(s)) < 0) return r;
  }
  return rc;
}
