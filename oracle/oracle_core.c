/*
 * oracle_core.c -- state, index maps, geometry, ghost cells, gradient,
 * bpres.  TEST INFRASTRUCTURE ONLY (the checker for the CUDA library).
 * Parity: find_intersection_point pinned by the reference's own
 * known-answer test (test_intersection_point.f90:8-38); setind, the ghost
 * cells, grad_gauss and bpres pinned against the reference's own routines
 * run from their source (see oracle.h).
 */
#include "oracle.h"
#include "oracle_internal.h"

#include <stdlib.h>
#include <string.h>
#include <math.h>

/* --------------------------------------------------------------- state */

/* setind.f90:21-40 */
static void setind(cap_state* s) {
  s->nim = s->ni - 1; s->njm = s->nj - 1; s->nkm = s->nk - 1;
  s->nimm = s->nim - 1; s->njmm = s->njm - 1; s->nkmm = s->nkm - 1;
  s->nij = s->ni * s->nj; s->nik = s->ni * s->nk; s->njk = s->nj * s->nk;
  s->nijk = s->nij * s->nk;
  for (int i = 1; i <= s->ni; ++i) s->li[i] = (i - 1) * s->nj;
  for (int k = 1; k <= s->nk; ++k) s->lk[k] = (k - 1) * s->nij;
}

cap_state* cap_new(int ni, int nj, int nk) {
  cap_state* s = (cap_state*)calloc(1, sizeof(cap_state));
  s->ni = ni; s->nj = nj; s->nk = nk;
  s->li = (int*)calloc((size_t)ni + 1, sizeof(int));
  s->lk = (int*)calloc((size_t)nk + 1, sizeof(int));
  setind(s);
  /* set_parameters.f90:22-57 leaves nxyza unassigned; the evident intent,
     used here, is nxyza = nxyz = nijk. Every array is zero-initialised. */
  for (int f = 0; f < CAP_NFIELDS; ++f) s->f[f] = (double*)calloc((size_t)s->nijk, sizeof(double));
  s->bc[CAP_LBW] = (int*)calloc((size_t)s->njk, sizeof(int));
  s->bc[CAP_LBE] = (int*)calloc((size_t)s->njk, sizeof(int));
  s->bc[CAP_LBS] = (int*)calloc((size_t)s->nik, sizeof(int));
  s->bc[CAP_LBN] = (int*)calloc((size_t)s->nik, sizeof(int));
  s->bc[CAP_LBB] = (int*)calloc((size_t)s->nij, sizeof(int));
  s->bc[CAP_LBT] = (int*)calloc((size_t)s->nij, sizeof(int));
  s->prm.alfa = 0.92;           /* init.f90:164 */
  s->prm.cappa = 0.41; s->prm.elog = 8.432;  /* init.f90:167-168 */
  s->prm.zero = 0.0;
  s->prm.densit = 1.0;
  s->prm.isol_p = CAPPGPU_SOLVER_CGSTAB_SIP;
  s->prm.piso_solver = CAPPGPU_SOLVER_PCGSIP;
  s->prm.ipr = s->prm.jpr = s->prm.kpr = 3;
  return s;
}

void cap_free(cap_state* s) {
  if (!s) return;
  for (int f = 0; f < CAP_NFIELDS; ++f) free(s->f[f]);
  for (int b = 0; b < CAP_NBC; ++b) free(s->bc[b]);
  free(s->li); free(s->lk); free(s);
}

double* cap_field(cap_state* s, int fid) { return (fid >= 0 && fid < CAP_NFIELDS) ? s->f[fid] : 0; }
int* cap_bc(cap_state* s, int face) { return (face >= 0 && face < CAP_NBC) ? s->bc[face] : 0; }
cappgpu_params* cap_params(cap_state* s) { return &s->prm; }
int* cap_li(cap_state* s) { return s->li; }
int* cap_lk(cap_state* s) { return s->lk; }
int cap_nijk(cap_state* s) { return s->nijk; }

/* ------------------------------------------------------------ geometry */

/* init.f90:49-136: face area vectors from the 4 corner nodes of each face
   (half the cross product of the face diagonals). */
static void face_area_loop(cap_state* s, int idns, int idtb, int i0, int i1, int j0, int j1,
                           int k0, int k1, double* ax, double* ay, double* az) {
  const double *x = s->f[CAP_X], *y = s->f[CAP_Y], *z = s->f[CAP_Z];
  for (int k = k0; k <= k1; ++k)
    for (int i = i0; i <= i1; ++i)
      for (int j = j0; j <= j1; ++j) {
        int inp = IXK(i, j, k);
        int ins = inp - idns, inb = inp - idtb, inbs = inb - idns;
        double dxet = 0.5 * (x[inp] - x[ins] + x[inb] - x[inbs]);
        double dyet = 0.5 * (y[inp] - y[ins] + y[inb] - y[inbs]);
        double dzet = 0.5 * (z[inp] - z[ins] + z[inb] - z[inbs]);
        double dxzd = 0.5 * (x[inp] - x[inb] + x[ins] - x[inbs]);
        double dyzd = 0.5 * (y[inp] - y[inb] + y[ins] - y[inbs]);
        double dzzd = 0.5 * (z[inp] - z[inb] + z[ins] - z[inbs]);
        ax[inp] = dyet * dzzd - dyzd * dzet;
        ay[inp] = dxzd * dzet - dxet * dzzd;
        az[inp] = dxet * dyzd - dyet * dxzd;
      }
}

void cap_face_areas(cap_state* s) {
  /* East faces  init.f90:50-77 (idns=1, idtb=nij, i=1..nim) */
  face_area_loop(s, 1, s->nij, 1, s->nim, 2, s->njm, 2, s->nkm,
                 s->f[CAP_AR1X], s->f[CAP_AR1Y], s->f[CAP_AR1Z]);
  /* North faces init.f90:80-107 (idns=nj, idtb=nij, j=1..njm) */
  face_area_loop(s, s->nj, s->nij, 2, s->nim, 1, s->njm, 2, s->nkm,
                 s->f[CAP_AR2X], s->f[CAP_AR2Y], s->f[CAP_AR2Z]);
  /* Top faces   init.f90:110-136 (idns=1, idtb=nj, k=1..nkm) */
  face_area_loop(s, 1, s->nj, 2, s->nim, 2, s->njm, 1, s->nkm,
                 s->f[CAP_AR3X], s->f[CAP_AR3Y], s->f[CAP_AR3Z]);
}

/* find_intersection_point.f90:1-76 (same formula as
   test_intersection_point.f90:58-74).  p15 = x1,y1,z1,...,x5,y5,z5. */
void cap_find_intersection_point(const double* p, double* out) {
  double x1 = p[0], y1 = p[1], z1 = p[2], x2 = p[3], y2 = p[4], z2 = p[5];
  double x3 = p[6], y3 = p[7], z3 = p[8], x4 = p[9], y4 = p[10], z4 = p[11];
  double x5 = p[12], y5 = p[13], z5 = p[14];
  double t = -(x2 * (y3 * z4 - y4 * z3) - x1 * (y3 * z4 - y4 * z3) - x3 * (y2 * z4 - y4 * z2) +
               x1 * (y2 * z4 - y4 * z2) + x3 * (y1 * z4 - y4 * z1) - x2 * (y1 * z4 - y4 * z1) +
               x4 * (y2 * z3 - y3 * z2) - x1 * (y2 * z3 - y3 * z2) - x4 * (y1 * z3 - y3 * z1) +
               x2 * (y1 * z3 - y3 * z1) + x4 * (y1 * z2 - y2 * z1) - x3 * (y1 * z2 - y2 * z1)) /
             (x2 * (y3 * (z5 - z4) - (y5 - y4) * z3) - x1 * (y3 * (z5 - z4) - (y5 - y4) * z3) -
              x3 * (y2 * (z5 - z4) - (y5 - y4) * z2) + x1 * (y2 * (z5 - z4) - (y5 - y4) * z2) +
              x3 * (y1 * (z5 - z4) - (y5 - y4) * z1) - x2 * (y1 * (z5 - z4) - (y5 - y4) * z1) +
              (x5 - x4) * (y2 * z3 - y3 * z2) - (x5 - x4) * (y1 * z3 - y3 * z1) +
              (x5 - x4) * (y1 * z2 - y2 * z1));
  out[0] = x4 + (x5 - x4) * t;
  out[1] = y4 + (y5 - y4) * t;
  out[2] = z4 + (z5 - z4) * t;
}

/* intfac.f90:4-48 */
static void intfac(cap_state* s, int idew, int idns, int idtb, double* lambda) {
  const double *x = s->f[CAP_X], *y = s->f[CAP_Y], *z = s->f[CAP_Z];
  const double *xc = s->f[CAP_XC], *yc = s->f[CAP_YC], *zc = s->f[CAP_ZC];
  for (int k = 2; k <= s->nkm; ++k)
    for (int i = 2; i <= s->nim; ++i)
      for (int j = 2; j <= s->njm; ++j) {
        int inp = IXK(i, j, k), inn = inp + idew;
        double p[15] = {x[inp], y[inp], z[inp], x[inp - idns], y[inp - idns], z[inp - idns],
                        x[inp - idtb], y[inp - idtb], z[inp - idtb], xc[inp], yc[inp], zc[inp],
                        xc[inp + idew], yc[inp + idew], zc[inp + idew]};
        double q[3];
        cap_find_intersection_point(p, q);
        double xf = q[0], yf = q[1], zf = q[2];
        double dx = xf - xc[inp], dy = yf - yc[inp], dz = zf - zc[inp];
        double ex = xc[inn] - xc[inp], ey = yc[inn] - yc[inp], ez = zc[inn] - zc[inp] + SMALL;
        lambda[inp] = sqrt(dx * dx + dy * dy + dz * dz) / (sqrt(ex * ex + ey * ey + ez * ez) + SMALL);
      }
}

void cap_intfac_all(cap_state* s) {
  /* init.f90:142-144 */
  intfac(s, s->nj, 1, s->nij, s->f[CAP_FX]);
  intfac(s, 1, s->nj, s->nij, s->f[CAP_FY]);
  intfac(s, s->nij, 1, s->nj, s->f[CAP_FZ]);
}

/* ---------------------------------------------------------- ghost cells */

/* update_values_at_ghostcells_nonperiodic.f90:47-640 */
static void ghost_nonperiodic(cap_state* s) {
  double *u = s->f[CAP_U], *v = s->f[CAP_V], *w = s->f[CAP_W];
  double *te = s->f[CAP_TE], *ed = s->f[CAP_ED], *t = s->f[CAP_T], *vis = s->f[CAP_VIS];
  const double *fx = s->f[CAP_FX], *fy = s->f[CAP_FY], *fz = s->f[CAP_FZ];
  const cappgpu_params* P = &s->prm;
  const int nj = s->nj, nk = s->nk, nij = s->nij;
  /* faces: 0 west 1 east 2 south 3 north 4 bottom 5 top */
  for (int face = 0; face < 6; ++face) {
    int na, nb;       /* outer loop (a) and inner loop (b) ranges */
    if (face <= 1) { na = s->nkmm; nb = s->njmm; }       /* k, j  */
    else if (face <= 3) { na = s->nkmm; nb = s->nimm; }  /* k, i  */
    else { na = s->nimm; nb = s->njmm; }                 /* i, j  */
    for (int a = 3; a <= na; ++a)
      for (int b = 3; b <= nb; ++b) {
        int inp, ingc, iface, inbc, lb, off;
        double fxp, *arx, *ary, *arz;
        switch (face) {
          case 0: inp = IXK(3, b, a); off = nj; ingc = inp - nj; iface = inp - nj;
                  inbc = (b - 1) * nk + a; lb = s->bc[CAP_LBW][inbc - 1]; fxp = fx[inp - nj];
                  arx = s->f[CAP_AR1X]; ary = s->f[CAP_AR1Y]; arz = s->f[CAP_AR1Z]; break;
          case 1: inp = IXK(s->nimm, b, a); off = nj; ingc = inp + nj; iface = inp;
                  inbc = (b - 1) * nk + a; lb = s->bc[CAP_LBE][inbc - 1]; fxp = 1.0 - fx[inp];
                  arx = s->f[CAP_AR1X]; ary = s->f[CAP_AR1Y]; arz = s->f[CAP_AR1Z]; break;
          case 2: inp = IXK(b, 3, a); off = 1; ingc = inp - 1; iface = inp - 1;
                  inbc = (b - 1) * nk + a; lb = s->bc[CAP_LBS][inbc - 1]; fxp = 1.0 - fy[inp];
                  arx = s->f[CAP_AR2X]; ary = s->f[CAP_AR2Y]; arz = s->f[CAP_AR2Z]; break;
          case 3: inp = IXK(b, s->njmm, a); off = 1; ingc = inp + 1; iface = inp;
                  inbc = (b - 1) * nk + a; lb = s->bc[CAP_LBN][inbc - 1]; fxp = 1.0 - fy[inp];
                  arx = s->f[CAP_AR2X]; ary = s->f[CAP_AR2Y]; arz = s->f[CAP_AR2Z]; break;
          case 4: inp = IXK(a, b, 3); off = nij; ingc = inp - nij; iface = inp - nij;
                  inbc = (a - 1) * nj + b; lb = s->bc[CAP_LBB][inbc - 1]; fxp = fz[ingc];
                  arx = s->f[CAP_AR3X]; ary = s->f[CAP_AR3Y]; arz = s->f[CAP_AR3Z]; break;
          default: inp = IXK(a, b, s->nkmm); off = nij; ingc = inp + nij; iface = inp;
                  inbc = (a - 1) * nj + b; lb = s->bc[CAP_LBT][inbc - 1]; fxp = 1.0 - fz[inp];
                  arx = s->f[CAP_AR3X]; ary = s->f[CAP_AR3Y]; arz = s->f[CAP_AR3Z]; break;
        }
        double fxe = 1.0 - fxp;
        double fxer = 1.0 / fxe;
        int lowside = (face == 0 || face == 2 || face == 4);
        if (lb == 1) { /* inlet :73-86 */
          u[ingc] = (P->uin - u[inp] * fxp) * fxer;
          v[ingc] = (P->vin - v[inp] * fxp) * fxer;
          w[ingc] = (P->win - w[inp] * fxp) * fxer;
          te[ingc] = (P->tein - te[inp] * fxp) * fxer;
          ed[ingc] = (P->edin - ed[inp] * fxp) * fxer;
          t[ingc] = (P->tin - t[inp] * fxp) * fxer;
          vis[ingc] = 0.09 * (te[ingc] * te[ingc]) / ed[ingc];
        }
        if (lb == 2) { /* outlet :88-101 (low side) / :185-198 (high side) */
          if (lowside) {
            const double* fif = (face == 0) ? fx : (face == 2) ? fy : fz;
            double f = fif[inp];
            u[ingc] = u[inp] - (u[inp + off] - u[inp]) * f;
            v[ingc] = v[inp] - (v[inp + off] - v[inp]) * f;
            w[ingc] = w[inp] - (w[inp + off] - w[inp]) * f;
            te[ingc] = te[inp] - (te[inp + off] - te[inp]) * f;
            ed[ingc] = ed[inp] - (ed[inp + off] - ed[inp]) * f;
            t[ingc] = t[inp] - (t[inp + off] - t[inp]) * f;
            vis[ingc] = vis[inp] - (vis[inp + off] - vis[inp]) * f;
          } else {
            const double* fif = (face == 1) ? fx : (face == 3) ? fy : fz;
            double f = 1.0 - fif[inp - off];
            u[ingc] = u[inp] + (u[inp] - u[inp - off]) * f;
            v[ingc] = v[inp] + (v[inp] - v[inp - off]) * f;
            w[ingc] = w[inp] + (w[inp] - w[inp - off]) * f;
            te[ingc] = te[inp] + (te[inp] - te[inp - off]) * f;
            ed[ingc] = ed[inp] + (ed[inp] - ed[inp - off]) * f;
            t[ingc] = t[inp] + (t[inp] - t[inp - off]) * f;
            vis[ingc] = vis[inp] + (vis[inp] - vis[inp - off]) * f;
          }
        }
        if (lb == 3) { /* symmetry :103-117 (area vector, not unit normal) */
          double unmag = u[inp] * arx[iface] + v[inp] * ary[iface] + w[inp] * arz[iface];
          u[ingc] = u[inp] - unmag * arx[iface];
          v[ingc] = v[inp] - unmag * ary[iface];
          w[ingc] = w[inp] - unmag * arz[iface];
          te[ingc] = te[inp];
          ed[ingc] = ed[inp];
          t[ingc] = t[inp];
          vis[ingc] = vis[inp];
        }
        if (lb == 4) { /* wall :119-137 (bottom/top keep vis, :528-529) */
          u[ingc] = (-u[inp] * fxp) * fxer;
          v[ingc] = (-v[inp] * fxp) * fxer;
          w[ingc] = (-w[inp] * fxp) * fxer;
          te[ingc] = (-te[inp] * fxp) * fxer;
          ed[ingc] = ed[inp];
          t[ingc] = (P->tin - t[inp] * fxp) * fxer;
          if (face >= 4) vis[ingc] = vis[inp];
          else vis[ingc] = (vis[ingc] - vis[inp] * fxp) * fxer;
        }
      }
  }
}

/* update_values_at_ghostcells.f90:40-145 (periodic in i and j, walls in k) */
static void ghost_periodic(cap_state* s) {
  double* fl[6] = {s->f[CAP_U], s->f[CAP_V], s->f[CAP_W], s->f[CAP_TE], s->f[CAP_ED], s->f[CAP_VIS]};
  const double* fz = s->f[CAP_FZ];
  for (int k = 3; k <= s->nkmm; ++k)
    for (int j = 3; j <= s->njmm; ++j) {
      int ingcw = IXK(2, j, k), inp = IXK(3, j, k), ine = IXK(s->nimm, j, k), ingce = IXK(s->nim, j, k);
      for (int q = 0; q < 6; ++q) fl[q][ingcw] = fl[q][ine];
      for (int q = 0; q < 6; ++q) fl[q][ingce] = fl[q][inp];
    }
  for (int k = 3; k <= s->nkmm; ++k)
    for (int i = 3; i <= s->nimm; ++i) {
      int ingcw = IXK(i, 2, k), inp = IXK(i, 3, k), ine = IXK(i, s->njmm, k), ingce = IXK(i, s->njm, k);
      for (int q = 0; q < 6; ++q) fl[q][ingcw] = fl[q][ine];
      for (int q = 0; q < 6; ++q) fl[q][ingce] = fl[q][inp];
    }
  double *u = s->f[CAP_U], *v = s->f[CAP_V], *w = s->f[CAP_W];
  double *te = s->f[CAP_TE], *ed = s->f[CAP_ED], *vis = s->f[CAP_VIS];
  for (int i = 3; i <= s->nimm; ++i)
    for (int j = 3; j <= s->njmm; ++j) {
      int ingc = IXK(i, j, 2), inp = IXK(i, j, 3);
      int ine = inp - s->nij;
      double fxp = fz[ine], fxe = 1.0 - fxp;
      u[ingc] = -u[inp] * fxp / fxe;
      v[ingc] = -v[inp] * fxp / fxe;
      w[ingc] = -w[inp] * fxp / fxe;
      te[ingc] = -te[inp] * fxp / fxe;
      ed[ingc] = ed[inp];
      vis[ingc] = (vis[ingc] - vis[inp] * fxp) / fxe;
    }
  for (int i = 3; i <= s->nimm; ++i)
    for (int j = 3; j <= s->njmm; ++j) {
      int ingc = IXK(i, j, s->nkm), inp = IXK(i, j, s->nkmm);
      double fxe = fz[inp], fxp = 1.0 - fxe;
      u[ingc] = -u[inp] * fxp / fxe;
      v[ingc] = -v[inp] * fxp / fxe;
      w[ingc] = -w[inp] * fxp / fxe;
      te[ingc] = -te[inp] * fxp / fxe;
      ed[ingc] = ed[inp];
      vis[ingc] = (vis[ingc] - vis[inp] * fxp) / fxe;
    }
}

void cap_update_values_at_ghostcells(cap_state* s) {
  if (s->prm.periodic) ghost_periodic(s);
  else ghost_nonperiodic(s);
}

/* ------------------------------------------------------------- gradient */

/* GRAD_GAUSS.f90:1-105 (scatter form, reference loop order) */
void cap_grad_gauss(cap_state* s, int uf, int dxf, int dyf, int dzf) {
  const double* u = s->f[uf];
  double *dudx = s->f[dxf], *dudy = s->f[dyf], *dudz = s->f[dzf];
  const double *fx = s->f[CAP_FX], *fy = s->f[CAP_FY], *fz = s->f[CAP_FZ];
  const double *a1x = s->f[CAP_AR1X], *a1y = s->f[CAP_AR1Y], *a1z = s->f[CAP_AR1Z];
  const double *a2x = s->f[CAP_AR2X], *a2y = s->f[CAP_AR2Y], *a2z = s->f[CAP_AR2Z];
  const double *a3x = s->f[CAP_AR3X], *a3y = s->f[CAP_AR3Y], *a3z = s->f[CAP_AR3Z];
  const double* vol = s->f[CAP_VOL];
  memset(dudx, 0, sizeof(double) * s->nijk);
  memset(dudy, 0, sizeof(double) * s->nijk);
  memset(dudz, 0, sizeof(double) * s->nijk);
  for (int k = 2; k <= s->nkm; ++k)
    for (int i = 2; i <= s->nimm; ++i)
      for (int j = 2; j <= s->njmm; ++j) {
        int inp = IXK(i, j, k), ine = inp + s->nj, inn = inp + 1, int_ = inp + s->nij;
        double ue = u[ine] * fx[inp] + u[inp] * (1.0 - fx[inp]);
        double un = u[inn] * fy[inp] + u[inp] * (1.0 - fy[inp]);
        double ut = u[int_] * fz[inp] + u[inp] * (1.0 - fz[inp]);
        dudx[inp] = dudx[inp] + (ue * a1x[inp] + un * a2x[inp] + ut * a3x[inp]);
        dudx[ine] = dudx[ine] - (ue * a1x[inp]);
        dudx[inn] = dudx[inn] - (un * a2x[inp]);
        dudx[int_] = dudx[int_] - (ut * a3x[inp]);
        dudy[inp] = dudy[inp] + (ue * a1y[inp] + un * a2y[inp] + ut * a3y[inp]);
        dudy[ine] = dudy[ine] - (ue * a1y[inp]);
        dudy[inn] = dudy[inn] - (un * a2y[inp]);
        dudy[int_] = dudy[int_] - (ut * a3y[inp]);
        dudz[inp] = dudz[inp] + (ue * a1z[inp] + un * a2z[inp] + ut * a3z[inp]);
        dudz[ine] = dudz[ine] - (ue * a1z[inp]);
        dudz[inn] = dudz[inn] - (un * a2z[inp]);
        dudz[int_] = dudz[int_] - (ut * a3z[inp]);
      }
  for (int k = 2; k <= s->nkm; ++k)
    for (int i = 3; i <= s->nimm; ++i)
      for (int j = 3; j <= s->njmm; ++j) {
        int inp = IXK(i, j, k);
        double volr = 1.0 / vol[inp];
        dudx[inp] = dudx[inp] * volr;
        dudy[inp] = dudy[inp] * volr;
        dudz[inp] = dudz[inp] * volr;
      }
}

/* ---------------------------------------------------------------- bpres */

/* bpres.f90:3-81 */
void cap_bpres(cap_state* s, int pf) {
  double* p = s->f[pf];
  const double *fx = s->f[CAP_FX], *fy = s->f[CAP_FY], *fz = s->f[CAP_FZ];
  const int nj = s->nj, nij = s->nij;
  for (int i = 3; i <= s->nimm; ++i)
    for (int j = 3; j <= s->njmm; ++j) {
      int ijk = IXK(i, j, 3);
      p[ijk - nij] = p[ijk] - (p[ijk + nij] - p[ijk]) * fz[ijk];
    }
  for (int i = 3; i <= s->nimm; ++i)
    for (int j = 3; j <= s->njmm; ++j) {
      int ijk = IXK(i, j, s->nkmm);
      p[ijk + nij] = p[ijk] + (p[ijk] - p[ijk - nij]) * (1.0 - fz[ijk - nij]);
    }
  for (int j = 3; j <= s->njmm; ++j)
    for (int k = 3; k <= s->nkmm; ++k) {
      int ijk = IXK(3, j, k);
      p[ijk - nj] = p[ijk] - (p[ijk + nj] - p[ijk]) * fx[ijk];
    }
  for (int j = 3; j <= s->njmm; ++j)
    for (int k = 3; k <= s->nkmm; ++k) {
      int ijk = IXK(s->nimm, j, k);
      p[ijk + nj] = p[ijk] + (p[ijk] - p[ijk - nj]) * (1.0 - fx[ijk - nj]);
    }
  for (int i = 3; i <= s->nimm; ++i)
    for (int k = 3; k <= s->nkmm; ++k) {
      int ijk = IXK(i, 3, k);
      p[ijk - 1] = p[ijk] - (p[ijk + 1] - p[ijk]) * fy[ijk];
    }
  for (int i = 3; i <= s->nimm; ++i)
    for (int k = 3; k <= s->nkmm; ++k) {
      int ijk = IXK(i, s->njmm, k);
      p[ijk + 1] = p[ijk] + (p[ijk] - p[ijk - 1]) * (1.0 - fy[ijk - 1]);
    }
}
