// assembly.cu -- momentum assembly (fluxuvw, calcuvw), PISO pressure
// equation and corrector, SIMPLE (fluxmass, fluxmc, calcp), Courant number
// and continuity errors as device kernels.  Each kernel keeps the
// reference routine's write set and per-element operation order; where the
// reference scatters into a neighbour (su(ine) updates) the device code
// gathers the same rounded terms in the reference's order.
#include <math.h>
#include <string.h>

#include <vector>

#include "common.cuh"
#include "kernels.cuh"

namespace cap {

#define BOX_LOOP(b)                                                                              \
  for (long long t_ = blockIdx.x * (long long)blockDim.x + threadIdx.x, n_ = (b).count(); t_ < n_; \
       t_ += (long long)gridDim.x * blockDim.x)

// ---------------------------------------------------------------- fluxuvw
struct FluxArgs {
  const double *arvx, *arvy, *arvz, *fif, *fcf;
  double *acfe, *acfw;
  const double *x, *y, *z, *xc, *yc, *zc;
  const double *u, *v, *w, *vis;
  const double *gux, *guy, *guz, *gvx, *gvy, *gvz, *gwx, *gwy, *gwz;
  const double *gud, *gvd, *gwd;   // gradient component along dir (LUDS)
  double *su, *sv, *sw, *bp, *bt, *bb;
  double gam, zero;
  int idew, idns, idtb;
  int lcds, lcds4, lluds, lquds, flux_limiter, lsmart, lavl, lmuscl, lumist, lgamma;
};

template <typename R>
__device__ inline R dmin_(R a, R b) { return a < b ? a : b; }
// square root in the compute type (FP32 form: sqrtf, IEEE-rounded)
__device__ inline double sqrt_(double x) { return sqrt(x); }
__device__ inline float sqrt_(float x) { return sqrtf(x); }
template <typename R>
__device__ inline R dmax_(R a, R b) { return a > b ? a : b; }

// ------------------------------------------------ per-face geometry cache
// The face kernels of the momentum and pressure assembly spend most of
// their FP64 work on quantities of the grid alone: the distance of the two
// cell centres and the face area (two square roots), the unit normal, the
// centre-line unit vector and their cosine, area/volume ratios and the
// offset of the face centre from the interpolation point (ten divisions).
// GB300 runs FP64 divisions and square roots slowly, and these values do
// not change between time steps, so the FP64 forms read them from arrays
// built once per grid (rebuilt when a geometry field is written).  Each
// array holds the very expression the reference evaluates per face, with
// the same operation order, so the cached forms give the same bits.
enum GeoQ { GQ_XPN, GQ_YPN, GQ_ZPN, GQ_DPN, GQ_ARE, GQ_COSTN, GQ_AVX, GQ_AVY, GQ_AVZ, GQ_DXF, GQ_DYF, GQ_DZF, GQ_N };

struct FaceGeoPtrs {
  const double* q[GQ_N];
};

struct FaceGeoCache {
  double* buf[3] = {};
  unsigned long long gen[3] = {0, 0, 0};
  int nijk = 0;
};
FaceGeoCache g_fg;

void facegeo_free() {
  for (auto& p : g_fg.buf) { if (p) cudaFree(p); p = nullptr; }
  g_fg = FaceGeoCache();
}

// PISO_assemble_pressure_eq.f90:60-120 / fluxuvw-overrelaxed-correction.f90:
// 135-205: the geometric part of one face
__global__ void k_face_geo(Dims d, Box b, int idew, int idns, int idtb, const double* __restrict__ arvx,
                           const double* __restrict__ arvy, const double* __restrict__ arvz,
                           const double* __restrict__ fif, const double* __restrict__ x,
                           const double* __restrict__ y, const double* __restrict__ z,
                           const double* __restrict__ xc, const double* __restrict__ yc,
                           const double* __restrict__ zc, double* __restrict__ out) {
  const size_t n = (size_t)d.nijk;
  BOX_LOOP(b) {
    int i, j, k;
    b.at(t_, i, j, k);
    const int inp = ixk(d, i, j, k);
    const int ine = inp + idew, ins = inp - idns, inb = inp - idtb, inbs = inb - idns;
    const double fxe = fif[inp], fxp = 1.0 - fxe;
    const double xf = 0.25 * (x[inp] + x[ins] + x[inb] + x[inbs]);
    const double yf = 0.25 * (y[inp] + y[ins] + y[inb] + y[inbs]);
    const double zf = 0.25 * (z[inp] + z[ins] + z[inb] + z[inbs]);
    const double xi = xc[inp] * fxp + xc[ine] * fxe;
    const double yi = yc[inp] * fxp + yc[ine] * fxe;
    const double zi = zc[inp] * fxp + zc[ine] * fxe;
    const double xpn = xc[ine] - xc[inp], ypn = yc[ine] - yc[inp], zpn = zc[ine] - zc[inp];
    const double dpn = sqrt(xpn * xpn + ypn * ypn + zpn * zpn);
    const double ixi1 = xpn / dpn, ixi2 = ypn / dpn, ixi3 = zpn / dpn;
    const double arx = arvx[inp], ary = arvy[inp], arz = arvz[inp];
    const double are = sqrt(arx * arx + ary * ary + arz * arz);
    const double vole = xpn * arx + ypn * ary + zpn * arz;
    const double nxx = arx / are, nyy = ary / are, nzz = arz / are;
    const double costheta = nxx * ixi1 + nyy * ixi2 + nzz * ixi3;
    out[GQ_XPN * n + inp] = xpn;
    out[GQ_YPN * n + inp] = ypn;
    out[GQ_ZPN * n + inp] = zpn;
    out[GQ_DPN * n + inp] = dpn;
    out[GQ_ARE * n + inp] = are;
    out[GQ_COSTN * n + inp] = costheta;
    out[GQ_AVX * n + inp] = arx / vole;
    out[GQ_AVY * n + inp] = ary / vole;
    out[GQ_AVZ * n + inp] = arz / vole;
    out[GQ_DXF * n + inp] = xf - xi;
    out[GQ_DYF * n + inp] = yf - yi;
    out[GQ_DZF * n + inp] = zf - zi;
  }
}

// The cache of the face direction given by the arguments, built if stale;
// false when the arguments are not one of the grid's three face sets (the
// caller then evaluates the geometry itself).
static int face_geo(int idew, int idns, int idtb, int arvx, int arvy, int arvz, int fif, FaceGeoPtrs* out,
                    bool* ok) {
  Ctx& c = ctx();
  const Dims& d = c.d;
  *ok = false;
  int dir = -1;
  if (idew == d.nj && idns == 1 && idtb == d.nij && arvx == CAP_AR1X && arvy == CAP_AR1Y && arvz == CAP_AR1Z &&
      fif == CAP_FX)
    dir = 0;
  else if (idew == 1 && idns == d.nij && idtb == d.nj && arvx == CAP_AR2X && arvy == CAP_AR2Y &&
           arvz == CAP_AR2Z && fif == CAP_FY)
    dir = 1;
  else if (idew == d.nij && idns == d.nj && idtb == 1 && arvx == CAP_AR3X && arvy == CAP_AR3Y &&
           arvz == CAP_AR3Z && fif == CAP_FZ)
    dir = 2;
  if (dir < 0 || !c.face_geo) return CAPPGPU_OK;
  const size_t n = (size_t)d.nijk;
  if (g_fg.nijk != d.nijk) {
    facegeo_free();
    g_fg.nijk = d.nijk;
  }
  if (!g_fg.buf[dir]) {
    if (cudaMalloc(&g_fg.buf[dir], GQ_N * n * sizeof(double)) != cudaSuccess) {
      cudaGetLastError();
      g_fg.buf[dir] = nullptr;
      return CAPPGPU_OK;   // no room: evaluate per call
    }
    CAP_CUDA(cudaMemsetAsync(g_fg.buf[dir], 0, GQ_N * n * sizeof(double), c.st));
    g_fg.gen[dir] = 0;
  }
  if (g_fg.gen[dir] != c.geo_gen) {
    double** F = c.f;
    // every face any caller visits: the pressure equation's box
    Box b{2, d.nimm, 2, d.njmm, 2, d.nkmm};
    launch(k_face_geo, grid_for(b.count()), kThreads, c.st, d, b, idew, idns, idtb, (const double*)F[arvx],
           (const double*)F[arvy], (const double*)F[arvz], (const double*)F[fif], (const double*)F[CAP_X],
           (const double*)F[CAP_Y], (const double*)F[CAP_Z], (const double*)F[CAP_XC], (const double*)F[CAP_YC],
           (const double*)F[CAP_ZC], g_fg.buf[dir]);
    CAP_CHECK_LAUNCH();
    g_fg.gen[dir] = c.geo_gen;
  }
  for (int q = 0; q < GQ_N; ++q) out->q[q] = g_fg.buf[dir] + q * n;
  *ok = true;
  return CAPPGPU_OK;
}

// QUICK's high-order fluxes of face inp (fluxuvw-overrelaxed-correction.f90:388-409)
template <typename R>
__device__ inline void quick_face(const FluxArgs& A, int inp, R& fu, R& fv, R& fw) {
  const double *u = A.u, *v = A.v, *w = A.w;
  const int ine = inp + A.idew, inw = inp - A.idew, inee = inp + 2 * A.idew;
  const R flcf = R(A.fcf[inp]);
  const R ce = dmin_(flcf, R(A.zero)), cp = dmax_(flcf, R(A.zero));
  R fm = R(A.fif[inw]), f0 = R(A.fif[inp]), fpl = R(A.fif[ine]);
  R g11 = ((2 - fm) * (f0 * f0)) / (1 + f0 - fm);
  R g12 = ((1 - f0) * ((1 - fm) * (1 - fm))) / (1 + f0 - fm);
  R g21 = ((1 + fpl) * ((1 - f0) * (1 - f0))) / (1 + fpl - f0);
  R g22 = ((fpl * fpl) * f0) / (1 + fpl - f0);
  fu = ce * (g21 * R(u[inp]) + (1 - g21 + g22) * R(u[ine]) - g22 * R(u[inee])) +
       cp * (g11 * R(u[ine]) + (1 - g11 + g12) * R(u[inp]) - g12 * R(u[inw]));
  fv = ce * (g21 * R(v[inp]) + (1 - g21 + g22) * R(v[ine]) - g22 * R(v[inee])) +
       cp * (g11 * R(v[ine]) + (1 - g11 + g12) * R(v[inp]) - g12 * R(v[inw]));
  fw = ce * (g21 * R(w[inp]) + (1 - g21 + g22) * R(w[ine]) - g22 * R(w[inee])) +
       cp * (g11 * R(w[ine]) + (1 - g11 + g12) * R(w[inp]) - g12 * R(w[inw]));
}

// The reference zeroes fuhigh, fvhigh, fwhigh once, before its face loop
// (fluxuvw-overrelaxed-correction.f90:90-92), and QUICK assigns them only
// inside 2 < i,j,k < n-1 (:383-385): a face outside that box where no
// earlier scheme assigned them carries the values of the last face of the
// loop order (k, i, j) that was inside.  The loop boxes (:96-110) leave
// out only the plane i = 2 (x faces), j = 2 (y faces) or k = 2 (z faces);
// the face carried is (k-1, nimm, njmm) or (k, i-1, njmm), and none at the
// start of the loop (the zeros).
__device__ inline bool quick_carried_face(const Dims& d, int idew, int i, int j, int k, int* pinp) {
  (void)j;
  if (idew == d.nj) {                  // x faces: k 3..nkmm, i 2..nimm, j 3..njmm
    if (k <= 3) return false;
    *pinp = ixk(d, d.nimm, d.njmm, k - 1);
    return true;
  }
  if (idew == 1) {                     // y faces: k 3..nkmm, i 3..nimm, j 2..njmm
    if (i > 3) { *pinp = ixk(d, i - 1, d.njmm, k); return true; }
    if (k <= 3) return false;
    *pinp = ixk(d, d.nimm, d.njmm, k - 1);
    return true;
  }
  return false;                        // z faces: the plane k = 2 opens the loop
}

// fluxuvw-overrelaxed-correction.f90:121-637 for one face inp; GEO: the
// geometric terms come from the per-face cache (FP64 form only)
template <typename R, bool GEO>
__global__ void k_fluxuvw_faces(Dims d, Box b, FluxArgs A, FaceGeoPtrs G) {
  BOX_LOOP(b) {
    int i, j, k;
    b.at(t_, i, j, k);
    int inp = ixk(d, i, j, k);
    int ine = inp + A.idew, inw = inp - A.idew, ins = inp - A.idns, inb = inp - A.idtb;
    int inee = inp + 2 * A.idew, inbs = inb - A.idns;
    R fxe = R(A.fif[inp]), fxp = R(1.0) - fxe;
    R fxpw = R(A.fif[inw]), fxw = R(1.0) - fxpw;
    R fxee = R(A.fif[ine]), fxew = R(1.0) - fxee;
    R arx = R(A.arvx[inp]), ary = R(A.arvy[inp]), arz = R(A.arvz[inp]);
    R xpn, ypn, zpn, dpn, are, avx, avy, avz, dxf, dyf, dzf;
    if constexpr (GEO) {
      xpn = G.q[GQ_XPN][inp]; ypn = G.q[GQ_YPN][inp]; zpn = G.q[GQ_ZPN][inp];
      dpn = G.q[GQ_DPN][inp]; are = G.q[GQ_ARE][inp];
      avx = G.q[GQ_AVX][inp]; avy = G.q[GQ_AVY][inp]; avz = G.q[GQ_AVZ][inp];
      dxf = G.q[GQ_DXF][inp]; dyf = G.q[GQ_DYF][inp]; dzf = G.q[GQ_DZF][inp];
    } else {
      xpn = R(A.xc[ine]) - R(A.xc[inp]); ypn = R(A.yc[ine]) - R(A.yc[inp]); zpn = R(A.zc[ine]) - R(A.zc[inp]);
      dpn = sqrt_(xpn * xpn + ypn * ypn + zpn * zpn);
      are = sqrt_(arx * arx + ary * ary + arz * arz);
      R vole = xpn * arx + ypn * ary + zpn * arz;
      avx = arx / vole; avy = ary / vole; avz = arz / vole;
      R xf = R(0.25) * (R(A.x[inp]) + R(A.x[ins]) + R(A.x[inb]) + R(A.x[inbs]));
      R yf = R(0.25) * (R(A.y[inp]) + R(A.y[ins]) + R(A.y[inb]) + R(A.y[inbs]));
      R zf = R(0.25) * (R(A.z[inp]) + R(A.z[ins]) + R(A.z[inb]) + R(A.z[inbs]));
      R xi = R(A.xc[inp]) * fxp + R(A.xc[ine]) * fxe;
      R yi = R(A.yc[inp]) * fxp + R(A.yc[ine]) * fxe;
      R zi = R(A.zc[inp]) * fxp + R(A.zc[ine]) * fxe;
      dxf = xf - xi; dyf = yf - yi; dzf = zf - zi;
    }
    const R costn = R(1.0);  // orthogonal correction (:178)
    R d1x = costn, d1y = costn, d1z = costn;
    R d2x = xpn * costn, d2y = ypn * costn, d2z = zpn * costn;
    R game = (R(A.vis[inp]) * fxp + R(A.vis[ine]) * fxe);
    const double *u = A.u, *v = A.v, *w = A.w;
    R duxi = R(A.gux[inp]) * fxp + R(A.gux[ine]) * fxe;
    R duyi = R(A.guy[inp]) * fxp + R(A.guy[ine]) * fxe;
    R duzi = R(A.guz[inp]) * fxp + R(A.guz[ine]) * fxe;
    R du = R(u[ine]) - R(u[inp]) - duxi * d2x - duyi * d2y - duzi * d2z;
    R duxii = duxi * d1x + avx * du;
    R duyii = duyi * d1y + avy * du;
    R duzii = duzi * d1z + avz * du;
    R dvxi = R(A.gvx[inp]) * fxp + R(A.gvx[ine]) * fxe;
    R dvyi = R(A.gvy[inp]) * fxp + R(A.gvy[ine]) * fxe;
    R dvzi = R(A.gvz[inp]) * fxp + R(A.gvz[ine]) * fxe;
    R dv = R(v[ine]) - R(v[inp]) - dvxi * d2x - dvyi * d2y - dvzi * d2z;
    R dvxii = dvxi * d1x + avx * dv;
    R dvyii = dvyi * d1y + avy * dv;
    R dvzii = dvzi * d1z + avz * dv;
    R dwxi = R(A.gwx[inp]) * fxp + R(A.gwx[ine]) * fxe;
    R dwyi = R(A.gwy[inp]) * fxp + R(A.gwy[ine]) * fxe;
    R dwzi = R(A.gwz[inp]) * fxp + R(A.gwz[ine]) * fxe;
    R dw = R(w[ine]) - R(w[inp]) - dwxi * d2x - dwyi * d2y - dwzi * d2z;
    R dwxii = dwxi * d1x + avx * dw;
    R dwyii = dwyi * d1y + avy * dw;
    R dwzii = dwzi * d1z + avz * dw;
    R fdue = game * ((duxii + duxii) * arx + (duyii + dvxii) * ary + (duzii + dwxii) * arz);
    R fdve = game * ((duyii + dvxii) * arx + (dvyii + dvyii) * ary + (dvzii + dwyii) * arz);
    R fdwe = game * ((duzii + dwxii) * arx + (dwyii + dvzii) * ary + (dwzii + dwzii) * arz);
    R gad = game * are / dpn;
    R fdui = gad * (duxi * xpn + duyi * ypn + duzi * zpn);
    R fdvi = gad * (dvxi * xpn + dvyi * ypn + dvzi * zpn);
    R fdwi = gad * (dwxi * xpn + dwyi * ypn + dwzi * zpn);
    R de = gad;
    R flcf = R(A.fcf[inp]);
    R ce = dmin_(flcf, R(A.zero));
    R cp = dmax_(flcf, R(A.zero));
    A.acfe[inp] = de - ce;
    A.acfw[ine] = de + cp;
    R fuuds = cp * R(u[inp]) + ce * R(u[ine]);
    R fvuds = cp * R(v[inp]) + ce * R(v[ine]);
    R fwuds = cp * R(w[inp]) + ce * R(w[ine]);
    R fuhigh = R(0.0), fvhigh = R(0.0), fwhigh = R(0.0);
    bool assigned = false;             // a scheme before QUICK set this face's fluxes
    if (A.lcds) {
      R ue = R(u[inp]) * fxp + R(u[ine]) * fxe + (duxi * dxf + duyi * dyf + duzi * dzf);
      R ve = R(v[inp]) * fxp + R(v[ine]) * fxe + (dvxi * dxf + dvyi * dyf + dvzi * dzf);
      R we = R(w[inp]) * fxp + R(w[ine]) * fxe + (dwxi * dxf + dwyi * dyf + dwzi * dzf);
      fuhigh = flcf * ue; fvhigh = flcf * ve; fwhigh = flcf * we;
      assigned = true;
    }
    if (A.lcds4 && (A.idew == d.nj || A.idew == 1)) {
      R ue = R(1.0) / R(48.0) * (R(27.0) * R(u[inp]) + R(27.0) * R(u[ine]) - R(3.0) * R(u[inw]) - R(3.0) * R(u[inee]));
      R ve = R(1.0) / R(48.0) * (R(27.0) * R(v[inp]) + R(27.0) * R(v[ine]) - R(3.0) * R(v[inw]) - R(3.0) * R(v[inee]));
      R we = R(1.0) / R(48.0) * (R(27.0) * R(w[inp]) + R(27.0) * R(w[ine]) - R(3.0) * R(w[inw]) - R(3.0) * R(w[inee]));
      fuhigh = flcf * ue; fvhigh = flcf * ve; fwhigh = flcf * we;
      assigned = true;
    }
    if (A.lluds) {
      R xf = R(0.25) * (R(A.x[inp]) + R(A.x[ins]) + R(A.x[inb]) + R(A.x[inbs]));
      R yf = R(0.25) * (R(A.y[inp]) + R(A.y[ins]) + R(A.y[inb]) + R(A.y[inbs]));
      R zf = R(0.25) * (R(A.z[inp]) + R(A.z[ins]) + R(A.z[inb]) + R(A.z[inbs]));
      R dxc = xf - R(A.xc[inp]), dyc = yf - R(A.yc[inp]), dzc = zf - R(A.zc[inp]);
      R dxe = R(A.xc[ine]) - xf, dye = R(A.yc[ine]) - yf, dze = R(A.zc[ine]) - zf;
      R dfidx_u = R(A.gud[inw]) * fxw + R(A.gud[inp]) * fxpw;
      R dfidy_u = R(A.gvd[inw]) * fxw + R(A.gvd[inp]) * fxpw;
      R dfidz_u = R(A.gwd[inw]) * fxw + R(A.gwd[inp]) * fxpw;
      R dfidx_u1 = R(A.gud[inee]) * fxee + R(A.gud[ine]) * fxew;
      R dfidy_u1 = R(A.gvd[inee]) * fxee + R(A.gvd[ine]) * fxew;
      R dfidz_u1 = R(A.gwd[inee]) * fxee + R(A.gwd[ine]) * fxew;
      fuhigh = ce * (R(u[ine]) + dxe * dfidx_u1) + cp * (R(u[inp]) + dxc * dfidx_u);
      fvhigh = ce * (R(v[ine]) + dye * dfidy_u1) + cp * (R(v[inp]) + dyc * dfidy_u);
      fwhigh = ce * (R(w[ine]) + dze * dfidz_u1) + cp * (R(w[inp]) + dzc * dfidz_u);
      assigned = true;
    }
    if (A.lquds) {
      int qf;
      if (k > 2 && k < d.nk - 1 && j > 2 && j < d.nj - 1 && i > 2 && i < d.ni - 1)
        quick_face<R>(A, inp, fuhigh, fvhigh, fwhigh);
      else if (!assigned && quick_carried_face(d, A.idew, i, j, k, &qf))
        quick_face<R>(A, qf, fuhigh, fvhigh, fwhigh);
    }
    if (A.flux_limiter) {
      R rr[6];
      rr[0] = (2 * R(A.gux[inp]) * xpn + 2 * R(A.guy[inp]) * ypn + 2 * R(A.guz[inp]) * zpn) / (R(u[ine]) - R(u[inp])) - R(1.0);
      rr[1] = (2 * R(A.gvx[inp]) * xpn + 2 * R(A.gvy[inp]) * ypn + 2 * R(A.gvz[inp]) * zpn) / (R(v[ine]) - R(v[inp])) - R(1.0);
      rr[2] = (2 * R(A.gwx[inp]) * xpn + 2 * R(A.gwy[inp]) * ypn + 2 * R(A.gwz[inp]) * zpn) / (R(w[ine]) - R(w[inp])) - R(1.0);
      rr[3] = (2 * R(A.gux[ine]) * xpn + 2 * R(A.guy[ine]) * ypn + 2 * R(A.guz[ine]) * zpn) / (R(u[inp]) - R(u[ine])) - R(1.0);
      rr[4] = (2 * R(A.gvx[ine]) * xpn + 2 * R(A.gvy[ine]) * ypn + 2 * R(A.gvz[ine]) * zpn) / (R(v[inp]) - R(v[ine])) - R(1.0);
      rr[5] = (2 * R(A.gwx[ine]) * xpn + 2 * R(A.gwy[ine]) * ypn + 2 * R(A.gwz[ine]) * zpn) / (R(w[inp]) - R(w[ine])) - R(1.0);
      R psi[6] = {0, 0, 0, 0, 0, 0};
#pragma unroll
      for (int q = 0; q < 6; ++q) {
        R r = rr[q];
        if (A.lsmart) psi[q] = dmax_(R(0.0), dmin_(dmin_(R(2.0) * r, R(0.75) * r + R(0.25)), R(4.0)));
        if (A.lavl) psi[q] = dmax_(R(0.0), dmin_(dmin_(R(1.5) * r, R(0.75) * r + R(0.25)), R(2.5)));
        if (A.lmuscl) psi[q] = dmax_(R(0.0), dmin_(dmin_(R(2.0) * r, R(0.5) * r + R(0.5)), R(2.0)));
        if (A.lumist) psi[q] = dmax_(R(0.0), dmin_(dmin_(dmin_(R(2.0) * r, R(0.75) * r + R(0.25)), R(0.25) * r + R(0.75)), R(2.0)));
        if (A.lgamma) psi[q] = dmax_(R(0.0), dmin_(r, R(2.0) * r / (r + R(1.0))));
      }
      fuhigh = ce * (R(u[ine]) + fxe * psi[3] * (R(u[inp]) - R(u[ine]))) + cp * (R(u[inp]) + fxp * psi[0] * (R(u[ine]) - R(u[inp])));
      fvhigh = ce * (R(v[ine]) + fxe * psi[4] * (R(v[inp]) - R(v[ine]))) + cp * (R(v[inp]) + fxp * psi[1] * (R(v[ine]) - R(v[inp])));
      fwhigh = ce * (R(w[ine]) + fxe * psi[5] * (R(w[inp]) - R(w[ine]))) + cp * (R(w[inp]) + fxp * psi[2] * (R(w[ine]) - R(w[inp])));
    }
    A.su[inp] = R(A.su[inp]) + R(A.gam) * (fuuds - fuhigh) + fdue - fdui;
    A.sv[inp] = R(A.sv[inp]) + R(A.gam) * (fvuds - fvhigh) + fdve - fdvi;
    A.sw[inp] = R(A.sw[inp]) + R(A.gam) * (fwuds - fwhigh) + fdwe - fdwi;
    A.bp[ine] = -R(A.gam) * (fuuds - fuhigh) - fdue + fdui;
    A.bt[ine] = -R(A.gam) * (fvuds - fvhigh) - fdve + fdvi;
    A.bb[ine] = -R(A.gam) * (fwuds - fwhigh) - fdwe + fdwi;
  }
}

// fluxuvw-overrelaxed-correction.f90:639-650 (reads bp/bt/bb over the whole
// shifted box, including cells the face loop did not write)
__global__ void k_add_staged(Dims d, Box b, int idew, double* su, double* sv, double* sw, const double* __restrict__ bp,
                             const double* __restrict__ bt, const double* __restrict__ bb) {
  BOX_LOOP(b) {
    int i, j, k;
    b.at(t_, i, j, k);
    int inp = ixk(d, i, j, k) + idew;
    su[inp] = su[inp] + bp[inp];
    if (sv) {
      sv[inp] = sv[inp] + bt[inp];
      sw[inp] = sw[inp] + bb[inp];
    }
  }
}

int fluxuvw(int idew, int idns, int idtb, int arvx, int arvy, int arvz, int fif, int acfe, int acfw, int fcf) {
  Ctx& c = ctx();
  const Dims& d = c.d;
  double** F = c.f;
  const cappgpu_params& P = c.prm;
  int dir = 0;
  if (idew == d.nj) dir = 1;
  if (idew == 1) dir = 2;
  if (idew == d.nij) dir = 3;
  if (!dir) { set_error("fluxuvw: idew must be nj, 1 or nij"); return CAPPGPU_E_ARG; }
  int kst = 2, kend = d.nkmm, ist = 2, iend = d.nimm, jst = 2, jend = d.njmm;
  if (dir == 1) { jst = 3; kst = 3; }
  else if (dir == 2) { ist = 3; kst = 3; }
  else { ist = 3; jst = 3; }
  Box b{ist, iend, jst, jend, kst, kend};
  int gd = dir == 1 ? 0 : dir == 2 ? 1 : 2;
  FluxArgs A{F[arvx], F[arvy], F[arvz], F[fif], F[fcf], F[acfe], F[acfw],
             F[CAP_X], F[CAP_Y], F[CAP_Z], F[CAP_XC], F[CAP_YC], F[CAP_ZC],
             F[CAP_U], F[CAP_V], F[CAP_W], F[CAP_VIS],
             F[CAP_GRADU_X], F[CAP_GRADU_Y], F[CAP_GRADU_Z], F[CAP_GRADV_X], F[CAP_GRADV_Y], F[CAP_GRADV_Z],
             F[CAP_GRADW_X], F[CAP_GRADW_Y], F[CAP_GRADW_Z],
             F[CAP_GRADU_X + gd], F[CAP_GRADV_X + gd], F[CAP_GRADW_X + gd],
             F[CAP_SU], F[CAP_SV], F[CAP_SW], F[CAP_BP], F[CAP_BT], F[CAP_BB],
             P.gds[CAP_IU - 1], P.zero, idew, idns, idtb,
             P.lcds, P.lcds4, P.lluds, P.lquds, P.flux_limiter, P.lsmart, P.lavl, P.lmuscl, P.lumist, P.lgamma};
  // precision modes 1-2 assemble in FP32 arithmetic (FP64 storage)
  FaceGeoPtrs G{};
  bool geo = false;
  if (c.fp32(4)) {
    launch(k_fluxuvw_faces<float, false>, grid_for(b.count()), kThreads, c.st, d, b, A, G);
  } else {
    int rc = face_geo(idew, idns, idtb, arvx, arvy, arvz, fif, &G, &geo);
    if (rc) return rc;
    if (geo)
      launch(k_fluxuvw_faces<double, true>, grid_for(b.count()), kThreads, c.st, d, b, A, G);
    else
      launch(k_fluxuvw_faces<double, false>, grid_for(b.count()), kThreads, c.st, d, b, A, G);
  }
  Box b2{2, d.nimm, 2, d.njmm, 2, d.nkmm};
  launch(k_add_staged, grid_for(b2.count()), kThreads, c.st, d, b2, idew, F[CAP_SU], F[CAP_SV], F[CAP_SW], F[CAP_BP],
                                                            F[CAP_BT], F[CAP_BB]);
  CAP_CHECK_LAUNCH();
  size_t nb = sizeof(double) * d.nijk;
  CAP_CUDA(cudaMemsetAsync(F[CAP_BP], 0, nb, c.st));
  CAP_CUDA(cudaMemsetAsync(F[CAP_BT], 0, nb, c.st));
  CAP_CUDA(cudaMemsetAsync(F[CAP_BB], 0, nb, c.st));
  return CAPPGPU_OK;
}

// ---------------------------------------------------------------- calcuvw
struct SrcArgs {
  double *ap, *spv, *sp, *su, *sv, *sw;
  const double *gpx, *gpy, *gpz, *vol, *den, *t, *uo, *vo, *wo, *uoo, *voo, *woo;
  double gradpcmf, densit, beta, tref, gravx, gravy, gravz, timestep, btime;
  int const_mflux, buoy, boussinesq, bdf;
};

// calcuvw.f90:56-125
__global__ void k_calcuvw_sources(Dims d, Box b, SrcArgs A) {
  BOX_LOOP(b) {
    int i, j, k;
    b.at(t_, i, j, k);
    int inp = ixk(d, i, j, k);
    double ap = 0.0, spv = 0.0, sp = 0.0;
    double su = -A.gpx[inp] * A.vol[inp];
    double sv = -A.gpy[inp] * A.vol[inp];
    double sw = -A.gpz[inp] * A.vol[inp];
    if (A.const_mflux) su = su + A.gradpcmf * A.vol[inp];
    if (A.buoy) {
      double heat = 0.0;
      if (A.boussinesq) heat = A.beta * A.densit * (A.t[inp] - A.tref) * A.vol[inp];
      else heat = (A.densit - A.den[inp]) * A.vol[inp];
      su = su - A.gravx * heat;
      sv = sv - A.gravy * heat;
      sw = sw - A.gravz * heat;
    }
    if (A.bdf) {
      double apotime = A.den[inp] * A.vol[inp] / A.timestep;
      double sut = apotime * ((1 + A.btime) * A.uo[inp] - 0.5 * A.btime * A.uoo[inp]);
      double svt = apotime * ((1 + A.btime) * A.vo[inp] - 0.5 * A.btime * A.voo[inp]);
      double swt = apotime * ((1 + A.btime) * A.wo[inp] - 0.5 * A.btime * A.woo[inp]);
      su = su + sut;
      sv = sv + svt;
      sw = sw + swt;
      ap = ap + apotime * (1 + 0.5 * A.btime);
      spv = spv + apotime * (1 + 0.5 * A.btime);
      sp = sp + apotime * (1 + 0.5 * A.btime);
    }
    A.ap[inp] = ap; A.spv[inp] = spv; A.sp[inp] = sp;
    A.su[inp] = su; A.sv[inp] = sv; A.sw[inp] = sw;
  }
}

// calcuvw.f90:161-337 (first-order wall model), one wall per launch
// top: 0 the bottom wall, else the k plane of the top wall's cells
__global__ void k_calcuvw_wall(Dims d, int top, const double* __restrict__ xc, const double* __restrict__ yc,
                               const double* __restrict__ zc, const double* __restrict__ fz,
                               const double* __restrict__ a3x, const double* __restrict__ a3y,
                               const double* __restrict__ a3z, const double* __restrict__ u,
                               const double* __restrict__ v, const double* __restrict__ w,
                               const double* __restrict__ vis, double* ap, double* spv, double* sp, double* su,
                               double* sv, double* sw) {
  Box b{3, d.nimm, 3, d.njmm, 1, 1};
  // nx,ny,nz of the dnw dot product are the integer extents ni,nj,nk
  // (set_parameters.f90:34-36; calcuvw.f90:187,277)
  const double nxi = (double)d.ni, nyi = (double)d.nj, nzi = (double)d.nk;
  BOX_LOOP(b) {
    int i, j, kk;
    b.at(t_, i, j, kk);
    int inbc, ingc, iface;
    double fxp, fxe;
    if (!top) {
      inbc = ixk(d, i, j, 3); ingc = inbc - d.nij; iface = ingc;
      fxp = fz[ingc]; fxe = 1.0 - fxp;
    } else {
      inbc = ixk(d, i, j, top); ingc = inbc + d.nij; iface = inbc;  // lk(nimm) (calcuvw.f90:254) or lk(nkmm)
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

__global__ void k_scale_all(long long n, double* a, double s) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
    a[t] = s * a[t];
}

struct AsmArgs {
  const double *ae, *aw, *an, *as, *at, *ab;
  double *ap, *su, *spx, *srcx, *apx;
  const double *fld, *old, *den, *vol;
  double urfrs, urfms, timestep;
  int cn, comp;
};

// calcuvw.f90:358-385 (u), 394-420 (v), 431-457 (w)
__global__ void k_calcuvw_assemble(Dims d, Box b, AsmArgs A) {
  BOX_LOOP(b) {
    int i, j, k;
    b.at(t_, i, j, k);
    int inp = ixk(d, i, j, k);
    double diag;
    if (A.cn) {
      double apotime = A.den[inp] * A.vol[inp] / A.timestep;
      A.srcx[inp] = A.srcx[inp] +
                    (A.ae[inp] * A.old[inp + d.nj] + A.aw[inp] * A.old[inp - d.nj] + A.an[inp] * A.old[inp + 1] +
                     A.as[inp] * A.old[inp - 1] + A.at[inp] * A.old[inp + d.nij] + A.ab[inp] * A.old[inp - d.nij]) +
                    (apotime - A.ae[inp] - A.aw[inp] - A.an[inp] - A.as[inp] - A.at[inp] - A.ab[inp]) * A.old[inp];
      if (A.comp == 0) A.ap[inp] = A.ap[inp] + apotime;
      else A.spx[inp] = A.spx[inp] + apotime;
    }
    diag = A.comp == 0 ? A.ap[inp] : A.spx[inp];
    double ap = A.ae[inp] + A.aw[inp] + A.an[inp] + A.as[inp] + A.at[inp] + A.ab[inp] + diag;
    ap = ap * A.urfrs;
    A.ap[inp] = ap;
    A.su[inp] = A.srcx[inp] + A.urfms * ap * A.fld[inp];
    A.apx[inp] = 1.0 / (ap + CAP_SMALL);
  }
}

static int calcuvw_assemble(int comp) {
  Ctx& c = ctx();
  const Dims& d = c.d;
  double** F = c.f;
  const cappgpu_params& P = c.prm;
  int ifi = CAP_IU + comp;
  AsmArgs A{F[CAP_AE], F[CAP_AW], F[CAP_AN], F[CAP_AS], F[CAP_AT], F[CAP_AB],
            F[CAP_AP], F[CAP_SU],
            comp == 0 ? nullptr : comp == 1 ? F[CAP_SPV] : F[CAP_SP],
            comp == 0 ? F[CAP_SU] : comp == 1 ? F[CAP_SV] : F[CAP_SW],
            comp == 0 ? F[CAP_APU] : comp == 1 ? F[CAP_APV] : F[CAP_APW],
            comp == 0 ? F[CAP_U] : comp == 1 ? F[CAP_V] : F[CAP_W],
            comp == 0 ? F[CAP_UO] : comp == 1 ? F[CAP_VO] : F[CAP_WO],
            F[CAP_DEN], F[CAP_VOL],
            1.0 / P.urf[ifi - 1], 1.0 - P.urf[ifi - 1], P.timestep, P.cn, comp};
  Box b{3, d.nimm, 3, d.njmm, 2, d.nkm};
  launch(k_calcuvw_assemble, grid_for(b.count()), kThreads, c.st, d, b, A);
  CAP_CHECK_LAUNCH();
  return CAPPGPU_OK;
}

// calcuvw.f90:3-464 with isol=1 and Gauss gradients
int calcuvw(cappgpu_solve_report* rep3) {
  Ctx& c = ctx();
  const Dims& d = c.d;
  double** F = c.f;
  const cappgpu_params& P = c.prm;
  int rc;
  // the top-wall loop addresses lk(nimm) (calcuvw.f90:254): inside the
  // array only when nimm+1 <= nk; params.top_plane = 1 takes lk(nkmm)
  const int ktop = P.top_plane ? d.nkmm : d.nimm;
  if (ktop + 1 > d.nk) {
    set_error("top wall index lk(nimm) of calcuvw.f90:254 leaves the array (ni=%d > nk=%d); "
              "params.top_plane = 1 takes lk(nkmm)", d.ni, d.nk);
    return CAPPGPU_E_ARG;
  }
  if ((rc = grad_gauss(CAP_U, CAP_GRADU_X, CAP_GRADU_Y, CAP_GRADU_Z))) return rc;
  if ((rc = grad_gauss(CAP_V, CAP_GRADV_X, CAP_GRADV_Y, CAP_GRADV_Z))) return rc;
  if ((rc = grad_gauss(CAP_W, CAP_GRADW_X, CAP_GRADW_Y, CAP_GRADW_Z))) return rc;
  if ((rc = grad_gauss(CAP_PP, CAP_GRADP_X, CAP_GRADP_Y, CAP_GRADP_Z))) return rc;
  SrcArgs S{F[CAP_AP], F[CAP_SPV], F[CAP_SP], F[CAP_SU], F[CAP_SV], F[CAP_SW],
            F[CAP_GRADP_X], F[CAP_GRADP_Y], F[CAP_GRADP_Z], F[CAP_VOL], F[CAP_DEN], F[CAP_T],
            F[CAP_UO], F[CAP_VO], F[CAP_WO], F[CAP_UOO], F[CAP_VOO], F[CAP_WOO],
            P.gradpcmf, P.densit, P.beta, P.tref, P.gravx, P.gravy, P.gravz, P.timestep, P.btime,
            P.const_mflux, P.lcal[CAP_IEN - 1] && P.lbuoy, P.boussinesq, P.bdf};
  Box bs{3, d.nimm, 3, d.njmm, 2, d.nkm};
  launch(k_calcuvw_sources, grid_for(bs.count()), kThreads, c.st, d, bs, S);
  CAP_CHECK_LAUNCH();
  if ((rc = fluxuvw(d.nj, 1, d.nij, CAP_AR1X, CAP_AR1Y, CAP_AR1Z, CAP_FX, CAP_AE, CAP_AW, CAP_F1))) return rc;
  if ((rc = fluxuvw(1, d.nij, d.nj, CAP_AR2X, CAP_AR2Y, CAP_AR2Z, CAP_FY, CAP_AN, CAP_AS, CAP_F2))) return rc;
  if ((rc = fluxuvw(d.nij, d.nj, 1, CAP_AR3X, CAP_AR3Y, CAP_AR3Z, CAP_FZ, CAP_AT, CAP_AB, CAP_F3))) return rc;
  int gw = grid_for((long long)(d.nimm - 2) * (d.njmm - 2));
  for (int top : {0, ktop})
    launch(k_calcuvw_wall, gw, kThreads, c.st, d, top, F[CAP_XC], F[CAP_YC], F[CAP_ZC], F[CAP_FZ], F[CAP_AR3X],
                                              F[CAP_AR3Y], F[CAP_AR3Z], F[CAP_U], F[CAP_V], F[CAP_W], F[CAP_VIS],
                                              F[CAP_AP], F[CAP_SPV], F[CAP_SP], F[CAP_SU], F[CAP_SV], F[CAP_SW]);
  CAP_CHECK_LAUNCH();
  if (P.cn) {
    for (int q : {CAP_AE, CAP_AN, CAP_AT, CAP_AW, CAP_AS, CAP_AB})
      launch(k_scale_all, grid_for(d.nijk), kThreads, c.st, d.nijk, F[q], 0.5);
    CAP_CHECK_LAUNCH();
  }
  int agg = 0;
  for (int comp = 0; comp < 3; ++comp) {
    if ((rc = calcuvw_assemble(comp))) return rc;
    rc = sipsol(CAP_U + comp, CAP_IU + comp, rep3 ? &rep3[comp] : nullptr);
    if (rc < 0) return rc;
    agg |= rc;
  }
  return agg;
}

// ----------------------------------------------- PISO pressure assembly
struct PeqArgs {
  const double *arvx, *arvy, *arvz, *fif;
  double *acfe, *acfw, *fcf, *bp, *su;
  const double *x, *y, *z, *xc, *yc, *zc, *u, *v, *w, *p, *den, *vol, *apu;
  const double *gux, *guy, *guz, *gvx, *gvy, *gvz, *gwx, *gwy, *gwz, *gpx, *gpy, *gpz;
  int idew, idns, idtb, ipc;
};

// PISO_assemble_pressure_eq.f90:48-237 for one face; GEO: the geometric
// terms come from the per-face cache (FP64 form only)
template <typename R, bool GEO>
__global__ void k_piso_peq_faces(Dims d, Box b, PeqArgs A, FaceGeoPtrs G) {
  BOX_LOOP(b) {
    int i, j, k;
    b.at(t_, i, j, k);
    int inp = ixk(d, i, j, k);
    int ine = inp + A.idew;
    R fxe = R(A.fif[inp]), fxp = R(1.0) - fxe;
    R arx = R(A.arvx[inp]), ary = R(A.arvy[inp]), arz = R(A.arvz[inp]);
    R xpn, ypn, zpn, dpn, are, costn, avx, avy, avz, dxf, dyf, dzf;
    if constexpr (GEO) {
      xpn = G.q[GQ_XPN][inp]; ypn = G.q[GQ_YPN][inp]; zpn = G.q[GQ_ZPN][inp];
      dpn = G.q[GQ_DPN][inp]; are = G.q[GQ_ARE][inp]; costn = G.q[GQ_COSTN][inp];
      avx = G.q[GQ_AVX][inp]; avy = G.q[GQ_AVY][inp]; avz = G.q[GQ_AVZ][inp];
      dxf = G.q[GQ_DXF][inp]; dyf = G.q[GQ_DYF][inp]; dzf = G.q[GQ_DZF][inp];
    } else {
      int ins = inp - A.idns, inb = inp - A.idtb, inbs = inb - A.idns;
      R xf = R(0.25) * (R(A.x[inp]) + R(A.x[ins]) + R(A.x[inb]) + R(A.x[inbs]));
      R yf = R(0.25) * (R(A.y[inp]) + R(A.y[ins]) + R(A.y[inb]) + R(A.y[inbs]));
      R zf = R(0.25) * (R(A.z[inp]) + R(A.z[ins]) + R(A.z[inb]) + R(A.z[inbs]));
      R xi = R(A.xc[inp]) * fxp + R(A.xc[ine]) * fxe;
      R yi = R(A.yc[inp]) * fxp + R(A.yc[ine]) * fxe;
      R zi = R(A.zc[inp]) * fxp + R(A.zc[ine]) * fxe;
      xpn = R(A.xc[ine]) - R(A.xc[inp]); ypn = R(A.yc[ine]) - R(A.yc[inp]); zpn = R(A.zc[ine]) - R(A.zc[inp]);
      dpn = sqrt_(xpn * xpn + ypn * ypn + zpn * zpn);
      R ixi1 = xpn / dpn, ixi2 = ypn / dpn, ixi3 = zpn / dpn;
      are = sqrt_(arx * arx + ary * ary + arz * arz);
      R vole = xpn * arx + ypn * ary + zpn * arz;
      R nxx = arx / are, nyy = ary / are, nzz = arz / are;
      costn = nxx * ixi1 + nyy * ixi2 + nzz * ixi3;
      avx = arx / vole; avy = ary / vole; avz = arz / vole;
      dxf = xf - xi; dyf = yf - yi; dzf = zf - zi;
    }
    R d1x = costn, d1y = costn, d1z = costn;
    R d2x = xpn * costn, d2y = ypn * costn, d2z = zpn * costn;
    R dene = R(A.den[inp]) * fxp + R(A.den[ine]) * fxe;
    R game = dene * (fxp * R(A.vol[inp]) * R(A.apu[inp]) + fxe * R(A.vol[ine]) * R(A.apu[ine]));
    R acf = game * are / dpn;
    A.acfe[inp] = acf;
    A.acfw[ine] = acf;
    if (A.ipc > 0) {
      R dfixi = R(A.gpx[inp]) * fxp + R(A.gpx[ine]) * fxe;
      R dfiyi = R(A.gpy[inp]) * fxp + R(A.gpy[ine]) * fxe;
      R dfizi = R(A.gpz[inp]) * fxp + R(A.gpz[ine]) * fxe;
      R dp = R(A.p[ine]) - R(A.p[inp]) - (dfixi * d2x + dfiyi * d2y + dfizi * d2z);
      R dfixii = dfixi * d1x + avx * dp;
      R dfiyii = dfiyi * d1y + avy * dp;
      R dfizii = dfizi * d1z + avz * dp;
      R fdfie = game * (dfixii * arx + dfiyii * ary + dfizii * arz);
      R fdfii = acf * (dfixi * xpn + dfiyi * ypn + dfizi * zpn);   // game*are/dpn*(...)
      R suadd = fdfie - fdfii;
      A.su[inp] = R(A.su[inp]) + suadd;
      A.bp[inp] = suadd;
      R duxi = R(A.gux[inp]) * fxp + R(A.gux[ine]) * fxe;
      R duyi = R(A.guy[inp]) * fxp + R(A.guy[ine]) * fxe;
      R duzi = R(A.guz[inp]) * fxp + R(A.guz[ine]) * fxe;
      R ui = R(A.u[inp]) * fxp + R(A.u[ine]) * fxe + duxi * dxf + duyi * dyf + duzi * dzf;
      duxi = R(A.gvx[inp]) * fxp + R(A.gvx[ine]) * fxe;
      duyi = R(A.gvy[inp]) * fxp + R(A.gvy[ine]) * fxe;
      duzi = R(A.gvz[inp]) * fxp + R(A.gvz[ine]) * fxe;
      R vi = R(A.v[inp]) * fxp + R(A.v[ine]) * fxe + duxi * dxf + duyi * dyf + duzi * dzf;
      duxi = R(A.gwx[inp]) * fxp + R(A.gwx[ine]) * fxe;
      duyi = R(A.gwy[inp]) * fxp + R(A.gwy[ine]) * fxe;
      duzi = R(A.gwz[inp]) * fxp + R(A.gwz[ine]) * fxe;
      R wi = R(A.w[inp]) * fxp + R(A.w[ine]) * fxe + duxi * dxf + duyi * dyf + duzi * dzf;
      A.fcf[inp] = dene * (ui * arx + vi * ary + wi * arz);
    }
  }
}

// PISO_assemble_pressure_eq.f90:241-257: su(inp+idew) -= bp(inp+idew)
__global__ void k_sub_staged(Dims d, Box b, int idew, double* su, const double* __restrict__ bp) {
  BOX_LOOP(b) {
    int i, j, k;
    b.at(t_, i, j, k);
    int inp = ixk(d, i, j, k) + idew;
    su[inp] = su[inp] - bp[inp];
  }
}

int piso_assemble(int idew, int idns, int idtb, int arvx, int arvy, int arvz, int fif, int acfe, int acfw, int fcf,
                  int ipc, int bp) {
  Ctx& c = ctx();
  const Dims& d = c.d;
  double** F = c.f;
  CAP_CUDA(cudaMemsetAsync(F[bp], 0, sizeof(double) * d.nijk, c.st));
  PeqArgs A{F[arvx], F[arvy], F[arvz], F[fif], F[acfe], F[acfw], F[fcf], F[bp], F[CAP_SU],
            F[CAP_X], F[CAP_Y], F[CAP_Z], F[CAP_XC], F[CAP_YC], F[CAP_ZC], F[CAP_U], F[CAP_V], F[CAP_W],
            F[CAP_P], F[CAP_DEN], F[CAP_VOL], F[CAP_APU],
            F[CAP_GRADU_X], F[CAP_GRADU_Y], F[CAP_GRADU_Z], F[CAP_GRADV_X], F[CAP_GRADV_Y], F[CAP_GRADV_Z],
            F[CAP_GRADW_X], F[CAP_GRADW_Y], F[CAP_GRADW_Z], F[CAP_GRADP_X], F[CAP_GRADP_Y], F[CAP_GRADP_Z],
            idew, idns, idtb, ipc};
  Box b{2, d.nimm, 2, d.njmm, 2, d.nkmm};
  FaceGeoPtrs G{};
  bool geo = false;
  if (c.fp32(16)) {
    launch(k_piso_peq_faces<float, false>, grid_for(b.count()), kThreads, c.st, d, b, A, G);
  } else {
    int rc = face_geo(idew, idns, idtb, arvx, arvy, arvz, fif, &G, &geo);
    if (rc) return rc;
    if (geo)
      launch(k_piso_peq_faces<double, true>, grid_for(b.count()), kThreads, c.st, d, b, A, G);
    else
      launch(k_piso_peq_faces<double, false>, grid_for(b.count()), kThreads, c.st, d, b, A, G);
  }
  CAP_CHECK_LAUNCH();
  if (ipc > 0) {
    Box bi{3, d.nimm, 3, d.njmm, 3, d.nkmm};
    launch(k_sub_staged, grid_for(bi.count()), kThreads, c.st, d, bi, idew, F[CAP_SU], F[bp]);
    CAP_CHECK_LAUNCH();
  }
  return CAPPGPU_OK;
}

// assemble_pressure_eq.f90:38-121
__global__ void k_apeq_faces(Dims d, Box b, const double* __restrict__ arvx, const double* __restrict__ arvy,
                             const double* __restrict__ arvz, const double* __restrict__ fif, double* acfe,
                             double* acfw, double* fcf, const double* __restrict__ xc, const double* __restrict__ yc,
                             const double* __restrict__ zc, const double* __restrict__ vol,
                             const double* __restrict__ su, const double* __restrict__ sv,
                             const double* __restrict__ sw, int idew) {
  BOX_LOOP(b) {
    int i, j, k;
    b.at(t_, i, j, k);
    int inp = ixk(d, i, j, k), ine = inp + idew;
    double fxe = fif[inp], fxp = 1.0 - fxe;
    double xpn = xc[ine] - xc[inp], ypn = yc[ine] - yc[inp], zpn = zc[ine] - zc[inp];
    double arx = arvx[inp], ary = arvy[inp], arz = arvz[inp];
    double are = sqrt(arx * arx + ary * ary + arz * arz);
    double nxx = arx / are, nyy = ary / are, nzz = arz / are;
    double smdpn = (arx * arx + ary * ary + arz * arz) / (arx * xpn * nxx + ary * ypn * nyy + arz * zpn * nzz);
    double a = (fxp * vol[inp] + fxe * vol[ine]) * smdpn;
    acfe[inp] = a;
    acfw[ine] = a;
    double ui = su[inp] * fxp + su[ine] * fxe;
    double vi = sv[inp] * fxp + sv[ine] * fxe;
    double wi = sw[inp] * fxp + sw[ine] * fxe;
    fcf[inp] = ui * arx + vi * ary + wi * arz;
  }
}

int assemble_pressure_eq(int idew, int idns, int idtb, int arvx, int arvy, int arvz, int fif, int acfe, int acfw,
                         int fcf) {
  Ctx& c = ctx();
  const Dims& d = c.d;
  double** F = c.f;
  (void)idns; (void)idtb;
  Box b{2, d.nimm, 2, d.njmm, 2, d.nkmm};
  launch(k_apeq_faces, grid_for(b.count()), kThreads, c.st, d, b, F[arvx], F[arvy], F[arvz], F[fif], F[acfe],
                                                          F[acfw], F[fcf], F[CAP_XC], F[CAP_YC], F[CAP_ZC],
                                                          F[CAP_VOL], F[CAP_SU], F[CAP_SV], F[CAP_SW], idew);
  CAP_CHECK_LAUNCH();
  return CAPPGPU_OK;
}

// ------------------------------------------------------------ PISO HbyA
struct HbyaArgs {
  double *sp, *su, *sv, *sw;
  const double *he, *hw, *hn, *hs, *ht, *hb;
  const double *u, *v, *w, *uo, *vo, *wo, *uoo, *voo, *woo, *den, *vol, *t;
  double densit, beta, tref, gravx, gravy, gravz, timestep, btime;
  int buoy, boussinesq, bdf, cn;
};

// PISO_getHbyA.f90:35-200: sources and H(U) for u, v, w (old U read
// everywhere; the velocity update is a separate pass).
__global__ void k_hbya_h(Dims d, Box b, HbyaArgs A) {
  BOX_LOOP(b) {
    int i, j, k;
    b.at(t_, i, j, k);
    int inp = ixk(d, i, j, k);
    double sv3[3] = {0.0, 0.0, 0.0};
    A.sp[inp] = 0.0;
    if (A.buoy) {
      double heat = 0.0;
      if (A.boussinesq) heat = A.beta * A.densit * (A.t[inp] - A.tref) * A.vol[inp];
      else heat = (A.densit - A.den[inp]) * A.vol[inp];
      sv3[0] = sv3[0] - A.gravx * heat;
      sv3[1] = sv3[1] - A.gravy * heat;
      sv3[2] = sv3[2] - A.gravz * heat;
    }
    if (A.bdf) {
      double apotime = A.den[inp] * A.vol[inp] / A.timestep;
      double sut = apotime * ((1 + A.btime) * A.uo[inp] - 0.5 * A.btime * A.uoo[inp]);
      double svt = apotime * ((1 + A.btime) * A.vo[inp] - 0.5 * A.btime * A.voo[inp]);
      double swt = apotime * ((1 + A.btime) * A.wo[inp] - 0.5 * A.btime * A.woo[inp]);
      sv3[0] = sv3[0] + sut;
      sv3[1] = sv3[1] + svt;
      sv3[2] = sv3[2] + swt;
    }
    const double* fl[3] = {A.u, A.v, A.w};
    const double* ol[3] = {A.uo, A.vo, A.wo};
    int ine = inp + d.nj, inw = inp - d.nj, inn = inp + 1, ins = inp - 1, int_ = inp + d.nij, inb = inp - d.nij;
    double he = A.he[inp], hw = A.hw[inp], hn = A.hn[inp], hs = A.hs[inp], ht = A.ht[inp], hb = A.hb[inp];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      const double* f = fl[q];
      const double* o = ol[q];
      if (A.cn) {
        double apotime = A.den[inp] * A.vol[inp] / A.timestep;
        sv3[q] = sv3[q] + (he * o[ine] + hw * o[inw] + hn * o[inn] + hs * o[ins] + ht * o[int_] + hb * o[inb]) +
                 (apotime - he - hw - hn - hs - ht - hb) * o[inp];
      }
      sv3[q] = sv3[q] + (he * f[ine] + hw * f[inw] + hn * f[inn] + hs * f[ins] + ht * f[int_] + hb * f[inb]);
    }
    A.su[inp] = sv3[0];
    A.sv[inp] = sv3[1];
    A.sw[inp] = sv3[2];
  }
}

// PISO_getHbyA.f90:204-216
__global__ void k_hbya_u(Dims d, Box b, double* u, double* v, double* w, const double* __restrict__ su,
                         const double* __restrict__ sv, const double* __restrict__ sw, const double* __restrict__ apu,
                         const double* __restrict__ apv, const double* __restrict__ apw) {
  BOX_LOOP(b) {
    int i, j, k;
    b.at(t_, i, j, k);
    int inp = ixk(d, i, j, k);
    u[inp] = su[inp] * apu[inp];
    v[inp] = sv[inp] * apv[inp];
    w[inp] = sw[inp] * apw[inp];
  }
}

int piso_gethbya() {
  Ctx& c = ctx();
  const Dims& d = c.d;
  double** F = c.f;
  const cappgpu_params& P = c.prm;
  HbyaArgs A{F[CAP_SP], F[CAP_SU], F[CAP_SV], F[CAP_SW], F[CAP_HE], F[CAP_HW], F[CAP_HN], F[CAP_HS], F[CAP_HT],
             F[CAP_HB], F[CAP_U], F[CAP_V], F[CAP_W], F[CAP_UO], F[CAP_VO], F[CAP_WO], F[CAP_UOO], F[CAP_VOO],
             F[CAP_WOO], F[CAP_DEN], F[CAP_VOL], F[CAP_T], P.densit, P.beta, P.tref, P.gravx, P.gravy, P.gravz,
             P.timestep, P.btime, P.lcal[CAP_IEN - 1] && P.lbuoy, P.boussinesq, P.bdf, P.cn};
  Box b{3, d.nimm, 3, d.njmm, 3, d.nkmm};
  launch(k_hbya_h, grid_for(b.count()), kThreads, c.st, d, b, A);
  launch(k_hbya_u, grid_for(b.count()), kThreads, c.st, d, b, F[CAP_U], F[CAP_V], F[CAP_W], F[CAP_SU], F[CAP_SV],
                                                       F[CAP_SW], F[CAP_APU], F[CAP_APV], F[CAP_APW]);
  CAP_CHECK_LAUNCH();
  int rc;
  if ((rc = grad_gauss(CAP_U, CAP_GRADU_X, CAP_GRADU_Y, CAP_GRADU_Z))) return rc;
  if ((rc = grad_gauss(CAP_V, CAP_GRADV_X, CAP_GRADV_Y, CAP_GRADV_Z))) return rc;
  return grad_gauss(CAP_W, CAP_GRADW_X, CAP_GRADW_Y, CAP_GRADW_Z);
}

// ------------------------------------------------- PISO corrector pieces
// su = -div(F) (PISO_multiple_correction.f90:91-98) and/or ap = sum(a_nb) (:103-110)
__global__ void k_div_ap(Dims d, Box b, int do_su, int do_ap, double* su, double* ap, const double* __restrict__ f1,
                         const double* __restrict__ f2, const double* __restrict__ f3, const double* __restrict__ ae,
                         const double* __restrict__ aw, const double* __restrict__ an, const double* __restrict__ as,
                         const double* __restrict__ at, const double* __restrict__ ab) {
  BOX_LOOP(b) {
    int i, j, k;
    b.at(t_, i, j, k);
    int inp = ixk(d, i, j, k);
    if (do_su) su[inp] = -f1[inp] + f1[inp - d.nj] - f2[inp] + f2[inp - 1] - f3[inp] + f3[inp - d.nij];
    if (do_ap) ap[inp] = ae[inp] + aw[inp] + an[inp] + as[inp] + at[inp] + ab[inp];
  }
}

// reference cell pin (PISO_multiple_correction.f90:117-129)
__global__ void k_pin(int inpr, double* ap, double* ae, double* aw, double* an, double* as, double* at, double* ab,
                      double* su, const double* p) {
  ap[inpr] = 1.0;
  ae[inpr] = 0.0; aw[inpr] = 0.0; an[inpr] = 0.0; as[inpr] = 0.0; at[inpr] = 0.0; ab[inpr] = 0.0;
  su[inpr] = p[inpr];
}

// F -= a (p_nb - p_P) (PISO_multiple_correction.f90:209-252)
__global__ void k_flux_corr(Dims d, Box b, double* f1, double* f2, double* f3, const double* __restrict__ ae,
                            const double* __restrict__ an, const double* __restrict__ at,
                            const double* __restrict__ p) {
  BOX_LOOP(b) {
    int i, j, k;
    b.at(t_, i, j, k);
    int inp = ixk(d, i, j, k);
    f1[inp] = f1[inp] - ae[inp] * (p[inp + d.nj] - p[inp]);
    f2[inp] = f2[inp] - an[inp] * (p[inp + 1] - p[inp]);
    f3[inp] = f3[inp] - at[inp] * (p[inp + d.nij] - p[inp]);
  }
}

// U -= apu gradp vol (PISO_multiple_correction.f90:270-282); SIMPLE form
// U -= vol apu gradp (calcp...f90:202-205) with simple=1 plus the p update.
__global__ void k_vel_corr(Dims d, Box b, int simple, double* u, double* v, double* w, const double* __restrict__ apu,
                           const double* __restrict__ apv, const double* __restrict__ apw,
                           const double* __restrict__ gpx, const double* __restrict__ gpy,
                           const double* __restrict__ gpz, const double* __restrict__ vol, double* p,
                           const double* __restrict__ pp, double urfp, const double* ppref_ptr) {
  BOX_LOOP(b) {
    int i, j, k;
    b.at(t_, i, j, k);
    int inp = ixk(d, i, j, k);
    if (!simple) {
      u[inp] = u[inp] - apu[inp] * gpx[inp] * vol[inp];
      v[inp] = v[inp] - apv[inp] * gpy[inp] * vol[inp];
      w[inp] = w[inp] - apw[inp] * gpz[inp] * vol[inp];
    } else {
      u[inp] = u[inp] - vol[inp] * apu[inp] * gpx[inp];
      v[inp] = v[inp] - vol[inp] * apv[inp] * gpy[inp];
      w[inp] = w[inp] - vol[inp] * apw[inp] * gpz[inp];
      p[inp] = p[inp] + urfp * (pp[inp] - *ppref_ptr);
    }
  }
}

// continuityErrors.h:59-81 partial sums (global, sum |local|) and the
// last cell's local error
__global__ void k_continuity(Dims d, Box b, const double* __restrict__ f1, const double* __restrict__ f2,
                             const double* __restrict__ f3, double* part, double* last) {
  double v[2] = {0.0, 0.0};
  BOX_LOOP(b) {
    int i, j, k;
    b.at(t_, i, j, k);
    int inp = ixk(d, i, j, k);
    double loc = -f1[inp] + f1[inp - d.nj] - f2[inp] + f2[inp - 1] - f3[inp] + f3[inp - d.nij];
    v[0] += loc;
    v[1] += fabs(loc);
    if (t_ == n_ - 1) *last = loc;
  }
  block_reduce_store<2>(v, part);
}

int continuity_errors() {
  Ctx& c = ctx();
  const Dims& d = c.d;
  cappgpu_params& P = c.prm;
  Box b{3, d.nimm, 3, d.njmm, 2, d.nkm};
  launch(k_continuity, kRedBlocks, kThreads, c.st, d, b, c.f[CAP_F1], c.f[CAP_F2], c.f[CAP_F3], c.partials,
                                                  c.redout + 3);
  CAP_CHECK_LAUNCH();
  int rc = finish_reduce(2);
  if (rc) return rc;
  double r[4];
  if ((rc = fetch_reduce(4, r))) return rc;
  P.globalconterr = r[0];
  P.sumlocalconterr = r[1];
  P.localconterr = r[3];
  P.cumulativeconterr = P.cumulativeconterr + r[0];
  return CAPPGPU_OK;
}

// CourantNo.h:29-52: su = sum |F| over the cell faces (su zeroed first),
// max(su/vol), sum vol, sum su.
__global__ void k_courant(Dims d, Box b, double* su, const double* __restrict__ f1, const double* __restrict__ f2,
                          const double* __restrict__ f3, const double* __restrict__ vol, double* part) {
  double v[2] = {0.0, 0.0};
  double mx = 0.0;
  BOX_LOOP(b) {
    int i, j, k;
    b.at(t_, i, j, k);
    int inp = ixk(d, i, j, k);
    double s = fabs(f1[inp]) + fabs(f1[inp - d.nj]) + fabs(f2[inp]) + fabs(f2[inp - 1]) + fabs(f3[inp]) +
               fabs(f3[inp - d.nij]);
    su[inp] = s;
    mx = fmax(mx, s / vol[inp]);
    v[0] += vol[inp];
    v[1] += s;
  }
  block_reduce_store<2>(v, part);
  __syncthreads();
  block_max_store(mx, part + 2 * kRedBlocks);
}

int courant() {
  Ctx& c = ctx();
  const Dims& d = c.d;
  cappgpu_params& P = c.prm;
  if (!P.ltransient) return CAPPGPU_OK;
  CAP_CUDA(cudaMemsetAsync(c.f[CAP_SU], 0, sizeof(double) * d.nijk, c.st));
  Box b{3, d.nimm, 3, d.njmm, 2, d.nkm};
  launch(k_courant, kRedBlocks, kThreads, c.st, d, b, c.f[CAP_SU], c.f[CAP_F1], c.f[CAP_F2], c.f[CAP_F3],
                                               c.f[CAP_VOL], c.partials);
  CAP_CHECK_LAUNCH();
  int rc = finish_reduce(2);
  if (rc) return rc;
  double r[2];
  if ((rc = fetch_reduce(2, r))) return rc;
  if ((rc = finish_reduce(1, true, 2))) return rc;   // max over the third partial slot
  double conum;
  if ((rc = fetch_reduce(1, &conum))) return rc;
  double suma = r[0], meanconum = r[1];
  conum = 0.5 * conum * P.timestep;
  meanconum = 0.5 * meanconum / suma * P.timestep;
  if (P.conumfix) {
    double dt = P.timestep;
    P.timestep = P.conumfixvalue / conum * P.timestep;
    conum = conum * P.timestep / dt;
    meanconum = meanconum * P.timestep / dt;
  }
  P.time = P.time + P.timestep;
  P.conum = conum;
  P.meanconum = meanconum;
  return CAPPGPU_OK;
}

// PISO_multiple_correction.f90:3-296
int piso_multiple_correction(cappgpu_solve_report* reps) {
  Ctx& c = ctx();
  const Dims& d = c.d;
  double** F = c.f;
  cappgpu_params& P = c.prm;
  double reltol = P.sor[CAP_IP - 1];
  size_t nb = sizeof(double) * d.nijk;
  const int hsrc[6] = {CAP_AE, CAP_AW, CAP_AN, CAP_AS, CAP_AT, CAP_AB};
  const int hdst[6] = {CAP_HE, CAP_HW, CAP_HN, CAP_HS, CAP_HT, CAP_HB};
  for (int q = 0; q < 6; ++q) CAP_CUDA(cudaMemcpyAsync(F[hdst[q]], F[hsrc[q]], nb, cudaMemcpyDeviceToDevice, c.st));
  for (int q : {CAP_GRADP_X, CAP_GRADP_Y, CAP_GRADP_Z, CAP_P}) CAP_CUDA(cudaMemsetAsync(F[q], 0, nb, c.st));
  int rc, agg = 0, nrep = 0;
  Box bi{3, d.nimm, 3, d.njmm, 3, d.nkmm};
  int inpr = ixk(d, P.ipr, P.jpr, P.kpr);
  for (P.icorr = 1; P.icorr <= P.ncorr; ++P.icorr) {
    if ((rc = piso_gethbya())) return rc;
    for (P.ipcorr = 1; P.ipcorr <= P.npcor; ++P.ipcorr) {
      int ipc = P.ipcorr;
      if ((rc = piso_assemble(d.nj, 1, d.nij, CAP_AR1X, CAP_AR1Y, CAP_AR1Z, CAP_FX, CAP_AE, CAP_AW, CAP_F1, ipc, CAP_BE))) return rc;
      if ((rc = piso_assemble(1, d.nij, d.nj, CAP_AR2X, CAP_AR2Y, CAP_AR2Z, CAP_FY, CAP_AN, CAP_AS, CAP_F2, ipc, CAP_BN))) return rc;
      if ((rc = piso_assemble(d.nij, d.nj, 1, CAP_AR3X, CAP_AR3Y, CAP_AR3Z, CAP_FZ, CAP_AT, CAP_AB, CAP_F3, ipc, CAP_BT))) return rc;
      int first = P.ipcorr == 1;
      if (first && !P.const_mflux) { if ((rc = outbc())) return rc; }
      launch(k_div_ap, grid_for(bi.count()), kThreads, c.st, d, bi, first, 1, F[CAP_SU], F[CAP_AP], F[CAP_F1], F[CAP_F2],
                                                           F[CAP_F3], F[CAP_AE], F[CAP_AW], F[CAP_AN], F[CAP_AS],
                                                           F[CAP_AT], F[CAP_AB]);
      launch(k_pin, 1, 1, c.st, inpr, F[CAP_AP], F[CAP_AE], F[CAP_AW], F[CAP_AN], F[CAP_AS], F[CAP_AT], F[CAP_AB],
                               F[CAP_SU], F[CAP_P]);
      CAP_CHECK_LAUNCH();
      // sor(ip) = 0.1 (default real) before the last corrector, :132; the
      // tight_correctors option solves every corrector to reltol
      if (P.icorr != P.ncorr && !c.tight_correctors) P.sor[CAP_IP - 1] = (double)0.1f;
      else P.sor[CAP_IP - 1] = reltol;
      cappgpu_solve_report prep{};
      CAP_CUDA(cudaEventRecord(c.ev[2], c.st));
      rc = solve(P.piso_solver, CAP_P, CAP_IP, &prep);
      if (reps) reps[nrep] = prep;
      ++nrep;
      if (rc < 0) return rc;
      agg |= rc;
      CAP_CUDA(cudaEventRecord(c.ev[3], c.st));
      CAP_CUDA(cudaEventSynchronize(c.ev[3]));
      {
        float f = 0.f;
        CAP_CUDA(cudaEventElapsedTime(&f, c.ev[2], c.ev[3]));
        c.p_solve_ms = f;
        c.p_rep = prep;
      }
      if ((rc = bpres(CAP_P))) return rc;
      if ((rc = grad_gauss(CAP_P, CAP_GRADP_X, CAP_GRADP_Y, CAP_GRADP_Z))) return rc;
      if (P.ipcorr == P.npcor) {
        Box bf{2, d.nimm, 2, d.njmm, 2, d.nkmm};
        launch(k_flux_corr, grid_for(bf.count()), kThreads, c.st, d, bf, F[CAP_F1], F[CAP_F2], F[CAP_F3], F[CAP_AE],
                                                                  F[CAP_AN], F[CAP_AT], F[CAP_P]);
        CAP_CHECK_LAUNCH();
      }
    }
    P.ipcorr = P.npcor + 1;
    if ((rc = continuity_errors())) return rc;
    launch(k_vel_corr, grid_for(bi.count()), kThreads, c.st, d, bi, 0, F[CAP_U], F[CAP_V], F[CAP_W], F[CAP_APU],
                                                            F[CAP_APV], F[CAP_APW], F[CAP_GRADP_X], F[CAP_GRADP_Y],
                                                            F[CAP_GRADP_Z], F[CAP_VOL], nullptr, nullptr, 0.0, nullptr);
    CAP_CHECK_LAUNCH();
  }
  CAP_CUDA(cudaMemcpyAsync(F[CAP_PP], F[CAP_P], nb, cudaMemcpyDeviceToDevice, c.st));
  return agg;
}

// ------------------------------------------------------------------ SIMPLE
struct FmArgs {
  const double *arvx, *arvy, *arvz, *fif;
  double *acfe, *acfw, *fcf;
  const double *x, *y, *z, *xc, *yc, *zc, *u, *v, *w, *p, *den, *vol, *apu, *apv, *apw;
  const double *gux, *guy, *guz, *gvx, *gvy, *gvz, *gwx, *gwy, *gwz, *gpx, *gpy, *gpz;
  int idew, idns, idtb;
};

// fluxmass2.f90:41-192
__global__ void k_fluxmass(Dims d, Box b, FmArgs A) {
  BOX_LOOP(b) {
    int i, j, k;
    b.at(t_, i, j, k);
    int inp = ixk(d, i, j, k);
    int ine = inp + A.idew, ins = inp - A.idns, inb = inp - A.idtb, inbs = inb - A.idns;
    double fxe = A.fif[inp], fxp = 1.0 - fxe;
    double xf = 0.25 * (A.x[inp] + A.x[ins] + A.x[inb] + A.x[inbs]);
    double yf = 0.25 * (A.y[inp] + A.y[ins] + A.y[inb] + A.y[inbs]);
    double zf = 0.25 * (A.z[inp] + A.z[ins] + A.z[inb] + A.z[inbs]);
    double xi = A.xc[inp] * fxp + A.xc[ine] * fxe;
    double yi = A.yc[inp] * fxp + A.yc[ine] * fxe;
    double zi = A.zc[inp] * fxp + A.zc[ine] * fxe;
    double xpn = A.xc[ine] - A.xc[inp], ypn = A.yc[ine] - A.yc[inp], zpn = A.zc[ine] - A.zc[inp];
    double arx = A.arvx[inp], ary = A.arvy[inp], arz = A.arvz[inp];
    double are = sqrt(arx * arx + ary * ary + arz * arz);
    double nxx = arx / are, nyy = ary / are, nzz = arz / are;
    double sfdpnr = 1.0 / (arx * xpn * nxx + ary * ypn * nyy + arz * zpn * nzz);
    double dene = A.den[inp] * fxp + A.den[ine] * fxe;
    double smdpn = (arx * arx + ary * ary + arz * arz) * sfdpnr;
    double a = dene * (fxp * A.vol[inp] * A.apu[inp] + fxe * A.vol[ine] * A.apu[ine]) * smdpn;
    A.acfe[inp] = a;
    A.acfw[ine] = a;
    double duxi = A.gux[inp] * fxp + A.gux[ine] * fxe;
    double duyi = A.guy[inp] * fxp + A.guy[ine] * fxe;
    double duzi = A.guz[inp] * fxp + A.guz[ine] * fxe;
    double ui = A.u[inp] * fxp + A.u[ine] * fxe + (duxi * (xf - xi) + duyi * (yf - yi) + duzi * (zf - zi));
    duxi = A.gvx[inp] * fxp + A.gvx[ine] * fxe;
    duyi = A.gvy[inp] * fxp + A.gvy[ine] * fxe;
    duzi = A.gvz[inp] * fxp + A.gvz[ine] * fxe;
    double vi = A.v[inp] * fxp + A.v[ine] * fxe + (duxi * (xf - xi) + duyi * (yf - yi) + duzi * (zf - zi));
    duxi = A.gwx[inp] * fxp + A.gwx[ine] * fxe;
    duyi = A.gwy[inp] * fxp + A.gwy[ine] * fxe;
    duzi = A.gwz[inp] * fxp + A.gwz[ine] * fxe;
    double wi = A.w[inp] * fxp + A.w[ine] * fxe + (duxi * (xf - xi) + duyi * (yf - yi) + duzi * (zf - zi));
    double cu = fxe * A.vol[ine] * A.apu[ine] + fxp * A.vol[inp] * A.apu[inp];
    double cv = fxe * A.vol[ine] * A.apv[ine] + fxp * A.vol[inp] * A.apv[inp];
    double cw = fxe * A.vol[ine] * A.apw[ine] + fxp * A.vol[inp] * A.apw[inp];
    double dpxi = cu * (fxe * A.gpx[ine] + fxp * A.gpx[inp]) * xpn * nxx;
    double dpyi = cv * (fxe * A.gpy[ine] + fxp * A.gpy[inp]) * ypn * nyy;
    double dpzi = cw * (fxe * A.gpz[ine] + fxp * A.gpz[inp]) * zpn * nzz;
    double xpp = xf - (xf - A.xc[inp]) * nxx, ypp = yf - (yf - A.yc[inp]) * nyy, zpp = zf - (zf - A.zc[inp]) * nzz;
    double xep = xf - (xf - A.xc[ine]) * nxx, yep = yf - (yf - A.yc[ine]) * nyy, zep = zf - (zf - A.zc[ine]) * nzz;
    xpp = xpp - A.xc[inp]; ypp = ypp - A.yc[inp]; zpp = zpp - A.zc[inp];
    xep = xep - A.xc[ine]; yep = yep - A.yc[ine]; zep = zep - A.zc[ine];
    // operator precedence of fluxmass2.f90:171-173 kept
    double dpe = (A.p[ine] - A.p[inp]) + (A.gpx[ine] * xep + A.gpy[ine] * yep + A.gpz[ine] * zep - A.gpx[inp] * xpp +
                                          A.gpy[inp] * ypp + A.gpz[inp] * zpp);
    double dpex = cu * (arx * sfdpnr) * dpe;
    double dpey = cv * (ary * sfdpnr) * dpe;
    double dpez = cw * (arz * sfdpnr) * dpe;
    double ue = ui - dpex + dpxi, ve = vi - dpey + dpyi, we = wi - dpez + dpzi;
    A.fcf[inp] = dene * (ue * arx + ve * ary + we * arz);
  }
}

int fluxmass(int idew, int idns, int idtb, int arvx, int arvy, int arvz, int fif, int acfe, int acfw, int fcf) {
  Ctx& c = ctx();
  const Dims& d = c.d;
  double** F = c.f;
  FmArgs A{F[arvx], F[arvy], F[arvz], F[fif], F[acfe], F[acfw], F[fcf],
           F[CAP_X], F[CAP_Y], F[CAP_Z], F[CAP_XC], F[CAP_YC], F[CAP_ZC], F[CAP_U], F[CAP_V], F[CAP_W], F[CAP_P],
           F[CAP_DEN], F[CAP_VOL], F[CAP_APU], F[CAP_APV], F[CAP_APW],
           F[CAP_GRADU_X], F[CAP_GRADU_Y], F[CAP_GRADU_Z], F[CAP_GRADV_X], F[CAP_GRADV_Y], F[CAP_GRADV_Z],
           F[CAP_GRADW_X], F[CAP_GRADW_Y], F[CAP_GRADW_Z], F[CAP_GRADP_X], F[CAP_GRADP_Y], F[CAP_GRADP_Z],
           idew, idns, idtb};
  Box b{2, d.nimm, 2, d.njmm, 2, d.nkm};
  launch(k_fluxmass, grid_for(b.count()), kThreads, c.st, d, b, A);
  CAP_CHECK_LAUNCH();
  return CAPPGPU_OK;
}

// fluxmc.f90:43-106 for one face (dir 0 east, 1 north, 2 top)
__device__ inline double fluxmc_face(const Dims& d, int inp, int dir, const double* const* F) {
  int idew = dir == 0 ? d.nj : dir == 1 ? 1 : d.nij;
  int idns = dir == 0 ? 1 : dir == 1 ? d.nij : d.nj;
  int idtb = dir == 0 ? d.nij : dir == 1 ? d.nj : 1;
  const double* fif = F[CAP_FX + dir];
  int ine = inp + idew, ins = inp - idns, inb = inp - idtb, inbs = inb - idns;
  double fxe = fif[inp], fxp = 1.0 - fxe;
  double arx = F[CAP_AR1X + 3 * dir][inp], ary = F[CAP_AR1Y + 3 * dir][inp], arz = F[CAP_AR1Z + 3 * dir][inp];
  const double *xc = F[CAP_XC], *yc = F[CAP_YC], *zc = F[CAP_ZC];
  double xpn = xc[ine] - xc[inp], ypn = yc[ine] - yc[inp], zpn = zc[ine] - zc[inp];
  double are = sqrt(arx * arx + ary * ary + arz * arz);
  double nxx = arx / are, nyy = ary / are, nzz = arz / are;
  double dppnnr = 1.0 / ((xpn * nxx) + (ypn * nyy) + (zpn * nzz));
  const double *x = F[CAP_X], *y = F[CAP_Y], *z = F[CAP_Z];
  double xf = 0.25 * (x[inp] + x[ins] + x[inb] + x[inbs]);
  double yf = 0.25 * (y[inp] + y[ins] + y[inb] + y[inbs]);
  double zf = 0.25 * (z[inp] + z[ins] + z[inb] + z[inbs]);
  double xpp = xf - (xf - xc[inp]) * nxx, ypp = yf - (yf - yc[inp]) * nyy, zpp = zf - (zf - zc[inp]) * nzz;
  double xep = xf - (xf - xc[ine]) * nxx, yep = yf - (yf - yc[ine]) * nyy, zep = zf - (zf - zc[ine]) * nzz;
  xpp = xpp - xc[inp]; ypp = ypp - yc[inp]; zpp = zpp - zc[inp];
  xep = xep - xc[ine]; yep = yep - yc[ine]; zep = zep - zc[ine];
  const double *apu = F[CAP_APU], *den = F[CAP_DEN], *vol = F[CAP_VOL];
  const double *gpx = F[CAP_GRADP_X], *gpy = F[CAP_GRADP_Y], *gpz = F[CAP_GRADP_Z];
  double rapr = (apu[inp] * den[inp] * vol[inp] * fxp + apu[ine] * den[ine] * vol[ine] * fxe);
  return rapr * are * ((gpx[ine] * xep - gpx[inp] * xpp) + (gpy[ine] * yep - gpy[inp] * ypp) + (gpz[ine] * zep - gpz[inp] * zpp)) *
         dppnnr;
}

struct FieldTable { const double* p[CAP_NFIELDS]; };

// fmcor per interior face into three scratch arrays
__global__ void k_fluxmc_faces(Dims d, Box b, FieldTable T, double* m1, double* m2, double* m3) {
  BOX_LOOP(b) {
    int i, j, k;
    b.at(t_, i, j, k);
    int inp = ixk(d, i, j, k);
    m1[inp] = fluxmc_face(d, inp, 0, T.p);
    m2[inp] = fluxmc_face(d, inp, 1, T.p);
    m3[inp] = fluxmc_face(d, inp, 2, T.p);
  }
}

// calcp...f90:122-160 in gather form: su was zeroed; for cell P the
// reference's loop order gives -m3(B), -m1(W), -m2(S), then (for interior
// P) f -= m and +m1(P), +m2(P), +m3(P).
__global__ void k_fluxmc_apply(Dims d, Box ib, double* su, double* f1, double* f2, double* f3,
                               const double* __restrict__ m1, const double* __restrict__ m2,
                               const double* __restrict__ m3) {
  Box b{3, d.nim, 3, d.njm, 3, d.nkm};
  BOX_LOOP(b) {
    int i, j, k;
    b.at(t_, i, j, k);
    int p = ixk(d, i, j, k);
    auto in = [&](int ii, int jj, int kk) {
      return ii >= ib.i0 && ii <= ib.i1 && jj >= ib.j0 && jj <= ib.j1 && kk >= ib.k0 && kk <= ib.k1;
    };
    double s = 0.0;
    if (in(i, j, k - 1)) s = s - m3[p - d.nij];
    if (in(i - 1, j, k)) s = s - m1[p - d.nj];
    if (in(i, j - 1, k)) s = s - m2[p - 1];
    if (in(i, j, k)) {
      f1[p] = f1[p] - m1[p];
      s = s + m1[p];
      f2[p] = f2[p] - m2[p];
      s = s + m2[p];
      f3[p] = f3[p] - m3[p];
      s = s + m3[p];
    }
    su[p] = s;
  }
}

__global__ void k_read(const double* a, int idx, double* out) { *out = a[idx]; }

// calcp-multiple_correction_SIMPLE.f90:3-238
int calcp(cappgpu_solve_report* reps) {
  Ctx& c = ctx();
  const Dims& d = c.d;
  double** F = c.f;
  cappgpu_params& P = c.prm;
  size_t nb = sizeof(double) * d.nijk;
  Box bi{3, d.nimm, 3, d.njmm, 3, d.nkmm};
  int rc, agg = 0, nrep = 0;
  for (P.icorr = 1; P.icorr <= P.ncorr; ++P.icorr) {
    if ((rc = grad_gauss(CAP_U, CAP_GRADU_X, CAP_GRADU_Y, CAP_GRADU_Z))) return rc;
    if ((rc = grad_gauss(CAP_V, CAP_GRADV_X, CAP_GRADV_Y, CAP_GRADV_Z))) return rc;
    if ((rc = grad_gauss(CAP_W, CAP_GRADW_X, CAP_GRADW_Y, CAP_GRADW_Z))) return rc;
    if ((rc = fluxmass(d.nj, 1, d.nij, CAP_AR1X, CAP_AR1Y, CAP_AR1Z, CAP_FX, CAP_AE, CAP_AW, CAP_F1))) return rc;
    if ((rc = fluxmass(1, d.nij, d.nj, CAP_AR2X, CAP_AR2Y, CAP_AR2Z, CAP_FY, CAP_AN, CAP_AS, CAP_F2))) return rc;
    if ((rc = fluxmass(d.nij, d.nj, 1, CAP_AR3X, CAP_AR3Y, CAP_AR3Z, CAP_FZ, CAP_AT, CAP_AB, CAP_F3))) return rc;
    if (!P.const_mflux) { if ((rc = outbc())) return rc; }
    launch(k_div_ap, grid_for(bi.count()), kThreads, c.st, d, bi, 1, 1, F[CAP_SU], F[CAP_AP], F[CAP_F1], F[CAP_F2],
                                                         F[CAP_F3], F[CAP_AE], F[CAP_AW], F[CAP_AN], F[CAP_AS],
                                                         F[CAP_AT], F[CAP_AB]);
    CAP_CHECK_LAUNCH();
    for (P.ipcorr = 1; P.ipcorr <= P.npcor; ++P.ipcorr) {
      CAP_CUDA(cudaMemsetAsync(F[CAP_PP], 0, nb, c.st));
      cappgpu_solve_report prep{};
      CAP_CUDA(cudaEventRecord(c.ev[2], c.st));
      rc = solve(P.isol_p, CAP_PP, CAP_IP, &prep);
      if (reps) reps[nrep] = prep;
      ++nrep;
      if (rc < 0) return rc;
      agg |= rc;
      CAP_CUDA(cudaEventRecord(c.ev[3], c.st));
      CAP_CUDA(cudaEventSynchronize(c.ev[3]));
      {
        float f = 0.f;
        CAP_CUDA(cudaEventElapsedTime(&f, c.ev[2], c.ev[3]));
        c.p_solve_ms = f;
        c.p_rep = prep;
      }
      double* ppref = c.dscal;   // device scalar pp(ijkpr)
      launch(k_read, 1, 1, c.st, F[CAP_PP], ixk(d, P.ipr, P.jpr, P.kpr), ppref);
      if ((rc = grad_gauss(CAP_PP, CAP_GRADP_X, CAP_GRADP_Y, CAP_GRADP_Z))) return rc;
      if (P.ipcorr != P.npcor) {
        CAP_CUDA(cudaMemsetAsync(F[CAP_SU], 0, nb, c.st));
        FieldTable T;
        for (int q = 0; q < CAP_NFIELDS; ++q) T.p[q] = F[q];
        launch(k_fluxmc_faces, grid_for(bi.count()), kThreads, c.st, d, bi, T, c.work[5], c.work[6], c.work[7]);
        Box bx{3, d.nim, 3, d.njm, 3, d.nkm};
        launch(k_fluxmc_apply, grid_for(bx.count()), kThreads, c.st, d, bi, F[CAP_SU], F[CAP_F1], F[CAP_F2], F[CAP_F3],
                                                                     c.work[5], c.work[6], c.work[7]);
        CAP_CHECK_LAUNCH();
      }
      launch(k_flux_corr, grid_for(bi.count()), kThreads, c.st, d, bi, F[CAP_F1], F[CAP_F2], F[CAP_F3], F[CAP_AE],
                                                               F[CAP_AN], F[CAP_AT], F[CAP_PP]);
      launch(k_vel_corr, grid_for(bi.count()), kThreads, c.st, d, bi, 1, F[CAP_U], F[CAP_V], F[CAP_W], F[CAP_APU],
                                                              F[CAP_APV], F[CAP_APW], F[CAP_GRADP_X], F[CAP_GRADP_Y],
                                                              F[CAP_GRADP_Z], F[CAP_VOL], F[CAP_P], F[CAP_PP],
                                                              P.urf[CAP_IP - 1], ppref);
      CAP_CHECK_LAUNCH();
    }
    P.ipcorr = P.npcor + 1;
    if ((rc = continuity_errors())) return rc;
    if ((rc = correct_bc())) return rc;
  }
  if ((rc = bpres(CAP_P))) return rc;
  CAP_CUDA(cudaMemcpyAsync(F[CAP_PP], F[CAP_P], nb, cudaMemcpyDeviceToDevice, c.st));
  return agg;
}

// ------------------------------------------------------------------ outbc
// outbc.f90:3-318.  With an outlet (lout), the mass flux through every
// outlet face (code 2) of the face sets flagged low..lot is formed --
// den(ghost) times u(interior) dotted with ar1x,ar1y,ar1z of the ghost for
// all six sets, as the reference writes it -- and summed in the routine's
// loop order; then each outlet ghost takes the interior velocity times
// fac = flowin/(flow+small), its flux is scaled by fac, and te, ed, vis, t
// are copied from the interior (vart, con, utt, vtt, wtt have no field
// here).  The face lists are built on the host in the reference's loop
// order, the fluxes are formed on the device and the flow is summed on the
// host in that order, so fac carries the reference's rounding.  Each face
// set is its own launch, in order: the corner ghosts that two sets share
// take the later set's values, and a later set may read an earlier set's
// ghost as its interior neighbour, as in the reference's sequence.  Face
// sets: 0 W, 1 E, 2 S, 3 N, 4 B, 5 T.
namespace {
struct OutbcBuf {
  int3* ent = nullptr;     // per face: ghost inp, interior inh, index of its flux
  double* val = nullptr;   // per face: its flux
  size_t cap = 0;
};
OutbcBuf g_ob;

__global__ void k_outbc_flux(int n, const int3* __restrict__ e, const double* __restrict__ den,
                             const double* __restrict__ a1x, const double* __restrict__ a1y,
                             const double* __restrict__ a1z, const double* __restrict__ u,
                             const double* __restrict__ v, const double* __restrict__ w, double* __restrict__ f,
                             double* __restrict__ val) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int3 q = e[t];
    const double fl = den[q.x] * (a1x[q.x] * u[q.y] + a1y[q.x] * v[q.y] + a1z[q.x] * w[q.y]);
    f[q.z] = fl;
    val[t] = fl;
  }
}

__global__ void k_outbc_scale(int n, const int3* __restrict__ e, double fac, double* u, double* v, double* w,
                              double* f, double* te, double* ed, double* vis, double* tt) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int3 q = e[t];
    u[q.x] = u[q.y] * fac;
    v[q.x] = v[q.y] * fac;
    w[q.x] = w[q.y] * fac;
    f[q.z] = f[q.z] * fac;
    te[q.x] = te[q.y];
    ed[q.x] = ed[q.y];
    vis[q.x] = vis[q.y];
    tt[q.x] = tt[q.y];
  }
}
}  // namespace

void outbc_free() {
  if (g_ob.ent) cudaFree(g_ob.ent);
  if (g_ob.val) cudaFree(g_ob.val);
  g_ob = OutbcBuf();
}

int outbc() {
  Ctx& c = ctx();
  const cappgpu_params& P = c.prm;
  if (!P.lout) return CAPPGPU_OK;   // outbc.f90:31
  const Dims& d = c.d;
  double** F = c.f;
  const int on[6] = {P.low, P.loe, P.los, P.lon, P.lob, P.lot};
  const int bcf[6] = {CAP_LBW, CAP_LBE, CAP_LBS, CAP_LBN, CAP_LBB, CAP_LBT};
  const int ff[6] = {CAP_F1, CAP_F1, CAP_F2, CAP_F2, CAP_F3, CAP_F3};
  std::vector<int3> ent;
  size_t start[7];
  for (int set = 0; set < 6; ++set) {
    start[set] = ent.size();
    if (!on[set]) continue;
    const int len = set < 2 ? d.njk : set < 4 ? d.nik : d.nij;
    std::vector<int> code((size_t)len);
    CAP_CUDA(cudaMemcpyAsync(code.data(), c.bc[bcf[set]], sizeof(int) * len, cudaMemcpyDeviceToHost, c.st));
    CAP_CUDA(cudaStreamSynchronize(c.st));
    // outer x inner loops: k,j (W/E); k,i (S/N); i,j (B/T)
    const int o_hi = set < 4 ? d.nkm : d.nim;
    const int i_hi = (set == 2 || set == 3) ? d.nim : d.njm;
    for (int o = 2; o <= o_hi; ++o)
      for (int q = 2; q <= i_hi; ++q) {
        int inp, inbc, inh, at;
        switch (set) {
          case 0: inp = ixk(d, 2, q, o); inbc = (q - 1) * d.nk + o; inh = inp + d.nj; at = inp; break;
          case 1: inp = ixk(d, d.nim, q, o); inbc = (q - 1) * d.nk + o; inh = inp - d.nj; at = inh; break;
          case 2: inp = ixk(d, q, 2, o); inbc = (q - 1) * d.nk + o; inh = inp + 1; at = inp; break;
          case 3: inp = ixk(d, q, d.njm, o); inbc = (q - 1) * d.nk + o; inh = inp - 1; at = inh; break;
          case 4: inp = ixk(d, o, q, 2); inbc = (o - 1) * d.nj + q; inh = inp + d.nij; at = inp; break;
          default: inp = ixk(d, o, q, d.nkm); inbc = (o - 1) * d.nj + q; inh = inp - d.nij; at = inh; break;
        }
        if (code[(size_t)inbc - 1] == 2) ent.push_back(make_int3(inp, inh, at));
      }
  }
  start[6] = ent.size();
  const size_t n = ent.size();
  if (n > g_ob.cap) {
    outbc_free();
    if (cudaMalloc(&g_ob.ent, sizeof(int3) * n) != cudaSuccess || cudaMalloc(&g_ob.val, sizeof(double) * n) != cudaSuccess) {
      outbc_free();
      set_error("outbc: out of device memory");
      return CAPPGPU_E_NOMEM;
    }
    g_ob.cap = n;
  }
  double flow = 0.0;
  std::vector<double> val(n);
  if (n) {
    CAP_CUDA(cudaMemcpyAsync(g_ob.ent, ent.data(), sizeof(int3) * n, cudaMemcpyHostToDevice, c.st));
    for (int set = 0; set < 6; ++set) {
      const int m = (int)(start[set + 1] - start[set]);
      if (m)
        launch(k_outbc_flux, grid_for(m), kThreads, c.st, m, (const int3*)g_ob.ent + start[set],
               (const double*)F[CAP_DEN], (const double*)F[CAP_AR1X], (const double*)F[CAP_AR1Y],
               (const double*)F[CAP_AR1Z], (const double*)F[CAP_U], (const double*)F[CAP_V], (const double*)F[CAP_W],
               F[ff[set]], g_ob.val + start[set]);
    }
    CAP_CHECK_LAUNCH();
    CAP_CUDA(cudaMemcpyAsync(val.data(), g_ob.val, sizeof(double) * n, cudaMemcpyDeviceToHost, c.st));
    CAP_CUDA(cudaStreamSynchronize(c.st));
    for (int set = 0; set < 6; ++set)   // flow in the routine's order: minus W/S/B, plus E/N/T
      for (size_t e = start[set]; e < start[set + 1]; ++e) flow = (set & 1) ? flow + val[e] : flow - val[e];
  }
  const double fac = P.flowin / (flow + CAP_SMALL);   // outbc.f90:147
  for (int set = 0; set < 6; ++set) {
    const int m = (int)(start[set + 1] - start[set]);
    if (m)
      launch(k_outbc_scale, grid_for(m), kThreads, c.st, m, (const int3*)g_ob.ent + start[set], fac, F[CAP_U],
             F[CAP_V], F[CAP_W], F[ff[set]], F[CAP_TE], F[CAP_ED], F[CAP_VIS], F[CAP_T]);
  }
  CAP_CHECK_LAUNCH();
  return CAPPGPU_OK;
}

}  // namespace cap

using namespace cap;

extern "C" {

static int check_fields(std::initializer_list<int> ids) {
  for (int f : ids)
    if (f < 0 || f >= CAP_NFIELDS) { set_error("bad field id %d", f); return CAPPGPU_E_ARG; }
  return CAPPGPU_OK;
}

static int sync_rc(int rc) {
  cudaError_t e = cudaStreamSynchronize(ctx().st);
  if (e != cudaSuccess) return cuda_fail(e, "stream sync", __FILE__, __LINE__);
  return rc;
}

int cappgpu_fluxuvw(int idew, int idns, int idtb, int arvx, int arvy, int arvz, int fif, int acfe, int acfw, int fcf) {
  CAP_REQUIRE_INIT();
  int rc = check_fields({arvx, arvy, arvz, fif, acfe, acfw, fcf});
  if (rc) return rc;
  return sync_rc(fluxuvw(idew, idns, idtb, arvx, arvy, arvz, fif, acfe, acfw, fcf));
}

int cappgpu_calcuvw(cappgpu_solve_report* rep) {
  CAP_REQUIRE_INIT();
  return sync_rc(calcuvw(rep));
}

int cappgpu_piso_assemble_pressure_eq(int idew, int idns, int idtb, int arvx, int arvy, int arvz, int fif, int acfe,
                                      int acfw, int fcf, int ipc, int bp) {
  CAP_REQUIRE_INIT();
  int rc = check_fields({arvx, arvy, arvz, fif, acfe, acfw, fcf, bp});
  if (rc) return rc;
  return sync_rc(piso_assemble(idew, idns, idtb, arvx, arvy, arvz, fif, acfe, acfw, fcf, ipc, bp));
}

int cappgpu_assemble_pressure_eq(int idew, int idns, int idtb, int arvx, int arvy, int arvz, int fif, int acfe,
                                 int acfw, int fcf) {
  CAP_REQUIRE_INIT();
  int rc = check_fields({arvx, arvy, arvz, fif, acfe, acfw, fcf});
  if (rc) return rc;
  return sync_rc(assemble_pressure_eq(idew, idns, idtb, arvx, arvy, arvz, fif, acfe, acfw, fcf));
}

int cappgpu_piso_gethbya(void) {
  CAP_REQUIRE_INIT();
  return sync_rc(piso_gethbya());
}

int cappgpu_piso_multiple_correction(cappgpu_solve_report* rep) {
  CAP_REQUIRE_INIT();
  return sync_rc(piso_multiple_correction(rep));
}

int cappgpu_fluxmass(int idew, int idns, int idtb, int arvx, int arvy, int arvz, int fif, int acfe, int acfw, int fcf) {
  CAP_REQUIRE_INIT();
  int rc = check_fields({arvx, arvy, arvz, fif, acfe, acfw, fcf});
  if (rc) return rc;
  return sync_rc(fluxmass(idew, idns, idtb, arvx, arvy, arvz, fif, acfe, acfw, fcf));
}

int cappgpu_calcp(cappgpu_solve_report* rep) {
  CAP_REQUIRE_INIT();
  return sync_rc(calcp(rep));
}

int cappgpu_outbc(void) {
  CAP_REQUIRE_INIT();
  return sync_rc(outbc());
}

int cappgpu_courant(void) {
  CAP_REQUIRE_INIT();
  return sync_rc(courant());
}

int cappgpu_continuity_errors(void) {
  CAP_REQUIRE_INIT();
  return sync_rc(continuity_errors());
}

}  // extern "C"
