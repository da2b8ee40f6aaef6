// stencil.cu -- ghost-cell fills, Green-Gauss gradient, pressure ghost
// extrapolation and the 7-point product of the reference, as device kernels
// with the reference's write sets and per-cell operation order.
#include "common.cuh"
#include "kernels.cuh"

namespace cap {

// ---------------------------------------------------------------- ghost cells
// update_values_at_ghostcells_nonperiodic.f90:47-640.  The six boundary
// loops write disjoint ghost cells and read only interior cells (plus the
// ghost's own old vis), so one launch covers all faces.
struct GhostArgs {
  double *u, *v, *w, *te, *ed, *t, *vis;
  const double *fx, *fy, *fz;
  const double *a1x, *a1y, *a1z, *a2x, *a2y, *a2z, *a3x, *a3y, *a3z;
  const int *lbw, *lbe, *lbs, *lbn, *lbb, *lbt;
  double uin, vin, win, tein, edin, tin;
};

__global__ void k_ghost_nonperiodic(Dims d, GhostArgs g) {
  const int nA[6] = {d.nkmm - 2, d.nkmm - 2, d.nkmm - 2, d.nkmm - 2, d.nimm - 2, d.nimm - 2};
  const int nB[6] = {d.njmm - 2, d.njmm - 2, d.nimm - 2, d.nimm - 2, d.njmm - 2, d.njmm - 2};
  long long off[7];
  off[0] = 0;
  for (int f = 0; f < 6; ++f) off[f + 1] = off[f] + (long long)nA[f] * nB[f];
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < off[6];
       t += (long long)gridDim.x * blockDim.x) {
    int face = 0;
    while (t >= off[face + 1]) ++face;
    long long r = t - off[face];
    int b = 3 + (int)(r % nB[face]);
    int a = 3 + (int)(r / nB[face]);
    int inp, ingc, iface, lb, step;
    double fxp;
    const double *arx, *ary, *arz, *fif;
    switch (face) {
      case 0: inp = ixk(d, 3, b, a); step = d.nj; ingc = inp - d.nj; iface = inp - d.nj;
              lb = g.lbw[(b - 1) * d.nk + a - 1]; fxp = g.fx[inp - d.nj];
              arx = g.a1x; ary = g.a1y; arz = g.a1z; fif = g.fx; break;
      case 1: inp = ixk(d, d.nimm, b, a); step = d.nj; ingc = inp + d.nj; iface = inp;
              lb = g.lbe[(b - 1) * d.nk + a - 1]; fxp = 1.0 - g.fx[inp];
              arx = g.a1x; ary = g.a1y; arz = g.a1z; fif = g.fx; break;
      case 2: inp = ixk(d, b, 3, a); step = 1; ingc = inp - 1; iface = inp - 1;
              lb = g.lbs[(b - 1) * d.nk + a - 1]; fxp = 1.0 - g.fy[inp];
              arx = g.a2x; ary = g.a2y; arz = g.a2z; fif = g.fy; break;
      case 3: inp = ixk(d, b, d.njmm, a); step = 1; ingc = inp + 1; iface = inp;
              lb = g.lbn[(b - 1) * d.nk + a - 1]; fxp = 1.0 - g.fy[inp];
              arx = g.a2x; ary = g.a2y; arz = g.a2z; fif = g.fy; break;
      case 4: inp = ixk(d, a, b, 3); step = d.nij; ingc = inp - d.nij; iface = inp - d.nij;
              lb = g.lbb[(a - 1) * d.nj + b - 1]; fxp = g.fz[ingc];
              arx = g.a3x; ary = g.a3y; arz = g.a3z; fif = g.fz; break;
      default: inp = ixk(d, a, b, d.nkmm); step = d.nij; ingc = inp + d.nij; iface = inp;
              lb = g.lbt[(a - 1) * d.nj + b - 1]; fxp = 1.0 - g.fz[inp];
              arx = g.a3x; ary = g.a3y; arz = g.a3z; fif = g.fz; break;
    }
    double fxe = 1.0 - fxp;
    double fxer = 1.0 / fxe;
    bool low = (face == 0 || face == 2 || face == 4);
    if (lb == 1) {  // inlet
      g.u[ingc] = (g.uin - g.u[inp] * fxp) * fxer;
      g.v[ingc] = (g.vin - g.v[inp] * fxp) * fxer;
      g.w[ingc] = (g.win - g.w[inp] * fxp) * fxer;
      g.te[ingc] = (g.tein - g.te[inp] * fxp) * fxer;
      g.ed[ingc] = (g.edin - g.ed[inp] * fxp) * fxer;
      g.t[ingc] = (g.tin - g.t[inp] * fxp) * fxer;
      double tg = g.te[ingc];
      g.vis[ingc] = 0.09 * (tg * tg) / g.ed[ingc];
    }
    if (lb == 2) {  // outlet: linear extrapolation from two inside cells
      double* fl[7] = {g.u, g.v, g.w, g.te, g.ed, g.t, g.vis};
      if (low) {
        double f = fif[inp];
#pragma unroll
        for (int q = 0; q < 7; ++q) fl[q][ingc] = fl[q][inp] - (fl[q][inp + step] - fl[q][inp]) * f;
      } else {
        double f = 1.0 - fif[inp - step];
#pragma unroll
        for (int q = 0; q < 7; ++q) fl[q][ingc] = fl[q][inp] + (fl[q][inp] - fl[q][inp - step]) * f;
      }
    }
    if (lb == 3) {  // symmetry (area vector, not unit normal, as the reference)
      double unmag = g.u[inp] * arx[iface] + g.v[inp] * ary[iface] + g.w[inp] * arz[iface];
      g.u[ingc] = g.u[inp] - unmag * arx[iface];
      g.v[ingc] = g.v[inp] - unmag * ary[iface];
      g.w[ingc] = g.w[inp] - unmag * arz[iface];
      g.te[ingc] = g.te[inp];
      g.ed[ingc] = g.ed[inp];
      g.t[ingc] = g.t[inp];
      g.vis[ingc] = g.vis[inp];
    }
    if (lb == 4) {  // wall
      g.u[ingc] = (-g.u[inp] * fxp) * fxer;
      g.v[ingc] = (-g.v[inp] * fxp) * fxer;
      g.w[ingc] = (-g.w[inp] * fxp) * fxer;
      g.te[ingc] = (-g.te[inp] * fxp) * fxer;
      g.ed[ingc] = g.ed[inp];
      g.t[ingc] = (g.tin - g.t[inp] * fxp) * fxer;
      if (face >= 4) g.vis[ingc] = g.vis[inp];
      else g.vis[ingc] = (g.vis[ingc] - g.vis[inp] * fxp) * fxer;
    }
  }
}

// update_values_at_ghostcells.f90:40-145 (periodic i and j, walls in k)
__global__ void k_ghost_periodic(Dims d, double* u, double* v, double* w, double* te, double* ed,
                                 double* vis, const double* __restrict__ fz) {
  long long nWE = (long long)(d.nkmm - 2) * (d.njmm - 2);
  long long nSN = (long long)(d.nkmm - 2) * (d.nimm - 2);
  long long nBT = (long long)(d.nimm - 2) * (d.njmm - 2);
  long long tot = nWE + nSN + 2 * nBT;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < tot; t += (long long)gridDim.x * blockDim.x) {
    double* fl[6] = {u, v, w, te, ed, vis};
    if (t < nWE) {
      int j = 3 + (int)(t % (d.njmm - 2)), k = 3 + (int)(t / (d.njmm - 2));
      int ingcw = ixk(d, 2, j, k), inp = ixk(d, 3, j, k), ine = ixk(d, d.nimm, j, k), ingce = ixk(d, d.nim, j, k);
#pragma unroll
      for (int q = 0; q < 6; ++q) { fl[q][ingcw] = fl[q][ine]; fl[q][ingce] = fl[q][inp]; }
    } else if (t < nWE + nSN) {
      long long r = t - nWE;
      int i = 3 + (int)(r % (d.nimm - 2)), k = 3 + (int)(r / (d.nimm - 2));
      int ingcw = ixk(d, i, 2, k), inp = ixk(d, i, 3, k), ine = ixk(d, i, d.njmm, k), ingce = ixk(d, i, d.njm, k);
#pragma unroll
      for (int q = 0; q < 6; ++q) { fl[q][ingcw] = fl[q][ine]; fl[q][ingce] = fl[q][inp]; }
    } else {
      long long r = t - nWE - nSN;
      bool top = r >= nBT;
      if (top) r -= nBT;
      int j = 3 + (int)(r % (d.njmm - 2)), i = 3 + (int)(r / (d.njmm - 2));
      int ingc, inp;
      double fxp, fxe;
      if (!top) {
        ingc = ixk(d, i, j, 2); inp = ixk(d, i, j, 3);
        fxp = fz[inp - d.nij]; fxe = 1.0 - fxp;
      } else {
        ingc = ixk(d, i, j, d.nkm); inp = ixk(d, i, j, d.nkmm);
        fxe = fz[inp]; fxp = 1.0 - fxe;
      }
      u[ingc] = -u[inp] * fxp / fxe;
      v[ingc] = -v[inp] * fxp / fxe;
      w[ingc] = -w[inp] * fxp / fxe;
      te[ingc] = -te[inp] * fxp / fxe;
      ed[ingc] = ed[inp];
      vis[ingc] = (vis[ingc] - vis[inp] * fxp) / fxe;
    }
  }
}

int ghost_update() {
  Ctx& c = ctx();
  const Dims& d = c.d;
  double** F = c.f;
  if (c.prm.periodic) {
    long long tot = (long long)(d.nkmm - 2) * (d.njmm - 2) + (long long)(d.nkmm - 2) * (d.nimm - 2) +
                    2LL * (d.nimm - 2) * (d.njmm - 2);
    launch(k_ghost_periodic, grid_for(tot), kThreads, c.st, d, F[CAP_U], F[CAP_V], F[CAP_W], F[CAP_TE], F[CAP_ED],
                                                           F[CAP_VIS], F[CAP_FZ]);
  } else {
    GhostArgs g{F[CAP_U], F[CAP_V], F[CAP_W], F[CAP_TE], F[CAP_ED], F[CAP_T], F[CAP_VIS],
                F[CAP_FX], F[CAP_FY], F[CAP_FZ],
                F[CAP_AR1X], F[CAP_AR1Y], F[CAP_AR1Z], F[CAP_AR2X], F[CAP_AR2Y], F[CAP_AR2Z],
                F[CAP_AR3X], F[CAP_AR3Y], F[CAP_AR3Z],
                c.bc[CAP_LBW], c.bc[CAP_LBE], c.bc[CAP_LBS], c.bc[CAP_LBN], c.bc[CAP_LBB], c.bc[CAP_LBT],
                c.prm.uin, c.prm.vin, c.prm.win, c.prm.tein, c.prm.edin, c.prm.tin};
    long long tot = 4LL * (d.nkmm - 2) * ((d.njmm - 2) + (d.nimm - 2)) / 2 + 2LL * (d.nimm - 2) * (d.njmm - 2);
    launch(k_ghost_nonperiodic, grid_for(tot), kThreads, c.st, d, g);
  }
  CAP_CHECK_LAUNCH();
  return CAPPGPU_OK;
}

// ------------------------------------------------------------------- gradient
// GRAD_GAUSS.f90:1-105 in gather form.  The reference scatters each face
// value into both neighbours in loop order (k,i,j) over faces
// k=2..nkm, i=2..nimm, j=2..njmm, then divides interior cells by vol.  For a
// cell P the scatter order is: bottom face (from k-1), west face (from i-1),
// south face (from j-1), own east/north/top faces.  The gather below adds
// the same rounded terms in the same order, so every element -- ghost and
// padding cells included -- is bit-identical.
template <typename R, bool VR>
__global__ void k_grad_gauss(Dims d, const double* __restrict__ u, const double* __restrict__ fx,
                             const double* __restrict__ fy, const double* __restrict__ fz,
                             const double* __restrict__ a1x, const double* __restrict__ a1y,
                             const double* __restrict__ a1z, const double* __restrict__ a2x,
                             const double* __restrict__ a2y, const double* __restrict__ a2z,
                             const double* __restrict__ a3x, const double* __restrict__ a3y,
                             const double* __restrict__ a3z, const double* __restrict__ vol,
                             const double* __restrict__ volr_c, double* __restrict__ dx, double* __restrict__ dy,
                             double* __restrict__ dz) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < d.nijk; t += (long long)gridDim.x * blockDim.x) {
    int p = (int)t;
    int k = p / d.nij + 1;
    int r = p - (k - 1) * d.nij;
    int i = r / d.nj + 1;
    int j = r - (i - 1) * d.nj + 1;
    // face box F = {k 2..nkm, i 2..nimm, j 2..njmm}
    auto inF = [&](int ii, int jj, int kk) {
      return kk >= 2 && kk <= d.nkm && ii >= 2 && ii <= d.nimm && jj >= 2 && jj <= d.njmm;
    };
    R gx = R(0.0), gy = R(0.0), gz = R(0.0);
    if (inF(i, j, k - 1)) {  // bottom face: this cell is 'int' of inp = p - nij
      int q = p - d.nij;
      R ut = R(u[p]) * R(fz[q]) + R(u[q]) * (R(1.0) - R(fz[q]));
      gx = gx - (ut * R(a3x[q]));
      gy = gy - (ut * R(a3y[q]));
      gz = gz - (ut * R(a3z[q]));
    }
    if (inF(i - 1, j, k)) {  // west face: this cell is 'ine' of inp = p - nj
      int q = p - d.nj;
      R ue = R(u[p]) * R(fx[q]) + R(u[q]) * (R(1.0) - R(fx[q]));
      gx = gx - (ue * R(a1x[q]));
      gy = gy - (ue * R(a1y[q]));
      gz = gz - (ue * R(a1z[q]));
    }
    if (inF(i, j - 1, k)) {  // south face: this cell is 'inn' of inp = p - 1
      int q = p - 1;
      R un = R(u[p]) * R(fy[q]) + R(u[q]) * (R(1.0) - R(fy[q]));
      gx = gx - (un * R(a2x[q]));
      gy = gy - (un * R(a2y[q]));
      gz = gz - (un * R(a2z[q]));
    }
    if (inF(i, j, k)) {  // own east, north, top faces
      R ue = R(u[p + d.nj]) * R(fx[p]) + R(u[p]) * (R(1.0) - R(fx[p]));
      R un = R(u[p + 1]) * R(fy[p]) + R(u[p]) * (R(1.0) - R(fy[p]));
      R ut = R(u[p + d.nij]) * R(fz[p]) + R(u[p]) * (R(1.0) - R(fz[p]));
      gx = gx + (ue * R(a1x[p]) + un * R(a2x[p]) + ut * R(a3x[p]));
      gy = gy + (ue * R(a1y[p]) + un * R(a2y[p]) + ut * R(a3y[p]));
      gz = gz + (ue * R(a1z[p]) + un * R(a2z[p]) + ut * R(a3z[p]));
    }
    if (k >= 2 && k <= d.nkm && i >= 3 && i <= d.nimm && j >= 3 && j <= d.njmm) {
      R volr;
      if constexpr (VR) volr = R(volr_c[p]);   // the same 1/vol, evaluated once per grid
      else volr = R(1.0) / R(vol[p]);
      gx = gx * volr;
      gy = gy * volr;
      gz = gz * volr;
    }
    dx[p] = gx;
    dy[p] = gy;
    dz[p] = gz;
  }
}

// The same gradient in FP32 arithmetic from FP32 copies of the geometry
// (fx, fy, fz, ar1x..ar3z and 1/vol, each rounded once per grid) and of the
// field (rounded once per call): the FP32 terms of k_grad_gauss<float> in
// the same order, so the same bits, without its ≈30 FP64 -> FP32
// conversions per cell (GB300 runs them on the FP64 pipe, 64 cycles per
// warp instruction) and with half the bytes read.  G holds the 13 geometry
// planes of n floats each in the order fx, fy, fz, a1x, a1y, a1z, a2x, a2y,
// a2z, a3x, a3y, a3z, 1/vol.
__global__ void k_grad_gauss32(Dims d, const float* __restrict__ u, const float* __restrict__ G, long long n,
                               double* __restrict__ dx, double* __restrict__ dy, double* __restrict__ dz) {
  const float *fx = G, *fy = G + n, *fz = G + 2 * n;
  const float *a1x = G + 3 * n, *a1y = G + 4 * n, *a1z = G + 5 * n;
  const float *a2x = G + 6 * n, *a2y = G + 7 * n, *a2z = G + 8 * n;
  const float *a3x = G + 9 * n, *a3y = G + 10 * n, *a3z = G + 11 * n, *volr = G + 12 * n;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < d.nijk; t += (long long)gridDim.x * blockDim.x) {
    int p = (int)t;
    int k = p / d.nij + 1;
    int r = p - (k - 1) * d.nij;
    int i = r / d.nj + 1;
    int j = r - (i - 1) * d.nj + 1;
    auto inF = [&](int ii, int jj, int kk) {
      return kk >= 2 && kk <= d.nkm && ii >= 2 && ii <= d.nimm && jj >= 2 && jj <= d.njmm;
    };
    float gx = 0.0f, gy = 0.0f, gz = 0.0f;
    if (inF(i, j, k - 1)) {  // bottom face
      int q = p - d.nij;
      float ut = u[p] * fz[q] + u[q] * (1.0f - fz[q]);
      gx = gx - (ut * a3x[q]);
      gy = gy - (ut * a3y[q]);
      gz = gz - (ut * a3z[q]);
    }
    if (inF(i - 1, j, k)) {  // west face
      int q = p - d.nj;
      float ue = u[p] * fx[q] + u[q] * (1.0f - fx[q]);
      gx = gx - (ue * a1x[q]);
      gy = gy - (ue * a1y[q]);
      gz = gz - (ue * a1z[q]);
    }
    if (inF(i, j - 1, k)) {  // south face
      int q = p - 1;
      float un = u[p] * fy[q] + u[q] * (1.0f - fy[q]);
      gx = gx - (un * a2x[q]);
      gy = gy - (un * a2y[q]);
      gz = gz - (un * a2z[q]);
    }
    if (inF(i, j, k)) {  // own east, north, top faces
      float ue = u[p + d.nj] * fx[p] + u[p] * (1.0f - fx[p]);
      float un = u[p + 1] * fy[p] + u[p] * (1.0f - fy[p]);
      float ut = u[p + d.nij] * fz[p] + u[p] * (1.0f - fz[p]);
      gx = gx + (ue * a1x[p] + un * a2x[p] + ut * a3x[p]);
      gy = gy + (ue * a1y[p] + un * a2y[p] + ut * a3y[p]);
      gz = gz + (ue * a1z[p] + un * a2z[p] + ut * a3z[p]);
    }
    if (k >= 2 && k <= d.nkm && i >= 3 && i <= d.nimm && j >= 3 && j <= d.njmm) {
      const float vr = volr[p];
      gx = gx * vr;
      gy = gy * vr;
      gz = gz * vr;
    }
    dx[p] = gx;
    dy[p] = gy;
    dz[p] = gz;
  }
}

// 1/vol of every cell for the FP64 gradient (an FP64 division per cell and
// call otherwise), and the FP32 geometry of k_grad_gauss32, rebuilt after a
// write into a geometry field or vol
namespace {
double* g_volr = nullptr;
unsigned long long g_volr_gen = 0;
int g_volr_n = 0;
float* g_geo32 = nullptr;   // 13 geometry planes, then the field's FP32 copy
unsigned long long g_geo32_gen = 0;
int g_geo32_n = 0;

__global__ void k_recip(long long n, const double* __restrict__ v, double* __restrict__ r) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
    r[t] = 1.0 / v[t];
}

struct Geo13 {
  const double* g[12];   // fx, fy, fz, a1x .. a3z
  const double* vol;
};

__global__ void k_geo32(long long n, Geo13 src, float* __restrict__ G) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
#pragma unroll
    for (int q = 0; q < 12; ++q) G[q * n + t] = (float)src.g[q][t];
    G[12 * n + t] = 1.0f / (float)src.vol[t];
  }
}

__global__ void k_to_f32(long long n, const double* __restrict__ x, float* __restrict__ y) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
    y[t] = (float)x[t];
}
}  // namespace

void volr_free() {
  if (g_volr) cudaFree(g_volr);
  g_volr = nullptr;
  g_volr_gen = 0;
  g_volr_n = 0;
  if (g_geo32) cudaFree(g_geo32);
  g_geo32 = nullptr;
  g_geo32_gen = 0;
  g_geo32_n = 0;
}

// the FP32 geometry planes followed by room for the field (14 x nijk
// floats), or null (no room, or option face_geo 0: convert per call)
static float* geo32_cache() {
  Ctx& c = ctx();
  if (!c.face_geo) return nullptr;
  const long long n = c.d.nijk;
  if (g_geo32_n != c.d.nijk) {
    if (g_geo32) cudaFree(g_geo32);
    g_geo32 = nullptr;
    g_geo32_n = 0;
    if (cudaMalloc(&g_geo32, sizeof(float) * 14 * (size_t)n) != cudaSuccess) {
      cudaGetLastError();
      g_geo32 = nullptr;
      return nullptr;
    }
    g_geo32_n = c.d.nijk;
    g_geo32_gen = 0;
  }
  if (g_geo32_gen != c.geo_gen) {
    double** F = c.f;
    Geo13 src{{F[CAP_FX], F[CAP_FY], F[CAP_FZ], F[CAP_AR1X], F[CAP_AR1Y], F[CAP_AR1Z], F[CAP_AR2X], F[CAP_AR2Y],
               F[CAP_AR2Z], F[CAP_AR3X], F[CAP_AR3Y], F[CAP_AR3Z]},
              F[CAP_VOL]};
    launch(k_geo32, grid_for(n), kThreads, c.st, n, src, g_geo32);
    g_geo32_gen = c.geo_gen;
  }
  return g_geo32;
}

static const double* volr_cache() {
  Ctx& c = ctx();
  if (!c.face_geo) return nullptr;
  if (g_volr_n != c.d.nijk) {
    volr_free();
    if (cudaMalloc(&g_volr, sizeof(double) * c.d.nijk) != cudaSuccess) {
      cudaGetLastError();
      g_volr = nullptr;
      return nullptr;   // no room: divide per call
    }
    g_volr_n = c.d.nijk;
  }
  if (g_volr_gen != c.geo_gen) {
    launch(k_recip, grid_for(c.d.nijk), kThreads, c.st, (long long)c.d.nijk, (const double*)c.f[CAP_VOL], g_volr);
    g_volr_gen = c.geo_gen;
  }
  return g_volr;
}

int grad_gauss(int uf, int dxf, int dyf, int dzf) {
  Ctx& c = ctx();
  double** F = c.f;
  // precision modes 1-2: velocity gradients (inputs of the coefficient
  // assembly) in FP32 arithmetic; the pressure gradient of the velocity
  // correction stays FP64
  const bool f32 = c.fp32(8) && uf != CAP_P;
  if (f32) {
    float* G = geo32_cache();
    if (G) {
      const long long n = c.d.nijk;
      float* u32 = G + 13 * n;
      launch(k_to_f32, grid_for(n), kThreads, c.st, n, (const double*)F[uf], u32);
      launch(k_grad_gauss32, grid_for(n), kThreads, c.st, c.d, (const float*)u32, (const float*)G, n, F[dxf], F[dyf],
             F[dzf]);
      CAP_CHECK_LAUNCH();
      return CAPPGPU_OK;
    }
  }
  const double* vr = f32 ? nullptr : volr_cache();
  auto k = f32 ? k_grad_gauss<float, false> : vr ? k_grad_gauss<double, true> : k_grad_gauss<double, false>;
  launch(k, grid_for(c.d.nijk), kThreads, c.st,
      c.d, F[uf], F[CAP_FX], F[CAP_FY], F[CAP_FZ], F[CAP_AR1X], F[CAP_AR1Y], F[CAP_AR1Z], F[CAP_AR2X],
      F[CAP_AR2Y], F[CAP_AR2Z], F[CAP_AR3X], F[CAP_AR3Y], F[CAP_AR3Z], F[CAP_VOL], vr, F[dxf], F[dyf], F[dzf]);
  CAP_CHECK_LAUNCH();
  return CAPPGPU_OK;
}

// ---------------------------------------------------------------------- bpres
// bpres.f90:3-81: the six planes write disjoint ghost cells from interior
// values, one launch.
__global__ void k_bpres(Dims d, double* p, const double* __restrict__ fx, const double* __restrict__ fy,
                        const double* __restrict__ fz) {
  long long nij_ = (long long)(d.nimm - 2) * (d.njmm - 2);
  long long njk_ = (long long)(d.njmm - 2) * (d.nkmm - 2);
  long long nik_ = (long long)(d.nimm - 2) * (d.nkmm - 2);
  long long tot = 2 * (nij_ + njk_ + nik_);
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < tot; t += (long long)gridDim.x * blockDim.x) {
    long long r = t;
    if (r < 2 * nij_) {
      bool top = r >= nij_;
      if (top) r -= nij_;
      int j = 3 + (int)(r % (d.njmm - 2)), i = 3 + (int)(r / (d.njmm - 2));
      if (!top) { int ijk = ixk(d, i, j, 3); p[ijk - d.nij] = p[ijk] - (p[ijk + d.nij] - p[ijk]) * fz[ijk]; }
      else { int ijk = ixk(d, i, j, d.nkmm); p[ijk + d.nij] = p[ijk] + (p[ijk] - p[ijk - d.nij]) * (1.0 - fz[ijk - d.nij]); }
      continue;
    }
    r -= 2 * nij_;
    if (r < 2 * njk_) {
      bool east = r >= njk_;
      if (east) r -= njk_;
      int k = 3 + (int)(r % (d.nkmm - 2)), j = 3 + (int)(r / (d.nkmm - 2));
      if (!east) { int ijk = ixk(d, 3, j, k); p[ijk - d.nj] = p[ijk] - (p[ijk + d.nj] - p[ijk]) * fx[ijk]; }
      else { int ijk = ixk(d, d.nimm, j, k); p[ijk + d.nj] = p[ijk] + (p[ijk] - p[ijk - d.nj]) * (1.0 - fx[ijk - d.nj]); }
      continue;
    }
    r -= 2 * njk_;
    bool north = r >= nik_;
    if (north) r -= nik_;
    int k = 3 + (int)(r % (d.nkmm - 2)), i = 3 + (int)(r / (d.nkmm - 2));
    if (!north) { int ijk = ixk(d, i, 3, k); p[ijk - 1] = p[ijk] - (p[ijk + 1] - p[ijk]) * fy[ijk]; }
    else { int ijk = ixk(d, i, d.njmm, k); p[ijk + 1] = p[ijk] + (p[ijk] - p[ijk - 1]) * (1.0 - fy[ijk - 1]); }
  }
}

int bpres(int pf) {
  Ctx& c = ctx();
  const Dims& d = c.d;
  long long tot = 2LL * ((long long)(d.nimm - 2) * (d.njmm - 2) + (long long)(d.njmm - 2) * (d.nkmm - 2) +
                         (long long)(d.nimm - 2) * (d.nkmm - 2));
  launch(k_bpres, grid_for(tot), kThreads, c.st, d, c.f[pf], c.f[CAP_FX], c.f[CAP_FY], c.f[CAP_FZ]);
  CAP_CHECK_LAUNCH();
  return CAPPGPU_OK;
}

// correctBoundaryConditions.f90:1-86 -- four padding-layer copies; the
// first two and the last two touch disjoint cells but the second reads
// layer li(njm) that the first does not write, so one launch per loop pair.
__global__ void k_correct_bc(Dims d, double* u, double* v, double* w, double* f1, double* f2, int pass) {
  long long n = pass == 0 ? (long long)(d.nkm - 1) * (d.njm - 1) : (long long)(d.nkm - 1) * (d.nim - 1);
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    if (pass == 0) {
      int j = 2 + (int)(t % (d.njm - 1)), k = 2 + (int)(t / (d.njm - 1));
      int inp = ixk(d, d.ni, j, k), inh = ixk(d, 2, j, k);
      u[inp] = u[inh]; v[inp] = v[inh]; w[inp] = w[inh];
      inp = ixk(d, 1, j, k);
      inh = (k - 1) * d.nij + (d.njm - 1) * d.nj + (j - 1);  // li(njm), correctBoundaryConditions.f90:44
      u[inp] = u[inh]; v[inp] = v[inh]; w[inp] = w[inh];
      f1[inp] = f1[inh];
    } else {
      int i = 2 + (int)(t % (d.nim - 1)), k = 2 + (int)(t / (d.nim - 1));
      int inp = ixk(d, i, d.nj, k), inh = ixk(d, i, 2, k);
      u[inp] = u[inh]; v[inp] = v[inh]; w[inp] = w[inh];
      inp = ixk(d, i, 1, k);
      inh = ixk(d, i, d.njm, k);
      u[inp] = u[inh]; v[inp] = v[inh]; w[inp] = w[inh];
      f2[inp] = f2[inh];
    }
  }
}

int correct_bc() {
  Ctx& c = ctx();
  const Dims& d = c.d;
  // loop 1 writes i=ni from i=2, loop 2 writes i=1 from li(njm): the source
  // cells of loop 2 are never written by loop 1 unless njm == ni; keep the
  // reference order with two launches per direction when they could alias.
  // the second loop reads row li(njm) (correctBoundaryConditions.f90:44):
  // a valid i row only when nj-1 <= ni, and a cell that the first loop
  // (which writes row ni) must not have written: nj-1 != ni
  if (d.njm >= d.ni) {
    set_error("correctBoundaryConditions reads row li(nj-1), which needs nj-1 < ni (ni=%d, nj=%d)", d.ni, d.nj);
    return CAPPGPU_E_ARG;
  }
  launch(k_correct_bc, grid_for((long long)(d.nkm - 1) * (d.njm - 1)), kThreads, c.st, d, c.f[CAP_U], c.f[CAP_V], c.f[CAP_W], c.f[CAP_F1], c.f[CAP_F2], 0);
  launch(k_correct_bc, grid_for((long long)(d.nkm - 1) * (d.nim - 1)), kThreads, c.st, d, c.f[CAP_U], c.f[CAP_V], c.f[CAP_W], c.f[CAP_F1], c.f[CAP_F2], 1);
  CAP_CHECK_LAUNCH();
  return CAPPGPU_OK;
}

}  // namespace cap

using namespace cap;

extern "C" {

int cappgpu_update_values_at_ghostcells(void) {
  CAP_REQUIRE_INIT();
  int rc = ghost_update();
  if (rc) return rc;
  CAP_CUDA(cudaStreamSynchronize(ctx().st));
  return CAPPGPU_OK;
}

int cappgpu_grad_gauss(int u, int dudx, int dudy, int dudz) {
  CAP_REQUIRE_INIT();
  for (int f : {u, dudx, dudy, dudz})
    if (f < 0 || f >= CAP_NFIELDS) { set_error("grad_gauss: bad field %d", f); return CAPPGPU_E_ARG; }
  if (u == dudx || u == dudy || u == dudz) { set_error("grad_gauss: input aliases an output"); return CAPPGPU_E_ARG; }
  int rc = grad_gauss(u, dudx, dudy, dudz);
  if (rc) return rc;
  CAP_CUDA(cudaStreamSynchronize(ctx().st));
  return CAPPGPU_OK;
}

int cappgpu_bpres(int p) {
  CAP_REQUIRE_INIT();
  if (p < 0 || p >= CAP_NFIELDS) { set_error("bpres: bad field %d", p); return CAPPGPU_E_ARG; }
  int rc = bpres(p);
  if (rc) return rc;
  CAP_CUDA(cudaStreamSynchronize(ctx().st));
  return CAPPGPU_OK;
}

int cappgpu_correct_boundary_conditions(void) {
  CAP_REQUIRE_INIT();
  int rc = correct_bc();
  if (rc) return rc;
  CAP_CUDA(cudaStreamSynchronize(ctx().st));
  return CAPPGPU_OK;
}

}  // extern "C"

extern "C" {

// Host-pointer drop-in for grad_gauss(u,dudx,dudy,dudz): u and the three
// outputs are host arrays of nijk doubles (for example the gfortran
// temporaries of gradu(1,:) sections, calcuvw.f90:43-45).  The inputs are
// staged through solver work vectors; the geometry comes from the context.
int cappgpu_grad_gauss_h(const double* u, double* dudx, double* dudy, double* dudz) {
  CAP_REQUIRE_INIT();
  if (!u || !dudx || !dudy || !dudz) { cap::set_error("grad_gauss_h: null pointer"); return CAPPGPU_E_ARG; }
  cap::Ctx& c = cap::ctx();
  size_t nb = sizeof(double) * c.d.nijk;
  double** F = c.f;
  double *du = c.work[4], *gx = c.work[5], *gy = c.work[6], *gz = c.work[7];
  CAP_CUDA(cudaMemcpyAsync(du, u, nb, cudaMemcpyHostToDevice, c.st));
  const double* vr = cap::volr_cache();
  cap::launch(vr ? cap::k_grad_gauss<double, true> : cap::k_grad_gauss<double, false>, cap::grid_for(c.d.nijk),
      cap::kThreads, c.st, c.d, (const double*)du, F[CAP_FX], F[CAP_FY], F[CAP_FZ], F[CAP_AR1X], F[CAP_AR1Y],
      F[CAP_AR1Z], F[CAP_AR2X], F[CAP_AR2Y], F[CAP_AR2Z], F[CAP_AR3X], F[CAP_AR3Y], F[CAP_AR3Z], F[CAP_VOL], vr, gx,
      gy, gz);
  CAP_CHECK_LAUNCH();
  CAP_CUDA(cudaMemcpyAsync(dudx, gx, nb, cudaMemcpyDeviceToHost, c.st));
  CAP_CUDA(cudaMemcpyAsync(dudy, gy, nb, cudaMemcpyDeviceToHost, c.st));
  CAP_CUDA(cudaMemcpyAsync(dudz, gz, nb, cudaMemcpyDeviceToHost, c.st));
  CAP_CUDA(cudaStreamSynchronize(c.st));
  return CAPPGPU_OK;
}

}  // extern "C"
