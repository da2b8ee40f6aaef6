// les.cu -- the Smagorinsky sub-grid viscosity of the LES path:
// find_strain_rate (find_strain_rate.f90:20-79, gauss branch) and
// calc_vis_les (calc_vis_les.f90:38-249) as device kernels, called by the
// step drivers after the pressure-velocity coupling when lcal(ivis) and lles
// are set (main.f90:205).  Each element keeps the reference's operation
// order; exp, log and pow are CUDA's, so results agree with the oracle's
// libm to a few ulps rather than bit for bit.  With the FP32 coefficient
// assembly of precision modes 1-2 the strain rate and the Smagorinsky
// viscosity are evaluated in FP32 arithmetic (FP64 storage), like the
// coefficients they feed.
#include <math.h>

#include "common.cuh"
#include "kernels.cuh"

namespace cap {

namespace {

// |S| = sqrt(2 s_ij s_ij) over k = 2..nkm, i = 3..nimm, j = 3..njmm
// (find_strain_rate.f90:33-76; the vorticity invariant of :77 is not kept);
// R = float in precision modes 1-2 with the FP32 coefficient assembly
__device__ __forceinline__ double sqrt_l(double x) { return sqrt(x); }
__device__ __forceinline__ float sqrt_l(float x) { return sqrtf(x); }
__device__ __forceinline__ double pow_l(double x, double y) { return pow(x, y); }
__device__ __forceinline__ float pow_l(float x, float y) { return powf(x, y); }
__device__ __forceinline__ double exp_l(double x) { return exp(x); }
__device__ __forceinline__ float exp_l(float x) { return expf(x); }

template <typename R>
__global__ void k_strain(Dims d, Box b, const double* __restrict__ gux, const double* __restrict__ guy,
                         const double* __restrict__ guz, const double* __restrict__ gvx,
                         const double* __restrict__ gvy, const double* __restrict__ gvz,
                         const double* __restrict__ gwx, const double* __restrict__ gwy,
                         const double* __restrict__ gwz, double* __restrict__ strain) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < b.count();
       t += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    b.at(t, i, j, k);
    const int inp = ixk(d, i, j, k);
    const R s11 = R(gux[inp]);
    const R s12 = R(0.5) * (R(guy[inp]) + R(gvx[inp]));
    const R s13 = R(0.5) * (R(guz[inp]) + R(gwx[inp]));
    const R s22 = R(gvy[inp]);
    const R s23 = R(0.5) * (R(gvz[inp]) + R(gwy[inp]));
    const R s33 = R(gwz[inp]);
    strain[inp] = sqrt_l(R(2) * (s11 * s11 + s22 * s22 + s33 * s33 + R(2) * (s12 * s12 + s13 * s13 + s23 * s23)));
  }
}

// Smagorinsky viscosity, Van Driest damping and Schumann's length limit
// (calc_vis_les.f90:42-73): the coefficient is the 0.17 assigned last (:66),
// C_delta the default-real 0.158, the exponent the default-real 1./3.
template <typename R>
__global__ void k_vis_les(Dims d, Box b, const double* __restrict__ u, const double* __restrict__ v,
                          const double* __restrict__ w, const double* __restrict__ wd,
                          const double* __restrict__ vol, const double* __restrict__ strain,
                          const double* __restrict__ den, double* __restrict__ vis, double viscos_d, double cappa_d,
                          double urf_d) {
  const R c_delta = R(0.158f), c_les = R(0.17f), third = R(1.f / 3.f);
  const R viscos = R(viscos_d), cappa = R(cappa_d), urf = R(urf_d);
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < b.count();
       t += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    b.at(t, i, j, k);
    const int inp = ixk(d, i, j, k);
    const R visold = R(vis[inp]);
    const R wldist = R(wd[inp]);
    const R uu = R(u[inp]), vv = R(v[inp]), ww = R(w[inp]);
    const R uref = sqrt_l(uu * uu + vv * vv + ww * ww);
    const R utau = sqrt_l(viscos * uref / wldist);
    const R zplus = wldist * utau / viscos;
    const R lm = c_les * pow_l(R(vol[inp]), third);
    const R ls = cappa / c_delta * wldist;
    const R l = (lm < ls ? lm : ls) * (R(1) - exp_l(-zplus / R(26.0)));
    const R vis_smag = l * l * R(strain[inp]) * R(den[inp]);
    const R vnew = vis_smag + viscos;
    vis[inp] = urf * vnew + (R(1) - urf) * visold;
  }
}

// wall-function viscosity of the bottom (top = 0) or top ghost layer
// (calc_vis_les.f90:80-246): dnw dotted with the integer extents nx,ny,nz
// and the top wall at lk(nimm), as in calcuvw (ktop: nimm, or nkmm with
// params.top_plane)
__global__ void k_vis_les_wall(Dims d, int top, int ktop, const double* __restrict__ xc, const double* __restrict__ yc,
                               const double* __restrict__ zc, const double* __restrict__ fz,
                               const double* __restrict__ a3x, const double* __restrict__ a3y,
                               const double* __restrict__ a3z, const double* __restrict__ u,
                               const double* __restrict__ v, const double* __restrict__ w,
                               double* __restrict__ vis, double viscos, double densit, double cappa, double elog,
                               double zero) {
  const int ni_ = d.nimm - 2, nj_ = d.njmm - 2;
  const double nxi = (double)d.ni, nyi = (double)d.nj, nzi = (double)d.nk;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < ni_ * nj_; t += gridDim.x * blockDim.x) {
    const int i = 3 + t / nj_, j = 3 + t % nj_;
    int inbc, ingc, iface;
    double fxp, fxe;
    if (!top) {
      inbc = ixk(d, i, j, 3);
      ingc = inbc - d.nij;
      iface = ingc;
      fxp = fz[ingc];
      fxe = 1.0 - fxp;
    } else {
      inbc = ixk(d, i, j, ktop);
      ingc = inbc + d.nij;
      iface = inbc;
      fxp = 1.0 - fz[inbc];
      fxe = 1.0 - fxp;
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
    const double utau = sqrt(tau / densit);
    const double ypl = densit * utau * dnw / viscos;
    double viscw = zero;
    if (ypl > (double)11.61f) viscw = ypl * viscos * cappa / log(elog * ypl);
    vis[ingc] = viscos > viscw ? viscos : viscw;
  }
}

}  // namespace

int find_strain_rate() {
  Ctx& c = ctx();
  const Dims& d = c.d;
  double** F = c.f;
  int rc;
  if ((rc = grad_gauss(CAP_U, CAP_GRADU_X, CAP_GRADU_Y, CAP_GRADU_Z))) return rc;
  if ((rc = grad_gauss(CAP_V, CAP_GRADV_X, CAP_GRADV_Y, CAP_GRADV_Z))) return rc;
  if ((rc = grad_gauss(CAP_W, CAP_GRADW_X, CAP_GRADW_Y, CAP_GRADW_Z))) return rc;
  Box b{3, d.nimm, 3, d.njmm, 2, d.nkm};
  // precision modes 1-2 with the FP32 coefficient assembly: FP32 arithmetic
  launch(c.fp32(4) ? k_strain<float> : k_strain<double>, grid_for(b.count()), kThreads, c.st, d, b,
         (const double*)F[CAP_GRADU_X],
         (const double*)F[CAP_GRADU_Y], (const double*)F[CAP_GRADU_Z], (const double*)F[CAP_GRADV_X],
         (const double*)F[CAP_GRADV_Y], (const double*)F[CAP_GRADV_Z], (const double*)F[CAP_GRADW_X],
         (const double*)F[CAP_GRADW_Y], (const double*)F[CAP_GRADW_Z], F[CAP_STRAIN]);
  CAP_CHECK_LAUNCH();
  return CAPPGPU_OK;
}

int calc_vis_les() {
  Ctx& c = ctx();
  const Dims& d = c.d;
  double** F = c.f;
  const cappgpu_params& P = c.prm;
  Box b{3, d.nimm, 3, d.njmm, 2, d.nkm};
  launch(c.fp32(4) ? k_vis_les<float> : k_vis_les<double>, grid_for(b.count()), kThreads, c.st, d, b,
         (const double*)F[CAP_U], (const double*)F[CAP_V],
         (const double*)F[CAP_W], (const double*)F[CAP_WALLDIST], (const double*)F[CAP_VOL],
         (const double*)F[CAP_STRAIN], (const double*)F[CAP_DEN], F[CAP_VIS], P.viscos, P.cappa,
         P.urf[CAP_IVIS - 1]);
  for (int top = 0; top < 2; ++top)
    launch(k_vis_les_wall, grid_for((long long)(d.nimm - 2) * (d.njmm - 2)), kThreads, c.st, d, top,
           c.prm.top_plane ? d.nkmm : d.nimm,
           (const double*)F[CAP_XC], (const double*)F[CAP_YC], (const double*)F[CAP_ZC], (const double*)F[CAP_FZ],
           (const double*)F[CAP_AR3X], (const double*)F[CAP_AR3Y], (const double*)F[CAP_AR3Z],
           (const double*)F[CAP_U], (const double*)F[CAP_V], (const double*)F[CAP_W], F[CAP_VIS], P.viscos,
           P.densit, P.cappa, P.elog, P.zero);
  CAP_CHECK_LAUNCH();
  return CAPPGPU_OK;
}

}  // namespace cap

using namespace cap;

extern "C" {

int cappgpu_find_strain_rate(void) {
  CAP_REQUIRE_INIT();
  int rc = find_strain_rate();
  CAP_CUDA(cudaStreamSynchronize(ctx().st));
  return rc;
}

int cappgpu_calc_vis_les(void) {
  CAP_REQUIRE_INIT();
  const Dims& d = ctx().d;
  if (!ctx().prm.top_plane && d.nimm + 1 > d.nk) {   // the top wall at lk(nimm), calc_vis_les.f90:174
    set_error("top wall index lk(nimm) of calc_vis_les.f90:174 leaves the array (ni=%d > nk=%d)", d.ni, d.nk);
    return CAPPGPU_E_ARG;
  }
  int rc = calc_vis_les();
  CAP_CUDA(cudaStreamSynchronize(ctx().st));
  return rc;
}

}  // extern "C"
