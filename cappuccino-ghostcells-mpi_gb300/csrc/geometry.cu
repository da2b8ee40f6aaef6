// geometry.cu -- face area vectors and interpolation factors from the grid
// nodes, computed on the device exactly as init.f90:49-144 does on the
// host (face areas init.f90:54-136; interpolation factors intfac.f90:4-48
// through find_intersection_point.f90:1-76).
#include "common.cuh"

namespace cap {

// init.f90:58-73 for one face.  idns/idtb select the face's two in-plane
// directions.  sgn = +1 reproduces the reference's cross product verbatim;
// sgn = -1 flips it (see cappgpu_build_geometry).
__global__ void k_face_areas(Dims d, Box b, int idns, int idtb, double sgn, const double* __restrict__ x,
                             const double* __restrict__ y, const double* __restrict__ z, double* ax,
                             double* ay, double* az) {
  long long n = b.count();
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    b.at(t, i, j, k);
    int inp = ixk(d, i, j, k);
    int ins = inp - idns, inb = inp - idtb, inbs = inb - idns;
    double dxet = 0.5 * (x[inp] - x[ins] + x[inb] - x[inbs]);
    double dyet = 0.5 * (y[inp] - y[ins] + y[inb] - y[inbs]);
    double dzet = 0.5 * (z[inp] - z[ins] + z[inb] - z[inbs]);
    double dxzd = 0.5 * (x[inp] - x[inb] + x[ins] - x[inbs]);
    double dyzd = 0.5 * (y[inp] - y[inb] + y[ins] - y[inbs]);
    double dzzd = 0.5 * (z[inp] - z[inb] + z[ins] - z[inbs]);
    double a1 = dyet * dzzd - dyzd * dzet;
    double a2 = dxzd * dzet - dxet * dzzd;
    double a3 = dxet * dyzd - dyet * dxzd;
    ax[inp] = sgn < 0 ? -a1 : a1;
    ay[inp] = sgn < 0 ? -a2 : a2;
    az[inp] = sgn < 0 ? -a3 : a3;
  }
}

// find_intersection_point.f90:39-56: intersection of the plane through
// p1,p2,p3 with the line p4-p5.
__device__ inline void intersection(double x1, double y1, double z1, double x2, double y2, double z2,
                                    double x3, double y3, double z3, double x4, double y4, double z4,
                                    double x5, double y5, double z5, double& xj, double& yj, double& zj) {
  double t = -(x2 * (y3 * z4 - y4 * z3) - x1 * (y3 * z4 - y4 * z3) - x3 * (y2 * z4 - y4 * z2) +
               x1 * (y2 * z4 - y4 * z2) + x3 * (y1 * z4 - y4 * z1) - x2 * (y1 * z4 - y4 * z1) +
               x4 * (y2 * z3 - y3 * z2) - x1 * (y2 * z3 - y3 * z2) - x4 * (y1 * z3 - y3 * z1) +
               x2 * (y1 * z3 - y3 * z1) + x4 * (y1 * z2 - y2 * z1) - x3 * (y1 * z2 - y2 * z1)) /
             (x2 * (y3 * (z5 - z4) - (y5 - y4) * z3) - x1 * (y3 * (z5 - z4) - (y5 - y4) * z3) -
              x3 * (y2 * (z5 - z4) - (y5 - y4) * z2) + x1 * (y2 * (z5 - z4) - (y5 - y4) * z2) +
              x3 * (y1 * (z5 - z4) - (y5 - y4) * z1) - x2 * (y1 * (z5 - z4) - (y5 - y4) * z1) +
              (x5 - x4) * (y2 * z3 - y3 * z2) - (x5 - x4) * (y1 * z3 - y3 * z1) +
              (x5 - x4) * (y1 * z2 - y2 * z1));
  xj = x4 + (x5 - x4) * t;
  yj = y4 + (y5 - y4) * t;
  zj = z4 + (z5 - z4) * t;
}

// intfac.f90:25-48
__global__ void k_intfac(Dims d, int idew, int idns, int idtb, const double* __restrict__ x,
                         const double* __restrict__ y, const double* __restrict__ z,
                         const double* __restrict__ xc, const double* __restrict__ yc,
                         const double* __restrict__ zc, double* lambda) {
  Box b{2, d.nim, 2, d.njm, 2, d.nkm};
  long long n = b.count();
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    b.at(t, i, j, k);
    int inp = ixk(d, i, j, k), inn = inp + idew;
    double xf, yf, zf;
    intersection(x[inp], y[inp], z[inp], x[inp - idns], y[inp - idns], z[inp - idns], x[inp - idtb],
                 y[inp - idtb], z[inp - idtb], xc[inp], yc[inp], zc[inp], xc[inp + idew], yc[inp + idew],
                 zc[inp + idew], xf, yf, zf);
    double dx = xf - xc[inp], dy = yf - yc[inp], dz = zf - zc[inp];
    double ex = xc[inn] - xc[inp], ey = yc[inn] - yc[inp], ez = zc[inn] - zc[inp] + CAP_SMALL;
    lambda[inp] = sqrt(dx * dx + dy * dy + dz * dz) / (sqrt(ex * ex + ey * ey + ez * ez) + CAP_SMALL);
  }
}

__global__ void k_intersection_kat(const double* p, double* out) {
  intersection(p[0], p[1], p[2], p[3], p[4], p[5], p[6], p[7], p[8], p[9], p[10], p[11], p[12], p[13],
               p[14], out[0], out[1], out[2]);
}

}  // namespace cap

using namespace cap;

extern "C" {

// Face areas and interpolation factors from the nodes x,y,z and the cell
// centres xc,yc,zc already in the context.
//   orient = 0: init.f90:54-136 verbatim.  On a right-handed grid its cross
//               products point east faces towards +i but north and top
//               faces towards -j and -k.
//   orient = 1: north and top area vectors negated, so that all three point
//               towards increasing index -- the orientation GRAD_GAUSS.f90:57-81,
//               fluxuvw and the pressure assembly assume.
int cappgpu_build_geometry(int orient) {
  CAP_REQUIRE_INIT();
  Ctx& c = ctx();
  const Dims& d = c.d;
  double s23 = orient ? -1.0 : 1.0;
  Box be{1, d.nim, 2, d.njm, 2, d.nkm};
  Box bn{2, d.nim, 1, d.njm, 2, d.nkm};
  Box bt{2, d.nim, 2, d.njm, 1, d.nkm};
  ++c.geo_gen;
  launch(k_face_areas, grid_for(be.count()), kThreads, c.st, d, be, 1, d.nij, 1.0, c.f[CAP_X], c.f[CAP_Y],
                                                            c.f[CAP_Z], c.f[CAP_AR1X], c.f[CAP_AR1Y], c.f[CAP_AR1Z]);
  launch(k_face_areas, grid_for(bn.count()), kThreads, c.st, d, bn, d.nj, d.nij, s23, c.f[CAP_X], c.f[CAP_Y],
                                                            c.f[CAP_Z], c.f[CAP_AR2X], c.f[CAP_AR2Y], c.f[CAP_AR2Z]);
  launch(k_face_areas, grid_for(bt.count()), kThreads, c.st, d, bt, 1, d.nj, s23, c.f[CAP_X], c.f[CAP_Y],
                                                            c.f[CAP_Z], c.f[CAP_AR3X], c.f[CAP_AR3Y], c.f[CAP_AR3Z]);
  CAP_CHECK_LAUNCH();
  long long n = (long long)(d.nim - 1) * (d.njm - 1) * (d.nkm - 1);
  launch(k_intfac, grid_for(n), kThreads, c.st, d, d.nj, 1, d.nij, c.f[CAP_X], c.f[CAP_Y], c.f[CAP_Z],
                                               c.f[CAP_XC], c.f[CAP_YC], c.f[CAP_ZC], c.f[CAP_FX]);
  launch(k_intfac, grid_for(n), kThreads, c.st, d, 1, d.nj, d.nij, c.f[CAP_X], c.f[CAP_Y], c.f[CAP_Z],
                                               c.f[CAP_XC], c.f[CAP_YC], c.f[CAP_ZC], c.f[CAP_FY]);
  launch(k_intfac, grid_for(n), kThreads, c.st, d, d.nij, 1, d.nj, c.f[CAP_X], c.f[CAP_Y], c.f[CAP_Z],
                                               c.f[CAP_XC], c.f[CAP_YC], c.f[CAP_ZC], c.f[CAP_FZ]);
  CAP_CHECK_LAUNCH();
  CAP_CUDA(cudaStreamSynchronize(c.st));
  return CAPPGPU_OK;
}

// find_intersection_point on the device for one point set (known-answer
// test of test_intersection_point.f90:8-38).  p: 15 doubles, out: 3.
int cappgpu_find_intersection_point(const double* p, double* out) {
  if (!p || !out) return CAPPGPU_E_ARG;
  double* dv = nullptr;
  CAP_CUDA(cudaMalloc(&dv, sizeof(double) * 18));
  CAP_CUDA(cudaMemcpy(dv, p, sizeof(double) * 15, cudaMemcpyHostToDevice));
  launch(k_intersection_kat, 1, 1, (cudaStream_t)0, (const double*)dv, dv + 15);
  CAP_CHECK_LAUNCH();
  CAP_CUDA(cudaMemcpy(out, dv + 15, sizeof(double) * 3, cudaMemcpyDeviceToHost));
  CAP_CUDA(cudaFree(dv));
  return CAPPGPU_OK;
}

}  // extern "C"
