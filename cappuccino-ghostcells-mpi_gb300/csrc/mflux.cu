// mflux.cu -- constant mass-flux forcing of the periodic channel:
// const_massflux_correction.f90:1-22, included at main.f90:252 at the end of
// a transient step when const_mflux is set.  Volume-weighted averages of U
// and APU over k = 2..nkm, i = 3..nimm, j = 3..njmm
// (fieldManipulation.f90:10-44), the pressure-gradient increment restoring
// the bulk velocity magUbar = uin (init.f90:356), U += APU * increment over
// the whole array, gradpcmf += increment (read by calcuvw.f90:78).  The
// sums are the library's fixed-order block reductions, not the reference's
// serial order.
#include "common.cuh"
#include "kernels.cuh"

namespace cap {

namespace {

__global__ void k_vw_sums(Dims d, Box b, const double* __restrict__ vol, const double* __restrict__ u,
                          const double* __restrict__ apu, double* part) {
  double v[3] = {0.0, 0.0, 0.0};
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < b.count();
       t += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    b.at(t, i, j, k);
    const int inp = ixk(d, i, j, k);
    v[0] += vol[inp];
    v[1] += vol[inp] * u[inp];
    v[2] += vol[inp] * apu[inp];
  }
  block_reduce_store<3>(v, part);
}

__global__ void k_add_apu(long long n, double* __restrict__ u, const double* __restrict__ apu, double g) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x)
    u[q] = u[q] + 1.0 * apu[q] * g;
}

}  // namespace

int const_massflux_correction() {
  Ctx& c = ctx();
  const Dims& d = c.d;
  double** F = c.f;
  Box b{3, d.nimm, 3, d.njmm, 2, d.nkm};
  launch(k_vw_sums, kRedBlocks, kThreads, c.st, d, b, (const double*)F[CAP_VOL], (const double*)F[CAP_U],
         (const double*)F[CAP_APU], c.partials);
  CAP_CHECK_LAUNCH();
  int rc = finish_reduce(3);
  if (rc) return rc;
  double s[3];
  if ((rc = fetch_reduce(3, s))) return rc;
  const double mag_ubar_star = s[1] / s[0];
  const double rua = s[2] / s[0];
  const double dgrad = (c.prm.uin - mag_ubar_star) / rua;
  launch(k_add_apu, grid_for(d.nijk), kThreads, c.st, (long long)d.nijk, F[CAP_U], (const double*)F[CAP_APU],
         dgrad);
  CAP_CHECK_LAUNCH();
  c.prm.gradpcmf = c.prm.gradpcmf + dgrad;
  return CAPPGPU_OK;
}

}  // namespace cap

using namespace cap;

extern "C" int cappgpu_const_massflux_correction(void) {
  CAP_REQUIRE_INIT();
  int rc = const_massflux_correction();
  CAP_CUDA(cudaStreamSynchronize(ctx().st));
  return rc;
}
