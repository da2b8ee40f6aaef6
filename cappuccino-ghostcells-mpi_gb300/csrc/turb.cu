// turb.cu -- Menter's k-omega SST on the device: calcscm (calcscm.f90:3-602)
// for te (k) and ed (omega), calculate_stuff_for_sst
// (calculate_stuff_for_sst.f90:27-70), fluxscm
// (fluxscm-overrelaxed-correction.f90:40-230) and modvis
// (modvis.f90:195-236), run by the step drivers after the pressure-velocity
// coupling when lcal(ite), lcal(ied) and sst are set (main.f90:196-203).
//
// Each element keeps the reference's operation order and literal kinds
// (the default-real model constants of init.f90:229-245 are single
// precision there); tanh is CUDA's, so the blending functions agree with
// the oracle's libm to a few ulps rather than bit for bit.  MAX/MIN over
// several arguments take the larger/smaller in argument order, a NaN
// argument losing to a number.  The linear solves are sipsol through the
// solver selector, so precision modes 1-2 run them in the FP32 refinement
// form.
#include <math.h>

#include "common.cuh"
#include "kernels.cuh"

namespace cap {

namespace {

constexpr double kSigmk1 = 1.0 / 1.176, kSigmk2 = 1.0, kSigmom1 = 1.0 / 2.0, kSigmom2 = 1.0 / 1.168;
constexpr double kBetai1 = (double)0.075f, kBetai2 = (double)0.0828f, kA1 = 0.31;
constexpr double kAlpha1 = (double)(5.0f / 9.0f), kAlpha2 = (double)0.44f, kBettast = (double)0.09f;

__device__ __forceinline__ double nmax(double a, double b) { return (b > a || a != a) ? b : a; }
__device__ __forceinline__ double nmin(double a, double b) { return (b < a || a != a) ? b : a; }
__device__ __forceinline__ double dmn(double a, double b) { return a < b ? a : b; }
__device__ __forceinline__ double dmx(double a, double b) { return a > b ? a : b; }

#define TURB_LOOP(b)                                                                                          \
  for (long long t_ = blockIdx.x * (long long)blockDim.x + threadIdx.x, n_ = (b).count(); t_ < n_;         \
       t_ += (long long)gridDim.x * blockDim.x)

// calcscm.f90:64-81: gen = |vis - viscos| S^2, limited by 0.9 rho k omega
__global__ void k_sst_gen(Dims d, Box b, const double* __restrict__ strain, const double* __restrict__ vis,
                          const double* __restrict__ den, const double* __restrict__ te,
                          const double* __restrict__ ed, double viscos, double* __restrict__ gen) {
  TURB_LOOP(b) {
    int i, j, k;
    b.at(t_, i, j, k);
    const int inp = ixk(d, i, j, k);
    const double ssq = strain[inp] * strain[inp];
    double g = fabs(vis[inp] - viscos) * ssq;
    g = dmn(g, (double)0.9f * den[inp] * te[inp] * ed[inp]);
    gen[inp] = g;
  }
}

struct SrcArgs {
  double *su, *sp, *sv;
  const double *gen, *vol, *den, *te, *ed, *vis, *fo, *foo, *wd;
  const double *gtx, *gty, *gtz, *gex, *gey, *gez;
  double *alphasst, *bettasst, *prt_te, *prt_ed, *domega;
  double viscos, densit, zero, timestep, btime;
  int bdf;
};

// k-equation volume sources (calcscm.f90:135-221, SST branch)
__global__ void k_sst_k_sources(Dims d, Box b, SrcArgs A) {
  TURB_LOOP(b) {
    int i, j, k;
    b.at(t_, i, j, k);
    const int inp = ixk(d, i, j, k);
    const double genp = dmx(A.gen[inp], A.zero), genn = dmn(A.gen[inp], A.zero);
    double su = genp * A.vol[inp];
    double sp = kBettast * A.ed[inp] * A.den[inp] * A.vol[inp];
    sp = sp - genn * A.vol[inp] / A.te[inp];
    if (A.bdf) {
      const double apotime = A.den[inp] * A.vol[inp] / A.timestep;
      const double sut = apotime * ((1 + A.btime) * A.fo[inp] - 0.5 * A.btime * A.foo[inp]);
      su = su + sut;
      sp = sp + apotime * (1 + 0.5 * A.btime);
    }
    A.su[inp] = su;
    A.sp[inp] = sp;
  }
}

// calculate_stuff_for_sst.f90:27-70, then the omega-equation volume
// sources (calcscm.f90:286-486, SST branch); the blending arrays are
// stored for fluxscm and the next step's k equation.
__global__ void k_sst_omega_sources(Dims d, Box b, SrcArgs A) {
  TURB_LOOP(b) {
    int i, j, k;
    b.at(t_, i, j, k);
    const int inp = ixk(d, i, j, k);
    const double wldist = A.wd[inp];
    const double den = A.den[inp], te = A.te[inp], ed = A.ed[inp];
    const double dot = A.gtx[inp] * A.gex[inp] + A.gty[inp] * A.gey[inp] + A.gtz[inp] * A.gez[inp];
    const double tmp1 = 2.0 * den / ((double)1.168f * ed) * dot;
    const double domegapl = nmax(tmp1, (double)1.e-10f);
    const double ksi = nmin(nmax(sqrt(te) / ((double)0.09f * wldist * ed), (500.0 * A.viscos / den) / (wldist * wldist * ed)),
                            4.0 * den * te / ((double)1.168f * domegapl * (wldist * wldist)));
    const double k2 = ksi * ksi;
    const double F = tanh(k2 * k2);
    const double alphasst = F * kAlpha1 + (1.0 - F) * kAlpha2;
    const double bettasst = F * kBetai1 + (1.0 - F) * kBetai2;
    A.alphasst[inp] = alphasst;
    A.bettasst[inp] = bettasst;
    A.prt_te[inp] = F * kSigmk1 + (1.0 - F) * kSigmk2;
    A.prt_ed[inp] = F * kSigmom1 + (1.0 - F) * kSigmom2;
    const double domega = nmax(2.0 * (1.0 - F) * den / ((double)1.168f * ed) * dot, 0.0);
    A.domega[inp] = domega;
    const double genp = dmx(A.gen[inp], A.zero), genn = dmn(A.gen[inp], A.zero);
    const double domegap = dmx(domega, A.zero);
    A.sv[inp] = 0.0;
    double vist = (A.vis[inp] - A.viscos) / A.densit;
    double su = alphasst * genp * A.vol[inp] / vist;
    su = su + domegap * A.vol[inp];
    vist = (A.vis[inp] - A.viscos) / A.densit;
    double sp = bettasst * den * ed * A.vol[inp];
    sp = sp - alphasst * genn * A.vol[inp] / (vist * ed);
    if (A.bdf) {
      const double apotime = den * A.vol[inp] / A.timestep;
      const double sut = apotime * ((1 + A.btime) * A.fo[inp] - 0.5 * A.btime * A.foo[inp]);
      su = su + sut;
      sp = sp + apotime * (1 + 0.5 * A.btime);
    }
    A.su[inp] = su;
    A.sp[inp] = sp;
  }
}

struct ScmFluxArgs {
  const double *arvx, *arvy, *arvz, *fif, *fcf, *x, *y, *z, *xc, *yc, *zc, *vis, *phi, *g1, *g2, *g3, *prt;
  double *acfe, *acfw, *su, *bp;
  double viscos, gam, zero;
  int idew, idns, idtb, lcds;
};

// fluxscm-overrelaxed-correction.f90:40-206 for one face inp
__global__ void k_fluxscm_faces(Dims d, Box b, ScmFluxArgs A) {
  TURB_LOOP(b) {
    int i, j, k;
    b.at(t_, i, j, k);
    const int inp = ixk(d, i, j, k);
    const int ine = inp + A.idew, ins = inp - A.idns, inb = inp - A.idtb, inbs = inb - A.idns;
    const double fxe = A.fif[inp], fxp = 1.0 - fxe;
    const double xpn = A.xc[ine] - A.xc[inp], ypn = A.yc[ine] - A.yc[inp], zpn = A.zc[ine] - A.zc[inp];
    const double dpn = sqrt(xpn * xpn + ypn * ypn + zpn * zpn);
    const double arx = A.arvx[inp], ary = A.arvy[inp], arz = A.arvz[inp];
    const double are = sqrt(arx * arx + ary * ary + arz * arz);
    const double costn = 1.0;
    const double vole = xpn * arx + ypn * ary + zpn * arz;
    const double d1x = costn, d1y = costn, d1z = costn;
    const double d2x = xpn * costn, d2y = ypn * costn, d2z = zpn * costn;
    const double prtr = A.prt[inp] * fxp + A.prt[ine] * fxe;
    const double viste = (A.vis[inp] - A.viscos) * fxp + (A.vis[ine] - A.viscos) * fxe;
    const double game = viste * prtr + A.viscos;
    const double xf = 0.25 * (A.x[inp] + A.x[ins] + A.x[inb] + A.x[inbs]);
    const double yf = 0.25 * (A.y[inp] + A.y[ins] + A.y[inb] + A.y[inbs]);
    const double zf = 0.25 * (A.z[inp] + A.z[ins] + A.z[inb] + A.z[inbs]);
    const double xi = A.xc[inp] * fxp + A.xc[ine] * fxe;
    const double yi = A.yc[inp] * fxp + A.yc[ine] * fxe;
    const double zi = A.zc[inp] * fxp + A.zc[ine] * fxe;
    const double dfixi = A.g1[inp] * fxp + A.g1[ine] * fxe;
    const double dfiyi = A.g2[inp] * fxp + A.g2[ine] * fxe;
    const double dfizi = A.g3[inp] * fxp + A.g3[ine] * fxe;
    const double pe = A.phi[ine], pp = A.phi[inp];
    const double dfixii = dfixi * d1x + arx / vole * (pe - pp - dfixi * d2x - dfiyi * d2y - dfizi * d2z);
    const double dfiyii = dfiyi * d1y + ary / vole * (pe - pp - dfixi * d2x - dfiyi * d2y - dfizi * d2z);
    const double dfizii = dfizi * d1z + arz / vole * (pe - pp - dfixi * d2x - dfiyi * d2y - dfizi * d2z);
    const double fdfie = game * (dfixii * arx + dfiyii * ary + dfizii * arz);
    const double fdfii = game * are / dpn * (dfixi * xpn + dfiyi * ypn + dfizi * zpn);
    const double de = game * are / dpn;
    const double fm = A.fcf[inp];
    const double ce = dmn(fm, A.zero), cp = dmx(fm, A.zero);
    A.acfe[inp] = de - ce;
    A.acfw[ine] = de + cp;
    double fcfie;
    if (A.lcds) {
      const double fii = pp * fxp + pe * fxe + (dfixi * (xf - xi) + dfiyi * (yf - yi) + dfizi * (zf - zi));
      fcfie = fm * fii;
    } else {
      const double r1 = (2 * A.g1[inp] * xpn + 2 * A.g2[inp] * ypn + 2 * A.g3[inp] * zpn) / (pe - pp) - 1.0;
      const double r2 = (2 * A.g1[ine] * xpn + 2 * A.g2[ine] * ypn + 2 * A.g3[ine] * zpn) / (pp - pe) - 1.0;
      const double psiw = nmax(0.0, nmin(nmin(2.0 * r1, 0.5 * r1 + 0.5), 2.0));
      const double psie = nmax(0.0, nmin(nmin(2.0 * r2, 0.5 * r2 + 0.5), 2.0));
      fcfie = ce * (pe + fxe * psie * (pp - pe)) + cp * (pp + fxp * psiw * (pe - pp));
    }
    const double fcfii = ce * pe + cp * pp;
    const double ffic = A.gam * (fcfie - fcfii);
    const double suadd = -ffic + fdfie - fdfii;
    A.su[inp] = A.su[inp] + suadd;
    A.bp[ine] = suadd;
  }
}

// fluxscm-overrelaxed-correction.f90:208-216: su(inp+idew) -= bp(inp+idew)
__global__ void k_scm_staged(Dims d, Box b, int idew, double* su, const double* __restrict__ bp) {
  TURB_LOOP(b) {
    int i, j, k;
    b.at(t_, i, j, k);
    const int inp = ixk(d, i, j, k) + idew;
    su[inp] = su[inp] - bp[inp];
  }
}

struct AsmArgs {
  double *ae, *aw, *an, *as, *at, *ab, *ap, *su, *sp;
  const double *phi, *fo, *den, *vol;
  double urfrs, urfms, timestep;
  int cn;
};

// calcscm.f90:546-586: Crank-Nicolson terms, ap, under-relaxation
__global__ void k_scm_assemble(Dims d, Box b, AsmArgs A) {
  TURB_LOOP(b) {
    int i, j, k;
    b.at(t_, i, j, k);
    const int inp = ixk(d, i, j, k);
    double ae = A.ae[inp], aw = A.aw[inp], an = A.an[inp], as = A.as[inp], at = A.at[inp], ab = A.ab[inp];
    double su = A.su[inp], sp = A.sp[inp];
    if (A.cn) {
      ae = 0.5 * ae; an = 0.5 * an; at = 0.5 * at; aw = 0.5 * aw; as = 0.5 * as; ab = 0.5 * ab;
      A.ae[inp] = ae; A.an[inp] = an; A.at[inp] = at; A.aw[inp] = aw; A.as[inp] = as; A.ab[inp] = ab;
      const double apotime = A.den[inp] * A.vol[inp] / A.timestep;
      const double* o = A.fo;
      su = su + (ae * o[inp + d.nj] + aw * o[inp - d.nj] + an * o[inp + 1] + as * o[inp - 1] + at * o[inp + d.nij] +
                 ab * o[inp - d.nij]) +
           (apotime - ae - aw - an - as - at - ab) * o[inp];
      sp = sp + apotime;
      A.sp[inp] = sp;
    }
    double ap = ae + aw + an + as + at + ab + sp;
    ap = ap * A.urfrs;
    A.ap[inp] = ap;
    A.su[inp] = su + A.urfms * ap * A.phi[inp];
  }
}

// calcscm.f90:595-599: fi >= small over the whole array
__global__ void k_clip_small(long long n, double* fi) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
    fi[t] = dmx(fi[t], CAP_SMALL);
}

// modvis.f90:207-233 (SST, high-Re)
__global__ void k_modvis_sst(Dims d, Box b, const double* __restrict__ wd, const double* __restrict__ te,
                             const double* __restrict__ ed, const double* __restrict__ den,
                             const double* __restrict__ strain, double* __restrict__ vis, double viscos, double cmu,
                             double urf) {
  TURB_LOOP(b) {
    int i, j, k;
    b.at(t_, i, j, k);
    const int inp = ixk(d, i, j, k);
    const double visold = vis[inp];
    const double wldist = wd[inp];
    const double etha = nmax(2 * sqrt(te[inp]) / (cmu * wldist * ed[inp]),
                             (500 * viscos / den[inp]) / (wldist * wldist * ed[inp]));
    const double f2 = tanh(etha * etha);
    double v = viscos + den[inp] * kA1 * te[inp] / nmax(nmax(kA1, ed[inp]), strain[inp] * f2);
    v = urf * v + (1.0 - urf) * visold;
    vis[inp] = v;
  }
}

int fluxscm(int idew, int idns, int idtb, int fi, int gx, int ifi, int arvx, int arvy, int arvz, int fif, int acfe,
            int acfw, int fcf) {
  Ctx& c = ctx();
  const Dims& d = c.d;
  double** F = c.f;
  const cappgpu_params& P = c.prm;
  ScmFluxArgs A{F[arvx], F[arvy], F[arvz], F[fif], F[fcf], F[CAP_X], F[CAP_Y], F[CAP_Z], F[CAP_XC], F[CAP_YC],
                F[CAP_ZC], F[CAP_VIS], F[fi], F[gx], F[gx + 1], F[gx + 2],
                ifi == CAP_ITE ? F[CAP_PRTINV_TE] : F[CAP_PRTINV_ED], F[acfe], F[acfw], F[CAP_SU], F[CAP_BP],
                P.viscos, P.gds[ifi - 1], P.zero, idew, idns, idtb, P.lcds};
  const Box b{2, d.nimm, 2, d.njmm, 2, d.nkmm};
  launch(k_fluxscm_faces, grid_for(b.count()), kThreads, c.st, d, b, A);
  launch(k_scm_staged, grid_for(b.count()), kThreads, c.st, d, b, idew, F[CAP_SU], (const double*)F[CAP_BP]);
  CAP_CHECK_LAUNCH();
  CAP_CUDA(cudaMemsetAsync(F[CAP_BP], 0, sizeof(double) * d.nijk, c.st));
  return CAPPGPU_OK;
}

}  // namespace

// calcscm.f90:3-602 for ifi = ite or ied (SST)
int calcscm(int ifi, cappgpu_solve_report* rep) {
  Ctx& c = ctx();
  const Dims& d = c.d;
  double** F = c.f;
  const cappgpu_params& P = c.prm;
  if (!P.sst) { set_error("calcscm: only the k-omega SST model is built (sst = 1)"); return CAPPGPU_E_ARG; }
  if (P.lbuoy) { set_error("calcscm: buoyancy sources of the turbulence equations are not built"); return CAPPGPU_E_ARG; }
  const int fi = ifi == CAP_ITE ? CAP_TE : CAP_ED;
  const int gx = ifi == CAP_ITE ? CAP_GRADTE_X : CAP_GRADED_X;
  const int fo = ifi == CAP_ITE ? CAP_TEO : CAP_EDO;
  const int foo = ifi == CAP_ITE ? CAP_TEOO : CAP_EDOO;
  int rc;
  if ((rc = grad_gauss(fi, gx, gx + 1, gx + 2))) return rc;   // calcscm.f90:53-55
  const Box b{3, d.nimm, 3, d.njmm, 3, d.nkmm};
  SrcArgs A{F[CAP_SU], F[CAP_SP], F[CAP_SV], F[CAP_GEN], F[CAP_VOL], F[CAP_DEN], F[CAP_TE], F[CAP_ED], F[CAP_VIS],
            F[fo], F[foo], F[CAP_WALLDIST], F[CAP_GRADTE_X], F[CAP_GRADTE_Y], F[CAP_GRADTE_Z], F[CAP_GRADED_X],
            F[CAP_GRADED_Y], F[CAP_GRADED_Z], F[CAP_ALPHASST], F[CAP_BETTASST], F[CAP_PRTINV_TE], F[CAP_PRTINV_ED],
            F[CAP_DOMEGA], P.viscos, P.densit, P.zero, P.timestep, P.btime, P.bdf};
  if (ifi == CAP_ITE) {
    if ((rc = find_strain_rate())) return rc;   // calcscm.f90:62
    launch(k_sst_gen, grid_for(b.count()), kThreads, c.st, d, b, (const double*)F[CAP_STRAIN],
           (const double*)F[CAP_VIS], (const double*)F[CAP_DEN], (const double*)F[CAP_TE], (const double*)F[CAP_ED],
           P.viscos, F[CAP_GEN]);
    launch(k_sst_k_sources, grid_for(b.count()), kThreads, c.st, d, b, A);
  } else {
    launch(k_sst_omega_sources, grid_for(b.count()), kThreads, c.st, d, b, A);
  }
  CAP_CHECK_LAUNCH();
  if ((rc = fluxscm(d.nj, 1, d.nij, fi, gx, ifi, CAP_AR1X, CAP_AR1Y, CAP_AR1Z, CAP_FX, CAP_AE, CAP_AW, CAP_F1)))
    return rc;
  if ((rc = fluxscm(1, d.nij, d.nj, fi, gx, ifi, CAP_AR2X, CAP_AR2Y, CAP_AR2Z, CAP_FY, CAP_AN, CAP_AS, CAP_F2)))
    return rc;
  if ((rc = fluxscm(d.nij, d.nj, 1, fi, gx, ifi, CAP_AR3X, CAP_AR3Y, CAP_AR3Z, CAP_FZ, CAP_AT, CAP_AB, CAP_F3)))
    return rc;
  AsmArgs M{F[CAP_AE], F[CAP_AW], F[CAP_AN], F[CAP_AS], F[CAP_AT], F[CAP_AB], F[CAP_AP], F[CAP_SU], F[CAP_SP],
            F[fi], F[fo], F[CAP_DEN], F[CAP_VOL], 1.0 / P.urf[ifi - 1], 1.0 - P.urf[ifi - 1], P.timestep, P.cn};
  launch(k_scm_assemble, grid_for(b.count()), kThreads, c.st, d, b, M);
  CAP_CHECK_LAUNCH();
  rc = solve(CAPPGPU_SOLVER_SIPSOL, fi, ifi, rep);   // calcscm.f90:591
  if (rc < 0) return rc;
  launch(k_clip_small, grid_for(d.nijk), kThreads, c.st, (long long)d.nijk, F[fi]);
  CAP_CHECK_LAUNCH();
  return rc;
}

// modvis.f90:195-236 (SST) over k = 2..nkm, i = 3..nimm, j = 3..njmm
int modvis() {
  Ctx& c = ctx();
  const Dims& d = c.d;
  double** F = c.f;
  const cappgpu_params& P = c.prm;
  if (!P.sst) return CAPPGPU_OK;
  const Box b{3, d.nimm, 3, d.njmm, 2, d.nkm};
  launch(k_modvis_sst, grid_for(b.count()), kThreads, c.st, d, b, (const double*)F[CAP_WALLDIST],
         (const double*)F[CAP_TE], (const double*)F[CAP_ED], (const double*)F[CAP_DEN], (const double*)F[CAP_STRAIN],
         F[CAP_VIS], P.viscos, P.cmu, P.urf[CAP_IVIS - 1]);
  CAP_CHECK_LAUNCH();
  return CAPPGPU_OK;
}

}  // namespace cap

using namespace cap;

extern "C" {

int cappgpu_calcscm(int ifi, cappgpu_solve_report* rep) {
  CAP_REQUIRE_INIT();
  if (ifi != CAP_ITE && ifi != CAP_IED) { set_error("calcscm: ifi must be ite (5) or ied (6)"); return CAPPGPU_E_ARG; }
  int rc = calcscm(ifi, rep);
  cudaError_t e = cudaStreamSynchronize(ctx().st);
  if (e != cudaSuccess) return cuda_fail(e, "calcscm", __FILE__, __LINE__);
  return rc;
}

int cappgpu_modvis(void) {
  CAP_REQUIRE_INIT();
  int rc = modvis();
  if (rc) return rc;
  CAP_CUDA(cudaStreamSynchronize(ctx().st));
  return CAPPGPU_OK;
}


}  // extern "C"
