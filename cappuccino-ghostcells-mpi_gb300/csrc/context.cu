// context.cu -- the library's module state on the device: lifecycle,
// fields, parameters, BC codes, host-address registry, index maps,
// geometry set-up and the single-rank communication entry points.
#include <stdarg.h>
#include <string.h>

#include <mutex>
#include <string>

#include "common.cuh"
#include "kernels.cuh"

namespace cap {

static Ctx g_ctx;
static char g_err[512] = "";

Ctx& ctx() { return g_ctx; }

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

int cuda_fail(cudaError_t e, const char* what, const char* file, int line) {
  set_error("CUDA error %s (%s) in %s at %s:%d", cudaGetErrorName(e), cudaGetErrorString(e), what,
            file, line);
  return CAPPGPU_E_CUDA;
}

__global__ void k_finish_reduce(const double* part, double* out, int nv, int is_max) {
  // one warp per value, fixed order: lane l sums partials l, l+32, ... then
  // a fixed shuffle tree combines the 32 lane sums.
  int v = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (v >= nv) return;
  const double* p = part + v * kRedBlocks;
  double s = 0.0;
  for (int b = lane; b < kRedBlocks; b += 32) s = is_max ? fmax(s, p[b]) : s + p[b];
  for (int o = 16; o > 0; o >>= 1) {
    double t = __shfl_down_sync(0xffffffffu, s, o);
    s = is_max ? fmax(s, t) : s + t;
  }
  if (lane == 0) out[v] = s;
}

int finish_reduce(int nv, bool is_max, int first) {
  Ctx& c = ctx();
  launch(k_finish_reduce, 1, 32 * kMaxRed, c.st, c.partials + first * kRedBlocks, c.redout, nv, is_max ? 1 : 0);
  CAP_CHECK_LAUNCH();
  return CAPPGPU_OK;
}

int fetch_reduce(int nv, double* out) {
  Ctx& c = ctx();
  CAP_CUDA(cudaMemcpyAsync(c.hred, c.redout, sizeof(double) * nv, cudaMemcpyDeviceToHost, c.st));
  CAP_CUDA(cudaStreamSynchronize(c.st));
  for (int q = 0; q < nv; ++q) out[q] = c.hred[q];
  return CAPPGPU_OK;
}

static const char* kFieldNames[CAP_NFIELDS] = {
    "x", "y", "z", "xc", "yc", "zc", "vol", "fx", "fy", "fz",
    "ar1x", "ar1y", "ar1z", "ar2x", "ar2y", "ar2z", "ar3x", "ar3y", "ar3z", "walldist",
    "u", "v", "w", "p", "pp", "f1", "f2", "f3", "vis", "den", "te", "ed", "t", "strain",
    "uo", "vo", "wo", "uoo", "voo", "woo",
    "ae", "aw", "an", "as", "at", "ab", "ap", "sp", "spv", "su", "sv", "sw", "res",
    "apu", "apv", "apw",
    "bb", "bs", "bw", "bp", "bn", "be", "bt",
    "he", "hw", "hn", "hs", "ht", "hb",
    "gradu_x", "gradu_y", "gradu_z", "gradv_x", "gradv_y", "gradv_z",
    "gradw_x", "gradw_y", "gradw_z", "gradp_x", "gradp_y", "gradp_z",
    "gradte_x", "gradte_y", "gradte_z", "graded_x", "graded_y", "graded_z",
    "gen", "alphasst", "bettasst", "domega", "prtinv_te", "prtinv_ed",
    "teo", "edo", "teoo", "edoo"};

// Output field of the 7-point products (cappgpu_spmv, cappgpu_spmv_noalloc):
// not one of the coefficients it reads (ae..ap, read through restrict
// pointers) nor a grid-geometry field (a product written there would
// leave the geometry caches stale).
bool spmv_output_ok(int q) {
  if (q >= CAP_AE && q <= CAP_AP) return false;
  if (q >= CAP_X && q <= CAP_AR3Z) return false;   // nodes, centres, vol, fx..fz, face areas
  return true;
}

void note_write(int q) {
  switch (q) {
    case CAP_X: case CAP_Y: case CAP_Z: case CAP_XC: case CAP_YC: case CAP_ZC:
    case CAP_FX: case CAP_FY: case CAP_FZ:
    case CAP_AR1X: case CAP_AR1Y: case CAP_AR1Z: case CAP_AR2X: case CAP_AR2Y: case CAP_AR2Z:
    case CAP_AR3X: case CAP_AR3Y: case CAP_AR3Z: case CAP_VOL:
      ++ctx().geo_gen;
      break;
    default:
      break;
  }
}

static void free_all() {
  fast_free();
  learned_free();
  facegeo_free();
  volr_free();
  outbc_free();
  Ctx& c = ctx();
  for (auto& p : c.f) { if (p) cudaFree(p); p = nullptr; }
  for (auto& p : c.bc) { if (p) cudaFree(p); p = nullptr; }
  for (auto& p : c.work) { if (p) cudaFree(p); p = nullptr; }
  if (c.li) cudaFree(c.li);
  if (c.lk) cudaFree(c.lk);
  if (c.partials) cudaFree(c.partials);
  if (c.redout) cudaFree(c.redout);
  if (c.hred) cudaFreeHost(c.hred);
  if (c.dscal) cudaFree(c.dscal);
  if (c.wf_flags) cudaFree(c.wf_flags);
  if (c.vec3buf) cudaFree(c.vec3buf);
  for (auto& e : c.ev) { if (e) cudaEventDestroy(e); e = nullptr; }
  for (auto& e : c.sw_ev) { if (e) cudaEventDestroy(e); e = nullptr; }
  if (c.st) cudaStreamDestroy(c.st);
  c = Ctx();
}

static int bc_len(const Dims& d, int face) {
  return face <= CAP_LBE ? d.njk : face <= CAP_LBN ? d.nik : d.nij;
}

}  // namespace cap

using namespace cap;

extern "C" {

const char* cappgpu_last_error(void) { return g_err; }

const char* cappgpu_field_name(int field) {
  return (field >= 0 && field < CAP_NFIELDS) ? kFieldNames[field] : "";
}

int cappgpu_field_id(const char* name) {
  if (!name) return -1;
  for (int q = 0; q < CAP_NFIELDS; ++q)
    if (strcmp(name, kFieldNames[q]) == 0) return q;
  return -1;
}

int cappgpu_init(int ni, int nj, int nk) {
  if (ni < 5 || nj < 5 || nk < 5) { set_error("grid %dx%dx%d too small", ni, nj, nk); return CAPPGPU_E_ARG; }
  if ((long long)ni * nj * nk > 0x7fffffffLL) { set_error("grid too large for int32 indices"); return CAPPGPU_E_ARG; }
  if (ctx().init) free_all();
  Ctx& c = ctx();
  Dims& d = c.d;
  // setind.f90:21-40
  d.ni = ni; d.nj = nj; d.nk = nk;
  d.nim = ni - 1; d.njm = nj - 1; d.nkm = nk - 1;
  d.nimm = d.nim - 1; d.njmm = d.njm - 1; d.nkmm = d.nkm - 1;
  d.nij = ni * nj; d.nik = ni * nk; d.njk = nj * nk; d.nijk = d.nij * nk;
  size_t nb = sizeof(double) * (size_t)d.nijk;
  CAP_CUDA(cudaGetDevice(&c.device));   // the context's stream and arrays live on this device
  CAP_CUDA(cudaStreamCreateWithFlags(&c.st, cudaStreamNonBlocking));
  for (int q = 0; q < CAP_NFIELDS; ++q) {
    if (cudaMalloc(&c.f[q], nb) != cudaSuccess) { free_all(); set_error("out of device memory"); return CAPPGPU_E_NOMEM; }
    CAP_CUDA(cudaMemsetAsync(c.f[q], 0, nb, c.st));
  }
  for (int q = 0; q < 8; ++q) {
    if (cudaMalloc(&c.work[q], nb) != cudaSuccess) { free_all(); set_error("out of device memory"); return CAPPGPU_E_NOMEM; }
    CAP_CUDA(cudaMemsetAsync(c.work[q], 0, nb, c.st));
  }
  for (int q = 0; q < CAP_NBC; ++q) {
    CAP_CUDA(cudaMalloc(&c.bc[q], sizeof(int) * bc_len(d, q)));
    CAP_CUDA(cudaMemsetAsync(c.bc[q], 0, sizeof(int) * bc_len(d, q), c.st));
  }
  // index maps li(1..ni), lk(1..nk) kept 1-based (element 0 unused)
  int* hli = new int[ni + 1];
  int* hlk = new int[nk + 1];
  hli[0] = hlk[0] = 0;
  for (int i = 1; i <= ni; ++i) hli[i] = (i - 1) * nj;
  for (int k = 1; k <= nk; ++k) hlk[k] = (k - 1) * d.nij;
  CAP_CUDA(cudaMalloc(&c.li, sizeof(int) * (ni + 1)));
  CAP_CUDA(cudaMalloc(&c.lk, sizeof(int) * (nk + 1)));
  CAP_CUDA(cudaMemcpy(c.li, hli, sizeof(int) * (ni + 1), cudaMemcpyHostToDevice));
  CAP_CUDA(cudaMemcpy(c.lk, hlk, sizeof(int) * (nk + 1), cudaMemcpyHostToDevice));
  delete[] hli;
  delete[] hlk;
  CAP_CUDA(cudaMalloc(&c.partials, sizeof(double) * kMaxRed * kRedBlocks));
  CAP_CUDA(cudaMalloc(&c.redout, sizeof(double) * kMaxRed));
  CAP_CUDA(cudaMallocHost(&c.hred, sizeof(double) * kMaxRed));
  CAP_CUDA(cudaMalloc(&c.dscal, sizeof(double) * 16));
  CAP_CUDA(cudaMemsetAsync(c.dscal, 0, sizeof(double) * 16, c.st));
  CAP_CUDA(cudaMalloc(&c.wf_flags, sizeof(int) * 1024 * 1024));
  CAP_CUDA(cudaMemsetAsync(c.wf_flags, 0, sizeof(int) * 1024 * 1024, c.st));
  // defaults of init.f90:164-168,342 and the solver switches of the reference
  memset(&c.prm, 0, sizeof(c.prm));
  c.prm.alfa = 0.92;
  c.prm.cappa = 0.41;
  c.prm.elog = 8.432;
  c.prm.densit = 1.0;
  c.prm.isol_p = CAPPGPU_SOLVER_CGSTAB_SIP;
  c.prm.piso_solver = CAPPGPU_SOLVER_PCGSIP;
  for (auto& e : c.ev) CAP_CUDA(cudaEventCreate(&e));
  CAP_CUDA(cudaStreamSynchronize(c.st));
  c.init = true;
  return CAPPGPU_OK;
}

int cappgpu_finalize(void) {
  if (ctx().init) {
    cudaStreamSynchronize(ctx().st);
    free_all();
  }
  return CAPPGPU_OK;
}

int cappgpu_set_field(int field, const double* host, int64_t n) {
  CAP_REQUIRE_INIT();
  Ctx& c = ctx();
  if (field < 0 || field >= CAP_NFIELDS || !host || n != c.d.nijk) {
    set_error("set_field: bad field %d or size %lld (nijk=%d)", field, (long long)n, c.d.nijk);
    return CAPPGPU_E_ARG;
  }
  note_write(field);
  CAP_CUDA(cudaMemcpyAsync(c.f[field], host, sizeof(double) * n, cudaMemcpyHostToDevice, c.st));
  CAP_CUDA(cudaStreamSynchronize(c.st));
  return CAPPGPU_OK;
}

int cappgpu_get_field(int field, double* host, int64_t n) {
  CAP_REQUIRE_INIT();
  Ctx& c = ctx();
  if (field < 0 || field >= CAP_NFIELDS || !host || n != c.d.nijk) {
    set_error("get_field: bad field %d or size %lld (nijk=%d)", field, (long long)n, c.d.nijk);
    return CAPPGPU_E_ARG;
  }
  CAP_CUDA(cudaMemcpyAsync(host, c.f[field], sizeof(double) * n, cudaMemcpyDeviceToHost, c.st));
  CAP_CUDA(cudaStreamSynchronize(c.st));
  return CAPPGPU_OK;
}

int cappgpu_set_bc(int face, const int* codes, int64_t n) {
  CAP_REQUIRE_INIT();
  Ctx& c = ctx();
  if (face < 0 || face >= CAP_NBC || !codes || n != bc_len(c.d, face)) {
    set_error("set_bc: bad face %d or size %lld", face, (long long)n);
    return CAPPGPU_E_ARG;
  }
  CAP_CUDA(cudaMemcpyAsync(c.bc[face], codes, sizeof(int) * n, cudaMemcpyHostToDevice, c.st));
  CAP_CUDA(cudaStreamSynchronize(c.st));
  return CAPPGPU_OK;
}

int cappgpu_set_params(const cappgpu_params* p) {
  CAP_REQUIRE_INIT();
  if (!p) { set_error("set_params: null"); return CAPPGPU_E_ARG; }
  Ctx& c = ctx();
  const Dims& d = c.d;
  if (p->ipr < 1 || p->ipr > d.ni || p->jpr < 1 || p->jpr > d.nj || p->kpr < 1 || p->kpr > d.nk) {
    set_error("set_params: reference cell (%d,%d,%d) outside the grid", p->ipr, p->jpr, p->kpr);
    return CAPPGPU_E_ARG;
  }
  c.prm = *p;
  return CAPPGPU_OK;
}

int cappgpu_get_params(cappgpu_params* p) {
  CAP_REQUIRE_INIT();
  if (!p) { set_error("get_params: null"); return CAPPGPU_E_ARG; }
  *p = ctx().prm;
  return CAPPGPU_OK;
}

int cappgpu_register(int field, double* host) {
  CAP_REQUIRE_INIT();
  if (field < 0 || field >= CAP_NFIELDS) { set_error("register: bad field %d", field); return CAPPGPU_E_ARG; }
  ctx().host_reg[field] = host;
  return CAPPGPU_OK;
}

int cappgpu_unregister_all(void) {
  CAP_REQUIRE_INIT();
  for (auto& p : ctx().host_reg) p = nullptr;
  return CAPPGPU_OK;
}

int cappgpu_get_index_maps(int* li, int* lk) {
  CAP_REQUIRE_INIT();
  Ctx& c = ctx();
  if (!li || !lk) { set_error("get_index_maps: null"); return CAPPGPU_E_ARG; }
  CAP_CUDA(cudaMemcpy(li, c.li + 1, sizeof(int) * c.d.ni, cudaMemcpyDeviceToHost));
  CAP_CUDA(cudaMemcpy(lk, c.lk + 1, sizeof(int) * c.d.nk, cudaMemcpyDeviceToHost));
  return CAPPGPU_OK;
}

// Run-time options: "wave" = 1 (persistent hyperplane wavefront, default)
// or 0 (one kernel launch per hyperplane, the simple form kept for checks).
int cappgpu_set_option(const char* key, int value) {
  CAP_REQUIRE_INIT();
  if (!key) return CAPPGPU_E_ARG;
  if (strcmp(key, "wave") == 0 && (value == 0 || value == 1)) { ctx().wave_impl = value; return CAPPGPU_OK; }
  if (strcmp(key, "cg_batch") == 0 && value >= 1 && value <= 64) {
    ctx().cg_batch = value;
    return CAPPGPU_OK;
  }
  if (strcmp(key, "inner_drop") == 0 && value >= 1 && value <= 9) {
    ctx().inner_drop = value;
    return CAPPGPU_OK;
  }
  if (strcmp(key, "fp32_parts") == 0 && value >= 0 && value <= 31) {
    ctx().fp32_parts = value;
    return CAPPGPU_OK;
  }
  if (strcmp(key, "learn_conv") == 0 && value >= 0 && value <= 2) return learned_set_conv(value);
  if (strcmp(key, "learn_loss") == 0 && value >= 0 && value <= 2) return learned_set_loss(value);
  if (strcmp(key, "sweep_timing") == 0 && (value == 0 || value == 1)) {
    Ctx& c = ctx();
    if (value && !c.sw_ev[0])
      for (auto& e : c.sw_ev) CAP_CUDA(cudaEventCreate(&e));
    c.sweep_timing = value;
    return CAPPGPU_OK;
  }
  if (strcmp(key, "fused_dot") == 0 && (value == 0 || value == 1)) {
    ctx().fused_dot = value;
    return CAPPGPU_OK;
  }
  if (strcmp(key, "lane_wave") == 0 && value >= 0 && value <= 2) {
    ctx().lane_wave = value;
    return CAPPGPU_OK;
  }
  if (strcmp(key, "face_geo") == 0 && (value == 0 || value == 1)) {
    ctx().face_geo = value;
    if (!value) {
      facegeo_free();
      volr_free();
    }
    return CAPPGPU_OK;
  }
  if (strcmp(key, "spin_limit") == 0 && value >= 1) {
    ctx().spin_limit = value;
    return CAPPGPU_OK;
  }
  if (strcmp(key, "sip_slabs") == 0 && value >= 1 && value <= 4096) {
    ctx().sip_slabs = value;
    return CAPPGPU_OK;
  }
  if (strcmp(key, "sip_slab_axis") == 0 && (value == 0 || value == 1)) {
    ctx().sip_slab_axis = value;
    return CAPPGPU_OK;
  }
  if (strcmp(key, "tight_correctors") == 0 && (value == 0 || value == 1)) {
    ctx().tight_correctors = value;
    return CAPPGPU_OK;
  }
  set_error("unknown option %s=%d", key, value);
  return CAPPGPU_E_ARG;
}

// Precision of the pressure solve (pcgsip): 0 = FP64 plain, the reference's
// arithmetic (default); 1 = FP32 SIP-preconditioned CG inside FP64
// iterative refinement; 2 = as 1, starting from the learned initial guess.
int cappgpu_precision(int mode) {
  CAP_REQUIRE_INIT();
  if (mode < 0 || mode > 2) {
    set_error("precision mode %d: 0 (FP64 plain), 1 (FP32 + FP64 refinement) or 2 (1 + learned guess)", mode);
    return CAPPGPU_E_ARG;
  }
  ctx().precision = mode;
  return CAPPGPU_OK;
}

int cappgpu_ijkpr(void) {
  if (!ctx().init) return CAPPGPU_E_NOINIT;
  const cappgpu_params& p = ctx().prm;
  // setind.f90:56, 1-based as in the reference
  return (p.kpr - 1) * ctx().d.nij + (p.ipr - 1) * ctx().d.nj + p.jpr;
}

// exchange_mpi.f90:4-89 -- the only neighbour of a single rank is itself
// (read_grid.f90:232, nproc-this with both 0), so SENDRECV_REPLACE returns
// the packed values unchanged: the identity on phi.
int cappgpu_exchange(int field) {
  CAP_REQUIRE_INIT();
  if (field < 0 || field >= CAP_NFIELDS) { set_error("exchange: bad field %d", field); return CAPPGPU_E_ARG; }
  return CAPPGPU_OK;
}

// global_sum_mpi.f90 / global_max_mpi.f90: MPI_ALLREDUCE over one rank.
int cappgpu_global_sum(double* phi) { return phi ? CAPPGPU_OK : CAPPGPU_E_ARG; }
int cappgpu_global_max(double* phi) { return phi ? CAPPGPU_OK : CAPPGPU_E_ARG; }

}  // extern "C"
