// One RK stage of the FP64 path that allocates no memory.
//
// Some callers cannot let a library call cudaMalloc: solvers that hand every
// device buffer out of their own pre-sized arena and must stay inside it,
// and latency-sensitive hosts for which the implicit device-wide
// synchronisation cudaMalloc/cudaFree can cause is not acceptable.  For
// them this entry point takes device pointers for all inputs and outputs
// (allocated by the caller) and keeps its only scratch -- the per-block
// partial sums of the stage-3 change norms and force integrals -- in a
// file-scope static __device__ array that every GPU loading this library
// holds until the process exits.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "../../include/bcm_gb300.h"
#include "bcm_kernels.h"

namespace {

// Block sums of 7 quantities; one block reduces kChunk interior cells, so
// the scratch bounds the case at kMaxBlocks * kChunk interior cells.
constexpr int kMaxBlocks = 8192;
constexpr long long kChunk = 4096;
constexpr long long kMaxCells = kMaxBlocks * kChunk;  // 33,554,432 cells

static __device__ __align__(256) double g_noalloc_partials[kMaxBlocks * 7];

constexpr int kMaxDevices = 64;
double *g_partials_addr[kMaxDevices] = {nullptr};
std::mutex g_setup_mu;

thread_local char g_msg[256];

int fail(const char *m) {
  snprintf(g_msg, sizeof g_msg, "%s", m);
  bcmg_internal_set_error(g_msg);
  return BCMG_ERR_ARG;
}
int fail_cuda(const char *what, cudaError_t e) {
  snprintf(g_msg, sizeof g_msg, "%s: %s", what, cudaGetErrorString(e));
  bcmg_internal_set_error(g_msg);
  return BCMG_ERR_CUDA;
}

// Device address of the static scratch on the current device, looked up
// once per device with that device current (host code only knows the
// symbol's host-side stand-in, not its device address).
int scratch_on_current_device(double **out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail_cuda("cudaGetDevice", e);
  if (dev < 0 || dev >= kMaxDevices) return fail("device ordinal beyond the supported 64");
  std::lock_guard<std::mutex> lock(g_setup_mu);
  if (!g_partials_addr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_partials);
    if (e != cudaSuccess) return fail_cuda("cudaGetSymbolAddress", e);
    g_partials_addr[dev] = static_cast<double *>(p);
  }
  *out = g_partials_addr[dev];
  return BCMG_OK;
}

}  // namespace

extern "C" int bcmg_flux_rk_stage_noalloc(int ncube, int RK, double deltaT, double deltaTau,
                                          double e, const int *FWS, const double *cube_size,
                                          double *U1_, const double *U1, const double *U1q,
                                          double *U1p1, double *U1p2, double *Rku1,
                                          double *Residual1, double *er, void *stream) {
  bcmg_internal_set_error(nullptr);
  if (ncube < 2 || RK < 1 || RK > 3 || !FWS || !cube_size || !U1_ || !U1 || !U1q || !U1p1 ||
      !U1p2 || !Rku1 || !Residual1 || (RK == 3 && !er))
    return fail("bcmg_flux_rk_stage_noalloc: bad arguments");
  bcmg_reference_config cfg;
  bcmg_get_reference_config(&cfg);
  if (cfg.ncube_x <= 0 || cfg.ncube_x % 4 != 0 || cfg.ncube_x > 256)
    return fail("bcmg_flux_rk_stage_noalloc: the reference configuration's ncube_x must be a "
                "positive multiple of 4 up to 256");
  const long long n3 = (long long)cfg.ncube_x * cfg.ncube_x * cfg.ncube_x;
  const long long total = (long long)(ncube - 1) * n3;
  if (total > kMaxCells)
    return fail("bcmg_flux_rk_stage_noalloc: case exceeds the fixed scratch (at most "
                "33,554,432 interior cells)");
  double *partials = nullptr;
  int r = scratch_on_current_device(&partials);
  if (r) return r;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  bcmg::Phys ph;
  ph.n = cfg.ncube_x;
  ph.mpi_ncube = cfg.mpi_ncube;
  ph.mu_L = cfg.mu_L;
  ph.rho0 = cfg.rho0;
  ph.U0 = cfg.U0;
  ph.Uin = cfg.Uin;
  ph.P0 = cfg.P0;
  bcmg::FluxArgs a;
  a.ph = ph;
  a.cube0 = 1;
  a.dT = deltaT;
  a.dTau = deltaTau;
  a.e = e;
  a.FWS = FWS;
  a.cube_size = cube_size;
  a.U1_ = U1_;
  a.U1 = U1;
  a.U1q = U1q;
  a.Rku1 = Rku1;
  a.Residual1 = Residual1;
  cudaError_t ce = bcmg::launch_flux_fp64(a, ncube - 1, s);
  if (ce != cudaSuccess) return fail_cuda("flux kernel", ce);
  bcmg::RkArgs k;
  k.ph = ph;
  k.ncube = ncube;
  k.RK = RK;
  k.FWS = FWS;
  k.U1_ = U1_;
  k.U1p1 = U1p1;
  k.U1p2 = U1p2;
  k.Rku1 = Rku1;
  k.Residual1 = Residual1;
  k.partials = partials;
  const int nblocks = (int)((total + kChunk - 1) / kChunk);
  ce = bcmg::launch_rk_chunked(k, kChunk, nblocks, s);
  if (ce != cudaSuccess) return fail_cuda("stage kernel", ce);
  if (RK == 3) {
    ce = bcmg::launch_norms(ph, partials, nblocks, er, s);
    if (ce != cudaSuccess) return fail_cuda("norm kernel", ce);
  }
  return BCMG_OK;
}
