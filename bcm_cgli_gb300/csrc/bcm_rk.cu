// RK stage combination, change norms and force sums.
//
// BCM_Flux_XYZ_Viscous_Runge_kutta.cpp:2417-2652.  Fluid cells only are
// updated; at stage 3 the L2 change norms of p, u, v, w, T over fluid cells
// and the force sums over all interior cells are formed.  The reference sums
// serially (its OpenMP accumulation at :2523 is unsynchronised); here each
// block sums a fixed contiguous range of cells in a fixed tree order and a
// single block adds the block sums in order, so the result is run-to-run
// reproducible and equal to the serial sum within rounding.
#include <cuda_runtime.h>

#include "bcm_common.cuh"
#include "bcm_kernels.h"

namespace bcmg {

constexpr int kRkThreads = 256;

__global__ void __launch_bounds__(kRkThreads) k_rk(RkArgs a, long long total, long long chunk) {
  const int n = a.ph.n, S = n + 4;
  long long beg = (long long)blockIdx.x * chunk;
  long long end = min(total, beg + chunk);
  if (a.blk_beg) {  // batches: the block's range lies inside one case
    beg = a.blk_beg[blockIdx.x];
    end = a.blk_beg[blockIdx.x + 1];
  }
  if (beg < end && !case_active(a.bt, 1 + (int)(beg / ((long long)n * n * n)))) return;
  double s[7] = {0, 0, 0, 0, 0, 0, 0};
  for (long long t = beg + threadIdx.x; t < end; t += kRkThreads) {
    const int c = 1 + (int)(t / ((long long)n * n * n));
    const int r = (int)(t % ((long long)n * n * n));
    const int i = 2 + r / (n * n), j = 2 + (r / n) % n, k = 2 + r % n;
    const size_t o = cell_index(S, c, i, j, k);
    double *q = a.U1_ + 5 * o;
    const double *rk = a.Rku1 + 5 * o;
    const bool fluid = a.FWS[o] == kFluid;
    if (a.RK == 1) {
      if (fluid) {
#pragma unroll
        for (int v = 0; v < 5; ++v) {
          double x = q[v] + rk[v];
          q[v] = x;
          a.U1p1[5 * o + v] = x;
        }
      }
    } else if (a.RK == 2) {
      if (fluid) {
#pragma unroll
        for (int v = 0; v < 5; ++v) {
          double x = 0.75 * q[v] + 0.25 * a.U1p1[5 * o + v] + 0.25 * rk[v];
          q[v] = x;
          a.U1p2[5 * o + v] = x;
        }
      }
    } else {
      if (fluid) {
        const double K = BCMG_K;
        (void)K;
        double rhoold = q[0];
        double Uold = q[1] / rhoold, Vold = q[2] / rhoold, Wold = q[3] / rhoold;
        double VVold = Uold * Uold + Vold * Vold + Wold * Wold;
        double Pold = (q[4] - 0.5 * rhoold * VVold) * (BCMG_K - 1);
        double Told = Pold / rhoold;
        double x[5];
#pragma unroll
        for (int v = 0; v < 5; ++v) {
          x[v] = 1.0 / 3.0 * q[v] + 2.0 / 3.0 * a.U1p2[5 * o + v] + 2.0 / 3.0 * rk[v];
          q[v] = x[v];
        }
        double rho = x[0];
        double U = x[1] / rho, V = x[2] / rho, W = x[3] / rho;
        double VV = U * U + V * V + W * W;
        double P = (x[4] - 0.5 * rho * VV) * (BCMG_K - 1);
        double T = P / rho;
        s[0] += (P - Pold) * (P - Pold);
        s[1] += (U - Uold) * (U - Uold);
        s[2] += (V - Vold) * (V - Vold);
        s[3] += (W - Wold) * (W - Wold);
        s[4] += (T - Told) * (T - Told);
      }
      s[5] += a.Residual1[5 * o + 0];
      s[6] += a.Residual1[5 * o + 1];
    }
  }
  if (a.RK != 3) return;
  // Fixed-shape block reduction: warp shuffles then one lane per warp.
  __shared__ double red[kRkThreads / 32][7];
#pragma unroll
  for (int m = 0; m < 7; ++m) {
    double v = s[m];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5][m] = v;
  }
  __syncthreads();
  if (threadIdx.x < 7) {
    double v = 0;
    for (int w = 0; w < kRkThreads / 32; ++w) v += red[w][threadIdx.x];
    a.partials[(size_t)blockIdx.x * 7 + threadIdx.x] = v;
  }
}

// Deterministic sum of partials[b][0..6] over blocks [b0, b1) into tot[7]
// (shared).  kNormWarps warps per quantity; lane l of warp w takes blocks
// b0 + 32 w + l, then every 32 kNormWarps-th, into four accumulators in turn
// (loads in flight), combined as (v0 + v1) + (v2 + v3); a fixed shuffle tree
// per warp and the warps' results in warp order.  The order depends only on
// b1 - b0, never on timing, so a batch's case and the same case alone sum
// identically.  Launch with 7 * kNormWarps warps.
constexpr int kNormWarps = 4;
__device__ void sum_partials(const double *partials, int b0, int b1, double *tot) {
  __shared__ double part[7][kNormWarps];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m = w / kNormWarps, sub = w % kNormWarps;
  constexpr int kStride = 32 * kNormWarps;
  if (m < 7) {
    double v0 = 0, v1 = 0, v2 = 0, v3 = 0;
    int b = b0 + sub * 32 + lane;
    for (; b + 3 * kStride < b1; b += 4 * kStride) {
      v0 += partials[(size_t)b * 7 + m];
      v1 += partials[(size_t)(b + kStride) * 7 + m];
      v2 += partials[(size_t)(b + 2 * kStride) * 7 + m];
      v3 += partials[(size_t)(b + 3 * kStride) * 7 + m];
    }
    for (; b < b1; b += kStride) v0 += partials[(size_t)b * 7 + m];
    double v = (v0 + v1) + (v2 + v3);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if (lane == 0) part[m][sub] = v;
  }
  __syncthreads();
  if (threadIdx.x < 7) {
    double t = part[threadIdx.x][0];
    for (int q = 1; q < kNormWarps; ++q) t += part[threadIdx.x][q];
    tot[threadIdx.x] = t;
  }
  __syncthreads();
}

// er[1..5] = L2 change norms / (MPI_Ncube n^3), er[6], er[7] = force sums /
// (0.5 rho0 U0^2 2.602) (BCM_Flux...cpp:2628-2650).
__device__ void write_norms(int n, int mpi_ncube, double rho0, double U0, const double *tot,
                            double *er) {
  double DN = 1. / (mpi_ncube * n * n * n);
  er[0] = 0;
  for (int m = 0; m < 5; ++m) er[1 + m] = sqrt(tot[m]) * DN;
  er[6] = tot[5] / (0.5 * rho0 * U0 * U0 * 2.602);
  er[7] = tot[6] / (0.5 * rho0 * U0 * U0 * 2.602);
}

__global__ void k_norms(Phys ph, const double *partials, int nblocks, double *er,
                        const int *active) {
  if (active && !active[0]) return;
  __shared__ double tot[7];
  sum_partials(partials, 0, nblocks, tot);
  if (threadIdx.x == 0) write_norms(ph.n, ph.mpi_ncube, ph.rho0, ph.U0, tot, er);
}

// Cube-sharded runs: the raw sums of this rank's blocks (the ranks' sums are
// then added, as the reference's MPI_Allreduce does, BCM_Flux...cpp
// :2641-2652), and the norms from the summed values.
__global__ void k_norm_sums(const double *partials, int nblocks, double *sums,
                            const int *active) {
  if (active && !active[0]) return;
  __shared__ double tot[7];
  sum_partials(partials, 0, nblocks, tot);
  if (threadIdx.x < 7) sums[threadIdx.x] = tot[threadIdx.x];
}

__global__ void k_norm_final(Phys ph, const double *sums, double *er, const int *active) {
  if (active && !active[0]) return;
  write_norms(ph.n, ph.mpi_ncube, ph.rho0, ph.U0, sums, er);
}

// One CTA per case of a batch.
__global__ void k_norms_batch(int n, const CaseConst *cases, const int *case_blk,
                              const double *partials, double *er, const int *active) {
  __shared__ double tot[7];
  const int q = blockIdx.x;
  if (active && !active[q]) return;
  sum_partials(partials, case_blk[q], case_blk[q + 1], tot);
  if (threadIdx.x == 0) {
    const CaseConst &c = cases[q];
    write_norms(n, c.mpi_ncube, c.rho0, c.U0, tot, er + 8 * (size_t)q);
  }
}

static void rk_geometry(const RkArgs &a, long long &total, long long &chunk, int &nb) {
  const long long n3 = (long long)a.ph.n * a.ph.n * a.ph.n;
  total = (long long)(a.ncube - 1) * n3;
  nb = (int)((total + 4 * kRkThreads - 1) / (4 * kRkThreads));
  if (nb > 152 * 16) nb = 152 * 16;
  if (nb < 1) nb = 1;
  chunk = (total + nb - 1) / nb;
}

int rk_partial_blocks(const RkArgs &a) {
  long long total, chunk;
  int nb;
  rk_geometry(a, total, chunk, nb);
  return nb;
}

cudaError_t launch_rk(const RkArgs &a, int *nblocks_out, cudaStream_t s) {
  long long total, chunk;
  int nb;
  rk_geometry(a, total, chunk, nb);
  if (nblocks_out) *nblocks_out = nb;
  if (total <= 0) return cudaSuccess;
  k_rk<<<nb, kRkThreads, 0, s>>>(a, total, chunk);
  return cudaGetLastError();
}

cudaError_t launch_norms(const Phys &ph, const double *partials, int nblocks, double *er,
                         cudaStream_t s, const int *active) {
  k_norms<<<1, 7 * 32 * kNormWarps, 0, s>>>(ph, partials, nblocks, er, active);
  return cudaGetLastError();
}

cudaError_t launch_norm_sums(const double *partials, int nblocks, double *sums, cudaStream_t s,
                             const int *active) {
  k_norm_sums<<<1, 7 * 32 * kNormWarps, 0, s>>>(partials, nblocks, sums, active);
  return cudaGetLastError();
}

cudaError_t launch_norm_final(const Phys &ph, const double *sums, double *er, cudaStream_t s,
                              const int *active) {
  k_norm_final<<<1, 1, 0, s>>>(ph, sums, er, active);
  return cudaGetLastError();
}

cudaError_t launch_norms_batch(int n, const CaseConst *cases, const int *case_blk, int ncase,
                               const double *partials, double *er, cudaStream_t s,
                               const int *active) {
  if (ncase <= 0) return cudaSuccess;
  k_norms_batch<<<ncase, 7 * 32 * kNormWarps, 0, s>>>(n, cases, case_blk, partials, er, active);
  return cudaGetLastError();
}

cudaError_t launch_rk_table(const RkArgs &a, int nblocks, cudaStream_t s) {
  if (nblocks <= 0 || !a.blk_beg) return cudaErrorInvalidValue;
  k_rk<<<nblocks, kRkThreads, 0, s>>>(a, 0, 0);
  return cudaGetLastError();
}

}  // namespace bcmg

namespace bcmg {

// Stage combination with a caller-chosen chunk (cells per block) and block
// count; partials must hold nblocks * 7 doubles.
cudaError_t launch_rk_chunked(const RkArgs &a, long long chunk, int nblocks, cudaStream_t s) {
  const long long n3 = (long long)a.ph.n * a.ph.n * a.ph.n;
  const long long total = (long long)(a.ncube - 1) * n3;
  if (total <= 0 || nblocks <= 0) return cudaSuccess;
  k_rk<<<nblocks, kRkThreads, 0, s>>>(a, total, chunk);
  return cudaGetLastError();
}

}  // namespace bcmg
