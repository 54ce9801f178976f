// LU-SGS dual-time sub-iteration (FP64).  No counterpart in the reference:
// BCM_LUSGS.h only re-declares an older BCM_Interface.  The scheme is a
// matrix-free lower-upper symmetric Gauss-Seidel step for the same discrete
// residual as the RK path (BDF2 source + inviscid + viscous), with the
// Jameson-Turkel split Jacobians A+- = (A +- omega r I)/2 (r = |u_d| + c), a
// scalar viscous term nu = mu K/(Pr rho) and an optional local pseudo-time
// term (cfl > 0).  Per cube, cube faces and non-fluid cells carry no
// increment (block Jacobi across cubes, like the interface treats cubes).
//
// Parallel form.  A cell's forward value needs only its three lower
// neighbours (i-1, j-1, k-1) and its backward value only its three upper
// neighbours, so every plane i+j+k = h of a cube is independent.  One CTA per
// cube walks the planes in order; thread column (a, b) owns the cells
// (a, b, h-a-b), so consecutive planes hand each column its own previous
// cell and the two neighbouring columns' cells of the previous plane.  The
// increments of the previous plane sit in a double-buffered shared array
// [2][n*n][5]; the per-cell coefficients formed in the forward sweep are kept
// in global scratch for the backward sweep.  Every cell's arithmetic is the
// same as the serial lexicographic sweep's, so the result is bit-identical
// to it (built with --fmad=false; IEEE division and square root).
//
// The backward sweep applies Q += dq on its cells as it finishes them (no
// other thread reads Q during the sweep: neighbours' coefficients come from
// the scratch) and sums the change norms of p, u, v, w, T and the force
// integrands per cube, like the RK path's third stage
// (BCM_Flux_XYZ_Viscous_Runge_kutta.cpp:2530-2650).
#include <cuda_runtime.h>

#include "bcm_common.cuh"
#include "bcm_kernels.h"

namespace bcmg {

namespace {

constexpr int kLuMaxThreads = 288;

// Cell coefficients: U, V, W, VV, H, r_x, r_y, r_z, nu, dg.
__device__ __forceinline__ void lu_coef(const double *q, double dx, double mu_L, double T0,
                                        double dT, double cfl, double omega, double *k) {
  const double rho = q[0];
  const double U = q[1] / rho, V = q[2] / rho, W = q[3] / rho;
  const double VV = U * U + V * V + W * W;
  const double P = (q[4] - 0.5 * rho * VV) * (BCMG_K - 1);
  const double c = sqrt(BCMG_K * P / rho);
  const double H = (q[4] + P) / rho;
  const double r0 = fabs(U) + c, r1 = fabs(V) + c, r2 = fabs(W) + c;
  const double T = P / rho / BCMG_R;
  const double temp = T / T0;
  const double mu = mu_L * temp * sqrt(temp) * (T0 + 110.) / (T + 110.);
  const double nu = mu * (BCMG_K / BCMG_PR) / rho;
  const double rs = r0 + r1 + r2;
  double dg = 1.5 / dT + omega * rs / dx + 6.0 * nu / (dx * dx);
  if (cfl > 0) dg = dg + rs / (cfl * dx);
  k[0] = U; k[1] = V; k[2] = W; k[3] = VV; k[4] = H;
  k[5] = r0; k[6] = r1; k[7] = r2; k[8] = nu; k[9] = dg;
}

// Split off-diagonal term of a neighbour (coefficients k, increment dq)
// across a face of direction D; LOWER: the A+ part (forward sweep), else A-.
template <int D, bool LOWER>
__device__ __forceinline__ void lu_off(const double *k, double dx, double omega, const double *dq,
                                       double *out) {
  const double U = k[0], V = k[1], W = k[2], VV = k[3], H = k[4];
  const double un = D == 0 ? U : (D == 1 ? V : W);
  const double dp = (BCMG_K - 1) * (dq[4] - (U * dq[1] + V * dq[2] + W * dq[3]) + 0.5 * VV * dq[0]);
  const double t = dq[1 + D] - un * dq[0];
  double a[5];
  a[0] = dq[1 + D];
  a[1] = un * dq[1] + U * t;
  a[2] = un * dq[2] + V * t;
  a[3] = un * dq[3] + W * t;
  a[1 + D] = a[1 + D] + dp;
  a[4] = un * (dq[4] + dp) + H * t;
  const double h = 0.5 / dx, w = omega * k[5 + D], v = k[8] / (dx * dx);
#pragma unroll
  for (int m = 0; m < 5; ++m)
    out[m] = LOWER ? h * (a[m] + w * dq[m]) + v * dq[m] : h * (a[m] - w * dq[m]) - v * dq[m];
}

// Coefficients of cell o: 5 in coefA, 5 in coefB (the RK path's U1p1 / U1p2
// buffers, unused by this method).
__device__ __forceinline__ void coef_store(const LusgsArgs &a, size_t o, const double *k) {
#pragma unroll
  for (int m = 0; m < 5; ++m) {
    a.coefA[5 * o + m] = k[m];
    a.coefB[5 * o + m] = k[5 + m];
  }
}
__device__ __forceinline__ void coef_load(const LusgsArgs &a, size_t o, double *k) {
#pragma unroll
  for (int m = 0; m < 5; ++m) {
    k[m] = a.coefA[5 * o + m];  // written earlier in this launch: plain loads
    k[5 + m] = a.coefB[5 * o + m];
  }
}

template <int D, bool LOWER>
__device__ __forceinline__ void add_nb(const LusgsArgs &a, size_t on, const double *dqn,
                                       double dx, double omega, double *s) {
  double kn[10], t[5];
  coef_load(a, on, kn);
  lu_off<D, LOWER>(kn, dx, omega, dqn, t);
#pragma unroll
  for (int m = 0; m < 5; ++m) s[m] = s[m] + t[m];
}

__global__ void __launch_bounds__(kLuMaxThreads) k_lusgs(LusgsArgs a) {
  extern __shared__ double buf[];  // [2][n*n][5] increments of the previous plane
  const int n = a.ph.n, S = n + 4, nn = n * n;
  const int cube = 1 + blockIdx.x;
  if (!case_active(a.bt, cube)) return;  // converged case
  double dT = a.dT, mu_L = a.ph.mu_L, rho0 = a.ph.rho0, P0 = a.ph.P0;
  if (a.bt.cube_case) {
    const CaseConst *q = a.bt.cases + a.bt.cube_case[cube];
    dT = q->dT; mu_L = q->mu_L; rho0 = q->rho0; P0 = q->P0;
  }
  const double T0 = P0 / rho0 / BCMG_R;
  const double omega = a.omega, cfl = a.cfl;
  const double dx = a.cube_size[cube] / n;
  const size_t cb = cell_index(S, cube, 0, 0, 0);
  auto cell = [&](int i, int j, int k) -> size_t {
    return cb + ((size_t)(i + 2) * S + (j + 2)) * S + (k + 2);
  };
  const int *F = a.FWS;

  // Forward sweep: dq* = (R + sum of lower A+ terms) / dg.
  for (int h = 0; h <= 3 * (n - 1); ++h) {
    double *cur = buf + (size_t)(h & 1) * nn * 5;
    const double *prv = buf + (size_t)((h + 1) & 1) * nn * 5;
    for (int col = threadIdx.x; col < nn; col += blockDim.x) {
      const int ci = col / n, cj = col - (col / n) * n, ck = h - ci - cj;
      if (ck < 0 || ck >= n) continue;
      const size_t o = cell(ci, cj, ck);
      double *slot = cur + 5 * col;
      if (F[o] != kFluid) {
#pragma unroll
        for (int m = 0; m < 5; ++m) slot[m] = 0;
        continue;
      }
      double k[10];
      lu_coef(a.U1_ + 5 * o, dx, mu_L, T0, dT, cfl, omega, k);
      coef_store(a, o, k);
      double s[5];
#pragma unroll
      for (int m = 0; m < 5; ++m) s[m] = a.Rku1[5 * o + m];
      if (ci > 0) {
        const size_t on = cell(ci - 1, cj, ck);
        if (F[on] == kFluid) add_nb<0, true>(a, on, prv + 5 * (col - n), dx, omega, s);
      }
      if (cj > 0) {
        const size_t on = cell(ci, cj - 1, ck);
        if (F[on] == kFluid) add_nb<1, true>(a, on, prv + 5 * (col - 1), dx, omega, s);
      }
      if (ck > 0) {
        const size_t on = cell(ci, cj, ck - 1);
        if (F[on] == kFluid) add_nb<2, true>(a, on, prv + 5 * col, dx, omega, s);
      }
#pragma unroll
      for (int m = 0; m < 5; ++m) {
        const double x = s[m] / k[9];
        a.Rku1[5 * o + m] = x;
        slot[m] = x;
      }
    }
    __syncthreads();
  }

  // Backward sweep: dq = dq* - (sum of upper A- terms) / dg, then the update.
  double e[7] = {0, 0, 0, 0, 0, 0, 0};
  for (int h = 3 * (n - 1); h >= 0; --h) {
    double *cur = buf + (size_t)(h & 1) * nn * 5;
    const double *prv = buf + (size_t)((h + 1) & 1) * nn * 5;
    for (int col = threadIdx.x; col < nn; col += blockDim.x) {
      const int ci = col / n, cj = col - (col / n) * n, ck = h - ci - cj;
      if (ck < 0 || ck >= n) continue;
      const size_t o = cell(ci, cj, ck);
      double *slot = cur + 5 * col;
      e[5] += a.Residual1[5 * o + 0];
      e[6] += a.Residual1[5 * o + 1];
      if (F[o] != kFluid) {
#pragma unroll
        for (int m = 0; m < 5; ++m) slot[m] = 0;
        continue;
      }
      double s[5] = {0, 0, 0, 0, 0};
      if (ci + 1 < n) {
        const size_t on = cell(ci + 1, cj, ck);
        if (F[on] == kFluid) add_nb<0, false>(a, on, prv + 5 * (col + n), dx, omega, s);
      }
      if (cj + 1 < n) {
        const size_t on = cell(ci, cj + 1, ck);
        if (F[on] == kFluid) add_nb<1, false>(a, on, prv + 5 * (col + 1), dx, omega, s);
      }
      if (ck + 1 < n) {
        const size_t on = cell(ci, cj, ck + 1);
        if (F[on] == kFluid) add_nb<2, false>(a, on, prv + 5 * col, dx, omega, s);
      }
      const double dg = a.coefB[5 * o + 4];
      double dq[5];
#pragma unroll
      for (int m = 0; m < 5; ++m) {
        dq[m] = a.Rku1[5 * o + m] - s[m] / dg;
        a.Rku1[5 * o + m] = dq[m];
        slot[m] = dq[m];
      }
      double *q = a.U1_ + 5 * o;
      const double rhoold = q[0];
      const double Uold = q[1] / rhoold, Vold = q[2] / rhoold, Wold = q[3] / rhoold;
      const double VVold = Uold * Uold + Vold * Vold + Wold * Wold;
      const double Pold = (q[4] - 0.5 * rhoold * VVold) * (BCMG_K - 1);
      const double Told = Pold / rhoold;
      double x[5];
#pragma unroll
      for (int m = 0; m < 5; ++m) {
        x[m] = q[m] + dq[m];
        q[m] = x[m];
      }
      const double rho = x[0];
      const double U = x[1] / rho, V = x[2] / rho, W = x[3] / rho;
      const double VV = U * U + V * V + W * W;
      const double P = (x[4] - 0.5 * rho * VV) * (BCMG_K - 1);
      const double T = P / rho;
      e[0] += (P - Pold) * (P - Pold);
      e[1] += (U - Uold) * (U - Uold);
      e[2] += (V - Vold) * (V - Vold);
      e[3] += (W - Wold) * (W - Wold);
      e[4] += (T - Told) * (T - Told);
    }
    __syncthreads();
  }

  // Per-cube partial sums (warp shuffles, then one lane per warp in order).
  double *red = buf;  // reused: [warps][7]
  const int nw = (blockDim.x + 31) / 32;
#pragma unroll
  for (int m = 0; m < 7; ++m) {
    double v = e[m];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if ((threadIdx.x & 31) == 0) red[(threadIdx.x >> 5) * 7 + m] = v;
  }
  __syncthreads();
  if (threadIdx.x < 7) {
    double v = 0;
    for (int w = 0; w < nw; ++w) v += red[w * 7 + threadIdx.x];
    a.partials[(size_t)blockIdx.x * 7 + threadIdx.x] = v;
  }
}

}  // namespace

int lusgs_threads(int n) {
  const int nn = n * n;
  const int t = (nn + 31) / 32 * 32;
  return t < kLuMaxThreads ? t : kLuMaxThreads;
}

cudaError_t launch_lusgs(const LusgsArgs &a, int ncubes, cudaStream_t s) {
  if (ncubes <= 0) return cudaSuccess;
  const int n = a.ph.n;
  const size_t smem = (size_t)2 * n * n * 5 * sizeof(double);
  const int threads = lusgs_threads(n);
  // the reduction reuses the buffer: needs threads/32 * 7 doubles
  if (smem < (size_t)(threads / 32) * 7 * sizeof(double)) return cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute(k_lusgs, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  k_lusgs<<<ncubes, threads, smem, s>>>(a);
  return cudaGetLastError();
}

}  // namespace bcmg
