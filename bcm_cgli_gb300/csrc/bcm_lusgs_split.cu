// Split-precision LU-SGS sub-iteration: the sweeps in FP32, the update and
// norm sums in FP64.  Same scheme and parallel form as the FP64 kernel
// (bcm_lusgs.cu): per cube, forward and backward sweeps over the planes
// i+j+k = const, thread column (a, b) owning cells (a, b, h-a-b), the
// previous plane's increments double-buffered in shared memory.  The sweep
// is a preconditioner of the dual-time iteration (the FP32 residual it is
// fed decides the converged state), so its coefficients come from the FP32
// mirror of the state: deltas from the case's reference state (rho0, 0, 0,
// 0, P0/(K-1)), pressure p = P0 + p'.  The increment is added to the FP64
// state and the change norms are formed from the FP32 increments and summed
// in FP64, as in the split RK path.
#include <cuda_runtime.h>

#include "bcm_common.cuh"
#include "bcm_kernels.h"

namespace bcmg {

int lusgs_threads(int n);

namespace {

constexpr int kLuMaxThreads = 288;

// Cell coefficients U, V, W, VV, H, r_x, r_y, r_z, nu, dg from the FP32
// deltas m (rho' = m0, rho u = m1.., E' = m4).
__device__ __forceinline__ void luf_coef(const float *m, float rho0, float P0, float T0,
                                         float mu_L, float idx, float dT, float cfl,
                                         float omega, float *k) {
  const float rho = rho0 + m[0];
  const float ir = 1.0f / rho;
  const float U = m[1] * ir, V = m[2] * ir, W = m[3] * ir;
  const float VV = U * U + V * V + W * W;
  const float P = P0 + (m[4] - 0.5f * rho * VV) * 0.4f;
  const float c = sqrtf(1.4f * P * ir);
  const float H = (m[4] + 2.5f * P0 + P) * ir;
  const float r0 = fabsf(U) + c, r1 = fabsf(V) + c, r2 = fabsf(W) + c;
  const float T = P * ir * (1.0f / 287.0f);
  const float temp = T / T0;
  const float mu = mu_L * temp * sqrtf(temp) * (T0 + 110.f) / (T + 110.f);
  const float nu = mu * (float)(BCMG_K / BCMG_PR) * ir;
  const float rs = r0 + r1 + r2;
  float dg = 1.5f / dT + omega * rs * idx + 6.0f * nu * idx * idx;
  if (cfl > 0) dg += rs * idx / cfl;
  k[0] = U; k[1] = V; k[2] = W; k[3] = VV; k[4] = H;
  k[5] = r0; k[6] = r1; k[7] = r2; k[8] = nu; k[9] = dg;
}

template <int D, bool LOWER>
__device__ __forceinline__ void luf_off(const float *k, float idx, float omega, const float *dq,
                                        float *s) {
  const float U = k[0], V = k[1], W = k[2], VV = k[3], H = k[4];
  const float un = D == 0 ? U : (D == 1 ? V : W);
  const float dp = 0.4f * (dq[4] - (U * dq[1] + V * dq[2] + W * dq[3]) + 0.5f * VV * dq[0]);
  const float t = dq[1 + D] - un * dq[0];
  float a[5];
  a[0] = dq[1 + D];
  a[1] = un * dq[1] + U * t;
  a[2] = un * dq[2] + V * t;
  a[3] = un * dq[3] + W * t;
  a[1 + D] += dp;
  a[4] = un * (dq[4] + dp) + H * t;
  const float h = 0.5f * idx, w = omega * k[5 + D], v = k[8] * idx * idx;
#pragma unroll
  for (int m = 0; m < 5; ++m)
    s[m] += LOWER ? h * (a[m] + w * dq[m]) + v * dq[m] : h * (a[m] - w * dq[m]) - v * dq[m];
}

template <int D, bool LOWER>
__device__ __forceinline__ void addf_nb(const float *coef, size_t on, const float *dqn, float idx,
                                        float omega, float *s) {
  float kn[10];
#pragma unroll
  for (int m = 0; m < 10; ++m) kn[m] = coef[10 * on + m];  // written in this launch
  luf_off<D, LOWER>(kn, idx, omega, dqn, s);
}

__global__ void __launch_bounds__(kLuMaxThreads) k_lusgs_split(LusgsSplitArgs a) {
  extern __shared__ __align__(16) float fbuf[];  // [2][n*n][5]; later the reduction's doubles
  const int n = a.ph.n, S = n + 4, nn = n * n;
  const int cube = 1 + blockIdx.x;
  if (!case_active(a.bt, cube)) return;  // converged case
  float dT = a.dTf, mu_L = a.mu_Lf, rho0 = a.rho0f, P0 = a.P0f, T0 = a.T0f;
  if (a.bt.cube_case) {
    const CaseConst *q = a.bt.cases + a.bt.cube_case[cube];
    dT = q->dTf; mu_L = q->mu_Lf; rho0 = q->rho0f; P0 = q->P0f; T0 = q->T0f;
  }
  const float omega = a.omegaf, cfl = a.cflf;
  const float idx = a.inv_dx[cube];
  const size_t cb = cell_index(S, cube, 0, 0, 0);
  auto cell = [&](int i, int j, int k) -> size_t {
    return cb + ((size_t)(i + 2) * S + (j + 2)) * S + (k + 2);
  };
  const int *F = a.FWS;

  for (int h = 0; h <= 3 * (n - 1); ++h) {
    float *cur = fbuf + (size_t)(h & 1) * nn * 5;
    const float *prv = fbuf + (size_t)((h + 1) & 1) * nn * 5;
    for (int col = threadIdx.x; col < nn; col += blockDim.x) {
      const int ci = col / n, cj = col - (col / n) * n, ck = h - ci - cj;
      if (ck < 0 || ck >= n) continue;
      const size_t o = cell(ci, cj, ck);
      float *slot = cur + 5 * col;
      if (F[o] != kFluid) {
#pragma unroll
        for (int m = 0; m < 5; ++m) slot[m] = 0.f;
        continue;
      }
      float k[10];
      luf_coef(a.M + 5 * o, rho0, P0, T0, mu_L, idx, dT, cfl, omega, k);
#pragma unroll
      for (int m = 0; m < 10; ++m) a.coef[10 * o + m] = k[m];
      float s[5];
#pragma unroll
      for (int m = 0; m < 5; ++m) s[m] = a.R32[5 * o + m];
      if (ci > 0 && F[cell(ci - 1, cj, ck)] == kFluid)
        addf_nb<0, true>(a.coef, cell(ci - 1, cj, ck), prv + 5 * (col - n), idx, omega, s);
      if (cj > 0 && F[cell(ci, cj - 1, ck)] == kFluid)
        addf_nb<1, true>(a.coef, cell(ci, cj - 1, ck), prv + 5 * (col - 1), idx, omega, s);
      if (ck > 0 && F[cell(ci, cj, ck - 1)] == kFluid)
        addf_nb<2, true>(a.coef, cell(ci, cj, ck - 1), prv + 5 * col, idx, omega, s);
      const float idg = 1.0f / k[9];
#pragma unroll
      for (int m = 0; m < 5; ++m) {
        const float x = s[m] * idg;
        a.R32[5 * o + m] = x;
        slot[m] = x;
      }
    }
    __syncthreads();
  }

  double e[7] = {0, 0, 0, 0, 0, 0, 0};
  for (int h = 3 * (n - 1); h >= 0; --h) {
    float *cur = fbuf + (size_t)(h & 1) * nn * 5;
    const float *prv = fbuf + (size_t)((h + 1) & 1) * nn * 5;
    for (int col = threadIdx.x; col < nn; col += blockDim.x) {
      const int ci = col / n, cj = col - (col / n) * n, ck = h - ci - cj;
      if (ck < 0 || ck >= n) continue;
      const size_t o = cell(ci, cj, ck);
      float *slot = cur + 5 * col;
      e[5] += a.Residual1[5 * o + 0];
      e[6] += a.Residual1[5 * o + 1];
      if (F[o] != kFluid) {
#pragma unroll
        for (int m = 0; m < 5; ++m) slot[m] = 0.f;
        continue;
      }
      float s[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
      if (ci + 1 < n && F[cell(ci + 1, cj, ck)] == kFluid)
        addf_nb<0, false>(a.coef, cell(ci + 1, cj, ck), prv + 5 * (col + n), idx, omega, s);
      if (cj + 1 < n && F[cell(ci, cj + 1, ck)] == kFluid)
        addf_nb<1, false>(a.coef, cell(ci, cj + 1, ck), prv + 5 * (col + 1), idx, omega, s);
      if (ck + 1 < n && F[cell(ci, cj, ck + 1)] == kFluid)
        addf_nb<2, false>(a.coef, cell(ci, cj, ck + 1), prv + 5 * col, idx, omega, s);
      const float idg = 1.0f / a.coef[10 * o + 9];
      float dq[5];
#pragma unroll
      for (int m = 0; m < 5; ++m) {
        dq[m] = a.R32[5 * o + m] - s[m] * idg;
        a.R32[5 * o + m] = dq[m];
        slot[m] = dq[m];
      }
      // FP64 update; change norms of p, u, v, w, T from the FP32 increment
      // (same formulas as the split RK path's third stage).
      double *q = a.U1_ + 5 * o;
      const float *mm_ = a.M + 5 * o;
      const float rf = rho0 + mm_[0];
      const float m1 = mm_[1], m2 = mm_[2], m3 = mm_[3];
      const float Pc = P0 + (mm_[4] - 0.5f * (m1 * m1 + m2 * m2 + m3 * m3) / rf) * 0.4f;
#pragma unroll
      for (int m = 0; m < 5; ++m) q[m] = q[m] + (double)dq[m];
      const float dr = dq[0], e1 = dq[1], e2 = dq[2], e3 = dq[3], dE = dq[4];
      const float den = 1.0f / (rf * (rf + dr));
      const float dU = (e1 * rf - m1 * dr) * den;
      const float dVv = (e2 * rf - m2 * dr) * den;
      const float dW = (e3 * rf - m3 * dr) * den;
      const float mm = m1 * m1 + m2 * m2 + m3 * m3;
      const float dKE =
          0.5f * ((2.f * (m1 * e1 + m2 * e2 + m3 * e3) + e1 * e1 + e2 * e2 + e3 * e3) * rf - mm * dr) * den;
      const float dP = 0.4f * (dE - dKE);
      const float dTt = (dP * rf - Pc * dr) * den;
      e[0] += (double)(dP * dP);
      e[1] += (double)(dU * dU);
      e[2] += (double)(dVv * dVv);
      e[3] += (double)(dW * dW);
      e[4] += (double)(dTt * dTt);
    }
    __syncthreads();
  }

  double *red = reinterpret_cast<double *>(fbuf);  // [warps][7]
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

cudaError_t launch_lusgs_split(const LusgsSplitArgs &a, int ncubes, cudaStream_t s) {
  if (ncubes <= 0) return cudaSuccess;
  const int n = a.ph.n;
  const int threads = lusgs_threads(n);
  size_t smem = (size_t)2 * n * n * 5 * sizeof(float);
  const size_t red = (size_t)(threads / 32) * 7 * sizeof(double);
  if (smem < red) smem = red;
  cudaError_t e = cudaFuncSetAttribute(k_lusgs_split,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k_lusgs_split<<<ncubes, threads, smem, s>>>(a);
  return cudaGetLastError();
}

}  // namespace bcmg
