// Split-precision LU-SGS sub-iteration: the sweeps in FP32, the update and
// norm sums in FP64.  Same scheme and parallel form as the FP64 kernel
// (bcm_lusgs.cu): per cube, forward and backward sweeps over the planes
// i+j+k = const, the previous plane's values double-buffered in shared memory.  The cube's
// inputs are first packed into a scratch in plane order, so the cells of a
// plane are consecutive: they go to consecutive threads (full warps) and the
// sequential sweeps read and write consecutive words; the update runs
// afterwards slab by slab in memory order.  The sweep
// is a preconditioner of the dual-time iteration (the FP32 residual it is
// fed decides the converged state), so its coefficients come from the FP32
// mirror of the state: deltas from the case's reference state (rho0, 0, 0,
// 0, P0/(K-1)), pressure p = P0 + p'.  The increment is added to the FP64
// state and the change norms are formed from the FP32 increments and summed
// in FP64, as in the split RK path.
#include <cuda_runtime.h>

#include <atomic>

#include "bcm_common.cuh"
#include "bcm_kernels.h"

namespace bcmg {

namespace {

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

// Per-cube scratch in plane order: the cells of plane h = i+j+k, i then j
// ascending, at positions pos = P[h] + Q[h][i] + (j - jlo(h, i)), one array
// per value (mirror 0..4, residual / increment 5..9, fluid flag 10).  The
// threads of a sweep plane (consecutive columns) and of a packing pass
// (consecutive cells of a slab's anti-diagonal) touch consecutive words, so
// every global access of the kernel is coalesced.
constexpr int kScr = 11;
// Shared slots of the previous plane, value-major [kSlot][n*n]: coefficients
// 0..9, increment 10..14, fluid flag 15.
constexpr int kSlot = 16;

__device__ __forceinline__ int jlo_of(int h, int i, int n) {
  const int x = h - i - (n - 1);
  return x > 0 ? x : 0;
}

template <int MAXT>
__global__ void __launch_bounds__(MAXT, MAXT <= 448 ? 2 : 1) k_lusgs_split(LusgsSplitArgs a) {
  extern __shared__ __align__(16) float fbuf[];
  const int n = a.ph.n, S = n + 4, nn = n * n, n3 = nn * n, np = 3 * n - 2;
  const int cube = 1 + blockIdx.x;
  if (!case_active(a.bt, cube)) return;  // converged case
  float dT = a.dTf, mu_L = a.mu_Lf, rho0 = a.rho0f, P0 = a.P0f, T0 = a.T0f;
  double rho0d = a.mir.rho0, E0d = a.mir.E0;  // mirror reference state (FP64)
  if (a.bt.cube_case) {
    const CaseConst *q = a.bt.cases + a.bt.cube_case[cube];
    dT = q->dTf; mu_L = q->mu_Lf; rho0 = q->rho0f; P0 = q->P0f; T0 = q->T0f;
    rho0d = q->rho0; E0d = q->E0;
  }
  // The mirror of the state, read by the pack and updated in place with the
  // state: this block reads only its own cube's interior cells of it, and
  // writes those and (same-level pushes) other cubes' ghost cells, which no
  // block of this launch reads.
  float *const Mc = mirror_current(a.mir);
  const float omega = a.omegaf, cfl = a.cflf;
  const float idx = a.inv_dx[cube];
  const size_t cb = cell_index(S, cube, 0, 0, 0);
  float *scr = a.scr + (size_t)blockIdx.x * kScr * n3;

  // Shared memory: slots (also the slab staging area), then the tables.
  float *slots = fbuf;                                   // [2][kSlot][nn]
  int *Pt = reinterpret_cast<int *>(fbuf + 2 * kSlot * nn);  // [np + 1]
  int *Qt = Pt + np + 1;                                 // [np][n]
  int *At = Qt + np * n;                                 // [2n] anti-diagonal starts
  int *sorder = At + 2 * n;                              // [nn] slab cells by anti-diagonal
  unsigned short *dec = reinterpret_cast<unsigned short *>(sorder + nn);  // [n3] column of a position
  const int tid = threadIdx.x, NT = blockDim.x;
  for (int h = tid; h < np; h += NT) {
    const int ilo = h - 2 * (n - 1) > 0 ? h - 2 * (n - 1) : 0, ihi = h < n - 1 ? h : n - 1;
    int acc = 0;
    for (int i = 0; i < n; ++i) {
      Qt[h * n + i] = acc;
      if (i >= ilo && i <= ihi) acc += (h - i < n - 1 ? h - i : n - 1) - jlo_of(h, i, n) + 1;
    }
  }
  if (tid == 0) {
    int acc = 0;
    for (int h = 0; h < np; ++h) {
      Pt[h] = acc;
      const int ilo = h - 2 * (n - 1) > 0 ? h - 2 * (n - 1) : 0, ihi = h < n - 1 ? h : n - 1;
      for (int i = ilo; i <= ihi; ++i)
        acc += (h - i < n - 1 ? h - i : n - 1) - jlo_of(h, i, n) + 1;
    }
    Pt[np] = acc;
    int d0 = 0;
    for (int d = 0; d <= 2 * n - 2; ++d) {
      At[d] = d0;
      d0 += (d < 2 * n - 2 - d ? d : 2 * n - 2 - d) + 1;
    }
  }
  __syncthreads();
  for (int jk = tid; jk < nn; jk += NT) {
    const int j = jk / n, k = jk - j * n, d = j + k;
    sorder[At[d] + j - (d - (n - 1) > 0 ? d - (n - 1) : 0)] = jk;
  }
  auto pos = [&](int h, int i, int j) { return Pt[h] + Qt[h * n + i] + (j - jlo_of(h, i, n)); };
  auto SV = [&](int v, int p) -> float & { return scr[(size_t)v * n3 + p]; };
  __syncthreads();
  for (int c = tid; c < n3; c += NT) {
    const int i = c / nn, j = (c / n) % n, k = c % n;
    dec[pos(i + j + k, i, j)] = (unsigned short)(i * n + j);
  }
  __syncthreads();

  // Pack, slab by slab (i fixed): coalesced loads in memory order into
  // shared memory, coalesced stores in plane order.
  float *stage = slots;  // [kScr][nn]
  for (int i = 0; i < n; ++i) {
    for (int jk = tid; jk < nn; jk += NT) {
      const int j = jk / n, k = jk - j * n;
      const size_t o = cb + ((size_t)(i + 2) * S + (j + 2)) * S + (k + 2);
#pragma unroll
      for (int v = 0; v < 5; ++v) {
        stage[v * nn + jk] = Mc[5 * o + v];
        stage[(5 + v) * nn + jk] = a.R32[5 * o + v];
      }
      stage[10 * nn + jk] = a.FWS[o] == kFluid ? 1.f : 0.f;
    }
    __syncthreads();
    for (int t = tid; t < nn; t += NT) {
      const int jk = sorder[t], j = jk / n, k = jk - j * n;
      const int p = pos(i + j + k, i, j);
#pragma unroll
      for (int v = 0; v < kScr; ++v) SV(v, p) = stage[v * nn + jk];
    }
    __syncthreads();
  }

  // Sweeps: the cells of plane h (positions Pt[h] .. Pt[h+1]) go to
  // consecutive threads, so every active warp is full; each cell finds its
  // neighbours' previous-plane values in the shared slot of their column.
  auto nb = [&](const float *prv, int c, float *kk, float *dd) {
#pragma unroll
    for (int v = 0; v < 10; ++v) kk[v] = prv[v * nn + c];
#pragma unroll
    for (int v = 0; v < 5; ++v) dd[v] = prv[(10 + v) * nn + c];
  };
  float m[5], r[5], fl = 0.f;     // this plane's cell
  float m2[5], r2[5], fl2 = 0.f;  // the next plane's, loaded a plane ahead
  auto fetch = [&](int pp) {
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      m[v] = SV(v, pp);
      r[v] = SV(5 + v, pp);
    }
    fl = SV(10, pp);
  };
  auto fetch2 = [&](int pp) {
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      m2[v] = SV(v, pp);
      r2[v] = SV(5 + v, pp);
    }
    fl2 = SV(10, pp);
  };
  auto take2 = [&]() {
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      m[v] = m2[v];
      r[v] = r2[v];
    }
    fl = fl2;
  };

  // Forward sweep: dq* = (R + sum of lower A+ terms) / dg.
  if (tid < Pt[1] - Pt[0]) fetch2(Pt[0] + tid);
  for (int h = 0; h < np; ++h) {
    float *cur = slots + (size_t)(h & 1) * kSlot * nn;
    const float *prv = slots + (size_t)((h + 1) & 1) * kSlot * nn;
    const int cnt = Pt[h + 1] - Pt[h];
    take2();
    if (h + 1 < np && tid < Pt[h + 2] - Pt[h + 1]) fetch2(Pt[h + 1] + tid);  // next plane
    for (int t = tid; t < cnt; t += NT) {
      const int pp = Pt[h] + t;
      if (t != tid) fetch(pp);  // further cells of a wide plane
      const int col = dec[pp], ci = col / n, cj = col - ci * n, k = h - ci - cj;
      cur[15 * nn + col] = fl;
      if (fl != 0.f) {
        float kc[10], kk[10], dd[5];
        luf_coef(m, rho0, P0, T0, mu_L, idx, dT, cfl, omega, kc);
        if (ci > 0 && prv[15 * nn + col - n] != 0.f) {
          nb(prv, col - n, kk, dd);
          luf_off<0, true>(kk, idx, omega, dd, r);
        }
        if (cj > 0 && prv[15 * nn + col - 1] != 0.f) {
          nb(prv, col - 1, kk, dd);
          luf_off<1, true>(kk, idx, omega, dd, r);
        }
        if (k > 0 && prv[15 * nn + col] != 0.f) {  // the column's previous cell
          nb(prv, col, kk, dd);
          luf_off<2, true>(kk, idx, omega, dd, r);
        }
        const float idg = 1.0f / kc[9];
#pragma unroll
        for (int v = 0; v < 5; ++v) {
          const float x = r[v] * idg;
          SV(5 + v, pp) = x;
          cur[(10 + v) * nn + col] = x;
        }
#pragma unroll
        for (int v = 0; v < 10; ++v) cur[v * nn + col] = kc[v];
      }
    }
    __syncthreads();
  }

  // Backward sweep: dq = dq* - (sum of upper A- terms) / dg.
  if (tid < Pt[np] - Pt[np - 1]) fetch2(Pt[np - 1] + tid);
  for (int h = np - 1; h >= 0; --h) {
    float *cur = slots + (size_t)(h & 1) * kSlot * nn;
    const float *prv = slots + (size_t)((h + 1) & 1) * kSlot * nn;
    const int cnt = Pt[h + 1] - Pt[h];
    take2();
    if (h > 0 && tid < Pt[h] - Pt[h - 1]) fetch2(Pt[h - 1] + tid);
    for (int t = tid; t < cnt; t += NT) {
      const int pp = Pt[h] + t;
      if (t != tid) fetch(pp);
      const int col = dec[pp], ci = col / n, cj = col - ci * n, k = h - ci - cj;
      cur[15 * nn + col] = fl;
      if (fl != 0.f) {
        float kc[10], kk[10], dd[5], s[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
        luf_coef(m, rho0, P0, T0, mu_L, idx, dT, cfl, omega, kc);
        if (ci + 1 < n && prv[15 * nn + col + n] != 0.f) {
          nb(prv, col + n, kk, dd);
          luf_off<0, false>(kk, idx, omega, dd, s);
        }
        if (cj + 1 < n && prv[15 * nn + col + 1] != 0.f) {
          nb(prv, col + 1, kk, dd);
          luf_off<1, false>(kk, idx, omega, dd, s);
        }
        if (k + 1 < n && prv[15 * nn + col] != 0.f) {
          nb(prv, col, kk, dd);
          luf_off<2, false>(kk, idx, omega, dd, s);
        }
        const float idg = 1.0f / kc[9];
#pragma unroll
        for (int v = 0; v < 5; ++v) {
          const float x = r[v] - s[v] * idg;
          SV(5 + v, pp) = x;
          cur[(10 + v) * nn + col] = x;
        }
#pragma unroll
        for (int v = 0; v < 10; ++v) cur[v * nn + col] = kc[v];
      }
    }
    __syncthreads();
  }

  // Update, slab by slab: increments gathered in plane order (coalesced)
  // into shared memory, then Q += dq on fluid cells in memory order (FP64),
  // change norms of p, u, v, w, T from the FP32 increment (the split RK
  // path's third-stage formulas) and the force integrands of every cell.
  double e[7] = {0, 0, 0, 0, 0, 0, 0};
  for (int i = 0; i < n; ++i) {
    for (int t = tid; t < nn; t += NT) {
      const int jk = sorder[t], j = jk / n, k = jk - j * n;
      const int pp = pos(i + j + k, i, j);
#pragma unroll
      for (int v = 0; v < 5; ++v) stage[v * nn + jk] = SV(5 + v, pp);
    }
    __syncthreads();
    for (int jk = tid; jk < nn; jk += NT) {
      const int j = jk / n, k = jk - j * n;
      const size_t o = cb + ((size_t)(i + 2) * S + (j + 2)) * S + (k + 2);
      e[5] += a.Residual1[5 * o + 0];
      e[6] += a.Residual1[5 * o + 1];
      if (a.FWS[o] != kFluid) continue;
      float dq[5];
#pragma unroll
      for (int v = 0; v < 5; ++v) dq[v] = stage[v * nn + jk];
      float *mm_ = Mc + 5 * o;
      const float rf = rho0 + mm_[0];
      const float m1 = mm_[1], m2 = mm_[2], m3 = mm_[3];
      const float mm = m1 * m1 + m2 * m2 + m3 * m3;
      const float Pc = P0 + (mm_[4] - 0.5f * mm / rf) * 0.4f;
      double un[5];
      float mn[5];
#pragma unroll
      for (int v = 0; v < 5; ++v) {
        un[v] = a.U1_[5 * o + v] + (double)dq[v];
        a.U1_[5 * o + v] = un[v];
        mn[v] = mirror_value_hw(un[v], v, rho0d, E0d);
        mm_[v] = mn[v];
      }
      // Same-level interface copy of this cell (state and mirror), done
      // here: no block reads another cube's cells during the sweep.
      if (a.push) {
        push_same_level(a.U1_, a.push, n, cube, i + 2, j + 2, k + 2, un);
        push_same_level(Mc, a.push, n, cube, i + 2, j + 2, k + 2, mn);
      }
      const float dr = dq[0], e1 = dq[1], e2 = dq[2], e3 = dq[3], dE = dq[4];
      const float den = 1.0f / (rf * (rf + dr));
      const float dU = (e1 * rf - m1 * dr) * den;
      const float dVv = (e2 * rf - m2 * dr) * den;
      const float dW = (e3 * rf - m3 * dr) * den;
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
  const int nw = (NT + 31) / 32;
#pragma unroll
  for (int v = 0; v < 7; ++v) {
    double x = e[v];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) x += __shfl_down_sync(0xffffffffu, x, off);
    if ((tid & 31) == 0) red[(tid >> 5) * 7 + v] = x;
  }
  __syncthreads();
  if (tid < 7) {
    double x = 0;
    for (int w = 0; w < nw; ++w) x += red[w * 7 + tid];
    a.partials[(size_t)blockIdx.x * 7 + tid] = x;
  }
}

}  // namespace

size_t lusgs_split_scratch(int n) { return (size_t)kScr * n * n * n; }

// Threads of the split LU-SGS kernel: the widest plane of a cube, in whole
// warps (every plane then takes one pass).
static int lusgs_split_threads(int n) {
  int mx = 0;
  for (int h = 0; h <= 3 * n - 3; ++h) {
    int c = 0;
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        const int k = h - i - j;
        c += k >= 0 && k < n;
      }
    mx = c > mx ? c : mx;
  }
  return (mx + 31) / 32 * 32;
}

int lusgs_split_default_threads(int n) { return lusgs_split_threads(n); }

cudaError_t launch_lusgs_split(const LusgsSplitArgs &a, int ncubes, cudaStream_t s) {
  if (ncubes <= 0) return cudaSuccess;
  const int n = a.ph.n;
  if (n * n > 1024) return cudaErrorInvalidValue;  // columns are 16-bit shared indices
  static std::atomic<int> cache[33];  // widest plane per n (0: not yet computed)
  int threads = cache[n].load(std::memory_order_relaxed);
  if (threads == 0) {
    threads = lusgs_split_threads(n);
    cache[n].store(threads, std::memory_order_relaxed);
  }
  if (a.threads > 0) {
    if (a.threads % 32 != 0 || a.threads > threads) return cudaErrorInvalidValue;
    threads = a.threads;  // fewer threads: wide planes take several passes
  }
  const int np = 3 * n - 2;
  size_t smem = (size_t)2 * n * n * kSlot * sizeof(float) +
                (size_t)(np + 1 + np * n + 2 * n + n * n) * sizeof(int) +
                (size_t)n * n * n * sizeof(unsigned short);
  const size_t red = (size_t)(threads / 32) * 7 * sizeof(double);
  if (smem < red) smem = red;
  cudaError_t e;
  if (threads <= 448) {
    e = cudaFuncSetAttribute(k_lusgs_split<448>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
    if (e != cudaSuccess) return e;
    k_lusgs_split<448><<<ncubes, threads, smem, s>>>(a);
  } else {
    e = cudaFuncSetAttribute(k_lusgs_split<1024>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
    if (e != cudaSuccess) return e;
    k_lusgs_split<1024><<<ncubes, threads, smem, s>>>(a);
  }
  return cudaGetLastError();
}

}  // namespace bcmg
