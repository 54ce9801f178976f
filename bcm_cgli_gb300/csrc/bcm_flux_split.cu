// Split-precision residual, preconditioned increment and stage update, fused.
//
// Same operator as BCM_Flux_XYZ_Viscous_Runge_kutta (BCM_Flux_XYZ_Viscous_
// Runge_kutta.cpp:326-2652) with the arithmetic split by where precision is
// needed:
//  * FP64: the conservative state Q (HBM), the time-level differences
//    Q - Q^n and Q^n - Q^(n-1) of the BDF2 source (the cancellation in
//    3Q - 4Q^n + Q^(n-1)), the state update Q += w * dQ, and the sums of the
//    residual/force norms;
//  * FP32: reconstruction, the preconditioned Roe flux, viscous gradients and
//    stresses, the residual sum and the pointwise 5x5 preconditioner.
// FP32 works on deltas from a per-case reference state (rho0, 0, 0, 0,
// P0/(K-1)) formed in FP64 (k_mirror), so pressure jumps are p' = p - P0
// differences and temperatures T' = T - T0 are O(1) numbers instead of
// 1e5 Pa / 300 K values whose FP32 rounding would swamp the low-Mach jumps.
// The constant P0 cancels exactly in every face-flux difference, so the
// momentum and force terms use p'.  The preconditioner's
// temp3 = H - H*K - VV + K*(T+VV) is formed as its exact identity
// 0.5*(K-1)*VV (C = K*T), avoiding a 1e5-scale cancellation in FP32.
#include <cuda_runtime.h>

#include "bcm_common.cuh"
#include "bcm_kernels.h"

namespace bcmg {

// ---------------------------------------------------------------------------
// FP64 -> FP32 deltas of the state, all cells of all cubes (ghosts included),
// into one or both mirror buffers: once per dual-time step, and whenever the
// state was set from outside.  16-byte loads and 8-byte stores (a cube holds
// S^3 cells, S even, so cells pair up within a cube); 32-bit indices within a
// cube.  The conversions (to_float_rn, delta_rn) are the integer-pipe IEEE
// roundings of bcm_mirror.cuh, which every other mirror writer uses too.
// ---------------------------------------------------------------------------
// One block row per cube (blockIdx.y); a thread converts two cells, i.e.
// five 16-byte pairs whose components are known at compile time, so only
// the density and energy components take an FP64 subtraction.
__global__ void __launch_bounds__(256) k_mirror(const double2 *__restrict__ U,
                                                float2 *__restrict__ M, float2 *__restrict__ M1,
                                                double rho0_, double E0_, Batch bt,
                                                int cube_cell_pairs, int ncubes) {
  for (int cube = 1 + blockIdx.y; cube <= ncubes; cube += gridDim.y) {
    double rho0 = rho0_, E0 = E0_;
    if (bt.cube_case) {  // the reference state of the cube's case
      const CaseConst *cq = bt.cases + bt.cube_case[cube];
      rho0 = cq->rho0;
      E0 = cq->E0;
    }
    const size_t base = (size_t)cube * cube_cell_pairs * 5;  // in 16-byte pairs
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      const int q = (blockIdx.x * 2 + r) * 256 + threadIdx.x;  // cell pair in the cube
      if (q < cube_cell_pairs) {
        const double2 *u = U + base + 5 * (size_t)q;
        const double2 a = u[0], b = u[1], c = u[2], d = u[3], e = u[4];
        // doubles: rho, mx, my, mz, E | rho, mx, my, mz, E
        const float2 m0 = make_float2(delta_rn(a.x, rho0), to_float_rn(a.y));
        const float2 m1 = make_float2(to_float_rn(b.x), to_float_rn(b.y));
        const float2 m2 = make_float2(delta_rn(c.x, E0), delta_rn(c.y, rho0));
        const float2 m3 = make_float2(to_float_rn(d.x), to_float_rn(d.y));
        const float2 m4 = make_float2(to_float_rn(e.x), delta_rn(e.y, E0));
        float2 *m = M + base + 5 * (size_t)q;
        m[0] = m0; m[1] = m1; m[2] = m2; m[3] = m3; m[4] = m4;
        if (M1) {
          float2 *o = M1 + base + 5 * (size_t)q;
          o[0] = m0; o[1] = m1; o[2] = m2; o[3] = m3; o[4] = m4;
        }
      }
    }
  }
}

cudaError_t launch_mirror(const double *U, float *M0, float *M1, int n, int ncube, double rho0,
                          double P0, const Batch &bt, cudaStream_t s) {
  if (ncube <= 1) return cudaSuccess;  // cube slot 0 is unused
  const int S = n + 4;
  const int cube_cell_pairs = S * S * S / 2;  // S is even
  const dim3 grid((cube_cell_pairs + 511) / 512, ncube - 1 < 65535 ? ncube - 1 : 65535);
  k_mirror<<<grid, 256, 0, s>>>(reinterpret_cast<const double2 *>(U),
                               reinterpret_cast<float2 *>(M0), reinterpret_cast<float2 *>(M1),
                               rho0, P0 / (BCMG_K - 1), bt, cube_cell_pairs, ncube - 1);
  return cudaGetLastError();
}

__global__ void k_mirror_flip(int *parity) { *parity ^= 1; }

cudaError_t launch_mirror_flip(int *parity, cudaStream_t s) {
  k_mirror_flip<<<1, 1, 0, s>>>(parity);
  return cudaGetLastError();
}

// Q^n - Q^(n-1) of the interior cells, formed in FP64 and stored in FP32,
// once per physical time step (it is constant over the step's stages).
__global__ void k_level_diff(const double *__restrict__ U1, const double *__restrict__ U1q,
                             float *__restrict__ D2, int n, long long total) {
  const int S = n + 4;
  const long long n3 = (long long)n * n * n;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int c = 1 + (int)(t / n3);
    const int r = (int)(t % n3);
    const size_t o = 5 * cell_index(S, c, 2 + r / (n * n), 2 + (r / n) % n, 2 + r % n);
#pragma unroll
    for (int v = 0; v < 5; ++v) D2[o + v] = (float)(U1[o + v] - U1q[o + v]);
  }
}

cudaError_t launch_level_diff(const double *U1, const double *U1q, float *D2, int n, int ncube,
                              cudaStream_t s) {
  const long long total = (long long)(ncube - 1) * n * n * n;
  if (total <= 0) return cudaSuccess;
  int blocks = (int)((total + 255) / 256);
  if (blocks > 152 * 8) blocks = 152 * 8;
  k_level_diff<<<blocks, 256, 0, s>>>(U1, U1q, D2, n, total);
  return cudaGetLastError();
}

struct PrimF {
  float U, V, W, Tp;  // velocity, T - T0
};

// Asynchronous 4-byte global -> shared copy (cp.async) and the wait for all
// of a thread's copies; an L2 prefetch hint.
__device__ __forceinline__ void cp_async4(void *smem_dst, const void *gmem_src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;\n" ::: "memory");
}
__device__ __forceinline__ void prefetch_l2(const void *p) {
  asm volatile("prefetch.global.L2 [%0];\n" ::"l"(p));
}

template <int T>
struct SplitSmem {
  static constexpr int B = T + 2;      // primitive box edge (tile + 1 halo)
  static constexpr int X = T + 6;      // stencil box edge (tile + 3 halo)
  static constexpr int nPrim = B * B * B;
  static constexpr int nCell = T * T * T;
  static constexpr int nBox = X * X * X;
  // Box pitches in floats: a row of X cells along k (5 floats each), a plane
  // of X rows.  For 8^3 tiles the pitches are padded (72 = 8 mod 32, 1011
  // odd) so that the stencil reads of a warp hit 32 distinct banks for x- and
  // z-faces (2 ways for y-faces) instead of 2 and 4 ways.
  static constexpr int RP = T == 8 ? 72 : 5 * X;
  static constexpr int PP = T == 8 ? 1011 : X * RP;
  static constexpr int nBoxF = X * PP;
  static constexpr int nFace = (T + 1) * T * T;  // faces of one axis
  static constexpr int nBits = (3 * nFace + 31) / 32;
  static constexpr size_t bytes = sizeof(float) * nBoxF /*state deltas*/ +
                                  sizeof(PrimF) * nPrim +
                                  sizeof(float) * 15 * nFace /*face fluxes, 3 axes*/ +
                                  sizeof(float) * 2 * nFace /*x, z face pressure halves*/ +
                                  sizeof(unsigned) * ((nBits + 3) / 4) * 4 /*second views*/ +
                                  ((nBox + 15) / 16) * 16 /*flags*/;
  static_assert(RP >= 5 * X && PP >= X * RP, "box pitches hold the rows");
  static_assert(T != 8 || bytes + 1024 <= 233472 / 2, "two CTAs per SM");
};

// Index of face fa (0..T along axis ax) at in-plane position (p, q) in the
// value-major face arrays.  The in-plane coordinates are (j, k) for x-faces,
// (i, k) for y-faces and (j, i) for z-faces.  For 8^3 tiles the plane index
// is rotated per face (by 8 fa for y-faces, by fa for z-faces) so that the
// 32 faces a warp stores (4 x 8 of one plane) and the faces 32 consecutive
// cells read (i, j, k order) land in distinct banks for every axis.
template <int T>
__device__ __forceinline__ int face_idx(int ax, int fa, int p, int q) {
  if (T == 8) {
    const int in = 8 * p + q;
    return fa * 64 + (ax == 0 ? in : ((in + (ax == 1 ? 8 * fa : fa)) & 63));
  }
  return (fa * T + p) * T + q;
}

// Delta-form preconditioned Roe flux (same formulas as face_flux in
// bcm_common.cuh, evaluated on deltas from the reference state).  Returns the
// flux with P replaced by p' in the momentum terms (P0 cancels in every face
// difference) and dPp = 0.5*(p'_L + p'_R).
template <int AX>
__device__ __forceinline__ void face_flux_delta(const float *ML, const float *MR, float e,
                                                float rho0, float P0, float *F, float &dPp) {
  const float K = 1.4f, Km1 = 0.4f;
  float dU1 = MR[0] - ML[0], dU2 = MR[1] - ML[1], dU3 = MR[2] - ML[2], dU4 = MR[3] - ML[3],
        dU5 = MR[4] - ML[4];
  float _rho = rho0 + ML[0];
  float _ir = 1.0f / _rho;
  float _U = ML[1] * _ir, _V = ML[2] * _ir, _W = ML[3] * _ir;
  float _VV = _U * _U + _V * _V + _W * _W;
  float _pp = (ML[4] - 0.5f * _rho * _VV) * Km1;  // p' = p - P0
  float _P = P0 + _pp;
  float _C = K * _P * _ir;
  float _H = 0.5f * _VV + _C * (1.0f / Km1);
  float rho_ = rho0 + MR[0];
  float ir_ = 1.0f / rho_;
  float U_ = MR[1] * ir_, V_ = MR[2] * ir_, W_ = MR[3] * ir_;
  float VV_ = U_ * U_ + V_ * V_ + W_ * W_;
  float pp_ = (MR[4] - 0.5f * rho_ * VV_) * Km1;
  float P_ = P0 + pp_;
  float C_ = K * P_ * ir_;
  float H_ = 0.5f * VV_ + C_ * (1.0f / Km1);
  float temp5 = sqrtf(_rho), temp6 = sqrtf(rho_);
  float it4 = 1.0f / (temp5 + temp6);
  float rho = temp5 * temp6;
  float U = (temp5 * _U + temp6 * U_) * it4;
  float V = (temp5 * _V + temp6 * V_) * it4;
  float W = (temp5 * _W + temp6 * W_) * it4;
  float VV = U * U + V * V + W * W;
  float H = (temp5 * _H + temp6 * H_) * it4;
  float C = (H - 0.5f * VV) * Km1;
  float q = VV / C;
  float beta = q > e ? q : e;
  const float un = AX == 0 ? U : (AX == 1 ? V : W);
  const float _un = AX == 0 ? _U : (AX == 1 ? _V : _W);
  const float un_ = AX == 0 ? U_ : (AX == 1 ? V_ : W_);
  float temp = 0.5f * (1.0f + beta) * un;
  float Sp = 0.5f * sqrtf(4.0f * beta * C + un * un * (1.0f - beta) * (1.0f - beta));
  float iS = 1.0f / Sp;
  float dp = pp_ - _pp;
  float temp1 = dp / (rho * beta * C);
  float tS = temp * iS;
  float temp2 = tS * (un_ - _un);
  float temp3 = 0.5f * (1.0f - beta) * un * temp * iS;
  float an = fabsf(un);
  float deltaU = (Sp - temp3 - beta * an) * temp1 + temp2;
  float deltaP = tS * dp + (Sp - an + temp3) * rho * (un_ - _un);
  float dr = deltaU * rho;
  float Fav1 = an * dU1 + dr;
  float Fav2 = an * dU2 + dr * U;
  float Fav3 = an * dU3 + dr * V;
  float Fav4 = an * dU4 + dr * W;
  if (AX == 0) Fav2 += deltaP;
  if (AX == 1) Fav3 += deltaP;
  if (AX == 2) Fav4 += deltaP;
  float Fav5 = an * dU5 + dr * H + deltaP * un;
  F[0] = 0.5f * ((_rho * _un + rho_ * un_) - Fav1);
  F[1] = AX == 0 ? 0.5f * ((_rho * _U * _U + _pp + rho_ * U_ * U_ + pp_) - Fav2)
                 : 0.5f * ((_rho * _U * _un + rho_ * U_ * un_) - Fav2);
  F[2] = AX == 1 ? 0.5f * ((_rho * _V * _V + _pp + rho_ * V_ * V_ + pp_) - Fav3)
                 : 0.5f * ((_rho * _V * _un + rho_ * V_ * un_) - Fav3);
  F[3] = AX == 2 ? 0.5f * ((_rho * _W * _W + _pp + rho_ * W_ * W_ + pp_) - Fav4)
                 : 0.5f * ((_rho * _W * _un + rho_ * W_ * un_) - Fav4);
  F[4] = 0.5f * ((_un * (3.5f * _P + 0.5f * _rho * _VV) + un_ * (3.5f * P_ + 0.5f * rho_ * VV_)) -
                 Fav5);
  dPp = 0.5f * (_pp + pp_);
}

// Packed FP32 pairs: Blackwell's FFMA2 / FADD2 / FMUL2 do the arithmetic of
// two independent evaluations (lane .x and lane .y) in one instruction, so
// a thread evaluating two faces at once issues about half the FP32
// instructions.  Subtraction is a - b = fma(b, -1, a) (exact: b * -1 is
// exact); reciprocals and square roots stay per lane (no packed form).
__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {
  return __ffma2_rn(b, make_float2(-1.0f, -1.0f), a);
}
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 rcp2(float2 a) { return make_float2(1.0f / a.x, 1.0f / a.y); }
__device__ __forceinline__ float2 sqrt2(float2 a) { return make_float2(sqrtf(a.x), sqrtf(a.y)); }

// face_flux_delta for two faces of one axis at once (same formulas; lane .x
// and .y are the two faces).
template <int AX>
__device__ __forceinline__ void face_flux_delta2(const float2 *ML, const float2 *MR, float e,
                                                 float rho0, float P0, float2 *F, float2 &dPp) {
  const float2 K = f2(1.4f), Km1 = f2(0.4f), half = f2(0.5f);
  const float2 dU1 = sub2(MR[0], ML[0]), dU2 = sub2(MR[1], ML[1]), dU3 = sub2(MR[2], ML[2]),
               dU4 = sub2(MR[3], ML[3]), dU5 = sub2(MR[4], ML[4]);
  const float2 r0 = f2(rho0), p0 = f2(P0);
  const float2 _rho = add2(r0, ML[0]);
  const float2 _ir = rcp2(_rho);
  const float2 _U = mul2(ML[1], _ir), _V = mul2(ML[2], _ir), _W = mul2(ML[3], _ir);
  const float2 _VV = fma2(_W, _W, fma2(_V, _V, mul2(_U, _U)));
  const float2 _pp = mul2(fma2(mul2(f2(-0.5f), _rho), _VV, ML[4]), Km1);
  const float2 _P = add2(p0, _pp);
  const float2 _C = mul2(mul2(K, _P), _ir);
  const float2 _H = fma2(_C, f2(2.5f), mul2(half, _VV));
  const float2 rho_ = add2(r0, MR[0]);
  const float2 ir_ = rcp2(rho_);
  const float2 U_ = mul2(MR[1], ir_), V_ = mul2(MR[2], ir_), W_ = mul2(MR[3], ir_);
  const float2 VV_ = fma2(W_, W_, fma2(V_, V_, mul2(U_, U_)));
  const float2 pp_ = mul2(fma2(mul2(f2(-0.5f), rho_), VV_, MR[4]), Km1);
  const float2 P_ = add2(p0, pp_);
  const float2 C_ = mul2(mul2(K, P_), ir_);
  const float2 H_ = fma2(C_, f2(2.5f), mul2(half, VV_));
  const float2 temp5 = sqrt2(_rho), temp6 = sqrt2(rho_);
  const float2 it4 = rcp2(add2(temp5, temp6));
  const float2 rho = mul2(temp5, temp6);
  const float2 U = mul2(fma2(temp6, U_, mul2(temp5, _U)), it4);
  const float2 V = mul2(fma2(temp6, V_, mul2(temp5, _V)), it4);
  const float2 W = mul2(fma2(temp6, W_, mul2(temp5, _W)), it4);
  const float2 VV = fma2(W, W, fma2(V, V, mul2(U, U)));
  const float2 H = mul2(fma2(temp6, H_, mul2(temp5, _H)), it4);
  const float2 C = mul2(fma2(f2(-0.5f), VV, H), Km1);
  const float2 q = mul2(VV, rcp2(C));
  const float2 beta = make_float2(fmaxf(q.x, e), fmaxf(q.y, e));
  const float2 un = AX == 0 ? U : (AX == 1 ? V : W);
  const float2 _un = AX == 0 ? _U : (AX == 1 ? _V : _W);
  const float2 un_ = AX == 0 ? U_ : (AX == 1 ? V_ : W_);
  const float2 omb = sub2(f2(1.0f), beta);
  const float2 temp = mul2(mul2(half, add2(f2(1.0f), beta)), un);
  const float2 Sp = mul2(half, sqrt2(fma2(mul2(f2(4.0f), beta), C, mul2(mul2(un, un), mul2(omb, omb)))));
  const float2 iS = rcp2(Sp);
  const float2 dp = sub2(pp_, _pp);
  const float2 temp1 = mul2(dp, rcp2(mul2(mul2(rho, beta), C)));
  const float2 tS = mul2(temp, iS);
  const float2 dun = sub2(un_, _un);
  const float2 temp2 = mul2(tS, dun);
  const float2 temp3 = mul2(mul2(mul2(mul2(half, omb), un), temp), iS);
  const float2 an = make_float2(fabsf(un.x), fabsf(un.y));
  const float2 deltaU = fma2(sub2(sub2(Sp, temp3), mul2(beta, an)), temp1, temp2);
  const float2 deltaP = fma2(mul2(add2(sub2(Sp, an), temp3), rho), dun, mul2(tS, dp));
  const float2 dr = mul2(deltaU, rho);
  float2 Fav1 = fma2(an, dU1, dr);
  float2 Fav2 = fma2(an, dU2, mul2(dr, U));
  float2 Fav3 = fma2(an, dU3, mul2(dr, V));
  float2 Fav4 = fma2(an, dU4, mul2(dr, W));
  if (AX == 0) Fav2 = add2(Fav2, deltaP);
  if (AX == 1) Fav3 = add2(Fav3, deltaP);
  if (AX == 2) Fav4 = add2(Fav4, deltaP);
  const float2 Fav5 = fma2(deltaP, un, fma2(an, dU5, mul2(dr, H)));
  const float2 _rhoun = mul2(_rho, _un), rhoun_ = mul2(rho_, un_);
  F[0] = mul2(half, sub2(add2(_rhoun, rhoun_), Fav1));
  F[1] = AX == 0 ? mul2(half, sub2(add2(fma2(_rhoun, _U, _pp), fma2(rhoun_, U_, pp_)), Fav2))
                 : mul2(half, sub2(fma2(rhoun_, U_, mul2(_rhoun, _U)), Fav2));
  F[2] = AX == 1 ? mul2(half, sub2(add2(fma2(_rhoun, _V, _pp), fma2(rhoun_, V_, pp_)), Fav3))
                 : mul2(half, sub2(fma2(rhoun_, V_, mul2(_rhoun, _V)), Fav3));
  F[3] = AX == 2 ? mul2(half, sub2(add2(fma2(_rhoun, _W, _pp), fma2(rhoun_, W_, pp_)), Fav4))
                 : mul2(half, sub2(fma2(rhoun_, W_, mul2(_rhoun, _W)), Fav4));
  const float2 EL = fma2(mul2(half, _rho), _VV, mul2(f2(3.5f), _P));
  const float2 ER = fma2(mul2(half, rho_), VV_, mul2(f2(3.5f), P_));
  F[4] = mul2(half, sub2(fma2(un_, ER, mul2(_un, EL)), Fav5));
  dPp = mul2(half, add2(_pp, pp_));
}

template <int AX, bool FWD>
__device__ __forceinline__ void visc_face_f(float mu_L, float T0, const PrimF &c, const PrimF &o,
                                            float inv, const PrimF &a0, const PrimF &a1,
                                            const PrimF &a2, const PrimF &a3, const PrimF &b0,
                                            const PrimF &b1, const PrimF &b2, const PrimF &b3,
                                            float *L) {
  float Tm = T0 + 0.5f * (c.Tp + o.Tp);
  float temp = Tm / T0;
  float mu_E = mu_L * temp * sqrtf(temp) * (T0 + 110.f) / (Tm + 110.f);
  float gn[4];
  if (FWD) {
    gn[0] = (o.U - c.U) * inv; gn[1] = (o.V - c.V) * inv;
    gn[2] = (o.W - c.W) * inv; gn[3] = (o.Tp - c.Tp) * inv;
  } else {
    gn[0] = (c.U - o.U) * inv; gn[1] = (c.V - o.V) * inv;
    gn[2] = (c.W - o.W) * inv; gn[3] = (c.Tp - o.Tp) * inv;
  }
  const float q = 0.25f * inv;
  float ga[3], gb[3];
  ga[0] = (a0.U + a1.U - a2.U - a3.U) * q;
  ga[1] = (a0.V + a1.V - a2.V - a3.V) * q;
  ga[2] = (a0.W + a1.W - a2.W - a3.W) * q;
  gb[0] = (b0.U + b1.U - b2.U - b3.U) * q;
  gb[1] = (b0.V + b1.V - b2.V - b3.V) * q;
  gb[2] = (b0.W + b1.W - b2.W - b3.W) * q;
  float d[3][3];
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    d[AX][m] = gn[m];
    d[AX == 0 ? 1 : 0][m] = ga[m];
    d[AX == 2 ? 1 : 2][m] = gb[m];
  }
  float div = d[0][0] + d[1][1] + d[2][2];
  float Um = 0.5f * (c.U + o.U), Vm = 0.5f * (c.V + o.V), Wm = 0.5f * (c.W + o.W);
  float s1, s2, s3;
  if (AX == 0) {
    s1 = mu_E * (2.f * d[0][0] - (2.f / 3.f) * div);
    s2 = mu_E * (d[1][0] + d[0][1]);
    s3 = mu_E * (d[2][0] + d[0][2]);
  } else if (AX == 1) {
    s1 = mu_E * (d[1][0] + d[0][1]);
    s2 = mu_E * (2.f * d[1][1] - (2.f / 3.f) * div);
    s3 = mu_E * (d[2][1] + d[1][2]);
  } else {
    s1 = mu_E * (d[2][0] + d[0][2]);
    s2 = mu_E * (d[2][1] + d[1][2]);
    s3 = mu_E * (2.f * d[2][2] - (2.f / 3.f) * div);
  }
  L[0] = s1;
  L[1] = s2;
  L[2] = s3;
  L[3] = Um * s1 + Vm * s2 + Wm * s3 + mu_E * (float)(BCMG_CV * BCMG_K / BCMG_PR) * gn[3];
}

// Threads per CTA: for 8^3 tiles, half the 576 faces of an axis (two faces
// and up to two cells per thread) so that two CTAs (~110 KB shared memory
// each) share an SM and one CTA's staging, barriers and FP64 tail overlap
// the other's FP32 work; for 4^3 tiles one face per thread.  Whole warps
// (the staging loop gives every warp whole rows).
template <int T>
__host__ __device__ constexpr int split_threads() {
  return T == 8 ? 288 : (((T + 1) * T * T) + 31) / 32 * 32;
}
template <int T>
__host__ __device__ constexpr int split_ctas_per_sm() { return T == 8 ? 2 : 1; }

// Reconstruction of the split path: the stencils of recon() (bcm_common.cuh)
// with the 1/60 and 1/6 factors folded into the coefficients (one multiply
// fewer per value; the FP64 path keeps the reference's form).
template <typename Ld>
__device__ __forceinline__ void recon_split(int ord, Ld ld, float *ML, float *MR) {
  if (ord == 5) {
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      const float a = ld(-3, v), b = ld(-2, v), c = ld(-1, v), d = ld(0, v), f = ld(1, v),
                  g = ld(2, v);
      ML[v] = (2.f / 60) * a - (13.f / 60) * b + (47.f / 60) * c + (27.f / 60) * d -
              (3.f / 60) * f;
      MR[v] = (-3.f / 60) * b + (27.f / 60) * c + (47.f / 60) * d - (13.f / 60) * f +
              (2.f / 60) * g;
    }
  } else if (ord == 3) {
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      const float b = ld(-2, v), c = ld(-1, v), d = ld(0, v), f = ld(1, v);
      ML[v] = (-1.f / 6) * b + (5.f / 6) * c + (2.f / 6) * d;
      MR[v] = (2.f / 6) * c + (5.f / 6) * d - (1.f / 6) * f;
    }
  } else {
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      ML[v] = ld(-1, v);
      MR[v] = ld(0, v);
    }
  }
}

// PACK (8^3 tiles only): each thread evaluates its two faces of an axis
// together in packed FP32 pairs; otherwise one after the other.
template <int T, bool VISCOUS, bool PACK>
__global__ void __launch_bounds__(split_threads<T>(), split_ctas_per_sm<T>())
    k_flux_split(FluxSplitArgs a) {
  static_assert(!PACK || (T == 8 && 2 * split_threads<T>() == (T + 1) * T * T),
                "packed face pairs: two faces of an axis per thread");
  using SM = SplitSmem<T>;
  constexpr int B = SM::B;
  constexpr int X = SM::X;
  constexpr int NT = split_threads<T>();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float *box = reinterpret_cast<float *>(smem_raw);  // [X][X][X][5] deltas, pitches RP, PP
  PrimF *prim = reinterpret_cast<PrimF *>(box + SM::nBoxF);
  // Face fluxes stored once per face: [3 axes][5][nFace], the x- and z-face
  // pressure halves [2][nFace], and one bit per face whose minus-side cell
  // takes a different reconstruction order (that cell recomputes its view).
  constexpr int NF = SM::nFace;
  float *FF = reinterpret_cast<float *>(prim + SM::nPrim);
  float *FdP = FF + 15 * NF;
  unsigned *dbits = reinterpret_cast<unsigned *>(FdP + 2 * NF);
  signed char *fbox =
      reinterpret_cast<signed char *>(dbits + ((SM::nBits + 3) / 4) * 4);  // [X][X][X] flags
  float *Fb = FF;  // staging area of the int flags (before the face pass)

  const int n = a.ph.n, S = n + 4, nx = n + 1;
  const int nt = n / T;
  const int tid = threadIdx.x;
  const int tiles = nt * nt * nt;
  const int cube = a.cube0 + blockIdx.x / tiles;
  if (!case_active(a.bt, cube)) return;  // converged case (uniform per CTA)
  const int tl = blockIdx.x % tiles;
  const int bi = 2 + (tl / (nt * nt)) * T, bj = 2 + ((tl / nt) % nt) * T, bk = 2 + (tl % nt) * T;
  // Mirror buffers: read the current one; stages 1..3 write the deltas of
  // the tile's cells into the other one.
  const int par = *a.mir.parity;
  const float *__restrict__ M = a.mir.buf[par];
  float *const Mw = a.RK >= 1 ? a.mir.buf[par ^ 1] : nullptr;
  const int *__restrict__ F = a.FWS;
  const size_t cb = cell_index(S, cube, 0, 0, 0);
  // Constants of the cube's case (kernel arguments for a single case).
  float rho0 = a.rho0f, P0 = a.P0f, RT0 = a.RT0f /* R * T0 */, ef = a.ef, T0c = a.T0f,
        mu_Lc = a.mu_Lf, i2dtc = a.i2dtf, dTc = a.dTf, dTauc = a.dTauf;
  double rho0d = a.mir.rho0, E0d = a.mir.E0;  // mirror reference state (FP64)
  if (a.bt.cube_case) {
    const CaseConst *cq = a.bt.cases + __ldg(a.bt.cube_case + cube);
    rho0 = cq->rho0f; P0 = cq->P0f; RT0 = cq->RT0f; ef = cq->ef; T0c = cq->T0f;
    mu_Lc = cq->mu_Lf; i2dtc = cq->i2dtf; dTc = cq->dTf; dTauc = cq->dTauf;
    rho0d = cq->rho0; E0d = cq->E0;
  }
  const float iR = 1.0f / 287.0f;

  // The FP64 state, the previous level and the level difference of the
  // tile's own cells are read at the end of the stage: start moving their
  // rows (8 cells: 320 B, 320 B, 160 B) into L2 now.
  for (int r = tid; r < T * T * 4; r += NT) {
    const int row = r >> 2, part = r & 3;
    const size_t go = cb + ((size_t)(bi + row / T) * S + (bj + row % T)) * S + bk;
    const int od = part == 3 ? 5 * T - 1 : 16 * part;  // doubles
    const int of = part == 3 ? 5 * T - 1 : (part == 2 ? 32 : 0);  // floats
    prefetch_l2(a.U1_ + 5 * go + od);
    prefetch_l2(a.U1 + 5 * go + od);
    prefetch_l2(a.D2 + 5 * go + of);
  }

  // Phase 0: stage the stencil box (tile +- 3 cells, clipped to the padded
  // cube) of FP32 deltas and flags into shared memory with asynchronous
  // 4-byte copies (the rows of the AoS layout start at any 4-byte boundary),
  // all in flight at once and waited for once.  Each box row along k is a
  // contiguous run of 5*X floats, so the copies are coalesced.  The flags go
  // as ints into the face buffers (unused until the face passes) and are
  // narrowed to bytes below.  Box cells outside the padded cube are never
  // read by the stencil (the reconstruction order falls back before reaching
  // them) and are left unset.
  int *ftmp = reinterpret_cast<int *>(Fb);
  static_assert(SM::nBox <= 17 * SM::nFace, "int flags fit the face buffers");
  for (int w = tid; w < SM::nBits; w += NT) dbits[w] = 0u;
  {
    const int k0 = bk - 3;
    const int klo = k0 < 0 ? -k0 : 0;                 // first valid column
    const int khi = (k0 + X > S) ? S - k0 : X;        // one past the last
    const int ncol = khi - klo;
    const int warp = tid >> 5, lane = tid & 31;
    constexpr int NW = (NT + 31) / 32;
    for (int row = warp; row < X * X; row += NW) {
      const int bi_ = row / X, bj_ = row - (row / X) * X;
      const int gi = bi - 3 + bi_, gj = bj - 3 + bj_;
      if (gi < 0 || gi >= S || gj < 0 || gj >= S) continue;
      const size_t g = cb + ((size_t)gi * S + gj) * S + (k0 + klo);
      const float *src = M + 5 * g;
      float *dst = box + bi_ * SM::PP + bj_ * SM::RP + klo * 5;
      for (int e = lane; e < 5 * ncol; e += 32) cp_async4(dst + e, src + e);
      const int *fsrc = F + g;
      int *fdst = ftmp + row * X + klo;
      for (int e = lane; e < ncol; e += 32) cp_async4(fdst + e, fsrc + e);
    }
    cp_async_wait_all();
  }
  __syncthreads();
  for (int p = tid; p < SM::nBox; p += NT) fbox[p] = (signed char)ftmp[p];
  auto BX = [&](int li, int lj, int lk) -> const float * {  // li.. relative to tile origin
    return box + (li + 3) * SM::PP + (lj + 3) * SM::RP + (lk + 3) * 5;
  };
  auto FL = [&](int li, int lj, int lk) -> int {
    return fbox[((li + 3) * X + (lj + 3)) * X + (lk + 3)];
  };

  // Phase 1: primitives (u, v, w, T - T0) over the tile plus one halo cell.
  for (int p = tid; p < SM::nPrim; p += NT) {
    int li = p / (B * B), lj = (p / B) % B, lk = p % B;
    const float *q = BX(li - 1, lj - 1, lk - 1);
    float r = q[0], m1 = q[1], m2 = q[2], m3 = q[3], e = q[4];
    float rho = rho0 + r;
    float ir = 1.0f / rho;
    PrimF pr;
    pr.U = m1 * ir;
    pr.V = m2 * ir;
    pr.W = m3 * ir;
    float pp = (e - 0.5f * rho * (pr.U * pr.U + pr.V * pr.V + pr.W * pr.W)) * 0.4f;
    pr.Tp = (pp - r * RT0) * ir * iR;  // T - T0 = (p' - rho' R T0) / (rho R)
    prim[p] = pr;
  }
  __syncthreads();  // byte flags complete; the face buffers are free again

  const float inv = a.inv_dx[cube];

  // The three axes are unrolled: every axis-dependent index, stride and
  // flux variant is then a compile-time choice (6% of the launch on the
  // 7 M-cell TGV case, measured).
  // One face f of axis ax: reconstruction order of the stored view, the
  // left/right states, the second-view bit; returns the face's slot.
  auto face_prep = [&](int ax, int f, float *ML, float *MR) -> int {
    const int fa = f / (T * T), p = (f / T) % T, q = f % T;
    int li, lj, lk;  // a warp covers 4 x 8 faces of a plane (8 x 4 for z-faces)
    if (ax == 0) { li = fa; lj = p; lk = q; }
    else if (ax == 1) { li = p; lj = fa; lk = q; }
    else { li = q; lj = p; lk = fa; }
    const int g = (ax == 0 ? bi + li : (ax == 1 ? bj + lj : bk + lk));
    const int di = ax == 0, dj = ax == 1, dk = ax == 2;
    const int fm2 = FL(li - 2 * di, lj - 2 * dj, lk - 2 * dk),
              fm1 = FL(li - di, lj - dj, lk - dk), f0 = FL(li, lj, lk),
              fp1 = FL(li + di, lj + dj, lk + dk);
    const bool needB = fa < T, needF = fa > 0;
    const int ob = order_backward(g, fm2, fm1, fp1);
    const int of = order_forward(g, nx, fm2, f0, fp1);
    const float *base = BX(li, lj, lk);
    const int sstride = ax == 0 ? SM::PP : (ax == 1 ? SM::RP : 5);
    auto ld = [&](int d, int v) -> float { return base[sstride * d + v]; };
    // The stored view is the plus-side cell's (the minus-side cell's for
    // the last face, which has no plus cell in the tile); where the
    // minus-side cell's order differs it recomputes its own view.
    recon_split(needB ? ob : of, ld, ML, MR);
    const int fi = face_idx<T>(ax, fa, p, q);
    if (needB && needF && ob != of) {
      const int bit = ax * NF + fi;
      atomicOr(dbits + (bit >> 5), 1u << (bit & 31));
    }
    return fi;
  };

  // The three axes are unrolled: every axis-dependent index, stride and
  // flux variant is then a compile-time choice (6% of the launch on the
  // 7 M-cell TGV case, measured).
#pragma unroll
  for (int ax = 0; ax < 3; ++ax) {
    if (PACK) {
      // 8^3 tiles: the axis's 576 faces are two per thread (f and f + 288),
      // evaluated together in packed pairs.
      float MLa[5], MRa[5], MLb[5], MRb[5];
      const int fa_ = face_prep(ax, tid, MLa, MRa);
      const int fb_ = face_prep(ax, tid + NT, MLb, MRb);
      float2 ML2[5], MR2[5], F2v[5], dP2;
#pragma unroll
      for (int v = 0; v < 5; ++v) {
        ML2[v] = make_float2(MLa[v], MLb[v]);
        MR2[v] = make_float2(MRa[v], MRb[v]);
      }
      if (ax == 0) face_flux_delta2<0>(ML2, MR2, ef, rho0, P0, F2v, dP2);
      else if (ax == 1) face_flux_delta2<1>(ML2, MR2, ef, rho0, P0, F2v, dP2);
      else face_flux_delta2<2>(ML2, MR2, ef, rho0, P0, F2v, dP2);
#pragma unroll
      for (int v = 0; v < 5; ++v) {
        FF[(5 * ax + v) * NF + fa_] = F2v[v].x;
        FF[(5 * ax + v) * NF + fb_] = F2v[v].y;
      }
      if (ax != 1) {
        FdP[(ax == 2) * NF + fa_] = dP2.x;
        FdP[(ax == 2) * NF + fb_] = dP2.y;
      }
    } else {
      for (int f = tid; f < (T + 1) * T * T; f += NT) {
        float ML[5], MR[5], Fx[5], dP;
        const int fi = face_prep(ax, f, ML, MR);
        if (ax == 0) face_flux_delta<0>(ML, MR, ef, rho0, P0, Fx, dP);
        else if (ax == 1) face_flux_delta<1>(ML, MR, ef, rho0, P0, Fx, dP);
        else face_flux_delta<2>(ML, MR, ef, rho0, P0, Fx, dP);
#pragma unroll
        for (int v = 0; v < 5; ++v) FF[(5 * ax + v) * NF + fi] = Fx[v];
        if (ax != 1) FdP[(ax == 2) * NF + fi] = dP;
      }
    }
  }
  __syncthreads();
  // Norm / force partial sums of this CTA (stage 3), reduced below by all
  // threads.
  double s5[7] = {0, 0, 0, 0, 0, 0, 0};
  // Not unrolled: with the packed face pass, two cells' tails interleaved
  // measured 2.5% slower per launch (n = 16; 1.9% at n = 24, same bits).
#pragma unroll 1
  for (int cl = tid; cl < SM::nCell; cl += NT) {
  const int mi = cl / (T * T), mj = (cl / T) % T, mk = cl % T;
  // Flux balance of the cell from its six faces, axis by axis.
  float acc[5], dPdx = 0.f, dPdz = 0.f;
#pragma unroll
  for (int ax = 0; ax < 3; ++ax) {
    const int m = ax == 0 ? mi : (ax == 1 ? mj : mk);
    const int p = ax == 2 ? mj : (ax == 0 ? mj : mi), q = ax == 2 ? mi : mk;
    const int fb = face_idx<T>(ax, m, p, q), ff = face_idx<T>(ax, m + 1, p, q);
    float Fbv[5], Ffv[5], dPbv = 0.f, dPfv = 0.f;
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      Fbv[v] = FF[(5 * ax + v) * NF + fb];
      Ffv[v] = FF[(5 * ax + v) * NF + ff];
    }
    if (ax != 1) {
      dPbv = FdP[(ax == 2) * NF + fb];
      dPfv = FdP[(ax == 2) * NF + ff];
    }
    const int bit = ax * NF + ff;
    if (m + 1 < T && ((dbits[bit >> 5] >> (bit & 31)) & 1u)) {
      // the forward face's stored view is the next cell's: form this cell's
      const int li = mi + (ax == 0), lj = mj + (ax == 1), lk = mk + (ax == 2);
      const int g = (ax == 0 ? bi + li : (ax == 1 ? bj + lj : bk + lk));
      const int di = ax == 0, dj = ax == 1, dk = ax == 2;
      const int of = order_forward(g, nx, FL(li - 2 * di, lj - 2 * dj, lk - 2 * dk),
                                   FL(li, lj, lk), FL(li + di, lj + dj, lk + dk));
      const float *base = BX(li, lj, lk);
      const int sstride = ax == 0 ? SM::PP : (ax == 1 ? SM::RP : 5);
      auto ld = [&](int d, int v) -> float { return base[sstride * d + v]; };
      float ML[5], MR[5];
      recon_split(of, ld, ML, MR);
      if (ax == 0) face_flux_delta<0>(ML, MR, ef, rho0, P0, Ffv, dPfv);
      else if (ax == 1) face_flux_delta<1>(ML, MR, ef, rho0, P0, Ffv, dPfv);
      else face_flux_delta<2>(ML, MR, ef, rho0, P0, Ffv, dPfv);
    }
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      const float t = (Ffv[v] - Fbv[v]) * inv;
      acc[v] = ax == 0 ? t : acc[v] + t;
    }
    if (ax == 0) dPdx = dPfv - dPbv;
    if (ax == 2) dPdz = dPfv - dPbv;
  }
  auto P = [&](int di, int dj, int dk) -> const PrimF & {
    return prim[((mi + 1 + di) * B + (mj + 1 + dj)) * B + (mk + 1 + dk)];
  };
  const PrimF &c = P(0, 0, 0);
  float vF[5] = {0, 0, 0, 0, 0};
  if (VISCOUS) {
    const float T0 = T0c;
    const float mu_L = mu_Lc;
    float Lb[4], Lf[4], Mb[4], Mf[4], Nb[4], Nf[4];
    visc_face_f<0, false>(mu_L, T0, c, P(-1, 0, 0), inv, P(0, 1, 0), P(-1, 1, 0), P(0, -1, 0),
                          P(-1, -1, 0), P(0, 0, 1), P(-1, 0, 1), P(0, 0, -1), P(-1, 0, -1), Lb);
    visc_face_f<0, true>(mu_L, T0, c, P(1, 0, 0), inv, P(0, 1, 0), P(1, 1, 0), P(0, -1, 0),
                         P(1, -1, 0), P(0, 0, 1), P(1, 0, 1), P(0, 0, -1), P(1, 0, -1), Lf);
    visc_face_f<1, false>(mu_L, T0, c, P(0, -1, 0), inv, P(1, 0, 0), P(1, -1, 0), P(-1, 0, 0),
                          P(-1, -1, 0), P(0, 0, 1), P(0, -1, 1), P(0, 0, -1), P(0, -1, -1), Mb);
    visc_face_f<1, true>(mu_L, T0, c, P(0, 1, 0), inv, P(1, 0, 0), P(1, 1, 0), P(-1, 0, 0),
                         P(-1, 1, 0), P(0, 0, 1), P(0, 1, 1), P(0, 0, -1), P(0, 1, -1), Mf);
    visc_face_f<2, false>(mu_L, T0, c, P(0, 0, -1), inv, P(1, 0, 0), P(1, 0, -1), P(-1, 0, 0),
                          P(-1, 0, -1), P(0, 1, 0), P(0, 1, -1), P(0, -1, 0), P(0, -1, -1), Nb);
    visc_face_f<2, true>(mu_L, T0, c, P(0, 0, 1), inv, P(1, 0, 0), P(1, 0, 1), P(-1, 0, 0),
                         P(-1, 0, 1), P(0, 1, 0), P(0, 1, 1), P(0, -1, 0), P(0, -1, 1), Nf);
#pragma unroll
    for (int v = 1; v < 5; ++v)
      vF[v] = ((Lf[v - 1] - Lb[v - 1]) + (Mf[v - 1] - Mb[v - 1]) + (Nf[v - 1] - Nb[v - 1])) * inv;
  }

  // BDF2 source from FP64 time-level differences, then FP32.  The FP64 <->
  // FP32 conversions of this tail are the hardware's (IEEE round to
  // nearest): here the FP64 pipe has room and the integer pipes do not
  // (measured: the integer-pipe routines of k_mirror made the launch 7-8%
  // longer).
  const size_t go = cb + ((size_t)(bi + mi) * S + (bj + mj)) * S + (bk + mk);
  double *u = a.U1_ + 5 * go;  // only this thread reads or writes these cells
  const double *uu = a.U1 + 5 * go;
  const float *d2p = a.D2 + 5 * go;
  const int IF = FL(mi, mj, mk);
  const float i2dt = i2dtc;
  float Rk[5];
  double xq[5], un[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    const double x = u[v], y = __ldg(uu + v);
    xq[v] = x;
    const float d1 = __double2float_rn(x - y), d2 = __ldg(d2p + v);
    const float Rp = -(3.0f * d1 - d2) * i2dt;
    Rk[v] = Rp - acc[v] + vF[v];
  }
  if (IF == kFluid && a.RK == 0) {
    // residual only: the LU-SGS right-hand side
#pragma unroll
    for (int v = 0; v < 5; ++v) a.R32[5 * go + v] = Rk[v];
  } else if (IF == kFluid) {
    const float K = 1.4f, Km1 = 0.4f;
    const float dT = dTc, dTau = dTauc;
    const float *qm = BX(mi, mj, mk);
    const float rho = rho0 + qm[0];
    const float Uc = c.U, Vc = c.V, Wc = c.W;
    const float VV = Uc * Uc + Vc * Vc + Wc * Wc;
    const float Pc = P0 + (qm[4] - 0.5f * rho * VV) * Km1;
    const float Tt = Pc / rho;  // P/rho (:2302)
    const float C = K * Tt;
    const float H = 0.5f * VV + C / Km1;
    const float qv = VV / C;
    const float beta = qv > ef ? qv : ef;
    const float itemp = 1.0f / (K * Tt * (2 * dT + 3 * dTau) * (2 * dT + 3 * beta * dTau));
    const float temp2 = Km1 * (beta - 1) * dT * dT;
    const float temp3 = 0.5f * Km1 * VV;  // == H - H*K - VV + K*(T+VV) since C = K*T
    const float bm1 = beta - 1;
    const float a4 = 4 * temp3 * bm1 * dT * dT;
    const float D = 3 * K * Tt * beta * dTau;
    float d[5][5];
    d[0][0] = (2 * dT * (-2 * (-Km1 * (H - VV) - temp3 * beta) * dT + D)) * itemp;
    d[0][1] = (-4 * Uc * temp2) * itemp;
    d[0][2] = (-4 * Vc * temp2) * itemp;
    d[0][3] = (-4 * Wc * temp2) * itemp;
    d[0][4] = (4 * temp2) * itemp;
    d[1][0] = Uc * a4 * itemp;
    d[1][1] = (2 * dT * (2 * K * (Tt - Uc * Uc * bm1) * dT + 2 * Uc * Uc * bm1 * dT + D)) * itemp;
    d[1][2] = (-4 * Uc * Vc * temp2) * itemp;
    d[1][3] = (-4 * Uc * Wc * temp2) * itemp;
    d[1][4] = (4 * Uc * temp2) * itemp;
    d[2][0] = Vc * a4 * itemp;
    d[2][1] = d[1][2];
    d[2][2] = (2 * dT * (2 * K * (Tt - Vc * Vc * bm1) * dT + 2 * Vc * Vc * bm1 * dT + D)) * itemp;
    d[2][3] = (-4 * Vc * Wc * temp2) * itemp;
    d[2][4] = (4 * Vc * temp2) * itemp;
    d[3][0] = Wc * a4 * itemp;
    d[3][1] = d[1][3];
    d[3][2] = d[2][3];
    d[3][3] = (2 * dT * (2 * K * (Tt - Wc * Wc * bm1) * dT + 2 * Wc * Wc * bm1 * dT + D)) * itemp;
    d[3][4] = (4 * Wc * temp2) * itemp;
    d[4][0] = H * a4 * itemp;
    d[4][1] = (-4 * H * Uc * temp2) * itemp;
    d[4][2] = (-4 * H * Vc * temp2) * itemp;
    d[4][3] = (-4 * H * Wc * temp2) * itemp;
    d[4][4] = (2 * dT * (2 * H * Km1 * bm1 * dT + K * Tt * (2 * dT + 3 * beta * dTau))) * itemp;
    // Stage update Q += w dQ (w = 1, 1/4, 2/3): the reference's RK
    // combinations with Q1 = Q2 = Q on fluid cells at stage entry.
    const float w = a.RK == 1 ? 1.0f : (a.RK == 2 ? 0.25f : 2.0f / 3.0f);
    float dq[5];
#pragma unroll
    for (int r = 0; r < 5; ++r) {
      dq[r] = w * dTau * (d[r][0] * Rk[0] + d[r][1] * Rk[1] + d[r][2] * Rk[2] +
                          d[r][3] * Rk[3] + d[r][4] * Rk[4]);
      un[r] = xq[r] + (double)dq[r];
      u[r] = un[r];
    }
    // Same-level interface copy of this cell, done here.  No CTA reads the
    // FP64 state of another cell during the stage, so the write races with
    // nothing.
    if (a.push) push_same_level(a.U1_, a.push, n, cube, bi + mi, bj + mj, bk + mk, un);
    if (a.RK == 3) {
      // Change norms of p, u, v, w, T from the increment, in FP32; summed
      // in FP64 (BCM_Flux...cpp:2530-2566).
      const float rf = rho, m1 = __double2float_rn(xq[1]), m2 = __double2float_rn(xq[2]),
                  m3 = __double2float_rn(xq[3]);
      const float dr = dq[0], e1 = dq[1], e2 = dq[2], e3 = dq[3], dE = dq[4];
      const float den = 1.0f / (rf * (rf + dr));
      const float dU = (e1 * rf - m1 * dr) * den;
      const float dVv = (e2 * rf - m2 * dr) * den;
      const float dW = (e3 * rf - m3 * dr) * den;
      const float mm = m1 * m1 + m2 * m2 + m3 * m3;
      const float dKE =
          0.5f * ((2.f * (m1 * e1 + m2 * e2 + m3 * e3) + e1 * e1 + e2 * e2 + e3 * e3) * rf - mm * dr) * den;
      const float dP = Km1 * (dE - dKE);
      const float dTt = (dP * rf - Pc * dr) * den;
      s5[0] += (double)(dP * dP);
      s5[1] += (double)(dU * dU);
      s5[2] += (double)(dVv * dVv);
      s5[3] += (double)(dW * dW);
      s5[4] += (double)(dTt * dTt);
    }
  } else {
    // Force integrands on non-fluid cells (:2395-2398); their sum over the
    // case is er[6], er[7].
    const double dx = a.cube_size[cube] / n;
    const double dV = dx * dx * dx;
    const double r0 = -((double)(-dPdx * inv) + (double)vF[1]) * dV;
    const double r1 = -((double)(-dPdz * inv) + (double)vF[3]) * dV;
    a.Residual1[5 * go + 0] = r0;
    a.Residual1[5 * go + 1] = r1;
    s5[5] += r0;
    s5[6] += r1;
  }
  if (Mw) {
    // The cell's mirror value after the stage into the next buffer (the
    // staged value where the cell did not change), and into the same-level
    // neighbour's ghost layers: every cell of those layers pushes, since the
    // next buffer's ghost layers hold values two stages old.
    // The conversion is the hardware's (IEEE round to nearest, the same bits
    // as the integer-pipe routine of the other writers): this kernel's FP64
    // pipe has room, its integer pipes do not (measured: the integer routine
    // made the launch 17% longer, this form 9%).
    float m5[5];
    if (IF == kFluid) {
#pragma unroll
      for (int v = 0; v < 5; ++v)
        m5[v] = __double2float_rn(v == 0 ? un[v] - rho0d : (v == 4 ? un[v] - E0d : un[v]));
    } else {
      const float *qm = BX(mi, mj, mk);
#pragma unroll
      for (int v = 0; v < 5; ++v) m5[v] = qm[v];
    }
    float *mw = Mw + 5 * go;
#pragma unroll
    for (int v = 0; v < 5; ++v) mw[v] = m5[v];
    if (a.push) push_same_level(Mw, a.push, n, cube, bi + mi, bj + mj, bk + mk, m5);
  }
  }  // cells of this thread
  if (a.RK != 3) return;
  __syncthreads();  // the face buffers are reused for the block reduction
  double *red = reinterpret_cast<double *>(Fb);  // [NW][7]
  constexpr int NWR = NT / 32;
#pragma unroll
  for (int m = 0; m < 7; ++m) {
    double v = s5[m];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if ((tid & 31) == 0) red[(tid >> 5) * 7 + m] = v;
  }
  __syncthreads();
  if (tid < 7) {
    double v = 0;
    for (int wv = 0; wv < NWR; ++wv) v += red[wv * 7 + tid];
    a.partials[(size_t)blockIdx.x * 7 + tid] = v;
  }
}

template <int T, bool VISCOUS, bool PACK>
static cudaError_t launch_split_k(const FluxSplitArgs &a, unsigned grid, cudaStream_t s) {
  const size_t smem = SplitSmem<T>::bytes;
  cudaError_t e = cudaFuncSetAttribute(k_flux_split<T, VISCOUS, PACK>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k_flux_split<T, VISCOUS, PACK><<<grid, split_threads<T>(), smem, s>>>(a);
  return cudaGetLastError();
}

template <int T>
static cudaError_t launch_split_t(const FluxSplitArgs &a, int ncubes, cudaStream_t s) {
  const int nt = a.ph.n / T;
  const unsigned grid = (unsigned)(ncubes * nt * nt * nt);
  if (grid == 0) return cudaSuccess;
  const bool visc = a.ph.mu_L != 0.0;
  if (T == 8 && a.form == 1)
    return visc ? launch_split_k<T, true, T == 8>(a, grid, s)
                : launch_split_k<T, false, T == 8>(a, grid, s);
  return visc ? launch_split_k<T, true, false>(a, grid, s) : launch_split_k<T, false, false>(a, grid, s);
}

int flux_tile(int n, int tile) {
  if (tile == 8 && n % 8 == 0) return 8;
  if (tile == 4 && n % 4 == 0) return 4;
  return n % 8 == 0 ? 8 : 4;
}

int flux_split_blocks(int n, int ncubes, int tile) {
  const int T = flux_tile(n, tile);
  const int nt = n / T;
  return ncubes * nt * nt * nt;
}

cudaError_t launch_flux_split(const FluxSplitArgs &a, int ncubes, cudaStream_t s) {
  if (a.ph.n % 4 != 0) return cudaErrorInvalidValue;
  if (flux_tile(a.ph.n, a.tile) == 8) return launch_split_t<8>(a, ncubes, s);
  return launch_split_t<4>(a, ncubes, s);
}

}  // namespace bcmg
