// Shared definitions for the BCM hot-path kernels (sm_103a).
//
// State layout in HBM is the reference's (Array.h:13-25): a cube-major
// array U[c][i][j][k][v] of doubles, S = n+4 cells per cube edge (two ghost
// layers per side), the five conservative variables contiguous (40 B per
// cell).  Keeping this layout makes the reference-facing entry points a
// plain memcpy and lets a thread read a whole cell with three vector loads.
// Cube 0 is unused (the reference numbers cubes from 1, main.cpp:90).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace bcmg {

constexpr int kFluid = 1;  // IFLUID, BCM.h:6

// prm.h constants that the reference spells as literals/macros.  K and R keep
// their literal values; (K-1) is formed as (1.4-1) exactly like the macro
// expansion (prm.h:1-2).
#define BCMG_K 1.4
#define BCMG_R 287
#define BCMG_CV 717.5
#define BCMG_PR 0.72

// Per-case constants: the reference's compile-time prm.h / Resolution.h
// values, carried at run time so one library serves every configuration.
struct Phys {
  int n;          // interior cells per cube edge (NcubeX)
  int mpi_ncube;  // residual-norm normaliser (MPI_Ncube)
  double mu_L;    // Sutherland reference viscosity (0: inviscid)
  double rho0, U0, Uin, P0;
};

__host__ __device__ inline size_t cell_index(int S, int c, int i, int j, int k) {
  return ((((size_t)c * S + i) * S + j) * S + k);
}

// Same-level interface copy of one updated interior cell (ci, cj, ck) of
// `cube`, made by the kernel that updates it (BCM_Interface.cpp:1745-1783
// copies exactly this after the update): a cell in layers 2, 3 (slot 0) or
// n, n+1 (slot 1) along an axis writes its new value un[5] into ghost
// layers n+2, n+3 or 0, 1 of the cube push[6 cube + 2 axis + slot] (0:
// none).  Safe only while no other thread reads those ghost layers of U
// (the FP64 state, or the FP32 mirror buffer being written).
template <typename T>
__device__ __forceinline__ void push_same_level(T *U, const int *push, int n, int cube, int ci,
                                                int cj, int ck, const T *un) {
  const int cg[3] = {ci, cj, ck};
#pragma unroll
  for (int ax = 0; ax < 3; ++ax) {
    const int x = cg[ax];
    const int slot = x <= 3 ? 0 : (x >= n ? 1 : -1);
    if (slot < 0) continue;
#ifdef __CUDA_ARCH__
    const int d = __ldg(push + 6 * cube + 2 * ax + slot);
#else
    const int d = push[6 * cube + 2 * ax + slot];
#endif
    if (d <= 0) continue;
    int dc[3] = {ci, cj, ck};
    dc[ax] = slot == 0 ? x + n : x - n;
    T *g = U + 5 * cell_index(n + 4, d, dc[0], dc[1], dc[2]);
#pragma unroll
    for (int r = 0; r < 5; ++r) g[r] = un[r];
  }
}

// ---------------------------------------------------------------------------
// Preconditioned Roe-type face flux (BCM_Flux_XYZ_Viscous_Runge_kutta.cpp
// :606-693 z, :1057-1146 x, :1503-1594 y).  AX is the face normal.
// Operation order is the reference's, so with contraction off the result is
// bit-identical to it.
// ---------------------------------------------------------------------------
template <int AX, typename R>
__device__ __forceinline__ void face_flux(const R *ML, const R *MR, R e, R *F, R &dP) {
  const R K = (R)BCMG_K;
  const R Km1 = (R)(BCMG_K - 1);
  R dU1 = MR[0] - ML[0], dU2 = MR[1] - ML[1], dU3 = MR[2] - ML[2], dU4 = MR[3] - ML[3],
    dU5 = MR[4] - ML[4];
  R _rho = ML[0];
  R _U = ML[1] / _rho, _V = ML[2] / _rho, _W = ML[3] / _rho;
  R _VV = _U * _U + _V * _V + _W * _W;
  R _P = (ML[4] - (R)0.5 * _rho * _VV) * Km1;
  R _C = K * _P / _rho;
  R _H = (R)0.5 * _VV + _C / Km1;
  R rho_ = MR[0];
  R U_ = MR[1] / rho_, V_ = MR[2] / rho_, W_ = MR[3] / rho_;
  R VV_ = U_ * U_ + V_ * V_ + W_ * W_;
  R P_ = (MR[4] - (R)0.5 * rho_ * VV_) * Km1;
  R C_ = K * P_ / rho_;
  R H_ = (R)0.5 * VV_ + C_ / Km1;
  R temp5 = sqrt(_rho), temp6 = sqrt(rho_);
  R temp4 = temp5 + temp6;
  R rho = sqrt(_rho * rho_);
  R U = (temp5 * _U + temp6 * U_) / temp4;
  R V = (temp5 * _V + temp6 * V_) / temp4;
  R W = (temp5 * _W + temp6 * W_) / temp4;
  R VV = U * U + V * V + W * W;
  R H = (temp5 * _H + temp6 * H_) / temp4;
  R C = (H - (R)0.5 * VV) * Km1;
  R q = VV / C;
  R beta = q > e ? q : e;
  const R un = AX == 0 ? U : (AX == 1 ? V : W);
  const R _un = AX == 0 ? _U : (AX == 1 ? _V : _W);
  const R un_ = AX == 0 ? U_ : (AX == 1 ? V_ : W_);
  R temp = (R)0.5 * ((R)1 + beta) * un;
  R Sp = (R)0.5 * sqrt((R)4 * beta * C + un * un * ((R)1 - beta) * ((R)1 - beta));
  R temp1 = (P_ - _P) / rho / beta / C;
  R tS = temp / Sp;
  R temp2 = tS * (un_ - _un);
  R temp3 = (R)0.5 * ((R)1 - beta) * un * temp / Sp;
  R an = fabs(un);
  R deltaU = (Sp - temp3 - beta * an) * temp1 + temp2;
  R deltaP = tS * (P_ - _P) + (Sp - an + temp3) * rho * (un_ - _un);
  R dr = deltaU * rho;
  R Fav1 = an * dU1 + dr;
  R Fav2 = an * dU2 + dr * U;
  R Fav3 = an * dU3 + dr * V;
  R Fav4 = an * dU4 + dr * W;
  if (AX == 0) Fav2 = Fav2 + deltaP;
  if (AX == 1) Fav3 = Fav3 + deltaP;
  if (AX == 2) Fav4 = Fav4 + deltaP;
  R Fav5 = an * dU5 + dr * H + deltaP * un;
  F[0] = (R)0.5 * ((_rho * _un + rho_ * un_) - Fav1);
  F[1] = AX == 0 ? (R)0.5 * ((_rho * _U * _U + _P + rho_ * U_ * U_ + P_) - Fav2)
                 : (R)0.5 * ((_rho * _U * _un + rho_ * U_ * un_) - Fav2);
  F[2] = AX == 1 ? (R)0.5 * ((_rho * _V * _V + _P + rho_ * V_ * V_ + P_) - Fav3)
                 : (R)0.5 * ((_rho * _V * _un + rho_ * V_ * un_) - Fav3);
  F[3] = AX == 2 ? (R)0.5 * ((_rho * _W * _W + _P + rho_ * W_ * W_ + P_) - Fav4)
                 : (R)0.5 * ((_rho * _W * _un + rho_ * W_ * un_) - Fav4);
  F[4] = (R)0.5 * ((_un * ((R)3.5 * _P + (R)0.5 * _rho * _VV) +
                    un_ * ((R)3.5 * P_ + (R)0.5 * rho_ * VV_)) - Fav5);
  dP = (R)0.5 * (_P + P_);
}

// Reconstruction order a cell uses for its backward face (view of the cell on
// the + side) and forward face (view of the cell on the - side), from the
// flags along the axis (BCM_Flux...cpp:497-596).  g is the + cell's index
// along the axis, fm2..fp1 the flags at g-2..g+1, nx = n+1.
__device__ __forceinline__ int order_backward(int g, int fm2, int fm1, int fp1) {
  if (!(fp1 == kFluid && fm1 == kFluid)) return 1;
  return (g == 2 || fm2 != kFluid) ? 3 : 5;
}
__device__ __forceinline__ int order_forward(int g, int nx, int fm2, int f0, int fp1) {
  if (!(f0 == kFluid && fm2 == kFluid)) return 1;
  return (g - 1 == nx || fp1 != kFluid) ? 3 : 5;
}

// Left/right states at the face between g-1 and g for a given order.  um3..up2
// point at the 5-vectors of cells g-3..g+2 (only those the order needs are
// touched).  Both views of one face produce identical (ML, MR) for equal
// orders, which is what lets a face be evaluated once.
template <typename R, typename Ld>
__device__ __forceinline__ void recon(int ord, Ld ld, R *ML, R *MR) {
  if (ord == 5) {
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      R a = ld(-3, v), b = ld(-2, v), c = ld(-1, v), d = ld(0, v), f = ld(1, v), g = ld(2, v);
      ML[v] = (R)(1. / 60) * ((R)2 * a - (R)13 * b + (R)47 * c + (R)27 * d - (R)3 * f);
      MR[v] = (R)(1. / 60) * ((R)-3 * b + (R)27 * c + (R)47 * d - (R)13 * f + (R)2 * g);
    }
  } else if (ord == 3) {
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      R b = ld(-2, v), c = ld(-1, v), d = ld(0, v), f = ld(1, v);
      ML[v] = (R)(1. / 6) * ((R)-1 * b + (R)5 * c + (R)2 * d);
      MR[v] = (R)(1. / 6) * ((R)2 * c + (R)5 * d - (R)1 * f);
    }
  } else {
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      ML[v] = ld(-1, v);
      MR[v] = ld(0, v);
    }
  }
}

}  // namespace bcmg
