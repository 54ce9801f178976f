// FP64 residual + pointwise-preconditioned increment for one RK stage.
//
// Replaces the cube loop of BCM_Flux_XYZ_Viscous_Runge_kutta
// (BCM_Flux_XYZ_Viscous_Runge_kutta.cpp:326-2411): for every interior cell
// it forms the BDF2 source, the upwind-biased inviscid flux balance, the
// viscous flux balance and Rku1 = dTau * D * Rk (0 on non-fluid cells), and
// the force integrands in Residual1 on non-fluid cells.  The RK combination
// itself runs in bcm_rk.cu once all increments exist (the reference also
// runs it after its cube loop, :2417-2599: cells read each other's old
// state).
//
// GB300 design: FP64 runs at a small fraction of the FP32 rate on this part,
// so the kernel does less FP64 work than the reference without changing a
// single rounding:
//  * one CTA per T^3 tile of a cube; the primitive variables (u,v,w,T) of
//    the tile plus a one-cell halo are formed once into shared memory
//    instead of 18 times per cell (the reference converts each neighbour
//    inside every cell's body, :1729-1895);
//  * each inviscid face flux is evaluated once and used by both cells that
//    share the face whenever both cells pick the same reconstruction order
//    (then their left/right states are identical bit for bit); only faces
//    next to non-fluid flags or cube edges get two evaluations;
//  * everything else keeps the reference's expression order, and this
//    translation unit is compiled with --fmad=false, so every value equals
//    the reference's (checked against the C oracle in tests/).
#include <cuda_runtime.h>

#include "bcm_common.cuh"
#include "bcm_kernels.h"

namespace bcmg {

struct Prim {
  double U, V, W, T;  // T = P/(rho*R): the neighbour form (:1734)
};

template <int T>
struct FluxSmem {
  static constexpr int B = T + 2;  // primitive box edge
  static constexpr int nPrim = B * B * B;
  static constexpr int nCell = T * T * T;
  static constexpr size_t bytes = sizeof(Prim) * nPrim + sizeof(double) * nCell /*Tc*/ +
                                  2 * sizeof(double) * 5 * nCell /*Fb, Ff*/ +
                                  2 * sizeof(double) * nCell /*dPb, dPf*/;
};

__device__ __forceinline__ Prim prim_of(double q0, double q1, double q2, double q3,
                                        double q4) {
  Prim p;
  double rho = q0;
  p.U = q1 / rho;
  p.V = q2 / rho;
  p.W = q3 / rho;
  double P = (q4 - 0.5 * rho * (p.U * p.U + p.V * p.V + p.W * p.W)) * (BCMG_K - 1);
  p.T = P / (rho * BCMG_R);
  return p;
}

// Viscous face (BCM_Flux...cpp:1906-2265).  c/o are the centre and normal
// neighbour primitives, Tc the centre temperature in its P/rho/R form,
// a0..a3 / b0..b3 the terms of the two transverse central differences in the
// reference's (a + b - c - d) order (transverse axes in x<y<z order).
template <int AX, bool FWD>
__device__ __forceinline__ void visc_face(double mu_L, double T0, double Tc, const Prim &c,
                                          const Prim &o, double inv, const Prim &a0,
                                          const Prim &a1, const Prim &a2, const Prim &a3,
                                          const Prim &b0, const Prim &b1, const Prim &b2,
                                          const Prim &b3, double *L) {
  double Tm = 0.5 * (Tc + o.T);
  double temp = Tm / T0;
  double mu_E = mu_L * temp * sqrt(temp) * (T0 + 110.) / (Tm + 110.);
  double gn[4];
  if (FWD) {
    gn[0] = (o.U - c.U) * inv; gn[1] = (o.V - c.V) * inv;
    gn[2] = (o.W - c.W) * inv; gn[3] = (o.T - Tc) * inv;
  } else {
    gn[0] = (c.U - o.U) * inv; gn[1] = (c.V - o.V) * inv;
    gn[2] = (c.W - o.W) * inv; gn[3] = (Tc - o.T) * inv;
  }
  double ga[3], gb[3];
  ga[0] = (a0.U + a1.U - a2.U - a3.U) / 4 * inv;
  ga[1] = (a0.V + a1.V - a2.V - a3.V) / 4 * inv;
  ga[2] = (a0.W + a1.W - a2.W - a3.W) / 4 * inv;
  gb[0] = (b0.U + b1.U - b2.U - b3.U) / 4 * inv;
  gb[1] = (b0.V + b1.V - b2.V - b3.V) / 4 * inv;
  gb[2] = (b0.W + b1.W - b2.W - b3.W) / 4 * inv;
  double d[3][3];
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    d[AX][m] = gn[m];
    d[AX == 0 ? 1 : 0][m] = ga[m];
    d[AX == 2 ? 1 : 2][m] = gb[m];
  }
  const double du_dx = d[0][0], dv_dx = d[0][1], dw_dx = d[0][2];
  const double du_dy = d[1][0], dv_dy = d[1][1], dw_dy = d[1][2];
  const double du_dz = d[2][0], dv_dz = d[2][1], dw_dz = d[2][2];
  double Um = 0.5 * (c.U + o.U), Vm = 0.5 * (c.V + o.V), Wm = 0.5 * (c.W + o.W);
  double div = du_dx + dv_dy + dw_dz;
  double s1, s2, s3;
  if (AX == 0) {
    s1 = mu_E * (2 * du_dx - 2.0 / 3.0 * div);
    s2 = mu_E * (du_dy + dv_dx);
    s3 = mu_E * (du_dz + dw_dx);
  } else if (AX == 1) {
    s1 = mu_E * (du_dy + dv_dx);
    s2 = mu_E * (2 * dv_dy - 2.0 / 3.0 * div);
    s3 = mu_E * (dv_dz + dw_dy);
  } else {
    s1 = mu_E * (du_dz + dw_dx);
    s2 = mu_E * (dv_dz + dw_dy);
    s3 = mu_E * (2 * dw_dz - 2.0 / 3.0 * div);
  }
  L[0] = s1;
  L[1] = s2;
  L[2] = s3;
  L[3] = Um * s1 + Vm * s2 + Wm * s3 + mu_E * BCMG_CV * BCMG_K * gn[3] / (BCMG_PR);
}

template <int T, bool VISCOUS>
__global__ void __launch_bounds__(T *T *T, 1) k_flux_fp64(FluxArgs a) {
  using SM = FluxSmem<T>;
  constexpr int B = SM::B;
  constexpr int NT = T * T * T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Prim *prim = reinterpret_cast<Prim *>(smem_raw);
  double *Tcs = reinterpret_cast<double *>(prim + SM::nPrim);
  double *Fb = Tcs + SM::nCell;
  double *Ff = Fb + 5 * SM::nCell;
  double *dPb = Ff + 5 * SM::nCell;
  double *dPf = dPb + SM::nCell;

  const int n = a.ph.n, S = n + 4, nx = n + 1;
  const int nt = n / T;
  const int tid = threadIdx.x;
  const int tiles = nt * nt * nt;
  const int cube = a.cube0 + blockIdx.x / tiles;
  if (!case_active(a.bt, cube)) return;  // converged case (uniform per CTA)
  const int tl = blockIdx.x % tiles;
  const int bi = 2 + (tl / (nt * nt)) * T, bj = 2 + ((tl / nt) % nt) * T, bk = 2 + (tl % nt) * T;
  const double *__restrict__ U = a.U1_;
  const int *__restrict__ F = a.FWS;
  const size_t cb = cell_index(S, cube, 0, 0, 0);
  // Constants of the cube's case (kernel arguments for a single case).
  double e = a.e, dT = a.dT, dTau = a.dTau, mu_L = a.ph.mu_L, rho0 = a.ph.rho0, P0 = a.ph.P0;
  if (a.bt.cube_case) {
    const CaseConst *q = a.bt.cases + __ldg(a.bt.cube_case + cube);
    e = q->e; dT = q->dT; dTau = q->dTau; mu_L = q->mu_L; rho0 = q->rho0; P0 = q->P0;
  }

  // Phase 1: primitives over the tile plus a one-cell halo (edges included).
  for (int p = tid; p < SM::nPrim; p += NT) {
    int li = p / (B * B), lj = (p / B) % B, lk = p % B;
    const double *q =
        U + 5 * (cb + ((size_t)(bi - 1 + li) * S + (bj - 1 + lj)) * S + (bk - 1 + lk));
    double q0 = __ldg(q), q1 = __ldg(q + 1), q2 = __ldg(q + 2), q3 = __ldg(q + 3),
           q4 = __ldg(q + 4);
    Prim pr = prim_of(q0, q1, q2, q3, q4);
    prim[p] = pr;
    if (li >= 1 && li <= T && lj >= 1 && lj <= T && lk >= 1 && lk <= T) {
      // Centre temperature as the viscous block forms it: P/rho/R (:1841).
      double VV = pr.U * pr.U + pr.V * pr.V + pr.W * pr.W;
      double P = (q4 - 0.5 * q0 * VV) * (BCMG_K - 1);
      Tcs[((li - 1) * T + (lj - 1)) * T + (lk - 1)] = P / q0 / BCMG_R;
    }
  }

  const double dx = a.cube_size[cube] / n;
  const double inv = 1. / dx;
  double acc[5];
  double dPdx = 0, dPdz = 0;  // dPf - dPb for the force integrands

  // Phase 2: inviscid face fluxes, axis by axis in x, y, z order so that the
  // per-cell sum Rfx/dx + Rfy/dy + Rfz/dz keeps the reference's order (:1710).
#pragma unroll 1
  for (int ax = 0; ax < 3; ++ax) {
    for (int f = tid; f < (T + 1) * T * T; f += NT) {
      const int fa = f / (T * T), p = (f / T) % T, q = f % T;
      int li, lj, lk;  // local index of the + cell of this face (fa may be T)
      if (ax == 0) { li = fa; lj = p; lk = q; }
      else if (ax == 1) { li = p; lj = fa; lk = q; }
      else { li = p; lj = q; lk = fa; }
      const int g = (ax == 0 ? bi + li : (ax == 1 ? bj + lj : bk + lk));
      const ptrdiff_t stride = ax == 0 ? (ptrdiff_t)S * S : (ax == 1 ? (ptrdiff_t)S : 1);
      const size_t c0 = cb + ((size_t)(bi + li) * S + (bj + lj)) * S + (bk + lk);
      const int fm2 = __ldg(F + c0 - 2 * stride), fm1 = __ldg(F + c0 - stride),
                f0 = __ldg(F + c0), fp1 = __ldg(F + c0 + stride);
      const bool needB = fa < T, needF = fa > 0;
      const int ob = order_backward(g, fm2, fm1, fp1);
      const int of = order_forward(g, nx, fm2, f0, fp1);
      const int slotB = (li * T + lj) * T + lk;  // valid when needB
      const int slotF = slotB - (ax == 0 ? T * T : (ax == 1 ? T : 1));  // valid when needF
      int nviews, ord0, ord1 = 0, dst0, dst1 = 0;  // dst bit0 backward, bit1 forward
      if (needB && needF && ob == of) { nviews = 1; ord0 = ob; dst0 = 3; }
      else if (needB && needF) { nviews = 2; ord0 = ob; dst0 = 1; ord1 = of; dst1 = 2; }
      else if (needB) { nviews = 1; ord0 = ob; dst0 = 1; }
      else { nviews = 1; ord0 = of; dst0 = 2; }
      const double *base = U + 5 * c0;
      auto ld = [&](int d, int v) -> double { return __ldg(base + 5 * stride * d + v); };
#pragma unroll 1
      for (int w = 0; w < nviews; ++w) {
        const int ord = w == 0 ? ord0 : ord1;
        const int dst = w == 0 ? dst0 : dst1;
        double ML[5], MR[5], Fx[5], dP;
        recon<double>(ord, ld, ML, MR);
        if (ax == 0) face_flux<0, double>(ML, MR, e, Fx, dP);
        else if (ax == 1) face_flux<1, double>(ML, MR, e, Fx, dP);
        else face_flux<2, double>(ML, MR, e, Fx, dP);
        if (dst & 1) {
#pragma unroll
          for (int v = 0; v < 5; ++v) Fb[5 * slotB + v] = Fx[v];
          dPb[slotB] = dP;
        }
        if (dst & 2) {
#pragma unroll
          for (int v = 0; v < 5; ++v) Ff[5 * slotF + v] = Fx[v];
          dPf[slotF] = dP;
        }
      }
    }
    __syncthreads();
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      double t = (Ff[5 * tid + v] - Fb[5 * tid + v]) / dx;
      acc[v] = ax == 0 ? t : acc[v] + t;
    }
    if (ax == 0) dPdx = dPf[tid] - dPb[tid];
    if (ax == 2) dPdz = dPf[tid] - dPb[tid];
    __syncthreads();
  }

  // Phase 3: viscous fluxes from the shared primitives (own cell).
  const int mi = tid / (T * T), mj = (tid / T) % T, mk = tid % T;
  auto P = [&](int di, int dj, int dk) -> const Prim & {
    return prim[((mi + 1 + di) * B + (mj + 1 + dj)) * B + (mk + 1 + dk)];
  };
  const Prim &c = P(0, 0, 0);
  double vF[5] = {0, 0, 0, 0, 0};
  if (VISCOUS) {
    const double T0 = P0 / rho0 / BCMG_R;
    const double Tc = Tcs[tid];
    double Lb[4], Lf[4], Mb[4], Mf[4], Nb[4], Nf[4];
    visc_face<0, false>(mu_L, T0, Tc, c, P(-1, 0, 0), inv, P(0, 1, 0), P(-1, 1, 0), P(0, -1, 0),
                        P(-1, -1, 0), P(0, 0, 1), P(-1, 0, 1), P(0, 0, -1), P(-1, 0, -1), Lb);
    visc_face<0, true>(mu_L, T0, Tc, c, P(1, 0, 0), inv, P(0, 1, 0), P(1, 1, 0), P(0, -1, 0),
                       P(1, -1, 0), P(0, 0, 1), P(1, 0, 1), P(0, 0, -1), P(1, 0, -1), Lf);
    visc_face<1, false>(mu_L, T0, Tc, c, P(0, -1, 0), inv, P(1, 0, 0), P(1, -1, 0), P(-1, 0, 0),
                        P(-1, -1, 0), P(0, 0, 1), P(0, -1, 1), P(0, 0, -1), P(0, -1, -1), Mb);
    visc_face<1, true>(mu_L, T0, Tc, c, P(0, 1, 0), inv, P(1, 0, 0), P(1, 1, 0), P(-1, 0, 0),
                       P(-1, 1, 0), P(0, 0, 1), P(0, 1, 1), P(0, 0, -1), P(0, 1, -1), Mf);
    visc_face<2, false>(mu_L, T0, Tc, c, P(0, 0, -1), inv, P(1, 0, 0), P(1, 0, -1), P(-1, 0, 0),
                        P(-1, 0, -1), P(0, 1, 0), P(0, 1, -1), P(0, -1, 0), P(0, -1, -1), Nb);
    visc_face<2, true>(mu_L, T0, Tc, c, P(0, 0, 1), inv, P(1, 0, 0), P(1, 0, 1), P(-1, 0, 0),
                       P(-1, 0, 1), P(0, 1, 0), P(0, 1, 1), P(0, -1, 0), P(0, -1, 1), Nf);
#pragma unroll
    for (int v = 1; v < 5; ++v)
      vF[v] = (Lf[v - 1] - Lb[v - 1]) * inv + (Mf[v - 1] - Mb[v - 1]) * inv +
              (Nf[v - 1] - Nb[v - 1]) * inv;
  }

  // Phase 4: BDF2 source, preconditioner, increment, force integrands.
  const size_t go = cb + ((size_t)(bi + mi) * S + (bj + mj)) * S + (bk + mk);
  const double *u = U + 5 * go;
  const double *uu = a.U1 + 5 * go;
  const double *uq = a.U1q + 5 * go;
  const int IF = __ldg(F + go);
  double Rk[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    double Rp = -(3 * __ldg(u + v) - 4 * __ldg(uu + v) + __ldg(uq + v)) / (2 * dT);
    double Rf = -acc[v];
    Rk[v] = v == 0 ? Rp + Rf : Rp + Rf + vF[v];
  }
  double *rk = a.Rku1 + 5 * go;
  if (IF == kFluid && a.raw) {
#pragma unroll
    for (int r = 0; r < 5; ++r) rk[r] = Rk[r];
  } else if (IF == kFluid) {
    const double K = BCMG_K;
    const double rho = __ldg(u);
    const double Uc = c.U, Vc = c.V, Wc = c.W;
    const double VV = Uc * Uc + Vc * Vc + Wc * Wc;
    const double Pc = (__ldg(u + 4) - 0.5 * rho * VV) * (BCMG_K - 1);
    const double C = K * Pc / rho;
    const double Tt = Pc / rho;
    const double H = 0.5 * VV + C / (BCMG_K - 1);
    const double qv = VV / C;
    const double beta = qv > e ? qv : e;
    const double temp = K * Tt * (2 * dT + 3 * dTau) * (2 * dT + 3 * beta * dTau);
    const double temp2 = (BCMG_K - 1) * (beta - 1) * dT * dT;
    const double temp3 = H - H * K - VV + K * (Tt + VV);
    double d[5][5];
    d[0][0] = (2 * dT * (-2 * (-(BCMG_K - 1) * (H - VV) - temp3 * beta) * dT + 3 * K * Tt * beta * dTau)) / temp;
    d[0][1] = (-4 * Uc * temp2) / temp;
    d[0][2] = (-4 * Vc * temp2) / temp;
    d[0][3] = (-4 * Wc * temp2) / temp;
    d[0][4] = (4 * temp2) / temp;
    d[1][0] = (4 * Uc * temp3 * (beta - 1) * dT * dT) / temp;
    d[1][1] = (2 * dT * (2 * K * (Tt - Uc * Uc * (beta - 1)) * dT + 2 * Uc * Uc * (beta - 1) * dT + 3 * K * Tt * beta * dTau)) / temp;
    d[1][2] = (-4 * Uc * Vc * temp2) / temp;
    d[1][3] = (-4 * Uc * Wc * temp2) / temp;
    d[1][4] = (4 * Uc * temp2) / temp;
    d[2][0] = (4 * Vc * temp3 * (beta - 1) * dT * dT) / temp;
    d[2][1] = (-4 * Uc * Vc * temp2) / temp;
    d[2][2] = (2 * dT * (2 * K * (Tt - Vc * Vc * (beta - 1)) * dT + 2 * Vc * Vc * (beta - 1) * dT + 3 * K * Tt * beta * dTau)) / temp;
    d[2][3] = (-4 * Vc * Wc * temp2) / temp;
    d[2][4] = (4 * Vc * temp2) / temp;
    d[3][0] = (4 * Wc * temp3 * (beta - 1) * dT * dT) / temp;
    d[3][1] = (-4 * Uc * Wc * temp2) / temp;
    d[3][2] = (-4 * Vc * Wc * temp2) / temp;
    d[3][3] = (2 * dT * (2 * K * (Tt - Wc * Wc * (beta - 1)) * dT + 2 * Wc * Wc * (beta - 1) * dT + 3 * K * Tt * beta * dTau)) / temp;
    d[3][4] = (4 * Wc * temp2) / temp;
    d[4][0] = (4 * H * temp3 * (beta - 1) * dT * dT) / temp;
    d[4][1] = (-4 * H * Uc * temp2) / temp;
    d[4][2] = (-4 * H * Vc * temp2) / temp;
    d[4][3] = (-4 * H * Wc * temp2) / temp;
    d[4][4] = (2 * dT * (2 * H * (BCMG_K - 1) * (beta - 1) * dT + K * Tt * (2 * dT + 3 * beta * dTau))) / temp;
#pragma unroll
    for (int r = 0; r < 5; ++r)
      rk[r] = dTau * (d[r][0] * Rk[0] + d[r][1] * Rk[1] + d[r][2] * Rk[2] + d[r][3] * Rk[3] +
                      d[r][4] * Rk[4]);
  } else {
#pragma unroll
    for (int r = 0; r < 5; ++r) rk[r] = 0;
    // Force integrands on non-fluid cells (:2395-2398).
    const double dV = dx;  // dx = dy = dz
    a.Residual1[5 * go + 0] = -(-(dPdx) / dx + vF[1]) * dx * dV * dV;
    a.Residual1[5 * go + 1] = -(-(dPdz) / dV + vF[3]) * dx * dV * dV;
  }
}

template <int T>
static cudaError_t launch_t(const FluxArgs &a, int ncubes, cudaStream_t s) {
  const int nt = a.ph.n / T;
  const size_t smem = FluxSmem<T>::bytes;
  const unsigned grid = (unsigned)(ncubes * nt * nt * nt);
  if (grid == 0) return cudaSuccess;
  cudaError_t e;
  if (a.ph.mu_L != 0.0) {
    e = cudaFuncSetAttribute(k_flux_fp64<T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
    if (e != cudaSuccess) return e;
    k_flux_fp64<T, true><<<grid, T * T * T, smem, s>>>(a);
  } else {
    e = cudaFuncSetAttribute(k_flux_fp64<T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
    if (e != cudaSuccess) return e;
    k_flux_fp64<T, false><<<grid, T * T * T, smem, s>>>(a);
  }
  return cudaGetLastError();
}

// Cubes [a.cube0, a.cube0 + ncubes) of the flat list.
cudaError_t launch_flux_fp64(const FluxArgs &a, int ncubes, cudaStream_t s) {
  if (a.ph.n % 4 != 0) return cudaErrorInvalidValue;
  if (flux_tile(a.ph.n, a.tile) == 8) return launch_t<8>(a, ncubes, s);
  return launch_t<4>(a, ncubes, s);
}

}  // namespace bcmg
