/*
 * ORACLE (test infrastructure; never part of the product path).
 *
 * A plain-C restatement of BCM_CGLI's per-stage hot path, runtime-sized in the
 * cube resolution, used as the CPU checker for the CUDA kernels and as the
 * "port" CPU baseline.  Every routine keeps the reference's IEEE operation
 * order so that, built with -ffp-contract=off, it reproduces the reference's
 * results bit for bit; that equality is pinned by tests/test_oracle_golden.py
 * against fixtures generated from the reference's own compiled sources
 * (oracle/ref_build.py, tests/golden/make_golden.py).
 *
 * Layout (same as the reference, Array.h:13-25): U[c][i][j][k][v] with
 * S = n+4 cells per edge (two ghost layers each side), v fastest; cube 0 is
 * unused (1-based cube numbering, main.cpp:90).  FWS[c][i][j][k] is the flag
 * (1 fluid, 0 IBM ghost, -1 solid; BCM.h:6-8).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "bcm_oracle.h"
#ifdef _OPENMP
#include <omp.h>
#endif

/* Thread count for the per-cell loops (results do not depend on it: every
 * order-sensitive reduction below runs serially). */
void bcmo_set_threads(int n) {
#ifdef _OPENMP
  omp_set_num_threads(n > 0 ? n : 1);
#else
  (void)n;
#endif
}

#define IFLUID 1
#define KG 1.4        /* K, prm.h:1 */
#define RGAS 287      /* R, prm.h:2 (an int in the reference) */
#define CV 717.5      /* Cv, prm.h:4 */
#define PR_L 0.72     /* Pr_L, prm.h:6 */

static inline size_t at(int S, int c, int i, int j, int k) {
  return ((((size_t)c * S + i) * S + j) * S + k);
}

/* ------------------------------------------------------------------------ */
/* Inviscid face flux.  BCM_Flux_XYZ_Viscous_Runge_kutta.cpp:606-693 (Z),     */
/* :1057-1146 (X), :1503-1594 (Y): the same preconditioned Roe-type flux with  */
/* the normal velocity component nd (0 x, 1 y, 2 z).  ML/MR are the left and  */
/* right reconstructed conservative states; F receives the flux and *dP the   */
/* face pressure 0.5*(pL+pR) used by the force integrand.                    */
/* ------------------------------------------------------------------------ */
static void face_flux(const double *ML, const double *MR, int nd, double e, double *F,
                      double *dP) {
  double dU1 = MR[0] - ML[0], dU2 = MR[1] - ML[1], dU3 = MR[2] - ML[2],
         dU4 = MR[3] - ML[3], dU5 = MR[4] - ML[4];
  double _rho = ML[0];
  double _U = ML[1] / _rho, _V = ML[2] / _rho, _W = ML[3] / _rho;
  double _VV = _U * _U + _V * _V + _W * _W;
  double _P = (ML[4] - 0.5 * _rho * _VV) * (KG - 1);
  double _C = KG * _P / _rho;
  double _H = 0.5 * _VV + _C / (KG - 1);
  double rho_ = MR[0];
  double U_ = MR[1] / rho_, V_ = MR[2] / rho_, W_ = MR[3] / rho_;
  double VV_ = U_ * U_ + V_ * V_ + W_ * W_;
  double P_ = (MR[4] - 0.5 * rho_ * VV_) * (KG - 1);
  double C_ = KG * P_ / rho_;
  double H_ = 0.5 * VV_ + C_ / (KG - 1);
  double temp5 = sqrt(_rho), temp6 = sqrt(rho_);
  double temp4 = temp5 + temp6;
  double rho = sqrt(_rho * rho_);
  double U = (temp5 * _U + temp6 * U_) / temp4;
  double V = (temp5 * _V + temp6 * V_) / temp4;
  double W = (temp5 * _W + temp6 * W_) / temp4;
  double VV = U * U + V * V + W * W;
  double H = (temp5 * _H + temp6 * H_) / temp4;
  double C = (H - 0.5 * VV) * (KG - 1);
  double q = VV / C;
  double beta = q > e ? q : e;
  double un = nd == 0 ? U : (nd == 1 ? V : W);
  double _un = nd == 0 ? _U : (nd == 1 ? _V : _W);
  double un_ = nd == 0 ? U_ : (nd == 1 ? V_ : W_);
  double temp = 0.5 * (1 + beta) * un;
  double S = 0.5 * sqrt(4 * beta * C + un * un * (1 - beta) * (1 - beta));
  double temp1 = (P_ - _P) / rho / beta / C;
  double temp2 = temp / S * (un_ - _un);
  double temp3 = 0.5 * (1 - beta) * un * temp / S;
  double deltaU = (S - temp3 - beta * fabs(un)) * temp1 + temp2;
  double deltaP = temp / S * (P_ - _P) + (S - fabs(un) + temp3) * rho * (un_ - _un);
  double an = fabs(un);
  double Fav1 = an * dU1 + deltaU * rho;
  double Fav2 = an * dU2 + deltaU * rho * U;
  double Fav3 = an * dU3 + deltaU * rho * V;
  double Fav4 = an * dU4 + deltaU * rho * W;
  if (nd == 0) Fav2 = Fav2 + deltaP;
  if (nd == 1) Fav3 = Fav3 + deltaP;
  if (nd == 2) Fav4 = Fav4 + deltaP;
  double Fav5 = an * dU5 + deltaU * rho * H + deltaP * un;
  F[0] = 0.5 * ((_rho * _un + rho_ * un_) - Fav1);
  double _vm[3] = {_U, _V, _W}, vm_[3] = {U_, V_, W_};
  double Fm[3] = {Fav2, Fav3, Fav4};
  for (int m = 0; m < 3; ++m) {
    if (m == nd)
      F[1 + m] = 0.5 * ((_rho * _vm[m] * _vm[m] + _P + rho_ * vm_[m] * vm_[m] + P_) - Fm[m]);
    else
      F[1 + m] = 0.5 * ((_rho * _vm[m] * _un + rho_ * vm_[m] * un_) - Fm[m]);
  }
  F[4] = 0.5 * ((_un * (3.5 * _P + 0.5 * _rho * _VV) + un_ * (3.5 * P_ + 0.5 * rho_ * VV_)) - Fav5);
  *dP = 0.5 * (_P + P_);
}

/* Reconstruction along one axis (BCM_Flux...cpp:497-596 for Z, :945-1044 X,
 * :1393-1492 Y).  u[-3..3] are the 5-vectors along the axis (u[0] the cell),
 * f[-2..2] the flags, pos the cell's index on that axis and n the interior
 * size.  Outputs the backward face (ML, MR) and forward face (MLi, MRi). */
static void reconstruct(const double *const *u, const int *f, int pos, int n, double *ML,
                        double *MR, double *MLi, double *MRi) {
  const double *m3 = u[0], *m2 = u[1], *m1 = u[2], *c0 = u[3], *p1 = u[4], *p2 = u[5],
               *p3 = u[6];
  int IF_1 = f[1], IF_2 = f[0], IF1 = f[3], IF2 = f[4];
  int nxpos = n + 1; /* nx (Resolution.h:12) */
  if (IF1 == IFLUID && IF_1 == IFLUID) {
    if ((pos == 2) | (IF_2 != IFLUID)) {
      for (int v = 0; v < 5; ++v) {
        ML[v] = 1. / 6 * (-1 * m2[v] + 5 * m1[v] + 2 * c0[v]);
        MR[v] = 1. / 6 * (2 * m1[v] + 5 * c0[v] - 1 * p1[v]);
      }
    } else {
      for (int v = 0; v < 5; ++v) {
        ML[v] = 1. / 60 * (2 * m3[v] - 13 * m2[v] + 47 * m1[v] + 27 * c0[v] - 3 * p1[v]);
        MR[v] = 1. / 60 * (-3 * m2[v] + 27 * m1[v] + 47 * c0[v] - 13 * p1[v] + 2 * p2[v]);
      }
    }
    if ((pos == nxpos) | (IF2 != IFLUID)) {
      for (int v = 0; v < 5; ++v) {
        MLi[v] = 1. / 6 * (-1 * m1[v] + 5 * c0[v] + 2 * p1[v]);
        MRi[v] = 1. / 6 * (2 * c0[v] + 5 * p1[v] - 1 * p2[v]);
      }
    } else {
      for (int v = 0; v < 5; ++v) {
        MLi[v] = 1. / 60 * (2 * m2[v] - 13 * m1[v] + 47 * c0[v] + 27 * p1[v] - 3 * p2[v]);
        MRi[v] = 1. / 60 * (-3 * m1[v] + 27 * c0[v] + 47 * p1[v] - 13 * p2[v] + 2 * p3[v]);
      }
    }
  } else {
    for (int v = 0; v < 5; ++v) {
      ML[v] = m1[v];
      MR[v] = c0[v];
      MLi[v] = c0[v];
      MRi[v] = p1[v];
    }
  }
}

/* Primitive (U,V,W,T) of a neighbour cell as the viscous block computes it
 * (BCM_Flux...cpp:1729-1895): T = P/(rho*R). */
typedef struct { double U, V, W, T; } prim_t;
static inline prim_t prim_nb(const double *q) {
  prim_t p;
  double rho = q[0];
  p.U = q[1] / rho;
  p.V = q[2] / rho;
  p.W = q[3] / rho;
  double P = (q[4] - 0.5 * rho * (p.U * p.U + p.V * p.V + p.W * p.W)) * (KG - 1);
  p.T = P / (rho * RGAS);
  return p;
}

/* Viscous face flux components 2..5 (BCM_Flux...cpp:1906-2265).  axis is the
 * face normal; sgn +1 forward face / -1 backward face.  c is the centre
 * primitive (with T = P/rho/R), o the normal neighbour, and g1/g2 the
 * transverse central differences' four terms as the reference orders them. */
static void visc_face(double mu_L, double T0, prim_t c, prim_t o, int axis, int fwd,
                      const double dxa[3], const double *tU, const double *tV,
                      const double *tW, const double *tT, double *L) {
  /* tX[4*t + 0..3] = the four values in (a + b - c - d) order for the two
   * transverse axes t=0,1 (in x<y<z order, skipping axis). */
  double Tm = 0.5 * (c.T + o.T);
  double temp = Tm / T0;
  double mu_E = mu_L * temp * sqrt(temp) * (T0 + 110.) / (Tm + 110.);
  double Pr_E = PR_L;
  double g[3][4]; /* d(u,v,w,T)/d(x,y,z) */
  double inv = dxa[axis];
  if (fwd) {
    g[axis][0] = (o.U - c.U) * inv;
    g[axis][1] = (o.V - c.V) * inv;
    g[axis][2] = (o.W - c.W) * inv;
    g[axis][3] = (o.T - c.T) * inv;
  } else {
    g[axis][0] = (c.U - o.U) * inv;
    g[axis][1] = (c.V - o.V) * inv;
    g[axis][2] = (c.W - o.W) * inv;
    g[axis][3] = (c.T - o.T) * inv;
  }
  int t = 0;
  for (int a = 0; a < 3; ++a) {
    if (a == axis) continue;
    const double *qU = tU + 4 * t, *qV = tV + 4 * t, *qW = tW + 4 * t, *qT = tT + 4 * t;
    g[a][0] = (qU[0] + qU[1] - qU[2] - qU[3]) / 4 * dxa[a];
    g[a][1] = (qV[0] + qV[1] - qV[2] - qV[3]) / 4 * dxa[a];
    g[a][2] = (qW[0] + qW[1] - qW[2] - qW[3]) / 4 * dxa[a];
    g[a][3] = (qT[0] + qT[1] - qT[2] - qT[3]) / 4 * dxa[a];
    ++t;
  }
  double du_dx = g[0][0], dv_dx = g[0][1], dw_dx = g[0][2];
  double du_dy = g[1][0], dv_dy = g[1][1], dw_dy = g[1][2];
  double du_dz = g[2][0], dv_dz = g[2][1], dw_dz = g[2][2];
  double dT = g[axis][3];
  double Um = 0.5 * (c.U + o.U), Vm = 0.5 * (c.V + o.V), Wm = 0.5 * (c.W + o.W);
  double div = du_dx + dv_dy + dw_dz;
  double s1, s2, s3;
  if (axis == 0) {
    s1 = mu_E * (2 * du_dx - 2.0 / 3.0 * div);
    s2 = mu_E * (du_dy + dv_dx);
    s3 = mu_E * (du_dz + dw_dx);
  } else if (axis == 1) {
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
  L[3] = Um * s1 + Vm * s2 + Wm * s3 + mu_E * CV * KG * dT / (Pr_E);
}

/* ------------------------------------------------------------------------ */
/* One RK stage of BCM_Flux_XYZ_Viscous_Runge_kutta (BCM_Flux...cpp:18-2659). */
/* ------------------------------------------------------------------------ */
void bcmo_flux_stage(const bcmo_phys *ph, int ncube, int RK, double deltaT, double deltaTau,
                     double e, const int *FWS, const double *cube_size, double *U1_,
                     const double *U1, const double *U1q, double *U1p1, double *U1p2,
                     double *Rku1, double *Residual1, double *er) {
  const int n = ph->n, S = n + 4;
  const int nx = n + 1;
  const double mu_L = ph->mu_L;
  const double T0 = ph->P0 / ph->rho0 / RGAS;

#pragma omp parallel for schedule(dynamic, 1)
  for (int c = 1; c < ncube; ++c) {
    double dx = cube_size[c] / n;
    double dy = dx, dz = dx;
    double inv = 1. / dx;
    double dxa[3] = {inv, inv, inv};
    for (int i = 2; i <= nx; ++i)
      for (int j = 2; j <= nx; ++j)
        for (int k = 2; k <= nx; ++k) {
          size_t o = at(S, c, i, j, k);
          const double *uu = U1 + 5 * o, *uq = U1q + 5 * o, *u = U1_ + 5 * o;
          int IF = FWS[o];
          double Rp[5];
          for (int v = 0; v < 5; ++v) Rp[v] = -(3 * u[v] - 4 * uu[v] + uq[v]) / (2 * deltaT);

          /* Inviscid fluxes: Z, X, Y (reference order; independent). */
          double Rfa[3][5], dPb[3], dPf[3];
          for (int ax = 0; ax < 3; ++ax) {
            const double *s[7];
            int f[5];
            int pos = ax == 0 ? i : (ax == 1 ? j : k);
            for (int d = -3; d <= 3; ++d) {
              int ii = i + (ax == 0 ? d : 0), jj = j + (ax == 1 ? d : 0), kk = k + (ax == 2 ? d : 0);
              /* Out-of-range ends are never used (pos==2 / pos==nx fallbacks). */
              if ((d == -3 && pos <= 2) || (d == 3 && pos >= nx)) { s[d + 3] = u; continue; }
              s[d + 3] = U1_ + 5 * at(S, c, ii, jj, kk);
              if (d >= -2 && d <= 2) f[d + 2] = FWS[at(S, c, ii, jj, kk)];
            }
            double ML[5], MR[5], MLi[5], MRi[5], Fb[5], Ff[5];
            reconstruct(s, f, pos, n, ML, MR, MLi, MRi);
            face_flux(ML, MR, ax, e, Fb, &dPb[ax]);
            face_flux(MLi, MRi, ax, e, Ff, &dPf[ax]);
            for (int v = 0; v < 5; ++v) Rfa[ax][v] = Ff[v] - Fb[v];
          }
          double Rf[5];
          for (int v = 0; v < 5; ++v) Rf[v] = -(Rfa[0][v] / dx + Rfa[1][v] / dy + Rfa[2][v] / dz);

          /* Viscous fluxes. */
#define NB(di, dj, dk) prim_nb(U1_ + 5 * at(S, c, i + (di), j + (dj), k + (dk)))
          prim_t C;
          {
            double rho = u[0];
            C.U = u[1] / u[0];
            C.V = u[2] / u[0];
            C.W = u[3] / u[0];
            double VV = C.U * C.U + C.V * C.V + C.W * C.W;
            double P = (u[4] - 0.5 * rho * VV) * (KG - 1);
            C.T = P / rho / RGAS;
          }
          prim_t im = NB(-1, 0, 0), ip = NB(1, 0, 0), jm = NB(0, -1, 0), jp = NB(0, 1, 0),
                 km = NB(0, 0, -1), kp = NB(0, 0, 1);
          prim_t imjp = NB(-1, 1, 0), imkp = NB(-1, 0, 1), ipjm = NB(1, -1, 0),
                 ipkm = NB(1, 0, -1), jmkp = NB(0, -1, 1), jpkm = NB(0, 1, -1),
                 imjm = NB(-1, -1, 0), jmkm = NB(0, -1, -1), imkm = NB(-1, 0, -1),
                 ipjp = NB(1, 1, 0), ipkp = NB(1, 0, 1), jpkp = NB(0, 1, 1);
#undef NB
          double LLb[4], LLf[4], MLb[4], MLf[4], NLb[4], NLf[4];
#define PACK4(a, b, c_, d, fld) {a.fld, b.fld, c_.fld, d.fld}
#define VISC(axis, fwd, o, A, B, C_, D, E, F_, G, H, out)                                   \
  {                                                                                       \
    double tU[8] = {A.U, B.U, C_.U, D.U, E.U, F_.U, G.U, H.U};                            \
    double tV[8] = {A.V, B.V, C_.V, D.V, E.V, F_.V, G.V, H.V};                            \
    double tW[8] = {A.W, B.W, C_.W, D.W, E.W, F_.W, G.W, H.W};                            \
    double tT[8] = {A.T, B.T, C_.T, D.T, E.T, F_.T, G.T, H.T};                            \
    visc_face(mu_L, T0, C, o, axis, fwd, dxa, tU, tV, tW, tT, out);                        \
  }
          /* X backward (:1920-1968): y terms (Uj+iUj-jU-ijU), z terms (Uk+iUk-kU-ikU). */
          VISC(0, 0, im, jp, imjp, jm, imjm, kp, imkp, km, imkm, LLb);
          /* X forward (:1977-2024): (Uj+Uij-jU-jUi), (Uk+Uik-kU-kUi). */
          VISC(0, 1, ip, jp, ipjp, jm, ipjm, kp, ipkp, km, ipkm, LLf);
          /* Y backward (:2040-2089): x (Ui+jUi-iU-ijU), z (Uk+jUk-kU-jkU). */
          VISC(1, 0, jm, ip, ipjm, im, imjm, kp, jmkp, km, jmkm, MLb);
          /* Y forward (:2099-2144): x (Ui+Uij-iU-iUj), z (Uk+Ujk-kU-kUj). */
          VISC(1, 1, jp, ip, ipjp, im, imjp, kp, jpkp, km, jpkm, MLf);
          /* Z backward (:2159-2208): x (Ui+kUi-iU-ikU), y (Uj+kUj-jU-jkU). */
          VISC(2, 0, km, ip, ipkm, im, imkm, jp, jpkm, jm, jmkm, NLb);
          /* Z forward (:2219-2265): x (Ui+Uik-iU-iUk), y (Uj+Ujk-jU-jUk). */
          VISC(2, 1, kp, ip, ipkp, im, imkp, jp, jpkp, jm, jmkp, NLf);
#undef VISC
#undef PACK4
          double vF[5];
          vF[0] = 0;
          for (int v = 1; v < 5; ++v)
            vF[v] = (LLf[v - 1] - LLb[v - 1]) * dxa[0] + (MLf[v - 1] - MLb[v - 1]) * dxa[1] +
                    (NLf[v - 1] - NLb[v - 1]) * dxa[2];
          double Rk[5];
          Rk[0] = Rp[0] + Rf[0];
          for (int v = 1; v < 5; ++v) Rk[v] = Rp[v] + Rf[v] + vF[v];

          /* Pointwise preconditioner (:2295-2366). */
          double rho = u[0];
          double U = u[1] / u[0], V = u[2] / u[0], W = u[3] / u[0];
          double VV = U * U + V * V + W * W;
          double P = (u[4] - 0.5 * rho * VV) * (KG - 1);
          double Cc = KG * P / rho;
          double T = P / rho;
          double H = 0.5 * VV + Cc / (KG - 1);
          double q = VV / Cc;
          double beta = q > e ? q : e;
          double temp = KG * T * (2 * deltaT + 3 * deltaTau) * (2 * deltaT + 3 * beta * deltaTau);
          double temp2 = (KG - 1) * (beta - 1) * deltaT * deltaT;
          double temp3 = H - H * KG - VV + KG * (T + VV);
          double d[5][5];
          d[0][0] = (2 * deltaT * (-2 * (-(KG - 1) * (H - VV) - temp3 * beta) * deltaT + 3 * KG * T * beta * deltaTau)) / temp;
          d[0][1] = (-4 * U * temp2) / temp;
          d[0][2] = (-4 * V * temp2) / temp;
          d[0][3] = (-4 * W * temp2) / temp;
          d[0][4] = (4 * temp2) / temp;
          d[1][0] = (4 * U * temp3 * (beta - 1) * deltaT * deltaT) / temp;
          d[1][1] = (2 * deltaT * (2 * KG * (T - U * U * (beta - 1)) * deltaT + 2 * U * U * (beta - 1) * deltaT + 3 * KG * T * beta * deltaTau)) / temp;
          d[1][2] = (-4 * U * V * temp2) / temp;
          d[1][3] = (-4 * U * W * temp2) / temp;
          d[1][4] = (4 * U * temp2) / temp;
          d[2][0] = (4 * V * temp3 * (beta - 1) * deltaT * deltaT) / temp;
          d[2][1] = (-4 * U * V * temp2) / temp;
          d[2][2] = (2 * deltaT * (2 * KG * (T - V * V * (beta - 1)) * deltaT + 2 * V * V * (beta - 1) * deltaT + 3 * KG * T * beta * deltaTau)) / temp;
          d[2][3] = (-4 * V * W * temp2) / temp;
          d[2][4] = (4 * V * temp2) / temp;
          d[3][0] = (4 * W * temp3 * (beta - 1) * deltaT * deltaT) / temp;
          d[3][1] = (-4 * U * W * temp2) / temp;
          d[3][2] = (-4 * V * W * temp2) / temp;
          d[3][3] = (2 * deltaT * (2 * KG * (T - W * W * (beta - 1)) * deltaT + 2 * W * W * (beta - 1) * deltaT + 3 * KG * T * beta * deltaTau)) / temp;
          d[3][4] = (4 * W * temp2) / temp;
          d[4][0] = (4 * H * temp3 * (beta - 1) * deltaT * deltaT) / temp;
          d[4][1] = (-4 * H * U * temp2) / temp;
          d[4][2] = (-4 * H * V * temp2) / temp;
          d[4][3] = (-4 * H * W * temp2) / temp;
          d[4][4] = (2 * deltaT * (2 * H * (KG - 1) * (beta - 1) * deltaT + KG * T * (2 * deltaT + 3 * beta * deltaTau))) / temp;
          double *rk = Rku1 + 5 * o;
          if (IF == IFLUID && RK == 0) {
            /* residual only (the LU-SGS sub-iteration's right-hand side) */
            for (int a = 0; a < 5; ++a) rk[a] = Rk[a];
          } else if (IF == IFLUID) {
            for (int a = 0; a < 5; ++a)
              rk[a] = deltaTau * (d[a][0] * Rk[0] + d[a][1] * Rk[1] + d[a][2] * Rk[2] +
                                  d[a][3] * Rk[3] + d[a][4] * Rk[4]);
          } else {
            for (int a = 0; a < 5; ++a) rk[a] = 0;
          }
          /* Force integrands on non-fluid cells (:2395-2398). */
          if (IF < IFLUID) {
            Residual1[5 * o + 0] = -(-(dPf[0] - dPb[0]) / dx + vF[1]) * dx * dy * dz;
            Residual1[5 * o + 1] = -(-(dPf[2] - dPb[2]) / dz + vF[3]) * dx * dy * dz;
          }
        }
  }

  /* Stage updates (:2417-2599). */
  if (RK == 1) {
    for (int c = 1; c < ncube; ++c)
      for (int i = 2; i <= nx; ++i)
        for (int j = 2; j <= nx; ++j)
          for (int k = 2; k <= nx; ++k) {
            size_t o = at(S, c, i, j, k);
            if (FWS[o] != IFLUID) continue;
            for (int v = 0; v < 5; ++v)
              U1p1[5 * o + v] = U1_[5 * o + v] = U1_[5 * o + v] + Rku1[5 * o + v];
          }
  }
  if (RK == 2) {
    for (int c = 1; c < ncube; ++c)
      for (int i = 2; i <= nx; ++i)
        for (int j = 2; j <= nx; ++j)
          for (int k = 2; k <= nx; ++k) {
            size_t o = at(S, c, i, j, k);
            if (FWS[o] != IFLUID) continue;
            for (int v = 0; v < 5; ++v)
              U1_[5 * o + v] = U1p2[5 * o + v] =
                  0.75 * U1_[5 * o + v] + 0.25 * U1p1[5 * o + v] + 0.25 * Rku1[5 * o + v];
          }
  }
  if (RK == 3) {
    double e1 = 0, e2 = 0, e3 = 0, e4 = 0, e5 = 0, e6 = 0, e7 = 0;
    for (int c = 1; c < ncube; ++c)
      for (int i = 2; i <= nx; ++i)
        for (int j = 2; j <= nx; ++j)
          for (int k = 2; k <= nx; ++k) {
            size_t o = at(S, c, i, j, k);
            double *q = U1_ + 5 * o;
            double rhoold = q[0];
            double Uold = q[1] / rhoold, Vold = q[2] / rhoold, Wold = q[3] / rhoold;
            double VVold = Uold * Uold + Vold * Vold + Wold * Wold;
            double Pold = (q[4] - 0.5 * rhoold * VVold) * (KG - 1);
            double Told = Pold / rhoold;
            if (FWS[o] == IFLUID) {
              for (int v = 0; v < 5; ++v)
                q[v] = 1.0 / 3.0 * q[v] + 2.0 / 3.0 * U1p2[5 * o + v] + 2.0 / 3.0 * Rku1[5 * o + v];
              double rho = q[0];
              double U = q[1] / rho, V = q[2] / rho, W = q[3] / rho;
              double VV = U * U + V * V + W * W;
              double P = (q[4] - 0.5 * rho * VV) * (KG - 1);
              double T = P / rho;
              e1 = e1 + (P - Pold) * (P - Pold);
              e2 = e2 + (U - Uold) * (U - Uold);
              e3 = e3 + (V - Vold) * (V - Vold);
              e4 = e4 + (W - Wold) * (W - Wold);
              e5 = e5 + (T - Told) * (T - Told);
            }
          }
    for (int c = 1; c < ncube; ++c)
      for (int i = 2; i <= nx; ++i)
        for (int j = 2; j <= nx; ++j)
          for (int k = 2; k <= nx; ++k) {
            size_t o = at(S, c, i, j, k);
            e6 = e6 + Residual1[5 * o + 0];
            e7 = e7 + Residual1[5 * o + 1];
          }
    double DN = 1. / (ph->mpi_ncube * n * n * n);
    er[1] = sqrt(e1) * DN;
    er[2] = sqrt(e2) * DN;
    er[3] = sqrt(e3) * DN;
    er[4] = sqrt(e4) * DN;
    er[5] = sqrt(e5) * DN;
    er[6] = e6 / (0.5 * ph->rho0 * ph->U0 * ph->U0 * 2.602);
    er[7] = e7 / (0.5 * ph->rho0 * ph->U0 * ph->U0 * 2.602);
  }
}

/* ------------------------------------------------------------------------ */
/* Boundary conditions, BCM_X/Y/Z_boundary_condition.cpp, in X, Y, Z order. */
/* Lists are 0-based arrays of cube numbers here.                            */
/* ------------------------------------------------------------------------ */
void bcmo_bc(const bcmo_phys *ph, int nxl, int nxu, const int *xl, const int *xu, int nyl,
             int nyu, const int *yl, const int *yu, int nzl, int nzu, const int *zl,
             const int *zu, double *U1_) {
  const int n = ph->n, S = n + 4, nx = n + 1, nxx = n + 2, nxxx = n + 3;
  /* X lower: inflow (BCM_X_boundary_condition.cpp:43-80). */
  for (int a = 0; a < nxl; ++a) {
    int c = xl[a];
    for (int j = 2; j <= nx; ++j)
      for (int k = 2; k <= nx; ++k) {
        const double *q = U1_ + 5 * at(S, c, 2, j, k);
        double rho = q[0];
        double U = q[1] / rho, V = q[2] / rho, W = q[3] / rho;
        double VV = U * U + V * V + W * W;
        double P = (q[4] - 0.5 * rho * VV) * (KG - 1);
        U = ph->Uin;
        V = 0.;
        W = 0;
        VV = U * U + V * V + W * W;
        double out[5] = {rho, rho * U, rho * V, rho * W, P / (KG - 1) + 0.5 * rho * VV};
        memcpy(U1_ + 5 * at(S, c, 1, j, k), out, sizeof out);
        memcpy(U1_ + 5 * at(S, c, 0, j, k), out, sizeof out);
      }
  }
  /* X upper: zero gradient (:85-118). */
  for (int a = 0; a < nxu; ++a) {
    int c = xu[a];
    for (int j = 2; j <= nx; ++j)
      for (int k = 2; k <= nx; ++k) {
        const double *q = U1_ + 5 * at(S, c, nx, j, k);
        memmove(U1_ + 5 * at(S, c, nxx, j, k), q, 5 * sizeof(double));
        memmove(U1_ + 5 * at(S, c, nxxx, j, k), q, 5 * sizeof(double));
      }
  }
  /* Y lower / upper: copies over all i (BCM_Y_boundary_condition.cpp:36-85). */
  for (int a = 0; a < nyl; ++a) {
    int c = yl[a];
    for (int i = 0; i <= nxxx; ++i)
      for (int k = 2; k <= nx; ++k) {
        const double *q = U1_ + 5 * at(S, c, i, 2, k);
        memmove(U1_ + 5 * at(S, c, i, 1, k), q, 5 * sizeof(double));
        memmove(U1_ + 5 * at(S, c, i, 0, k), q, 5 * sizeof(double));
      }
  }
  for (int a = 0; a < nyu; ++a) {
    int c = yu[a];
    for (int i = 0; i <= nxxx; ++i)
      for (int k = 2; k <= nx; ++k) {
        const double *q = U1_ + 5 * at(S, c, i, nx, k);
        memmove(U1_ + 5 * at(S, c, i, nxx, k), q, 5 * sizeof(double));
        memmove(U1_ + 5 * at(S, c, i, nxxx, k), q, 5 * sizeof(double));
      }
  }
  /* Z lower: slip wall, rho*w negated; Z upper: copy (BCM_Z_boundary_condition.cpp:42-92). */
  for (int a = 0; a < nzl; ++a) {
    int c = zl[a];
    for (int i = 0; i <= nxxx; ++i)
      for (int j = 0; j <= nxxx; ++j) {
        const double *q = U1_ + 5 * at(S, c, i, j, 2);
        double out[5] = {q[0], q[1], q[2], -q[3], q[4]};
        memcpy(U1_ + 5 * at(S, c, i, j, 1), out, sizeof out);
        memcpy(U1_ + 5 * at(S, c, i, j, 0), out, sizeof out);
      }
  }
  for (int a = 0; a < nzu; ++a) {
    int c = zu[a];
    for (int i = 0; i <= nxxx; ++i)
      for (int j = 0; j <= nxxx; ++j) {
        const double *q = U1_ + 5 * at(S, c, i, j, nx);
        memmove(U1_ + 5 * at(S, c, i, j, nxx), q, 5 * sizeof(double));
        memmove(U1_ + 5 * at(S, c, i, j, nxxx), q, 5 * sizeof(double));
      }
  }
}

/* ------------------------------------------------------------------------ */
/* IBM ghost cells, BCM_Ghostcell_minus.cpp:72-489 (plus is identical).      */
/* Entries are processed in list order (the reference's serial order).       */
/* GCindex/IPsur/weight are 1-based packed like BCM_Reading_IBM.cpp:53-73.    */
/* ------------------------------------------------------------------------ */
void bcmo_ghost(const bcmo_phys *ph, int nbc, const double *weight, const int *GCindex,
                const int *IPsur, double *U1_) {
  const int S = ph->n + 4;
  const double rho0 = ph->rho0, P0 = ph->P0;
  for (int e = 1; e <= nbc; ++e) {
    int b = (e - 1) * 4;
    int c = IPsur[b + 1], i = IPsur[b + 2], j = IPsur[b + 3], k = IPsur[b + 4];
    double rh[8], Uu[8], Vv[8], Ww[8], Pp[8];
    for (int m = 0; m < 8; ++m) {
      /* Order 000,100,010,001,110,101,011,111 (:81-145). */
      static const int off[8][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1},
                                    {1, 1, 0}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1}};
      const double *q = U1_ + 5 * at(S, c, i + off[m][0], j + off[m][1], k + off[m][2]);
      rh[m] = q[0];
      Uu[m] = q[1] / rh[m];
      Vv[m] = q[2] / rh[m];
      Ww[m] = q[3] / rh[m];
      double VV = Uu[m] * Uu[m] + Vv[m] * Vv[m] + Ww[m] * Ww[m];
      Pp[m] = (q[4] - 0.5 * rh[m] * VV) * (KG - 1);
    }
    const double *w = weight + (e - 1) * 8 + 1;
    int gc = GCindex[b + 1], gi = GCindex[b + 2], gj = GCindex[b + 3], gk = GCindex[b + 4];
    double rho = w[0] * (rh[0] - rho0) + w[1] * (rh[1] - rho0) + w[2] * (rh[2] - rho0) +
                 w[3] * (rh[3] - rho0) + w[4] * (rh[4] - rho0) + w[5] * (rh[5] - rho0) +
                 w[6] * (rh[6] - rho0) + w[7] * (rh[7] - rho0) + rho0;
    double P = w[0] * (Pp[0] - P0) + w[1] * (Pp[1] - P0) + w[2] * (Pp[2] - P0) +
               w[3] * (Pp[3] - P0) + w[4] * (Pp[4] - P0) + w[5] * (Pp[5] - P0) +
               w[6] * (Pp[6] - P0) + w[7] * (Pp[7] - P0) + P0;
    double U = w[0] * Uu[0] + w[1] * Uu[1] + w[2] * Uu[2] + w[3] * Uu[3] + w[4] * Uu[4] +
               w[5] * Uu[5] + w[6] * Uu[6] + w[7] * Uu[7];
    double V = w[0] * Vv[0] + w[1] * Vv[1] + w[2] * Vv[2] + w[3] * Vv[3] + w[4] * Vv[4] +
               w[5] * Vv[5] + w[6] * Vv[6] + w[7] * Vv[7];
    double W = w[0] * Ww[0] + w[1] * Ww[1] + w[2] * Ww[2] + w[3] * Ww[3] + w[4] * Ww[4] +
               w[5] * Ww[5] + w[6] * Ww[6] + w[7] * Ww[7];
    double VV = U * U + V * V + W * W;
    double *g = U1_ + 5 * at(S, gc, gi, gj, gk);
    g[0] = rho;
    g[1] = 0.5 * rho * U;
    g[2] = 0.5 * rho * V;
    g[3] = 0.5 * rho * W;
    g[4] = P / (KG - 1) + 0.5 * rho * 0.25 * VV;
    /* Ghost inside its own stencil (:192-449): the cube index is not compared. */
    static const int off[8][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1},
                                  {1, 1, 0}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1}};
    for (int s = 0; s < 8; ++s) {
      if (!((gi == i + off[s][0]) & (gj == j + off[s][1]) & (gk == k + off[s][2]))) continue;
      double r2, p2, su = 0, sv = 0, sw = 0;
      if (w[s] > 0.9999) {
        r2 = rh[s];
        p2 = Pp[s];
      } else {
        double ar = 0, ap = 0;
        int first = 1;
        for (int m = 0; m < 8; ++m) {
          if (m == s) continue;
          double tr = w[m] * (rh[m] - rho0), tp = w[m] * (Pp[m] - P0);
          if (first) { ar = tr; ap = tp; first = 0; }
          else { ar = ar + tr; ap = ap + tp; }
        }
        r2 = ar / (1 - w[s]) + rho0;
        p2 = ap / (1 - w[s]) + P0;
      }
      int first = 1;
      for (int m = 0; m < 8; ++m) {
        if (m == s) continue;
        if (first) { su = w[m] * Uu[m]; sv = w[m] * Vv[m]; sw = w[m] * Ww[m]; first = 0; }
        else { su = su + w[m] * Uu[m]; sv = sv + w[m] * Vv[m]; sw = sw + w[m] * Ww[m]; }
      }
      double U2 = su / (2 - w[s]), V2 = sv / (2 - w[s]), W2 = sw / (2 - w[s]);
      double VV2 = U2 * U2 + V2 * V2 + W2 * W2;
      g[0] = r2;
      g[1] = r2 * U2;
      g[2] = r2 * V2;
      g[3] = r2 * W2;
      g[4] = p2 / (KG - 1) + 0.5 * r2 * VV2;
    }
  }
}

/* ------------------------------------------------------------------------ */
/* Interface: same-level face copies and the ordered edge fill.              */
/* BCM_Interface.cpp:1745-1783 (X), :2608-2642 (Y), :3478-3512 (Z),          */
/* :5640-5732 (edges).  adj is [ncube][5][7] (BCM_Grid.cpp layout); the same- */
/* level lists are rebuilt here like BCM_Interface_table.cpp:96-208.         */
/* Level jumps are not restated here (see bcmo_interface_levels).            */
/* ------------------------------------------------------------------------ */
static int plus_neighbour(const int *adj, int c, int dir) {
  /* max over the four slots of adj_number[c][1..4][dir]. */
  int a = adj[(c * 5 + 1) * 7 + dir];
  for (int s = 2; s <= 4; ++s) {
    int b = adj[(c * 5 + s) * 7 + dir];
    if (b > a) a = b;
  }
  return a;
}

void bcmo_interface(const bcmo_phys *ph, int ncube, const int *adj, const int *csl,
                    double *U1_) {
  const int n = ph->n, S = n + 4, nx = n + 1, nyy = n + 2;
  /* Same-level copies for +X, +Y, +Z pairs. */
  for (int ax = 0; ax < 3; ++ax) {
    int dir = 2 + 2 * ax;
    for (int c0 = 1; c0 < ncube; ++c0) {
      int any = 0;
      for (int s = 1; s <= 4; ++s) any |= adj[(c0 * 5 + s) * 7 + dir] > 0;
      if (!any) continue;
      int a = plus_neighbour(adj, c0, dir);
      if (csl[c0] != csl[a]) continue;
      int c2 = adj[(c0 * 5 + 1) * 7 + dir];
      for (int l = 0; l < 2; ++l)
        for (int p = 2; p <= nx; ++p)
          for (int q = 2; q <= nx; ++q) {
            int src0[3], dst2[3], src2[3], dst0[3];
            /* axis coordinate, then the two transverse ones in x<y<z order. */
            int t0 = ax == 0 ? 1 : 0, t1 = ax == 2 ? 1 : 2;
            src0[ax] = n + l; dst2[ax] = l;
            src2[ax] = 2 + l; dst0[ax] = 2 + n + l;
            src0[t0] = dst2[t0] = src2[t0] = dst0[t0] = p;
            src0[t1] = dst2[t1] = src2[t1] = dst0[t1] = q;
            memmove(U1_ + 5 * at(S, c2, dst2[0], dst2[1], dst2[2]),
                    U1_ + 5 * at(S, c0, src0[0], src0[1], src0[2]), 5 * sizeof(double));
            memmove(U1_ + 5 * at(S, c0, dst0[0], dst0[1], dst0[2]),
                    U1_ + 5 * at(S, c2, src2[0], src2[1], src2[2]), 5 * sizeof(double));
          }
    }
  }
  bcmo_interface_levels(ph, ncube, adj, csl, U1_);
  /* Edge fill, three ordered phases per cube (:5640-5732). */
  for (int c = 1; c < ncube; ++c) {
#define Q(i, j, k) (U1_ + 5 * at(S, c, (i), (j), (k)))
#define AVG(d, a, b) { double *dd = d; const double *aa = a, *bb = b; \
    for (int v = 0; v < 5; ++v) dd[v] = 0.5 * (aa[v] + bb[v]); }
    for (int i = 2; i <= nx; ++i) {
      AVG(Q(i, 1, 1), Q(i, 1, 2), Q(i, 2, 1));
      AVG(Q(i, nyy, 1), Q(i, nyy, 2), Q(i, nx, 1));
      AVG(Q(i, 1, nyy), Q(i, 1, nx), Q(i, 2, nyy));
      AVG(Q(i, nyy, nyy), Q(i, nyy, nx), Q(i, nx, nyy));
    }
    for (int j = 1; j <= nyy; ++j) {
      AVG(Q(1, j, 1), Q(1, j, 2), Q(2, j, 1));
      AVG(Q(1, j, nyy), Q(2, j, nyy), Q(1, j, nx));
      AVG(Q(nyy, j, 1), Q(nx, j, 1), Q(nyy, j, 2));
      AVG(Q(nyy, j, nyy), Q(nx, j, nyy), Q(nyy, j, nx));
    }
    for (int k = 1; k <= nyy; ++k) {
      AVG(Q(1, 1, k), Q(1, 2, k), Q(2, 1, k));
      AVG(Q(1, nyy, k), Q(2, nyy, k), Q(1, nx, k));
      AVG(Q(nyy, 1, k), Q(nx, 1, k), Q(nyy, 2, k));
      AVG(Q(nyy, nyy, k), Q(nx, nyy, k), Q(nyy, nx, k));
    }
#undef AVG
#undef Q
  }
}

/* Level jumps between a cube B and its four half-size neighbours across one
 * face (BCM_Interface.cpp:1790-2599 x, :2651-3470 y, :3518-4358 z; lists as
 * BCM_Interface_table.cpp:96-308 builds them).  For axis a with tangential
 * axes t0 < t1, sub-face slot s (1..4) offsets (t0, t1) by
 * ((s==2||s==4)*n/2, (s==3||s==4)*n/2).  Four blocks per axis:
 *  (a) B bigger than its +a neighbours: each small cube's low ghost layers
 *      l=0,1 <- B's cell (n+1, p/2+1+o0, q/2+1+o1) (injection, :1790-1899);
 *  (b) B bigger than its -a neighbours: each small cube's high ghost layers
 *      n+2+l <- B's cell (2, p/2+1+o0, q/2+1+o1) (:1903-2022);
 *  (c) B's high ghost layers n+2+l over the slot's quadrant <- 0.125 * the sum
 *      of the small cube's 2x2x2 cells at along-axis 2l+2 (:2026-2314);
 *  (d) B's low ghost layers l <- 0.125 * sum at along-axis n-2+2l (:2318-2599).
 * Every read is an interior cell, every write a ghost cell, so the blocks
 * commute with each other and with the same-level copies. */
static void lvl_index(int ax, int g, int p, int q, int *ijk) {
  int t0 = ax == 0 ? 1 : 0, t1 = ax == 2 ? 1 : 2;
  ijk[ax] = g;
  ijk[t0] = p;
  ijk[t1] = q;
}

void bcmo_interface_levels(const bcmo_phys *ph, int ncube, const int *adj, const int *csl,
                           double *U1_) {
  const int n = ph->n, S = n + 4, h = n / 2;
  static const int off8[8][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1},
                                 {1, 1, 0}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1}};
  for (int ax = 0; ax < 3; ++ax) {
    for (int pm = 0; pm < 2; ++pm) { /* pm 0: +a neighbours (bs_plus), 1: -a (bs_minus) */
      const int dir = pm == 0 ? 2 + 2 * ax : 1 + 2 * ax;
      for (int B = 1; B < ncube; ++B) {
        int any = 0, acube = 0;
        for (int sl = 1; sl <= 4; ++sl) {
          int v = adj[(B * 5 + sl) * 7 + dir];
          any |= v > 0;
          if (v > acube) acube = v;
        }
        if (!any || !(csl[B] > csl[acube])) continue;
        for (int sl = 1; sl <= 4; ++sl) {
          const int sc = adj[(B * 5 + sl) * 7 + dir];
          if (sc <= 0) continue;
          const int o0 = (sl == 2 || sl == 4) ? h : 0, o1 = (sl == 3 || sl == 4) ? h : 0;
          /* (a) / (b): coarse -> fine injection into the small cube */
          for (int l = 0; l < 2; ++l)
            for (int p = 2; p <= n + 1; ++p)
              for (int q = 2; q <= n + 1; ++q) {
                int d[3], sidx[3];
                lvl_index(ax, pm == 0 ? l : n + 2 + l, p, q, d);
                lvl_index(ax, pm == 0 ? n + 1 : 2, p / 2 + 1 + o0, q / 2 + 1 + o1, sidx);
                memmove(U1_ + 5 * at(S, sc, d[0], d[1], d[2]),
                        U1_ + 5 * at(S, B, sidx[0], sidx[1], sidx[2]), 5 * sizeof(double));
              }
          /* (c) / (d): fine -> coarse 8-cell average into B */
          for (int l = 0; l < 2; ++l)
            for (int p = 2; p <= h + 1; ++p)
              for (int q = 2; q <= h + 1; ++q) {
                int d[3], b[3];
                lvl_index(ax, pm == 0 ? n + 2 + l : l, p + o0, q + o1, d);
                lvl_index(ax, pm == 0 ? 2 * (l + 1) : n - 2 + 2 * l, (p - 1) * 2, (q - 1) * 2, b);
                double *dst = U1_ + 5 * at(S, B, d[0], d[1], d[2]);
                for (int v = 0; v < 5; ++v) {
                  double sum = 0;
                  for (int m = 0; m < 8; ++m) {
                    double x = U1_[5 * at(S, sc, b[0] + off8[m][0], b[1] + off8[m][1],
                                          b[2] + off8[m][2]) + v];
                    sum = m == 0 ? x : sum + x;
                  }
                  dst[v] = 0.125 * sum;
                }
              }
        }
      }
    }
  }
}

/* Time-level shift on interior cells (main.cpp:1292-1315). */
void bcmo_time_shift(const bcmo_phys *ph, int ncube, const double *U1_, double *U1,
                     double *U1q) {
  const int n = ph->n, S = n + 4, nx = n + 1;
  for (int c = 1; c < ncube; ++c)
    for (int i = 2; i <= nx; ++i)
      for (int j = 2; j <= nx; ++j)
        for (int k = 2; k <= nx; ++k) {
          size_t o = 5 * at(S, c, i, j, k);
          for (int v = 0; v < 5; ++v) {
            U1q[o + v] = U1[o + v];
            U1[o + v] = U1_[o + v];
          }
        }
}

/* ------------------------------------------------------------------------ */
/* The reference time loop (main.cpp:1146-1357) with a fixed sub-iteration   */
/* count per physical step; same per-stage order as the reference:           */
/* BCs -> IBM minus -> IBM plus -> interface -> flux/RK -> interface.        */
/* ------------------------------------------------------------------------ */
void bcmo_run(const bcmo_phys *ph, int ncube, int steps, int subiters, double deltaT,
              double deltaTau, double e, const int *FWS, const int *adj, const int *csl,
              const double *cube_size, double *U1_, double *U1, double *U1q, double *U1p1,
              double *U1p2, double *Rku1, double *Residual1, int nxl, int nxu, const int *xl,
              const int *xu, int nyl, int nyu, const int *yl, const int *yu, int nzl, int nzu,
              const int *zl, const int *zu, int nminus, const double *wm, const int *gm,
              const int *im, int nplus, const double *wp, const int *gp, const int *ip,
              double *er, double *Emax) {
  for (int step = 1; step <= steps; ++step) {
    for (int it = 1; it <= subiters; ++it) {
      for (int RK = 1; RK < 4; ++RK) {
        bcmo_bc(ph, nxl, nxu, xl, xu, nyl, nyu, yl, yu, nzl, nzu, zl, zu, U1_);
        if (nminus > 0) bcmo_ghost(ph, nminus, wm, gm, im, U1_);
        if (nplus > 0) bcmo_ghost(ph, nplus, wp, gp, ip, U1_);
        bcmo_interface(ph, ncube, adj, csl, U1_);
        bcmo_flux_stage(ph, ncube, RK, deltaT, deltaTau, e, FWS, cube_size, U1_, U1, U1q, U1p1,
                        U1p2, Rku1, Residual1, er);
        bcmo_interface(ph, ncube, adj, csl, U1_);
      }
      /* main.cpp:1249-1259 */
      for (int v = 1; v <= 5; ++v) {
        Emax[v] = er[v] > Emax[v] ? er[v] : Emax[v];
        er[v] = er[v] / Emax[v];
      }
    }
    bcmo_time_shift(ph, ncube, U1_, U1, U1q);
  }
}
