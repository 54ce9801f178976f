/*
 * ORACLE (test infrastructure; never part of the product path).
 *
 * LU-SGS dual-time sub-iteration.  The reference has no implementation
 * (BCM_LUSGS.h only re-declares an older BCM_Interface), so this file is the
 * CPU definition of the scheme the GPU kernel must reproduce: a matrix-free
 * LU-SGS (Yoon & Jameson's lower-upper symmetric Gauss-Seidel, in the
 * Jameson-Turkel split-Jacobian form A+- = (A +- omega*r I)/2 with a scalar
 * viscous term) for the same discrete residual as the RK path,
 *
 *   R(Q) = -(3Q - 4Q^n + Q^(n-1))/(2 dT) - div F_inviscid + div F_viscous,
 *
 * one pseudo-time step per sub-iteration, per cube (cube faces and non-fluid
 * cells carry no increment).  Per interior fluid cell with state q:
 *   u, v, w, p, c = sqrt(K p / rho), H = (E + p)/rho, r_d = |u_d| + c,
 *   nu = mu(T) K / (Pr rho) (Sutherland mu as in the viscous flux),
 *   dg = 3/(2 dT) + omega * sum_d r_d / dx + 6 nu / dx^2 [+ sum_d r_d/(cfl dx)]
 * Forward sweep, cells in lexicographic (i, j, k) order:
 *   dq*_i = (R_i + sum_{d=x,y,z} L_d(i - e_d)) / dg_i,
 *   L_d(m) = (A_d(q_m) dq*_m + omega r_d,m dq*_m) / (2 dx) + nu_m/dx^2 dq*_m
 * Backward sweep, reverse order:
 *   dq_i = dq*_i - (sum_{d=x,y,z} U_d(i + e_d)) / dg_i,
 *   U_d(m) = (A_d(q_m) dq_m - omega r_d,m dq_m) / (2 dx) - nu_m/dx^2 dq_m
 * where A_d(q) dq is the exact linearisation of the Euler flux in direction d
 * and neighbours outside the cube's interior or not fluid contribute nothing.
 * Then Q += dq on fluid cells with the change / force norms of the RK path's
 * third stage (BCM_Flux_XYZ_Viscous_Runge_kutta.cpp:2530-2650).
 *
 * A cell's forward value depends only on its three lower neighbours and its
 * backward value only on its three upper neighbours, so the planes
 * i + j + k = const can be swept in parallel (the GPU kernel does) with
 * results identical to this serial order.  The converged state (R = 0) is
 * the RK path's converged state; tests check both facts.
 */
#include <math.h>
#include <stddef.h>

#include "bcm_oracle.h"

#define IFLUID 1
#define KG 1.4
#define RGAS 287
#define PR_L 0.72

static inline size_t at(int S, int c, int i, int j, int k) {
  return ((((size_t)c * S + i) * S + j) * S + k);
}

typedef struct {
  double U, V, W, VV, H, r[3], nu, dg;
} lu_coef;

static lu_coef lu_coef_of(const double *q, double dx, double mu_L, double T0, double deltaT,
                          double cfl, double omega) {
  lu_coef k;
  double rho = q[0];
  k.U = q[1] / rho;
  k.V = q[2] / rho;
  k.W = q[3] / rho;
  k.VV = k.U * k.U + k.V * k.V + k.W * k.W;
  double P = (q[4] - 0.5 * rho * k.VV) * (KG - 1);
  double c = sqrt(KG * P / rho);
  k.H = (q[4] + P) / rho;
  k.r[0] = fabs(k.U) + c;
  k.r[1] = fabs(k.V) + c;
  k.r[2] = fabs(k.W) + c;
  double T = P / rho / RGAS;
  double temp = T / T0;
  double mu = mu_L * temp * sqrt(temp) * (T0 + 110.) / (T + 110.);
  k.nu = mu * (KG / PR_L) / rho;
  double rs = k.r[0] + k.r[1] + k.r[2];
  double dg = 1.5 / deltaT + omega * rs / dx + 6.0 * k.nu / (dx * dx);
  if (cfl > 0) dg = dg + rs / (cfl * dx);
  k.dg = dg;
  return k;
}

/* out = sgn-split off-diagonal term of cell m (coefficients k, increment dq)
 * across a face of direction d: sgn > 0 lower neighbour, sgn < 0 upper. */
static void lu_off(const lu_coef *k, int d, int sgn, double dx, double omega,
                   const double *dq, double *out) {
  double un = d == 0 ? k->U : (d == 1 ? k->V : k->W);
  double dp = (KG - 1) * (dq[4] - (k->U * dq[1] + k->V * dq[2] + k->W * dq[3]) +
                          0.5 * k->VV * dq[0]);
  double t = dq[1 + d] - un * dq[0];
  double a[5];
  a[0] = dq[1 + d];
  a[1] = un * dq[1] + k->U * t;
  a[2] = un * dq[2] + k->V * t;
  a[3] = un * dq[3] + k->W * t;
  a[1 + d] = a[1 + d] + dp;
  a[4] = un * (dq[4] + dp) + k->H * t;
  double h = 0.5 / dx, w = omega * k->r[d], v = k->nu / (dx * dx);
  for (int m = 0; m < 5; ++m)
    out[m] = sgn > 0 ? h * (a[m] + w * dq[m]) + v * dq[m] : h * (a[m] - w * dq[m]) - v * dq[m];
}

void bcmo_lusgs(const bcmo_phys *ph, int ncube, double deltaT, double cfl, double omega,
                const int *FWS, const double *cube_size, double *U1_, double *Rku1,
                const double *Residual1, double *er) {
  const int n = ph->n, S = n + 4, nx = n + 1;
  const double T0 = ph->P0 / ph->rho0 / RGAS;
#pragma omp parallel for schedule(dynamic, 1)
  for (int c = 1; c < ncube; ++c) {
    const double dx = cube_size[c] / n;
    /* forward sweep */
    for (int i = 2; i <= nx; ++i)
      for (int j = 2; j <= nx; ++j)
        for (int k = 2; k <= nx; ++k) {
          size_t o = at(S, c, i, j, k);
          if (FWS[o] != IFLUID) continue;
          lu_coef kc = lu_coef_of(U1_ + 5 * o, dx, ph->mu_L, T0, deltaT, cfl, omega);
          double s[5];
          for (int m = 0; m < 5; ++m) s[m] = Rku1[5 * o + m];
          for (int d = 0; d < 3; ++d) {
            int ii = i - (d == 0), jj = j - (d == 1), kk = k - (d == 2);
            if (ii < 2 || jj < 2 || kk < 2) continue;
            size_t on = at(S, c, ii, jj, kk);
            if (FWS[on] != IFLUID) continue;
            lu_coef kn = lu_coef_of(U1_ + 5 * on, dx, ph->mu_L, T0, deltaT, cfl, omega);
            double t[5];
            lu_off(&kn, d, +1, dx, omega, Rku1 + 5 * on, t);
            for (int m = 0; m < 5; ++m) s[m] = s[m] + t[m];
          }
          for (int m = 0; m < 5; ++m) Rku1[5 * o + m] = s[m] / kc.dg;
        }
    /* backward sweep */
    for (int i = nx; i >= 2; --i)
      for (int j = nx; j >= 2; --j)
        for (int k = nx; k >= 2; --k) {
          size_t o = at(S, c, i, j, k);
          if (FWS[o] != IFLUID) continue;
          lu_coef kc = lu_coef_of(U1_ + 5 * o, dx, ph->mu_L, T0, deltaT, cfl, omega);
          double s[5] = {0, 0, 0, 0, 0};
          for (int d = 0; d < 3; ++d) {
            int ii = i + (d == 0), jj = j + (d == 1), kk = k + (d == 2);
            if (ii > nx || jj > nx || kk > nx) continue;
            size_t on = at(S, c, ii, jj, kk);
            if (FWS[on] != IFLUID) continue;
            lu_coef kn = lu_coef_of(U1_ + 5 * on, dx, ph->mu_L, T0, deltaT, cfl, omega);
            double t[5];
            lu_off(&kn, d, -1, dx, omega, Rku1 + 5 * on, t);
            for (int m = 0; m < 5; ++m) s[m] = s[m] + t[m];
          }
          for (int m = 0; m < 5; ++m) Rku1[5 * o + m] = Rku1[5 * o + m] - s[m] / kc.dg;
        }
  }
  /* update and norms (serial order) */
  double e1 = 0, e2 = 0, e3 = 0, e4 = 0, e5 = 0, e6 = 0, e7 = 0;
  for (int c = 1; c < ncube; ++c)
    for (int i = 2; i <= nx; ++i)
      for (int j = 2; j <= nx; ++j)
        for (int k = 2; k <= nx; ++k) {
          size_t o = at(S, c, i, j, k);
          if (FWS[o] == IFLUID) {
            double *q = U1_ + 5 * o;
            double rhoold = q[0];
            double Uold = q[1] / rhoold, Vold = q[2] / rhoold, Wold = q[3] / rhoold;
            double VVold = Uold * Uold + Vold * Vold + Wold * Wold;
            double Pold = (q[4] - 0.5 * rhoold * VVold) * (KG - 1);
            double Told = Pold / rhoold;
            for (int v = 0; v < 5; ++v) q[v] = q[v] + Rku1[5 * o + v];
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

/* The time loop of bcmo_run with one LU-SGS update per sub-iteration:
 * BCs -> IBM minus -> IBM plus -> interface -> residual -> LU-SGS update ->
 * interface; the same convergence normalisation and time shift. */
void bcmo_run_lusgs(const bcmo_phys *ph, int ncube, int steps, int subiters, double deltaT,
                    double cfl, double omega, double e, const int *FWS, const int *adj,
                    const int *csl, const double *cube_size, double *U1_, double *U1,
                    double *U1q, double *Rku1, double *Residual1, int nxl, int nxu,
                    const int *xl, const int *xu, int nyl, int nyu, const int *yl,
                    const int *yu, int nzl, int nzu, const int *zl, const int *zu, int nminus,
                    const double *wm, const int *gm, const int *im, int nplus,
                    const double *wp, const int *gp, const int *ip, double *er, double *Emax) {
  for (int step = 1; step <= steps; ++step) {
    for (int it = 1; it <= subiters; ++it) {
      bcmo_bc(ph, nxl, nxu, xl, xu, nyl, nyu, yl, yu, nzl, nzu, zl, zu, U1_);
      if (nminus > 0) bcmo_ghost(ph, nminus, wm, gm, im, U1_);
      if (nplus > 0) bcmo_ghost(ph, nplus, wp, gp, ip, U1_);
      bcmo_interface(ph, ncube, adj, csl, U1_);
      bcmo_flux_stage(ph, ncube, 0, deltaT, deltaT, e, FWS, cube_size, U1_, U1, U1q, NULL, NULL,
                      Rku1, Residual1, er);
      bcmo_lusgs(ph, ncube, deltaT, cfl, omega, FWS, cube_size, U1_, Rku1, Residual1, er);
      bcmo_interface(ph, ncube, adj, csl, U1_);
      for (int v = 1; v <= 5; ++v) {
        Emax[v] = er[v] > Emax[v] ? er[v] : Emax[v];
        er[v] = er[v] / Emax[v];
      }
    }
    bcmo_time_shift(ph, ncube, U1_, U1, U1q);
  }
}

/* The reference time loop with its convergence test (main.cpp:1146-1357):
 * per step, sub-iterations (method 0: three RK stages as in bcmo_run;
 * method 1: one LU-SGS update) until every normalised change norm er[1..5]
 * is below tol or max_subiters ran (the reference's iteration_end_step),
 * then the time shift.  iters_out[step] receives the sub-iteration counts. */
void bcmo_run_converged(const bcmo_phys *ph, int ncube, int steps, int max_subiters, double tol,
                        int method, double deltaT, double deltaTau, double cfl, double omega,
                        double e, const int *FWS, const int *adj, const int *csl,
                        const double *cube_size, double *U1_, double *U1, double *U1q,
                        double *U1p1, double *U1p2, double *Rku1, double *Residual1, int nxl,
                        int nxu, const int *xl, const int *xu, int nyl, int nyu, const int *yl,
                        const int *yu, int nzl, int nzu, const int *zl, const int *zu,
                        int nminus, const double *wm, const int *gm, const int *im, int nplus,
                        const double *wp, const int *gp, const int *ip, double *er, double *Emax,
                        int *iters_out) {
  for (int step = 1; step <= steps; ++step) {
    int it;
    for (it = 1; it <= max_subiters; ++it) {
      for (int RK = 1; RK <= (method == 1 ? 1 : 3); ++RK) {
        bcmo_bc(ph, nxl, nxu, xl, xu, nyl, nyu, yl, yu, nzl, nzu, zl, zu, U1_);
        if (nminus > 0) bcmo_ghost(ph, nminus, wm, gm, im, U1_);
        if (nplus > 0) bcmo_ghost(ph, nplus, wp, gp, ip, U1_);
        bcmo_interface(ph, ncube, adj, csl, U1_);
        if (method == 1) {
          bcmo_flux_stage(ph, ncube, 0, deltaT, deltaT, e, FWS, cube_size, U1_, U1, U1q, U1p1,
                          U1p2, Rku1, Residual1, er);
          bcmo_lusgs(ph, ncube, deltaT, cfl, omega, FWS, cube_size, U1_, Rku1, Residual1, er);
        } else {
          bcmo_flux_stage(ph, ncube, RK, deltaT, deltaTau, e, FWS, cube_size, U1_, U1, U1q, U1p1,
                          U1p2, Rku1, Residual1, er);
        }
        bcmo_interface(ph, ncube, adj, csl, U1_);
      }
      for (int v = 1; v <= 5; ++v) {
        Emax[v] = er[v] > Emax[v] ? er[v] : Emax[v];
        er[v] = er[v] / Emax[v];
      }
      if (er[1] < tol && er[2] < tol && er[3] < tol && er[4] < tol && er[5] < tol) break;
    }
    iters_out[step - 1] = it > max_subiters ? max_subiters : it;
    bcmo_time_shift(ph, ncube, U1_, U1, U1q);
  }
}
