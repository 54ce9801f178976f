/*
 * ORACLE (test infrastructure).  C restatement of BCM_CGLI's per-stage hot
 * path; see bcm_oracle.c.  Arrays use the reference layout
 * U[c][i][j][k][5] with S = n+4 cells per edge, cube 0 unused.
 */
#ifndef BCM_ORACLE_H
#define BCM_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct bcmo_phys {
  int n;          /* interior cells per cube edge (NcubeX, Resolution.h:9) */
  int mpi_ncube;  /* norm normaliser MPI_Ncube (Resolution.h:3) */
  double mu_L;    /* prm.h:5 */
  double rho0;    /* prm.h:27 */
  double U0;      /* prm.h:29 */
  double Uin;     /* prm.h:31 */
  double P0;      /* prm.h:37 */
} bcmo_phys;

/* RK 1..3: one stage; RK 0: the raw residual R into Rku1 (fluid cells) and
 * the force integrands, no update. */
void bcmo_flux_stage(const bcmo_phys *ph, int ncube, int RK, double deltaT, double deltaTau,
                     double e, const int *FWS, const double *cube_size, double *U1_,
                     const double *U1, const double *U1q, double *U1p1, double *U1p2,
                     double *Rku1, double *Residual1, double *er);
void bcmo_bc(const bcmo_phys *ph, int nxl, int nxu, const int *xl, const int *xu, int nyl,
             int nyu, const int *yl, const int *yu, int nzl, int nzu, const int *zl,
             const int *zu, double *U1_);
void bcmo_ghost(const bcmo_phys *ph, int nbc, const double *weight, const int *GCindex,
                const int *IPsur, double *U1_);
void bcmo_interface(const bcmo_phys *ph, int ncube, const int *adj, const int *csl,
                    double *U1_);
void bcmo_interface_levels(const bcmo_phys *ph, int ncube, const int *adj, const int *csl,
                           double *U1_);
void bcmo_time_shift(const bcmo_phys *ph, int ncube, const double *U1_, double *U1,
                     double *U1q);
void bcmo_run(const bcmo_phys *ph, int ncube, int steps, int subiters, double deltaT,
              double deltaTau, double e, const int *FWS, const int *adj, const int *csl,
              const double *cube_size, double *U1_, double *U1, double *U1q, double *U1p1,
              double *U1p2, double *Rku1, double *Residual1, int nxl, int nxu, const int *xl,
              const int *xu, int nyl, int nyu, const int *yl, const int *yu, int nzl, int nzu,
              const int *zl, const int *zu, int nminus, const double *wm, const int *gm,
              const int *im, int nplus, const double *wp, const int *gp, const int *ip,
              double *er, double *Emax);
/* LU-SGS sub-iteration (bcm_oracle_lusgs.c; no reference counterpart).
 * Rku1 holds the residual (bcmo_flux_stage with RK = 0) on entry and the
 * increment on return; U1_ is updated on fluid cells and er[1..7] set. */
void bcmo_lusgs(const bcmo_phys *ph, int ncube, double deltaT, double cfl, double omega,
                const int *FWS, const double *cube_size, double *U1_, double *Rku1,
                const double *Residual1, double *er);
void bcmo_run_lusgs(const bcmo_phys *ph, int ncube, int steps, int subiters, double deltaT,
                    double cfl, double omega, double e, const int *FWS, const int *adj,
                    const int *csl, const double *cube_size, double *U1_, double *U1,
                    double *U1q, double *Rku1, double *Residual1, int nxl, int nxu,
                    const int *xl, const int *xu, int nyl, int nyu, const int *yl,
                    const int *yu, int nzl, int nzu, const int *zl, const int *zu, int nminus,
                    const double *wm, const int *gm, const int *im, int nplus,
                    const double *wp, const int *gp, const int *ip, double *er, double *Emax);
void bcmo_run_converged(const bcmo_phys *ph, int ncube, int steps, int max_subiters, double tol,
                        int method, double deltaT, double deltaTau, double cfl, double omega,
                        double e, const int *FWS, const int *adj, const int *csl,
                        const double *cube_size, double *U1_, double *U1, double *U1q,
                        double *U1p1, double *U1p2, double *Rku1, double *Residual1, int nxl,
                        int nxu, const int *xl, const int *xu, int nyl, int nyu, const int *yl,
                        const int *yu, int nzl, int nzu, const int *zl, const int *zu,
                        int nminus, const double *wm, const int *gm, const int *im, int nplus,
                        const double *wp, const int *gp, const int *ip, double *er, double *Emax,
                        int *iters_out);
/* IBM preprocessing (bcm_oracle_ibm.c): triangles tri_in[ntri][9], FWS
 * updated in place, entries 0-based packed (GCindex / IPsur 4 ints, weight 8
 * doubles per entry), tri_scratch holds ntri*9 doubles.  Returns 0, or -1
 * when an output table would exceed cap entries. */
int bcmo_ibm(int n, int ncube, const double *cube_size, const int *csl, const double *Xcube,
             const double *Ycube, const double *Zcube, int *FWS, int ntri_in, const double *tri_in,
             int cap, int *nminus, int *gc_m, int *ip_m, double *w_m, int *nplus, int *gc_p,
             int *ip_p, double *w_p, double *tri_scratch);
void bcmo_set_threads(int n);

#ifdef __cplusplus
}
#endif
#endif
