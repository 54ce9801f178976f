// C++ link shim for the reference's own driver (main.cpp).
//
// The reference declares its hot-path routines in main.h with C++ linkage
// and fixed-size array parameters, e.g. `double (*U1_)[X_size][Y_size]
// [Z_size][Ndim]`.  Including this header in exactly ONE translation unit of
// the host program (after Resolution.h, so X_size/Ndim are defined), and
// dropping the reference's BCM_Flux_XYZ_Viscous_Runge_kutta.cpp,
// BCM_Interface.cpp, BCM_Ghostcell_minus.cpp, BCM_Ghostcell_plus.cpp,
// BCM_X/Y/Z_boundary_condition.cpp, BCM_Immersed_boundary.cpp and
// BCM_FWS_Interface.cpp from the link, gives main.cpp the same
// C++ symbols, now running through the C ABI of bcm_gb300.h (the per-stage
// routines and the IBM preprocessing on the GPU, the flag setup on the
// host).
// Call bcmg_set_reference_config() once at start-up with the values of
// Resolution.h / prm.h (NcubeX, MPI_Ncube, mu_L, rho0, U0, Uin, P0).
#pragma once

#include "bcm_gb300.h"

#ifndef X_size
#error "include Resolution.h before bcm_gb300_reference_shim.hpp"
#endif

typedef double bcmg_shim_cell_t[X_size][Y_size][Z_size][Ndim];
typedef int bcmg_shim_flag_t[X_size][Y_size][Z_size];

// main.h:473-513
void BCM_Flux_XYZ_Viscous_Runge_kutta(int myid, int ncube, int RK, double deltaT,
                                      double deltaTau, double e, bcmg_shim_flag_t *FWS, int *csl,
                                      double *cube_size, bcmg_shim_cell_t *U1_,
                                      bcmg_shim_cell_t *U1, bcmg_shim_cell_t *U1q,
                                      bcmg_shim_cell_t *U1p1, bcmg_shim_cell_t *U1p2,
                                      bcmg_shim_cell_t *Rku1, bcmg_shim_cell_t *Residual1,
                                      double *er) {
  ::BCM_Flux_XYZ_Viscous_Runge_kutta(myid, ncube, RK, deltaT, deltaTau, e, (int *)FWS, csl,
                                     cube_size, (double *)U1_, (double *)U1, (double *)U1q,
                                     (double *)U1p1, (double *)U1p2, (double *)Rku1,
                                     (double *)Residual1, er);
}

// main.h:418-470
void BCM_X_boundary_condition(int myid, int nXbc_l, int nXbc_u, int *Xbc_l, int *Xbc_u,
                              bcmg_shim_cell_t *U1_) {
  ::BCM_X_boundary_condition(myid, nXbc_l, nXbc_u, Xbc_l, Xbc_u, (double *)U1_);
}
void BCM_Y_boundary_condition(int nYbc_l, int nYbc_u, int *Ybc_l, int *Ybc_u,
                              bcmg_shim_cell_t *U1_) {
  ::BCM_Y_boundary_condition(nYbc_l, nYbc_u, Ybc_l, Ybc_u, (double *)U1_);
}
void BCM_Z_boundary_condition(int nZbc_l, int nZbc_u, int *Zbc_l, int *Zbc_u,
                              bcmg_shim_cell_t *U1_) {
  ::BCM_Z_boundary_condition(nZbc_l, nZbc_u, Zbc_l, Zbc_u, (double *)U1_);
}

// main.h:378-413
void BCM_Ghostcell_minus(int myid, int *NNBC, double *weight, int *GCindex, int *IPsur,
                         bcmg_shim_flag_t *FWS, bcmg_shim_cell_t *U1_) {
  ::BCM_Ghostcell_minus(myid, NNBC, weight, GCindex, IPsur, (int *)FWS, (double *)U1_);
}
void BCM_Ghostcell_plus(int myid, int *NNBC, double *weight, int *GCindex, int *IPsur,
                        bcmg_shim_flag_t *FWS, bcmg_shim_cell_t *U1_) {
  ::BCM_Ghostcell_plus(myid, NNBC, weight, GCindex, IPsur, (int *)FWS, (double *)U1_);
}

// main.h:224-354
void BCM_Interface(int myid, int ncube, int mPI_Nadj, int ncpu_bs, int ncpu_eq, int ncpu_sb,
                   int max_nei_bs, int max_nei_eq, int max_nei_sb, int nadjX_eq, int nadjY_eq,
                   int nadjZ_eq, int nadjX_bs_plus, int nadjX_sb_plus, int nadjX_bs_minus,
                   int nadjX_sb_minus, int nadjY_bs_plus, int nadjY_sb_plus,
                   int nadjY_bs_minus, int nadjY_sb_minus, int nadjZ_bs_plus,
                   int nadjZ_sb_plus, int nadjZ_bs_minus, int nadjZ_sb_minus,
                   int (*rank_map)[MPI_Ncube], int *MPI_cpu, int *MPI_cube, int *MPI_cpu_adj,
                   int *MPI_cube_adj, int *MPI_direction, int *MPI_interface,
                   int *neighbor_cpu_eq, int *Ncube_Ncpu_eq, int *neighbor_cpu_sb,
                   int *Ncube_Ncpu_sb, int *neighbor_cpu_bs, int *Ncube_Ncpu_bs,
                   int *Scube_Ncpu_eq, int *Rcube_Ncpu_eq, double *send_data_curr_eq,
                   double *recv_data_curr_eq, double *send_data_neig_eq,
                   double *recv_data_neig_eq, int *Sdir_eq, int *Rdir_eq, int *Scube_Ncpu_sb,
                   int *Rcube_Ncpu_sb, double *send_data_curr_sb, double *recv_data_curr_sb,
                   double *send_data_neig_sb, double *recv_data_neig_sb, int *Sdir_sb,
                   int *Rdir_sb, int *Scube_Ncpu_bs, int *Rcube_Ncpu_bs,
                   double *send_data_curr_bs, double *recv_data_curr_bs,
                   double *send_data_neig_bs, double *recv_data_neig_bs, int *Sdir_bs,
                   int *Rdir_bs, int *ist_eq, int *ist_sb, int *ist_bs, int *adjN_sb,
                   int *RadjN_bs, int *SadjN_bs, int *csl, int (*adj_number)[5][7],
                   int *adjX_eq, int *adjY_eq, int *adjZ_eq, int *adjX_bs_plus,
                   int *adjX_sb_plus, int *adjX_bs_minus, int *adjX_sb_minus,
                   int *adjY_bs_plus, int *adjY_sb_plus, int *adjY_bs_minus,
                   int *adjY_sb_minus, int *adjZ_bs_plus, int *adjZ_sb_plus,
                   int *adjZ_bs_minus, int *adjZ_sb_minus, bcmg_shim_cell_t *U1_) {
  ::BCM_Interface(myid, ncube, mPI_Nadj, ncpu_bs, ncpu_eq, ncpu_sb, max_nei_bs, max_nei_eq,
                  max_nei_sb, nadjX_eq, nadjY_eq, nadjZ_eq, nadjX_bs_plus, nadjX_sb_plus,
                  nadjX_bs_minus, nadjX_sb_minus, nadjY_bs_plus, nadjY_sb_plus, nadjY_bs_minus,
                  nadjY_sb_minus, nadjZ_bs_plus, nadjZ_sb_plus, nadjZ_bs_minus, nadjZ_sb_minus,
                  (int *)rank_map, MPI_cpu, MPI_cube, MPI_cpu_adj, MPI_cube_adj, MPI_direction,
                  MPI_interface, neighbor_cpu_eq, Ncube_Ncpu_eq, neighbor_cpu_sb, Ncube_Ncpu_sb,
                  neighbor_cpu_bs, Ncube_Ncpu_bs, Scube_Ncpu_eq, Rcube_Ncpu_eq,
                  send_data_curr_eq, recv_data_curr_eq, send_data_neig_eq, recv_data_neig_eq,
                  Sdir_eq, Rdir_eq, Scube_Ncpu_sb, Rcube_Ncpu_sb, send_data_curr_sb,
                  recv_data_curr_sb, send_data_neig_sb, recv_data_neig_sb, Sdir_sb, Rdir_sb,
                  Scube_Ncpu_bs, Rcube_Ncpu_bs, send_data_curr_bs, recv_data_curr_bs,
                  send_data_neig_bs, recv_data_neig_bs, Sdir_bs, Rdir_bs, ist_eq, ist_sb,
                  ist_bs, adjN_sb, RadjN_bs, SadjN_bs, csl, (int *)adj_number, adjX_eq,
                  adjY_eq, adjZ_eq, adjX_bs_plus, adjX_sb_plus, adjX_bs_minus, adjX_sb_minus,
                  adjY_bs_plus, adjY_sb_plus, adjY_bs_minus, adjY_sb_minus, adjZ_bs_plus,
                  adjZ_sb_plus, adjZ_bs_minus, adjZ_sb_minus, (double *)U1_);
}

// main.h:113-144 (setup, called once at main.cpp:811)
void BCM_Immersed_boundary(int myid, int ncube, int n_wallcube, int *NBC, double Xmin,
                           double Xmax, double Ymin, double Ymax, double Zmin, double Zmax,
                           double *cube_size, int *csl, double *Xcube, double *Ycube,
                           double *Zcube, double (*Xcnt)[X_size], double (*Ycnt)[Y_size],
                           double (*Zcnt)[Z_size], bcmg_shim_flag_t *FWS, int *wallcube) {
  ::BCM_Immersed_boundary(myid, ncube, n_wallcube, NBC, Xmin, Xmax, Ymin, Ymax, Zmin, Zmax,
                          cube_size, csl, Xcube, Ycube, Zcube, (double *)Xcnt, (double *)Ycnt,
                          (double *)Zcnt, (int *)FWS, wallcube);
}

// main.h:55-110 (setup, called at main.cpp:634 and :1070)
void BCM_FWS_Interface(int myid, int ncube, int mPI_Nadj, int ncpu_eq, int max_nei_eq,
                       int nadjX_eq, int nadjY_eq, int nadjZ_eq, int (*rank_map)[MPI_Ncube],
                       int *MPI_cpu, int *MPI_cube, int *MPI_cpu_adj, int *MPI_cube_adj,
                       int *MPI_direction, int *MPI_interface, int *neighbor_cpu_eq,
                       int *Ncube_Ncpu_eq, int *Scube_Ncpu_eq, int *Rcube_Ncpu_eq,
                       double *send_data_curr_eq, double *recv_data_curr_eq,
                       double *send_data_neig_eq, double *recv_data_neig_eq, int *Sdir_eq,
                       int *Rdir_eq, int *ist_eq, int *csl, int (*adj_number)[5][7],
                       int *adjX_eq, int *adjY_eq, int *adjZ_eq, bcmg_shim_flag_t *FWS) {
  ::BCM_FWS_Interface(myid, ncube, mPI_Nadj, ncpu_eq, max_nei_eq, nadjX_eq, nadjY_eq, nadjZ_eq,
                      (int *)rank_map, MPI_cpu, MPI_cube, MPI_cpu_adj, MPI_cube_adj,
                      MPI_direction, MPI_interface, neighbor_cpu_eq, Ncube_Ncpu_eq,
                      Scube_Ncpu_eq, Rcube_Ncpu_eq, send_data_curr_eq, recv_data_curr_eq,
                      send_data_neig_eq, recv_data_neig_eq, Sdir_eq, Rdir_eq, ist_eq, csl,
                      (int *)adj_number, adjX_eq, adjY_eq, adjZ_eq, (int *)FWS);
}
