// Kernel argument blocks and launchers shared by the C-ABI layer.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "bcm_common.cuh"
#include "bcm_mirror.cuh"

extern "C" void bcmg_internal_set_error(const char *msg);

namespace bcmg {

// Constants of one case in a batch: several independent cases laid end to
// end in one flat cube list (same n), each with the values the reference
// takes from its own prm.h / Resolution.h and its own time steps.  FP32
// copies for the split path are formed once on the host.
struct CaseConst {
  double mu_L, rho0, U0, Uin, P0;
  double E0;  // P0 / (K - 1), the energy of the mirror's reference state
  double dT, dTau, e;
  int mpi_ncube;
  float ef, rho0f, P0f, RT0f, T0f, mu_Lf, i2dtf, dTf, dTauf;
};
// Cube -> case map of a batch.  cube_case == nullptr: a single case whose
// constants are the scalar fields of the argument block.
struct Batch {
  const int *cube_case = nullptr;    // [ncube] case of each cube (slot 0 unused)
  const CaseConst *cases = nullptr;  // [ncase]
  // Convergence-driven sub-iterations: active[q] == 0 once case q met the
  // convergence test; kernels then leave its cubes alone.  nullptr: all
  // cases active.
  const int *active = nullptr;
};
__device__ __forceinline__ int case_of(const Batch &bt, int cube) {
  return bt.cube_case ? bt.cube_case[cube] : 0;
}
__device__ __forceinline__ bool case_active(const Batch &bt, int cube) {
  return !bt.active || bt.active[case_of(bt, cube)] != 0;
}
#ifdef __CUDACC__
// Reference state (rho0, E0 = P0/(K-1)) of the mirror deltas of a cube.
__device__ __forceinline__ void mirror_base(const Mirror &m, const Batch &bt, int cube,
                                            double &rho0, double &E0) {
  if (bt.cube_case) {
    const CaseConst &q = bt.cases[bt.cube_case[cube]];
    rho0 = q.rho0;
    E0 = q.E0;
  } else {
    rho0 = m.rho0;
    E0 = m.E0;
  }
}
#endif

struct FluxArgs {
  Phys ph;
  int cube0;  // first cube of this launch (cubes are 1-based)
  double dT, dTau, e;
  const int *FWS;
  const double *cube_size;
  const double *U1_, *U1, *U1q;
  double *Rku1, *Residual1;
  Batch bt;
  int raw = 0;  // 1: write the residual R itself (LU-SGS right-hand side)
  int tile = 0;  // tile edge 8 or 4 (0: 8 when n is a multiple of 8, else 4)
};

// FP64 residual + increment (bit-exact with the reference).
cudaError_t launch_flux_fp64(const FluxArgs &a, int ncubes, cudaStream_t s);

// Split-precision path (bcm_flux_split.cu): FP32 reconstruction, fluxes,
// viscous terms and preconditioner on deltas from a reference state; FP64
// state, time-level differences, update and norm sums.
struct FluxSplitArgs {
  Phys ph;
  int cube0;
  double dT, dTau;
  float ef;  // e (beta floor)
  // FP32 constants formed once on the host (FP64 arithmetic on the device
  // costs 64 FP32 issue slots per instruction on this part)
  float rho0f, P0f, RT0f, T0f, mu_Lf, i2dtf, dTf, dTauf;
  const float *inv_dx;  // [ncube] n / cube_size
  const int *FWS;
  const double *cube_size;
  // FP32 deltas of U1_: the kernel reads the current buffer; at stages 1..3
  // it writes the deltas of every interior cell of its tile (updated or
  // not) and of the same-level ghost layers it pushes into the other buffer
  // (launch_mirror_flip then makes that one current).
  Mirror mir;
  double *U1_;     // updated in place for the CTA's own cells
  const double *U1, *U1q;
  const float *D2;  // FP32 of the FP64 difference U1 - U1q (k_level_diff)
  int RK;              // stage 1..3: the kernel applies the stage update;
                       // 0: it writes the FP32 residual to R32 instead
  float *R32 = nullptr;  // [ncell][5] (RK == 0)
  int tile = 0;          // tile edge 8 or 4 (0: 8 when n is a multiple of 8, else 4)
  int form = 0;          // 8^3 tiles: 0 faces one at a time, 1 in packed FP32 pairs
  double *partials;    // [blocks][7] norm/force partial sums (stage 3)
  double *Residual1;
  Batch bt;
  // [ncube][6] (stages 1..3, optional): push[6c + 2 axis + 0] is the cube
  // whose high ghost layers copy cube c's low interior layers (2, 3) along
  // axis at the same level, push[6c + 2 axis + 1] the cube whose low ghost
  // layers copy its high layers (n, n+1); 0 where none.  Updated fluid
  // cells in those layers write their new value there too.
  const int *push = nullptr;
};
// Tile edge a flux launch uses (tile: 0 default, else 8 or 4 when it divides n).
int flux_tile(int n, int tile);
// Blocks of one split flux launch over ncubes cubes (one per tile).
int flux_split_blocks(int n, int ncubes, int tile = 0);
// Full mirror of U into M0 and, when not null, M1 (all cells of all cubes).
cudaError_t launch_mirror(const double *U, float *M0, float *M1, int n, int ncube, double rho0,
                          double P0, const Batch &bt, cudaStream_t s);
// Makes the other mirror buffer current (after an RK-stage flux launch).
cudaError_t launch_mirror_flip(int *parity, cudaStream_t s);
cudaError_t launch_flux_split(const FluxSplitArgs &a, int ncubes, cudaStream_t s);
cudaError_t launch_level_diff(const double *U1, const double *U1q, float *D2, int n, int ncube,
                              cudaStream_t s);

struct RkArgs {
  Phys ph;
  int ncube;  // cube slots incl. slot 0
  int RK;
  const int *FWS;
  double *U1_, *U1p1, *U1p2;
  const double *Rku1, *Residual1;
  double *partials;  // [nblocks][7] norm/force partial sums (RK == 3)
  // Batches: block b sums interior cells [blk_beg[b], blk_beg[b+1]) of the
  // flat numbering (c-1)*n^3 + r, so no block straddles two cases.  nullptr:
  // equal chunks over all cubes.
  const long long *blk_beg = nullptr;
  Batch bt;
};

// Stage combination (BCM_Flux...cpp:2417-2599) and, at RK 3, the per-block
// partial sums of the change norms and force integrands.
cudaError_t launch_rk(const RkArgs &a, int *nblocks_out, cudaStream_t s);
// Number of partial-sum blocks launch_rk uses for this case (for sizing).
int rk_partial_blocks(const RkArgs &a);
// Same combination with an explicit chunk (cells per block) and block count.
cudaError_t launch_rk_chunked(const RkArgs &a, long long chunk, int nblocks, cudaStream_t s);
// Deterministic final reduction of partials -> er[1..7] (device, 8 doubles).
cudaError_t launch_norms(const Phys &ph, const double *partials, int nblocks, double *er,
                         cudaStream_t s, const int *active = nullptr);
// Cube-sharded runs: raw sums of the partial blocks (sums[7]), and the norms
// er[1..7] from sums added over the ranks.
cudaError_t launch_norm_sums(const double *partials, int nblocks, double *sums, cudaStream_t s,
                             const int *active = nullptr);
cudaError_t launch_norm_final(const Phys &ph, const double *sums, double *er, cudaStream_t s,
                              const int *active = nullptr);
// Batches: case q reduces partial blocks [case_blk[q], case_blk[q+1]) into
// er[8q .. 8q+7] with its own normalisers.
cudaError_t launch_norms_batch(int n, const CaseConst *cases, const int *case_blk, int ncase,
                               const double *partials, double *er, cudaStream_t s,
                               const int *active = nullptr);
// Batch form of launch_rk over an explicit block table (nblocks blocks).
cudaError_t launch_rk_table(const RkArgs &a, int nblocks, cudaStream_t s);

// LU-SGS sub-iteration (bcm_lusgs.cu; no reference counterpart): per cube,
// forward and backward Gauss-Seidel sweeps over the planes i+j+k = const,
// then Q += dq on fluid cells with per-cube norm/force partial sums.
struct LusgsArgs {
  Phys ph;
  double dT, cfl, omega;
  const int *FWS;
  const double *cube_size;
  double *U1_;             // updated in place on fluid cells
  double *Rku1;            // in: residual; out: increment
  double *coefA, *coefB;   // [ncell][5] each: scratch for the cell coefficients
  const double *Residual1; // force integrands (summed into the partials)
  double *partials;        // [ncube-1][7]
  Batch bt;
};
cudaError_t launch_lusgs(const LusgsArgs &a, int ncubes, cudaStream_t s);

// Split-precision LU-SGS: FP32 sweeps on the FP32 mirror of the state (deltas
// from the case's reference state), FP64 update and norm sums.
struct LusgsSplitArgs {
  Phys ph;
  float dTf, cflf, omegaf;
  float rho0f, P0f, T0f, mu_Lf;
  const int *FWS;
  const float *inv_dx;     // [ncube] n / cube_size
  Mirror mir;              // FP32 deltas of the state: read and updated in place
  double *U1_;             // updated in place on fluid cells
  const float *R32;        // residual (FP32) of every cell
  float *scr;              // [ncube-1][11][n^3] sweep scratch (lusgs_split_scratch)
  int threads = 0;         // threads per cube (0: the widest plane, in whole warps)
  const double *Residual1;
  double *partials;        // [ncube-1][7]
  Batch bt;
  const int *push = nullptr;  // same-level push table (FluxSplitArgs::push)
};
cudaError_t launch_lusgs_split(const LusgsSplitArgs &a, int ncubes, cudaStream_t s);
// Floats of that scratch per cube.
size_t lusgs_split_scratch(int n);
// Default threads per cube of the split LU-SGS kernel (the widest plane).
int lusgs_split_default_threads(int n);

// PLOT3D byte images of BCM_Output (bcm_output.cu) for cubes
// [cube0, cube0 + ncubes): solution (4 + 5 (n+2)^3 doubles per cube) and
// grid (3 (n+2)^3 doubles per cube; origin [ncubes][3] of those cubes).
cudaError_t launch_plot3d_q(const double *U, double *out, int n, int cube0, int ncubes,
                            cudaStream_t s);
cudaError_t launch_plot3d_x(const double *cube_size, const double *origin, double *out, int n,
                            int cube0, int ncubes, cudaStream_t s);

// Interface: face-copy tasks (destination cube, source cube, axis, side) built
// on the host, then the ordered three-phase edge fill of every cube.
struct FaceTask {
  int32_t src;   // source cube
  int8_t axis;   // 0 x, 1 y, 2 z
  int8_t side;   // 0: destination's low ghost layers, 1: its high ghost layers
  int8_t kind;   // 0 same-level copy, 1 coarse->fine injection, 2 fine->coarse average
  int8_t slot;   // kinds 1, 2: sub-face slot 1..4 of the small cube on the big face
};
struct InterfaceArgs {
  int n;
  int ntasks;             // face tasks (all destination cubes)
  const int *task_cube;   // [ntasks] destination cube of each task
  const FaceTask *tasks;  // [ntasks]
  double *U1_;
  Batch bt;
  Mirror mir;  // split precision: every written cell's mirror value too
  bool edge_list = false;           // the edge fill over edge_cubes only (else all)
  const int *edge_cubes = nullptr;  // [nedge] cube numbers
  int nedge = 0;
};
cudaError_t launch_interface(const InterfaceArgs &a, int ndst, cudaStream_t s);

// Halo exchange of cube-sharded runs: band b = bands[4b..4b+3] = (cube slot,
// axis, side 1 high / 0 low face, layers); its cells are the `layers`
// interior layers next to that face over the whole n x n face, starting at
// cell offs[b] of the buffer; the buffer holds every cell's five doubles,
// then (split precision) its five mirror floats.  unpack = 0 gathers U (and
// the current mirror buffer) into the buffer, 1 scatters the buffer into
// them.
cudaError_t launch_halo(double *U, const Mirror &mir, const int *bands, const long long *offs,
                        int nband, long long total_cells, int n, void *buf, int unpack,
                        cudaStream_t s);

// X/Y/Z boundary conditions for a list of (cube, mask) pairs; mask bits
// 0..5 = x lower, x upper, y lower, y upper, z lower, z upper.  axes selects
// which of the three phases run (bit 0 x, 1 y, 2 z).
struct BcArgs {
  int n;
  double Uin;
  const int *cubes;
  const int *masks;
  int axes;
  double *U1_;
  Batch bt;  // batches: Uin of the cube's case
  Mirror mir;  // split precision: every written cell's mirror value too
};
cudaError_t launch_bc(const BcArgs &a, int ncubes, cudaStream_t s);

// IBM ghost-cell fill for one dependency level of the combined entry list.
struct GhostArgs {
  int n;
  double rho0, P0;
  const int *entries;      // entry numbers (1-based) of this level
  const double *weight;    // 1-based packed [8*nbc+1]
  const int *GCindex;      // 1-based packed [4*nbc+1]
  const int *IPsur;        // 1-based packed [4*nbc+1]
  double *U1_;
  Batch bt;  // batches: rho0, P0 of the ghost cell's case
  Mirror mir;  // split precision: the ghost cell's mirror value too
};
// priority != 0: launched with that scheduling priority (a launch
// attribute, kept by stream capture), so its blocks go ahead of pending
// blocks of lower-priority kernels running beside it
cudaError_t launch_ghost(const GhostArgs &a, int count, cudaStream_t s, int priority = 0);

}  // namespace bcmg
