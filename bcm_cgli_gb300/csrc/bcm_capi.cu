// C ABI: drop-in twins of the reference routines and the device-resident
// case context.  See include/bcm_gb300.h for the contract of every entry
// point.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <thread>
#include <map>
#include <vector>

#include <unistd.h>

#include "../../include/bcm_gb300.h"
#include "bcm_kernels.h"
#include "bcm_tables.h"
#include "bcm_trace.h"

using namespace bcmg;

namespace {

thread_local std::string g_err;
thread_local bool g_has_err = false;

void set_err(const std::string &s) {
  g_err = s;
  g_has_err = true;
}
void clear_err() { g_has_err = false; }

#define CK(expr)                                                                     \
  do {                                                                               \
    cudaError_t e__ = (expr);                                                        \
    if (e__ != cudaSuccess) {                                                        \
      set_err(std::string(#expr) + ": " + cudaGetErrorString(e__));                  \
      cudaGetLastError(); /* a non-sticky error must not reach the next call */      \
      return BCMG_ERR_CUDA;                                                          \
    }                                                                                \
  } while (0)

template <typename T>
cudaError_t dalloc(T **p, size_t count) {
  *p = nullptr;
  if (count == 0) count = 1;
  return cudaMalloc((void **)p, sizeof(T) * count);
}

template <typename T>
void dfree(T *&p) {
  if (p) cudaFree(p);
  p = nullptr;
}

__global__ void k_time_shift(int n, int ncubes, const double2 *__restrict__ U1_,
                             double2 *__restrict__ U1, double2 *__restrict__ U1q) {
  // main.cpp:1292-1315: U1q <- U1, U1 <- U1_ on interior cells.  An interior
  // row (cube, i, j) is 5n contiguous doubles starting at an even cell index
  // (S even), so it moves as 5n/2 aligned 16-byte pairs; cubes on blockIdx.y.
  const int S = n + 4, rl = 5 * n / 2, per = n * n * rl;
  for (int cube = 1 + blockIdx.y; cube <= ncubes; cube += gridDim.y)
    for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < per; w += gridDim.x * blockDim.x) {
      const int row = w / rl, e = w - row * rl;
      const size_t o = 5 * cell_index(S, cube, 2 + row / n, 2 + row % n, 2) / 2 + e;
      const double2 a = U1[o], b = U1_[o];
      U1q[o] = a;
      U1[o] = b;
    }
}

// Split-precision flux twin: the stage's new state of the fluid interior
// cells into U1p1 (RK 1) or U1p2 (RK 2), as the reference's stage
// combination leaves them (BCM_Flux_XYZ_Viscous_Runge_kutta.cpp:2417-2599).
__global__ void k_copy_fluid(int n, int ncubes, const double *__restrict__ U1_,
                             const int *__restrict__ FWS, double *__restrict__ dst) {
  const int S = n + 4;
  const long long n3 = (long long)n * n * n, total = n3 * ncubes;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int c = 1 + (int)(t / n3), r = (int)(t % n3);
    const size_t o = cell_index(S, c, 2 + r / (n * n), 2 + (r / n) % n, 2 + r % n);
    if (FWS[o] != kFluid) continue;
#pragma unroll
    for (int v = 0; v < 5; ++v) dst[5 * o + v] = U1_[5 * o + v];
  }
}

__global__ void k_emax(double *er, double *emax, const int *active) {
  // main.cpp:1249-1259: E_k = max(E_k, er_k); er_k /= E_k.  One block per
  // case: er[8q..], emax[6q..]; converged cases keep theirs.
  if (active && !active[blockIdx.x]) return;
  er += 8 * (size_t)blockIdx.x;
  emax += 6 * (size_t)blockIdx.x;
  const int v = threadIdx.x + 1;
  if (v <= 5) {
    double E = emax[v] > er[v] ? emax[v] : er[v];
    emax[v] = E;
    er[v] = er[v] / E;
  }
}

// Convergence-driven sub-iterations (main.cpp:1249-1271): before a step
// every case is active with zero sub-iterations; after each sub-iteration
// (and its E normalisation) a case whose normalised change norms er[1..5]
// are all below tol, or that reached max_subiters, becomes inactive; the
// loop continues while any case is active.  With a graph handle the
// decision drives the step graph's while node on the device.
__global__ void k_conv_reset(int *active, int *iters, int ncase) {
  for (int q = threadIdx.x; q < ncase; q += blockDim.x) {
    active[q] = 1;
    iters[q] = 0;
  }
}

__global__ void k_conv_check(const double *er, int *active, int *iters, int ncase, double tol,
                             int max_subiters, int *cont, cudaGraphConditionalHandle h,
                             int use_handle) {
  if (threadIdx.x != 0) return;
  int any = 0;
  for (int q = 0; q < ncase; ++q) {
    if (!active[q]) continue;
    const double *e = er + 8 * (size_t)q;
    const int it = ++iters[q];
    const bool conv = e[1] < tol && e[2] < tol && e[3] < tol && e[4] < tol && e[5] < tol;
    if (conv || it >= max_subiters)
      active[q] = 0;
    else
      any = 1;
  }
  *cont = any;
  if (use_handle) cudaGraphSetConditional(h, any ? 1u : 0u);
}

__global__ void k_store_iters(const int *iters, int *dst, int ncase) {
  for (int q = threadIdx.x; q < ncase; q += blockDim.x) dst[q] = iters[q];
}

struct Ibm {
  int nbc = 0;
  double *w = nullptr;
  int *gc = nullptr, *ip = nullptr, *order = nullptr;
  std::vector<int> level_off;
  void release() {
    dfree(w);
    dfree(gc);
    dfree(ip);
    dfree(order);
    nbc = 0;
    level_off.clear();
  }
};

// Upload one IBM table (1-based packed) and its dependency levels.
int ibm_upload(Ibm &t, int nbc, const double *w, const int *gc, const int *ip, int n, int ncube,
               cudaStream_t s) {
  t.release();
  if (nbc <= 0) return BCMG_OK;
  std::vector<int> order;
  std::string err;
  if (!build_ibm_levels(nbc, gc, ip, n, ncube, order, t.level_off, err)) {
    set_err(err);
    return BCMG_ERR_ARG;
  }
  t.nbc = nbc;
  CK(dalloc(&t.w, (size_t)8 * nbc + 1));
  CK(dalloc(&t.gc, (size_t)4 * nbc + 1));
  CK(dalloc(&t.ip, (size_t)4 * nbc + 1));
  CK(dalloc(&t.order, (size_t)nbc));
  CK(cudaMemcpyAsync(t.w, w, sizeof(double) * (8 * (size_t)nbc + 1), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(t.gc, gc, sizeof(int) * (4 * (size_t)nbc + 1), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(t.ip, ip, sizeof(int) * (4 * (size_t)nbc + 1), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(t.order, order.data(), sizeof(int) * nbc, cudaMemcpyHostToDevice, s));
  CK(cudaStreamSynchronize(s));
  return BCMG_OK;
}

int ibm_run(const Ibm &t, int n, double rho0, double P0, double *U, cudaStream_t s,
            long long *launches, const Batch &bt = Batch(), const Mirror &mir = Mirror(),
            int priority = 0) {
  for (size_t l = 1; l < t.level_off.size(); ++l) {
    GhostArgs g;
    g.n = n;
    g.rho0 = rho0;
    g.P0 = P0;
    g.entries = t.order + t.level_off[l - 1];
    g.weight = t.w;
    g.GCindex = t.gc;
    g.IPsur = t.ip;
    g.U1_ = U;
    g.bt = bt;
    g.mir = mir;
    CK(launch_ghost(g, t.level_off[l] - t.level_off[l - 1], s, priority));
    if (launches) ++*launches;
  }
  return BCMG_OK;
}

bool valid_n(int n) { return n >= 4 && n % 4 == 0 && n <= 256; }

}  // namespace

// ===========================================================================
// Device-resident case context
// ===========================================================================
struct bcmg_case {
  Phys ph{};
  int ncube = 0, S = 0;
  // Cube-sharded runs (bcmg_case_create_shard): cube slots 1..nreal are this
  // rank's cubes, the rest proxies of remote cubes (read by face tasks,
  // filled by the halo exchange, never advanced).  nreal = ncube - 1 else.
  int nreal = 0;
  bcmg_exchange_fn xchg = nullptr;
  void *xchg_user = nullptr;
  double *nsum = nullptr;  // device [7]: raw norm sums handed to the exchange hook
  struct Halo {
    int *send = nullptr, *recv = nullptr;            // device band tables (4 ints each)
    long long *soff = nullptr, *roff = nullptr;      // device first cell of each band
    int nsend = 0, nrecv = 0;
    long long send_cells = 0, recv_cells = 0;
  };
  std::vector<Halo> halo;
  double dT = 0, dTau = 0, e = 0;
  int precision = 0;
  size_t ncell = 0;
  cudaStream_t stream = nullptr;
  double *U1_ = nullptr, *U1 = nullptr, *U1q = nullptr, *U1p1 = nullptr, *U1p2 = nullptr,
         *Rku1 = nullptr, *Residual1 = nullptr;
  // Split precision: the FP32 mirror of U1_ (deltas from each case's
  // reference state) in two buffers, the device flag naming the current one
  // (bcm_mirror.cuh), and whether the whole mirror is re-formed before every
  // flux launch (the old per-stage pass; kept to check the incremental
  // mirror against it) instead of once per dual-time step.
  float *M = nullptr, *M2 = nullptr;
  int *mpar = nullptr;
  bool mirror_each_stage = false;
  Mirror mir() const {
    Mirror m;
    if (M) {
      m.buf[0] = M;
      m.buf[1] = M2;
      m.parity = mpar;
      m.rho0 = ph.rho0;
      m.E0 = ph.P0 / (BCMG_K - 1);
    }
    return m;
  }
  float *D2 = nullptr;                   // split precision: FP32 of U1 - U1q
  float *inv_dx = nullptr;               // split precision: n / cube_size per cube
  int *FWS = nullptr;
  double *cube_size = nullptr;
  int *task_cube = nullptr;  // destination cube of each face task
  FaceTask *tasks = nullptr;
  int ntasks = 0;
  // The face tasks a stage's first interface call must repeat after the
  // previous stage's last one (main.cpp:1161-1204 runs the interface before
  // and after every update): level jumps, faces the boundary fill writes and
  // faces whose source or destination layers hold IBM ghost cells.  The
  // other copies would write the values already there: between the two
  // calls only the boundary fill (its own ghost faces) and the IBM ghost
  // fill (its listed cells) write the state.
  int *task_cube_p = nullptr;
  FaceTask *tasks_p = nullptr;
  int ntasks_p = 0;
  // Split-precision RK stages and LU-SGS sweeps make the same-level face
  // copies of the cells they update inside the updating kernel (push table,
  // see FluxSplitArgs::push); their closing interface call then runs only
  // the level-jump tasks (and the edge fill).  push == nullptr: the table
  // could not be formed (one source layer pair feeding two faces).
  int *push = nullptr;
  bool push_on = true;  // bcmg_case_set_face_copies
  const int *push_table() const { return push_on ? push : nullptr; }
  int *task_cube_q = nullptr;
  FaceTask *tasks_q = nullptr;
  int ntasks_q = 0;
  // the closing call of split RK stages 1 and 2: the level jumps and edge
  // fills read before the next stage's opening call rewrites them
  int *task_cube_r = nullptr, *edge_r = nullptr;
  FaceTask *tasks_r = nullptr;
  int ntasks_r = 0, nedge_r = 0;
  bool closing_reduced = false;
  int *bc_cubes = nullptr, *bc_masks = nullptr;
  int nbc = 0;
  // The IBM ghost fill on a side stream beside the boundary fill: allowed
  // when no cube holds both an IBM entry's cells (ghost or stencil) and a
  // boundary face, so neither reads or writes a cell of the other; the
  // interface call after them waits for both.
  bool ghost_beside_bc = false;  // a side table exists
  Ibm ibm_side;                  // the entries filled beside the boundary fill
  bool ghost_side_on = true;     // bcmg_case_set_concurrent_ghosts
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  int side_priority = 0;  // the device's highest scheduling priority
  Ibm ibm;  // minus entries then plus entries, one combined schedule
  double *partials = nullptr;
  int nparts = 0;
  double *er = nullptr, *emax = nullptr;  // device [8 ncase], [6 ncase]
  // Batches (bcmg_batch_create): several cases end to end in one flat cube
  // list; case q owns cubes [case_cube0[q], case_cube0[q+1]).
  bool batched = false;
  int ncase = 1;
  std::vector<int> case_cube0;
  std::vector<CaseConst> hcases;
  CaseConst *cases = nullptr;   // device [ncase]
  int *cube_case = nullptr;     // device [ncube]
  long long *rk_blk = nullptr;  // device [nrk+1]: FP64 stage-update blocks
  int nrk = 0;
  int *case_blk_rk = nullptr, *case_blk_flux = nullptr;  // device [ncase+1]
  int *case_blk_cube = nullptr;                           // device [ncase+1]
  // Sub-iteration method (bcmg_case_set_method): RK3 (the reference's) or
  // LU-SGS with its pseudo-time CFL (0: none) and relaxation factor.
  int method = BCMG_METHOD_RK3;
  // Launch shapes (bcmg_case_set_tuning / bcmg_case_autotune): flux tile
  // edge (0: default) and threads per cube of the split LU-SGS sweep.
  int tile = 0, lu_threads = 0;
  int form = 0;  // split flux on 8^3 tiles: 0 default (packed pairs), 1 packed, 2 one face at a time
  double lu_cfl = 0.0, lu_omega = 1.5;
  // Convergence-driven stepping (bcmg_case_advance_converged)
  bool conv = false;                 // kernels see the active masks
  int *active = nullptr, *iters = nullptr, *cont = nullptr;  // device
  cudaGraphExec_t cgraph = nullptr;  // step graph with the while node
  int cgraph_max = -1, cgraph_method = -1;
  double cgraph_tol = -1;
  float *lu_scr = nullptr;  // split LU-SGS sweep scratch
  // PLOT3D output (bcmg_case_output_*): device byte image, a side stream for
  // the copies, two pinned chunks and the writer thread.
  int device = 0;
  double *out_dev = nullptr;
  size_t out_cap = 0;  // doubles
  cudaStream_t out_stream = nullptr;
  cudaEvent_t out_ready = nullptr, out_chunk[2] = {nullptr, nullptr};
  char *out_host[2] = {nullptr, nullptr};
  std::thread out_thread;
  int out_status = 0;
  std::string out_err;
  Batch bt() const {
    Batch b;
    if (batched) {
      b.cube_case = cube_case;
      b.cases = cases;
    }
    if (conv) b.active = active;
    return b;
  }
  cudaGraphExec_t graph = nullptr;
  int graph_subiters = -1;
  // Kernel nodes of the captured step graph, counted while capturing; of
  // the convergence-driven graph, per pass of the while body and outside it.
  long long graph_launches = 0, cgraph_body = 0, cgraph_outer = 0;
  long long launches = 0;
  bool profile = false;
  std::vector<cudaEvent_t> ev;
  size_t ev_used = 0;
  double flux_ms = 0;
  long long flux_launches = 0;
  std::vector<cudaEvent_t> marks;  // bcmg_case_timer_mark slots

  void join_output() {
    if (out_thread.joinable()) out_thread.join();
  }
  void release() {
    join_output();
    if (out_dev) cudaFree(out_dev);
    out_dev = nullptr;
    for (int i = 0; i < 2; ++i) {
      if (out_host[i]) cudaFreeHost(out_host[i]);
      out_host[i] = nullptr;
      if (out_chunk[i]) cudaEventDestroy(out_chunk[i]);
      out_chunk[i] = nullptr;
    }
    if (out_ready) cudaEventDestroy(out_ready);
    out_ready = nullptr;
    if (out_stream) cudaStreamDestroy(out_stream);
    out_stream = nullptr;
    for (auto x : marks)
      if (x) cudaEventDestroy(x);
    marks.clear();
    if (graph) cudaGraphExecDestroy(graph);
    graph = nullptr;
    if (cgraph) cudaGraphExecDestroy(cgraph);
    cgraph = nullptr;
    dfree(active); dfree(iters); dfree(cont); dfree(lu_scr);
    for (auto x : ev) cudaEventDestroy(x);
    ev.clear();
    dfree(U1_); dfree(U1); dfree(U1q); dfree(U1p1); dfree(U1p2); dfree(Rku1); dfree(Residual1);
    dfree(M); dfree(M2); dfree(mpar); dfree(D2); dfree(inv_dx);
    dfree(FWS); dfree(cube_size); dfree(task_cube); dfree(tasks); dfree(task_cube_p);
    dfree(tasks_p); dfree(push); dfree(task_cube_q); dfree(tasks_q); dfree(bc_cubes);
    dfree(task_cube_r); dfree(tasks_r); dfree(edge_r);
    dfree(bc_masks); dfree(partials); dfree(er); dfree(emax);
    dfree(cases); dfree(cube_case); dfree(rk_blk); dfree(case_blk_rk); dfree(case_blk_flux);
    dfree(case_blk_cube);
    dfree(nsum);
    for (auto &h : halo) {
      dfree(h.send); dfree(h.recv); dfree(h.soff); dfree(h.roff);
    }
    halo.clear();
    ibm.release();
    ibm_side.release();
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_join) cudaEventDestroy(ev_join);
    ev_fork = ev_join = nullptr;
    if (side) cudaStreamDestroy(side);
    side = nullptr;
    if (stream) cudaStreamDestroy(stream);
    stream = nullptr;
  }
};

namespace {

int case_flux(bcmg_case *c, int RK) {
  FluxArgs a;
  a.ph = c->ph;
  a.cube0 = 1;
  a.dT = c->dT;
  a.dTau = c->dTau;
  a.e = c->e;
  a.FWS = c->FWS;
  a.cube_size = c->cube_size;
  a.U1_ = c->U1_;
  a.U1 = c->U1;
  a.U1q = c->U1q;
  a.Rku1 = c->Rku1;
  a.Residual1 = c->Residual1;
  a.bt = c->bt();
  a.raw = RK == 0;  // residual only (LU-SGS)
  a.tile = c->tile;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (c->profile) {
    while (c->ev.size() < c->ev_used + 2) {
      cudaEvent_t x;
      CK(cudaEventCreate(&x));
      c->ev.push_back(x);
    }
    e0 = c->ev[c->ev_used];
    e1 = c->ev[c->ev_used + 1];
    c->ev_used += 2;
  }
  if (c->precision == BCMG_PRECISION_SPLIT && c->mirror_each_stage) {
    CK(launch_mirror(c->U1_, c->M, c->M2, c->ph.n, c->ncube, c->ph.rho0, c->ph.P0, c->bt(),
                     c->stream));
    ++c->launches;
  }
  // the timed span is the flux kernel alone
  if (c->profile) CK(cudaEventRecord(e0, c->stream));
  if (c->precision == BCMG_PRECISION_SPLIT) {
    FluxSplitArgs sa;
    sa.ph = c->ph;
    sa.cube0 = 1;
    sa.dT = c->dT;
    sa.dTau = c->dTau;
    sa.ef = (float)c->e;
    sa.rho0f = (float)c->ph.rho0;
    sa.P0f = (float)c->ph.P0;
    sa.RT0f = (float)(c->ph.P0 / c->ph.rho0);
    sa.T0f = (float)(c->ph.P0 / c->ph.rho0 / BCMG_R);
    sa.mu_Lf = (float)c->ph.mu_L;
    sa.i2dtf = (float)(1.0 / (2.0 * c->dT));
    sa.dTf = (float)c->dT;
    sa.dTauf = (float)c->dTau;
    sa.inv_dx = c->inv_dx;
    sa.FWS = c->FWS;
    sa.cube_size = c->cube_size;
    sa.mir = c->mir();
    sa.U1_ = c->U1_;
    sa.U1 = c->U1;
    sa.U1q = c->U1q;
    sa.D2 = c->D2;
    sa.RK = RK;
    // RK 0 (LU-SGS): FP32 residual into the Rku1 buffer, which the split
    // path does not otherwise use
    sa.R32 = reinterpret_cast<float *>(c->Rku1);
    sa.tile = c->tile;
    sa.form = c->form == 2 ? 0 : 1;
    sa.partials = c->partials;
    sa.Residual1 = c->Residual1;
    sa.bt = c->bt();
    sa.push = RK >= 1 ? c->push_table() : nullptr;
    CK(launch_flux_split(sa, c->nreal, c->stream));
  } else {
    CK(launch_flux_fp64(a, c->nreal, c->stream));
  }
  if (c->profile) CK(cudaEventRecord(e1, c->stream));
  ++c->launches;
  if (c->precision == BCMG_PRECISION_SPLIT && RK >= 1) {
    // the flux kernel wrote the stage's mirror into the other buffer
    CK(launch_mirror_flip(c->mpar, c->stream));
    ++c->launches;
  }
  return BCMG_OK;
}

// Which face tasks an interface call runs.
enum IfaceList { kIfaceFull, kIfacePrologue, kIfaceClosing, kIfaceClosingReduced };

int case_interface(bcmg_case *c, IfaceList list = kIfaceFull) {
  if (c->xchg) {  // sharded: the proxies' face bands first
    if (c->xchg(c->xchg_user, BCMG_XCHG_HALO, c->stream) != 0) {
      set_err("exchange hook failed (halo)");
      return BCMG_ERR_CUDA;
    }
  }
  InterfaceArgs ia;
  ia.n = c->ph.n;
  ia.ntasks = c->ntasks;
  ia.task_cube = c->task_cube;
  ia.tasks = c->tasks;
  if (list == kIfacePrologue) {
    ia.ntasks = c->ntasks_p;
    ia.task_cube = c->task_cube_p;
    ia.tasks = c->tasks_p;
  } else if (list == kIfaceClosing) {
    ia.ntasks = c->ntasks_q;
    ia.task_cube = c->task_cube_q;
    ia.tasks = c->tasks_q;
  } else if (list == kIfaceClosingReduced) {
    ia.ntasks = c->ntasks_r;
    ia.task_cube = c->task_cube_r;
    ia.tasks = c->tasks_r;
    ia.edge_list = true;
    ia.edge_cubes = c->edge_r;
    ia.nedge = c->nedge_r;
  }
  ia.U1_ = c->U1_;
  ia.bt = c->bt();
  ia.mir = c->mir();
  CK(launch_interface(ia, c->ncube, c->stream));
  c->launches += (ia.ntasks > 0 ? 1 : 0) + (ia.edge_list && ia.nedge == 0 ? 0 : 1);
  return BCMG_OK;
}

// Boundary conditions, IBM ghost cells and interface ahead of each update
// (main.cpp:1161-1204).  full == false: the stage follows another stage's
// closing interface call, so only the face copies that can change run.
int case_prologue(bcmg_case *c, bool full = true) {
  int r;
  const bool beside = c->ghost_beside_bc && c->ghost_side_on;
  if (beside) {  // fork: the side table's ghost levels on the side stream
    CK(cudaEventRecord(c->ev_fork, c->stream));
    CK(cudaStreamWaitEvent(c->side, c->ev_fork, 0));
    if ((r = ibm_run(c->ibm_side, c->ph.n, c->ph.rho0, c->ph.P0, c->U1_, c->side, &c->launches,
                     c->bt(), c->mir(), c->side_priority)))
      return r;
    CK(cudaEventRecord(c->ev_join, c->side));
  }
  if (c->nbc > 0) {
    BcArgs b;
    b.n = c->ph.n;
    b.Uin = c->ph.Uin;
    b.cubes = c->bc_cubes;
    b.masks = c->bc_masks;
    b.axes = 7;
    b.U1_ = c->U1_;
    b.bt = c->bt();
    b.mir = c->mir();
    CK(launch_bc(b, c->nbc, c->stream));
    ++c->launches;
  }
  if (beside) {  // join; the other cases' entries after the boundary fill
    CK(cudaStreamWaitEvent(c->stream, c->ev_join, 0));
  } else if ((r = ibm_run(c->ibm_side, c->ph.n, c->ph.rho0, c->ph.P0, c->U1_, c->stream,
                          &c->launches, c->bt(), c->mir()))) {
    return r;
  }
  if ((r = ibm_run(c->ibm, c->ph.n, c->ph.rho0, c->ph.P0, c->U1_, c->stream, &c->launches,
                   c->bt(), c->mir())))
    return r;
  return case_interface(c, full ? kIfaceFull : kIfacePrologue);
}

// One LU-SGS sub-iteration: prologue, residual, sweeps with the update and
// per-cube norm partials, norms, interface.
LusgsSplitArgs lusgs_split_args(bcmg_case *c) {
  LusgsSplitArgs l;
  l.ph = c->ph;
  l.dTf = (float)c->dT;
  l.cflf = (float)c->lu_cfl;
  l.omegaf = (float)c->lu_omega;
  l.rho0f = (float)c->ph.rho0;
  l.P0f = (float)c->ph.P0;
  l.T0f = (float)(c->ph.P0 / c->ph.rho0 / BCMG_R);
  l.mu_Lf = (float)c->ph.mu_L;
  l.FWS = c->FWS;
  l.inv_dx = c->inv_dx;
  l.mir = c->mir();
  l.U1_ = c->U1_;
  l.R32 = reinterpret_cast<const float *>(c->Rku1);
  l.scr = c->lu_scr;
  l.Residual1 = c->Residual1;
  l.partials = c->partials;
  l.bt = c->bt();
  l.threads = c->lu_threads;
  l.push = c->push_table();
  return l;
}

// Norms of one case over nb partial blocks; sharded contexts hand the raw
// sums to the exchange hook, which adds them over the ranks.
int case_norms(bcmg_case *c, int nb) {
  if (!c->xchg) {
    CK(launch_norms(c->ph, c->partials, nb, c->er, c->stream, c->bt().active));
    ++c->launches;
    return BCMG_OK;
  }
  CK(launch_norm_sums(c->partials, nb, c->nsum, c->stream, c->bt().active));
  if (c->xchg(c->xchg_user, BCMG_XCHG_NORMS, c->stream) != 0) {
    set_err("exchange hook failed (norms)");
    return BCMG_ERR_CUDA;
  }
  CK(launch_norm_final(c->ph, c->nsum, c->er, c->stream, c->bt().active));
  c->launches += 2;
  return BCMG_OK;
}

int case_lusgs(bcmg_case *c, bool full = true) {
  int r;
  if ((r = case_prologue(c, full))) return r;
  if ((r = case_flux(c, 0))) return r;
  if (c->precision == BCMG_PRECISION_SPLIT) {
    CK(launch_lusgs_split(lusgs_split_args(c), c->nreal, c->stream));
  } else {
    LusgsArgs l;
    l.ph = c->ph;
    l.dT = c->dT;
    l.cfl = c->lu_cfl;
    l.omega = c->lu_omega;
    l.FWS = c->FWS;
    l.cube_size = c->cube_size;
    l.U1_ = c->U1_;
    l.Rku1 = c->Rku1;
    l.coefA = c->U1p1;
    l.coefB = c->U1p2;
    l.Residual1 = c->Residual1;
    l.partials = c->partials;
    l.bt = c->bt();
    CK(launch_lusgs(l, c->nreal, c->stream));
  }
  ++c->launches;
  if (c->batched)
    CK(launch_norms_batch(c->ph.n, c->cases, c->case_blk_cube, c->ncase, c->partials, c->er,
                          c->stream, c->bt().active));
  else if ((r = case_norms(c, c->nreal)))
    return r;
  if (c->batched) ++c->launches;
  // the split sweep made the same-level copies of the updated cells
  return case_interface(c, c->precision == BCMG_PRECISION_SPLIT && c->push_table()
                               ? kIfaceClosing
                               : kIfaceFull);
}

// reduced: the stage is RK 1 or 2 of a sub-iteration that goes on (not a
// single-stage call), so its closing interface call may leave out what the
// next stage's opening call rewrites before anything reads it.
int case_stage(bcmg_case *c, int RK, bool full = true, bool reduced = false) {
  int r;
  if ((r = case_prologue(c, full))) return r;
  if ((r = case_flux(c, RK))) return r;
  int nb = 0;
  if (c->precision == BCMG_PRECISION_SPLIT) {
    // the split flux kernel applied the stage update and wrote the partials
    nb = flux_split_blocks(c->ph.n, c->nreal, c->tile);
    if (RK == 3) {
      if (c->batched) {
        CK(launch_norms_batch(c->ph.n, c->cases, c->case_blk_flux, c->ncase, c->partials, c->er,
                              c->stream, c->bt().active));
        ++c->launches;
      } else if ((r = case_norms(c, nb))) {
        return r;
      }
    }
    // the flux kernel made the same-level copies of the updated cells
    if (!c->push_table()) return case_interface(c, kIfaceFull);
    return case_interface(c, reduced && c->closing_reduced && !c->xchg ? kIfaceClosingReduced
                                                                      : kIfaceClosing);
  }
  RkArgs k;
  k.ph = c->ph;
  k.ncube = c->nreal + 1;
  k.RK = RK;
  k.FWS = c->FWS;
  k.U1_ = c->U1_;
  k.U1p1 = c->U1p1;
  k.U1p2 = c->U1p2;
  k.Rku1 = c->Rku1;
  k.Residual1 = c->Residual1;
  k.partials = c->partials;
  k.bt = c->bt();
  if (c->batched) {
    k.blk_beg = c->rk_blk;
    CK(launch_rk_table(k, c->nrk, c->stream));
  } else {
    CK(launch_rk(k, &nb, c->stream));
  }
  ++c->launches;
  if (RK == 3) {
    if (c->batched) {
      CK(launch_norms_batch(c->ph.n, c->cases, c->case_blk_rk, c->ncase, c->partials, c->er,
                            c->stream, c->bt().active));
      ++c->launches;
    } else {
      int r = case_norms(c, nb);
      if (r) return r;
    }
  }
  return case_interface(c);
}

// One sub-iteration (three RK stages or one LU-SGS update) and the E
// normalisation of its norms (main.cpp:1249-1259).
int case_subiter(bcmg_case *c, bool full = true) {
  int r;
  if (c->method == BCMG_METHOD_LUSGS) {
    if ((r = case_lusgs(c, full))) return r;
  } else {
    for (int RK = 1; RK <= 3; ++RK)
      if ((r = case_stage(c, RK, full && RK == 1, RK < 3))) return r;
  }
  k_emax<<<c->ncase, 32, 0, c->stream>>>(c->er, c->emax, c->bt().active);
  CK(cudaGetLastError());
  ++c->launches;
  return BCMG_OK;
}

// Time-level shift at the end of a dual-time step (main.cpp:1292-1315).
int case_shift(bcmg_case *c) {
  const long long total = (long long)(c->ncube - 1) * c->ph.n * c->ph.n * c->ph.n;
  if (total > 0) {
    const int n = c->ph.n, per = n * n * (5 * n / 2);
    const dim3 grid((per + 255) / 256, std::min(c->ncube - 1, 65535));
    k_time_shift<<<grid, 256, 0, c->stream>>>(n, c->ncube - 1,
                                              reinterpret_cast<const double2 *>(c->U1_),
                                              reinterpret_cast<double2 *>(c->U1),
                                              reinterpret_cast<double2 *>(c->U1q));
    CK(cudaGetLastError());
    ++c->launches;
    if (c->precision == BCMG_PRECISION_SPLIT) {
      CK(launch_level_diff(c->U1, c->U1q, c->D2, c->ph.n, c->ncube, c->stream));
      ++c->launches;
    }
  }
  return BCMG_OK;
}

// The whole mirror of the current state, into both buffers: at the start of
// every dual-time step (and of a single-stage call), so that a state set or
// changed from outside, or a case that sat out sub-iterations after it
// converged, is mirrored exactly; within the step the kernels that write the
// state keep it current.
int case_mirror_all(bcmg_case *c) {
  if (c->precision != BCMG_PRECISION_SPLIT) return BCMG_OK;
  CK(launch_mirror(c->U1_, c->M, c->M2, c->ph.n, c->ncube, c->ph.rho0, c->ph.P0, c->bt(),
                   c->stream));
  ++c->launches;
  return BCMG_OK;
}

int case_step(bcmg_case *c, int subiters) {
  int r;
  if ((r = case_mirror_all(c))) return r;
  for (int it = 0; it < subiters; ++it)  // the step's first stage runs every face copy
    if ((r = case_subiter(c, it == 0))) return r;
  return case_shift(c);
}

// The step graph of convergence-driven stepping: reset of the masks, a
// while node whose body is one sub-iteration plus the convergence check
// (which sets the node's condition on the device), then the time shift.
int build_conv_graph(bcmg_case *c, int max_subiters, double tol) {
  if (c->cgraph) cudaGraphExecDestroy(c->cgraph);
  c->cgraph = nullptr;
  const cudaStreamCaptureMode mode = cudaStreamCaptureModeThreadLocal;
  cudaGraph_t g = nullptr;
  CK(cudaGraphCreate(&g, 0));
  struct Guard {
    cudaGraph_t *g;
    ~Guard() { if (*g) cudaGraphDestroy(*g); }
  } guard{&g};
  cudaGraphConditionalHandle h;
  CK(cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault));
  CK(cudaStreamBeginCaptureToGraph(c->stream, g, nullptr, nullptr, 0, mode));
  k_conv_reset<<<1, 128, 0, c->stream>>>(c->active, c->iters, c->ncase);
  cudaError_t le = cudaGetLastError();
  const long long l_pre = c->launches;
  int rm = le == cudaSuccess ? case_mirror_all(c) : BCMG_OK;
  const long long pre_nodes = 1 + (c->launches - l_pre);
  CK(cudaStreamEndCapture(c->stream, &g));
  if (rm) return rm;
  CK(le);
  // the node the while node follows: the last of the nodes captured above
  // (reset, then the mirror on the split path), which form a chain
  std::vector<cudaGraphNode_t> pre((size_t)pre_nodes);
  size_t nn = pre.size();
  CK(cudaGraphGetNodes(g, pre.data(), &nn));
  cudaGraphNode_t reset = nullptr;
  for (size_t i = 0; i < nn; ++i) {
    size_t ndep = 0;
    CK(cudaGraphNodeGetDependentNodes(pre[i], nullptr, nullptr, &ndep));
    if (ndep == 0) reset = pre[i];
  }
  cudaGraphNodeParams p = {};
  p.type = cudaGraphNodeTypeConditional;
  p.conditional.handle = h;
  p.conditional.type = cudaGraphCondTypeWhile;
  p.conditional.size = 1;
  cudaGraphNode_t wnode;
  CK(cudaGraphAddNode(&wnode, g, &reset, nullptr, 1, &p));
  cudaGraph_t body = p.conditional.phGraph_out[0];
  CK(cudaStreamBeginCaptureToGraph(c->stream, body, nullptr, nullptr, 0, mode));
  const long long l0 = c->launches;
  int r = case_subiter(c);
  if (!r) {
    k_conv_check<<<1, 32, 0, c->stream>>>(c->er, c->active, c->iters, c->ncase, tol,
                                          max_subiters, c->cont, h, 1);
    le = cudaGetLastError();
  }
  c->cgraph_body = c->launches - l0 + 1;  // + the check
  cudaError_t ce = cudaStreamEndCapture(c->stream, &body);
  if (r) return r;
  CK(le);
  CK(ce);
  CK(cudaStreamBeginCaptureToGraph(c->stream, g, &wnode, nullptr, 1, mode));
  const long long l1 = c->launches;
  r = case_shift(c);
  c->cgraph_outer = c->launches - l1 + pre_nodes;  // + the reset and the step's mirror
  ce = cudaStreamEndCapture(c->stream, &g);
  if (r) return r;
  CK(ce);
  // per-node priorities: the IBM ghost levels beside the boundary fill
  CK(cudaGraphInstantiate(&c->cgraph, g, cudaGraphInstantiateFlagUseNodePriority));
  c->cgraph_max = max_subiters;
  c->cgraph_tol = tol;
  c->cgraph_method = c->method;
  return BCMG_OK;
}

}  // namespace

extern "C" {

// Sets (msg != NULL) or clears (msg == NULL) the calling thread's last error;
// used by entry points defined in other translation units.
void bcmg_internal_set_error(const char *msg) {
  if (msg)
    set_err(msg);
  else
    clear_err();
}

const char *bcmg_last_error(void) { return g_has_err ? g_err.c_str() : nullptr; }
const char *bcmg_version(void) { return "bcm_gb300 0.1 (sm_103a)"; }

}  // extern "C"

namespace {

// Per-case tables of a batch, formed by bcmg_batch_create.
struct BatchInit {
  std::vector<CaseConst> cases;
  std::vector<int> case_cube0;  // [ncase+1]
};

CaseConst case_const(const bcmg_case_desc &d) {
  CaseConst q{};
  q.mu_L = d.mu_L;
  q.rho0 = d.rho0;
  q.U0 = d.U0;
  q.Uin = d.Uin;
  q.P0 = d.P0;
  q.E0 = d.P0 / (BCMG_K - 1);
  q.dT = d.deltaT;
  q.dTau = d.deltaTau;
  q.e = d.e;
  q.mpi_ncube = d.mpi_ncube;
  q.ef = (float)d.e;
  q.rho0f = (float)d.rho0;
  q.P0f = (float)d.P0;
  q.RT0f = (float)(d.P0 / d.rho0);
  q.T0f = (float)(d.P0 / d.rho0 / BCMG_R);
  q.mu_Lf = (float)d.mu_L;
  q.i2dtf = (float)(1.0 / (2.0 * d.deltaT));
  q.dTf = (float)d.deltaT;
  q.dTauf = (float)d.deltaTau;
  return q;
}

int create_common(const bcmg_case_desc *d, const BatchInit *bi, bcmg_case **out,
                  int nproxy = 0);

}  // namespace

extern "C" int bcmg_case_create(const bcmg_case_desc *d, bcmg_case **out) {
  TraceRange trace("bcmg_case_create");
  return create_common(d, nullptr, out);
}

extern "C" int bcmg_case_create_shard(const bcmg_case_desc *d, int nproxy, bcmg_case **out) {
  TraceRange trace("bcmg_case_create_shard");
  return create_common(d, nullptr, out, nproxy);
}

extern "C" int bcmg_case_set_exchange(bcmg_case *c, bcmg_exchange_fn fn, void *user) {
  clear_err();
  if (!c) { set_err("null context"); return BCMG_ERR_ARG; }
  if (c->batched && fn) { set_err("batches are not sharded"); return BCMG_ERR_UNSUPPORTED; }
  c->xchg = fn;
  c->xchg_user = user;
  if (c->graph) cudaGraphExecDestroy(c->graph);  // captured steps lack the hook
  c->graph = nullptr;
  c->graph_subiters = -1;
  if (c->cgraph) cudaGraphExecDestroy(c->cgraph);
  c->cgraph = nullptr;
  return BCMG_OK;
}

extern "C" int bcmg_case_set_halo(bcmg_case *c, int npeer, const int *nsend,
                                  const int *const *send, const int *nrecv,
                                  const int *const *recv) {
  clear_err();
  if (!c || npeer < 0 || (npeer > 0 && (!nsend || !send || !nrecv || !recv))) {
    set_err("bad arguments");
    return BCMG_ERR_ARG;
  }
  const int n = c->ph.n;
  // Every band names an own cube (send) or a proxy (recv), an axis, a side
  // and 1..n layers: the kernels then stay inside the case's arrays.
  auto valid = [&](int cnt, const int *b, bool own) {
    if (cnt < 0 || (cnt > 0 && !b)) return false;
    for (int i = 0; i < cnt; ++i) {
      const int cube = b[4 * i], ax = b[4 * i + 1], side = b[4 * i + 2], L = b[4 * i + 3];
      const bool cube_ok = own ? (cube >= 1 && cube <= c->nreal)
                               : (cube > c->nreal && cube < c->ncube);
      if (!cube_ok || ax < 0 || ax > 2 || side < 0 || side > 1 || L < 1 || L > n) return false;
    }
    return true;
  };
  for (int p = 0; p < npeer; ++p)
    if (!valid(nsend[p], send[p], true) || !valid(nrecv[p], recv[p], false)) {
      set_err("halo band outside the context (send: own cubes, recv: proxy slots)");
      return BCMG_ERR_ARG;
    }
  for (auto &h : c->halo) {
    dfree(h.send); dfree(h.recv); dfree(h.soff); dfree(h.roff);
  }
  c->halo.assign((size_t)npeer, bcmg_case::Halo());
  auto upload = [&](int cnt, const int *b, int **tab, long long **off, long long &cells) {
    std::vector<long long> o((size_t)cnt);
    cells = 0;
    for (int i = 0; i < cnt; ++i) {
      o[i] = cells;
      cells += (long long)b[4 * i + 3] * n * n;
    }
    if (cnt == 0) return BCMG_OK;
    CK(dalloc(tab, 4 * (size_t)cnt));
    CK(dalloc(off, (size_t)cnt));
    CK(cudaMemcpy(*tab, b, sizeof(int) * 4 * cnt, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(*off, o.data(), sizeof(long long) * cnt, cudaMemcpyHostToDevice));
    return BCMG_OK;
  };
  for (int p = 0; p < npeer; ++p) {
    bcmg_case::Halo &h = c->halo[p];
    h.nsend = nsend[p];
    h.nrecv = nrecv[p];
    int r = upload(h.nsend, send[p], &h.send, &h.soff, h.send_cells);
    if (!r) r = upload(h.nrecv, recv[p], &h.recv, &h.roff, h.recv_cells);
    if (r) return r;
  }
  return BCMG_OK;
}

extern "C" int bcmg_case_halo_bytes(const bcmg_case *c, int peer, size_t *send_bytes,
                                    size_t *recv_bytes) {
  if (!c || peer < 0 || peer >= (int)c->halo.size()) return BCMG_ERR_ARG;
  const size_t per = 5 * sizeof(double) + (c->M ? 5 * sizeof(float) : 0);
  if (send_bytes) *send_bytes = per * (size_t)c->halo[peer].send_cells;
  if (recv_bytes) *recv_bytes = per * (size_t)c->halo[peer].recv_cells;
  return BCMG_OK;
}

static int halo_move(bcmg_case *c, int peer, void *buf, int unpack) {
  clear_err();
  if (!c || peer < 0 || peer >= (int)c->halo.size() || !buf) {
    set_err("bad context, peer or buffer");
    return BCMG_ERR_ARG;
  }
  const bcmg_case::Halo &h = c->halo[peer];
  if (unpack)
    CK(launch_halo(c->U1_, c->mir(), h.recv, h.roff, h.nrecv, h.recv_cells, c->ph.n, buf, 1,
                   c->stream));
  else
    CK(launch_halo(c->U1_, c->mir(), h.send, h.soff, h.nsend, h.send_cells, c->ph.n, buf, 0,
                   c->stream));
  return BCMG_OK;
}

extern "C" int bcmg_case_halo_pack(bcmg_case *c, int peer, void *dev_buf) {
  return halo_move(c, peer, dev_buf, 0);
}

extern "C" int bcmg_case_halo_unpack(bcmg_case *c, int peer, const void *dev_buf) {
  return halo_move(c, peer, const_cast<void *>(dev_buf), 1);
}

extern "C" int bcmg_case_norm_sums(bcmg_case *c, double **dev_sums) {
  if (!c || !dev_sums) return BCMG_ERR_ARG;
  *dev_sums = c->nsum;
  return BCMG_OK;
}

extern "C" int bcmg_case_norm_sums_host(bcmg_case *c, double *sums, int write) {
  clear_err();
  if (!c || !sums) { set_err("null argument"); return BCMG_ERR_ARG; }
  if (write)
    CK(cudaMemcpyAsync(c->nsum, sums, 7 * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  else
    CK(cudaMemcpyAsync(sums, c->nsum, 7 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return BCMG_OK;
}

namespace {

int create_common(const bcmg_case_desc *d, const BatchInit *bi, bcmg_case **out,
                  int nproxy) {
  clear_err();
  if (!d || !out) {
    set_err("null argument");
    return BCMG_ERR_ARG;
  }
  if (nproxy < 0 || nproxy > d->ncube - 2 || (nproxy > 0 && bi)) {
    set_err("nproxy must leave at least one own cube (and batches are not sharded)");
    return BCMG_ERR_ARG;
  }
  *out = nullptr;
  if (!valid_n(d->n)) {
    set_err("n must be a multiple of 4 in [4, 256]");
    return BCMG_ERR_ARG;
  }
  if (d->ncube < 2 || !d->cube_size || !d->csl || !d->adj_number || !d->FWS) {
    set_err("ncube < 2 or missing geometry arrays");
    return BCMG_ERR_ARG;
  }
  if (d->precision != BCMG_PRECISION_FP64 && d->precision != BCMG_PRECISION_SPLIT) {
    set_err("unknown precision");
    return BCMG_ERR_ARG;
  }
  for (int i = 1; i < d->ncube; ++i)
    if (!(d->cube_size[i] > 0)) {
      set_err("cube_size must be positive for cubes 1..ncube-1");
      return BCMG_ERR_ARG;
    }
  bcmg_case *c = new bcmg_case();
  auto fail = [&](int code) {
    c->release();
    delete c;
    return code;
  };
  c->ph.n = d->n;
  c->ph.mpi_ncube = d->mpi_ncube;
  c->ph.mu_L = d->mu_L;
  c->ph.rho0 = d->rho0;
  c->ph.U0 = d->U0;
  c->ph.Uin = d->Uin;
  c->ph.P0 = d->P0;
  c->ncube = d->ncube;
  c->nreal = d->ncube - 1 - nproxy;
  c->S = d->n + 4;
  c->dT = d->deltaT;
  c->dTau = d->deltaTau;
  c->e = d->e;
  c->precision = d->precision;
  c->ncell = (size_t)d->ncube * c->S * c->S * c->S;
  cudaGetDevice(&c->device);
  if (bi) {
    c->batched = true;
    c->ncase = (int)bi->cases.size();
    c->hcases = bi->cases;
    c->case_cube0 = bi->case_cube0;
  }
  std::vector<int> off;
  std::vector<FaceTask> tasks;
  std::string err;
  if (!build_interface_tasks(d->ncube, d->adj_number, d->csl, off, tasks, err)) {
    set_err(err);
    return fail(BCMG_ERR_ARG);
  }
  std::vector<int> task_cube(tasks.size());
  for (int cc = 1; cc < d->ncube; ++cc)
    for (int t = off[cc]; t < off[cc + 1]; ++t) task_cube[t] = cc;
  if (nproxy > 0) {  // proxies are read, never written
    std::vector<FaceTask> kt;
    std::vector<int> kc;
    for (size_t t = 0; t < tasks.size(); ++t)
      if (task_cube[t] <= c->nreal) {
        kt.push_back(tasks[t]);
        kc.push_back(task_cube[t]);
      }
    tasks.swap(kt);
    task_cube.swap(kc);
  }
  c->ntasks = (int)tasks.size();
  const int *lists[6] = {d->xl, d->xu, d->yl, d->yu, d->zl, d->zu};
  const int counts[6] = {d->nxl, d->nxu, d->nyl, d->nyu, d->nzl, d->nzu};
  for (int l = 0; l < 6; ++l)
    if (counts[l] > 0 && !lists[l]) {
      set_err("boundary list pointer missing");
      return fail(BCMG_ERR_ARG);
    }
  std::vector<int> bcc, bcm;
  if (!build_bc_entries(d->ncube, lists, counts, bcc, bcm, err)) {
    set_err(err);
    return fail(BCMG_ERR_ARG);
  }
  auto ck = [&](cudaError_t e, const char *what) {
    if (e != cudaSuccess) set_err(std::string(what) + ": " + cudaGetErrorString(e));
    return e == cudaSuccess;
  };
  if (!ck(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "stream"))
    return fail(BCMG_ERR_CUDA);
  const size_t nd = c->ncell * 5;
  bool ok = ck(dalloc(&c->U1_, nd), "alloc") && ck(dalloc(&c->U1, nd), "alloc") &&
            ck(dalloc(&c->U1q, nd), "alloc") && ck(dalloc(&c->U1p1, nd), "alloc") &&
            ck(dalloc(&c->U1p2, nd), "alloc") && ck(dalloc(&c->Rku1, nd), "alloc") &&
            ck(dalloc(&c->Residual1, nd), "alloc") && ck(dalloc(&c->FWS, c->ncell), "alloc") &&
            ck(dalloc(&c->cube_size, (size_t)d->ncube), "alloc") &&
            ck(dalloc(&c->task_cube, tasks.size()), "alloc") &&
            ck(dalloc(&c->tasks, tasks.size()), "alloc") &&
            ck(dalloc(&c->bc_cubes, bcc.size()), "alloc") &&
            ck(dalloc(&c->bc_masks, bcm.size()), "alloc") &&
            ck(dalloc(&c->er, 8 * (size_t)c->ncase), "alloc") &&
            ck(dalloc(&c->nsum, 7), "alloc") &&
            ck(dalloc(&c->emax, 6 * (size_t)c->ncase), "alloc");
  if (!ok) return fail(BCMG_ERR_CUDA);
  if (d->precision == BCMG_PRECISION_SPLIT &&
      !(ck(dalloc(&c->M, nd), "alloc") && ck(dalloc(&c->M2, nd), "alloc") &&
        ck(dalloc(&c->mpar, 1), "alloc") && ck(cudaMemset(c->mpar, 0, sizeof(int)), "memset") &&
        ck(dalloc(&c->D2, nd), "alloc") && ck(cudaMemset(c->D2, 0, nd * sizeof(float)), "memset") &&
        ck(dalloc(&c->inv_dx, (size_t)d->ncube), "alloc") &&
        ck(cudaMemset(c->M, 0, nd * sizeof(float)), "memset") &&
        ck(cudaMemset(c->M2, 0, nd * sizeof(float)), "memset") &&
        true))
    return fail(BCMG_ERR_CUDA);
  if (c->inv_dx) {
    std::vector<float> inv((size_t)d->ncube, 0.f);
    for (int i = 1; i < d->ncube; ++i) inv[i] = (float)(d->n / d->cube_size[i]);
    if (!ck(cudaMemcpy(c->inv_dx, inv.data(), sizeof(float) * inv.size(), cudaMemcpyHostToDevice),
            "copy"))
      return fail(BCMG_ERR_CUDA);
  }
  RkArgs probe{};
  probe.ph = c->ph;
  probe.ncube = c->ncube;
  c->nparts = rk_partial_blocks(probe);
  if (d->precision == BCMG_PRECISION_SPLIT)  // room for either tile edge
    c->nparts = std::max(c->nparts, flux_split_blocks(d->n, d->ncube - 1, 4));
  c->nparts = std::max(c->nparts, d->ncube - 1);  // LU-SGS: one block per cube
  if (c->batched) {
    // Stage-update blocks of about equal size that never straddle two cases
    // (per-case norms), the flux kernel's per-case block ranges (one block
    // per tile, cubes in order), and the cube -> case map.
    const long long n3 = (long long)d->n * d->n * d->n;
    const long long total = (long long)(d->ncube - 1) * n3;
    long long nbt = std::min<long long>(std::max<long long>((total + 1023) / 1024, 1), 152 * 16);
    const long long chunk = (total + nbt - 1) / nbt;
    const int tiles = flux_split_blocks(d->n, 1);
    std::vector<long long> blk;
    std::vector<int> cbr(c->ncase + 1), cbf(c->ncase + 1), cbc(c->ncase + 1),
        cube_case(d->ncube, 0);
    for (int q = 0; q <= c->ncase; ++q) cbc[q] = c->case_cube0[q] - 1;
    for (int q = 0; q < c->ncase; ++q) {
      cbr[q] = (int)blk.size();
      cbf[q] = (c->case_cube0[q] - 1) * tiles;
      const long long b0 = (c->case_cube0[q] - 1) * n3, b1 = (c->case_cube0[q + 1] - 1) * n3;
      for (long long x = b0; x < b1; x += chunk) blk.push_back(x);
      for (int g = c->case_cube0[q]; g < c->case_cube0[q + 1]; ++g) cube_case[g] = q;
    }
    cbr[c->ncase] = (int)blk.size();
    cbf[c->ncase] = (d->ncube - 1) * tiles;
    blk.push_back(total);
    c->nrk = (int)blk.size() - 1;
    if (d->precision == BCMG_PRECISION_FP64) c->nparts = std::max(c->nparts, c->nrk);
    ok = ck(dalloc(&c->cases, (size_t)c->ncase), "alloc") &&
         ck(dalloc(&c->cube_case, (size_t)d->ncube), "alloc") &&
         ck(dalloc(&c->rk_blk, blk.size()), "alloc") &&
         ck(dalloc(&c->case_blk_rk, cbr.size()), "alloc") &&
         ck(dalloc(&c->case_blk_flux, cbf.size()), "alloc") &&
         ck(dalloc(&c->case_blk_cube, cbc.size()), "alloc") &&
         ck(cudaMemcpy(c->case_blk_cube, cbc.data(), sizeof(int) * cbc.size(),
                       cudaMemcpyHostToDevice), "copy") &&
         ck(cudaMemcpy(c->cases, c->hcases.data(), sizeof(CaseConst) * c->ncase,
                       cudaMemcpyHostToDevice), "copy") &&
         ck(cudaMemcpy(c->cube_case, cube_case.data(), sizeof(int) * cube_case.size(),
                       cudaMemcpyHostToDevice), "copy") &&
         ck(cudaMemcpy(c->rk_blk, blk.data(), sizeof(long long) * blk.size(),
                       cudaMemcpyHostToDevice), "copy") &&
         ck(cudaMemcpy(c->case_blk_rk, cbr.data(), sizeof(int) * cbr.size(),
                       cudaMemcpyHostToDevice), "copy") &&
         ck(cudaMemcpy(c->case_blk_flux, cbf.data(), sizeof(int) * cbf.size(),
                       cudaMemcpyHostToDevice), "copy");
    if (!ok) return fail(BCMG_ERR_CUDA);
  }
  if (!ck(dalloc(&c->partials, (size_t)c->nparts * 7), "alloc")) return fail(BCMG_ERR_CUDA);
  cudaStream_t s = c->stream;
  ok = ck(cudaMemsetAsync(c->U1_, 0, nd * 8, s), "memset") &&
       ck(cudaMemsetAsync(c->U1, 0, nd * 8, s), "memset") &&
       ck(cudaMemsetAsync(c->U1q, 0, nd * 8, s), "memset") &&
       ck(cudaMemsetAsync(c->U1p1, 0, nd * 8, s), "memset") &&
       ck(cudaMemsetAsync(c->U1p2, 0, nd * 8, s), "memset") &&
       ck(cudaMemsetAsync(c->Rku1, 0, nd * 8, s), "memset") &&
       ck(cudaMemsetAsync(c->Residual1, 0, nd * 8, s), "memset") &&
       ck(cudaMemsetAsync(c->er, 0, 8 * 8 * (size_t)c->ncase, s), "memset") &&
       ck(cudaMemsetAsync(c->emax, 0, 6 * 8 * (size_t)c->ncase, s), "memset") &&
       ck(cudaMemcpyAsync(c->FWS, d->FWS, c->ncell * sizeof(int), cudaMemcpyHostToDevice, s),
          "copy") &&
       ck(cudaMemcpyAsync(c->cube_size, d->cube_size, sizeof(double) * d->ncube,
                          cudaMemcpyHostToDevice, s), "copy") &&
       (tasks.empty() || ck(cudaMemcpyAsync(c->task_cube, task_cube.data(),
                                            sizeof(int) * task_cube.size(),
                                            cudaMemcpyHostToDevice, s), "copy")) &&
       (tasks.empty() || ck(cudaMemcpyAsync(c->tasks, tasks.data(), sizeof(FaceTask) * tasks.size(),
                                            cudaMemcpyHostToDevice, s), "copy")) &&
       (bcc.empty() || (ck(cudaMemcpyAsync(c->bc_cubes, bcc.data(), sizeof(int) * bcc.size(),
                                           cudaMemcpyHostToDevice, s), "copy") &&
                        ck(cudaMemcpyAsync(c->bc_masks, bcm.data(), sizeof(int) * bcm.size(),
                                           cudaMemcpyHostToDevice, s), "copy"))) &&
       ck(cudaStreamSynchronize(s), "sync");
  if (!ok) return fail(BCMG_ERR_CUDA);
  c->nbc = (int)bcc.size();
  // Combined IBM table: minus entries 1..nm then plus entries nm+1..nm+np
  // (main.cpp:1168-1174 applies minus before plus).
  const int nm = std::max(0, d->nminus), np = std::max(0, d->nplus);
  if (nm + np > 0) {
    if ((nm && (!d->w_minus || !d->gc_minus || !d->ip_minus)) ||
        (np && (!d->w_plus || !d->gc_plus || !d->ip_plus))) {
      set_err("IBM table pointer missing");
      return fail(BCMG_ERR_ARG);
    }
    std::vector<double> w(8 * (size_t)(nm + np) + 1, 0.0);
    std::vector<int> gc(4 * (size_t)(nm + np) + 1, 0), ip(4 * (size_t)(nm + np) + 1, 0);
    if (nm) {
      std::copy(d->w_minus + 1, d->w_minus + 1 + 8 * (size_t)nm, w.begin() + 1);
      std::copy(d->gc_minus + 1, d->gc_minus + 1 + 4 * (size_t)nm, gc.begin() + 1);
      std::copy(d->ip_minus + 1, d->ip_minus + 1 + 4 * (size_t)nm, ip.begin() + 1);
    }
    if (np) {
      std::copy(d->w_plus + 1, d->w_plus + 1 + 8 * (size_t)np, w.begin() + 1 + 8 * (size_t)nm);
      std::copy(d->gc_plus + 1, d->gc_plus + 1 + 4 * (size_t)np, gc.begin() + 1 + 4 * (size_t)nm);
      std::copy(d->ip_plus + 1, d->ip_plus + 1 + 4 * (size_t)np, ip.begin() + 1 + 4 * (size_t)nm);
    }
    // Cases in which no IBM entry's cell (ghost cell or stencil) lies where
    // the boundary fill reads or writes: the three layers at each boundary
    // face of its cube (ghost layers written, the next interior layer read,
    // and the y and z faces over whole planes).  Their entries form the side
    // table, filled beside the boundary fill; the other cases' entries stay
    // in the reference's order after it.  Cases never share cubes, so
    // splitting the table by case keeps every dependency inside one table.
    const int ne = nm + np;
    auto case_of = [&](int cube) -> int {
      if (!bi) return 0;
      const auto &b0 = bi->case_cube0;
      return (int)(std::upper_bound(b0.begin(), b0.end(), cube) - b0.begin()) - 1;
    };
    const int ncs = bi ? (int)bi->cases.size() : 1;
    std::vector<int> c0 = bi ? bi->case_cube0 : std::vector<int>{1, d->ncube};
    std::vector<char> shared;
    ghost_shared_cases(d->n, d->ncube, bcc, bcm, gc.data(), ip.data(), ne, c0, shared);
    std::vector<char> to_side((size_t)ne, 0);
    int nside = 0;
    if (!bcc.empty())
      for (int e = 0; e < ne; ++e) {
        const int q = case_of(gc[4 * (size_t)e + 1]);
        if (q >= 0 && q < ncs && !shared[q]) {
          to_side[e] = 1;
          ++nside;
        }
      }
    auto upload = [&](Ibm &t, char which) -> int {
      std::vector<double> ws(1, 0.0);
      std::vector<int> gs(1, 0), is(1, 0);
      int cnt = 0;
      for (int e = 0; e < ne; ++e) {
        if (to_side[e] != which) continue;
        ws.insert(ws.end(), w.begin() + 1 + 8 * (size_t)e, w.begin() + 9 + 8 * (size_t)e);
        gs.insert(gs.end(), gc.begin() + 1 + 4 * (size_t)e, gc.begin() + 5 + 4 * (size_t)e);
        is.insert(is.end(), ip.begin() + 1 + 4 * (size_t)e, ip.begin() + 5 + 4 * (size_t)e);
        ++cnt;
      }
      return cnt ? ibm_upload(t, cnt, ws.data(), gs.data(), is.data(), d->n, d->ncube, s)
                 : BCMG_OK;
    };
    int r = nside == 0 ? ibm_upload(c->ibm, ne, w.data(), gc.data(), ip.data(), d->n, d->ncube, s)
                       : upload(c->ibm, 0);
    if (!r && nside > 0) r = upload(c->ibm_side, 1);
    if (r) return fail(r);
    if (nside > 0) {
      int least = 0, greatest = 0;
      if (!ck(cudaDeviceGetStreamPriorityRange(&least, &greatest), "priority range"))
        return fail(BCMG_ERR_CUDA);
      c->side_priority = greatest;
      if (!ck(cudaStreamCreateWithPriority(&c->side, cudaStreamNonBlocking, greatest), "stream") ||
          !ck(cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming), "event") ||
          !ck(cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming), "event"))
        return fail(BCMG_ERR_CUDA);
      c->ghost_beside_bc = true;
    }
  }
  // Reduced face-task list of the prologue interface calls.
  {
    std::vector<char> keep;
    prologue_task_mask(d->n, d->ncube, tasks, task_cube, bcc, bcm, d->gc_minus, nm, d->gc_plus,
                       np, keep);
    // a proxy's bands are refilled by the exchange before every call
    for (size_t t = 0; t < tasks.size(); ++t)
      if (tasks[t].src > c->nreal) keep[t] = 1;
    std::vector<FaceTask> tp;
    std::vector<int> cp;
    for (size_t t = 0; t < tasks.size(); ++t)
      if (keep[t]) {
        tp.push_back(tasks[t]);
        cp.push_back(task_cube[t]);
      }
    c->ntasks_p = (int)tp.size();
    if (!tp.empty() &&
        !(ck(dalloc(&c->tasks_p, tp.size()), "alloc") &&
          ck(dalloc(&c->task_cube_p, cp.size()), "alloc") &&
          ck(cudaMemcpy(c->tasks_p, tp.data(), sizeof(FaceTask) * tp.size(),
                        cudaMemcpyHostToDevice), "copy") &&
          ck(cudaMemcpy(c->task_cube_p, cp.data(), sizeof(int) * cp.size(),
                        cudaMemcpyHostToDevice), "copy")))
      return fail(BCMG_ERR_CUDA);
  }
  // Push table of the split-precision flux kernel and the closing list that
  // goes with it (level-jump tasks only).
  if (d->precision == BCMG_PRECISION_SPLIT) {
    std::vector<int> push;
    const bool ok_push = build_push_table(d->ncube, tasks, task_cube, push);
    std::vector<FaceTask> tq;
    std::vector<int> cq;
    for (size_t t = 0; t < tasks.size(); ++t)
      if (tasks[t].kind != 0 || tasks[t].src > c->nreal) {  // proxies push nothing
        tq.push_back(tasks[t]);
        cq.push_back(task_cube[t]);
      }
    if (ok_push) {
      c->ntasks_q = (int)tq.size();
      if (!(ck(dalloc(&c->push, push.size()), "alloc") &&
            ck(cudaMemcpy(c->push, push.data(), sizeof(int) * push.size(),
                          cudaMemcpyHostToDevice), "copy")))
        return fail(BCMG_ERR_CUDA);
      if (!tq.empty() &&
          !(ck(dalloc(&c->tasks_q, tq.size()), "alloc") &&
            ck(dalloc(&c->task_cube_q, cq.size()), "alloc") &&
            ck(cudaMemcpy(c->tasks_q, tq.data(), sizeof(FaceTask) * tq.size(),
                          cudaMemcpyHostToDevice), "copy") &&
            ck(cudaMemcpy(c->task_cube_q, cq.data(), sizeof(int) * cq.size(),
                          cudaMemcpyHostToDevice), "copy")))
        return fail(BCMG_ERR_CUDA);
      // the closing call of RK stages 1 and 2 (not for sharded contexts,
      // whose proxies are refilled by each call's exchange)
      if (c->nreal == d->ncube - 1) {
        std::vector<char> keep_r, edge;
        closing_plan(d->n, d->ncube, tasks, task_cube, bcc, bcm, d->ip_minus, nm, d->ip_plus,
                     np, keep_r, edge);
        std::vector<FaceTask> tr;
        std::vector<int> cr, er_;
        for (size_t t = 0; t < tasks.size(); ++t)
          if (keep_r[t]) {
            tr.push_back(tasks[t]);
            cr.push_back(task_cube[t]);
          }
        for (int cb = 1; cb < d->ncube; ++cb)
          if (edge[cb]) er_.push_back(cb);
        c->ntasks_r = (int)tr.size();
        c->nedge_r = (int)er_.size();
        if ((!tr.empty() &&
             !(ck(dalloc(&c->tasks_r, tr.size()), "alloc") &&
               ck(dalloc(&c->task_cube_r, cr.size()), "alloc") &&
               ck(cudaMemcpy(c->tasks_r, tr.data(), sizeof(FaceTask) * tr.size(),
                             cudaMemcpyHostToDevice), "copy") &&
               ck(cudaMemcpy(c->task_cube_r, cr.data(), sizeof(int) * cr.size(),
                             cudaMemcpyHostToDevice), "copy"))) ||
            (!er_.empty() &&
             !(ck(dalloc(&c->edge_r, er_.size()), "alloc") &&
               ck(cudaMemcpy(c->edge_r, er_.data(), sizeof(int) * er_.size(),
                             cudaMemcpyHostToDevice), "copy"))))
          return fail(BCMG_ERR_CUDA);
        c->closing_reduced = true;
      }
    }
  }
  *out = c;
  return BCMG_OK;
}

}  // namespace

extern "C" {

void bcmg_case_destroy(bcmg_case *c) {
  if (!c) return;
  if (c->stream) cudaStreamSynchronize(c->stream);
  c->release();
  delete c;
}

int bcmg_case_set_state(bcmg_case *c, const double *U1_, const double *U1, const double *U1q) {
  TraceRange trace("bcmg_case_set_state");
  clear_err();
  if (!c) { set_err("null context"); return BCMG_ERR_ARG; }
  const size_t b = c->ncell * 5 * sizeof(double);
  if (U1_) CK(cudaMemcpyAsync(c->U1_, U1_, b, cudaMemcpyHostToDevice, c->stream));
  if (U1) CK(cudaMemcpyAsync(c->U1, U1, b, cudaMemcpyHostToDevice, c->stream));
  if (U1q) CK(cudaMemcpyAsync(c->U1q, U1q, b, cudaMemcpyHostToDevice, c->stream));
  if (c->precision == BCMG_PRECISION_SPLIT && (U1 || U1q))
    CK(launch_level_diff(c->U1, c->U1q, c->D2, c->ph.n, c->ncube, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return BCMG_OK;
}

int bcmg_case_get_state(bcmg_case *c, double *U1_, double *U1, double *U1q) {
  TraceRange trace("bcmg_case_get_state");
  clear_err();
  if (!c) { set_err("null context"); return BCMG_ERR_ARG; }
  const size_t b = c->ncell * 5 * sizeof(double);
  if (U1_) CK(cudaMemcpyAsync(U1_, c->U1_, b, cudaMemcpyDeviceToHost, c->stream));
  if (U1) CK(cudaMemcpyAsync(U1, c->U1, b, cudaMemcpyDeviceToHost, c->stream));
  if (U1q) CK(cudaMemcpyAsync(U1q, c->U1q, b, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return BCMG_OK;
}

int bcmg_case_get_scratch(bcmg_case *c, double *U1p1, double *U1p2, double *Rku1,
                          double *Residual1) {
  clear_err();
  if (!c) { set_err("null context"); return BCMG_ERR_ARG; }
  const size_t b = c->ncell * 5 * sizeof(double);
  if (U1p1) CK(cudaMemcpyAsync(U1p1, c->U1p1, b, cudaMemcpyDeviceToHost, c->stream));
  if (U1p2) CK(cudaMemcpyAsync(U1p2, c->U1p2, b, cudaMemcpyDeviceToHost, c->stream));
  if (Rku1) CK(cudaMemcpyAsync(Rku1, c->Rku1, b, cudaMemcpyDeviceToHost, c->stream));
  if (Residual1)
    CK(cudaMemcpyAsync(Residual1, c->Residual1, b, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return BCMG_OK;
}

int bcmg_case_stage(bcmg_case *c, int RK) {
  TraceRange trace("bcmg_case_stage");
  clear_err();
  if (!c || RK < 1 || RK > 3) { set_err("bad context or RK"); return BCMG_ERR_ARG; }
  c->launches = 0;
  int r = case_mirror_all(c);
  if (!r) r = case_stage(c, RK);
  if (r) return r;
  CK(cudaStreamSynchronize(c->stream));
  return BCMG_OK;
}

int bcmg_case_advance(bcmg_case *c, int steps, int subiters, int use_graph, double *er,
                      double *emax) {
  TraceRange trace("bcmg_case_advance");
  clear_err();
  if (!c || steps < 0 || subiters < 1) { set_err("bad arguments"); return BCMG_ERR_ARG; }
  if (use_graph && c->xchg) {
    set_err("a context with an exchange hook steps without CUDA graphs (use_graph = 0)");
    return BCMG_ERR_UNSUPPORTED;
  }
  if (emax)
    CK(cudaMemcpyAsync(c->emax, emax, 6 * sizeof(double) * c->ncase, cudaMemcpyHostToDevice,
                       c->stream));
  c->launches = 0;
  c->ev_used = 0;
  if (use_graph && !c->profile) {
    if (!c->graph || c->graph_subiters != subiters) {
      if (c->graph) cudaGraphExecDestroy(c->graph);
      c->graph = nullptr;
      cudaGraph_t g;
      CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
      long long saved = c->launches;
      int r = case_step(c, subiters);
      c->graph_launches = c->launches - saved;
      cudaError_t ce = cudaStreamEndCapture(c->stream, &g);
      if (r) return r;
      if (ce != cudaSuccess) { set_err(cudaGetErrorString(ce)); return BCMG_ERR_CUDA; }
      // per-node priorities: the IBM ghost levels beside the boundary fill
      ce = cudaGraphInstantiate(&c->graph, g, cudaGraphInstantiateFlagUseNodePriority);
      cudaGraphDestroy(g);
      if (ce != cudaSuccess) { set_err(cudaGetErrorString(ce)); return BCMG_ERR_CUDA; }
      c->graph_subiters = subiters;
      c->launches = saved;
    }
    const long long per = c->graph_launches;  // kernel nodes of one step
    for (int s = 0; s < steps; ++s) CK(cudaGraphLaunch(c->graph, c->stream));
    c->launches = per * steps;
  } else {
    for (int s = 0; s < steps; ++s) {
      int r = case_step(c, subiters);
      if (r) return r;
    }
  }
  if (er)
    CK(cudaMemcpyAsync(er, c->er, 8 * sizeof(double) * c->ncase, cudaMemcpyDeviceToHost,
                       c->stream));
  if (emax)
    CK(cudaMemcpyAsync(emax, c->emax, 6 * sizeof(double) * c->ncase, cudaMemcpyDeviceToHost,
                       c->stream));
  CK(cudaStreamSynchronize(c->stream));
  if (c->profile) {
    for (size_t i = 0; i + 1 < c->ev_used; i += 2) {
      float ms = 0;
      CK(cudaEventElapsedTime(&ms, c->ev[i], c->ev[i + 1]));
      c->flux_ms += ms;
      ++c->flux_launches;
    }
  }
  return BCMG_OK;
}

int bcmg_case_advance_async(bcmg_case *c, int steps, int subiters) {
  TraceRange trace("bcmg_case_advance_async");
  clear_err();
  if (!c || steps < 0 || subiters < 1) { set_err("bad arguments"); return BCMG_ERR_ARG; }
  if (c->profile || c->xchg) {
    set_err("asynchronous steps need graphs: profiling and exchange hooks are synchronous");
    return BCMG_ERR_UNSUPPORTED;
  }
  if (!c->graph || c->graph_subiters != subiters) {
    // capture the step graph as bcmg_case_advance does (no step launched;
    // this first call waits for the capture)
    int r = bcmg_case_advance(c, 0, subiters, 1, nullptr, nullptr);
    if (r) return r;
  }
  for (int s = 0; s < steps; ++s) CK(cudaGraphLaunch(c->graph, c->stream));
  c->launches = c->graph_launches * steps;
  return BCMG_OK;
}

int bcmg_case_copy_state_async(bcmg_case *c, int to_device, double *U1_, double *U1,
                               double *U1q) {
  clear_err();
  if (!c) { set_err("null context"); return BCMG_ERR_ARG; }
  const size_t b = c->ncell * 5 * sizeof(double);
  const cudaMemcpyKind k = to_device ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost;
  double *dev[3] = {c->U1_, c->U1, c->U1q};
  double *host[3] = {U1_, U1, U1q};
  for (int i = 0; i < 3; ++i)
    if (host[i])
      CK(cudaMemcpyAsync(to_device ? dev[i] : host[i], to_device ? host[i] : dev[i], b, k,
                         c->stream));
  if (to_device && c->precision == BCMG_PRECISION_SPLIT && (U1 || U1q))
    CK(launch_level_diff(c->U1, c->U1q, c->D2, c->ph.n, c->ncube, c->stream));
  return BCMG_OK;
}

int bcmg_case_get_norms(bcmg_case *c, double *er, double *emax) {
  clear_err();
  if (!c) { set_err("null context"); return BCMG_ERR_ARG; }
  if (er)
    CK(cudaMemcpyAsync(er, c->er, 8 * sizeof(double) * c->ncase, cudaMemcpyDeviceToHost,
                       c->stream));
  if (emax)
    CK(cudaMemcpyAsync(emax, c->emax, 6 * sizeof(double) * c->ncase, cudaMemcpyDeviceToHost,
                       c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return BCMG_OK;
}

int bcmg_case_sync(bcmg_case *c) {
  clear_err();
  if (!c) { set_err("null context"); return BCMG_ERR_ARG; }
  CK(cudaStreamSynchronize(c->stream));
  return BCMG_OK;
}

int bcmg_case_device_state(bcmg_case *c, double **U1_, double **U1, double **U1q) {
  clear_err();
  if (!c) { set_err("null context"); return BCMG_ERR_ARG; }
  if (U1_) *U1_ = c->U1_;
  if (U1) *U1 = c->U1;
  if (U1q) *U1q = c->U1q;
  return BCMG_OK;
}

long long bcmg_case_launch_count(const bcmg_case *c) { return c ? c->launches : 0; }

int bcmg_case_time_flux(bcmg_case *c, int reps, double *ms) {
  clear_err();
  if (!c || reps < 1 || !ms) { set_err("bad arguments"); return BCMG_ERR_ARG; }
  cudaEvent_t a, b;
  CK(cudaEventCreate(&a));
  CK(cudaEventCreate(&b));
  bool prof = c->profile;
  c->profile = false;
  const size_t bytes = c->ncell * 5 * sizeof(double);
  // The split kernel applies its stage update in place: keep a copy of the
  // state in the (split-unused) U1p1 buffer and restore it afterwards.
  if (c->precision == BCMG_PRECISION_SPLIT)
    CK(cudaMemcpyAsync(c->U1p1, c->U1_, bytes, cudaMemcpyDeviceToDevice, c->stream));
  int r = case_mirror_all(c);
  if (!r) r = case_flux(c, 1);  // warm-up
  if (!r) {
    cudaEventRecord(a, c->stream);
    for (int i = 0; i < reps && !r; ++i) r = case_flux(c, 1);
    cudaEventRecord(b, c->stream);
  }
  if (c->precision == BCMG_PRECISION_SPLIT) {
    CK(cudaMemcpyAsync(c->U1_, c->U1p1, bytes, cudaMemcpyDeviceToDevice, c->stream));
    if (!r) r = case_mirror_all(c);
  }
  c->profile = prof;
  if (r) { cudaEventDestroy(a); cudaEventDestroy(b); return r; }
  CK(cudaEventSynchronize(b));
  float t = 0;
  CK(cudaEventElapsedTime(&t, a, b));
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  *ms = t / reps;
  return BCMG_OK;
}

// Per-launch timing of the flux kernel inside bcmg_case_advance (events on
// the context's stream around every flux launch; graphs are not used while
// profiling is on).  Totals accumulate until reset.
int bcmg_case_set_profiling(bcmg_case *c, int on) {
  clear_err();
  if (!c) { set_err("null context"); return BCMG_ERR_ARG; }
  c->profile = on != 0;
  c->flux_ms = 0;
  c->flux_launches = 0;
  return BCMG_OK;
}
int bcmg_case_profile(const bcmg_case *c, double *flux_ms_total, long long *flux_launches) {
  if (!c) return BCMG_ERR_ARG;
  if (flux_ms_total) *flux_ms_total = c->flux_ms;
  if (flux_launches) *flux_launches = c->flux_launches;
  return BCMG_OK;
}

// ---------------------------------------------------------------------------
// Batches: independent cases (same n and precision) laid end to end in one
// flat cube list.  Case q's cube l (1-based) becomes cube case_cube0[q]+l-1;
// its adjacency, boundary lists and IBM tables are renumbered the same way,
// so every table-driven kernel (interface, boundaries, ghost cells) runs over
// all cases at once and no task crosses from one case into another.  The
// constants each case takes from its own prm.h / time steps go to a device
// table indexed through a cube -> case map.
// ---------------------------------------------------------------------------
int bcmg_batch_create(int ncase, const bcmg_case_desc *descs, bcmg_case **out) {
  TraceRange trace("bcmg_batch_create");
  clear_err();
  if (!out || !descs || ncase < 1) {
    set_err("null argument or ncase < 1");
    return BCMG_ERR_ARG;
  }
  *out = nullptr;
  const int n = descs[0].n, prec = descs[0].precision;
  const int S = n + 4;
  const size_t S3 = (size_t)S * S * S;
  long long total = 1;
  for (int q = 0; q < ncase; ++q) {
    const bcmg_case_desc &d = descs[q];
    char msg[160];
    if (d.n != n || d.precision != prec) {
      std::snprintf(msg, sizeof msg, "case %d: every case of a batch needs the same n and precision", q);
      set_err(msg);
      return BCMG_ERR_ARG;
    }
    if (d.ncube < 2 || !d.cube_size || !d.csl || !d.adj_number || !d.FWS) {
      std::snprintf(msg, sizeof msg, "case %d: ncube < 2 or missing geometry arrays", q);
      set_err(msg);
      return BCMG_ERR_ARG;
    }
    if (!(d.deltaT > 0) || !(d.deltaTau > 0) || d.mpi_ncube < 1 || !(d.rho0 > 0)) {
      std::snprintf(msg, sizeof msg, "case %d: deltaT, deltaTau, rho0 must be positive and mpi_ncube >= 1", q);
      set_err(msg);
      return BCMG_ERR_ARG;
    }
    total += d.ncube - 1;
  }
  if (total > (1LL << 30)) {
    set_err("batch too large");
    return BCMG_ERR_ARG;
  }
  const int ncube = (int)total;
  std::vector<double> cube_size(ncube, 0.0);
  std::vector<int> csl(ncube, 0), adj((size_t)ncube * 35, 0);
  std::vector<int> fws;
  try {
    fws.assign((size_t)ncube * S3, 1);
  } catch (const std::bad_alloc &) {
    set_err("host memory for the batch's flag array");
    return BCMG_ERR_ARG;
  }
  std::vector<int> bc[6];
  std::vector<double> w(1, 0.0);
  std::vector<int> gc(1, 0), ip(1, 0);
  BatchInit bi;
  bi.case_cube0.push_back(1);
  double mu_any = 0.0;
  for (int q = 0; q < ncase; ++q) {
    const bcmg_case_desc &d = descs[q];
    const int g0 = bi.case_cube0.back();
    const int shift = g0 - 1;
    char msg[200];
    auto bad = [&](const char *what) {
      std::snprintf(msg, sizeof msg, "case %d: %s", q, what);
      set_err(msg);
      return BCMG_ERR_ARG;
    };
    for (int l = 1; l < d.ncube; ++l) {
      if (!(d.cube_size[l] > 0)) return bad("cube_size must be positive for cubes 1..ncube-1");
      cube_size[shift + l] = d.cube_size[l];
      csl[shift + l] = d.csl[l];
      for (int t = 0; t < 35; ++t) {
        const int v = d.adj_number[(size_t)l * 35 + t];
        if (v < 0 || v >= d.ncube) return bad("adj_number out of range");
        adj[(size_t)(shift + l) * 35 + t] = v > 0 ? v + shift : 0;
      }
    }
    std::copy(d.FWS + S3, d.FWS + (size_t)d.ncube * S3, fws.begin() + (size_t)g0 * S3);
    const int *lists[6] = {d.xl, d.xu, d.yl, d.yu, d.zl, d.zu};
    const int counts[6] = {d.nxl, d.nxu, d.nyl, d.nyu, d.nzl, d.nzu};
    for (int k = 0; k < 6; ++k) {
      if (counts[k] < 0 || (counts[k] > 0 && !lists[k])) return bad("boundary list missing");
      for (int m = 0; m < counts[k]; ++m) {
        const int v = lists[k][m];
        if (v < 1 || v >= d.ncube) return bad("boundary list entry out of range");
        bc[k].push_back(v + shift);
      }
    }
    // IBM entries: this case's minus list, then its plus list (main.cpp
    // applies minus before plus); cube numbers renumbered.
    for (int side = 0; side < 2; ++side) {
      const int cnt = side == 0 ? d.nminus : d.nplus;
      const double *W = side == 0 ? d.w_minus : d.w_plus;
      const int *G = side == 0 ? d.gc_minus : d.gc_plus;
      const int *I = side == 0 ? d.ip_minus : d.ip_plus;
      if (cnt <= 0) continue;
      if (!W || !G || !I) return bad("IBM table pointer missing");
      for (int e = 0; e < cnt; ++e) {
        for (int m = 0; m < 8; ++m) w.push_back(W[8 * (size_t)e + 1 + m]);
        for (int m = 0; m < 4; ++m) {
          int gv = G[4 * (size_t)e + 1 + m], iv = I[4 * (size_t)e + 1 + m];
          if (m == 0) {
            if (gv < 1 || gv >= d.ncube || iv < 1 || iv >= d.ncube)
              return bad("IBM cube number out of range");
            gv += shift;
            iv += shift;
          }
          gc.push_back(gv);
          ip.push_back(iv);
        }
      }
    }
    bi.cases.push_back(case_const(d));
    bi.case_cube0.push_back(g0 + d.ncube - 1);
    if (mu_any == 0.0 && d.mu_L != 0.0) mu_any = d.mu_L;
  }
  bcmg_case_desc m = descs[0];
  m.ncube = ncube;
  m.mu_L = mu_any;  // viscous kernels when any case is viscous
  m.cube_size = cube_size.data();
  m.csl = csl.data();
  m.adj_number = adj.data();
  m.FWS = fws.data();
  m.nxl = (int)bc[0].size(); m.nxu = (int)bc[1].size(); m.nyl = (int)bc[2].size();
  m.nyu = (int)bc[3].size(); m.nzl = (int)bc[4].size(); m.nzu = (int)bc[5].size();
  m.xl = bc[0].data(); m.xu = bc[1].data(); m.yl = bc[2].data();
  m.yu = bc[3].data(); m.zl = bc[4].data(); m.zu = bc[5].data();
  m.nminus = (int)((gc.size() - 1) / 4);
  m.w_minus = w.data();
  m.gc_minus = gc.data();
  m.ip_minus = ip.data();
  m.nplus = 0;
  m.w_plus = nullptr;
  m.gc_plus = m.ip_plus = nullptr;
  return create_common(&m, &bi, out);
}

int bcmg_case_set_method(bcmg_case *c, int method, double cfl, double omega) {
  clear_err();
  if (!c) { set_err("null context"); return BCMG_ERR_ARG; }
  if (method != BCMG_METHOD_RK3 && method != BCMG_METHOD_LUSGS) {
    set_err("unknown method");
    return BCMG_ERR_ARG;
  }
  if (method == BCMG_METHOD_LUSGS && !(cfl >= 0 && omega >= 1 && omega <= 4)) {
    set_err("LU-SGS needs cfl >= 0 (0: no pseudo-time term) and 1 <= omega <= 4");
    return BCMG_ERR_ARG;
  }
  if (method == BCMG_METHOD_LUSGS && c->ph.n * c->ph.n > 1024) {
    set_err("LU-SGS needs n <= 32 (one thread per cube column)");
    return BCMG_ERR_ARG;
  }
  if (method == BCMG_METHOD_LUSGS && c->precision == BCMG_PRECISION_SPLIT && !c->lu_scr)
    CK(dalloc(&c->lu_scr, lusgs_split_scratch(c->ph.n) * (size_t)(c->ncube - 1)));
  c->method = method;
  c->lu_cfl = cfl;
  c->lu_omega = omega;
  if (c->graph) cudaGraphExecDestroy(c->graph);  // the captured step changes
  c->graph = nullptr;
  c->graph_subiters = -1;
  return BCMG_OK;
}

int bcmg_case_advance_converged(bcmg_case *c, int steps, int max_subiters, double tol,
                                int use_graph, int *subiters_out, double *er, double *emax) {
  TraceRange trace("bcmg_case_advance_converged");
  clear_err();
  if (!c || steps < 0 || max_subiters < 1 || !(tol > 0)) {
    set_err("bad arguments");
    return BCMG_ERR_ARG;
  }
  if (use_graph && c->xchg) {
    set_err("a context with an exchange hook steps without CUDA graphs (use_graph = 0)");
    return BCMG_ERR_UNSUPPORTED;
  }
  if (!c->active) {
    CK(dalloc(&c->active, (size_t)c->ncase));
    CK(dalloc(&c->iters, (size_t)c->ncase));
    CK(dalloc(&c->cont, 1));
  }
  int *hist = nullptr;
  CK(dalloc(&hist, (size_t)std::max(1, steps) * c->ncase));
  struct Restore {
    bcmg_case *c;
    int *hist;
    ~Restore() {
      c->conv = false;
      if (hist) cudaFree(hist);
    }
  } restore{c, hist};
  if (emax)
    CK(cudaMemcpyAsync(c->emax, emax, 6 * sizeof(double) * c->ncase, cudaMemcpyHostToDevice,
                       c->stream));
  c->conv = true;
  c->launches = 0;
  c->ev_used = 0;
  int r;
  if (use_graph && !c->profile) {
    if (!c->cgraph || c->cgraph_max != max_subiters || c->cgraph_tol != tol ||
        c->cgraph_method != c->method) {
      long long saved = c->launches;
      if ((r = build_conv_graph(c, max_subiters, tol))) return r;
      c->launches = saved;
    }
    for (int st = 0; st < steps; ++st) {
      CK(cudaGraphLaunch(c->cgraph, c->stream));
      k_store_iters<<<1, 128, 0, c->stream>>>(c->iters, hist + (size_t)st * c->ncase, c->ncase);
      CK(cudaGetLastError());
    }
  } else {
    for (int st = 0; st < steps; ++st) {
      k_conv_reset<<<1, 128, 0, c->stream>>>(c->active, c->iters, c->ncase);
      CK(cudaGetLastError());
      for (int it = 0; it < max_subiters; ++it) {
        if ((r = case_subiter(c))) return r;
        k_conv_check<<<1, 32, 0, c->stream>>>(c->er, c->active, c->iters, c->ncase, tol,
                                              max_subiters, c->cont, 0, 0);
        CK(cudaGetLastError());
        int more = 0;
        CK(cudaMemcpyAsync(&more, c->cont, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        if (!more) break;
      }
      if ((r = case_shift(c))) return r;
      k_store_iters<<<1, 128, 0, c->stream>>>(c->iters, hist + (size_t)st * c->ncase, c->ncase);
      CK(cudaGetLastError());
    }
  }
  std::vector<int> h((size_t)std::max(1, steps) * c->ncase, 0);
  CK(cudaMemcpyAsync(h.data(), hist, sizeof(int) * h.size(), cudaMemcpyDeviceToHost, c->stream));
  if (er)
    CK(cudaMemcpyAsync(er, c->er, 8 * sizeof(double) * c->ncase, cudaMemcpyDeviceToHost,
                       c->stream));
  if (emax)
    CK(cudaMemcpyAsync(emax, c->emax, 6 * sizeof(double) * c->ncase, cudaMemcpyDeviceToHost,
                       c->stream));
  CK(cudaStreamSynchronize(c->stream));
  if (subiters_out) std::copy(h.begin(), h.begin() + (size_t)steps * c->ncase, subiters_out);
  if (use_graph && !c->profile) {
    // kernel launches of the replayed graphs: the while body once per
    // sub-iteration of the slowest case, plus reset and shift
    long long tot = 0;
    for (int st = 0; st < steps; ++st) {
      int mx = 0;
      for (int q = 0; q < c->ncase; ++q) mx = std::max(mx, h[(size_t)st * c->ncase + q]);
      tot += mx * c->cgraph_body + c->cgraph_outer;
    }
    c->launches = tot;
  }
  return BCMG_OK;
}

// ---------------------------------------------------------------------------
// PLOT3D output (BCM_Output.cpp:16-300).  The byte image is formed on the
// device on the context's stream (a snapshot: later solver work may proceed
// at once); a writer thread copies it to the host in pinned chunks on a side
// stream and writes the file, so the copy and the disk write overlap the
// solver.  Only one output is in flight: the next output call (or
// bcmg_case_output_wait / destroy) waits for it.
// ---------------------------------------------------------------------------
namespace {

constexpr size_t kOutChunk = (size_t)32 << 20;  // bytes per pinned chunk

int out_range(bcmg_case *c, int q, int *g0, int *ng) {
  if (q < 0) {
    *g0 = 1;
    *ng = c->ncube - 1;
    return BCMG_OK;
  }
  int nq = 0;
  int r = bcmg_case_case_cubes(c, q, g0, &nq);
  *ng = nq - 1;
  return r;
}

int out_prepare(bcmg_case *c, size_t ndoubles) {
  c->join_output();
  if (!c->out_stream) {
    CK(cudaStreamCreateWithFlags(&c->out_stream, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&c->out_ready, cudaEventDisableTiming));
    for (int i = 0; i < 2; ++i) {
      CK(cudaEventCreateWithFlags(&c->out_chunk[i], cudaEventDisableTiming));
      CK(cudaMallocHost((void **)&c->out_host[i], kOutChunk));
    }
  }
  if (ndoubles > c->out_cap) {
    if (c->out_dev) cudaFree(c->out_dev);
    c->out_dev = nullptr;
    c->out_cap = 0;
    CK(cudaMalloc((void **)&c->out_dev, ndoubles * sizeof(double)));
    c->out_cap = ndoubles;
  }
  return BCMG_OK;
}

// Writer thread body: header, then the device image in pinned chunks.
void out_write(bcmg_case *c, std::string path, std::vector<int> header, size_t bytes) {
  auto fail = [&](const std::string &m) {
    c->out_status = BCMG_ERR_CUDA;
    c->out_err = m;
  };
  cudaSetDevice(c->device);
  FILE *f = std::fopen(path.c_str(), "wb");
  if (!f) {
    c->out_status = BCMG_ERR_ARG;
    c->out_err = "cannot open " + path;
    return;
  }
  bool ok = std::fwrite(header.data(), sizeof(int), header.size(), f) == header.size();
  const char *src = reinterpret_cast<const char *>(c->out_dev);
  auto issue = [&](size_t off, int slot) {
    const size_t len = std::min(kOutChunk, bytes - off);
    cudaError_t e = cudaMemcpyAsync(c->out_host[slot], src + off, len, cudaMemcpyDeviceToHost,
                                    c->out_stream);
    if (e == cudaSuccess) e = cudaEventRecord(c->out_chunk[slot], c->out_stream);
    return e;
  };
  cudaError_t e = cudaSuccess;
  if (bytes > 0) e = issue(0, 0);
  int slot = 0;
  for (size_t off = 0; ok && e == cudaSuccess && off < bytes; off += kOutChunk, slot ^= 1) {
    if (off + kOutChunk < bytes) e = issue(off + kOutChunk, slot ^ 1);
    if (e != cudaSuccess) break;
    e = cudaEventSynchronize(c->out_chunk[slot]);
    if (e != cudaSuccess) break;
    const size_t len = std::min(kOutChunk, bytes - off);
    ok = std::fwrite(c->out_host[slot], 1, len, f) == len;
  }
  if (std::fclose(f) != 0) ok = false;
  if (e != cudaSuccess)
    fail(std::string("output copy: ") + cudaGetErrorString(e));
  else if (!ok)
    fail("write failed: " + path);
  else
    c->out_status = BCMG_OK;
}

int out_launch(bcmg_case *c, const char *path, int ncube_out, int ng, size_t ndoubles) {
  std::vector<int> header(1 + 3 * (size_t)ncube_out, c->ph.n + 2);
  header[0] = ncube_out;
  CK(cudaEventRecord(c->out_ready, c->stream));
  CK(cudaStreamWaitEvent(c->out_stream, c->out_ready, 0));
  c->out_status = BCMG_OK;
  c->out_err.clear();
  c->out_thread = std::thread(out_write, c, std::string(path), std::move(header),
                              ndoubles * sizeof(double));
  (void)ng;
  return BCMG_OK;
}

}  // namespace

int bcmg_case_output_q(bcmg_case *c, int q, int ncube_out, const char *path) {
  TraceRange trace("bcmg_case_output_q");
  clear_err();
  if (!c || !path) { set_err("null argument"); return BCMG_ERR_ARG; }
  int g0 = 0, ng = 0, r;
  if ((r = out_range(c, q, &g0, &ng))) return r;
  if (ncube_out <= 0) ncube_out = ng;
  const size_t m = c->ph.n + 2;
  const size_t nd = (4 + 5 * m * m * m) * (size_t)ng;
  if ((r = out_prepare(c, nd))) return r;
  CK(launch_plot3d_q(c->U1_, c->out_dev, c->ph.n, g0, ng, c->stream));
  return out_launch(c, path, ncube_out, ng, nd);
}

int bcmg_case_output_x(bcmg_case *c, int q, int ncube_out, const char *path,
                       const double *origin) {
  TraceRange trace("bcmg_case_output_x");
  clear_err();
  if (!c || !path || !origin) { set_err("null argument"); return BCMG_ERR_ARG; }
  int g0 = 0, ng = 0, r;
  if ((r = out_range(c, q, &g0, &ng))) return r;
  if (ncube_out <= 0) ncube_out = ng;
  const size_t m = c->ph.n + 2;
  const size_t nd = 3 * m * m * m * (size_t)ng;
  if ((r = out_prepare(c, nd))) return r;
  double *dorig = nullptr;
  CK(dalloc(&dorig, 3 * (size_t)std::max(ng, 1)));
  // origin rows of the written cubes: the case's own cubes 1.. (q >= 0) or
  // the flat list's cubes 1.. (q < 0)
  cudaError_t e = cudaMemcpyAsync(dorig, origin + 3, 3 * sizeof(double) * ng,
                                  cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess)
    e = launch_plot3d_x(c->cube_size, dorig, c->out_dev, c->ph.n, g0, ng, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  cudaFree(dorig);
  CK(e);
  if ((r = out_launch(c, path, ncube_out, ng, nd))) return r;
  return bcmg_case_output_wait(c);
}

int bcmg_case_output_wait(bcmg_case *c) {
  clear_err();
  if (!c) { set_err("null context"); return BCMG_ERR_ARG; }
  c->join_output();
  if (c->out_status) set_err(c->out_err);
  return c->out_status;
}

int bcmg_case_mirror(bcmg_case *c, float *M) {
  clear_err();
  if (!c || !M) { set_err("null argument"); return BCMG_ERR_ARG; }
  if (c->precision != BCMG_PRECISION_SPLIT) {
    set_err("the FP32 mirror exists on the split-precision path only");
    return BCMG_ERR_ARG;
  }
  CK(launch_mirror(c->U1_, c->M, c->M2, c->ph.n, c->ncube, c->ph.rho0, c->ph.P0, c->bt(),
                   c->stream));
  CK(cudaMemcpyAsync(M, c->M, c->ncell * 5 * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return BCMG_OK;
}

// The current mirror buffer as the kernels keep it, not re-formed.
int bcmg_case_mirror_current(bcmg_case *c, float *M) {
  clear_err();
  if (!c || !M) { set_err("null argument"); return BCMG_ERR_ARG; }
  if (c->precision != BCMG_PRECISION_SPLIT) {
    set_err("the FP32 mirror exists on the split-precision path only");
    return BCMG_ERR_ARG;
  }
  int par = 0;
  CK(cudaMemcpyAsync(&par, c->mpar, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  CK(cudaMemcpyAsync(M, par ? c->M2 : c->M, c->ncell * 5 * sizeof(float), cudaMemcpyDeviceToHost,
                     c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return BCMG_OK;
}

// ---------------------------------------------------------------------------
// Launch-shape tuning.  The choices change how work is split across CTAs,
// never the arithmetic of a cell: the FP64 path stays bit-identical to the
// reference with either tile edge (each cell's operations are the same), the
// split path's results change only by where a CTA boundary falls in its
// fixed-order norm sums.
// ---------------------------------------------------------------------------
int bcmg_case_set_tuning(bcmg_case *c, const bcmg_tuning *t) {
  clear_err();
  if (!c || !t) { set_err("null argument"); return BCMG_ERR_ARG; }
  const int n = c->ph.n;
  if (!(t->flux_tile == 0 || ((t->flux_tile == 4 || t->flux_tile == 8) && n % t->flux_tile == 0))) {
    set_err("flux_tile must be 0, or 4 or 8 dividing n");
    return BCMG_ERR_ARG;
  }
  if (t->lusgs_threads != 0 &&
      (n * n > 1024 || t->lusgs_threads % 32 != 0 || t->lusgs_threads < 32 ||
       t->lusgs_threads > lusgs_split_default_threads(n))) {
    set_err("lusgs_threads must be 0 or a multiple of 32 up to the widest plane of a cube");
    return BCMG_ERR_ARG;
  }
  if (t->flux_form < 0 || t->flux_form > 2) {
    set_err("flux_form must be 0, 1 or 2");
    return BCMG_ERR_ARG;
  }
  const int old_tiles = flux_split_blocks(n, 1, c->tile);
  c->tile = t->flux_tile;
  c->lu_threads = t->lusgs_threads;
  c->form = t->flux_form;
  const int tiles = flux_split_blocks(n, 1, c->tile);
  if (c->batched && tiles != old_tiles) {
    std::vector<int> cbf(c->ncase + 1);
    for (int q = 0; q <= c->ncase; ++q) cbf[q] = (c->case_cube0[q] - 1) * tiles;
    CK(cudaMemcpy(c->case_blk_flux, cbf.data(), sizeof(int) * cbf.size(), cudaMemcpyHostToDevice));
  }
  if (c->graph) cudaGraphExecDestroy(c->graph);  // captured steps hold the old shapes
  c->graph = nullptr;
  c->graph_subiters = -1;
  if (c->cgraph) cudaGraphExecDestroy(c->cgraph);
  c->cgraph = nullptr;
  return BCMG_OK;
}

int bcmg_case_set_mirror_each_stage(bcmg_case *c, int on) {
  clear_err();
  if (!c) { set_err("null context"); return BCMG_ERR_ARG; }
  c->mirror_each_stage = on != 0;
  if (c->graph) cudaGraphExecDestroy(c->graph);
  c->graph = nullptr;
  c->graph_subiters = -1;
  if (c->cgraph) cudaGraphExecDestroy(c->cgraph);
  c->cgraph = nullptr;
  c->cgraph_max = -1;
  return BCMG_OK;
}

int bcmg_case_set_face_copies(bcmg_case *c, int in_flux) {
  clear_err();
  if (!c) { set_err("null context"); return BCMG_ERR_ARG; }
  c->push_on = in_flux != 0;
  if (c->graph) cudaGraphExecDestroy(c->graph);  // captured steps hold the old lists
  c->graph = nullptr;
  c->graph_subiters = -1;
  if (c->cgraph) cudaGraphExecDestroy(c->cgraph);
  c->cgraph = nullptr;
  return BCMG_OK;
}

int bcmg_case_set_concurrent_ghosts(bcmg_case *c, int on) {
  clear_err();
  if (!c) { set_err("null context"); return BCMG_ERR_ARG; }
  c->ghost_side_on = on != 0;
  if (c->graph) cudaGraphExecDestroy(c->graph);  // captured steps hold the old order
  c->graph = nullptr;
  c->graph_subiters = -1;
  if (c->cgraph) cudaGraphExecDestroy(c->cgraph);
  c->cgraph = nullptr;
  return BCMG_OK;
}

int bcmg_case_concurrent_ghosts(bcmg_case *c) {
  if (!c) return 0;
  return c->ghost_beside_bc && c->ghost_side_on ? 1 : 0;
}

int bcmg_case_autotune(bcmg_case *c, int reps, bcmg_tuning *out) {
  clear_err();
  if (!c || reps < 1) { set_err("bad arguments"); return BCMG_ERR_ARG; }
  const int n = c->ph.n;
  bcmg_tuning best{};
  best.flux_tile = c->tile;
  best.lusgs_threads = c->lu_threads;
  best.flux_form = c->form;
  // Flux: tile 8 with packed face pairs, tile 8 one face at a time (the two
  // forms differ on the split path only), tile 4; each timed on the
  // context's own state (bcmg_case_time_flux restores it).
  const int tiles[3] = {8, 8, 4}, forms[3] = {1, 2, 0};
  double best_ms = 1e300;
  for (int v = 0; v < 3; ++v) {
    if (n % tiles[v] != 0) continue;
    if (v == 1 && c->precision != BCMG_PRECISION_SPLIT) continue;
    bcmg_tuning t = best;
    t.flux_tile = tiles[v];
    t.flux_form = forms[v];
    int r = bcmg_case_set_tuning(c, &t);
    if (r) return r;
    double ms = 0;
    if ((r = bcmg_case_time_flux(c, reps, &ms))) return r;
    best.flux_ms[v] = ms;
    if (ms < best_ms) {
      best_ms = ms;
      best.flux_tile = tiles[v];
      best.flux_form = forms[v];
    }
  }
  {
    int r = bcmg_case_set_tuning(c, &best);  // the LU-SGS candidates run on the chosen flux
    if (r) return r;
  }
  // Split LU-SGS sweep: the widest plane's threads or half of them (wide
  // planes then take two passes), timed on the residual of the current
  // state; the state is restored afterwards.
  if (c->precision == BCMG_PRECISION_SPLIT && c->method == BCMG_METHOD_LUSGS && c->lu_scr) {
    const int full = lusgs_split_default_threads(n);
    const int cand[2] = {full, ((full / 2) + 31) / 32 * 32};
    const size_t bytes = c->ncell * 5 * sizeof(double);
    CK(cudaMemcpyAsync(c->U1p1, c->U1_, bytes, cudaMemcpyDeviceToDevice, c->stream));
    int r = case_mirror_all(c);
    if (!r) r = case_flux(c, 0);  // residual of the current state
    if (r) return r;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    double lbest = 1e300;
    for (int v = 0; v < 2; ++v) {
      c->lu_threads = cand[v];
      LusgsSplitArgs l = lusgs_split_args(c);
      cudaError_t e = launch_lusgs_split(l, c->ncube - 1, c->stream);  // warm-up
      if (e == cudaSuccess) e = cudaEventRecord(e0, c->stream);
      for (int i = 0; i < reps && e == cudaSuccess; ++i)
        e = launch_lusgs_split(l, c->ncube - 1, c->stream);
      if (e == cudaSuccess) e = cudaEventRecord(e1, c->stream);
      if (e == cudaSuccess) e = cudaEventSynchronize(e1);
      float ms = 0;
      if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
      if (e != cudaSuccess) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        CK(e);
      }
      best.lusgs_ms[v] = ms / reps;
      if (ms / reps < lbest) {
        lbest = ms / reps;
        best.lusgs_threads = v == 0 ? 0 : cand[v];
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    CK(cudaMemcpyAsync(c->U1_, c->U1p1, bytes, cudaMemcpyDeviceToDevice, c->stream));
    if ((r = case_mirror_all(c))) return r;  // the sweeps updated the mirror in place
    CK(cudaStreamSynchronize(c->stream));
  }
  int r = bcmg_case_set_tuning(c, &best);
  if (r) return r;
  if (out) *out = best;
  return BCMG_OK;
}

int bcmg_case_ncase(const bcmg_case *c) { return c ? c->ncase : 0; }

int bcmg_case_case_cubes(const bcmg_case *c, int q, int *cube0, int *ncube) {
  clear_err();
  if (!c || q < 0 || q >= c->ncase) { set_err("bad context or case"); return BCMG_ERR_ARG; }
  const int a = c->batched ? c->case_cube0[q] : 1;
  const int b = c->batched ? c->case_cube0[q + 1] : c->ncube;
  if (cube0) *cube0 = a;
  if (ncube) *ncube = b - a + 1;  // the case's own cube slots incl. its unused slot 0
  return BCMG_OK;
}

// Copies between one case's own arrays [ncube_q][S][S][S][5] (slot 0
// skipped) and its cubes in the flat list.
static int case_copy(bcmg_case *c, int q, double *const host[3], bool to_device) {
  int g0 = 0, nq = 0;
  int r = bcmg_case_case_cubes(c, q, &g0, &nq);
  if (r) return r;
  const size_t cube_d = (size_t)c->S * c->S * c->S * 5;
  const size_t bytes = (size_t)(nq - 1) * cube_d * sizeof(double);
  double *dev[3] = {c->U1_, c->U1, c->U1q};
  for (int a = 0; a < 3; ++a) {
    if (!host[a]) continue;
    if (to_device)
      CK(cudaMemcpyAsync(dev[a] + (size_t)g0 * cube_d, host[a] + cube_d, bytes,
                         cudaMemcpyHostToDevice, c->stream));
    else
      CK(cudaMemcpyAsync(host[a] + cube_d, dev[a] + (size_t)g0 * cube_d, bytes,
                         cudaMemcpyDeviceToHost, c->stream));
  }
  if (to_device && c->precision == BCMG_PRECISION_SPLIT && (host[1] || host[2]))
    CK(launch_level_diff(c->U1, c->U1q, c->D2, c->ph.n, c->ncube, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return BCMG_OK;
}

int bcmg_case_set_case_state(bcmg_case *c, int q, const double *U1_, const double *U1,
                             const double *U1q) {
  clear_err();
  double *h[3] = {const_cast<double *>(U1_), const_cast<double *>(U1), const_cast<double *>(U1q)};
  return case_copy(c, q, h, true);
}

int bcmg_case_get_case_state(bcmg_case *c, int q, double *U1_, double *U1, double *U1q) {
  clear_err();
  double *h[3] = {U1_, U1, U1q};
  return case_copy(c, q, h, false);
}

}  // extern "C"

// ===========================================================================
// Drop-in twins of the reference routines (reference compile-time config
// held at run time).  Each call moves the caller's host arrays to the GPU,
// runs the same kernels as the resident context, and moves results back.
// ===========================================================================
namespace {

struct Compat {
  bcmg_reference_config cfg = {16, 1150, 0.0000185, 1.1842, 38.889, 38.889, 101300.0};
  cudaStream_t s = nullptr;
  int S = 0;                     // cube edge with ghosts of the current call
  int ncube = 0, full_S = 0;     // the whole-array buffers' geometry
  size_t ncell = 0;
  double *U1_ = nullptr, *U1 = nullptr, *U1q = nullptr, *U1p1 = nullptr, *U1p2 = nullptr,
         *Rku1 = nullptr, *Residual1 = nullptr, *cube_size = nullptr, *partials = nullptr,
         *er = nullptr;
  int *FWS = nullptr;
  int nparts = 0;
  // compact per-call cube buffer for routines that only touch listed cubes
  double *cubes = nullptr;
  size_t cubes_cap = 0;
  int *ibuf = nullptr;
  size_t ibuf_cap = 0;
  FaceTask *tasks = nullptr;
  size_t tasks_cap = 0;
  Ibm ibm;
  // split-precision flux twin (bcmg_set_reference_precision): mirror
  // buffers and flag, FP32 level difference, n / cube_size
  int precision = BCMG_PRECISION_FP64;
  float *M = nullptr, *M2 = nullptr, *D2 = nullptr, *inv_dx = nullptr;
  int *mpar = nullptr;

  Phys phys() const {
    Phys p;
    p.n = cfg.ncube_x;
    p.mpi_ncube = cfg.mpi_ncube;
    p.mu_L = cfg.mu_L;
    p.rho0 = cfg.rho0;
    p.U0 = cfg.U0;
    p.Uin = cfg.Uin;
    p.P0 = cfg.P0;
    return p;
  }
  int stream() {
    if (!s) CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    return BCMG_OK;
  }
  int ensure_full(int nc) {
    int r;
    if ((r = stream())) return r;
    // The full arrays' own geometry: S alone is also set by the boundary
    // and ghost-cell twins for the cube gathers, before any full call.
    const int Sx = cfg.ncube_x + 4;
    if (nc == ncube && Sx == full_S && U1_) return BCMG_OK;
    dfree(U1_); dfree(U1); dfree(U1q); dfree(U1p1); dfree(U1p2); dfree(Rku1);
    dfree(Residual1); dfree(cube_size); dfree(partials); dfree(er); dfree(FWS);
    dfree(M); dfree(M2); dfree(D2); dfree(inv_dx); dfree(mpar);
    ncube = nc;
    S = full_S = Sx;
    ncell = (size_t)nc * S * S * S;
    const size_t nd = ncell * 5;
    CK(dalloc(&U1_, nd)); CK(dalloc(&U1, nd)); CK(dalloc(&U1q, nd)); CK(dalloc(&U1p1, nd));
    CK(dalloc(&U1p2, nd)); CK(dalloc(&Rku1, nd)); CK(dalloc(&Residual1, nd));
    CK(dalloc(&cube_size, (size_t)nc)); CK(dalloc(&FWS, ncell)); CK(dalloc(&er, 8));
    RkArgs probe{};
    probe.ph = phys();
    probe.ncube = nc;
    nparts = std::max(rk_partial_blocks(probe), flux_split_blocks(cfg.ncube_x, nc - 1));
    CK(dalloc(&partials, (size_t)nparts * 7));
    return BCMG_OK;
  }
  int ensure_split() {
    if (M) return BCMG_OK;
    const size_t nd = ncell * 5;
    CK(dalloc(&M, nd)); CK(dalloc(&M2, nd)); CK(dalloc(&D2, nd));
    CK(dalloc(&inv_dx, (size_t)ncube)); CK(dalloc(&mpar, 1));
    CK(cudaMemsetAsync(mpar, 0, sizeof(int), s));
    return BCMG_OK;
  }
  template <typename T>
  int grow(T **p, size_t &cap, size_t need) {
    if (need <= cap && *p) return BCMG_OK;
    dfree(*p);
    CK(dalloc(p, need));
    cap = need;
    return BCMG_OK;
  }
};

Compat g_compat;

// Caller arrays of the twins, page-locked once (cudaHostRegister) when the
// caller opts in (bcmg_set_host_pinning(1)), so that every later copy of
// them runs at the host link's full rate instead of through pageable
// staging.  Opt-in because a registration must end before its memory is
// freed: a caller that frees arrays the twins have seen (a scripting
// front end, say) would leave registrations behind that a later array at
// the same address trips over.  The registration lasts until
// bcmg_release_host_arrays() or the process ends.
//
// Only the whole pages inside an array are registered.  The pages at its
// two ends may hold other objects (heap arrays of a few hundred KB sit side
// by side, and this host's pages may be 64 KB): registering them would make
// the runtime take a neighbour that starts there for page-locked memory
// and refuse its copy ("invalid argument") where the neighbour runs past
// the registration.  host_copy() therefore moves the registered middle of a
// range as one page-locked copy and the ends through pageable staging.  A
// region with no whole page, or that cannot be registered, is copied
// pageable.
struct HostPins {
  struct Reg {
    size_t bytes;
    const char *lo;  // registered span [lo, hi): the array's whole pages
  };
  std::map<const void *, Reg> reg;              // array base -> registration
  std::map<const char *, const char *> spans;   // lo -> hi, disjoint
  std::map<const void *, size_t> refused;
  bool enabled = false;
  static size_t page() {
    static const size_t p = [] {
      const long v = sysconf(_SC_PAGESIZE);
      return v > 0 ? (size_t)v : (size_t)4096;
    }();
    return p;
  }
  void pin(const void *p, size_t bytes) {
    if (!enabled || !p || bytes == 0) return;
    auto it = reg.find(p);
    if (it != reg.end() && it->second.bytes >= bytes) return;
    auto rf = refused.find(p);
    if (rf != refused.end() && rf->second >= bytes) return;
    if (it != reg.end()) {  // grown: register the larger region afresh
      cudaHostUnregister(const_cast<char *>(it->second.lo));
      spans.erase(it->second.lo);
      reg.erase(it);
    }
    const size_t P = page();
    const uintptr_t a = reinterpret_cast<uintptr_t>(p), e = a + bytes;
    const uintptr_t lo = (a + P - 1) / P * P, hi = e / P * P;
    if (hi > lo && cudaHostRegister(reinterpret_cast<void *>(lo), hi - lo,
                                    cudaHostRegisterDefault) == cudaSuccess) {
      reg[p] = Reg{bytes, reinterpret_cast<const char *>(lo)};
      spans[reinterpret_cast<const char *>(lo)] = reinterpret_cast<const char *>(hi);
    } else {
      cudaGetLastError();  // not sticky: the copies run pageable
      refused[p] = bytes;
    }
  }
  void release() {
    for (auto &kv : spans) cudaHostUnregister(const_cast<char *>(kv.first));
    spans.clear();
    reg.clear();
    refused.clear();
  }
  // Length of the piece of [h, h + bytes) that starts at h and lies either
  // wholly inside one registered span or wholly outside all of them.
  size_t piece(const char *h, size_t bytes, bool *locked) const {
    auto it = spans.upper_bound(h);  // first span starting after h
    if (it != spans.begin()) {
      auto pv = std::prev(it);
      if (pv->second > h) {
        *locked = true;
        return std::min(bytes, (size_t)(pv->second - h));
      }
    }
    *locked = false;
    return it == spans.end() ? bytes : std::min(bytes, (size_t)(it->first - h));
  }
};
HostPins g_pins;

// Copy between a caller's host array and the device, piece by piece so that
// no single copy mixes registered and unregistered pages.
cudaError_t host_copy(void *dst, const void *src, size_t bytes, cudaMemcpyKind kind,
                      cudaStream_t s) {
  const bool up = kind == cudaMemcpyHostToDevice;
  const char *h = static_cast<const char *>(up ? src : dst);
  size_t off = 0;
  while (off < bytes) {
    bool locked = false;
    const size_t len = g_pins.piece(h + off, bytes - off, &locked);
    cudaError_t e = cudaMemcpyAsync(static_cast<char *>(dst) + off,
                                    static_cast<const char *>(src) + off, len, kind, s);
    if (e != cudaSuccess) return e;
    off += len;
  }
  return cudaSuccess;
}

// A twin that stops on an error may leave copies of the caller's arrays in
// flight on its stream; they finish before the twin returns, so the caller
// may free or reuse its arrays (and end their registration) at once.
void twin_drain(int status) {
  if (status != BCMG_OK && g_compat.s) cudaStreamSynchronize(g_compat.s);
  cudaGetLastError();
}

// Host arrays of the flux twin whose device copies already hold the cells
// the routine never writes (uploaded once per host pointer): U1p1, U1p2,
// Rku1, Residual1 when a stage only writes them.  Only with
// bcmg_set_twin_scratch_kept(1): by default every array a stage returns is
// uploaded too, since a freed array's address may come back for another.
struct TwinSeen {
  const void *p[4] = {nullptr, nullptr, nullptr, nullptr};
  size_t ncell = 0;
};
TwinSeen g_twin_seen;
bool g_scratch_kept = false;

// Gather the listed cubes of a host array into the compact device buffer
// (slot 0 unused, slot m = cubes[m-1]); returns cube count.
int gather_cubes(Compat &C, const std::vector<int> &cubes, const double *hostU) {
  const size_t per = (size_t)C.S * C.S * C.S * 5;
  int r;
  if ((r = C.grow(&C.cubes, C.cubes_cap, per * (cubes.size() + 1)))) return r;
  int top = 0;
  for (int c : cubes) top = std::max(top, c);
  g_pins.pin(hostU, per * (top + 1) * sizeof(double));  // the array up to the last cube used
  for (size_t m = 0; m < cubes.size(); ++m)
    CK(host_copy(C.cubes + per * (m + 1), hostU + per * cubes[m], per * sizeof(double),
                 cudaMemcpyHostToDevice, C.s));
  return BCMG_OK;
}
int scatter_cubes(Compat &C, const std::vector<int> &cubes, double *hostU) {
  const size_t per = (size_t)C.S * C.S * C.S * 5;
  for (size_t m = 0; m < cubes.size(); ++m)
    CK(host_copy(hostU + per * cubes[m], C.cubes + per * (m + 1), per * sizeof(double),
                 cudaMemcpyDeviceToHost, C.s));
  CK(cudaStreamSynchronize(C.s));
  return BCMG_OK;
}

// One boundary-condition axis for the twins: lists are 1-based with counts.
int compat_bc(int axis, int nl, int nu, const int *lo, const int *up, double *U) {
  Compat &C = g_compat;
  int r;
  if ((r = C.stream())) return r;
  C.S = C.cfg.ncube_x + 4;
  if (nl < 0 || nu < 0 || (nl && !lo) || (nu && !up) || !U) {
    set_err("bad boundary-condition arguments");
    return BCMG_ERR_ARG;
  }
  std::vector<int> uniq;
  for (int a = 1; a <= nl; ++a) uniq.push_back(lo[a]);
  for (int a = 1; a <= nu; ++a) uniq.push_back(up[a]);
  for (int c : uniq)
    if (c <= 0) { set_err("boundary list holds a cube number < 1"); return BCMG_ERR_ARG; }
  std::sort(uniq.begin(), uniq.end());
  uniq.erase(std::unique(uniq.begin(), uniq.end()), uniq.end());
  if (uniq.empty()) return BCMG_OK;
  std::vector<int> slot(uniq.back() + 1, 0);
  for (size_t m = 0; m < uniq.size(); ++m) slot[uniq[m]] = (int)m + 1;
  std::vector<int> cubes(uniq.size()), masks(uniq.size(), 0);
  for (size_t m = 0; m < uniq.size(); ++m) cubes[m] = (int)m + 1;
  for (int a = 1; a <= nl; ++a) masks[slot[lo[a]] - 1] |= 1 << (2 * axis);
  for (int a = 1; a <= nu; ++a) masks[slot[up[a]] - 1] |= 2 << (2 * axis);
  if ((r = gather_cubes(C, uniq, U))) return r;
  if ((r = C.grow(&C.ibuf, C.ibuf_cap, 2 * cubes.size()))) return r;
  CK(cudaMemcpyAsync(C.ibuf, cubes.data(), sizeof(int) * cubes.size(), cudaMemcpyHostToDevice, C.s));
  CK(cudaMemcpyAsync(C.ibuf + cubes.size(), masks.data(), sizeof(int) * masks.size(),
                     cudaMemcpyHostToDevice, C.s));
  BcArgs b;
  b.n = C.cfg.ncube_x;
  b.Uin = C.cfg.Uin;
  b.cubes = C.ibuf;
  b.masks = C.ibuf + cubes.size();
  b.axes = 1 << axis;
  b.U1_ = C.cubes;
  CK(launch_bc(b, (int)cubes.size(), C.s));
  return scatter_cubes(C, uniq, U);
}

int compat_ghost(const int *NNBC, const double *weight, const int *GCindex, const int *IPsur,
                 double *U) {
  Compat &C = g_compat;
  int r;
  if ((r = C.stream())) return r;
  C.S = C.cfg.ncube_x + 4;
  if (!NNBC || *NNBC < 0 || !U || (*NNBC > 0 && (!weight || !GCindex || !IPsur))) {
    set_err("bad ghost-cell arguments");
    return BCMG_ERR_ARG;
  }
  const int nb = *NNBC;
  if (nb == 0) return BCMG_OK;
  // Remap the touched cubes to compact slots.
  std::vector<int> uniq;
  for (int e = 1; e <= nb; ++e) {
    uniq.push_back(IPsur[4 * (e - 1) + 1]);
    uniq.push_back(GCindex[4 * (e - 1) + 1]);
  }
  for (int c : uniq)
    if (c <= 0) { set_err("IBM table holds a cube number < 1"); return BCMG_ERR_ARG; }
  std::sort(uniq.begin(), uniq.end());
  uniq.erase(std::unique(uniq.begin(), uniq.end()), uniq.end());
  std::vector<int> slot(uniq.back() + 1, 0);
  for (size_t m = 0; m < uniq.size(); ++m) slot[uniq[m]] = (int)m + 1;
  std::vector<int> gc(GCindex, GCindex + 4 * (size_t)nb + 1), ip(IPsur, IPsur + 4 * (size_t)nb + 1);
  for (int e = 1; e <= nb; ++e) {
    gc[4 * (e - 1) + 1] = slot[gc[4 * (e - 1) + 1]];
    ip[4 * (e - 1) + 1] = slot[ip[4 * (e - 1) + 1]];
  }
  if ((r = ibm_upload(C.ibm, nb, weight, gc.data(), ip.data(), C.cfg.ncube_x,
                      (int)uniq.size() + 1, C.s)))
    return r;
  if ((r = gather_cubes(C, uniq, U))) return r;
  if ((r = ibm_run(C.ibm, C.cfg.ncube_x, C.cfg.rho0, C.cfg.P0, C.cubes, C.s, nullptr))) return r;
  return scatter_cubes(C, uniq, U);
}

}  // namespace

extern "C" {

int bcmg_set_reference_config(const bcmg_reference_config *cfg) {
  clear_err();
  if (!cfg || !valid_n(cfg->ncube_x) || cfg->mpi_ncube < 1) {
    set_err("invalid reference config (ncube_x multiple of 4, mpi_ncube >= 1)");
    return BCMG_ERR_ARG;
  }
  g_compat.cfg = *cfg;
  return BCMG_OK;
}

void bcmg_release_host_arrays(void) {
  clear_err();
  g_pins.release();
  g_twin_seen = TwinSeen{};
}

int bcmg_set_reference_precision(int precision) {
  clear_err();
  if (precision != BCMG_PRECISION_FP64 && precision != BCMG_PRECISION_SPLIT) {
    set_err("precision must be BCMG_PRECISION_FP64 or BCMG_PRECISION_SPLIT");
    return BCMG_ERR_ARG;
  }
  g_compat.precision = precision;
  return BCMG_OK;
}

void bcmg_set_twin_scratch_kept(int on) {
  g_scratch_kept = on != 0;
  g_twin_seen = TwinSeen{};
}

void bcmg_set_host_pinning(int on) {
  g_pins.enabled = on != 0;
  if (!on) g_pins.release();
}

void bcmg_get_reference_config(bcmg_reference_config *cfg) {
  if (cfg) *cfg = g_compat.cfg;
}

void BCM_Flux_XYZ_Viscous_Runge_kutta(int myid, int ncube, int RK, double deltaT,
                                      double deltaTau, double e, int *FWS, int *csl,
                                      double *cube_size, double *U1_, double *U1, double *U1q,
                                      double *U1p1, double *U1p2, double *Rku1,
                                      double *Residual1, double *er) {
  TraceRange trace("BCM_Flux_XYZ_Viscous_Runge_kutta");
  (void)myid;
  (void)csl;
  clear_err();
  Compat &C = g_compat;
  if (ncube < 1 || RK < 1 || RK > 3 || !FWS || !cube_size || !U1_ || !U1 || !U1q || !U1p1 ||
      !U1p2 || !Rku1 || !Residual1 || (RK == 3 && !er)) {
    set_err("BCM_Flux_XYZ_Viscous_Runge_kutta: bad arguments");
    return;
  }
  for (int i = 1; i < ncube; ++i)
    if (!(cube_size[i] > 0)) {
      set_err("BCM_Flux_XYZ_Viscous_Runge_kutta: cube_size must be positive");
      return;
    }
  auto run = [&]() -> int {
    int r;
    if ((r = C.ensure_full(ncube))) return r;
    const size_t b = C.ncell * 5 * sizeof(double);
    cudaStream_t s = C.s;
    TwinSeen &seen = g_twin_seen;
    if (seen.ncell != C.ncell) seen = TwinSeen{nullptr, nullptr, nullptr, nullptr, C.ncell};
    // Per stage, the arrays it reads go up (RK 1: U1_, U1, U1q; RK 2: also
    // U1p1; RK 3: also U1p2 and Residual1, whose fluid cells the norms sum);
    // the ones it only writes go up once per host array, since the routine
    // never writes their other cells.  Results come back whole.
    auto up = [&](double *dev, const double *host) -> int {
      g_pins.pin(host, b);
      CK(host_copy(dev, host, b, cudaMemcpyHostToDevice, s));
      return BCMG_OK;
    };
    auto up_once = [&](double *dev, const double *host, int slot) -> int {
      if (g_scratch_kept && seen.p[slot] == host) return BCMG_OK;
      int rr = up(dev, host);
      if (!rr) seen.p[slot] = host;
      return rr;
    };
    g_pins.pin(FWS, C.ncell * sizeof(int));
    CK(host_copy(C.FWS, FWS, C.ncell * sizeof(int), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(C.cube_size, cube_size, sizeof(double) * ncube, cudaMemcpyHostToDevice, s));
    if ((r = up(C.U1_, U1_)) || (r = up(C.U1, U1)) || (r = up(C.U1q, U1q))) return r;
    if (RK == 1 && (r = up_once(C.U1p1, U1p1, 0))) return r;
    if (RK == 2 && ((r = up(C.U1p1, U1p1)) || (r = up_once(C.U1p2, U1p2, 1)))) return r;
    if (RK == 3 && (r = up(C.U1p2, U1p2))) return r;
    if ((r = up_once(C.Rku1, Rku1, 2))) return r;
    if (RK == 3 ? (r = up(C.Residual1, Residual1)) : (r = up_once(C.Residual1, Residual1, 3)))
      return r;
    if (RK == 3) seen.p[3] = Residual1;
    for (double *h : {U1_, Rku1, Residual1}) g_pins.pin(h, b);
    if (RK == 1) g_pins.pin(U1p1, b);
    if (RK == 2) g_pins.pin(U1p2, b);
    int nb = 0;
    if (C.precision == BCMG_PRECISION_SPLIT) {
      // Split precision: FP32 mirror and level difference of this call's
      // state, then the split flux kernel applies the stage update in place
      // (Q += w dQ; Rku1 is not formed); U1p1 / U1p2 take the new state of
      // the fluid cells as the reference's combination leaves them.
      if ((r = C.ensure_split())) return r;
      const Phys ph = C.phys();
      std::vector<float> inv((size_t)ncube, 0.f);
      for (int i = 1; i < ncube; ++i) inv[i] = (float)(ph.n / cube_size[i]);
      CK(cudaMemcpyAsync(C.inv_dx, inv.data(), sizeof(float) * ncube, cudaMemcpyHostToDevice, s));
      CK(launch_mirror(C.U1_, C.M, C.M2, ph.n, ncube, ph.rho0, ph.P0, Batch(), s));
      CK(launch_level_diff(C.U1, C.U1q, C.D2, ph.n, ncube, s));
      FluxSplitArgs sa;
      sa.ph = ph;
      sa.cube0 = 1;
      sa.dT = deltaT;
      sa.dTau = deltaTau;
      sa.ef = (float)e;
      sa.rho0f = (float)ph.rho0;
      sa.P0f = (float)ph.P0;
      sa.RT0f = (float)(ph.P0 / ph.rho0);
      sa.T0f = (float)(ph.P0 / ph.rho0 / BCMG_R);
      sa.mu_Lf = (float)ph.mu_L;
      sa.i2dtf = (float)(1.0 / (2.0 * deltaT));
      sa.dTf = (float)deltaT;
      sa.dTauf = (float)deltaTau;
      sa.inv_dx = C.inv_dx;
      sa.FWS = C.FWS;
      sa.cube_size = C.cube_size;
      sa.mir.buf[0] = C.M;
      sa.mir.buf[1] = C.M2;
      sa.mir.parity = C.mpar;
      sa.mir.rho0 = ph.rho0;
      sa.mir.E0 = ph.P0 / (BCMG_K - 1);
      sa.U1_ = C.U1_;
      sa.U1 = C.U1;
      sa.U1q = C.U1q;
      sa.D2 = C.D2;
      sa.RK = RK;
      sa.form = 1;
      sa.partials = C.partials;
      sa.Residual1 = C.Residual1;
      CK(launch_flux_split(sa, ncube - 1, s));
      const long long total = (long long)(ncube - 1) * ph.n * ph.n * ph.n;
      const int blocks = (int)std::min<long long>(152 * 8, (total + 255) / 256);
      if (RK == 1 || RK == 2) {
        k_copy_fluid<<<blocks, 256, 0, s>>>(ph.n, ncube - 1, C.U1_, C.FWS,
                                            RK == 1 ? C.U1p1 : C.U1p2);
        CK(cudaGetLastError());
      }
      nb = flux_split_blocks(ph.n, ncube - 1);
      if (RK == 3) CK(launch_norms(ph, C.partials, nb, C.er, s));
      CK(host_copy(U1_, C.U1_, b, cudaMemcpyDeviceToHost, s));
      CK(host_copy(Residual1, C.Residual1, b, cudaMemcpyDeviceToHost, s));
      if (RK == 1) CK(host_copy(U1p1, C.U1p1, b, cudaMemcpyDeviceToHost, s));
      if (RK == 2) CK(host_copy(U1p2, C.U1p2, b, cudaMemcpyDeviceToHost, s));
      if (RK == 3) CK(cudaMemcpyAsync(er + 1, C.er + 1, 7 * sizeof(double), cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      return BCMG_OK;
    }
    FluxArgs a;
    a.ph = C.phys();
    a.cube0 = 1;
    a.dT = deltaT;
    a.dTau = deltaTau;
    a.e = e;
    a.FWS = C.FWS;
    a.cube_size = C.cube_size;
    a.U1_ = C.U1_;
    a.U1 = C.U1;
    a.U1q = C.U1q;
    a.Rku1 = C.Rku1;
    a.Residual1 = C.Residual1;
    CK(launch_flux_fp64(a, ncube - 1, s));
    RkArgs k;
    k.ph = C.phys();
    k.ncube = ncube;
    k.RK = RK;
    k.FWS = C.FWS;
    k.U1_ = C.U1_;
    k.U1p1 = C.U1p1;
    k.U1p2 = C.U1p2;
    k.Rku1 = C.Rku1;
    k.Residual1 = C.Residual1;
    k.partials = C.partials;
    CK(launch_rk(k, &nb, s));
    if (RK == 3) CK(launch_norms(C.phys(), C.partials, nb, C.er, s));
    CK(host_copy(U1_, C.U1_, b, cudaMemcpyDeviceToHost, s));
    CK(host_copy(Rku1, C.Rku1, b, cudaMemcpyDeviceToHost, s));
    CK(host_copy(Residual1, C.Residual1, b, cudaMemcpyDeviceToHost, s));
    if (RK == 1) CK(host_copy(U1p1, C.U1p1, b, cudaMemcpyDeviceToHost, s));
    if (RK == 2) CK(host_copy(U1p2, C.U1p2, b, cudaMemcpyDeviceToHost, s));
    if (RK == 3) CK(cudaMemcpyAsync(er + 1, C.er + 1, 7 * sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return BCMG_OK;
  };
  twin_drain(run());
}

void BCM_X_boundary_condition(int myid, int nXbc_l, int nXbc_u, int *Xbc_l, int *Xbc_u,
                              double *U1_) {
  (void)myid;
  clear_err();
  twin_drain(compat_bc(0, nXbc_l, nXbc_u, Xbc_l, Xbc_u, U1_));
}
void BCM_Y_boundary_condition(int nYbc_l, int nYbc_u, int *Ybc_l, int *Ybc_u, double *U1_) {
  clear_err();
  twin_drain(compat_bc(1, nYbc_l, nYbc_u, Ybc_l, Ybc_u, U1_));
}
void BCM_Z_boundary_condition(int nZbc_l, int nZbc_u, int *Zbc_l, int *Zbc_u, double *U1_) {
  clear_err();
  twin_drain(compat_bc(2, nZbc_l, nZbc_u, Zbc_l, Zbc_u, U1_));
}

void BCM_Ghostcell_minus(int myid, int *NNBC, double *weight, int *GCindex, int *IPsur,
                         int *FWS, double *U1_) {
  (void)myid;
  (void)FWS;
  clear_err();
  twin_drain(compat_ghost(NNBC, weight, GCindex, IPsur, U1_));
}
void BCM_Ghostcell_plus(int myid, int *NNBC, double *weight, int *GCindex, int *IPsur,
                        int *FWS, double *U1_) {
  (void)myid;
  (void)FWS;
  clear_err();
  twin_drain(compat_ghost(NNBC, weight, GCindex, IPsur, U1_));
}

void BCM_Interface(int myid, int ncube, int mPI_Nadj, int ncpu_bs, int ncpu_eq, int ncpu_sb,
                   int max_nei_bs, int max_nei_eq, int max_nei_sb, int nadjX_eq, int nadjY_eq,
                   int nadjZ_eq, int nadjX_bs_plus, int nadjX_sb_plus, int nadjX_bs_minus,
                   int nadjX_sb_minus, int nadjY_bs_plus, int nadjY_sb_plus,
                   int nadjY_bs_minus, int nadjY_sb_minus, int nadjZ_bs_plus,
                   int nadjZ_sb_plus, int nadjZ_bs_minus, int nadjZ_sb_minus, int *rank_map,
                   int *MPI_cpu, int *MPI_cube, int *MPI_cpu_adj, int *MPI_cube_adj,
                   int *MPI_direction, int *MPI_interface, int *neighbor_cpu_eq,
                   int *Ncube_Ncpu_eq, int *neighbor_cpu_sb, int *Ncube_Ncpu_sb,
                   int *neighbor_cpu_bs, int *Ncube_Ncpu_bs, int *Scube_Ncpu_eq,
                   int *Rcube_Ncpu_eq, double *send_data_curr_eq, double *recv_data_curr_eq,
                   double *send_data_neig_eq, double *recv_data_neig_eq, int *Sdir_eq,
                   int *Rdir_eq, int *Scube_Ncpu_sb, int *Rcube_Ncpu_sb,
                   double *send_data_curr_sb, double *recv_data_curr_sb,
                   double *send_data_neig_sb, double *recv_data_neig_sb, int *Sdir_sb,
                   int *Rdir_sb, int *Scube_Ncpu_bs, int *Rcube_Ncpu_bs,
                   double *send_data_curr_bs, double *recv_data_curr_bs,
                   double *send_data_neig_bs, double *recv_data_neig_bs, int *Sdir_bs,
                   int *Rdir_bs, int *ist_eq, int *ist_sb, int *ist_bs, int *adjN_sb,
                   int *RadjN_bs, int *SadjN_bs, int *csl, int *adj_number, int *adjX_eq,
                   int *adjY_eq, int *adjZ_eq, int *adjX_bs_plus, int *adjX_sb_plus,
                   int *adjX_bs_minus, int *adjX_sb_minus, int *adjY_bs_plus,
                   int *adjY_sb_plus, int *adjY_bs_minus, int *adjY_sb_minus,
                   int *adjZ_bs_plus, int *adjZ_sb_plus, int *adjZ_bs_minus,
                   int *adjZ_sb_minus, double *U1_) {
  TraceRange trace("BCM_Interface");
  (void)myid; (void)mPI_Nadj; (void)max_nei_bs; (void)max_nei_eq; (void)max_nei_sb;
  (void)rank_map; (void)MPI_cpu; (void)MPI_cube; (void)MPI_cpu_adj; (void)MPI_cube_adj;
  (void)MPI_direction; (void)MPI_interface; (void)neighbor_cpu_eq; (void)Ncube_Ncpu_eq;
  (void)neighbor_cpu_sb; (void)Ncube_Ncpu_sb; (void)neighbor_cpu_bs; (void)Ncube_Ncpu_bs;
  (void)Scube_Ncpu_eq; (void)Rcube_Ncpu_eq; (void)send_data_curr_eq; (void)recv_data_curr_eq;
  (void)send_data_neig_eq; (void)recv_data_neig_eq; (void)Sdir_eq; (void)Rdir_eq;
  (void)Scube_Ncpu_sb; (void)Rcube_Ncpu_sb; (void)send_data_curr_sb; (void)recv_data_curr_sb;
  (void)send_data_neig_sb; (void)recv_data_neig_sb; (void)Sdir_sb; (void)Rdir_sb;
  (void)Scube_Ncpu_bs; (void)Rcube_Ncpu_bs; (void)send_data_curr_bs; (void)recv_data_curr_bs;
  (void)send_data_neig_bs; (void)recv_data_neig_bs; (void)Sdir_bs; (void)Rdir_bs;
  (void)ist_eq; (void)ist_sb; (void)ist_bs; (void)adjN_sb; (void)RadjN_bs; (void)SadjN_bs;
  (void)adjX_sb_plus; (void)adjX_sb_minus; (void)adjY_sb_plus; (void)adjY_sb_minus;
  (void)adjZ_sb_plus; (void)adjZ_sb_minus; (void)nadjX_sb_plus; (void)nadjX_sb_minus;
  (void)nadjY_sb_plus; (void)nadjY_sb_minus; (void)nadjZ_sb_plus; (void)nadjZ_sb_minus;
  clear_err();
  if (ncpu_bs || ncpu_eq || ncpu_sb) {
    set_err("BCM_Interface: cross-rank exchange lists are not supported on one GPU");
    return;
  }
  const int *lists[9] = {adjX_eq, adjX_bs_plus, adjX_bs_minus, adjY_eq, adjY_bs_plus,
                         adjY_bs_minus, adjZ_eq, adjZ_bs_plus, adjZ_bs_minus};
  const int counts[9] = {nadjX_eq, nadjX_bs_plus, nadjX_bs_minus, nadjY_eq, nadjY_bs_plus,
                         nadjY_bs_minus, nadjZ_eq, nadjZ_bs_plus, nadjZ_bs_minus};
  bool bad = ncube < 2 || !adj_number || !U1_ || !csl;
  for (int l = 0; l < 9; ++l) bad |= counts[l] < 0 || (counts[l] > 0 && !lists[l]);
  if (bad) {
    set_err("BCM_Interface: bad arguments");
    return;
  }
  Compat &C = g_compat;
  auto run = [&]() -> int {
    int r;
    std::vector<int> off;
    std::vector<FaceTask> tasks;
    std::string err;
    if (!build_interface_tasks_from_lists(ncube, adj_number, csl, lists, counts, off, tasks,
                                          err)) {
      set_err("BCM_Interface: " + err);
      return BCMG_ERR_ARG;
    }
    if ((r = C.ensure_full(ncube))) return r;
    std::vector<int> task_cube(tasks.size());
    for (int cc = 1; cc < ncube; ++cc)
      for (int t = off[cc]; t < off[cc + 1]; ++t) task_cube[t] = cc;
    if ((r = C.grow(&C.ibuf, C.ibuf_cap, task_cube.size()))) return r;
    if ((r = C.grow(&C.tasks, C.tasks_cap, tasks.size()))) return r;
    const size_t b = C.ncell * 5 * sizeof(double);
    if (!task_cube.empty())
      CK(cudaMemcpyAsync(C.ibuf, task_cube.data(), sizeof(int) * task_cube.size(),
                         cudaMemcpyHostToDevice, C.s));
    if (!tasks.empty())
      CK(cudaMemcpyAsync(C.tasks, tasks.data(), sizeof(FaceTask) * tasks.size(),
                         cudaMemcpyHostToDevice, C.s));
    g_pins.pin(U1_, b);
    CK(host_copy(C.U1_, U1_, b, cudaMemcpyHostToDevice, C.s));
    InterfaceArgs ia;
    ia.n = C.cfg.ncube_x;
    ia.ntasks = (int)tasks.size();
    ia.task_cube = C.ibuf;
    ia.tasks = C.tasks;
    ia.U1_ = C.U1_;
    CK(launch_interface(ia, ncube, C.s));
    CK(host_copy(U1_, C.U1_, b, cudaMemcpyDeviceToHost, C.s));
    CK(cudaStreamSynchronize(C.s));
    return BCMG_OK;
  };
  twin_drain(run());
}

}  // extern "C"

// ===========================================================================
// Timing helpers: CUDA events on the context's stream, and a measured FP64
// FMA rate (the ALU roof of the FP64 path; GB300's FP64 rate is a small
// fraction of its FP32 rate).
// ===========================================================================
namespace {
__global__ void k_dfma_chain(double *out, int iters, double a, double b) {
  // 8 independent FMA chains per thread keep the FP64 pipe busy.
  double x[8];
#pragma unroll
  for (int m = 0; m < 8; ++m) x[m] = threadIdx.x * 1e-9 + m;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int m = 0; m < 8; ++m) x[m] = fma(x[m], a, b);
  }
  double s = 0;
#pragma unroll
  for (int m = 0; m < 8; ++m) s += x[m];
  if (s == 12345.678) out[0] = s;  // keeps the chains alive
}
}  // namespace

extern "C" {

int bcmg_case_timer_mark(bcmg_case *c, int slot) {
  clear_err();
  if (!c || slot < 0 || slot > 15) { set_err("bad timer slot"); return BCMG_ERR_ARG; }
  static_assert(sizeof(cudaEvent_t) == sizeof(void *), "event handle size");
  if (c->marks.empty()) {
    c->marks.resize(16, nullptr);
  }
  if (!c->marks[slot]) CK(cudaEventCreate(&c->marks[slot]));
  CK(cudaEventRecord(c->marks[slot], c->stream));
  return BCMG_OK;
}

int bcmg_case_timer_elapsed(bcmg_case *c, int a, int b, double *ms) {
  clear_err();
  if (!c || !ms || a < 0 || b < 0 || a > 15 || b > 15 || c->marks.empty() || !c->marks[a] ||
      !c->marks[b]) {
    set_err("timer marks not recorded");
    return BCMG_ERR_ARG;
  }
  CK(cudaEventSynchronize(c->marks[b]));
  float t = 0;
  CK(cudaEventElapsedTime(&t, c->marks[a], c->marks[b]));
  *ms = t;
  return BCMG_OK;
}

int bcmg_probe_fp64_rate(double *gflops) {
  clear_err();
  if (!gflops) { set_err("null argument"); return BCMG_ERR_ARG; }
  int dev = 0, sms = 0;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  double *out;
  CK(cudaMalloc(&out, sizeof(double)));
  cudaEvent_t a, b;
  CK(cudaEventCreate(&a));
  CK(cudaEventCreate(&b));
  const int blocks = sms * 4, threads = 256, iters = 4096;
  k_dfma_chain<<<blocks, threads>>>(out, 64, 1.0000001, 1e-9);  // warm-up
  CK(cudaEventRecord(a));
  k_dfma_chain<<<blocks, threads>>>(out, iters, 1.0000001, 1e-9);
  CK(cudaEventRecord(b));
  CK(cudaEventSynchronize(b));
  float ms = 0;
  CK(cudaEventElapsedTime(&ms, a, b));
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(out);
  const double flops = 2.0 * 8.0 * iters * (double)blocks * threads;
  *gflops = flops / (ms * 1e-3) / 1e9;
  return BCMG_OK;
}

}  // extern "C"
