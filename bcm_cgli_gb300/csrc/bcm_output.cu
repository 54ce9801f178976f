// PLOT3D output gathers (BCM_Output.cpp:16-300).  The reference writes, per
// cube, the padded indices 1..n+2 of every array with the FIRST array index
// fastest (a transpose of the cube-major [i][j][k][v] layout), the five
// conservative variables as separate blocks after four 1.0 doubles, and the
// grid as X, Y, Z blocks of cell centres Xcube + (i - 1.5) dx
// (BCM_Grid.cpp:124-148).  These kernels form that byte image on the device
// (one output double per thread, coalesced writes), so the host only copies
// and writes contiguous bytes.  Built with --fmad=false: the coordinates are
// a separately rounded multiply and add, like the reference's.
#include <cuda_runtime.h>

#include "bcm_common.cuh"
#include "bcm_kernels.h"

namespace bcmg {

namespace {

__global__ void k_plot3d_q(const double *__restrict__ U, double *__restrict__ out, int n,
                           int cube0, int ncubes) {
  const int m = n + 2, S = n + 4;
  const size_t m3 = (size_t)m * m * m;
  const size_t per = 4 + 5 * m3;
  const size_t total = per * (size_t)ncubes;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const size_t cl = t / per, r = t - cl * per;
    double v = 1.0;
    if (r >= 4) {
      const size_t e = r - 4;
      const int var = (int)(e / m3);
      const size_t p = e - (size_t)var * m3;
      const int a = (int)(p / ((size_t)m * m)), b = (int)((p / m) % m), g = (int)(p % m);
      v = U[5 * cell_index(S, cube0 + (int)cl, 1 + g, 1 + b, 1 + a) + var];
    }
    out[t] = v;
  }
}

__global__ void k_plot3d_x(const double *__restrict__ cube_size,
                           const double *__restrict__ origin, double *__restrict__ out, int n,
                           int cube0, int ncubes) {
  const int m = n + 2;
  const size_t m3 = (size_t)m * m * m;
  const size_t per = 3 * m3;
  const size_t total = per * (size_t)ncubes;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const size_t cl = t / per, r = t - cl * per;
    const int ax = (int)(r / m3);
    const size_t p = r - (size_t)ax * m3;
    const int a = (int)(p / ((size_t)m * m)), b = (int)((p / m) % m), g = (int)(p % m);
    const int c = cube0 + (int)cl;
    const double dx = cube_size[c] / n;
    const int idx = 1 + (ax == 0 ? g : (ax == 1 ? b : a));  // X by the first index, ...
    out[t] = origin[3 * (size_t)cl + ax] + (idx - 1.5) * dx;
  }
}

int grid_for(size_t total) {
  size_t b = (total + 255) / 256;
  return (int)(b < 152 * 16 ? (b ? b : 1) : 152 * 16);
}

}  // namespace

cudaError_t launch_plot3d_q(const double *U, double *out, int n, int cube0, int ncubes,
                            cudaStream_t s) {
  if (ncubes <= 0) return cudaSuccess;
  const size_t m = n + 2;
  k_plot3d_q<<<grid_for((4 + 5 * m * m * m) * ncubes), 256, 0, s>>>(U, out, n, cube0, ncubes);
  return cudaGetLastError();
}

cudaError_t launch_plot3d_x(const double *cube_size, const double *origin, double *out, int n,
                            int cube0, int ncubes, cudaStream_t s) {
  if (ncubes <= 0) return cudaSuccess;
  const size_t m = n + 2;
  k_plot3d_x<<<grid_for(3 * m * m * m * ncubes), 256, 0, s>>>(cube_size, origin, out, n, cube0,
                                                              ncubes);
  return cudaGetLastError();
}

}  // namespace bcmg
