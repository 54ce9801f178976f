// FP32 mirror of the state for the split-precision path.
//
// The split kernels read the state as FP32 deltas from each case's reference
// state (rho0, 0, 0, 0, P0/(K-1)), rounded to nearest even from the FP64
// values.  Two buffers hold it: during an RK stage the flux kernel reads the
// current buffer (the halo of its tile belongs to other CTAs, which update
// their cells during the launch) and writes the deltas of its own cells
// into the other one; the kernel after it flips a device flag naming the
// current buffer.  Every other kernel that writes the FP64 state (boundary
// fill, IBM ghost cells, interface copies, edge fill, LU-SGS update) writes
// the same cells of the current buffer too, so the mirror stays the exact
// rounding of the state without a pass over all cells each stage.
#pragma once

#include <cuda_runtime.h>

#include "bcm_common.cuh"

namespace bcmg {

#ifdef __CUDACC__
// double -> float, round to nearest even (IEEE 754), on the integer pipes:
// this part's FP64 pipe, where the hardware conversion runs, is its
// narrowest (1/64 of FP32).  Results outside the normal float range
// (|x| < 2^-126, overflow, zero, inf/nan) take the hardware conversion.
__device__ __forceinline__ float to_float_rn(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
  if ((b << 1) == 0) return __uint_as_float(hi);  // signed zero (common: rest momenta)
  const int e = (int)((hi >> 20) & 0x7FF) - 1023 + 127;  // float exponent field
  if (e <= 0 || e >= 255) return (float)x;
  const unsigned m = ((hi & 0xFFFFFu) << 3) | (lo >> 29);  // top 23 fraction bits
  const unsigned rem = lo & 0x1FFFFFFFu, half = 0x10000000u;
  unsigned r = ((unsigned)e << 23) | m;
  r += (rem > half || (rem == half && (m & 1u))) ? 1u : 0u;  // a carry may raise the exponent
  return __uint_as_float((hi & 0x80000000u) | r);
}

// float -> double (exact) on the integer pipes, for the same reason; zero,
// subnormal, inf and nan inputs take the hardware conversion.
__device__ __forceinline__ double to_double_exact(float f) {
  const unsigned b = __float_as_uint(f);
  const unsigned e = (b >> 23) & 0xFFu;
  if ((b & 0x7FFFFFFFu) == 0) return __hiloint2double((int)(b & 0x80000000u), 0);
  if (e == 0 || e == 255) return (double)f;
  const unsigned hi = (b & 0x80000000u) | ((e + 896u) << 20) | ((b & 0x7FFFFFu) >> 3);
  return __hiloint2double((int)hi, (int)(b << 29));
}

// (float)(x - r) without FP64 arithmetic when x and r have the same sign and
// binade: their difference is then exact in FP64 (Sterbenz), so the integer
// difference of the 53-bit significands, rounded once to nearest even, is
// bit for bit the FP64 subtraction followed by the conversion.  Other inputs
// take that subtraction.
__device__ __forceinline__ float delta_rn(double x, double r) {
  const unsigned long long bx = (unsigned long long)__double_as_longlong(x),
                           br = (unsigned long long)__double_as_longlong(r);
  const int ex = (int)((bx >> 52) & 0x7FF);
  if (ex != (int)((br >> 52) & 0x7FF) || ex == 0 || ex == 0x7FF || ((bx ^ br) >> 63))
    return to_float_rn(x - r);
  const long long mx = (long long)((bx & 0xFFFFFFFFFFFFFull) | (1ull << 52));
  const long long mr = (long long)((br & 0xFFFFFFFFFFFFFull) | (1ull << 52));
  long long d = mx - mr;  // value = d * 2^(ex - 1075)
  if (bx >> 63) d = -d;
  if (d == 0) return 0.0f;  // x - x is +0 when rounding to nearest
  const unsigned sign = d < 0 ? 0x80000000u : 0u;
  const unsigned long long a = d < 0 ? (unsigned long long)(-d) : (unsigned long long)d;
  const int bl = 64 - __clzll((long long)a);  // bit length, at most 53
  int fe = (bl - 1) + (ex - 1075) + 127;     // float exponent field
  if (fe <= 0) return to_float_rn(x - r);    // subnormal float: hardware path
  unsigned m;
  if (bl <= 24) {
    m = (unsigned)(a << (24 - bl));
  } else {
    const int sh = bl - 24;
    const unsigned long long keep = a >> sh, rem = a & ((1ull << sh) - 1), half = 1ull << (sh - 1);
    m = (unsigned)keep;
    if (rem > half || (rem == half && (keep & 1))) {
      m += 1;
      if (m == (1u << 24)) {  // the carry raises the exponent
        m >>= 1;
        fe += 1;
      }
    }
  }
  if (fe >= 255) return to_float_rn(x - r);
  return __uint_as_float(sign | ((unsigned)fe << 23) | (m & 0x7FFFFFu));
}

// Mirror value of component v (0..4) of a state cell: density and energy as
// deltas from rho0 and E0 = P0/(K-1), momenta as they are.  Two routes to
// the same bits: on the integer pipes (for the whole-state pass k_mirror,
// where the FP64 pipe is the bottleneck) and through the hardware
// conversion (one FP64 subtraction and one conversion: for the kernels
// that write a few cells each, where the integer routine's instructions
// and branches cost more).
__device__ __forceinline__ float mirror_value(double x, int v, double rho0, double E0) {
  return v == 0 ? delta_rn(x, rho0) : (v == 4 ? delta_rn(x, E0) : to_float_rn(x));
}
__device__ __forceinline__ float mirror_value_hw(double x, int v, double rho0, double E0) {
  return __double2float_rn(v == 0 ? x - rho0 : (v == 4 ? x - E0 : x));
}
#endif  // __CUDACC__

// The two mirror buffers, the device flag naming the current one, and the
// reference state of a single case (batches take each cube's case).
// buf[0] == nullptr: no mirror (the FP64 path); kernels then skip it.
struct Mirror {
  float *buf[2] = {nullptr, nullptr};
  const int *parity = nullptr;  // device [1]: index of the current buffer
  double rho0 = 0, E0 = 0;
};

#ifdef __CUDACC__
// (a select, not m.buf[*m.parity]: indexing a kernel argument's array with
// a run-time value would copy the argument to local memory)
__device__ __forceinline__ float *mirror_current(const Mirror &m) {
  return m.buf[0] ? (*m.parity ? m.buf[1] : m.buf[0]) : nullptr;
}
#endif

}  // namespace bcmg
