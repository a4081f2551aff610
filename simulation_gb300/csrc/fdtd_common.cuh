// Shared device code for the FDTD kernels: the per-cell update formulas,
// status reporting and small PTX helpers.
//
// Every kernel of the library (per-function drop-ins, the fused streaming 2D
// kernel, the 1D kernels) calls the SAME inline formulas below, written with
// explicit round-to-nearest intrinsics, so their FP32 results are bitwise
// identical whatever the tiling, the number of fused time steps or the launch
// shape.  The operation order follows the reference's expressions
// (dsarvan/simulation fd2d/python/fd2d_3_2.py:66-88, fd2d/python/fd2d_3_4.py:131-136,
// fd1d/program/fd1d_1_3.py:55-62).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/fdtd.h"

namespace fdtd {

// ---------------------------------------------------------------- 2D TM cell
// Dz update, fd2d/python/fd2d_3_2.py:66-67:
//   dz = gx3[i]*gy3[j]*dz + gx2[i]*gy2[j]*0.5*(hy[i,j]-hy[i-1,j]-hx[i,j]+hx[i,j-1])
__device__ __forceinline__ float d_update(float dz, float hy, float hy_im1, float hx, float hx_jm1,
                                          float gx3, float gy3, float gx2, float gy2) {
  const float curl = __fadd_rn(__fsub_rn(__fsub_rn(hy, hy_im1), hx), hx_jm1);
  const float ca = __fmul_rn(gx3, gy3);
  const float cb = __fmul_rn(__fmul_rn(gx2, gy2), 0.5f);
  return __fmaf_rn(ca, dz, __fmul_rn(cb, curl));
}

// Ez from Dz, lossy medium, fd2d/python/fd2d_3_4.py:135-136:
//   ez = naz*(dz - iz); iz += nbz*ez
__device__ __forceinline__ float e_update_lossy(float dz, float& iz, float naz, float nbz) {
  const float ez = __fmul_rn(naz, __fsub_rn(dz, iz));
  iz = __fmaf_rn(nbz, ez, iz);
  return ez;
}

// Ez from Dz, lossless medium, fd2d/python/fd2d_3_2.py:75: ez = naz*dz
__device__ __forceinline__ float e_update(float dz, float naz) { return __fmul_rn(naz, dz); }

// Hx/Hy update with PML accumulators, fd2d/python/fd2d_3_2.py:84-87:
//   ihx += ez[i,j]-ez[i,j+1];  ihy += ez[i,j]-ez[i+1,j]
//   hx = fy3[j]*hx + fy2[j]*(0.5*ez[i,j] - 0.5*ez[i,j+1] + fx1[i]*ihx)
//   hy = fx3[i]*hy - fx2[i]*(0.5*ez[i,j] - 0.5*ez[i+1,j] + fy1[j]*ihy)
// (0.5*a - 0.5*b equals 0.5*(a-b) exactly in binary floating point.)
__device__ __forceinline__ void h_update_pml(float ez, float ez_jp1, float ez_ip1, float& hx, float& hy,
                                             float& ihx, float& ihy, float fx1, float fx2, float fx3,
                                             float fy1, float fy2, float fy3) {
  const float cx = __fsub_rn(ez, ez_jp1);
  const float cy = __fsub_rn(ez, ez_ip1);
  ihx = __fadd_rn(ihx, cx);
  ihy = __fadd_rn(ihy, cy);
  hx = __fmaf_rn(fy3, hx, __fmul_rn(fy2, __fmaf_rn(fx1, ihx, __fmul_rn(0.5f, cx))));
  hy = __fmaf_rn(fx3, hy, -__fmul_rn(fx2, __fmaf_rn(fy1, ihy, __fmul_rn(0.5f, cy))));
}

// The same two updates where every PML coefficient of the cell is the unit
// profile (gx2 = gx3 = gy2 = gy3 = 1, fx1 = fy1 = 0, fx2 = fx3 = fy2 = fy3 = 1,
// i.e. outside the absorbing layer).  The general formulas then reduce
// exactly: gx3*gy3 = 1 and gx2*gy2*0.5 = 0.5 are exact, fma(1, a, b) rounds
// a + b once, and fma(0, ihx, y) = y for finite ihx (up to the sign of a
// zero).  So these return the same values as d_update / h_update_pml called
// with the unit coefficients, with 2 and 6 fewer operations per cell.
__device__ __forceinline__ float d_update_unit(float dz, float hy, float hy_im1, float hx, float hx_jm1) {
  const float curl = __fadd_rn(__fsub_rn(__fsub_rn(hy, hy_im1), hx), hx_jm1);
  return __fadd_rn(dz, __fmul_rn(0.5f, curl));
}
__device__ __forceinline__ void h_update_pml_unit(float ez, float ez_jp1, float ez_ip1, float& hx, float& hy,
                                                  float& ihx, float& ihy) {
  const float cx = __fsub_rn(ez, ez_jp1);
  const float cy = __fsub_rn(ez, ez_ip1);
  ihx = __fadd_rn(ihx, cx);
  ihy = __fadd_rn(ihy, cy);
  hx = __fadd_rn(hx, __fmul_rn(0.5f, cx));
  hy = __fsub_rn(hy, __fmul_rn(0.5f, cy));
}

// Hx/Hy update without PML, fd2d/python/fd2d_3_1.py:70-71:
//   hx += 0.5*(ez[i,j]-ez[i,j+1]);  hy -= 0.5*(ez[i,j]-ez[i+1,j])
__device__ __forceinline__ void h_update_free(float ez, float ez_jp1, float ez_ip1, float& hx, float& hy) {
  hx = __fmaf_rn(0.5f, __fsub_rn(ez, ez_jp1), hx);
  hy = __fmaf_rn(-0.5f, __fsub_rn(ez, ez_ip1), hy);
}

// ---------------------------------------------------------------- 1D cell
// Ex update, dielectric form, fd1d/program/fd1d_1_3.py:55: ex += cb*(hy[i-1]-hy[i])
__device__ __forceinline__ float ex_update_cb(float ex, float hy_im1, float hy, float cb) {
  return __fmaf_rn(cb, __fsub_rn(hy_im1, hy), ex);
}
// Ex update, lossy form, fd1d/program/fd1d_1_5.py:65: ex = ca*ex + cb*(hy[i-1]-hy[i])
__device__ __forceinline__ float ex_update_cacb(float ex, float hy_im1, float hy, float ca, float cb) {
  return __fmaf_rn(ca, ex, __fmul_rn(cb, __fsub_rn(hy_im1, hy)));
}
// Dx update, fd1d/program/fd1d_2_2.py:76: dx += 0.5*(hy[i-1]-hy[i])
__device__ __forceinline__ float dx_update(float dx, float hy_im1, float hy) {
  return __fmaf_rn(0.5f, __fsub_rn(hy_im1, hy), dx);
}
// Ex from Dx, fd1d/program/fd1d_2_2.py:83-84: ex = nax*(dx-ix); ix += nbx*ex
__device__ __forceinline__ float ex_from_dx(float dx, float& ix, float nax, float nbx) {
  const float ex = __fmul_rn(nax, __fsub_rn(dx, ix));
  ix = __fmaf_rn(nbx, ex, ix);
  return ex;
}
// Debye medium, fd1d/program/fd1d_2_3.py:84-86:
//   ex = nax*(dx - ix - ncx*sx); ix += nbx*ex; sx = ncx*sx + ndx*ex
__device__ __forceinline__ float ex_from_dx_debye(float dx, float& ix, float& sx, float nax, float nbx,
                                                  float ncx, float ndx) {
  const float ex = __fmul_rn(nax, __fsub_rn(__fsub_rn(dx, ix), __fmul_rn(ncx, sx)));
  ix = __fmaf_rn(nbx, ex, ix);
  sx = __fmaf_rn(ncx, sx, __fmul_rn(ndx, ex));
  return ex;
}
// Hy update, fd1d/program/fd1d_1_3.py:62: hy += 0.5*(ex[i]-ex[i+1])
__device__ __forceinline__ float hy_update(float hy, float ex, float ex_ip1) {
  return __fmaf_rn(0.5f, __fsub_rn(ex, ex_ip1), hy);
}

// ---------------------------------------------------------------- status
// Device-side status word (an int in device memory owned by the caller).
// Kernels never trap: they OR a bit in and return.
enum : int {
  ST_NONFINITE = 1,   // a field value became Inf/NaN
  ST_TIMEOUT = 2,     // a bounded wait ran out
  ST_BOUNDS = 4,      // a bounds check (debug build) caught an index
};

__device__ __forceinline__ void raise_status(int* status, int bit) {
  if (status) atomicOr(status, bit);
}

__device__ __forceinline__ bool finite4(float a) { return isfinite(a); }

#ifdef FDTD_BOUNDS_CHECK
#define FDTD_CHECK_INDEX(idx, n, status)                         \
  do {                                                           \
    if ((long long)(idx) < 0 || (long long)(idx) >= (long long)(n)) { \
      fdtd::raise_status((status), fdtd::ST_BOUNDS);             \
      return;                                                    \
    }                                                            \
  } while (0)
#else
#define FDTD_CHECK_INDEX(idx, n, status) \
  do {                                   \
  } while (0)
#endif

}  // namespace fdtd

// ---------------------------------------------------------------- host side
namespace fdtd_host {
// Records the last CUDA error seen by an entry point (read by fdtd_last_cuda_error).
void note_cuda_error(cudaError_t e);
int check_launch();  // returns FDTD_OK or FDTD_ERR_CUDA after a launch
}  // namespace fdtd_host
