// 2D TM kernels at the reference's granularity: one launch per reference
// function (dfield, efield, hfield, the TF/SF pieces, fourier), plus the
// device-side material map and a finite-value check.
//
// These are the per-function drop-ins of the C-ABI (fdtd2d_dfield ...) and the
// path fdtd2d_step_n takes when the TF/SF source or the full-field DFT is on.
// Each kernel updates the caller's arrays in place exactly like the reference
// loop it replaces; the serial order inside a reference function (e.g. the ABC
// of ezinct after the incident-line update) is kept, which the reference's own
// CUDA version does not do (fd2d/cuda/fd2d_3_4.cu:66-71 races on ezi[ny-2]).
#include "fd2d_internal.cuh"

namespace fdtd {

// ---------------------------------------------------------------- dfield
// fd2d/python/fd2d_3_2.py:62-69: i in [1,nx), j in [1,ny), then the source.
template <bool PML>
__global__ void k_dfield(int nx, int ny, fdtd2d_pml pml, float* __restrict__ dz, const float* __restrict__ hx,
                         const float* __restrict__ hy, int src_kind, int src_i, int src_j,
                         const float* __restrict__ src_table, float* __restrict__ ezi,
                         const float* __restrict__ tfsf_table, int t) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= nx || j >= ny) return;
  const float src_val = (src_kind != FDTD_SRC_NONE && i == src_i && j == src_j) ? src_table[t - 1] : 0.f;
  const size_t n = (size_t)i * ny + j;
  if (i >= 1 && j >= 1) {
    float gx3 = 1.f, gy3 = 1.f, gx2 = 1.f, gy2 = 1.f;
    if (PML) {
      gx3 = __ldg(pml.gx3 + i);
      gy3 = __ldg(pml.gy3 + j);
      gx2 = __ldg(pml.gx2 + i);
      gy2 = __ldg(pml.gy2 + j);
    }
    float d = d_update(dz[n], hy[n], hy[n - ny], hx[n], hx[n - 1], gx3, gy3, gx2, gy2);
    if (src_kind != FDTD_SRC_NONE && i == src_i && j == src_j)
      d = (src_kind == FDTD_SRC_HARD) ? src_val : __fadd_rn(d, src_val);
    dz[n] = d;
  } else if (src_kind != FDTD_SRC_NONE && i == src_i && j == src_j) {
    dz[n] = (src_kind == FDTD_SRC_HARD) ? src_val : __fadd_rn(dz[n], src_val);
  }
  // fd2d/python/fd2d_3_4.py:119: ezi[3] = gaussian(t, 20, 8.0)
  if (ezi && i == 0 && j == 0) ezi[3] = tfsf_table[t - 1];
}

// ---------------------------------------------------------------- efield
template <bool LOSSY>
__global__ void k_efield(size_t ncell, const float* __restrict__ naz, const float* __restrict__ nbz,
                         const float* __restrict__ dz, float* __restrict__ iz, float* __restrict__ ez) {
  for (size_t n = blockIdx.x * (size_t)blockDim.x + threadIdx.x; n < ncell; n += (size_t)gridDim.x * blockDim.x) {
    if (LOSSY) {
      float izv = iz[n];
      ez[n] = e_update_lossy(dz[n], izv, __ldg(naz + n), __ldg(nbz + n));
      iz[n] = izv;
    } else {
      ez[n] = e_update(dz[n], __ldg(naz + n));
    }
  }
}

// ---------------------------------------------------------------- hfield
// fd2d/python/fd2d_3_2.py:80-88: i in [0,nx-1), j in [0,ny-1).
template <bool PML>
__global__ void k_hfield(int nx, int ny, fdtd2d_pml pml, const float* __restrict__ ez, float* __restrict__ ihx,
                         float* __restrict__ ihy, float* __restrict__ hx, float* __restrict__ hy) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= nx - 1 || j >= ny - 1) return;
  const size_t n = (size_t)i * ny + j;
  const float e = ez[n];
  float hxv = hx[n], hyv = hy[n];
  if (PML) {
    float ihxv = ihx[n], ihyv = ihy[n];
    h_update_pml(e, ez[n + 1], ez[n + ny], hxv, hyv, ihxv, ihyv, __ldg(pml.fx1 + i), __ldg(pml.fx2 + i),
                 __ldg(pml.fx3 + i), __ldg(pml.fy1 + j), __ldg(pml.fy2 + j), __ldg(pml.fy3 + j));
    ihx[n] = ihxv;
    ihy[n] = ihyv;
  } else {
    h_update_free(e, ez[n + 1], ez[n + ny], hxv, hyv);
  }
  hx[n] = hxv;
  hy[n] = hyv;
}

// ---------------------------------------------------------------- TF/SF
// ezinct, fd2d/python/fd2d_3_4.py:103-110.  One block: the update loop, a
// barrier, then the two-step-back ABC on the updated values.
__global__ void k_ezinct(int ny, float* __restrict__ ezi, const float* __restrict__ hxi, float* __restrict__ bc) {
  for (int j = 1 + threadIdx.x; j < ny; j += blockDim.x)
    ezi[j] = __fmaf_rn(0.5f, __fsub_rn(hxi[j - 1], hxi[j]), ezi[j]);
  __syncthreads();
  if (threadIdx.x == 0) {
    ezi[0] = bc[0];
    bc[0] = bc[1];
    bc[1] = ezi[1];
    ezi[ny - 1] = bc[3];
    bc[3] = bc[2];
    bc[2] = ezi[ny - 2];
  }
}

// The incident line advanced nsteps steps in one block, in shared memory,
// with the same operations as k_ezinct (+ the ABC and the ezi[3] source of
// k_step_d), the ezi[6] input-probe DFT of k_step_e and k_hxinct, so the
// line equals the per-step kernels bit for bit.  Per step s it records what
// the 2D update reads: inc_e[s][:] = ezi after the E update and source, and
// inc_h[s] = hxi[npml-2], hxi[ny-npml] before the H update.
__global__ void k_inc_line(int ny, int npml, int t0, int nsteps, float* __restrict__ ezi, float* __restrict__ hxi,
                           float* __restrict__ bc, const float* __restrict__ tfsf_table, int nf,
                           const float* __restrict__ dft_cos, const float* __restrict__ dft_sin,
                           float* __restrict__ r_in, float* __restrict__ i_in, float* __restrict__ inc_e,
                           float* __restrict__ inc_h) {
  extern __shared__ float line[];
  float* e = line;
  float* h = line + ny;
  __shared__ float sbc[4];
  const int tid = threadIdx.x, nth = blockDim.x;
  for (int j = tid; j < ny; j += nth) {
    e[j] = ezi[j];
    h[j] = hxi[j];
  }
  if (tid < 4) sbc[tid] = bc[tid];
  float rin = 0.f, iin = 0.f;
  if (tid < nf) {
    rin = r_in[tid];
    iin = i_in[tid];
  }
  __syncthreads();
  for (int s = 0; s < nsteps; ++s) {
    const int t = t0 + s + 1;
    if (tid == 0) {
      inc_h[2 * s] = h[npml - 2];
      inc_h[2 * s + 1] = h[ny - npml];
    }
    for (int j = 1 + tid; j < ny; j += nth) e[j] = __fmaf_rn(0.5f, __fsub_rn(h[j - 1], h[j]), e[j]);
    __syncthreads();
    if (tid == 0) {
      e[0] = sbc[0];
      sbc[0] = sbc[1];
      sbc[1] = e[1];
      e[ny - 1] = sbc[3];
      sbc[3] = sbc[2];
      sbc[2] = e[ny - 2];
      e[3] = tfsf_table[t - 1];
    }
    __syncthreads();
    float* row = inc_e + (size_t)s * ny;
    for (int j = tid; j < ny; j += nth) row[j] = e[j];
    if (tid < nf) {
      const size_t k = (size_t)(t - 1) * nf + tid;
      rin = __fmaf_rn(dft_cos[k], e[6], rin);
      iin = __fmaf_rn(-dft_sin[k], e[6], iin);
    }
    for (int j = tid; j < ny - 1; j += nth) h[j] = __fmaf_rn(0.5f, __fsub_rn(e[j], e[j + 1]), h[j]);
    __syncthreads();
  }
  for (int j = tid; j < ny; j += nth) {
    ezi[j] = e[j];
    hxi[j] = h[j];
  }
  if (tid < 4) bc[tid] = sbc[tid];
  if (tid < nf) {
    r_in[tid] = rin;
    i_in[tid] = iin;
  }
}

// inctdz, fd2d/python/fd2d_3_4.py:123-127
__global__ void k_inctdz(int nx, int ny, int npml, const float* __restrict__ hxi, float* __restrict__ dz) {
  const int i = npml - 1 + blockIdx.x * blockDim.x + threadIdx.x;
  if (i > nx - npml) return;
  dz[(size_t)i * ny + (npml - 1)] = __fmaf_rn(0.5f, hxi[npml - 2], dz[(size_t)i * ny + (npml - 1)]);
  dz[(size_t)i * ny + (ny - npml)] = __fmaf_rn(-0.5f, hxi[ny - npml], dz[(size_t)i * ny + (ny - npml)]);
}

// hxinct, fd2d/python/fd2d_3_4.py:140-143
__global__ void k_hxinct(int ny, const float* __restrict__ ezi, float* __restrict__ hxi) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= ny - 1) return;
  hxi[j] = __fmaf_rn(0.5f, __fsub_rn(ezi[j], ezi[j + 1]), hxi[j]);
}

// incthx + incthy, fd2d/python/fd2d_3_4.py:158-170 (they touch disjoint arrays)
__global__ void k_incth(int nx, int ny, int npml, const float* __restrict__ ezi, float* __restrict__ hx,
                        float* __restrict__ hy) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = npml - 1 + k;
  if (i <= nx - npml) {
    hx[(size_t)i * ny + (npml - 2)] = __fmaf_rn(0.5f, ezi[npml - 1], hx[(size_t)i * ny + (npml - 2)]);
    hx[(size_t)i * ny + (ny - npml)] = __fmaf_rn(-0.5f, ezi[ny - npml], hx[(size_t)i * ny + (ny - npml)]);
  }
  const int j = npml - 1 + k;
  if (j <= ny - npml) {
    hy[(size_t)(npml - 2) * ny + j] = __fmaf_rn(-0.5f, ezi[j], hy[(size_t)(npml - 2) * ny + j]);
    hy[(size_t)(nx - npml) * ny + j] = __fmaf_rn(0.5f, ezi[j], hy[(size_t)(nx - npml) * ny + j]);
  }
}

// ---------------------------------------------------------------- fourier
// fd2d/python/fd2d_3_4.py:90-99: r += cos*ez, i -= sin*ez at every cell, plus
// the input probe ezi[6].
__global__ void k_fourier2d(size_t ncell, int nf, const float* __restrict__ cs, const float* __restrict__ sn,
                            const float* __restrict__ ez, const float* __restrict__ ezi, float* __restrict__ r_pt,
                            float* __restrict__ i_pt, float* __restrict__ r_in, float* __restrict__ i_in) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t n = blockIdx.x * (size_t)blockDim.x + threadIdx.x; n < ncell; n += stride) {
    const float e = ez[n];
    for (int f = 0; f < nf; ++f) {
      const size_t m = (size_t)f * ncell + n;
      r_pt[m] = __fmaf_rn(cs[f], e, r_pt[m]);
      i_pt[m] = __fmaf_rn(-sn[f], e, i_pt[m]);
    }
  }
  if (blockIdx.x == 0 && threadIdx.x < nf && ezi) {
    const int f = threadIdx.x;
    r_in[f] = __fmaf_rn(cs[f], ezi[6], r_in[f]);
    i_in[f] = __fmaf_rn(-sn[f], ezi[6], i_in[f]);
  }
}

// ---------------------------------------------------------------- dielectric
// fd2d/python/fd2d_3_4.py:174-194 in float64, same operation order
// (x = nx/2-1-i+m/3, d = sqrt(x*x+y*y), sequential sums of (epsr-1)/9, sigma/9).
__global__ void k_dielectric(int nx, int ny, int npml, double rgrid, double dt, double epsr, double sigma,
                             float* __restrict__ naz, float* __restrict__ nbz) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= nx || j >= ny) return;
  const size_t n = (size_t)i * ny + j;
  if (i < npml || i >= nx - npml || j < npml || j >= ny - npml) {
    naz[n] = 1.0f;
    nbz[n] = 0.0f;
    return;
  }
  const double eps0 = 8.854e-12;
  const double ce = (epsr - 1.0) / 9.0;
  const double cs = sigma / 9.0;
  double epsn = 1.0, cond = 0.0;
  for (int m = -1; m <= 1; ++m) {
    const double x = ((double)nx / 2.0 - 1.0 - (double)i) + (double)m / 3.0;
    for (int q = -1; q <= 1; ++q) {
      const double y = ((double)ny / 2.0 - 1.0 - (double)j) + (double)q / 3.0;
      const double d = __dsqrt_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)));
      if (d <= rgrid) {
        epsn = __dadd_rn(epsn, ce);
        cond = __dadd_rn(cond, cs);
      }
    }
  }
  const double nb = __ddiv_rn(__dmul_rn(cond, dt), eps0);
  naz[n] = (float)__ddiv_rn(1.0, __dadd_rn(epsn, nb));
  nbz[n] = (float)nb;
}

__global__ void k_check_finite(const float* __restrict__ x, size_t n, int* status) {
  bool bad = false;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
    bad |= !isfinite(x[k]);
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) raise_status(status, ST_NONFINITE);
}

// ================================================================ one step in three launches
// The TF/SF + DFT program (fd2d/python/fd2d_3_4.py:268-277) runs nine
// reference functions per step.  These three kernels do the same work in the
// same per-cell order, so the result is bitwise equal to the nine per-function
// launches:
//   S1  ezinct (block 0, after its cells) | dfield + source + inctdz per cell;
//   S2  efield + fourier per cell | hxinct + the input probe (block 0);
//   S3  hfield + incthx + incthy per cell.
// Race-free: S1 reads hxi and writes ezi/dz, S2 reads ezi and writes hxi/ez,
// S3 reads ezi/ez and writes hx/hy; no kernel reads what a peer block writes.

// S1: 2D grid of (32, 8) blocks; block (0, 0) also runs the incident line
template <bool PML>
__global__ void k_step_d(int nx, int ny, int npml, fdtd2d_pml pml, float* __restrict__ dz,
                         const float* __restrict__ hx, const float* __restrict__ hy, int src_kind, int src_i,
                         int src_j, const float* __restrict__ src_table, float* __restrict__ ezi,
                         const float* __restrict__ hxi, float* __restrict__ bc, const float* __restrict__ tfsf_table,
                         int t) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i < nx && j < ny) {
    const size_t n = (size_t)i * ny + j;
    const bool src_here = src_kind != FDTD_SRC_NONE && i == src_i && j == src_j;
    const float src_val = src_here ? src_table[t - 1] : 0.f;
    float d = dz[n];
    if (i >= 1 && j >= 1) {
      float gx3 = 1.f, gy3 = 1.f, gx2 = 1.f, gy2 = 1.f;
      if (PML) {
        gx3 = __ldg(pml.gx3 + i);
        gy3 = __ldg(pml.gy3 + j);
        gx2 = __ldg(pml.gx2 + i);
        gy2 = __ldg(pml.gy2 + j);
      }
      d = d_update(d, hy[n], hy[n - ny], hx[n], hx[n - 1], gx3, gy3, gx2, gy2);
    }
    if (src_here) d = (src_kind == FDTD_SRC_HARD) ? src_val : __fadd_rn(d, src_val);
    if (ezi && i >= npml - 1 && i <= nx - npml) {  // inctdz (fd2d/python/fd2d_3_4.py:123-127)
      if (j == npml - 1) d = __fmaf_rn(0.5f, hxi[npml - 2], d);
      if (j == ny - npml) d = __fmaf_rn(-0.5f, hxi[ny - npml], d);
    }
    dz[n] = d;
  }
  if (ezi && blockIdx.x == 0 && blockIdx.y == 0) {
    // ezinct (fd2d/python/fd2d_3_4.py:103-110), then ezi[3] of dfield (:119)
    const int tid = threadIdx.y * blockDim.x + threadIdx.x, nth = blockDim.x * blockDim.y;
    for (int k = 1 + tid; k < ny; k += nth) ezi[k] = __fmaf_rn(0.5f, __fsub_rn(hxi[k - 1], hxi[k]), ezi[k]);
    __syncthreads();
    if (tid == 0) {
      ezi[0] = bc[0];
      bc[0] = bc[1];
      bc[1] = ezi[1];
      ezi[ny - 1] = bc[3];
      bc[3] = bc[2];
      bc[2] = ezi[ny - 2];
      ezi[3] = tfsf_table[t - 1];
    }
  }
}

// S2: grid-stride over cells; block 0 also advances the incident hx line and
// accumulates the input probe ezi[6]
template <bool LOSSY>
__global__ void k_step_e(size_t ncell, int ny, const float* __restrict__ naz, const float* __restrict__ nbz,
                         const float* __restrict__ dz, float* __restrict__ iz, float* __restrict__ ez, int nf,
                         const float* __restrict__ cs, const float* __restrict__ sn, float* __restrict__ r_pt,
                         float* __restrict__ i_pt, const float* __restrict__ ezi, float* __restrict__ hxi,
                         float* __restrict__ r_in, float* __restrict__ i_in) {
  for (size_t n = blockIdx.x * (size_t)blockDim.x + threadIdx.x; n < ncell; n += (size_t)gridDim.x * blockDim.x) {
    float e;
    if (LOSSY) {
      float izv = iz[n];
      e = e_update_lossy(dz[n], izv, __ldg(naz + n), __ldg(nbz + n));
      iz[n] = izv;
    } else {
      e = e_update(dz[n], __ldg(naz + n));
    }
    ez[n] = e;
    for (int f = 0; f < nf; ++f) {  // fourier (fd2d/python/fd2d_3_4.py:90-99)
      const size_t m = (size_t)f * ncell + n;
      r_pt[m] = __fmaf_rn(cs[f], e, r_pt[m]);
      i_pt[m] = __fmaf_rn(-sn[f], e, i_pt[m]);
    }
  }
  if (blockIdx.x == 0 && ezi) {
    if (threadIdx.x < nf) {
      const int f = threadIdx.x;
      r_in[f] = __fmaf_rn(cs[f], ezi[6], r_in[f]);
      i_in[f] = __fmaf_rn(-sn[f], ezi[6], i_in[f]);
    }
    if (hxi)  // hxinct (fd2d/python/fd2d_3_4.py:140-143)
      for (int k = threadIdx.x; k < ny - 1; k += blockDim.x) hxi[k] = __fmaf_rn(0.5f, __fsub_rn(ezi[k], ezi[k + 1]), hxi[k]);
  }
}

// S3: hfield, then incthx/incthy on the TF/SF box edges (fd2d/python/fd2d_3_4.py:158-170)
template <bool PML>
__global__ void k_step_h(int nx, int ny, int npml, fdtd2d_pml pml, const float* __restrict__ ez,
                         float* __restrict__ ihx, float* __restrict__ ihy, float* __restrict__ hx,
                         float* __restrict__ hy, const float* __restrict__ ezi) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= nx - 1 || j >= ny - 1) return;
  const size_t n = (size_t)i * ny + j;
  const float e = ez[n];
  float hxv = hx[n], hyv = hy[n];
  if (PML) {
    float ihxv = ihx[n], ihyv = ihy[n];
    h_update_pml(e, ez[n + 1], ez[n + ny], hxv, hyv, ihxv, ihyv, __ldg(pml.fx1 + i), __ldg(pml.fx2 + i),
                 __ldg(pml.fx3 + i), __ldg(pml.fy1 + j), __ldg(pml.fy2 + j), __ldg(pml.fy3 + j));
    ihx[n] = ihxv;
    ihy[n] = ihyv;
  } else {
    h_update_free(e, ez[n + 1], ez[n + ny], hxv, hyv);
  }
  if (ezi) {
    if (i >= npml - 1 && i <= nx - npml) {
      if (j == npml - 2) hxv = __fmaf_rn(0.5f, ezi[npml - 1], hxv);
      if (j == ny - npml) hxv = __fmaf_rn(-0.5f, ezi[ny - npml], hxv);
    }
    if (j >= npml - 1 && j <= ny - npml) {
      if (i == npml - 2) hyv = __fmaf_rn(-0.5f, ezi[j], hyv);
      if (i == nx - npml) hyv = __fmaf_rn(0.5f, ezi[j], hyv);
    }
  }
  hx[n] = hxv;
  hy[n] = hyv;
}

// ================================================================ launchers
static inline dim3 grid2d(int nx, int ny, dim3 blk) {
  return dim3((unsigned)((ny + blk.x - 1) / blk.x), (unsigned)((nx + blk.y - 1) / blk.y));
}

int launch_dfield(int t, const fdtd2d_params& p, const fdtd2d_state& s, cudaStream_t st) {
  const dim3 blk(32, 8);
  float* ezi = p.tfsf_npml > 0 ? s.ezi : nullptr;
  if (has_pml(p))
    k_dfield<true><<<grid2d(p.nx, p.ny, blk), blk, 0, st>>>(p.nx, p.ny, p.pml, s.dz, s.hx, s.hy, p.src.kind, p.src.i,
                                                            p.src.j, p.src.table, ezi, p.tfsf_table, t);
  else
    k_dfield<false><<<grid2d(p.nx, p.ny, blk), blk, 0, st>>>(p.nx, p.ny, p.pml, s.dz, s.hx, s.hy, p.src.kind,
                                                             p.src.i, p.src.j, p.src.table, ezi, p.tfsf_table, t);
  return fdtd_host::check_launch();
}

int launch_efield(const fdtd2d_params& p, const fdtd2d_state& s, cudaStream_t st) {
  const size_t ncell = (size_t)p.nx * p.ny;
  const int blocks = (int)std::min<size_t>((ncell + 255) / 256, (size_t)152 * 16);
  if (p.nbz)
    k_efield<true><<<blocks, 256, 0, st>>>(ncell, p.naz, p.nbz, s.dz, s.iz, s.ez);
  else
    k_efield<false><<<blocks, 256, 0, st>>>(ncell, p.naz, nullptr, s.dz, nullptr, s.ez);
  return fdtd_host::check_launch();
}

int launch_hfield(const fdtd2d_params& p, const fdtd2d_state& s, cudaStream_t st) {
  const dim3 blk(32, 8);
  if (has_pml(p))
    k_hfield<true><<<grid2d(p.nx, p.ny, blk), blk, 0, st>>>(p.nx, p.ny, p.pml, s.ez, s.ihx, s.ihy, s.hx, s.hy);
  else
    k_hfield<false><<<grid2d(p.nx, p.ny, blk), blk, 0, st>>>(p.nx, p.ny, p.pml, s.ez, nullptr, nullptr, s.hx, s.hy);
  return fdtd_host::check_launch();
}

int launch_ezinct(const fdtd2d_params& p, const fdtd2d_state& s, cudaStream_t st) {
  k_ezinct<<<1, 1024, 0, st>>>(p.ny, s.ezi, s.hxi, s.bc);
  return fdtd_host::check_launch();
}

int launch_inctdz(const fdtd2d_params& p, const fdtd2d_state& s, cudaStream_t st) {
  const int n = p.nx - 2 * p.tfsf_npml + 2;
  k_inctdz<<<(n + 255) / 256, 256, 0, st>>>(p.nx, p.ny, p.tfsf_npml, s.hxi, s.dz);
  return fdtd_host::check_launch();
}

int launch_hxinct(const fdtd2d_params& p, const fdtd2d_state& s, cudaStream_t st) {
  k_hxinct<<<(p.ny + 255) / 256, 256, 0, st>>>(p.ny, s.ezi, s.hxi);
  return fdtd_host::check_launch();
}

int launch_incth(const fdtd2d_params& p, const fdtd2d_state& s, cudaStream_t st) {
  const int n = std::max(p.nx, p.ny) - 2 * p.tfsf_npml + 2;
  k_incth<<<(n + 255) / 256, 256, 0, st>>>(p.nx, p.ny, p.tfsf_npml, s.ezi, s.hx, s.hy);
  return fdtd_host::check_launch();
}

int launch_step3(int t, const fdtd2d_params& p, const fdtd2d_state& s, cudaStream_t st) {
  const dim3 blk(32, 8);
  const bool tfsf = p.tfsf_npml > 0;
  float* ezi = tfsf ? s.ezi : nullptr;
  const int npml = p.tfsf_npml;
  if (has_pml(p))
    k_step_d<true><<<grid2d(p.nx, p.ny, blk), blk, 0, st>>>(p.nx, p.ny, npml, p.pml, s.dz, s.hx, s.hy, p.src.kind,
                                                            p.src.i, p.src.j, p.src.table, ezi, s.hxi, s.bc,
                                                            p.tfsf_table, t);
  else
    k_step_d<false><<<grid2d(p.nx, p.ny, blk), blk, 0, st>>>(p.nx, p.ny, npml, p.pml, s.dz, s.hx, s.hy, p.src.kind,
                                                             p.src.i, p.src.j, p.src.table, ezi, s.hxi, s.bc,
                                                             p.tfsf_table, t);
  int rc = fdtd_host::check_launch();
  if (rc) return rc;
  const size_t ncell = (size_t)p.nx * p.ny;
  const int blocks = (int)std::min<size_t>((ncell + 255) / 256, (size_t)152 * 16);
  const int nf = p.nf > 0 ? p.nf : 0;
  const float* cs = nf ? p.dft_cos + (size_t)(t - 1) * nf : nullptr;
  const float* sn = nf ? p.dft_sin + (size_t)(t - 1) * nf : nullptr;
  // the input probe ezi[6] is accumulated only when the DFT is on (as fourier does)
  const float* ezi_e = tfsf ? s.ezi : nullptr;
  float* r_in = nf ? s.r_in : nullptr;
  float* i_in = nf ? s.i_in : nullptr;
  if (p.nbz)
    k_step_e<true><<<blocks, 256, 0, st>>>(ncell, p.ny, p.naz, p.nbz, s.dz, s.iz, s.ez, nf, cs, sn, s.r_pt, s.i_pt,
                                           ezi_e, tfsf ? s.hxi : nullptr, r_in, i_in);
  else
    k_step_e<false><<<blocks, 256, 0, st>>>(ncell, p.ny, p.naz, nullptr, s.dz, nullptr, s.ez, nf, cs, sn, s.r_pt,
                                            s.i_pt, ezi_e, tfsf ? s.hxi : nullptr, r_in, i_in);
  if ((rc = fdtd_host::check_launch())) return rc;
  if (has_pml(p))
    k_step_h<true><<<grid2d(p.nx, p.ny, blk), blk, 0, st>>>(p.nx, p.ny, npml, p.pml, s.ez, s.ihx, s.ihy, s.hx, s.hy,
                                                            ezi);
  else
    k_step_h<false><<<grid2d(p.nx, p.ny, blk), blk, 0, st>>>(p.nx, p.ny, npml, p.pml, s.ez, nullptr, nullptr, s.hx,
                                                             s.hy, ezi);
  return fdtd_host::check_launch();
}

int launch_inc_line(const fdtd2d_params& p, const fdtd2d_state& s, int t0, int nsteps, float* inc_e, float* inc_h,
                    cudaStream_t st) {
  const size_t smem = (size_t)2 * p.ny * sizeof(float);
  if (smem > 48 * 1024) {
    const cudaError_t e = cudaFuncSetAttribute(k_inc_line, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) {
      fdtd_host::note_cuda_error(e);
      return FDTD_ERR_CUDA;
    }
  }
  // the input probe is accumulated only with the DFT on (as in fourier)
  const int nf = p.nf > 0 ? p.nf : 0;
  k_inc_line<<<1, 1024, smem, st>>>(p.ny, p.tfsf_npml, t0, nsteps, s.ezi, s.hxi, s.bc, p.tfsf_table, nf, p.dft_cos,
                                    p.dft_sin, s.r_in, s.i_in, inc_e, inc_h);
  return fdtd_host::check_launch();
}

int launch_fourier(int t, const fdtd2d_params& p, const fdtd2d_state& s, cudaStream_t st) {
  const size_t ncell = (size_t)p.nx * p.ny;
  const int blocks = (int)std::min<size_t>((ncell + 255) / 256, (size_t)152 * 8);
  const float* cs = p.dft_cos + (size_t)(t - 1) * p.nf;
  const float* sn = p.dft_sin + (size_t)(t - 1) * p.nf;
  k_fourier2d<<<blocks, 256, 0, st>>>(ncell, p.nf, cs, sn, s.ez, p.tfsf_npml > 0 ? s.ezi : nullptr, s.r_pt, s.i_pt,
                                      s.r_in, s.i_in);
  return fdtd_host::check_launch();
}

int launch_dielectric(int nx, int ny, int npml, double rgrid, double dt, double epsr, double sigma, float* naz,
                      float* nbz, cudaStream_t st) {
  const dim3 blk(32, 8);
  k_dielectric<<<grid2d(nx, ny, blk), blk, 0, st>>>(nx, ny, npml, rgrid, dt, epsr, sigma, naz, nbz);
  return fdtd_host::check_launch();
}

int launch_check_finite(const float* x, size_t n, int* status, cudaStream_t st) {
  const int blocks = (int)std::min<size_t>((n + 255) / 256, (size_t)152 * 8);
  if (blocks > 0) k_check_finite<<<blocks, 256, 0, st>>>(x, n, status);
  return fdtd_host::check_launch();
}

}  // namespace fdtd
