// Internal declarations shared by the 2D translation units.
#pragma once

#include <algorithm>
#include <cstddef>

#include "fdtd_common.cuh"

namespace fdtd {

inline bool has_pml(const fdtd2d_params& p) { return p.pml.fx1 != nullptr; }

// per-function launchers (fd2d_simple.cu)
int launch_dfield(int t, const fdtd2d_params& p, const fdtd2d_state& s, cudaStream_t st);
int launch_efield(const fdtd2d_params& p, const fdtd2d_state& s, cudaStream_t st);
int launch_hfield(const fdtd2d_params& p, const fdtd2d_state& s, cudaStream_t st);
int launch_ezinct(const fdtd2d_params& p, const fdtd2d_state& s, cudaStream_t st);
int launch_inctdz(const fdtd2d_params& p, const fdtd2d_state& s, cudaStream_t st);
int launch_hxinct(const fdtd2d_params& p, const fdtd2d_state& s, cudaStream_t st);
int launch_incth(const fdtd2d_params& p, const fdtd2d_state& s, cudaStream_t st);
int launch_fourier(int t, const fdtd2d_params& p, const fdtd2d_state& s, cudaStream_t st);
// one whole step (TF/SF, source, DFT included) in three launches, bitwise
// equal to the per-function sequence
int launch_step3(int t, const fdtd2d_params& p, const fdtd2d_state& s, cudaStream_t st);
int launch_dielectric(int nx, int ny, int npml, double rgrid, double dt, double epsr, double sigma, float* naz,
                      float* nbz, cudaStream_t st);
int launch_check_finite(const float* x, size_t n, int* status, cudaStream_t st);

// One pass of the fused streaming kernel (fd2d_march.cu): reads the level-0
// fields from `in`, writes the fields after `k` time steps (t0+1 .. t0+k) to
// `out` and Ez to s.ez.  `in` and `out` must not alias.
struct FieldSet {
  float *dz, *iz, *hx, *hy, *ihx, *ihy;
};
int launch_march(const fdtd2d_params& p, const FieldSet& in, const FieldSet& out, float* ez, int t0, int k,
                 int* status, float* probe_ez, cudaStream_t st);
// columns a warp of the fused kernel owns (for workspace/grid sizing)
int march_max_steps_per_pass();
// steps per pass the library picks for a grid (steps_per_pass = 0)
int march_default_steps(int nx, int ny);
// A pass that also records the state after each of its steps (the adjoint's
// recompute): rec[s] receives dz, iz, hx, hy after step t0+s+1, s < k.
// Point source only, with PML (plain kernels, 64-column stripes).
struct RecSet {
  float *dz, *iz, *hx, *hy;
};
int launch_march_record(const fdtd2d_params& p, const FieldSet& in, const FieldSet& out, float* ez, int t0, int k,
                        const RecSet* rec, cudaStream_t st);

// The fd2d_3_4 extras inside a fused pass (fd2d/python/fd2d_3_4.py:90-170):
// the TF/SF box corrections (inctdz, incthx, incthy) from a precomputed
// incident line, and the running DFT of Ez at every cell.
struct MarchExt {
  int tfsf_npml;       // 0: no TF/SF
  const float* inc_e;  // [k][ny]: ezi after step t0+s+1's ezinct and source (row s)
  const float* inc_h;  // [k][2]: hxi[npml-2], hxi[ny-npml] before step t0+s+1's hxinct
  int nf;              // 0: no DFT
  const float* dft_cos;  // [t-1][nf] tables of the whole run
  const float* dft_sin;
  float *r_pt, *i_pt;  // [nf][nx][ny] accumulators
};
constexpr int kMarchMaxNf = 8;         // DFT frequencies the fused pass carries
constexpr int kLineMaxNy = 16384;      // incident line held in shared memory
constexpr int kLineChunkSteps = 64;    // incident-line steps per table
bool march_ext_supported(const fdtd2d_params& p);
int launch_march_ext(const fdtd2d_params& p, const FieldSet& in, const FieldSet& out, float* ez, int t0, int k,
                     int* status, const MarchExt& ext, cudaStream_t st);
// Advance the incident line (ezinct, hxinct, the input-probe DFT) by nsteps
// steps t0+1 .. t0+nsteps and record what the 2D update reads of it
// (fd2d_simple.cu holds the per-step kernels it must equal bit for bit).
int launch_inc_line(const fdtd2d_params& p, const fdtd2d_state& s, int t0, int nsteps, float* inc_e, float* inc_h,
                    cudaStream_t st);

}  // namespace fdtd
