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

}  // namespace fdtd
