// Single-warp fused 1D run without the running DFT, and the dispatch.
#include "fd1d_warp.cuh"

namespace fdtd {

int launch_fd1d_warp_plain(const Warp1DArgs& a, int cpt, bool hi_end, cudaStream_t st) {
  return launch_fd1d_warp_half<false>(a, cpt, hi_end, st);
}

int launch_fd1d_warp(const fdtd1d_params& p, const fdtd1d_state& s, int t0, int nsteps, cudaStream_t st) {
  const int nx = p.nx;
  if (nx > 32 * 16) return FDTD_ERR_SIZE;
  // fewest cells per lane that cover the line with 32 lanes
  const int cpt = nx <= 64 ? 2 : nx <= 128 ? 4 : nx <= 256 ? 8 : 16;
  const Warp1DArgs a{p, s, t0, nsteps};
  const bool hi_end = nx % cpt == 0;
  return p.nf > 0 ? launch_fd1d_warp_dft(a, cpt, hi_end, st) : launch_fd1d_warp_plain(a, cpt, hi_end, st);
}

}  // namespace fdtd
