// Single-warp fused 1D run with the running DFT (probes and full field).
#include "fd1d_warp.cuh"

namespace fdtd {

int launch_fd1d_warp_dft(const Warp1DArgs& a, int cpt, bool hi_end, cudaStream_t st) {
  return launch_fd1d_warp_half<true>(a, cpt, hi_end, st);
}

}  // namespace fdtd
