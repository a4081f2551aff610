// Fused passes with the fd2d_3_4 extras for 4 DFT frequencies.
#include "fd2d_march.cuh"

namespace fdtd {
namespace march {
int launch_ext_nf4(const MarchArgs& a, int k, bool lossy, bool pml, cudaStream_t st) {
  return launch_ext_nfc<4>(a, k, lossy, pml, st);
}
}  // namespace march
}  // namespace fdtd
