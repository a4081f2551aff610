// Fused passes with the fd2d_3_4 extras for 3 DFT frequencies.
#include "fd2d_march.cuh"

namespace fdtd {
namespace march {
int launch_ext_nf3(const MarchArgs& a, int k, bool lossy, bool pml, cudaStream_t st) {
  return launch_ext_nfc<3>(a, k, lossy, pml, st);
}
}  // namespace march
}  // namespace fdtd
