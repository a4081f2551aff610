// Fused passes with the fd2d_3_4 extras for a DFT frequency count read at run time (5 .. kMarchMaxNf).
#include "fd2d_march.cuh"

namespace fdtd {
namespace march {
int launch_ext_nfrt(const MarchArgs& a, int k, bool lossy, bool pml, cudaStream_t st) {
  return launch_ext_nfc<-1>(a, k, lossy, pml, st);
}
}  // namespace march
}  // namespace fdtd
