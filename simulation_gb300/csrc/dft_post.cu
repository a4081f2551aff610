// Amplitude and phase of the running-DFT accumulators against the input
// probe, the post-processing the reference runs after its time loop:
//   amplt = 1/hypot(r_in, i_in) * hypot(r_pt, i_pt)
//   phase = arctan2(i_pt, r_pt) - arctan2(i_in, r_in)
// (fd1d/program/fd1d_2_2.py:145-146 over every cell, fd2d/python/fd2d_3_4.py:280-284
// along one row).  The FP32 accumulators are widened to double and the
// reference's float64 expressions are evaluated in its order.
#include "fdtd_common.cuh"

namespace {

__global__ void k_amp_phase(int nf, long long n, const float* __restrict__ r_pt, const float* __restrict__ i_pt,
                            long long ld, const float* __restrict__ r_in, const float* __restrict__ i_in,
                            double* __restrict__ amp, double* __restrict__ phase) {
  const long long total = (long long)nf * n;
  for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < total;
       x += (long long)gridDim.x * blockDim.x) {
    const int f = (int)(x / n);
    const long long k = x - (long long)f * n;
    const double rp = r_pt[(long long)f * ld + k], ip = i_pt[(long long)f * ld + k];
    const double ri = r_in[f], ii = i_in[f];
    if (amp) amp[x] = 1.0 / hypot(ri, ii) * hypot(rp, ip);
    if (phase) phase[x] = atan2(ip, rp) - atan2(ii, ri);
  }
}

}  // namespace

extern "C" int fdtd_dft_amplitude_phase(int nf, long long n, const float* r_pt, const float* i_pt, long long ld,
                                        const float* r_in, const float* i_in, double* amp, double* phase,
                                        fdtd_stream_t stream) {
  if (!r_pt || !i_pt || !r_in || !i_in) return FDTD_ERR_NULL;
  if (!amp && !phase) return FDTD_ERR_NULL;
  if (nf < 1 || n < 1 || ld < n) return FDTD_ERR_SIZE;
  const long long total = (long long)nf * n;
  const int threads = 256;
  const long long want = (total + threads - 1) / threads;
  const int blocks = (int)(want < 4096 ? want : 4096);
  k_amp_phase<<<blocks, threads, 0, (cudaStream_t)stream>>>(nf, n, r_pt, i_pt, ld, r_in, i_in, amp, phase);
  return fdtd_host::check_launch();
}
