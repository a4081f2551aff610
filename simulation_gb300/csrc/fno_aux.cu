// Element-wise and reduction kernels of the 1D Fourier-neural-operator
// surrogate (the GEMMs run in gemm_tc.cu): lift, mode permutes between the
// DFT layout [B][C][2M] and the mode-major mixing layout [M][B][2C], complex
// weight expansion, GELU backward, mean pooling, column sums, per-sample
// partial sums, MSE loss and Adam.  No reference counterpart.
#include <cuda_bf16.h>

#include <algorithm>

#include "fdtd_common.cuh"

namespace fdtd {
namespace {

using bf16 = __nv_bfloat16;

// GELU, tanh form (Hendrycks & Gimpel 2016), the same function as the GEMM
// epilogue: 0.5 z (1 + tanh(u)), u = sqrt(2/pi) (z + 0.044715 z^3)
__device__ __forceinline__ float tanh_hw(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float gelu_f(float z) {
  const float u = 0.7978845608028654f * fmaf(0.044715f * z, z * z, z);
  return 0.5f * z * (1.0f + tanh_hw(u));
}
__device__ __forceinline__ float gelu_grad(float z) {
  // d/dz = 0.5 (1 + t) + 0.5 z (1 - t^2) sqrt(2/pi) (1 + 3*0.044715 z^2)
  const float u = 0.7978845608028654f * fmaf(0.044715f * z, z * z, z);
  const float t = tanh_hw(u);
  return 0.5f * (1.0f + t) + 0.5f * z * (1.0f - t * t) * 0.7978845608028654f * fmaf(0.134145f * z, z, 1.0f);
}

// Network inputs of slab profiles, built from their layer tables (the
// surrogate's profile_features): out[q][b][0..2] = (eps_r - 1)/eps_scale of
// cells 2b-1, 2b, 2b+1 of run run_idx[q], out[q][b][3..5] = sigma/sig_scale
// of the same cells; cells in no layer (or before cell 0) are vacuum, 0.
// The quotients are formed in double and rounded once, as the host form does.
__global__ void k_profile_features(int n, const int* __restrict__ run_idx, const int* __restrict__ layer_off,
                                   const int* __restrict__ layer_start, const int* __restrict__ layer_end,
                                   const double* __restrict__ epsr, const double* __restrict__ sigma, int nbins,
                                   double eps_scale, double sig_scale, float* __restrict__ out) {
  const long long total = (long long)n * nbins;
  for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < total;
       x += (long long)gridDim.x * blockDim.x) {
    const int q = (int)(x / nbins), b = (int)(x - (long long)q * nbins);
    const int r = run_idx ? run_idx[q] : q;
    const int l0 = layer_off[r], l1 = layer_off[r + 1];
    float v[6];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const int cell = 2 * b - 1 + c;
      double e = 0.0, g = 0.0;
      for (int l = l0; l < l1; ++l)
        if (cell >= layer_start[l] && cell < layer_end[l]) {
          e = (epsr[l] - 1.0) / eps_scale;
          g = sigma[l] / sig_scale;
        }
      v[c] = (float)e;
      v[3 + c] = (float)g;
    }
    float2* o = reinterpret_cast<float2*>(out + x * 6);
    o[0] = make_float2(v[0], v[1]);
    o[1] = make_float2(v[2], v[3]);
    o[2] = make_float2(v[4], v[5]);
  }
}

inline dim3 grid1(size_t n, int t = 256) {
  size_t b = (n + t - 1) / t;
  if (b > 152 * 64) b = 152 * 64;
  return dim3((unsigned)b);
}

// lift: x0[r][c] = sum_j P[c][j]*in[r][j] + p[c]   (r = b*N + n, j < cin)
__global__ void k_lift_fwd(size_t rows, int C, int cin, const float* __restrict__ in, const float* __restrict__ P,
                           const float* __restrict__ p, bf16* __restrict__ x0) {
  const size_t total = rows * C;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const size_t r = i / C;
    const int c = (int)(i % C);
    float v = p[c];
    for (int j = 0; j < cin; ++j) v = fmaf(P[c * cin + j], in[r * cin + j], v);
    x0[i] = __float2bfloat16_rn(v);
  }
}

constexpr int kLiftMaxIn = 8;

// The same lift, one thread per (row, 8 channels), 32-bit indices: block
// (C/8, 256/(C/8)) threads, x = channel group, y = row.  The thread's 8 x CIN
// weights stay in registers; each iteration loads the inputs of ROWS rows
// before computing, so several rows' loads are in flight per thread (one row
// at a time left the kernel waiting on memory latency), and every row leaves
// as one 16-byte store per thread.  Same accumulation order per element as
// k_lift_fwd, so results are identical.
template <int CIN, int ROWS>
__global__ void k_lift_fwd8(int rows, int C, const float* __restrict__ in, const float* __restrict__ P,
                            const float* __restrict__ p, bf16* __restrict__ x0) {
  const int c0 = threadIdx.x * 8;
  float pv[8], pw[8][CIN];
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    pv[k] = p[c0 + k];
#pragma unroll
    for (int j = 0; j < CIN; ++j) pw[k][j] = P[(c0 + k) * CIN + j];
  }
  const int stride = gridDim.x * blockDim.y;
  for (int r0 = blockIdx.x * blockDim.y + threadIdx.y; r0 < rows; r0 += ROWS * stride) {
    float xin[ROWS][CIN];
#pragma unroll
    for (int q = 0; q < ROWS; ++q) {
      const int r = r0 + q * stride;
#pragma unroll
      for (int j = 0; j < CIN; ++j) xin[q][j] = r < rows ? in[(size_t)r * CIN + j] : 0.f;
    }
#pragma unroll
    for (int q = 0; q < ROWS; ++q) {
      const int r = r0 + q * stride;
      if (r >= rows) break;
      float v[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        v[k] = pv[k];
#pragma unroll
        for (int j = 0; j < CIN; ++j) v[k] = fmaf(pw[k][j], xin[q][j], v[k]);
      }
      uint32_t w[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const __nv_bfloat162 h = __floats2bfloat162_rn(v[2 * k], v[2 * k + 1]);
        w[k] = *reinterpret_cast<const uint32_t*>(&h);
      }
      *reinterpret_cast<uint4*>(x0 + (size_t)r * C + c0) = make_uint4(w[0], w[1], w[2], w[3]);
    }
  }
}

// dP[c][j] += sum_r dx0[r][c]*in[r][j]; dp[c] += sum_r dx0[r][c]   (block per channel group)
__global__ void k_lift_bwd(size_t rows, int C, int cin, const float* __restrict__ in, const bf16* __restrict__ dx0,
                           float* __restrict__ dP, float* __restrict__ dp) {
  const int c = blockIdx.y;
  float s[kLiftMaxIn], sb = 0.f;
#pragma unroll
  for (int j = 0; j < kLiftMaxIn; ++j) s[j] = 0.f;
  for (size_t r = blockIdx.x * (size_t)blockDim.x + threadIdx.x; r < rows; r += (size_t)gridDim.x * blockDim.x) {
    const float d = __bfloat162float(dx0[r * C + c]);
#pragma unroll
    for (int j = 0; j < kLiftMaxIn; ++j)
      if (j < cin) s[j] = fmaf(d, in[r * cin + j], s[j]);
    sb += d;
  }
  for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
    for (int j = 0; j < kLiftMaxIn; ++j) s[j] += __shfl_down_sync(0xffffffffu, s[j], o);
    sb += __shfl_down_sync(0xffffffffu, sb, o);
  }
  if ((threadIdx.x & 31) == 0) {
#pragma unroll
    for (int j = 0; j < kLiftMaxIn; ++j)
      if (j < cin) atomicAdd(&dP[c * cin + j], s[j]);
    atomicAdd(&dp[c], sb);
  }
}

// ------------------------------------------------------------ propagation frame
// The surrogate predicts the spectrum in the frame of the single-pass
// propagation factor P(f) = exp(-i sum_cells k(f, cell)) from the entry probe
// to the exit probe, where k is the complex wavenumber of the 1D Yee update
// ex = ca ex + cb (hy[k-1] - hy[k]), hy += 0.5 (ex[k] - ex[k+1]) for a plane
// wave exp(i(w t - k x)):   sin^2(k/2) = (z^1/2 - ca z^-1/2) sin(w dt/2) / (i cb),
// z = exp(i w dt).  The branch is the wave travelling to the right, Re k > 0
// (in a passive cell that root also decays, Im k <= 0; choosing by the sign
// of Im k instead would let rounding flip lossless cells).
//
// cos k = 1 - 2 sin^2(k/2) = 1 - 2Q and sin k = sqrt(4Q(1-Q)) (no cancellation
// for small Q), so exp(ik) = cos k + i sin k and k = arg - i log|.|: one
// complex square root, one log and one atan2 per material and frequency, in
// FP32 (relative error ~1e-7; GB300's FP64 rate is a small fraction of FP32).
// The sums over cells (thousands of radians), and exp(-iK) at the end, are
// FP64: a layer of d cells adds d*k exactly to within k's own rounding, so the
// phase error stays near 1e-4 rad across a whole stack.
// s = sin(w dt/2), c = cos(w dt/2) are per-frequency constants.
__device__ float2 yee_wavenumber(float ca, float inv_cb, float s, float c) {
  const float qr = s * s * (1.0f + ca) * inv_cb, qi = -s * c * (1.0f - ca) * inv_cb;
  // 4 Q (1 - Q)
  const float ar = 4.0f * (qr * (1.0f - qr) + qi * qi), ai = 4.0f * (qi * (1.0f - qr) - qr * qi);
  // principal square root without cancellation: the small part is ai / (2 t)
  const float t = sqrtf(0.5f * (hypotf(ar, ai) + fabsf(ar)));
  float snr, sni;
  if (ar >= 0.0f) {
    snr = t;
    sni = t > 0.0f ? ai / (2.0f * t) : 0.0f;
  } else {
    snr = fabsf(ai) / (2.0f * t);
    sni = copysignf(t, ai);
  }
  const float wr = 1.0f - 2.0f * qr - sni, wi = -2.0f * qi + snr;
  float2 k = make_float2(atan2f(wi, wr), -0.5f * logf(wr * wr + wi * wi));
  if (k.x < 0.0f || (k.x == 0.0f && k.y > 0.0f)) k = make_float2(-k.x, -k.y);
  return k;
}

// Profile features, 6 channels per bin b: (eps_r - 1)/eps_scale of cells
// 2b-1, 2b, 2b+1, then sigma/sig_scale of the same cells; vacuum is all zero.
__device__ __forceinline__ void cell_material(const float* __restrict__ f, int nbins, int c, float& e, float& s) {
  if (c < 0 || c >= 2 * nbins) {
    e = 0.f;
    s = 0.f;
    return;
  }
  const float* b = f + (size_t)(c >> 1) * 6;
  e = b[1 + (c & 1)];
  s = b[4 + (c & 1)];
}

// one warp per sample; lane l handles frequencies l and l + 32
__global__ void k_propagation(int n, int nbins, const float* __restrict__ feat, int nf, const double* __restrict__ wdt,
                              double eps_scale, double sig_scale, double loss_scale, int probe_in, int probe_gap,
                              float* __restrict__ P) {
  const int sample = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (sample >= n) return;
  const float* f = feat + (size_t)sample * nbins * 6;
  int last = -1;
  for (int c = lane; c < 2 * nbins; c += 32) {
    float e, s;
    cell_material(f, nbins, c, e, s);
    if (e != 0.f || s != 0.f) last = c;
  }
  for (int o = 16; o > 0; o >>= 1) last = max(last, __shfl_xor_sync(0xffffffffu, last, o));
  const int probe_out = max(last + 1, probe_in) + probe_gap;
  float sh[2], ch[2];
  bool on[2];
  float2 k0[2];  // vacuum (ca = 1, cb = 0.5): the cells before and behind every stack
  for (int q = 0; q < 2; ++q) {
    on[q] = lane + 32 * q < nf;
    double sd, cd;
    sincos(0.5 * (on[q] ? wdt[lane + 32 * q] : 0.0), &sd, &cd);
    sh[q] = (float)sd;
    ch[q] = (float)cd;
    k0[q] = on[q] ? yee_wavenumber(1.0f, 2.0f, sh[q], ch[q]) : make_float2(0.f, 0.f);
  }
  double Kr[2] = {0.0, 0.0}, Ki[2] = {0.0, 0.0};
  float2 kc[2] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
  float ce = -1.f, cs = -1.f;  // current material (none yet: the first cell starts a run)
  int run_start = probe_in;
  // 32 cells per iteration, one per lane; material changes found by ballot and
  // handled in order by the whole warp (each lane for its two frequencies)
  for (int c0 = probe_in; c0 < probe_out; c0 += 32) {
    const int c = c0 + lane;
    float e = 0.f, s = 0.f;
    if (c < probe_out) cell_material(f, nbins, c, e, s);
    float pe = __shfl_up_sync(0xffffffffu, e, 1), ps = __shfl_up_sync(0xffffffffu, s, 1);
    if (lane == 0) {
      pe = ce;
      ps = cs;
    }
    unsigned chg = __ballot_sync(0xffffffffu, c < probe_out && (e != pe || s != ps));
    while (chg) {
      const int pos = __ffs(chg) - 1;
      chg &= chg - 1;
      const int run = c0 + pos - run_start;
      for (int q = 0; q < 2; ++q) {
        Kr[q] = fma((double)run, (double)kc[q].x, Kr[q]);
        Ki[q] = fma((double)run, (double)kc[q].y, Ki[q]);
      }
      run_start = c0 + pos;
      ce = __shfl_sync(0xffffffffu, e, pos);
      cs = __shfl_sync(0xffffffffu, s, pos);
      if (ce == 0.f && cs == 0.f) {
        kc[0] = k0[0];
        kc[1] = k0[1];
      } else {
        // the FDTD's float32 coefficients (lossy layer formula of fd1d/program/fd1d_1_5.py:37-44)
        const double er = 1.0 + eps_scale * (double)ce, sg = sig_scale * (double)cs;
        const double eaf = loss_scale * sg / er;
        const float ca = (float)((1.0 - eaf) / (1.0 + eaf));
        const float inv_cb = 1.0f / (float)(0.5 / (er * (1.0 + eaf)));
        for (int q = 0; q < 2; ++q) kc[q] = on[q] ? yee_wavenumber(ca, inv_cb, sh[q], ch[q]) : make_float2(0.f, 0.f);
      }
    }
  }
  const int run = probe_out - run_start;
  for (int q = 0; q < 2; ++q) {
    Kr[q] = fma((double)run, (double)kc[q].x, Kr[q]);
    Ki[q] = fma((double)run, (double)kc[q].y, Ki[q]);
    if (!on[q]) continue;
    // P = exp(-i K) = exp(Im K) (cos Re K - i sin Re K)
    const double a = exp(Ki[q]);
    double sn, cn;
    sincos(Kr[q], &sn, &cn);
    P[(size_t)sample * 2 * nf + lane + 32 * q] = (float)(a * cn);
    P[(size_t)sample * 2 * nf + nf + lane + 32 * q] = (float)(-a * sn);
  }
}

// out = P (.) y  or conj(P) (.) y per sample, spectra stored [Re(nf) | Im(nf)]
__global__ void k_cmul(size_t n, int nf, const float* __restrict__ P, const float* __restrict__ y, int conj_p,
                       float* __restrict__ out) {
  const size_t total = n * nf;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const size_t b = i / nf;
    const int k = (int)(i % nf);
    const size_t o = b * 2 * nf + k;
    const float pr = P[o], pi = conj_p ? -P[o + nf] : P[o + nf];
    const float yr = y[o], yi = y[o + nf];
    out[o] = fmaf(pr, yr, -pi * yi);
    out[o + nf] = fmaf(pr, yi, pi * yr);
  }
}

// DFT layout [B][C][2M] (cos rows 0..M-1, -sin rows M..2M-1) <-> mode-major
// [M][B][2C] with [Re | Im] along the last axis.  One block per sample b,
// through shared memory, so that both the [C][2M] side (rows of 2M) and the
// mode-major side (rows of C for each (k, part)) are read and written in
// contiguous runs.  The scalar versions are kept for shapes that do not fit.
constexpr int kPermSmem = 128 * 64 + 256;  // staged floats per block: 2M rows of C+1 (padded), 33 KB

__global__ void k_dft_to_modes_t(int B, int C, int M, const float* __restrict__ F, bf16* __restrict__ Fm) {
  __shared__ float t[kPermSmem];
  const int b = blockIdx.x;
  const int W = 2 * M, n = C * W;
  // read F_b [C][2M] as float4 (W % 4 == 0), scatter into the padded transpose
  const float4* src = reinterpret_cast<const float4*>(F + (size_t)b * n);
  for (int i = threadIdx.x; i < n / 4; i += blockDim.x) {
    const int c = (4 * i) / W, j = 4 * i - c * W;
    const float4 v = src[i];
    t[(j + 0) * (C + 1) + c] = v.x;
    t[(j + 1) * (C + 1) + c] = v.y;
    t[(j + 2) * (C + 1) + c] = v.z;
    t[(j + 3) * (C + 1) + c] = v.w;
  }
  __syncthreads();
  // destination rows (k, part) -> Fm[k][b][part*C + c .. +7] as 16-byte stores (C % 8 == 0)
  for (int i = threadIdx.x; i < n / 8; i += blockDim.x) {
    const int j = (8 * i) / C, c = 8 * i - j * C;  // j = part*M + k
    const int part = j / M, k = j - part * M;
    const float* r = t + j * (C + 1) + c;
    uint32_t w[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const __nv_bfloat162 h2 = __floats2bfloat162_rn(r[2 * e], r[2 * e + 1]);
      w[e] = *reinterpret_cast<const uint32_t*>(&h2);
    }
    *reinterpret_cast<uint4*>(Fm + ((size_t)k * B + b) * 2 * C + part * C + c) = make_uint4(w[0], w[1], w[2], w[3]);
  }
}

__global__ void k_modes_to_dft_t(int B, int C, int M, const float* __restrict__ Gm, bf16* __restrict__ G) {
  __shared__ float t[kPermSmem];
  const int b = blockIdx.x;
  const int W = 2 * M, n = C * W;
  // read the 2M mode rows of this sample (C contiguous floats each) as float4
  for (int i = threadIdx.x; i < n / 4; i += blockDim.x) {
    const int j = (4 * i) / C, c = 4 * i - j * C;  // j = part*M + k
    const int part = j / M, k = j - part * M;
    const float4 v = *reinterpret_cast<const float4*>(Gm + ((size_t)k * B + b) * 2 * C + part * C + c);
    float* r = t + j * (C + 1) + c;
    r[0] = v.x;
    r[1] = v.y;
    r[2] = v.z;
    r[3] = v.w;
  }
  __syncthreads();
  // G_b [C][2M] rows as 16-byte stores (W % 8 == 0)
  uint4* dst = reinterpret_cast<uint4*>(G + (size_t)b * n);
  for (int i = threadIdx.x; i < n / 8; i += blockDim.x) {
    const int c = (8 * i) / W, j = 8 * i - c * W;
    uint32_t w[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const __nv_bfloat162 h2 = __floats2bfloat162_rn(t[(j + 2 * e) * (C + 1) + c], t[(j + 2 * e + 1) * (C + 1) + c]);
      w[e] = *reinterpret_cast<const uint32_t*>(&h2);
    }
    dst[i] = make_uint4(w[0], w[1], w[2], w[3]);
  }
}

__global__ void k_dft_to_modes(int B, int C, int M, const float* __restrict__ F, bf16* __restrict__ Fm) {
  const size_t total = (size_t)B * C * 2 * M;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const int j = (int)(i % (2 * M));
    const size_t bc = i / (2 * M);
    const int c = (int)(bc % C);
    const int b = (int)(bc / C);
    const int k = j < M ? j : j - M;
    const int part = j < M ? 0 : 1;
    Fm[((size_t)k * B + b) * 2 * C + part * C + c] = __float2bfloat16_rn(F[i]);
  }
}

__global__ void k_modes_to_dft(int B, int C, int M, const float* __restrict__ Gm, bf16* __restrict__ G) {
  const size_t total = (size_t)B * C * 2 * M;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const int j = (int)(i % (2 * M));
    const size_t bc = i / (2 * M);
    const int c = (int)(bc % C);
    const int b = (int)(bc / C);
    const int k = j < M ? j : j - M;
    const int part = j < M ? 0 : 1;
    G[i] = __float2bfloat16_rn(Gm[((size_t)k * B + b) * 2 * C + part * C + c]);
  }
}

// complex per-mode weights R = Rr + i Ri acting on [Re|Im]: Rbig = [[Rr, -Ri], [Ri, Rr]]
__global__ void k_build_rbig(int M, int C, const float* __restrict__ Rr, const float* __restrict__ Ri,
                             bf16* __restrict__ Rbig) {
  const size_t total = (size_t)M * 4 * C * C;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const int col = (int)(i % (2 * C));
    const int row = (int)((i / (2 * C)) % (2 * C));
    const int k = (int)(i / (4 * (size_t)C * C));
    const int ro = row % C, co = col % C;
    const size_t s = ((size_t)k * C + ro) * C + co;
    float v;
    if (row < C) v = (col < C) ? Rr[s] : -Ri[s];
    else v = (col < C) ? Ri[s] : Rr[s];
    Rbig[i] = __float2bfloat16_rn(v);
  }
}

// Rectangular Rbig for the folded first layer: Rr, Ri are [M][Co][Ci],
// Rbig [M][2Co][2Ci] = [[Rr, -Ri], [Ri, Rr]]
__global__ void k_build_rbig_rect(int M, int Co, int Ci, const float* __restrict__ Rr, const float* __restrict__ Ri,
                                  bf16* __restrict__ Rbig) {
  const size_t total = (size_t)M * 4 * Co * Ci;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const int col = (int)(i % (2 * Ci));
    const int row = (int)((i / (2 * Ci)) % (2 * Co));
    const int k = (int)(i / (4 * (size_t)Co * Ci));
    const int ro = row % Co, co = col % Ci;
    const size_t s = ((size_t)k * Co + ro) * Ci + co;
    float v;
    if (row < Co) v = (col < Ci) ? Rr[s] : -Ri[s];
    else v = (col < Ci) ? Ri[s] : Rr[s];
    Rbig[i] = __float2bfloat16_rn(v);
  }
}

// C[b] = A[b] . B in FP32 (row-major, B shared), one thread per output: the
// small weight products of the folded first layer (W0 P', R_k P')
__global__ void k_small_matmul(int batch, int M, int N, int K, const float* __restrict__ A, const float* __restrict__ B,
                               float* __restrict__ Cm) {
  const size_t total = (size_t)batch * M * N;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const int n = (int)(i % N);
    const size_t bm = i / N;
    const float* a = A + bm * K;
    float t = 0.f;
    for (int k = 0; k < K; ++k) t = fmaf(a[k], B[(size_t)k * N + n], t);
    Cm[i] = t;
  }
}

// inputs for the folded first layer, one thread per row (b, n): the row
// (bf16(in[b][n][0..cin-1]), 1, 0 ... 0) goes to out[b][n][0..ldo-1]
// (sample-major, for the pointwise product; 64 wide, because narrower rows
// make the GEMM's TMA loads of A slow: 1.5 ms at K = 16 against 0.83 ms at
// K = 64 for 4096 spectra) and, when outT is given, to outT[n][b][0..15]
// (position-major, so the DFT of every sample's channels is one GEMM with the
// samples along M)
__global__ void k_pack_inputs16(int B, int N, int cin, int ldo, int write_pad, const float* __restrict__ in,
                                bf16* __restrict__ out, bf16* __restrict__ outT) {
  const long long rows = (long long)B * N;
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < rows; r += (long long)gridDim.x * blockDim.x) {
    const int b = (int)(r / N), n = (int)(r - (long long)b * N);
    uint32_t w[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const int j0 = 2 * k, j1 = 2 * k + 1;
      const float v0 = j0 < cin ? in[r * cin + j0] : (j0 == cin ? 1.0f : 0.0f);
      const float v1 = j1 < cin ? in[r * cin + j1] : (j1 == cin ? 1.0f : 0.0f);
      const __nv_bfloat162 h = __floats2bfloat162_rn(v0, v1);
      w[k] = *reinterpret_cast<const uint32_t*>(&h);
    }
    uint4* o = reinterpret_cast<uint4*>(out + r * ldo);
    o[0] = make_uint4(w[0], w[1], w[2], w[3]);
    o[1] = make_uint4(w[4], w[5], w[6], w[7]);
    if (write_pad)  // a caller reusing a zeroed buffer skips the constant padding
      for (int k = 2; k < ldo / 8; ++k) o[k] = make_uint4(0u, 0u, 0u, 0u);
    if (outT) {
      uint4* t = reinterpret_cast<uint4*>(outT + ((long long)n * B + b) * 16);
      t[0] = make_uint4(w[0], w[1], w[2], w[3]);
      t[1] = make_uint4(w[4], w[5], w[6], w[7]);
    }
  }
}

__global__ void k_fold_drbig(int M, int C, const float* __restrict__ dRbig, float* __restrict__ dRr,
                             float* __restrict__ dRi) {
  const size_t total = (size_t)M * C * C;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const int co = (int)(i % C);
    const int ro = (int)((i / C) % C);
    const int k = (int)(i / ((size_t)C * C));
    const size_t b = (size_t)k * 4 * C * C;
    const size_t w = 2 * (size_t)C;
    const float a00 = dRbig[b + ro * w + co], a01 = dRbig[b + ro * w + C + co];
    const float a10 = dRbig[b + (C + ro) * w + co], a11 = dRbig[b + (C + ro) * w + C + co];
    dRr[i] += a00 + a11;
    dRi[i] += a10 - a01;
  }
}

// dz = dy * gelu'(z)   (z = stored pre-activation, BF16)
__global__ void k_gelu_bwd(size_t n, const bf16* __restrict__ dy16, const float* __restrict__ dy32,
                           const bf16* __restrict__ pre, bf16* __restrict__ dz) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float d = dy16 ? __bfloat162float(dy16[i]) : dy32[i];
    dz[i] = __float2bfloat16_rn(d * gelu_grad(__bfloat162float(pre[i])));
  }
}

// h[b][c] = mean_n x[b][n][c]
__global__ void k_meanpool(int B, int N, int C, const bf16* __restrict__ x, bf16* __restrict__ h) {
  const int b = blockIdx.x;
  for (int c = threadIdx.x; c < C; c += blockDim.x) {
    float s = 0.f;
    for (int n = 0; n < N; ++n) s += __bfloat162float(x[((size_t)b * N + n) * C + c]);
    h[(size_t)b * C + c] = __float2bfloat16_rn(s / N);
  }
}

// The same mean with 16-byte loads: thread (g, y) of a 256-thread block sums
// channels 8g..8g+7 over rows y, y + ry, ...; the ry partial sums are added
// in shared memory in a fixed order (C % 8 == 0, C / 8 <= 256).
__global__ void k_meanpool8(int B, int N, int C, const bf16* __restrict__ x, bf16* __restrict__ h) {
  __shared__ float part[256 * 8];
  const int b = blockIdx.x;
  const int groups = C / 8, ry = blockDim.x / groups;
  const int g = threadIdx.x % groups, y = threadIdx.x / groups;
  float s[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  if (y < ry) {
    const bf16* base = x + (size_t)b * N * C + g * 8;
    for (int n = y; n < N; n += ry) {
      const uint4 u = *reinterpret_cast<const uint4*>(base + (size_t)n * C);
      const uint32_t w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const __nv_bfloat162 h2 = *reinterpret_cast<const __nv_bfloat162*>(&w[e]);
        s[2 * e] += __low2float(h2);
        s[2 * e + 1] += __high2float(h2);
      }
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) part[(y * groups + g) * 8 + k] = s[k];
  }
  __syncthreads();
  for (int c = threadIdx.x; c < C; c += blockDim.x) {
    const int gg = c / 8, k = c % 8;
    float t = 0.f;
    for (int yy = 0; yy < ry; ++yy) t += part[(yy * groups + gg) * 8 + k];
    h[(size_t)b * C + c] = __float2bfloat16_rn(t / N);
  }
}

// dx[b][n][c] = dh[b][c] / N
__global__ void k_meanpool_bwd(int B, int N, int C, const float* __restrict__ dh, bf16* __restrict__ dx) {
  const size_t total = (size_t)B * N * C;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const int c = (int)(i % C);
    const int b = (int)(i / ((size_t)N * C));
    dx[i] = __float2bfloat16_rn(dh[(size_t)b * C + c] / N);
  }
}

// out[c] += sum_r x[r][c]   (BF16 or FP32 input)
__global__ void k_colsum(size_t rows, int C, const bf16* __restrict__ x16, const float* __restrict__ x32,
                         float* __restrict__ out) {
  const int c = blockIdx.y * blockDim.x + threadIdx.x;
  if (c >= C) return;
  float s = 0.f;
  for (size_t r = blockIdx.x; r < rows; r += gridDim.x)
    s += x16 ? __bfloat162float(x16[r * C + c]) : x32[r * C + c];
  atomicAdd(&out[c], s);
}

// out[i] += sum_b parts[b][i]
__global__ void k_sum_parts(int nb, size_t n, const float* __restrict__ parts, float* __restrict__ out) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int b = 0; b < nb; ++b) s += parts[(size_t)b * n + i];
    out[i] += s;
  }
}

// loss = sum (o - y)^2 / (B * D); dO = 2 (o - y) / (B * D)
__global__ void k_mse(int B, int D, const float* __restrict__ o, const float* __restrict__ y, float* __restrict__ dO,
                      float* __restrict__ loss) {
  const size_t n = (size_t)B * D;
  const float inv = 1.0f / (float)n;
  float s = 0.f;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float d = o[i] - y[i];
    dO[i] = 2.0f * d * inv;
    s += d * d * inv;
  }
  for (int k = 16; k > 0; k >>= 1) s += __shfl_down_sync(0xffffffffu, s, k);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, s);
}

// relative loss per sample: w_b = 1 / max(||y_b||^2, floor2);
// loss = mean_b w_b ||o_b - y_b||^2, dO = 2 w_b (o_b - y_b) / B   (one block per sample)
__global__ void k_rel_mse(int B, int D, float floor2, const float* __restrict__ o, const float* __restrict__ y,
                          float* __restrict__ dO, float* __restrict__ loss) {
  const int b = blockIdx.x;
  __shared__ float red[2][32];
  float sy = 0.f, sd = 0.f;
  for (int d = threadIdx.x; d < D; d += blockDim.x) {
    const float yy = y[(size_t)b * D + d], dd = o[(size_t)b * D + d] - yy;
    sy += yy * yy;
    sd += dd * dd;
  }
  for (int k = 16; k > 0; k >>= 1) {
    sy += __shfl_down_sync(0xffffffffu, sy, k);
    sd += __shfl_down_sync(0xffffffffu, sd, k);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    red[0][w] = sy;
    red[1][w] = sd;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float ty = 0.f, td = 0.f;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
      ty += red[0][k];
      td += red[1][k];
    }
    red[0][0] = 1.0f / fmaxf(ty, floor2);
    atomicAdd(loss, td * red[0][0] / B);
  }
  __syncthreads();
  const float wb = red[0][0];
  for (int d = threadIdx.x; d < D; d += blockDim.x)
    dO[(size_t)b * D + d] = 2.0f * wb * (o[(size_t)b * D + d] - y[(size_t)b * D + d]) / B;
}

// Adam (Kingma & Ba 2015) on FP32 master weights; writes a BF16 copy if given
__global__ void k_adam(size_t n, float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, float lr, float b1, float b2, float eps, float bc1, float bc2,
                       bf16* __restrict__ w16) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
    w[i] = wi;
    if (w16) w16[i] = __float2bfloat16_rn(wi);
  }
}

__global__ void k_to_bf16(size_t n, const float* __restrict__ x, bf16* __restrict__ y) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    y[i] = __float2bfloat16_rn(x[i]);
}

__global__ void k_gelu_fwd(size_t n, const float* __restrict__ z, bf16* __restrict__ y, bf16* __restrict__ pre) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    if (pre) pre[i] = __float2bfloat16_rn(z[i]);
    y[i] = __float2bfloat16_rn(gelu_f(z[i]));
  }
}

}  // namespace
}  // namespace fdtd

// ======================================================================= C-ABI
// One entry point per surrogate helper; sizes are validated, pointers are
// device pointers, nothing synchronises the host.
using fdtd::bf16;
#define FNO_LAUNCH(kern, grid, block, ...)                       \
  do {                                                           \
    kern<<<grid, block, 0, (cudaStream_t)stream>>>(__VA_ARGS__); \
    return fdtd_host::check_launch();                            \
  } while (0)

extern "C" {

int fno_lift_fwd(long long rows, int C, int cin, const float* in, const float* P, const float* p, void* x0,
                 fdtd_stream_t stream) {
  if (!in || !P || !p || !x0) return FDTD_ERR_NULL;
  if (rows < 1 || C < 1 || cin < 1 || cin > fdtd::kLiftMaxIn) return FDTD_ERR_SIZE;
  if ((cin == 2 || cin == 6) && C % 8 == 0 && C <= 2048 && rows < (1LL << 30) && ((uintptr_t)x0 & 15) == 0) {
    const dim3 blk(C / 8, std::max(1, 256 / (C / 8)));
    const long long nblk = std::min<long long>((rows + blk.y - 1) / blk.y, 152LL * 16);
    if (cin == 6)
      FNO_LAUNCH((fdtd::k_lift_fwd8<6, 8>), dim3((unsigned)nblk), blk, (int)rows, C, in, P, p, (bf16*)x0);
    FNO_LAUNCH((fdtd::k_lift_fwd8<2, 8>), dim3((unsigned)nblk), blk, (int)rows, C, in, P, p, (bf16*)x0);
  }
  FNO_LAUNCH(fdtd::k_lift_fwd, fdtd::grid1((size_t)rows * C), 256, (size_t)rows, C, cin, in, P, p, (bf16*)x0);
}

int fno_lift_bwd(long long rows, int C, int cin, const float* in, const void* dx0, float* dP, float* dp,
                 fdtd_stream_t stream) {
  if (!in || !dx0 || !dP || !dp) return FDTD_ERR_NULL;
  if (rows < 1 || C < 1 || C > 65535 || cin < 1 || cin > fdtd::kLiftMaxIn) return FDTD_ERR_SIZE;
  FNO_LAUNCH(fdtd::k_lift_bwd, dim3(64, C), 256, (size_t)rows, C, cin, in, (const bf16*)dx0, dP, dp);
}

int fno_propagation(int n, int nbins, const float* feat, int nf, const double* wdt, double eps_scale,
                    double sig_scale, double loss_scale, int probe_in, int probe_gap, float* P,
                    fdtd_stream_t stream) {
  if (!feat || !wdt || !P) return FDTD_ERR_NULL;
  if (n < 1 || nbins < 1 || nf < 1 || nf > 64 || probe_in < 0 || probe_gap < 0 || !(eps_scale > 0))
    return FDTD_ERR_SIZE;
  const long long threads = 32LL * n;
  FNO_LAUNCH(fdtd::k_propagation, dim3((unsigned)((threads + 255) / 256)), 256, n, nbins, feat, nf, wdt, eps_scale,
             sig_scale, loss_scale, probe_in, probe_gap, P);
}

int fno_profile_features(int n, const int* run_idx, const int* layer_off, const int* layer_start,
                         const int* layer_end, const double* epsr, const double* sigma, int nbins, double eps_scale,
                         double sig_scale, float* out, fdtd_stream_t stream) {
  if (!layer_off || !layer_start || !layer_end || !epsr || !sigma || !out) return FDTD_ERR_NULL;
  if (n < 1 || nbins < 1 || !(eps_scale > 0) || !(sig_scale > 0)) return FDTD_ERR_SIZE;
  if ((uintptr_t)out & 7) return FDTD_ERR_ALIGN;
  FNO_LAUNCH(fdtd::k_profile_features, fdtd::grid1((size_t)n * nbins), 256, n, run_idx, layer_off, layer_start,
             layer_end, epsr, sigma, nbins, eps_scale, sig_scale, out);
}

int fno_cmul(long long n, int nf, const float* P, const float* y, int conj_p, float* out, fdtd_stream_t stream) {
  if (!P || !y || !out) return FDTD_ERR_NULL;
  if (n < 1 || nf < 1) return FDTD_ERR_SIZE;
  FNO_LAUNCH(fdtd::k_cmul, fdtd::grid1((size_t)n * nf), 256, (size_t)n, nf, P, y, conj_p, out);
}

int fno_dft_to_modes(int B, int C, int M, const float* F, void* Fm, fdtd_stream_t stream) {
  if (!F || !Fm) return FDTD_ERR_NULL;
  if (B < 1 || C < 1 || M < 1) return FDTD_ERR_SIZE;
  if ((C + 1) * 2 * M <= fdtd::kPermSmem && C % 8 == 0 && M % 4 == 0 && ((uintptr_t)F & 15) == 0 &&
      ((uintptr_t)Fm & 15) == 0)
    FNO_LAUNCH(fdtd::k_dft_to_modes_t, dim3(B), 256, B, C, M, F, (bf16*)Fm);
  FNO_LAUNCH(fdtd::k_dft_to_modes, fdtd::grid1((size_t)B * C * 2 * M), 256, B, C, M, F, (bf16*)Fm);
}

int fno_modes_to_dft(int B, int C, int M, const float* Gm, void* G, fdtd_stream_t stream) {
  if (!Gm || !G) return FDTD_ERR_NULL;
  if (B < 1 || C < 1 || M < 1) return FDTD_ERR_SIZE;
  if ((C + 1) * 2 * M <= fdtd::kPermSmem && C % 8 == 0 && M % 4 == 0 && ((uintptr_t)Gm & 15) == 0 &&
      ((uintptr_t)G & 15) == 0)
    FNO_LAUNCH(fdtd::k_modes_to_dft_t, dim3(B), 256, B, C, M, Gm, (bf16*)G);
  FNO_LAUNCH(fdtd::k_modes_to_dft, fdtd::grid1((size_t)B * C * 2 * M), 256, B, C, M, Gm, (bf16*)G);
}

int fno_build_rbig(int M, int C, const float* Rr, const float* Ri, void* Rbig, fdtd_stream_t stream) {
  if (!Rr || !Ri || !Rbig) return FDTD_ERR_NULL;
  if (M < 1 || C < 1) return FDTD_ERR_SIZE;
  FNO_LAUNCH(fdtd::k_build_rbig, fdtd::grid1((size_t)M * 4 * C * C), 256, M, C, Rr, Ri, (bf16*)Rbig);
}

int fno_build_rbig_rect(int M, int Co, int Ci, const float* Rr, const float* Ri, void* Rbig, fdtd_stream_t stream) {
  if (!Rr || !Ri || !Rbig) return FDTD_ERR_NULL;
  if (M < 1 || Co < 1 || Ci < 1) return FDTD_ERR_SIZE;
  FNO_LAUNCH(fdtd::k_build_rbig_rect, fdtd::grid1((size_t)M * 4 * Co * Ci), 256, M, Co, Ci, Rr, Ri, (bf16*)Rbig);
}

int fno_small_matmul(int batch, int M, int N, int K, const float* A, const float* B, float* Cm, fdtd_stream_t stream) {
  if (!A || !B || !Cm) return FDTD_ERR_NULL;
  if (batch < 1 || M < 1 || N < 1 || K < 1) return FDTD_ERR_SIZE;
  FNO_LAUNCH(fdtd::k_small_matmul, fdtd::grid1((size_t)batch * M * N), 256, batch, M, N, K, A, B, Cm);
}

int fno_pack_inputs(int B, int N, int cin, int ldo, int write_pad, const float* in, void* out, void* out_t,
                    fdtd_stream_t stream) {
  if (!in || !out) return FDTD_ERR_NULL;
  if (B < 1 || N < 1 || cin < 1 || cin > 15 || ldo < 16 || ldo % 8) return FDTD_ERR_SIZE;
  if (((uintptr_t)out & 15) || ((uintptr_t)out_t & 15)) return FDTD_ERR_ALIGN;
  FNO_LAUNCH(fdtd::k_pack_inputs16, fdtd::grid1((size_t)B * N), 256, B, N, cin, ldo, write_pad, in, (bf16*)out,
             (bf16*)out_t);
}

int fno_fold_drbig(int M, int C, const float* dRbig, float* dRr, float* dRi, fdtd_stream_t stream) {
  if (!dRbig || !dRr || !dRi) return FDTD_ERR_NULL;
  if (M < 1 || C < 1) return FDTD_ERR_SIZE;
  FNO_LAUNCH(fdtd::k_fold_drbig, fdtd::grid1((size_t)M * C * C), 256, M, C, dRbig, dRr, dRi);
}

int fno_gelu_bwd(long long n, const void* dy16, const float* dy32, const void* pre, void* dz, fdtd_stream_t stream) {
  if ((!dy16 && !dy32) || !pre || !dz) return FDTD_ERR_NULL;
  if (n < 1) return FDTD_ERR_SIZE;
  FNO_LAUNCH(fdtd::k_gelu_bwd, fdtd::grid1((size_t)n), 256, (size_t)n, (const bf16*)dy16, dy32, (const bf16*)pre,
             (bf16*)dz);
}

int fno_gelu_fwd(long long n, const float* z, void* y, void* pre, fdtd_stream_t stream) {
  if (!z || !y) return FDTD_ERR_NULL;
  if (n < 1) return FDTD_ERR_SIZE;
  FNO_LAUNCH(fdtd::k_gelu_fwd, fdtd::grid1((size_t)n), 256, (size_t)n, z, (bf16*)y, (bf16*)pre);
}

int fno_meanpool(int B, int N, int C, const void* x, void* h, fdtd_stream_t stream) {
  if (!x || !h) return FDTD_ERR_NULL;
  if (B < 1 || N < 1 || C < 1) return FDTD_ERR_SIZE;
  if (C % 8 == 0 && C / 8 <= 256 && ((uintptr_t)x & 15) == 0)
    FNO_LAUNCH(fdtd::k_meanpool8, dim3(B), 256, B, N, C, (const bf16*)x, (bf16*)h);
  FNO_LAUNCH(fdtd::k_meanpool, dim3(B), 128, B, N, C, (const bf16*)x, (bf16*)h);
}

int fno_meanpool_bwd(int B, int N, int C, const float* dh, void* dx, fdtd_stream_t stream) {
  if (!dh || !dx) return FDTD_ERR_NULL;
  if (B < 1 || N < 1 || C < 1) return FDTD_ERR_SIZE;
  FNO_LAUNCH(fdtd::k_meanpool_bwd, fdtd::grid1((size_t)B * N * C), 256, B, N, C, dh, (bf16*)dx);
}

int fno_colsum(long long rows, int C, const void* x16, const float* x32, float* out, fdtd_stream_t stream) {
  if ((!x16 && !x32) || !out) return FDTD_ERR_NULL;
  if (rows < 1 || C < 1) return FDTD_ERR_SIZE;
  FNO_LAUNCH(fdtd::k_colsum, dim3(256, (C + 127) / 128), 128, (size_t)rows, C, (const bf16*)x16, x32, out);
}

int fno_sum_parts(int nb, long long n, const float* parts, float* out, fdtd_stream_t stream) {
  if (!parts || !out) return FDTD_ERR_NULL;
  if (nb < 1 || n < 1) return FDTD_ERR_SIZE;
  FNO_LAUNCH(fdtd::k_sum_parts, fdtd::grid1((size_t)n), 256, nb, (size_t)n, parts, out);
}

int fno_mse(int B, int D, const float* o, const float* y, float* dO, float* loss, fdtd_stream_t stream) {
  if (!o || !y || !dO || !loss) return FDTD_ERR_NULL;
  if (B < 1 || D < 1) return FDTD_ERR_SIZE;
  FNO_LAUNCH(fdtd::k_mse, fdtd::grid1((size_t)B * D), 256, B, D, o, y, dO, loss);
}

int fno_rel_mse(int B, int D, float floor2, const float* o, const float* y, float* dO, float* loss,
                fdtd_stream_t stream) {
  if (!o || !y || !dO || !loss) return FDTD_ERR_NULL;
  if (B < 1 || D < 1 || !(floor2 > 0)) return FDTD_ERR_SIZE;
  FNO_LAUNCH(fdtd::k_rel_mse, dim3(B), 128, B, D, floor2, o, y, dO, loss);
}

int fno_adam(long long n, float* w, const float* g, float* m, float* v, float lr, float b1, float b2, float eps,
             int step, void* w16, fdtd_stream_t stream) {
  if (!w || !g || !m || !v) return FDTD_ERR_NULL;
  if (n < 1 || step < 1) return FDTD_ERR_SIZE;
  const float bc1 = 1.f - powf(b1, (float)step), bc2 = 1.f - powf(b2, (float)step);
  FNO_LAUNCH(fdtd::k_adam, fdtd::grid1((size_t)n), 256, (size_t)n, w, g, m, v, lr, b1, b2, eps, bc1, bc2,
             (bf16*)w16);
}

int fno_to_bf16(long long n, const float* x, void* y, fdtd_stream_t stream) {
  if (!x || !y) return FDTD_ERR_NULL;
  if (n < 1) return FDTD_ERR_SIZE;
  FNO_LAUNCH(fdtd::k_to_bf16, fdtd::grid1((size_t)n), 256, (size_t)n, x, (bf16*)y);
}

}  // extern "C"
