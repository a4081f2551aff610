// BF16 tensor-core GEMM for sm_103a (tcgen05 + TMA + TMEM), FP32 accumulation,
// with a fused epilogue (scale, bias, residual, GELU, accumulate, BF16/FP32
// output).  Written for the neural-operator surrogate's contractions
// (truncated DFT, inverse DFT, channel mixing, pointwise layers and their
// gradients).
//
// 128 x BN output tiles, persistent CTAs of 10 warps:
//   * warp 8, one lane: TMA producer.  Each pipeline stage holds a 128 x 64
//     A tile and a BN x 64 B tile in 128-byte-swizzled shared memory, loaded
//     by cp.async.bulk.tensor with mbarrier completion;
//   * warp 9, one lane: issues tcgen05.mma (kind::f16, BF16 inputs, FP32
//     accumulator in TMEM), four 16-deep MMAs per stage, and tcgen05.commit
//     to release the stage and, per tile, to signal the epilogue;
//   * warps 0-7: read the accumulator with tcgen05.ld (warp w owns TMEM lanes
//     32(w%4)..32(w%4)+31 = output rows, and half w/4 of the columns), return
//     the TMEM buffer, apply the epilogue and store; two accumulator buffers
//     overlap a tile's epilogue with the next tile's MMAs.  Eight epilogue
//     warps (two per SM sub-partition) rather than four: with four, the
//     pointwise layer's GEMM (K = 192) spent most of its time in the
//     epilogue and moved 3.6 TB/s; with eight it moves about 4.7 TB/s, and
//     sixteen (one 32-column chunk each) measured no faster.
// Operands may be K-major or MN-major (the transposed products of the
// backward pass need MN-major), selected per call.  Every wait on an mbarrier
// is bounded (about 2 s): on expiry the kernel records FDTD_STATUS_TIMEOUT in
// the status word and finishes without further waits.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <mutex>

#include "fdtd_common.cuh"

namespace fdtd {
namespace {

constexpr int BM = 128;
constexpr int BK = 64;      // one 128-byte swizzle atom of BF16 along K
constexpr int EPI_WARPS = 8;
constexpr int THREADS = 32 * (EPI_WARPS + 2);

struct GemmArgs {
  int M, N, K, batch;
  int a_mn, b_mn;
  float* c32;
  __nv_bfloat16* c16;
  long long ldc, stride_c;
  const float* bias;
  const __nv_bfloat16* res16;
  long long ldr, stride_r;
  float alpha;
  int act;
  int accumulate;
  __nv_bfloat16* pre16;  // optional pre-activation output (same layout as C)
  unsigned lbo_mn, sbo_mn;
  int a_shared, b_shared;  // operand shared by every batch entry (batch stride 0)
  int vec_ok;              // epilogue pointers/strides allow 16-byte vector access
  // optional second operand pair accumulated into the same tile: D += A2.B2'
  int K2;
  int a2_mn, b2_mn, a2_shared, b2_shared;
  int* status;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint32_t a, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t a, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(a), "r"(bytes) : "memory");
}

// bounded wait on an mbarrier phase; false (and TIMEOUT recorded) on expiry
__device__ __forceinline__ bool mbar_wait(uint32_t a, uint32_t parity, int* status) {
  const long long t0 = clock64();
  for (;;) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    if (ok) return true;
    if (clock64() - t0 > 4000000000LL) {
      raise_status(status, ST_TIMEOUT);
      return false;
    }
  }
}

__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap* tm, int c0, int c1, int c2,
                                            uint32_t mbar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(tm)), "r"(c0), "r"(c1), "r"(c2), "r"(mbar)
      : "memory");
}

// shared-memory matrix descriptor (tcgen05): start address, leading and
// stride byte offsets (16-byte units), descriptor version 1, 128B swizzle
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

// instruction descriptor, kind::f16: BF16 A and B, FP32 accumulator, M x N
__host__ __device__ constexpr uint32_t instr_desc(int m, int n, int a_mn, int b_mn) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)a_mn << 15) | ((uint32_t)b_mn << 16) |
         ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

// GELU, tanh form (Hendrycks & Gimpel 2016): 0.5 z (1 + tanh(sqrt(2/pi) (z + 0.044715 z^3)))
// with the hardware tanh approximation
__device__ __forceinline__ float tanh_hw(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float gelu(float z) {
  const float u = 0.7978845608028654f * fmaf(0.044715f * z, z * z, z);
  return 0.5f * z * (1.0f + tanh_hw(u));
}

// Persistent, warp-specialised kernel: warps 0-7 drain accumulators
// (epilogue), warp 8 is the TMA producer, warp 9 issues the MMAs.  Two TMEM
// accumulator buffers let the epilogue of one tile overlap the MMAs of the
// next; tiles are taken round-robin (tile = blockIdx.x + i * gridDim.x, M tiles
// fastest so neighbouring CTAs share B tiles in L2).
template <int BN, int STAGES>
__global__ void __launch_bounds__(THREADS, 1)
    k_gemm(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
           const __grid_constant__ CUtensorMap tmA2, const __grid_constant__ CUtensorMap tmB2, const GemmArgs a) {
  constexpr uint32_t A_BYTES = BM * BK * 2;
  constexpr uint32_t B_BYTES = BN * BK * 2;
  constexpr uint32_t STAGE_BYTES = A_BYTES + B_BYTES;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* tiles = reinterpret_cast<unsigned char*>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* bars = reinterpret_cast<uint64_t*>(tiles + STAGES * STAGE_BYTES);
  uint64_t* full = bars;
  uint64_t* empty = bars + STAGES;
  uint64_t* tfull = bars + 2 * STAGES;
  uint64_t* tempty = bars + 2 * STAGES + 2;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * STAGES + 4);
  // the bias of a one-column-tile GEMM (N <= BN: the same BN columns for every
  // tile) is staged once, so the epilogue reads it from shared memory
  float* sbias = reinterpret_cast<float*>(bars + 2 * STAGES + 6);  // 16-byte aligned for float4 reads

  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int kb1 = (a.K + BK - 1) / BK;                       // k-blocks of the first pair
  const int kblocks = kb1 + (a.K2 > 0 ? (a.K2 + BK - 1) / BK : 0);
  const int mt = (a.M + BM - 1) / BM;
  const int nt = (a.N + BN - 1) / BN;
  const long long total = (long long)mt * nt * a.batch;
  const bool bias_smem = a.bias != nullptr && nt == 1;
  if (bias_smem)
    for (int c = threadIdx.x; c < BN; c += blockDim.x) sbias[c] = c < a.N ? a.bias[c] : 0.f;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(smem_u32(&full[s]), 1);
      mbar_init(smem_u32(&empty[s]), 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(smem_u32(&tfull[b]), 1);
      mbar_init(smem_u32(&tempty[b]), EPI_WARPS);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(2 * BN)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  if (warp == EPI_WARPS) {
    // ------------------------------------------------ producer
    if (lane == 0) {
      long long g = 0;
      bool ok = true;
      for (long long t = blockIdx.x; t < total && ok; t += gridDim.x) {
        const int bz = (int)(t / ((long long)mt * nt));
        const int rem = (int)(t % ((long long)mt * nt));
        const int m0 = (rem % mt) * BM, n0 = (rem / mt) * BN;
        const int za = a.a_shared ? 0 : bz, zb = a.b_shared ? 0 : bz;
        for (int kb = 0; kb < kblocks; ++kb, ++g) {
          const int s = (int)(g % STAGES);
          if (g >= STAGES && !(ok = mbar_wait(smem_u32(&empty[s]), (uint32_t)(((g / STAGES) - 1) & 1), a.status)))
            break;
          const uint32_t fb = smem_u32(&full[s]);
          mbar_expect_tx(fb, STAGE_BYTES);
          const uint32_t sa = smem_u32(tiles + s * STAGE_BYTES);
          const uint32_t sb = sa + A_BYTES;
          const bool second = kb >= kb1;
          const CUtensorMap* ma = second ? &tmA2 : &tmA;
          const CUtensorMap* mb = second ? &tmB2 : &tmB;
          const int k0 = (second ? kb - kb1 : kb) * BK;
          const int amn = second ? a.a2_mn : a.a_mn, bmn = second ? a.b2_mn : a.b_mn;
          const int za2 = second ? (a.a2_shared ? 0 : bz) : za, zb2 = second ? (a.b2_shared ? 0 : bz) : zb;
          if (!amn) {
            tma_load_3d(sa, ma, k0, m0, za2, fb);
          } else {
            tma_load_3d(sa, ma, m0, k0, za2, fb);
            tma_load_3d(sa + A_BYTES / 2, ma, m0 + 64, k0, za2, fb);
          }
          if (!bmn) {
            tma_load_3d(sb, mb, k0, n0, zb2, fb);
          } else {
#pragma unroll
            for (int h = 0; h < BN / 64; ++h) tma_load_3d(sb + h * (BK * 128), mb, n0 + 64 * h, k0, zb2, fb);
          }
        }
      }
    }
  } else if (warp == EPI_WARPS + 1) {
    // ------------------------------------------------ MMA issuer
    if (lane == 0) {
      const uint32_t idesc1 = instr_desc(BM, BN, a.a_mn, a.b_mn);
      const uint32_t idesc2 = instr_desc(BM, BN, a.a2_mn, a.b2_mn);
      long long g = 0;
      int i = 0;
      bool ok = true;
      for (long long t = blockIdx.x; t < total && ok; t += gridDim.x, ++i) {
        const int b = i & 1;
        if (i >= 2 && !(ok = mbar_wait(smem_u32(&tempty[b]), (uint32_t)(((i >> 1) - 1) & 1), a.status))) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t dacc = tmem + (uint32_t)(b * BN);
        for (int kb = 0; kb < kblocks; ++kb, ++g) {
          const int s = (int)(g % STAGES);
          if (!(ok = mbar_wait(smem_u32(&full[s]), (uint32_t)((g / STAGES) & 1), a.status))) break;
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t sa = smem_u32(tiles + s * STAGE_BYTES);
          const uint32_t sb = sa + A_BYTES;
          const bool second = kb >= kb1;
          const int amn = second ? a.a2_mn : a.a_mn, bmn = second ? a.b2_mn : a.b_mn;
          const uint32_t idesc = second ? idesc2 : idesc1;
#pragma unroll
          for (int kk = 0; kk < BK / 16; ++kk) {
            // K-major: 32 bytes inside the swizzle atom; MN-major: 16 K rows of 128 bytes
            const uint64_t ad =
                amn ? smem_desc(sa + kk * 2048, a.lbo_mn, a.sbo_mn) : smem_desc(sa + kk * 32, 16, 1024);
            const uint64_t bd =
                bmn ? smem_desc(sb + kk * 2048, a.lbo_mn, a.sbo_mn) : smem_desc(sb + kk * 32, 16, 1024);
            const uint32_t acc = (kb > 0 || kk > 0) ? 1u : 0u;
            asm volatile(
                "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(dacc),
                "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
                : "memory");
          }
          asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                           smem_u32(&empty[s]))
                       : "memory");
        }
        if (ok)
          asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                           smem_u32(&tfull[b]))
                       : "memory");
      }
    }
  } else {
    // ------------------------------------------------ epilogue warps 0-7
    const int lg = warp & 3;                       // TMEM lane group = 32 output rows
    const int c_begin = (warp >> 2) * (BN / 2), c_end = c_begin + BN / 2;
    int i = 0;
    for (long long t = blockIdx.x; t < total; t += gridDim.x, ++i) {
      const int bz = (int)(t / ((long long)mt * nt));
      const int rem = (int)(t % ((long long)mt * nt));
      const int m0 = (rem % mt) * BM, n0 = (rem / mt) * BN;
      const int b = i & 1;
      const bool have =
          __all_sync(0xffffffffu, mbar_wait(smem_u32(&tfull[b]), (uint32_t)((i >> 1) & 1), a.status));
      if (!have) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const int row = m0 + lg * 32 + lane;
      const size_t cbase = (size_t)bz * a.stride_c + (size_t)row * a.ldc;
      const size_t rbase = (size_t)bz * a.stride_r + (size_t)row * a.ldr;
#pragma unroll 1
      for (int c0 = c_begin; c0 < c_end; c0 += 32) {
        uint32_t r[32];
        const uint32_t taddr = tmem + ((uint32_t)(lg * 32) << 16) + (uint32_t)(b * BN + c0);
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
            "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
              "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
              "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
              "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
            : "r"(taddr)
            : "memory");
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        if (c0 + 32 >= c_end) {
          // this warp's part of the accumulator has been read: release it
          asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
          __syncwarp();
          if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&tempty[b])) : "memory");
        }
      if (row < a.M && a.vec_ok && n0 + c0 + 32 <= a.N) {
        // 32 consecutive columns of this thread's row: 16-byte vector loads/stores
        const int col0 = n0 + c0;
        float z[32];
  #pragma unroll
        for (int q = 0; q < 32; ++q) z[q] = __uint_as_float(r[q]);
        if (a.alpha != 1.0f) {  // alpha = 1 (every surrogate product): no multiply, the same values
  #pragma unroll
          for (int q = 0; q < 32; ++q) z[q] = __fmul_rn(a.alpha, z[q]);
        }
        if (a.bias) {
          const float* bsrc = bias_smem ? sbias + c0 : a.bias + col0;
  #pragma unroll
          for (int v = 0; v < 8; ++v) {
            const float4 b = *reinterpret_cast<const float4*>(bsrc + 4 * v);
            z[4 * v] = __fadd_rn(z[4 * v], b.x);
            z[4 * v + 1] = __fadd_rn(z[4 * v + 1], b.y);
            z[4 * v + 2] = __fadd_rn(z[4 * v + 2], b.z);
            z[4 * v + 3] = __fadd_rn(z[4 * v + 3], b.w);
          }
        }
        if (a.res16) {
  #pragma unroll
          for (int v = 0; v < 4; ++v) {
            const uint4 u = *reinterpret_cast<const uint4*>(a.res16 + rbase + col0 + 8 * v);
            const uint32_t w[4] = {u.x, u.y, u.z, u.w};
  #pragma unroll
            for (int e = 0; e < 4; ++e) {
              const __nv_bfloat162 h2 = *reinterpret_cast<const __nv_bfloat162*>(&w[e]);
              z[8 * v + 2 * e] = __fadd_rn(z[8 * v + 2 * e], __low2float(h2));
              z[8 * v + 2 * e + 1] = __fadd_rn(z[8 * v + 2 * e + 1], __high2float(h2));
            }
          }
        }
        auto store_bf16 = [&](__nv_bfloat16* dst, const float* v32) {
  #pragma unroll
          for (int v = 0; v < 4; ++v) {
            uint32_t w[4];
  #pragma unroll
            for (int e = 0; e < 4; ++e) {
              const __nv_bfloat162 h2 = __floats2bfloat162_rn(v32[8 * v + 2 * e], v32[8 * v + 2 * e + 1]);
              w[e] = *reinterpret_cast<const uint32_t*>(&h2);
            }
            *reinterpret_cast<uint4*>(dst + 8 * v) = make_uint4(w[0], w[1], w[2], w[3]);
          }
        };
        if (a.pre16) store_bf16(a.pre16 + cbase + col0, z);
        if (a.act == 1) {
  #pragma unroll
          for (int q = 0; q < 32; ++q) z[q] = gelu(z[q]);
        }
        if (a.c32) {
          float* dst = a.c32 + cbase + col0;
  #pragma unroll
          for (int v = 0; v < 8; ++v) {
            float4 o = make_float4(z[4 * v], z[4 * v + 1], z[4 * v + 2], z[4 * v + 3]);
            if (a.accumulate) {
              const float4 c = *reinterpret_cast<const float4*>(dst + 4 * v);
              o.x = __fadd_rn(o.x, c.x);
              o.y = __fadd_rn(o.y, c.y);
              o.z = __fadd_rn(o.z, c.z);
              o.w = __fadd_rn(o.w, c.w);
            }
            *reinterpret_cast<float4*>(dst + 4 * v) = o;
          }
        } else {
          __nv_bfloat16* dst = a.c16 + cbase + col0;
          if (a.accumulate) {
  #pragma unroll
            for (int q = 0; q < 32; ++q) z[q] = __fadd_rn(z[q], __bfloat162float(dst[q]));
          }
          store_bf16(dst, z);
        }
      } else if (row < a.M) {
  #pragma unroll
        for (int q = 0; q < 32; ++q) {
          const int col = n0 + c0 + q;
          if (col < a.N) {
            float z = __fmul_rn(a.alpha, __uint_as_float(r[q]));
            if (a.bias) z = __fadd_rn(z, a.bias[col]);
            if (a.res16) z = __fadd_rn(z, __bfloat162float(a.res16[rbase + col]));
            if (a.pre16) a.pre16[cbase + col] = __float2bfloat16_rn(z);
            float y = a.act == 1 ? gelu(z) : z;
            if (a.c32) {
              if (a.accumulate) y = __fadd_rn(y, a.c32[cbase + col]);
              a.c32[cbase + col] = y;
            } else {
              if (a.accumulate) y = __fadd_rn(y, __bfloat162float(a.c16[cbase + col]));
              a.c16[cbase + col] = __float2bfloat16_rn(y);
            }
          }
        }
      }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * BN) : "memory");
  }
}

// ----------------------------------------------------------------- host
PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
std::mutex g_encode_mu;

int get_encode() {
  std::lock_guard<std::mutex> lk(g_encode_mu);
  if (g_encode) return FDTD_OK;
  void* fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
  if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !fn) {
    fdtd_host::note_cuda_error(e);
    return FDTD_ERR_CUDA;
  }
  g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  return FDTD_OK;
}

// 3D tensor map over a BF16 operand: dims {inner, outer, batch}
int make_map(CUtensorMap* tm, const void* base, uint64_t inner, uint64_t outer, uint64_t batch, uint64_t ld_elems,
             uint64_t stride_elems, uint32_t box_inner, uint32_t box_outer) {
  cuuint64_t dims[3] = {inner, outer, batch};
  cuuint64_t strides[2] = {ld_elems * 2, stride_elems * 2};
  cuuint32_t box[3] = {box_inner, box_outer, 1};
  cuuint32_t es[3] = {1, 1, 1};
  const CUresult r = g_encode(tm, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(base), dims, strides, box,
                              es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? FDTD_OK : FDTD_ERR_ARG;
}

template <int BN, int STAGES>
size_t smem_bytes() {
  return 1024 + (size_t)STAGES * (BM * BK * 2 + BN * BK * 2) + 8 * (2 * STAGES + 6) + sizeof(float) * BN;
}

template <int BN, int STAGES>
int launch_gemm_t(const CUtensorMap& ta, const CUtensorMap& tb, const CUtensorMap& ta2, const CUtensorMap& tb2,
                  const GemmArgs& g, cudaStream_t st) {
  auto kern = k_gemm<BN, STAGES>;
  const size_t smem = smem_bytes<BN, STAGES>();
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) {
    fdtd_host::note_cuda_error(e);
    return FDTD_ERR_CUDA;
  }
  int dev = 0, nsm = 0, occ = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, THREADS, smem);
  if (occ < 1) occ = 1;
  const long long tiles = (long long)((g.M + BM - 1) / BM) * ((g.N + BN - 1) / BN) * g.batch;
  const long long grid = std::min<long long>(tiles, (long long)nsm * occ);
  kern<<<(unsigned)grid, THREADS, smem, st>>>(ta, tb, ta2, tb2, g);
  return fdtd_host::check_launch();
}

}  // namespace
}  // namespace fdtd

extern "C" int fdtd_gemm_bf16(const fdtd_gemm_desc* d, int* status, fdtd_stream_t stream) {
  using namespace fdtd;
  if (!d || !d->A || !d->B) return FDTD_ERR_NULL;
  if (!d->C32 == !d->C16) return FDTD_ERR_ARG;  // exactly one output
  if (d->M < 1 || d->N < 1 || d->K < 1 || d->batch < 1) return FDTD_ERR_SIZE;
  if (d->N > 65535 * 64 || d->batch > 65535) return FDTD_ERR_SIZE;
  auto al16 = [](const void* p) { return ((uintptr_t)p & 15u) == 0; };
  if (!al16(d->A) || !al16(d->B)) return FDTD_ERR_ALIGN;
  if (d->lda % 8 || d->ldb % 8 || (d->batch > 1 && (d->stride_a % 8 || d->stride_b % 8))) return FDTD_ERR_ALIGN;
  if (d->act < 0 || d->act > 1) return FDTD_ERR_ARG;
  if ((d->a_mn_major ? d->lda < d->M : d->lda < d->K) || (d->b_mn_major ? d->ldb < d->N : d->ldb < d->K))
    return FDTD_ERR_SIZE;
  int rc = get_encode();
  if (rc) return rc;
  const int BN = (d->N <= 64) ? 64 : 128;
  CUtensorMap ta, tb;
  // an operand with batch stride 0 is shared: one batch slice in its map
  const bool a_sh = d->batch == 1 || d->stride_a == 0;
  const bool b_sh = d->batch == 1 || d->stride_b == 0;
  const uint64_t sa = a_sh ? (uint64_t)d->lda * (d->a_mn_major ? d->K : d->M) : (uint64_t)d->stride_a;
  const uint64_t sb = b_sh ? (uint64_t)d->ldb * (d->b_mn_major ? d->K : d->N) : (uint64_t)d->stride_b;
  const uint64_t ba = a_sh ? 1 : (uint64_t)d->batch, bb = b_sh ? 1 : (uint64_t)d->batch;
  if (!d->a_mn_major) rc = make_map(&ta, d->A, d->K, d->M, ba, d->lda, sa, BK, BM);
  else rc = make_map(&ta, d->A, d->M, d->K, ba, d->lda, sa, 64, BK);
  if (rc) return rc;
  if (!d->b_mn_major) rc = make_map(&tb, d->B, d->K, d->N, bb, d->ldb, sb, BK, BN);
  else rc = make_map(&tb, d->B, d->N, d->K, bb, d->ldb, sb, 64, BK);
  if (rc) return rc;
  CUtensorMap ta2 = ta, tb2 = tb;
  int a2_sh = 0, b2_sh = 0;
  if (d->K2 > 0) {
    if (!d->A2 || !d->B2) return FDTD_ERR_NULL;
    if (!al16(d->A2) || !al16(d->B2)) return FDTD_ERR_ALIGN;
    if (d->lda2 % 8 || d->ldb2 % 8 || (d->batch > 1 && (d->stride_a2 % 8 || d->stride_b2 % 8))) return FDTD_ERR_ALIGN;
    if ((d->a2_mn_major ? d->lda2 < d->M : d->lda2 < d->K2) || (d->b2_mn_major ? d->ldb2 < d->N : d->ldb2 < d->K2))
      return FDTD_ERR_SIZE;
    a2_sh = (d->batch == 1 || d->stride_a2 == 0);
    b2_sh = (d->batch == 1 || d->stride_b2 == 0);
    const uint64_t sa2 = a2_sh ? (uint64_t)d->lda2 * (d->a2_mn_major ? d->K2 : d->M) : (uint64_t)d->stride_a2;
    const uint64_t sb2 = b2_sh ? (uint64_t)d->ldb2 * (d->b2_mn_major ? d->K2 : d->N) : (uint64_t)d->stride_b2;
    const uint64_t ba2 = a2_sh ? 1 : (uint64_t)d->batch, bb2 = b2_sh ? 1 : (uint64_t)d->batch;
    if (!d->a2_mn_major) rc = make_map(&ta2, d->A2, d->K2, d->M, ba2, d->lda2, sa2, BK, BM);
    else rc = make_map(&ta2, d->A2, d->M, d->K2, ba2, d->lda2, sa2, 64, BK);
    if (rc) return rc;
    if (!d->b2_mn_major) rc = make_map(&tb2, d->B2, d->K2, d->N, bb2, d->ldb2, sb2, BK, BN);
    else rc = make_map(&tb2, d->B2, d->N, d->K2, bb2, d->ldb2, sb2, 64, BK);
    if (rc) return rc;
  }
  GemmArgs g{};
  g.K2 = d->K2 > 0 ? d->K2 : 0;
  g.a2_mn = d->a2_mn_major;
  g.b2_mn = d->b2_mn_major;
  g.a2_shared = a2_sh;
  g.b2_shared = b2_sh;
  g.M = d->M;
  g.N = d->N;
  g.K = d->K;
  g.batch = d->batch;
  g.a_mn = d->a_mn_major;
  g.b_mn = d->b_mn_major;
  g.c32 = d->C32;
  g.c16 = reinterpret_cast<__nv_bfloat16*>(d->C16);
  g.ldc = d->ldc;
  g.stride_c = d->stride_c;
  g.bias = d->bias;
  g.res16 = reinterpret_cast<const __nv_bfloat16*>(d->res16);
  g.ldr = d->ldr;
  g.stride_r = d->stride_r;
  g.alpha = d->alpha;
  g.act = d->act;
  g.accumulate = d->accumulate;
  g.pre16 = reinterpret_cast<__nv_bfloat16*>(d->pre16);
  g.lbo_mn = d->mn_lbo ? (unsigned)d->mn_lbo : (unsigned)(BK * 128);
  g.sbo_mn = d->mn_sbo ? (unsigned)d->mn_sbo : 1024u;
  {
    const void* cptr = d->C32 ? (const void*)d->C32 : d->C16;
    bool v = al16(cptr) && d->ldc % 8 == 0 && d->stride_c % 8 == 0;
    if (d->bias) v = v && al16(d->bias);
    if (d->res16) v = v && al16(d->res16) && d->ldr % 8 == 0 && d->stride_r % 8 == 0;
    if (d->pre16) v = v && al16(d->pre16);
    g.vec_ok = v ? 1 : 0;
  }
  g.a_shared = a_sh ? 1 : 0;
  g.b_shared = b_sh ? 1 : 0;
  g.status = status;
  // 4 pipeline stages throughout: with 2, a product of only one or two
  // k-blocks per tile (K = 16 + 64 in the folded first layer) cannot load the
  // next tile while the current one computes (1.6 ms instead of 0.9 at 4096)
  cudaStream_t st = (cudaStream_t)stream;
  if (BN == 64) return launch_gemm_t<64, 4>(ta, tb, ta2, tb2, g, st);
  return launch_gemm_t<128, 4>(ta, tb, ta2, tb2, g, st);
}
