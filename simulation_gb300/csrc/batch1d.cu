// Batched uneven 1D runs (thousands of independent lossy-slab simulations in
// one persistent launch), with the running-DFT probes fused in.
//
// Each run is the ca/cb lossy 1D program of fd1d/program/fd1d_1_5.py:63-72
// (E update, soft Gaussian source, two-step-back ABC, H update) with per-run
// layered coefficients and two DFT probes accumulated as in
// fd1d/program/fd1d_2_2.py:65-71 (after E, before the ABC).  The reference has
// no batched form; this is the library's extension for spectra sweeps.
//
// Execution model:
//   * a run is executed by a TEAM of warps inside a thread block: each thread
//     holds CPT consecutive cells (ex, hy) in registers; warp shuffles carry
//     the neighbour values inside a warp and a few shared-memory slots carry
//     them across warps; two team barriers per time step (a named barrier
//     `bar.sync id, n` for multi-warp teams, __syncwarp for one-warp teams);
//   * the per-cell (ca, cb) pairs are expanded from the run's layer table into
//     shared memory once per run;
//   * the host planner (fdtd1d_batch_plan, C++ below) sizes each team as
//     ceil(ke / CPT) rounded up to whole warps, so every run costs about the
//     same per step, and packs teams into "bundles" that fill a block
//     (first-fit decreasing, <= 15 multi-warp teams per block);
//   * persistent blocks take bundles from a device counter (atomicAdd); there
//     is no spin-wait anywhere.  An optional clock budget stops a block from
//     taking new bundles and raises FDTD_STATUS_TIMEOUT; per-run `done` flags
//     say which runs finished.
#include <algorithm>
#include <cstring>
#include <numeric>
#include <vector>

#include "fdtd_common.cuh"

namespace fdtd {

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int MAX_WARPS = 32;
constexpr int ENTRY_INTS = 4;  // run, threads, thread offset, barrier id (0 = single warp)

struct BatchArgs {
  fdtd1d_batch_params p;
  fdtd1d_batch_out o;
  const int* plan;  // device copy of the plan
  int nbundles;
  const int* bstart;  // [nbundles+1] entry offsets (into plan)
  const int* entries;
  long long max_cycles;
};

__device__ __forceinline__ void team_sync(int bar_id, int nthreads) {
  if (bar_id == 0) {
    __syncwarp();
  } else {
    asm volatile("bar.sync %0, %1;" ::"r"(bar_id), "r"(nthreads) : "memory");
  }
}

// a[c] for a runtime c: a switch (an indexed branch taken by the calling
// lane), not a compare-and-select per cell; callers keep it to one thread
#define FDTD_CELL_CASE(k)        \
  case k:                        \
    if constexpr (k < CPT) body(a[k < CPT ? k : 0]); \
    break;
template <int CPT, class A, class F>
__device__ __forceinline__ void cell_at(A& a, int c, F&& body) {
  static_assert(CPT <= 64, "cells per thread");
  switch (c) { FDTD_CELL_CASE(0) FDTD_CELL_CASE(1) FDTD_CELL_CASE(2) FDTD_CELL_CASE(3) FDTD_CELL_CASE(4) FDTD_CELL_CASE(5) FDTD_CELL_CASE(6) FDTD_CELL_CASE(7) FDTD_CELL_CASE(8) FDTD_CELL_CASE(9) FDTD_CELL_CASE(10) FDTD_CELL_CASE(11) FDTD_CELL_CASE(12) FDTD_CELL_CASE(13) FDTD_CELL_CASE(14) FDTD_CELL_CASE(15) FDTD_CELL_CASE(16) FDTD_CELL_CASE(17) FDTD_CELL_CASE(18) FDTD_CELL_CASE(19) FDTD_CELL_CASE(20) FDTD_CELL_CASE(21) FDTD_CELL_CASE(22) FDTD_CELL_CASE(23) FDTD_CELL_CASE(24) FDTD_CELL_CASE(25) FDTD_CELL_CASE(26) FDTD_CELL_CASE(27) FDTD_CELL_CASE(28) FDTD_CELL_CASE(29) FDTD_CELL_CASE(30) FDTD_CELL_CASE(31) FDTD_CELL_CASE(32) FDTD_CELL_CASE(33) FDTD_CELL_CASE(34) FDTD_CELL_CASE(35) FDTD_CELL_CASE(36) FDTD_CELL_CASE(37) FDTD_CELL_CASE(38) FDTD_CELL_CASE(39) FDTD_CELL_CASE(40) FDTD_CELL_CASE(41) FDTD_CELL_CASE(42) FDTD_CELL_CASE(43) FDTD_CELL_CASE(44) FDTD_CELL_CASE(45) FDTD_CELL_CASE(46) FDTD_CELL_CASE(47) FDTD_CELL_CASE(48) FDTD_CELL_CASE(49) FDTD_CELL_CASE(50) FDTD_CELL_CASE(51) FDTD_CELL_CASE(52) FDTD_CELL_CASE(53) FDTD_CELL_CASE(54) FDTD_CELL_CASE(55) FDTD_CELL_CASE(56) FDTD_CELL_CASE(57) FDTD_CELL_CASE(58) FDTD_CELL_CASE(59) FDTD_CELL_CASE(60) FDTD_CELL_CASE(61) FDTD_CELL_CASE(62) FDTD_CELL_CASE(63) }
}
#undef FDTD_CELL_CASE
template <int CPT>
__device__ __forceinline__ float cell_get(const float (&a)[CPT], int c) {
  float r = 0.f;
  cell_at<CPT>(a, c, [&](const float& x) { r = x; });
  return r;
}
template <int CPT>
__device__ __forceinline__ void cell_set(float (&a)[CPT], int c, float v) {
  cell_at<CPT>(a, c, [&](float& x) { x = v; });
}

template <int CPT>
__device__ void run_team(const BatchArgs& A, int run, int T, int tt, int bar_id, int warp_base, float2* coef,
                         float* x_last_hy, float* x_first_ex, float* x_last_ex, float* x_probe, float* acc) {
  const fdtd1d_batch_params& p = A.p;
  const int lane = threadIdx.x & 31;
  const int w = tt >> 5;              // warp index inside the team
  const int nw = T >> 5;
  const int nx = p.ke[run];

  // expand the layer table: background ca=1, cb=0.5 (free space of fd1d_1_5);
  // cells past the run's end get ca=cb=0, which keeps them exactly 0, so the
  // cell loops below need no range test (their H update adds 0.5*(0-0)).
  // Cell c of thread (warp w, lane l) is stored at coef[(w*CPT + c)*32 + l]:
  // the warp's read of its c-th cells touches 32 consecutive float2 (a
  // thread-major layout puts lanes CPT*8 bytes apart: 8-way bank conflicts),
  // and each thread reads at constant offsets c*256 bytes from its own base.
  const int l0 = p.layer_off[run], l1 = p.layer_off[run + 1];
  for (int i = tt; i < T * CPT; i += T) {
    float ca = i < nx ? 1.f : 0.f, cb = i < nx ? 0.5f : 0.f;
    for (int l = l0; l < l1; ++l)
      if (i >= p.layer_start[l] && i < p.layer_end[l]) {
        ca = p.layer_ca[l];
        cb = p.layer_cb[l];
      }
    const int th = i / CPT, c = i - th * CPT;
    coef[((th >> 5) * CPT + c) * 32 + (th & 31)] = make_float2(ca, cb);
  }
  const float2* my_coef = coef + (size_t)w * CPT * 32 + lane;
  const int pin = p.probe_in[run], pout = p.probe_out[run];
  const int nf = p.nf;
  // DFT accumulators of the team in shared memory: acc[4][nf] (re/im at the
  // entry probe, re/im at the exit probe); thread tt owns frequencies tt, tt+T
  for (int f = tt; f < 4 * nf; f += T) acc[f] = 0.f;

  float ex[CPT], hy[CPT];
#pragma unroll
  for (int c = 0; c < CPT; ++c) ex[c] = hy[c] = 0.f;
  const bool own_lo = (tt == 0);
  const int hi_thr = (nx - 1) / CPT;
  const int hi_c = (nx - 1) - hi_thr * CPT;
  const bool own_hi = (tt == hi_thr);
  // the threads (and their cells) holding the source and the two probes
  const bool own_src = tt == p.src_k / CPT, own_pin = tt == pin / CPT, own_pout = tt == pout / CPT;
  const int src_c = p.src_k % CPT, pin_c = pin % CPT, pout_c = pout % CPT;
  float bc0 = 0.f, bc1 = 0.f, bc2 = 0.f, bc3 = 0.f;
  if (lane == 31) x_last_hy[warp_base + w] = 0.f;
  team_sync(bar_id, T);

  for (int t = 1; t <= p.nsteps; ++t) {
    // DFT factors of this step, loaded early (consumed after barrier A)
    float cf[2], sf[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      const int f = tt + k * T;
      cf[k] = (f < nf) ? __ldg(p.dft_cos + (size_t)(t - 1) * nf + f) : 0.f;
      sf[k] = (f < nf) ? __ldg(p.dft_sin + (size_t)(t - 1) * nf + f) : 0.f;
    }
    const float v = __ldg(p.src_table + t - 1);
    // ---------------- E stage: ex = ca*ex + cb*(hy[i-1]-hy[i])
    float hy_left = __shfl_up_sync(FULL, hy[CPT - 1], 1);
    if (lane == 0) hy_left = (w > 0) ? x_last_hy[warp_base + w - 1] : 0.f;
    const float ex0 = ex[0];
#pragma unroll
    for (int c = 0; c < CPT; ++c) {
      const float hym = (c == 0) ? hy_left : hy[c - 1];
      const float2 k = my_coef[c * 32];
      ex[c] = ex_update_cacb(ex[c], hym, hy[c], k.x, k.y);
    }
    if (own_lo) ex[0] = ex0;  // cell 0 is not E-updated
    // soft source, fd1d/program/fd1d_1_5.py:67, then the probes read their cells
    if (own_src) cell_set<CPT>(ex, src_c, __fadd_rn(cell_get<CPT>(ex, src_c), v));
    if (own_pin) x_probe[0] = cell_get<CPT>(ex, pin_c);
    if (own_pout) x_probe[1] = cell_get<CPT>(ex, pout_c);
    // ABC (fd1d/program/fd1d_1_2.py:47-48): low side here, high side's
    // ex[nx-1] here and its state shift after barrier A
    if (own_lo) {
      const float e1 = ex[1];
      ex[0] = bc0;
      bc0 = bc1;
      bc1 = e1;
    }
    if (own_hi) cell_set<CPT>(ex, hi_c, bc3);
    const float prev_last_ex = __shfl_up_sync(FULL, ex[CPT - 1], 1);
    if (lane == 0) x_first_ex[warp_base + w] = ex[0];
    if (lane == 31) x_last_ex[warp_base + w] = ex[CPT - 1];
    team_sync(bar_id, T);  // barrier A

    // ---------------- DFT probes, ABC high-side state, H stage
    {
      const float ein = x_probe[0], eout = x_probe[1];
#pragma unroll
      for (int k = 0; k < 2; ++k) {
        const int f = tt + k * T;
        if (f < nf) {
          acc[0 * nf + f] = __fmaf_rn(cf[k], ein, acc[0 * nf + f]);
          acc[1 * nf + f] = __fmaf_rn(-sf[k], ein, acc[1 * nf + f]);
          acc[2 * nf + f] = __fmaf_rn(cf[k], eout, acc[2 * nf + f]);
          acc[3 * nf + f] = __fmaf_rn(-sf[k], eout, acc[3 * nf + f]);
        }
      }
    }
    float hy_hi = 0.f;  // hy[nx-1] is never updated: kept across the unmasked H loop
    if (own_hi) {
      const float e_nm2 = hi_c >= 1 ? cell_get<CPT>(ex, hi_c - 1)
                                    : ((lane > 0) ? prev_last_ex : x_last_ex[warp_base + w - 1]);
      bc3 = bc2;
      bc2 = e_nm2;
      hy_hi = cell_get<CPT>(hy, hi_c);
    }
    float ex_right = __shfl_down_sync(FULL, ex[0], 1);
    if (lane == 31) ex_right = (w + 1 < nw) ? x_first_ex[warp_base + w + 1] : 0.f;
#pragma unroll
    for (int c = 0; c < CPT; ++c) hy[c] = hy_update(hy[c], ex[c], (c == CPT - 1) ? ex_right : ex[c + 1]);
    if (own_hi) cell_set<CPT>(hy, hi_c, hy_hi);
    if (lane == 31) x_last_hy[warp_base + w] = hy[CPT - 1];
    team_sync(bar_id, T);  // barrier B
  }
  bool fin = true;
  float* sp = A.o.spec + (size_t)run * 4 * nf;
  for (int f = tt; f < 4 * nf; f += T) {
    sp[f] = acc[f];
    fin &= isfinite(acc[f]);
  }
  if (!fin) raise_status(A.o.status, ST_NONFINITE);
  if (tt == 0 && A.o.done) A.o.done[run] = 1;
}

template <int CPT, int BLOCK>
__global__ void __launch_bounds__(BLOCK, 1) k_batch(const BatchArgs A) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* coef = reinterpret_cast<float2*>(smem_raw);  // [blockDim * CPT]
  float* x = reinterpret_cast<float*>(coef + (size_t)blockDim.x * CPT);
  float* x_last_hy = x;                    // [MAX_WARPS]
  float* x_first_ex = x + MAX_WARPS;       // [MAX_WARPS]
  float* x_last_ex = x + 2 * MAX_WARPS;    // [MAX_WARPS]
  float* x_probe = x + 3 * MAX_WARPS;      // [MAX_WARPS][2] (per team, indexed by its first warp)
  float* x_acc = x + 5 * MAX_WARPS;        // [MAX_WARPS][4*64] DFT accumulators (per team)
  __shared__ int s_bundle;
  const long long t_start = clock64();
  for (;;) {
    if (threadIdx.x == 0) {
      int b = -1;
      if (A.max_cycles > 0 && clock64() - t_start > A.max_cycles) {
        // budget spent: take nothing more; report if work was left
        if (*(volatile unsigned*)A.o.queue < (unsigned)A.nbundles) raise_status(A.o.status, ST_TIMEOUT);
      } else {
        b = (int)atomicAdd(A.o.queue, 1u);
      }
      s_bundle = b;
    }
    __syncthreads();
    const int b = s_bundle;
    if (b < 0 || b >= A.nbundles) break;
    for (int e = A.bstart[b]; e < A.bstart[b + 1]; ++e) {
      const int* en = A.entries + (size_t)e * ENTRY_INTS;
      const int off = en[2], T = en[1];
      if ((int)threadIdx.x >= off && (int)threadIdx.x < off + T) {
        run_team<CPT>(A, en[0], T, threadIdx.x - off, en[3], off >> 5, coef + (size_t)off * CPT, x_last_hy,
                      x_first_ex, x_last_ex, x_probe + 2 * (off >> 5), x_acc + (size_t)256 * (off >> 5));
      }
    }
    __syncthreads();
  }
}

}  // namespace

// smem bytes of one block
static size_t batch_smem(int threads, int cpt) {
  return (size_t)threads * cpt * sizeof(float2) + (size_t)MAX_WARPS * (5 + 256) * sizeof(float);
}

template <int CPT, int BLOCK>
static int launch_batch_t(const BatchArgs& A, int threads, int ctas_per_sm, cudaStream_t st) {
  if (threads > BLOCK) return FDTD_ERR_ARG;
  auto kern = k_batch<CPT, BLOCK>;
  const size_t smem = batch_smem(threads, CPT);
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) {
    fdtd_host::note_cuda_error(e);
    return FDTD_ERR_CUDA;
  }
  int dev = 0, nsm = 0, occ = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, threads, smem);
  if (occ < 1) return FDTD_ERR_UNSUPPORTED;
  if (ctas_per_sm > 0) occ = std::min(occ, ctas_per_sm);
  const int grid = std::max(1, std::min(nsm * occ, A.nbundles));
  kern<<<grid, threads, smem, st>>>(A);
  return fdtd_host::check_launch();
}

}  // namespace fdtd

// ======================================================================= C-ABI
extern "C" {

int fdtd1d_batch_plan(const int* ke_host, int nruns, int cells_per_thread, int block_threads, int* plan,
                      size_t plan_ints, int* plan_len) {
  using fdtd::ENTRY_INTS;
  if (!ke_host || !plan_len) return FDTD_ERR_NULL;
  if (nruns <= 0) return FDTD_ERR_SIZE;
  if (cells_per_thread <= 1 || block_threads < 32 || block_threads > 1024 || block_threads % 32) return FDTD_ERR_ARG;
  std::vector<int> team(nruns);
  for (int r = 0; r < nruns; ++r) {
    if (ke_host[r] < 4) return FDTD_ERR_SIZE;
    const int thr = (ke_host[r] + cells_per_thread - 1) / cells_per_thread;
    team[r] = ((thr + 31) / 32) * 32;
    if (team[r] > block_threads) return FDTD_ERR_SIZE;
  }
  // first-fit decreasing by team size into blocks of block_threads threads,
  // at most 15 multi-warp teams (named barriers 1..15) per block
  std::vector<int> order(nruns);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return team[a] > team[b]; });
  struct Bin {
    int used = 0, named = 0;
    std::vector<int> runs;
  };
  std::vector<Bin> bins;
  for (int r : order) {
    const bool multi = team[r] > 32;
    bool placed = false;
    for (Bin& b : bins) {
      if (b.used + team[r] <= block_threads && (!multi || b.named < 15)) {
        b.runs.push_back(r);
        b.used += team[r];
        b.named += multi;
        placed = true;
        break;
      }
    }
    if (!placed) {
      Bin b;
      b.runs.push_back(r);
      b.used = team[r];
      b.named = multi;
      bins.push_back(b);
    }
  }
  const int nb = (int)bins.size();
  // layout: [0] nbundles, [1] cells_per_thread, [2] block_threads, [3] reserved,
  //         [4 .. 4+nb] bundle start (entry index), then entries (ENTRY_INTS each)
  const size_t need = 4 + (size_t)(nb + 1) + (size_t)nruns * ENTRY_INTS;
  *plan_len = (int)need;
  if (!plan) return FDTD_OK;  // size query
  if (plan_ints < need) return FDTD_ERR_WORKSPACE;
  plan[0] = nb;
  plan[1] = cells_per_thread;
  plan[2] = block_threads;
  plan[3] = 0;
  int* bstart = plan + 4;
  int* ent = plan + 4 + nb + 1;
  int e = 0;
  for (int b = 0; b < nb; ++b) {
    bstart[b] = e;
    int off = 0, bar = 1;
    for (int r : bins[b].runs) {
      ent[e * ENTRY_INTS + 0] = r;
      ent[e * ENTRY_INTS + 1] = team[r];
      ent[e * ENTRY_INTS + 2] = off;
      ent[e * ENTRY_INTS + 3] = team[r] > 32 ? bar++ : 0;
      off += team[r];
      ++e;
    }
  }
  bstart[nb] = e;
  return FDTD_OK;
}

int fdtd1d_batch_run(const fdtd1d_batch_params* p, fdtd1d_batch_out* o, const int* plan_device, int plan_len,
                     int nbundles, int cells_per_thread, int block_threads, int ctas_per_sm, long long max_cycles,
                     fdtd_stream_t stream) {
  if (!p || !o || !plan_device) return FDTD_ERR_NULL;
  if (p->nruns <= 0 || p->nsteps < 0 || nbundles <= 0 || plan_len < 4 + nbundles + 1) return FDTD_ERR_SIZE;
  if (!p->ke || !p->layer_off || !p->probe_in || !p->probe_out || !p->src_table || !o->spec || !o->queue)
    return FDTD_ERR_NULL;
  if (p->nf < 1 || p->nf > 64 || !p->dft_cos || !p->dft_sin) return FDTD_ERR_SIZE;
  if (p->nlayers > 0 && (!p->layer_start || !p->layer_end || !p->layer_ca || !p->layer_cb)) return FDTD_ERR_NULL;
  if (p->src_k < 1) return FDTD_ERR_ARG;
  if (block_threads < 32 || block_threads > 1024 || block_threads % 32) return FDTD_ERR_ARG;
  if (p->nsteps == 0) return FDTD_OK;
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = cudaMemsetAsync(o->queue, 0, sizeof(unsigned), st);
  if (e != cudaSuccess) {
    fdtd_host::note_cuda_error(e);
    return FDTD_ERR_CUDA;
  }
  // done[] is not cleared here: a plan may cover only some of the runs (one
  // call per tuning group), and clearing all nruns flags would erase the
  // flags an earlier group's launch set.  The caller zeroes done[] once.
  fdtd::BatchArgs A{};
  A.p = *p;
  A.o = *o;
  A.plan = plan_device;
  A.nbundles = nbundles;
  A.bstart = plan_device + 4;
  A.entries = plan_device + 4 + nbundles + 1;
  A.max_cycles = max_cycles;
  // cells per thread and the largest block each supports (register budget:
  // 64 per thread for 1024-thread blocks, 128 for 512)
  switch (cells_per_thread) {
    case 8: return fdtd::launch_batch_t<8, 1024>(A, block_threads, ctas_per_sm, st);
    case 16: return fdtd::launch_batch_t<16, 1024>(A, block_threads, ctas_per_sm, st);
    case 24: return fdtd::launch_batch_t<24, 512>(A, block_threads, ctas_per_sm, st);
    case 32: return fdtd::launch_batch_t<32, 512>(A, block_threads, ctas_per_sm, st);
    case 40: return fdtd::launch_batch_t<40, 512>(A, block_threads, ctas_per_sm, st);
    default: return FDTD_ERR_ARG;
  }
}

}  // extern "C"
