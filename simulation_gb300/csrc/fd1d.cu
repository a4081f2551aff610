// 1D Ex/Hy FDTD (fd1d): per-function kernels and the fused single-run kernel.
//
// Per-function kernels (fdtd1d_efield / fdtd1d_hfield / fdtd1d_fourier) update
// the caller's arrays in place with one launch per reference function.
//
// The fused kernel (fdtd1d_step_n) runs a whole time loop in ONE launch: one
// thread-block cluster holds the line, each thread CPT consecutive cells in
// registers (lines of up to 512 cells run in one warp instead, fd1d_warp.cuh).  Per time step it needs exactly two cluster-wide barriers:
//   E stage  : ex (or dx -> ex) from hy, with the left neighbour's last hy
//              read from shared memory (same block) or through distributed
//              shared memory (previous block of the cluster); then the source,
//              the running DFT (before the ABC, as fourier() precedes hyfield()
//              in fd1d/program/fd1d_2_2.py:138-142) and the low-side ABC;
//   barrier A: publishes each thread's first/last ex;
//   H stage  : the high-side ABC state update, then hy from ex with the right
//              neighbour's first ex;
//   barrier B: publishes each thread's last hy.
// This keeps the reference's serial order E -> source -> ABC -> H exactly; the
// reference's own CUDA kernels race on ex[1] and ex[nx-1]
// (fd1d/cuda/fd1d_1_3.cu:25-28, :35-39).
#include <cooperative_groups.h>

#include <algorithm>

#include "fd1d_warp.cuh"
#include "fdtd_common.cuh"

namespace cg = cooperative_groups;

namespace fdtd {

// ============================================================ per-function
// E stage, one thread per cell (fd1d/program/fd1d_1_3.py:55-57,
// fd1d/program/fd1d_1_5.py:65-67, fd1d/program/fd1d_2_2.py:74-84)
template <int FORM>
__global__ void k_fd1d_efield(fdtd1d_params p, fdtd1d_state s, int t) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < 1 || i >= p.nx) return;
  const float v = (p.src_kind != FDTD_SRC_NONE && i == p.src_k) ? p.src_table[t - 1] : 0.f;
  if (FORM == FDTD1D_FORM_CB || FORM == FDTD1D_FORM_CACB) {
    float e = (FORM == FDTD1D_FORM_CB) ? ex_update_cb(s.ex[i], s.hy[i - 1], s.hy[i], p.cb[i])
                                        : ex_update_cacb(s.ex[i], s.hy[i - 1], s.hy[i], p.ca[i], p.cb[i]);
    if (p.src_kind != FDTD_SRC_NONE && i == p.src_k) e = (p.src_kind == FDTD_SRC_HARD) ? v : __fadd_rn(e, v);
    s.ex[i] = e;
  } else {
    float d = dx_update(s.dx[i], s.hy[i - 1], s.hy[i]);
    if (p.src_kind != FDTD_SRC_NONE && i == p.src_k) d = (p.src_kind == FDTD_SRC_HARD) ? v : __fadd_rn(d, v);
    s.dx[i] = d;
    float ixv = s.ix[i];
    if (FORM == FDTD1D_FORM_DFORM) {
      s.ex[i] = ex_from_dx(d, ixv, p.nax[i], p.nbx[i]);
    } else {
      float sxv = s.sx[i];
      s.ex[i] = ex_from_dx_debye(d, ixv, sxv, p.nax[i], p.nbx[i], p.ncx[i], p.ndx[i]);
      s.sx[i] = sxv;
    }
    s.ix[i] = ixv;
  }
}

// source at cell 0 (never updated by the E loop, which starts at 1)
__global__ void k_fd1d_src0(fdtd1d_params p, fdtd1d_state s, int t) {
  const float v = p.src_table[t - 1];
  float* f = (p.form == FDTD1D_FORM_CB || p.form == FDTD1D_FORM_CACB) ? s.ex : s.dx;
  f[0] = (p.src_kind == FDTD_SRC_HARD) ? v : __fadd_rn(f[0], v);
  if (p.form >= FDTD1D_FORM_DFORM) {
    // ex[0] is not recomputed from dx[0] by the reference (exfield covers 1..nx-1)
  }
}

// ABC then H (fd1d/program/fd1d_2_2.py:87-92).  Thread 0 owns the low-side
// ABC and hy[0]; the thread of cell nx-2 owns the high-side ABC and hy[nx-2],
// so each boundary value is set before the only H update that reads it.
__global__ void k_fd1d_hfield(fdtd1d_params p, fdtd1d_state s) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int nx = p.nx;
  if (i > nx - 2) return;
  float e0, e1;
  if (p.abc && i == 0) {
    const float b0 = s.bc[0], b1 = s.bc[1];
    e1 = s.ex[1];
    s.ex[0] = b0;
    s.bc[0] = b1;
    s.bc[1] = e1;
    e0 = b0;
  } else {
    e0 = s.ex[i];
    e1 = s.ex[i + 1];
  }
  if (p.abc && i == nx - 2) {
    const float b2 = s.bc[2], b3 = s.bc[3];
    // ex[nx-2] (e0, nx >= 4 so i > 0) is final for this step; ex[nx-1] becomes bc[3]
    s.ex[nx - 1] = b3;
    s.bc[3] = b2;
    s.bc[2] = e0;
    e1 = b3;
  }
  s.hy[i] = hy_update(s.hy[i], e0, e1);
}

// running DFT (fd1d/program/fd1d_2_2.py:65-71): probes and, optionally, every cell
__global__ void k_fd1d_fourier(fdtd1d_params p, fdtd1d_state s, int t) {
  const float* cs = p.dft_cos + (size_t)(t - 1) * p.nf;
  const float* sn = p.dft_sin + (size_t)(t - 1) * p.nf;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (p.full_dft && i < p.nx) {
    const float e = s.ex[i];
    for (int f = 0; f < p.nf; ++f) {
      const size_t m = (size_t)f * p.nx + i;
      s.r_pt[m] = __fmaf_rn(cs[f], e, s.r_pt[m]);
      s.i_pt[m] = __fmaf_rn(-sn[f], e, s.i_pt[m]);
    }
  }
  if (i < p.nf) {
    for (int q = 0; q < p.nprobe; ++q) {
      const float e = s.ex[p.probe_k[q]];
      const size_t m = (size_t)q * p.nf + i;
      s.r_pr[m] = __fmaf_rn(cs[i], e, s.r_pr[m]);
      s.i_pr[m] = __fmaf_rn(-sn[i], e, s.i_pr[m]);
    }
  }
}

// ============================================================ fused run
struct Run1DArgs {
  fdtd1d_params p;
  fdtd1d_state s;
  int t0, nsteps;
};

constexpr int RUN1D_MAX_THREADS = 1024;
// block size limit per cells-per-thread, so the register budget grows with CPT
__host__ __device__ constexpr int run1d_max_threads(int cpt) { return cpt <= 8 ? 1024 : 512; }

template <int FORM, int CPT, bool CLUSTER>
__global__ void __launch_bounds__(run1d_max_threads(CPT)) k_fd1d_run(const Run1DArgs a) {
  const fdtd1d_params& p = a.p;
  const fdtd1d_state& s = a.s;
  __shared__ float x_first_ex[RUN1D_MAX_THREADS];
  __shared__ float x_last_ex[RUN1D_MAX_THREADS];
  __shared__ float x_last_hy[RUN1D_MAX_THREADS];
  __shared__ float x_probe[FDTD1D_MAX_PROBES];

  const int tid = threadIdx.x;
  const int T = blockDim.x;
  int rank = 0, C = 1;
  if (CLUSTER) {
    cg::cluster_group cl = cg::this_cluster();
    rank = (int)cl.block_rank();
    C = (int)cl.num_blocks();
  }
  auto sync_all = [&]() {
    if (CLUSTER) cg::this_cluster().sync();
    else __syncthreads();
  };
  const int lane = tid & 31, w = tid >> 5, nw = T >> 5;
  auto remote = [&](float* base, int r, int idx) -> float {
    if (CLUSTER) {
      float* rp = cg::this_cluster().map_shared_rank(base, r);
      return rp[idx];
    }
    return 0.f;
  };

  const int nx = p.nx;
  const int gthr = rank * T + tid;
  const int g0 = gthr * CPT;
  constexpr bool DF = (FORM == FDTD1D_FORM_DFORM || FORM == FDTD1D_FORM_DEBYE);

  float ex[CPT], hy[CPT], dx[CPT], ixa[CPT], sxa[CPT];
#pragma unroll
  for (int c = 0; c < CPT; ++c) {
    const int g = g0 + c;
    const bool in = g < nx;
    ex[c] = in ? s.ex[g] : 0.f;
    hy[c] = in ? s.hy[g] : 0.f;
    dx[c] = (DF && in) ? s.dx[g] : 0.f;
    ixa[c] = (DF && in) ? s.ix[g] : 0.f;
    sxa[c] = (FORM == FDTD1D_FORM_DEBYE && in) ? s.sx[g] : 0.f;
  }
  // per-cell coefficients: in registers for the whole run when the register
  // budget allows (few cells per thread), else read from L1 each step
  constexpr bool KREG = CPT <= 4;
  float k0[CPT], k1[CPT], k2[CPT], k3[CPT];
#pragma unroll
  for (int c = 0; c < CPT; ++c) {
    const int g = g0 + c;
    const bool in = g >= 1 && g < nx;
    k0[c] = k1[c] = k2[c] = k3[c] = 0.f;
    if (KREG && in) {
      if (FORM == FDTD1D_FORM_CB) k0[c] = __ldg(p.cb + g);
      if (FORM == FDTD1D_FORM_CACB) {
        k0[c] = __ldg(p.ca + g);
        k1[c] = __ldg(p.cb + g);
      }
      if (DF) {
        k0[c] = __ldg(p.nax + g);
        k1[c] = __ldg(p.nbx + g);
      }
      if (FORM == FDTD1D_FORM_DEBYE) {
        k2[c] = __ldg(p.ncx + g);
        k3[c] = __ldg(p.ndx + g);
      }
    }
  }
  // the source value of the next step is fetched one step ahead
  const bool have_src = p.src_kind != FDTD_SRC_NONE;
  const bool src_here = have_src && p.src_k >= g0 && p.src_k < g0 + CPT;
  float v_next = (src_here && a.nsteps > 0) ? __ldg(p.src_table + a.t0) : 0.f;
  // ABC owners: gthr 0 (cells 0,1 since CPT >= 2) and the thread of cell nx-1
  const bool own_lo = p.abc && gthr == 0;
  const int hi_thr = (nx - 1) / CPT;
  const int hi_c = (nx - 1) - hi_thr * CPT;
  const bool own_hi = p.abc && gthr == hi_thr;
  float bc0 = 0.f, bc1 = 0.f, bc2 = 0.f, bc3 = 0.f;
  if (own_lo) {
    bc0 = s.bc[0];
    bc1 = s.bc[1];
  }
  if (own_hi) {
    bc2 = s.bc[2];
    bc3 = s.bc[3];
  }
  // probe DFT: thread f of the block that owns a probe cell accumulates it in
  // registers when nf <= threads per block, else the block's threads stride
  // over f and accumulate in place in global memory
  const bool pr_reg = p.nf <= T;
  float pr_r[FDTD1D_MAX_PROBES], pr_i[FDTD1D_MAX_PROBES];
#pragma unroll
  for (int q = 0; q < FDTD1D_MAX_PROBES; ++q) {
    pr_r[q] = 0.f;
    pr_i[q] = 0.f;
  }
  unsigned my_probes = 0;  // probes owned by this block
  for (int q = 0; q < p.nprobe; ++q)
    if (p.probe_k[q] / (CPT * T) == rank) my_probes |= 1u << q;
  if (pr_reg && tid < p.nf) {
#pragma unroll
    for (int q = 0; q < FDTD1D_MAX_PROBES; ++q)
      if (my_probes & (1u << q)) {
        pr_r[q] = s.r_pr[(size_t)q * p.nf + tid];
        pr_i[q] = s.i_pr[(size_t)q * p.nf + tid];
      }
  }

  // neighbour values travel by warp shuffle; only a warp's edge lanes go
  // through shared memory (one slot per warp) or, across blocks, through
  // distributed shared memory
  if (lane == 31) x_last_hy[w] = hy[CPT - 1];
  sync_all();

  for (int t = a.t0 + 1; t <= a.t0 + a.nsteps; ++t) {
    // ---------------- E stage
    float hy_left = __shfl_up_sync(0xffffffffu, hy[CPT - 1], 1);
    if (lane == 0) {
      if (w > 0) hy_left = x_last_hy[w - 1];
      else if (rank > 0) hy_left = remote(x_last_hy, rank - 1, nw - 1);
      else hy_left = 0.f;
    }
    const float v = v_next;
    if (src_here && t < a.t0 + a.nsteps) v_next = __ldg(p.src_table + t);
#pragma unroll
    for (int c = 0; c < CPT; ++c) {
      const int g = g0 + c;
      const float hym = (c == 0) ? hy_left : hy[c - 1];
      if (g >= 1 && g < nx) {
        if (FORM == FDTD1D_FORM_CB) {
          ex[c] = ex_update_cb(ex[c], hym, hy[c], KREG ? k0[c] : __ldg(p.cb + g));
        } else if (FORM == FDTD1D_FORM_CACB) {
          ex[c] = ex_update_cacb(ex[c], hym, hy[c], KREG ? k0[c] : __ldg(p.ca + g), KREG ? k1[c] : __ldg(p.cb + g));
        } else {
          dx[c] = dx_update(dx[c], hym, hy[c]);
        }
      }
      if (src_here && g == p.src_k) {
        if (DF) dx[c] = (p.src_kind == FDTD_SRC_HARD) ? v : __fadd_rn(dx[c], v);
        else ex[c] = (p.src_kind == FDTD_SRC_HARD) ? v : __fadd_rn(ex[c], v);
      }
      if (DF && g >= 1 && g < nx) {
        if (FORM == FDTD1D_FORM_DFORM)
          ex[c] = ex_from_dx(dx[c], ixa[c], KREG ? k0[c] : __ldg(p.nax + g), KREG ? k1[c] : __ldg(p.nbx + g));
        else
          ex[c] = ex_from_dx_debye(dx[c], ixa[c], sxa[c], KREG ? k0[c] : __ldg(p.nax + g),
                                   KREG ? k1[c] : __ldg(p.nbx + g), KREG ? k2[c] : __ldg(p.ncx + g),
                                   KREG ? k3[c] : __ldg(p.ndx + g));
      }
    }
    // running DFT: probes published here, full field accumulated in place
    if (p.nf > 0) {
      for (int q = 0; q < p.nprobe; ++q) {
        const int k = p.probe_k[q];
        if (k >= g0 && k < g0 + CPT) {
#pragma unroll
          for (int c = 0; c < CPT; ++c)
            if (g0 + c == k) x_probe[q] = ex[c];
        }
      }
      if (p.full_dft) {
        const float* cs = p.dft_cos + (size_t)(t - 1) * p.nf;
        const float* sn = p.dft_sin + (size_t)(t - 1) * p.nf;
        for (int f = 0; f < p.nf; ++f) {
          const float cf = __ldg(cs + f), sf = __ldg(sn + f);
#pragma unroll
          for (int c = 0; c < CPT; ++c) {
            const int g = g0 + c;
            if (g < nx) {
              const size_t m = (size_t)f * nx + g;
              s.r_pt[m] = __fmaf_rn(cf, ex[c], s.r_pt[m]);
              s.i_pt[m] = __fmaf_rn(-sf, ex[c], s.i_pt[m]);
            }
          }
        }
      }
    }
    // ABC (fd1d/program/fd1d_1_2.py:47-48): low side complete; high side sets
    // ex[nx-1] now and shifts its state after barrier A
    if (own_lo) {
      const float e1 = ex[1];
      ex[0] = bc0;
      bc0 = bc1;
      bc1 = e1;
    }
    if (own_hi) {
#pragma unroll
      for (int c = 0; c < CPT; ++c)
        if (c == hi_c) ex[c] = bc3;
    }
    const float prev_last_ex = __shfl_up_sync(0xffffffffu, ex[CPT - 1], 1);
    const float next_first_ex = __shfl_down_sync(0xffffffffu, ex[0], 1);
    if (lane == 0) x_first_ex[w] = ex[0];
    if (lane == 31) x_last_ex[w] = ex[CPT - 1];
    sync_all();  // barrier A

    // ---------------- H stage
    if (own_hi) {
      float e_nm2;
      if (hi_c >= 1) {
        e_nm2 = 0.f;
#pragma unroll
        for (int c = 1; c < CPT; ++c)
          if (c == hi_c) e_nm2 = ex[c - 1];
      } else if (lane > 0) {
        e_nm2 = prev_last_ex;
      } else if (w > 0) {
        e_nm2 = x_last_ex[w - 1];
      } else {
        e_nm2 = remote(x_last_ex, rank - 1, nw - 1);
      }
      bc3 = bc2;
      bc2 = e_nm2;
    }
    if (p.nf > 0 && my_probes) {
      if (pr_reg) {
        if (tid < p.nf) {
          const float cf = __ldg(p.dft_cos + (size_t)(t - 1) * p.nf + tid);
          const float sf = __ldg(p.dft_sin + (size_t)(t - 1) * p.nf + tid);
#pragma unroll
          for (int q = 0; q < FDTD1D_MAX_PROBES; ++q)
            if (my_probes & (1u << q)) {
              const float e = x_probe[q];
              pr_r[q] = __fmaf_rn(cf, e, pr_r[q]);
              pr_i[q] = __fmaf_rn(-sf, e, pr_i[q]);
            }
        }
      } else {
        for (int f = tid; f < p.nf; f += T) {
          const float cf = __ldg(p.dft_cos + (size_t)(t - 1) * p.nf + f);
          const float sf = __ldg(p.dft_sin + (size_t)(t - 1) * p.nf + f);
          for (int q = 0; q < p.nprobe; ++q)
            if (my_probes & (1u << q)) {
              const float e = x_probe[q];
              const size_t m = (size_t)q * p.nf + f;
              s.r_pr[m] = __fmaf_rn(cf, e, s.r_pr[m]);
              s.i_pr[m] = __fmaf_rn(-sf, e, s.i_pr[m]);
            }
        }
      }
    }
    float ex_right = next_first_ex;
    if (lane == 31) {
      if (w + 1 < nw) ex_right = x_first_ex[w + 1];
      else if (rank < C - 1) ex_right = remote(x_first_ex, rank + 1, 0);
      else ex_right = 0.f;
    }
#pragma unroll
    for (int c = 0; c < CPT; ++c) {
      const int g = g0 + c;
      if (g <= nx - 2) hy[c] = hy_update(hy[c], ex[c], (c == CPT - 1) ? ex_right : ex[c + 1]);
    }
    if (lane == 31) x_last_hy[w] = hy[CPT - 1];
    sync_all();  // barrier B
  }

  bool fin = true;
#pragma unroll
  for (int c = 0; c < CPT; ++c) {
    const int g = g0 + c;
    if (g < nx) {
      s.ex[g] = ex[c];
      s.hy[g] = hy[c];
      fin &= isfinite(ex[c]) && isfinite(hy[c]);
      if (DF) {
        s.dx[g] = dx[c];
        s.ix[g] = ixa[c];
      }
      if (FORM == FDTD1D_FORM_DEBYE) s.sx[g] = sxa[c];
    }
  }
  if (!fin) raise_status(s.status, ST_NONFINITE);
  if (own_lo) {
    s.bc[0] = bc0;
    s.bc[1] = bc1;
  }
  if (own_hi) {
    s.bc[2] = bc2;
    s.bc[3] = bc3;
  }
  if (pr_reg && tid < p.nf) {
#pragma unroll
    for (int q = 0; q < FDTD1D_MAX_PROBES; ++q)
      if (my_probes & (1u << q)) {
        s.r_pr[(size_t)q * p.nf + tid] = pr_r[q];
        s.i_pr[(size_t)q * p.nf + tid] = pr_i[q];
      }
  }
}

// ============================================================ launchers
namespace {

template <int FORM, int CPT, bool CLUSTER>
int launch_run_t(const Run1DArgs& a, int threads, int cluster, cudaStream_t st) {
  auto kern = k_fd1d_run<FORM, CPT, CLUSTER>;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(cluster, 1, 1);
  cfg.blockDim = dim3(threads, 1, 1);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  int nattr = 0;
  if (CLUSTER) {
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    nattr = 1;
  }
  cfg.attrs = attr;
  cfg.numAttrs = nattr;
  const cudaError_t e = cudaLaunchKernelEx(&cfg, kern, a);
  if (e != cudaSuccess) {
    fdtd_host::note_cuda_error(e);
    return FDTD_ERR_CUDA;
  }
  return fdtd_host::check_launch();
}

// registers of the cluster variant (queried once per process)
template <int FORM, int CPT>
int regs_of() {
  static const int regs = [] {
    cudaFuncAttributes fa{};
    if (cudaFuncGetAttributes(&fa, k_fd1d_run<FORM, CPT, true>) != cudaSuccess) {
      (void)cudaGetLastError();
      return 255;
    }
    return fa.numRegs;
  }();
  return regs;
}

template <int FORM, int CPT>
int launch_run_cpt(const Run1DArgs& a, int threads, int cluster, cudaStream_t st) {
  if (cluster > 1) return launch_run_t<FORM, CPT, true>(a, threads, cluster, st);
  return launch_run_t<FORM, CPT, false>(a, threads, cluster, st);
}

template <int FORM>
int launch_run_form(const Run1DArgs& a, cudaStream_t st) {
  const int nx = a.p.nx;
  // candidates in order of preference: fewest cells per thread that fit one
  // block of <= 256 threads, else larger blocks, else a cluster of blocks
  struct Cand {
    int cpt, regs;
  };
  const Cand cands[4] = {{2, regs_of<FORM, 2>()}, {4, regs_of<FORM, 4>()}, {8, regs_of<FORM, 8>()},
                         {16, regs_of<FORM, 16>()}};
  auto max_threads = [](int regs, int cpt) {
    const int r = ((regs + 7) / 8) * 8;
    int t = 65536 / (r > 0 ? r : 1);
    t = (t / 32) * 32;
    return std::min(t, run1d_max_threads(cpt));
  };
  for (int pass = 0; pass < 3; ++pass) {
    const int limit_threads = pass == 0 ? 256 : RUN1D_MAX_THREADS;
    for (const Cand& c : cands) {
      const int tmax = std::min(limit_threads, max_threads(c.regs, c.cpt));
      const int cells_per_block = tmax * c.cpt;
      int cluster = (nx + cells_per_block - 1) / cells_per_block;
      if (pass < 2 && cluster > 1) continue;
      if (cluster > 8) continue;  // portable cluster size
      int threads = (nx + cluster * c.cpt - 1) / (cluster * c.cpt);
      threads = ((threads + 31) / 32) * 32;
      if (threads > tmax) continue;
      // the thread owning cell nx-1 and the thread owning cell 1 must exist
      switch (c.cpt) {
        case 2: return launch_run_cpt<FORM, 2>(a, threads, cluster, st);
        case 4: return launch_run_cpt<FORM, 4>(a, threads, cluster, st);
        case 8: return launch_run_cpt<FORM, 8>(a, threads, cluster, st);
        default: return launch_run_cpt<FORM, 16>(a, threads, cluster, st);
      }
    }
  }
  return FDTD_ERR_SIZE;
}

}  // namespace

int launch_fd1d_run(const fdtd1d_params& p, const fdtd1d_state& s, int t0, int nsteps, cudaStream_t st) {
  // a line of up to 512 cells runs in ONE warp (no block barrier at all)
  if (p.nx <= 32 * 16) return launch_fd1d_warp(p, s, t0, nsteps, st);
  Run1DArgs a{p, s, t0, nsteps};
  switch (p.form) {
    case FDTD1D_FORM_CB: return launch_run_form<FDTD1D_FORM_CB>(a, st);
    case FDTD1D_FORM_CACB: return launch_run_form<FDTD1D_FORM_CACB>(a, st);
    case FDTD1D_FORM_DFORM: return launch_run_form<FDTD1D_FORM_DFORM>(a, st);
    case FDTD1D_FORM_DEBYE: return launch_run_form<FDTD1D_FORM_DEBYE>(a, st);
    default: return FDTD_ERR_ARG;
  }
}

int launch_fd1d_efield(int t, const fdtd1d_params& p, const fdtd1d_state& s, cudaStream_t st) {
  const int blocks = (p.nx + 255) / 256;
  switch (p.form) {
    case FDTD1D_FORM_CB: k_fd1d_efield<FDTD1D_FORM_CB><<<blocks, 256, 0, st>>>(p, s, t); break;
    case FDTD1D_FORM_CACB: k_fd1d_efield<FDTD1D_FORM_CACB><<<blocks, 256, 0, st>>>(p, s, t); break;
    case FDTD1D_FORM_DFORM: k_fd1d_efield<FDTD1D_FORM_DFORM><<<blocks, 256, 0, st>>>(p, s, t); break;
    case FDTD1D_FORM_DEBYE: k_fd1d_efield<FDTD1D_FORM_DEBYE><<<blocks, 256, 0, st>>>(p, s, t); break;
    default: return FDTD_ERR_ARG;
  }
  int rc = fdtd_host::check_launch();
  if (rc) return rc;
  if (p.src_kind != FDTD_SRC_NONE && p.src_k == 0) {
    k_fd1d_src0<<<1, 1, 0, st>>>(p, s, t);
    rc = fdtd_host::check_launch();
  }
  return rc;
}

int launch_fd1d_hfield(const fdtd1d_params& p, const fdtd1d_state& s, cudaStream_t st) {
  k_fd1d_hfield<<<(p.nx + 255) / 256, 256, 0, st>>>(p, s);
  return fdtd_host::check_launch();
}

int launch_fd1d_fourier(int t, const fdtd1d_params& p, const fdtd1d_state& s, cudaStream_t st) {
  const int n = std::max(p.full_dft ? p.nx : 0, p.nf);
  k_fd1d_fourier<<<(n + 255) / 256, 256, 0, st>>>(p, s, t);
  return fdtd_host::check_launch();
}

}  // namespace fdtd

// ============================================================ C-ABI
namespace {

int check1d(const fdtd1d_params* p, const fdtd1d_state* s, int t_last) {
  if (!p || !s) return FDTD_ERR_NULL;
  if (p->nx < 4) return FDTD_ERR_SIZE;
  if (!s->ex || !s->hy) return FDTD_ERR_NULL;
  switch (p->form) {
    case FDTD1D_FORM_CB:
      if (!p->cb) return FDTD_ERR_NULL;
      break;
    case FDTD1D_FORM_CACB:
      if (!p->ca || !p->cb) return FDTD_ERR_NULL;
      break;
    case FDTD1D_FORM_DFORM:
      if (!p->nax || !p->nbx || !s->dx || !s->ix) return FDTD_ERR_NULL;
      break;
    case FDTD1D_FORM_DEBYE:
      if (!p->nax || !p->nbx || !p->ncx || !p->ndx || !s->dx || !s->ix || !s->sx) return FDTD_ERR_NULL;
      break;
    default: return FDTD_ERR_ARG;
  }
  if (p->src_kind < FDTD_SRC_NONE || p->src_kind > FDTD_SRC_SOFT) return FDTD_ERR_ARG;
  if (p->src_kind != FDTD_SRC_NONE) {
    if (p->src_k < 0 || p->src_k >= p->nx) return FDTD_ERR_ARG;
    if (!p->src_table) return FDTD_ERR_NULL;
    if (t_last > p->src_table_len) return FDTD_ERR_SIZE;
  }
  if (p->abc && !s->bc) return FDTD_ERR_NULL;
  if (p->nf < 0 || p->nf > 1024) return FDTD_ERR_SIZE;
  if (p->nprobe < 0 || p->nprobe > FDTD1D_MAX_PROBES) return FDTD_ERR_SIZE;
  if (p->nf > 0) {
    if (!p->dft_cos || !p->dft_sin) return FDTD_ERR_NULL;
    if (t_last > p->dft_table_len) return FDTD_ERR_SIZE;
    if (p->full_dft && (!s->r_pt || !s->i_pt)) return FDTD_ERR_NULL;
    if (p->nprobe > 0 && (!s->r_pr || !s->i_pr)) return FDTD_ERR_NULL;
    for (int q = 0; q < p->nprobe; ++q)
      if (p->probe_k[q] < 0 || p->probe_k[q] >= p->nx) return FDTD_ERR_ARG;
  }
  return FDTD_OK;
}

}  // namespace

extern "C" {

int fdtd1d_efield(int t, const fdtd1d_params* p, fdtd1d_state* s, fdtd_stream_t stream) {
  int rc = check1d(p, s, t);
  if (rc) return rc;
  if (t < 1) return FDTD_ERR_ARG;
  return fdtd::launch_fd1d_efield(t, *p, *s, (cudaStream_t)stream);
}

int fdtd1d_hfield(const fdtd1d_params* p, fdtd1d_state* s, fdtd_stream_t stream) {
  int rc = check1d(p, s, 0);
  if (rc) return rc;
  return fdtd::launch_fd1d_hfield(*p, *s, (cudaStream_t)stream);
}

int fdtd1d_fourier(int t, const fdtd1d_params* p, fdtd1d_state* s, fdtd_stream_t stream) {
  int rc = check1d(p, s, t);
  if (rc) return rc;
  if (t < 1 || p->nf <= 0) return FDTD_ERR_ARG;
  return fdtd::launch_fd1d_fourier(t, *p, *s, (cudaStream_t)stream);
}

int fdtd1d_step_n(const fdtd1d_params* p, fdtd1d_state* s, int t0, int nsteps, fdtd_stream_t stream) {
  if (t0 < 0 || nsteps < 0) return FDTD_ERR_ARG;
  int rc = check1d(p, s, t0 + nsteps);
  if (rc) return rc;
  if (nsteps == 0) return FDTD_OK;
  if (p->nx > FDTD1D_MAX_FUSED_NX) return FDTD_ERR_SIZE;
  return fdtd::launch_fd1d_run(*p, *s, t0, nsteps, (cudaStream_t)stream);
}

}  // extern "C"
