// Single-warp fused 1D run: a line of up to 512 cells held by ONE warp, CPT
// consecutive cells per lane in registers, the whole time loop in one launch.
//
// The step keeps the reference's serial order (E -> source -> DFT -> ABC -> H,
// fd1d/program/fd1d_2_2.py:138-142) and calls the same per-cell formulas as
// the per-function kernels, so the fields are bitwise equal to them.  What
// makes it short is that nothing per step depends on where the line ends:
//   * every lane runs the same branch-free cell loops; the cells that differ
//     (the source cell, nx-1 and nx-2) are picked by one bitwise select per
//     cell against one-hot lane masks, not by branches or predicates.  Cells
//     past the end of the line are ghosts whose coefficients are zero, so
//     they stay exactly 0, and the H update takes its factor from a per-cell
//     register (0.5, or 0 for hy[nx-1] and the ghosts).  hy[nx-1] is never updated by the
//     reference; hy + 0*(finite) returns hy (a -0.0 there becomes +0.0);
//   * cell 0 (never E-updated) is lane 0's first cell, a compile-time
//     position, and so are the low-side ABC cells 0 and 1;
//   * when nx is a multiple of CPT (HI_END) the high-side ABC cells nx-2 and
//     nx-1 are the last two cells of their lane, also compile-time positions;
//     otherwise the mask selects find them;
//   * the left neighbour's last hy and the right neighbour's first ex travel
//     by one warp shuffle each; no barrier and no shared memory in the step
//     (the probe DFT publishes its cells through a shared slot per step
//     parity);
//   * the source values of 32 steps are read by one coalesced load, one per
//     lane, a chunk ahead, and broadcast by shuffle in the step.
// Probe DFT accumulators sit in registers of lane f when nf <= 32, else they
// are accumulated in place in global memory (lanes stride over f).
#pragma once

#include "fdtd_common.cuh"

namespace fdtd {

struct Warp1DArgs {
  fdtd1d_params p;
  fdtd1d_state s;
  int t0, nsteps;
};

// a if the mask is all ones, b if it is zero: one bitwise select, no predicate
__device__ __forceinline__ float bsel(unsigned m, float a, float b) {
  return __uint_as_float((__float_as_uint(a) & m) | (__float_as_uint(b) & ~m));
}

// SOFT: the source adds to the field (else it replaces it, or is absent)
template <int FORM, int CPT, bool HI_END, bool DFT, bool SOFT>
__global__ void __launch_bounds__(32) k_fd1d_warp(const Warp1DArgs a) {
  constexpr bool DF = (FORM == FDTD1D_FORM_DFORM || FORM == FDTD1D_FORM_DEBYE);
  constexpr bool DB = (FORM == FDTD1D_FORM_DEBYE);
  constexpr unsigned kAll = 0xffffffffu;
  const fdtd1d_params& p = a.p;
  const fdtd1d_state& s = a.s;
  __shared__ float x_probe[2][FDTD1D_MAX_PROBES];

  const int lane = threadIdx.x;
  const int nx = p.nx;
  const int g0 = lane * CPT;

  // source: lane src_k / CPT, cell sp of it (-1 elsewhere)
  const bool have_src = p.src_kind != FDTD_SRC_NONE;
  const int sp = (have_src && p.src_k / CPT == lane) ? p.src_k - g0 : -1;
  // two-step-back ABC: lane 0 holds cells 0 and 1; lane hi_lane holds nx-1
  const bool abc = p.abc != 0;
  const bool own_lo = abc && lane == 0;
  const int hi_lane = (nx - 1) / CPT;
  const int hi_c = (nx - 1) - hi_lane * CPT;  // CPT-1 when HI_END
  const bool own_hi = abc && lane == hi_lane;

  float ex[CPT], hy[CPT], dx[CPT], ixa[CPT], sxa[CPT];
  float k0[CPT], k1[CPT], k2[CPT], k3[CPT], hc[CPT];
  unsigned sm[CPT], hm[CPT], nm[CPT];  // one-hot masks: source cell, nx-1, nx-2
#pragma unroll
  for (int c = 0; c < CPT; ++c) {
    const int g = g0 + c;
    const bool in = g < nx;
    const bool e_in = g >= 1 && g < nx;
    ex[c] = in ? s.ex[g] : 0.f;
    hy[c] = in ? s.hy[g] : 0.f;
    dx[c] = (DF && in) ? s.dx[g] : 0.f;
    ixa[c] = (DF && in) ? s.ix[g] : 0.f;
    sxa[c] = (DB && in) ? s.sx[g] : 0.f;
    k0[c] = k1[c] = k2[c] = k3[c] = 0.f;
    if (e_in) {
      if (FORM == FDTD1D_FORM_CB) k0[c] = __ldg(p.cb + g);
      if (FORM == FDTD1D_FORM_CACB) {
        k0[c] = __ldg(p.ca + g);
        k1[c] = __ldg(p.cb + g);
      }
      if (DF) {
        k0[c] = __ldg(p.nax + g);
        k1[c] = __ldg(p.nbx + g);
      }
      if (DB) {
        k2[c] = __ldg(p.ncx + g);
        k3[c] = __ldg(p.ndx + g);
      }
    }
    hc[c] = (g <= nx - 2) ? 0.5f : 0.f;
    sm[c] = (c == sp) ? kAll : 0u;
    hm[c] = (own_hi && c == hi_c) ? kAll : 0u;
    nm[c] = (own_hi && c + 1 == hi_c) ? kAll : 0u;
  }
  const unsigned z0 = lane == 0 ? kAll : 0u;  // this lane's first cell is cell 0 (no E update)
  const unsigned lo_m = own_lo ? kAll : 0u;
  const unsigned hi_m = own_hi ? kAll : 0u;
  float bc0 = 0.f, bc1 = 0.f, bc2 = 0.f, bc3 = 0.f;
  if (own_lo) {
    bc0 = s.bc[0];
    bc1 = s.bc[1];
  }
  if (own_hi) {
    bc2 = s.bc[2];
    bc3 = s.bc[3];
  }

  // probe DFT (lane f holds frequency f when nf <= 32)
  const int nf = DFT ? p.nf : 0;
  const int npr = DFT ? p.nprobe : 0;
  const bool pr_reg = nf <= 32;
  float pr_r[FDTD1D_MAX_PROBES], pr_i[FDTD1D_MAX_PROBES];
#pragma unroll
  for (int q = 0; q < FDTD1D_MAX_PROBES; ++q) {
    pr_r[q] = 0.f;
    pr_i[q] = 0.f;
    if (DFT && q < npr && pr_reg && lane < nf) {
      pr_r[q] = s.r_pr[(size_t)q * nf + lane];
      pr_i[q] = s.i_pr[(size_t)q * nf + lane];
    }
  }

  // one time step t with source value v; branch-free except the DFT
  auto step = [&](const int t, const float v) {
    // ---------------- E stage (+ source)
    // lane 0 receives its own value: cell 0 is never E-updated
    const float hy_left = __shfl_up_sync(kAll, hy[CPT - 1], 1);
#pragma unroll
    for (int c = 0; c < CPT; ++c) {
      const float hym = (c == 0) ? hy_left : hy[c - 1];
      if (FORM == FDTD1D_FORM_CB) {
        const float e = ex_update_cb(ex[c], hym, hy[c], k0[c]);
        ex[c] = c == 0 ? bsel(z0, ex[0], e) : e;
      } else if (FORM == FDTD1D_FORM_CACB) {
        const float e = ex_update_cacb(ex[c], hym, hy[c], k0[c], k1[c]);
        ex[c] = c == 0 ? bsel(z0, ex[0], e) : e;
      } else {
        const float d = dx_update(dx[c], hym, hy[c]);
        dx[c] = c == 0 ? bsel(z0, dx[0], d) : d;
      }
    }
#pragma unroll
    for (int c = 0; c < CPT; ++c) {
      float& f = DF ? dx[c] : ex[c];
      f = bsel(sm[c], SOFT ? __fadd_rn(f, v) : v, f);
    }
    if (DF) {
#pragma unroll
      for (int c = 0; c < CPT; ++c) {
        float ixn = ixa[c], sxn = sxa[c];
        const float e = (FORM == FDTD1D_FORM_DFORM) ? ex_from_dx(dx[c], ixn, k0[c], k1[c])
                                                    : ex_from_dx_debye(dx[c], ixn, sxn, k0[c], k1[c], k2[c], k3[c]);
        if (c == 0) {
          ex[0] = bsel(z0, ex[0], e);
          ixa[0] = bsel(z0, ixa[0], ixn);
          if (DB) sxa[0] = bsel(z0, sxa[0], sxn);
        } else {
          ex[c] = e;
          ixa[c] = ixn;
          if (DB) sxa[c] = sxn;
        }
      }
    }

    // ---------------- running DFT (before the ABC, as fourier() precedes hfield())
    if (DFT) {
      const int buf = t & 1;
      for (int q = 0; q < npr; ++q) {
        const int k = p.probe_k[q];
        if (k / CPT == lane) {
          float e = 0.f;
#pragma unroll
          for (int c = 0; c < CPT; ++c)
            if (g0 + c == k) e = ex[c];
          x_probe[buf][q] = e;
        }
      }
      const float* cs = p.dft_cos + (size_t)(t - 1) * nf;
      const float* sn = p.dft_sin + (size_t)(t - 1) * nf;
      if (p.full_dft) {
        for (int f = 0; f < nf; ++f) {
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
      __syncwarp();
      if (pr_reg) {
        if (lane < nf) {
          const float cf = __ldg(cs + lane), sf = __ldg(sn + lane);
#pragma unroll
          for (int q = 0; q < FDTD1D_MAX_PROBES; ++q)
            if (q < npr) {
              const float e = x_probe[buf][q];
              pr_r[q] = __fmaf_rn(cf, e, pr_r[q]);
              pr_i[q] = __fmaf_rn(-sf, e, pr_i[q]);
            }
        }
      } else {
        for (int f = lane; f < nf; f += 32) {
          const float cf = __ldg(cs + f), sf = __ldg(sn + f);
          for (int q = 0; q < npr; ++q) {
            const float e = x_probe[buf][q];
            const size_t m = (size_t)q * nf + f;
            s.r_pr[m] = __fmaf_rn(cf, e, s.r_pr[m]);
            s.i_pr[m] = __fmaf_rn(-sf, e, s.i_pr[m]);
          }
        }
      }
    }

    // ---------------- ABC (fd1d/program/fd1d_1_2.py:47-48); the state moves in
    // every lane, only the owners' values are kept
    const float e1 = ex[1];
    ex[0] = bsel(lo_m, bc0, ex[0]);
    bc0 = bc1;
    bc1 = e1;
    if (HI_END) {
      ex[CPT - 1] = bsel(hi_m, bc3, ex[CPT - 1]);
    } else {
#pragma unroll
      for (int c = 0; c < CPT; ++c) ex[c] = bsel(hm[c], bc3, ex[c]);
    }
    // ---------------- H stage
    // lane 31 receives its own value: its last cell is nx-1 or a ghost (factor 0)
    const float ex_right = __shfl_down_sync(kAll, ex[0], 1);
    float e_nm2;
    if (HI_END) {
      e_nm2 = ex[CPT - 2];
    } else {
      // nx-2 is a cell of the same lane, or (hi_c == 0) the last cell of the lane before
      const float prev_last = __shfl_up_sync(kAll, ex[CPT - 1], 1);
      unsigned acc = 0u;
#pragma unroll
      for (int c = 0; c < CPT; ++c) acc |= __float_as_uint(ex[c]) & nm[c];
      e_nm2 = hi_c == 0 ? prev_last : __uint_as_float(acc);
    }
    bc3 = bc2;
    bc2 = e_nm2;
#pragma unroll
    for (int c = 0; c < CPT; ++c) {
      const float er = (c == CPT - 1) ? ex_right : ex[c + 1];
      hy[c] = __fmaf_rn(hc[c], __fsub_rn(ex[c], er), hy[c]);
    }
  };

  const int t_end = a.t0 + a.nsteps;
  // source values of steps t+1 .. t+32 (table rows t .. t+31), one per lane
  float vc = (have_src && a.t0 + lane < t_end) ? __ldg(p.src_table + a.t0 + lane) : 0.f;
  for (int tc = a.t0; tc < t_end; tc += 32) {
    const int nchunk = min(32, t_end - tc);
    const int tn = tc + 32 + lane;
    const float vn = (have_src && tn < t_end) ? __ldg(p.src_table + tn) : 0.f;
    int j = 0;
    if (!DFT) {
      // 16 steps unrolled: the scheduler interleaves neighbouring steps
      // (47 us per config-1 run against 51 us for 4 and 55 us for none)
      for (; j + 16 <= nchunk; j += 16) {
#pragma unroll
        for (int i = 0; i < 16; ++i) step(tc + j + i + 1, __shfl_sync(kAll, vc, j + i));
      }
    }
    for (; j < nchunk; ++j) step(tc + j + 1, __shfl_sync(kAll, vc, j));
    vc = vn;
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
      if (DB) s.sx[g] = sxa[c];
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
  if (DFT && pr_reg && lane < nf) {
#pragma unroll
    for (int q = 0; q < FDTD1D_MAX_PROBES; ++q)
      if (q < npr) {
        s.r_pr[(size_t)q * nf + lane] = pr_r[q];
        s.i_pr[(size_t)q * nf + lane] = pr_i[q];
      }
  }
}

// Launches the single-warp run; FDTD_ERR_SIZE when nx > 32 * 16.
int launch_fd1d_warp(const fdtd1d_params& p, const fdtd1d_state& s, int t0, int nsteps, cudaStream_t st);
// the two halves of the dispatch (one per translation unit)
int launch_fd1d_warp_plain(const Warp1DArgs& a, int cpt, bool hi_end, cudaStream_t st);
int launch_fd1d_warp_dft(const Warp1DArgs& a, int cpt, bool hi_end, cudaStream_t st);

template <bool DFT>
int launch_fd1d_warp_half(const Warp1DArgs& a, int cpt, bool hi_end, cudaStream_t st) {
  auto go = [&](auto kern) -> int {
    kern<<<1, 32, 0, st>>>(a);
    return fdtd_host::check_launch();
  };
  const bool soft = a.p.src_kind == FDTD_SRC_SOFT;
#define FDTD_WARP_CASE(F, C)                                                          \
  if (a.p.form == F && cpt == C) {                                                    \
    if (soft) return hi_end ? go(k_fd1d_warp<F, C, true, DFT, true>) : go(k_fd1d_warp<F, C, false, DFT, true>); \
    return hi_end ? go(k_fd1d_warp<F, C, true, DFT, false>) : go(k_fd1d_warp<F, C, false, DFT, false>);       \
  }
#define FDTD_WARP_FORM(F) \
  FDTD_WARP_CASE(F, 2) FDTD_WARP_CASE(F, 4) FDTD_WARP_CASE(F, 8) FDTD_WARP_CASE(F, 16)
  FDTD_WARP_FORM(FDTD1D_FORM_CB)
  FDTD_WARP_FORM(FDTD1D_FORM_CACB)
  FDTD_WARP_FORM(FDTD1D_FORM_DFORM)
  FDTD_WARP_FORM(FDTD1D_FORM_DEBYE)
#undef FDTD_WARP_FORM
#undef FDTD_WARP_CASE
  return FDTD_ERR_ARG;
}

}  // namespace fdtd
