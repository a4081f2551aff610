// Fused, temporally blocked 2D TM update: the hot kernel of fdtd2d_step_n.
//
// One pass advances the whole grid by K time steps (K = 1..4) while reading
// every field once from HBM and writing it once: 60 bytes per cell per pass
// for the lossy PML update (dz, iz, hx, hy, ihx, ihy, naz, nbz in; dz, iz, hx,
// hy, ihx, ihy, ez out), i.e. 60/K bytes per cell-update.
//
// Work decomposition ("streaming march"):
//   * a warp owns a stripe of 32*CPL columns (CPL = columns per lane, loaded
//     as one float4/float2), of which the middle 32*CPL-8 are its output and
//     4 on each side are halo recomputed redundantly;
//   * the warp walks down a segment of rows.  At row iteration r, level 1
//     takes input row r, computes D and E on it and completes H on row r-1;
//     level s takes the row level s-1 just completed (r-s+1) and completes
//     row r-s at time step s; level K's completed row is stored.  The state a
//     level carries from one row to the next (the previous row's H, E, D
//     values) lives in registers, so each cell's K time steps never touch
//     memory in between;
//   * the j-neighbours needed by the stencil (hx[j-1] for D, ez[j+1] for H)
//     come from the adjacent lane by warp shuffle; there is no __syncthreads
//     and no shared-memory staging of fields at all;
//   * the i-neighbours come from the row carried in registers.  Segments
//     overlap by K rows (the dependence cone), so warps are independent.
// Passes read one copy of the evolving fields and write the other (ping-pong),
// which makes the overlapping reads race-free.  Out-of-grid lanes/rows load
// zeros and are masked by the same predicates as the reference loops (no D on
// row/column 0, no H on the last row/column), so boundary cells see exactly
// the reference's update.
//
// The per-cell arithmetic is the shared inline formulas of fdtd_common.cuh,
// so a pass of K steps is bitwise identical to K rounds of the per-function
// kernels (dfield -> source -> efield -> hfield).
#include <cstdio>
#include <cstdlib>

#include "fd2d_internal.cuh"

namespace fdtd {

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int HALO = 4;  // halo columns on each side (>= K, multiple of 4 for aligned vectors)

struct MarchArgs {
  int nx, ny;
  FieldSet in, out;
  float* ez;
  const float* naz;
  const float* nbz;
  fdtd2d_pml pml;
  int src_kind, src_i, src_j;
  const float* src_table;
  int t0;
  int seg_rows, n_stripes, n_segs;
  int* status;
  int check_finite;
  int probe_i, probe_j;  // Ez trace cell (probe_ez != nullptr)
  float* probe_ez;       // probe_ez[t-1] = ez at the probe after step t
};

template <int CPL>
__device__ __forceinline__ void ld_row(const float* __restrict__ p, bool ok, float (&v)[CPL]) {
  if (ok) {
    if constexpr (CPL == 4) {
      const float4 x = __ldg(reinterpret_cast<const float4*>(p));
      v[0] = x.x; v[1] = x.y; v[2] = x.z; v[3] = x.w;
    } else {
      const float2 x = __ldg(reinterpret_cast<const float2*>(p));
      v[0] = x.x; v[1] = x.y;
    }
  } else {
#pragma unroll
    for (int c = 0; c < CPL; ++c) v[c] = 0.f;
  }
}

template <int CPL>
__device__ __forceinline__ void st_row(float* __restrict__ p, const float (&v)[CPL]) {
  if constexpr (CPL == 4) {
    __stcs(reinterpret_cast<float4*>(p), make_float4(v[0], v[1], v[2], v[3]));
  } else {
    __stcs(reinterpret_cast<float2*>(p), make_float2(v[0], v[1]));
  }
}

template <int CPL>
__device__ __forceinline__ bool all_finite(const float (&v)[CPL]) {
  bool ok = true;
#pragma unroll
  for (int c = 0; c < CPL; ++c) ok &= isfinite(v[c]);
  return ok;
}

// The Ez probe (the adjoint's objective trace) is a separate instantiation,
// so the benchmark kernels carry no per-cell probe test.  Kernels with
// 64-column stripes are held to four 4-warp blocks per SM (128 registers, no
// spills); left free, the compiler takes 138-142 registers and the SM runs
// three blocks (-9% to -20% at 8192^2, K = 4).  128-column stripes need more
// registers and are left free.
template <int K, int CPL, bool LOSSY, bool PML, int WARPS, bool PROBE>
__global__ void __launch_bounds__(WARPS * 32, CPL == 2 ? 4 : 1) k_march(const MarchArgs a) {
  constexpr int W = 32 * CPL;
  constexpr int OUTW = W - 2 * HALO;
  static_assert(K >= 1 && K <= HALO, "steps per pass must not exceed the halo");
  extern __shared__ float smem[];  // per warp: gy2, gy3, fy1, fy2, fy3 of its columns

  const int lane = threadIdx.x & 31;
  const int wid = threadIdx.x >> 5;
  const int gw = blockIdx.x * WARPS + wid;
  const int stripe = gw % a.n_stripes;
  const int seg = gw / a.n_stripes;
  if (seg >= a.n_segs) return;  // whole warp leaves; nothing below syncs the block

  const int nx = a.nx, ny = a.ny;
  const int j0 = stripe * OUTW - HALO + lane * CPL;  // first column of this lane (multiple of 4 or 2)
  const bool vin = (j0 >= 0) && (j0 + CPL <= ny);    // ny % 4 == 0: a vector is wholly in or out
  const bool vout = vin && (lane * CPL >= HALO) && (lane * CPL < HALO + OUTW);

  float* cg = smem + wid * 5 * W + lane * CPL;
  if (PML) {
#pragma unroll
    for (int c = 0; c < CPL; ++c) {
      const int j = j0 + c;
      const bool ok = (j >= 0) && (j < ny);
      cg[0 * W + c] = ok ? __ldg(a.pml.gy2 + j) : 1.f;
      cg[1 * W + c] = ok ? __ldg(a.pml.gy3 + j) : 1.f;
      cg[2 * W + c] = ok ? __ldg(a.pml.fy1 + j) : 0.f;
      cg[3 * W + c] = ok ? __ldg(a.pml.fy2 + j) : 1.f;
      cg[4 * W + c] = ok ? __ldg(a.pml.fy3 + j) : 1.f;
    }
    __syncwarp();
  }

  // level state: values of the row each level will complete next
  float p_hy[K][CPL], p_hx[K][CPL], p_ihx[K][CPL], p_ihy[K][CPL], p_ez[K][CPL], p_dz[K][CPL], p_iz[K][CPL];
#pragma unroll
  for (int s = 0; s < K; ++s)
#pragma unroll
    for (int c = 0; c < CPL; ++c) {
      p_hy[s][c] = p_hx[s][c] = p_ihx[s][c] = p_ihy[s][c] = 0.f;
      p_ez[s][c] = p_dz[s][c] = p_iz[s][c] = 0.f;
    }

  const int i_s = seg * a.seg_rows;
  const int i_e = min(nx, i_s + a.seg_rows);
  const int r_begin = max(0, i_s - K);
  const int r_end = i_e - 1 + K;
  bool finite_ok = true;

  for (int r = r_begin; r <= r_end; ++r) {
    float in_dz[CPL], in_iz[CPL], in_hx[CPL], in_hy[CPL], in_ihx[CPL], in_ihy[CPL];
    {
      const bool ok = vin && (r < nx);
      const size_t off = ok ? (size_t)r * ny + j0 : 0;
      ld_row<CPL>(a.in.dz + off, ok, in_dz);
      ld_row<CPL>(a.in.hx + off, ok, in_hx);
      ld_row<CPL>(a.in.hy + off, ok, in_hy);
      if (LOSSY) ld_row<CPL>(a.in.iz + off, ok, in_iz);
      else {
#pragma unroll
        for (int c = 0; c < CPL; ++c) in_iz[c] = 0.f;
      }
      if (PML) {
        ld_row<CPL>(a.in.ihx + off, ok, in_ihx);
        ld_row<CPL>(a.in.ihy + off, ok, in_ihy);
      } else {
#pragma unroll
        for (int c = 0; c < CPL; ++c) in_ihx[c] = in_ihy[c] = 0.f;
      }
    }

#pragma unroll
    for (int s = 0; s < K; ++s) {
      const int q = r - s;   // row entering level s+1 (time step t0+s+1)
      const int qc = q - 1;  // row level s+1 completes now
      const bool qok = (q >= 0) && (q < nx);

      // ---- D (+ point source) and E on row q
      float naz[CPL], nbz[CPL];
      {
        const bool ok = qok && vin;
        const size_t off = ok ? (size_t)q * ny + j0 : 0;
        ld_row<CPL>(a.naz + off, ok, naz);
        if (LOSSY) ld_row<CPL>(a.nbz + off, ok, nbz);
      }
      float gx3q = 1.f, gx2q = 1.f;
      if (PML && qok) {
        gx3q = __ldg(a.pml.gx3 + q);
        gx2q = __ldg(a.pml.gx2 + q);
      }
      const float hx_left = __shfl_up_sync(FULL, in_hx[CPL - 1], 1);
      const bool drow = (q >= 1) && (q < nx);
      float nd[CPL], ne[CPL], niz[CPL];
#pragma unroll
      for (int c = 0; c < CPL; ++c) {
        const int j = j0 + c;
        float d = in_dz[c];
        if (drow && j >= 1 && j < ny) {
          const float hxm = (c == 0) ? hx_left : in_hx[c - 1];
          const float gy2 = PML ? cg[0 * W + c] : 1.f;
          const float gy3 = PML ? cg[1 * W + c] : 1.f;
          d = d_update(d, in_hy[c], p_hy[s][c], in_hx[c], hxm, gx3q, gy3, gx2q, gy2);
        }
        if (a.src_kind != FDTD_SRC_NONE && q == a.src_i && j == a.src_j) {
          const float v = __ldg(a.src_table + a.t0 + s);
          d = (a.src_kind == FDTD_SRC_HARD) ? v : __fadd_rn(d, v);
        }
        float izv = in_iz[c];
        const float e = LOSSY ? e_update_lossy(d, izv, naz[c], nbz[c]) : e_update(d, naz[c]);
        nd[c] = d;
        niz[c] = izv;
        ne[c] = e;
        // the probe cell's Ez is recorded by the warp that owns it (output
        // column, row inside the segment), where every level is valid
        if (PROBE && q == a.probe_i && j == a.probe_j && vout && q >= i_s && q < i_e) a.probe_ez[a.t0 + s] = e;
      }

      // ---- H on row qc (needs Ez of rows qc and q at this level)
      const float ez_right = __shfl_down_sync(FULL, p_ez[s][0], 1);
      const bool hrow = (qc >= 0) && (qc <= nx - 2);
      float fx1 = 0.f, fx2 = 1.f, fx3 = 1.f;
      if (PML && hrow) {
        fx1 = __ldg(a.pml.fx1 + qc);
        fx2 = __ldg(a.pml.fx2 + qc);
        fx3 = __ldg(a.pml.fx3 + qc);
      }
      float ohx[CPL], ohy[CPL], oihx[CPL], oihy[CPL];
#pragma unroll
      for (int c = 0; c < CPL; ++c) {
        const int j = j0 + c;
        float hxv = p_hx[s][c], hyv = p_hy[s][c], ihxv = p_ihx[s][c], ihyv = p_ihy[s][c];
        if (hrow && j >= 0 && j <= ny - 2) {
          const float er = (c == CPL - 1) ? ez_right : p_ez[s][c + 1];
          if (PML)
            h_update_pml(p_ez[s][c], er, ne[c], hxv, hyv, ihxv, ihyv, fx1, fx2, fx3, cg[2 * W + c], cg[3 * W + c],
                         cg[4 * W + c]);
          else
            h_update_free(p_ez[s][c], er, ne[c], hxv, hyv);
        }
        ohx[c] = hxv;
        ohy[c] = hyv;
        oihx[c] = ihxv;
        oihy[c] = ihyv;
      }

      // ---- level K stores its completed row
      if (s == K - 1 && vout && qc >= i_s && qc < i_e) {
        const size_t off = (size_t)qc * ny + j0;
        st_row<CPL>(a.out.dz + off, p_dz[s]);
        st_row<CPL>(a.out.hx + off, ohx);
        st_row<CPL>(a.out.hy + off, ohy);
        st_row<CPL>(a.ez + off, p_ez[s]);
        if (LOSSY) st_row<CPL>(a.out.iz + off, p_iz[s]);
        if (PML) {
          st_row<CPL>(a.out.ihx + off, oihx);
          st_row<CPL>(a.out.ihy + off, oihy);
        }
        if (a.check_finite) {
          finite_ok &= all_finite<CPL>(p_dz[s]) & all_finite<CPL>(ohx) & all_finite<CPL>(ohy) &
                       all_finite<CPL>(p_ez[s]);
          if (LOSSY) finite_ok &= all_finite<CPL>(p_iz[s]);
          if (PML) finite_ok &= all_finite<CPL>(oihx) & all_finite<CPL>(oihy);
        }
      }

      // ---- shift: this level's incoming row becomes its "previous" row, and
      //      the row it completed is the next level's incoming row
#pragma unroll
      for (int c = 0; c < CPL; ++c) {
        const float t_hy = in_hy[c], t_hx = in_hx[c], t_ihx = in_ihx[c], t_ihy = in_ihy[c];
        in_dz[c] = p_dz[s][c];
        in_iz[c] = p_iz[s][c];
        in_hx[c] = ohx[c];
        in_hy[c] = ohy[c];
        in_ihx[c] = oihx[c];
        in_ihy[c] = oihy[c];
        p_hy[s][c] = t_hy;
        p_hx[s][c] = t_hx;
        p_ihx[s][c] = t_ihx;
        p_ihy[s][c] = t_ihy;
        p_ez[s][c] = ne[c];
        p_dz[s][c] = nd[c];
        p_iz[s][c] = niz[c];
      }
    }
  }
  if (a.check_finite && __any_sync(FULL, !finite_ok) && lane == 0) raise_status(a.status, ST_NONFINITE);
}

// ------------------------------------------------------------- dispatch
struct MarchConfig {
  int cpl = 0;       // columns per lane; 0 = automatic (measured best: 4 for K <= 2, 2 for K >= 3)
  int warps = 4;
  int seg_rows = 0;  // 0 = automatic
};

MarchConfig g_cfg;  // tuning knob (fdtd2d_set_march_config)

// Shortest automatic segment: 4K rows (the recomputed cone is 2K), at least 8.
// Measured at 1024^2 (adjoint forward/recompute): 8 rows for K <= 2 and 16 for
// K = 4 beat 16/32 by 1.3-2x, because small grids otherwise leave most SMs idle.
constexpr int min_seg_rows(int K) { return K * 4 > 8 ? K * 4 : 8; }

template <int K, int CPL, bool LOSSY, bool PML, bool PROBE>
int launch_t(const MarchArgs& a0, int warps_cfg, int seg_cfg, cudaStream_t st) {
  constexpr int WARPS = 4;
  (void)warps_cfg;
  MarchArgs a = a0;
  constexpr int W = 32 * CPL;
  constexpr int OUTW = W - 2 * HALO;
  auto kern = k_march<K, CPL, LOSSY, PML, WARPS, PROBE>;
  const size_t smem = PML ? (size_t)WARPS * 5 * W * sizeof(float) : 0;
  a.n_stripes = (a.ny + OUTW - 1) / OUTW;
  int seg_rows = seg_cfg;
  if (seg_rows <= 0) {
    int dev = 0, nsm = 0, blocks_per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, kern, WARPS * 32, smem);
    if (blocks_per_sm < 1) blocks_per_sm = 1;
    const long resident = (long)nsm * blocks_per_sm * WARPS;
    // one wave of warps: n_stripes * n_segs ~= resident warps
    long n_segs = resident / a.n_stripes;
    if (n_segs < 1) n_segs = 1;
    seg_rows = (int)((a.nx + n_segs - 1) / n_segs);
    // keep the recomputed cone (2K rows per segment) small
    seg_rows = std::max(seg_rows, min_seg_rows(K));
  }
  a.seg_rows = seg_rows;
  a.n_segs = (a.nx + seg_rows - 1) / seg_rows;
  const long warps = (long)a.n_stripes * a.n_segs;
  const int blocks = (int)((warps + WARPS - 1) / WARPS);
  kern<<<blocks, WARPS * 32, smem, st>>>(a);
  return fdtd_host::check_launch();
}

template <int K, int CPL>
int launch_k(const MarchArgs& a, bool lossy, bool pml, cudaStream_t st) {
  if (a.probe_ez) {
    if (lossy && pml) return launch_t<K, CPL, true, true, true>(a, g_cfg.warps, g_cfg.seg_rows, st);
    if (lossy) return launch_t<K, CPL, true, false, true>(a, g_cfg.warps, g_cfg.seg_rows, st);
    if (pml) return launch_t<K, CPL, false, true, true>(a, g_cfg.warps, g_cfg.seg_rows, st);
    return launch_t<K, CPL, false, false, true>(a, g_cfg.warps, g_cfg.seg_rows, st);
  }
  if (lossy && pml) return launch_t<K, CPL, true, true, false>(a, g_cfg.warps, g_cfg.seg_rows, st);
  if (lossy) return launch_t<K, CPL, true, false, false>(a, g_cfg.warps, g_cfg.seg_rows, st);
  if (pml) return launch_t<K, CPL, false, true, false>(a, g_cfg.warps, g_cfg.seg_rows, st);
  return launch_t<K, CPL, false, false, false>(a, g_cfg.warps, g_cfg.seg_rows, st);
}

template <int CPL>
int launch_cpl(const MarchArgs& a, int k, bool lossy, bool pml, cudaStream_t st) {
  switch (k) {
    case 1: return launch_k<1, CPL>(a, lossy, pml, st);
    case 2: return launch_k<2, CPL>(a, lossy, pml, st);
    case 3: return launch_k<3, CPL>(a, lossy, pml, st);
    case 4: return launch_k<4, CPL>(a, lossy, pml, st);
    default: return FDTD_ERR_ARG;
  }
}

}  // namespace

int march_max_steps_per_pass() { return HALO; }

int launch_march(const fdtd2d_params& p, const FieldSet& in, const FieldSet& out, float* ez, int t0, int k,
                 int* status, float* probe_ez, cudaStream_t st) {
  MarchArgs a{};
  a.nx = p.nx;
  a.ny = p.ny;
  a.in = in;
  a.out = out;
  a.ez = ez;
  a.naz = p.naz;
  a.nbz = p.nbz;
  a.pml = p.pml;
  a.src_kind = p.src.kind;
  a.src_i = p.src.i;
  a.src_j = p.src.j;
  a.src_table = p.src.table;
  a.t0 = t0;
  a.status = status;
  a.check_finite = status != nullptr;
  a.probe_i = p.probe_i;
  a.probe_j = p.probe_j;
  a.probe_ez = probe_ez;
  const bool lossy = p.nbz != nullptr;
  const bool pml = has_pml(p);
  int cpl = g_cfg.cpl ? g_cfg.cpl : (k >= 3 ? 2 : 4);
  if (!g_cfg.cpl && cpl == 4 && k >= 1 && k <= HALO) {
    // small grids: if 128-column stripes times the shortest segments would not
    // fill one wave of warps (32 per SM), use 64-column stripes instead
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const long stripes = (p.ny + (32 * 4 - 2 * HALO) - 1) / (32 * 4 - 2 * HALO);
    const long segs = (p.nx + min_seg_rows(k) - 1) / min_seg_rows(k);
    if (stripes * segs < 32L * nsm) cpl = 2;
  }
  if (cpl == 2) return launch_cpl<2>(a, k, lossy, pml, st);
  return launch_cpl<4>(a, k, lossy, pml, st);
}

}  // namespace fdtd

extern "C" int fdtd2d_set_march_config(int cols_per_lane, int warps_per_block, int seg_rows) {
  if (cols_per_lane != 0 && cols_per_lane != 2 && cols_per_lane != 4) return FDTD_ERR_ARG;
  if (seg_rows < 0) return FDTD_ERR_ARG;
  fdtd::g_cfg.cpl = cols_per_lane;
  fdtd::g_cfg.warps = warps_per_block;
  fdtd::g_cfg.seg_rows = seg_rows;
  return FDTD_OK;
}
