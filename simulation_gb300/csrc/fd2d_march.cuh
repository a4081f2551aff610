// Fused, temporally blocked 2D TM update: the hot kernel of fdtd2d_step_n.
//
// This header holds the kernel template; fd2d_march.cu instantiates the
// plain passes and dispatches, fd2d_march_nf*.cu instantiate the passes with
// the fd2d_3_4 extras, one translation unit per DFT frequency count.
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
//     come from the adjacent lane by warp shuffle; there is no __syncthreads;
//   * the i-neighbours come from the row carried in registers.  Segments
//     overlap by K rows (the dependence cone), so warps are independent;
//   * each lane copies its own columns of the next input row (the evolving
//     fields, and naz/nbz, which every level reads again) into per-warp
//     shared-memory rings with cp.async one row ahead, so the levels read
//     shared memory instead of waiting on global loads (+16% at 8192^2,
//     K = 4: 204 -> 236 Gcell-updates/s).  Only the lane that copied a value
//     reads it, so its own cp.async.wait_group is the only wait.
// Passes read one copy of the evolving fields and write the other (ping-pong),
// which makes the overlapping reads race-free.  Out-of-grid lanes/rows load
// zeros and are masked by the same predicates as the reference loops (no D on
// row/column 0, no H on the last row/column), so boundary cells see exactly
// the reference's update.
//
// The per-cell arithmetic is the shared inline formulas of fdtd_common.cuh,
// so a pass of K steps is bitwise identical to K rounds of the per-function
// kernels (dfield -> source -> efield -> hfield).
#pragma once

#include <cstdio>
#include <cstdlib>
#include <type_traits>

#include "fd2d_internal.cuh"

namespace fdtd {
namespace march {


constexpr unsigned FULL = 0xffffffffu;
constexpr int HALO = 4;  // halo columns on each side (>= K, multiple of 4 for aligned vectors)
constexpr int kPlain = -2;        // NFC of the kernels without the fd2d_3_4 extras
constexpr int kExtMinBlocks = 3;  // blocks per SM the extras kernels are held to
constexpr bool kPlainPrefetch = true;  // the plain kernels prefetch rows too (false: direct loads)
constexpr int kWarps = 4;              // warps per block of every fused kernel
constexpr int kTraceNone = 0, kTraceProbe = 1, kTraceRecord = 2;  // what a plain pass keeps besides its output

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
  // plain kernels: the n_gen_lo + n_gen_hi stripes at the grid's left and
  // right edges (which the absorbing layer or the grid boundary make general)
  // have their own, shorter segments (seg_rows_g rows, n_segs_g of them); the
  // other stripes' first and last segments are seg_first rows, the rest
  // seg_rows.  Only the balance of the one wave of warps depends on this.
  int n_gen_lo, n_gen_hi, seg_rows_g, n_segs_g, seg_first;
  int* status;
  int check_finite;
  int probe_i, probe_j;  // Ez trace cell (probe_ez != nullptr)
  float* probe_ez;       // probe_ez[t-1] = ez at the probe after step t
  MarchExt ext;          // TF/SF corrections and the running DFT (EXT kernels)
  RecSet rec[HALO];      // recording passes: rec[s] <- dz, iz, hx, hy after step t0+s+1
  int pml_hint;          // absorbing-layer thickness in cells if known (host: work layout only)
};

// Shared memory per warp beyond the PML columns, in floats (each part a
// multiple of 4): the DFT ring (K+1 rows; lane stride 4*nf floats made an odd
// number of 16-byte units, so 16-byte accesses are conflict-free), the
// twiddles, the field-row ring (2 rows of the 3-6 evolving fields) and the
// material-row ring (K+1 rows of naz and nbz)
__host__ __device__ constexpr int ext_lane_stride(int nf) { return 4 * (nf | 1); }
__host__ __device__ constexpr int ext_nfields(bool lossy, bool pml) { return 3 + (lossy ? 1 : 0) + (pml ? 2 : 0); }
__host__ __device__ constexpr int ext_dft_floats(int k, int nf) {
  return nf > 0 ? (k + 1) * 32 * ext_lane_stride(nf) + ((2 * nf * k + 3) & ~3) : 0;
}
__host__ __device__ constexpr int ext_warp_floats(int k, int nf, bool lossy, bool pml, int w) {
  return ext_dft_floats(k, nf) + 2 * ext_nfields(lossy, pml) * w + (k + 1) * (lossy ? 2 : 1) * w;
}
// dynamic shared memory of a block of `warps` warps with w-column stripes:
// the PML column coefficients (5 rows of w) and the rings above, per warp
__host__ __device__ constexpr size_t march_smem_bytes(int warps, int k, int nf, bool lossy, bool pml, int w,
                                                     bool prefetch) {
  return (size_t)warps * ((pml ? 5 * w : 0) + (prefetch ? ext_warp_floats(k, nf, lossy, pml, w) : 0)) * sizeof(float);
}

struct MarchConfig {
  int cpl = 0;       // columns per lane; 0 = automatic (measured best: 4 for K <= 2, 2 for K >= 3)
  int warps = 4;
  int seg_rows = 0;  // 0 = automatic
  // time of a general row iteration over an interior one (load balance);
  // 0 = the measured best for the stripe width: 8192^2 K = 4 lossy PML,
  // 128-column stripes 386 Gcell/s at 3.5-5 (297 at 2, 349 at 8), 64-column
  // stripes 350 at 2.5 (338 at 3)
  float gen_cost = 0.f;
};

extern MarchConfig g_cfg;  // tuning knob (fdtd2d_set_march_config)

// Shortest automatic segment: 4K rows (the recomputed cone is 2K), at least 8.
// Measured at 1024^2 (adjoint forward/recompute): 8 rows for K <= 2 and 16 for
// K = 4 beat 16/32 by 1.3-2x, because small grids otherwise leave most SMs idle.
constexpr int min_seg_rows(int K) { return K * 4 > 8 ? K * 4 : 8; }

// Passes with the extras for one DFT frequency count: nf = 0..4 compiled in,
// 5..kMarchMaxNf through the runtime-count kernel (fd2d_march_nf*.cu)
int launch_ext_nf0(const MarchArgs& a, int k, bool lossy, bool pml, cudaStream_t st);
int launch_ext_nf1(const MarchArgs& a, int k, bool lossy, bool pml, cudaStream_t st);
int launch_ext_nf2(const MarchArgs& a, int k, bool lossy, bool pml, cudaStream_t st);
int launch_ext_nf3(const MarchArgs& a, int k, bool lossy, bool pml, cudaStream_t st);
int launch_ext_nf4(const MarchArgs& a, int k, bool lossy, bool pml, cudaStream_t st);
int launch_ext_nfrt(const MarchArgs& a, int k, bool lossy, bool pml, cudaStream_t st);

}  // namespace march

namespace {  // kernels are instantiated per translation unit

using namespace march;

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

// global -> shared copy of one lane's accumulator vector, completed by
// cp_async_wait_all in the same thread (no other thread reads it); a zero
// fill instead of the read where !ok (src must still be a valid address)
template <int CPL>
__device__ __forceinline__ void cp_async_acc_zfill(float* smem_dst, const float* gsrc, bool ok) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
  const unsigned n = ok ? 4u * CPL : 0u;
  if constexpr (CPL == 4)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(gsrc), "r"(n) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(d), "l"(gsrc), "r"(n) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_1() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

// one lane's CPL floats from shared memory (rows the lane copied in itself)
template <int CPL>
__device__ __forceinline__ void ld_acc2(const float* p, float (&v)[CPL]) {
  if constexpr (CPL == 4) {
    const float4 x = *reinterpret_cast<const float4*>(p);
    v[0] = x.x; v[1] = x.y; v[2] = x.z; v[3] = x.w;
  } else {
    const float2 x = *reinterpret_cast<const float2*>(p);
    v[0] = x.x; v[1] = x.y;
  }
}

template <int CPL>
__device__ __forceinline__ bool all_finite(const float (&v)[CPL]) {
  bool ok = true;
#pragma unroll
  for (int c = 0; c < CPL; ++c) ok &= isfinite(v[c]);
  return ok;
}

// Prefetch of one row by cp.async (zero fill outside the grid, as ld_row
// does): the evolving fields into a field-ring slot `fr` ([NFA][W], this
// lane's columns), naz/nbz into a material-ring slot `mr`, the DFT
// accumulators of owned cells into a DFT-ring slot `rg`
template <int CPL, bool LOSSY, bool PML>
__device__ __forceinline__ void pf_fields(const MarchArgs& a, float* fr, int row, int nx, int ny, int j0, bool vin) {
  constexpr int W = 32 * CPL;
  constexpr int F_IZ = 3, F_IHX = 3 + (LOSSY ? 1 : 0), F_IHY = F_IHX + 1;
  const bool ok = vin && row < nx;
  const size_t off = ok ? (size_t)row * ny + j0 : 0;
  cp_async_acc_zfill<CPL>(fr + 0 * W, a.in.dz + off, ok);
  cp_async_acc_zfill<CPL>(fr + 1 * W, a.in.hx + off, ok);
  cp_async_acc_zfill<CPL>(fr + 2 * W, a.in.hy + off, ok);
  if (LOSSY) cp_async_acc_zfill<CPL>(fr + F_IZ * W, a.in.iz + off, ok);
  if (PML) {
    cp_async_acc_zfill<CPL>(fr + F_IHX * W, a.in.ihx + off, ok);
    cp_async_acc_zfill<CPL>(fr + F_IHY * W, a.in.ihy + off, ok);
  }
}
template <int CPL, bool LOSSY>
__device__ __forceinline__ void pf_material(const MarchArgs& a, float* mr, int row, int nx, int ny, int j0, bool vin) {
  const bool ok = vin && row >= 0 && row < nx;
  const size_t off = ok ? (size_t)row * ny + j0 : 0;
  cp_async_acc_zfill<CPL>(mr, a.naz + off, ok);
  if (LOSSY) cp_async_acc_zfill<CPL>(mr + 32 * CPL, a.nbz + off, ok);
}
template <int CPL, int NFC, int NFMAX>
__device__ __forceinline__ void pf_dft(const MarchArgs& a, float* rg, int row, int ny, int j0, bool own, size_t ncell,
                                       int nf) {
  const size_t goff = own ? (size_t)row * ny + j0 : 0;
#pragma unroll
  for (int f = 0; f < NFMAX; ++f) {
    if (NFC < 0 && f >= nf) break;
    cp_async_acc_zfill<CPL>(rg + 4 * f, a.ext.r_pt + f * ncell + goff, own);
    cp_async_acc_zfill<CPL>(rg + 4 * f + 2, a.ext.i_pt + f * ncell + goff, own);
  }
}

// The Ez probe (the adjoint's objective trace) is a separate instantiation,
// so the benchmark kernels carry no per-cell probe test.  Plain kernels with
// 64-column stripes are held to four 4-warp blocks per SM (128 registers; the
// K = 4 lossy PML one spills 8 bytes since the row prefetch); left free, the
// compiler takes 138-142 registers and the SM runs three blocks (-9% to -20%
// at 8192^2, K = 4).  128-column stripes need more registers and are left
// free.  The EXT kernels need about 160 and are held to three blocks.
//
// EXT kernels add the fd2d_3_4 extras (fd2d/python/fd2d_3_4.py:90-170) at the
// same points of each cell's update as the per-step kernels, so they stay
// bitwise equal to them:
//   * TF/SF: after D (and the point source), inctdz adds +-hxi/2 on the box's
//     two j-edges; after H, incthx adds +-ezi/2 to hx on the two j-edges and
//     incthy +-ezi[j]/2 to hy on the two i-edges.  The incident line is a 1D
//     problem of its own, advanced ahead of the pass (k_inc_line), so the
//     pass only reads one table row per time step;
//   * DFT: each owned cell's accumulators enter a per-warp shared-memory ring
//     of K+1 rows by cp.async with the row's fields (one global read), take
//     one fma per level and frequency there, and leave at level K (one
//     global write): 16*nf bytes per cell per pass instead of per step, in
//     the reference's summation order.
// The level loop is straight-line code that the compiler interleaves across
// levels; the extras keep it so: edge tests are per-cell selects on uniform
// table loads, the DFT count is a template constant (NFC = 0..4; NFC = -1
// reads it at run time) and the ring is updated for every row and lane, with
// zero-filled copies and predicated stores where the warp does not own the
// cell.  Branches there cost the EXT kernel 40% at 2048^2.  The edge logic
// is compiled into the general form of the iteration only (TF = true when
// the TF/SF source is on): the interior form runs away from the box's edge
// rows and outside the stripes that hold its edge columns.
// One row iteration of a warp's march, in two forms sharing the same register
// state:
//   * the general form (GEN) handles every case: PML coefficients per row and
//     column, the grid's first/last rows and columns (the reference loops'
//     bounds), the point source, the probe trace and the TF/SF edges;
//   * the interior form (INT) runs where none of these can occur in any row
//     the iteration touches (rows r-K .. r) nor in the warp's columns: unit
//     PML coefficients (d_update_unit / h_update_pml_unit give the same values
//     as the general formulas there), no bounds tests, no source or probe
//     test.  It cuts the per-cell work roughly in half.
// The warp decides per iteration, on warp-uniform data: its columns are
// classified once (cint), its rows 32 at a time by a ballot over the lanes
// (one row per lane, see row_ok) into `run`, the count of good rows ending at
// the row entering level 1.  An iteration is interior when cint and run > K.
template <int K, int CPL, bool LOSSY, bool PML, int WARPS, int TRACE, int NFC, bool TF>
__device__ __forceinline__ void march_body(const MarchArgs& a, const int stripe, const int i_s, const int i_e) {
  constexpr bool PROBE = TRACE == kTraceProbe;  // Ez at one cell every step
  constexpr bool REC = TRACE == kTraceRecord;   // dz, iz, hx, hy after every step
  constexpr bool EXT = NFC != kPlain;
  constexpr bool TFS = EXT && TF;  // this body applies the TF/SF edge corrections
  constexpr bool PF = EXT || kPlainPrefetch;  // rows prefetched by cp.async into shared rings
  constexpr bool DFT = EXT && NFC != 0;  // NFC = -1: count at run time (1..kMarchMaxNf)
  constexpr int NFMAX = NFC >= 0 ? NFC : kMarchMaxNf;
  constexpr int W = 32 * CPL;
  constexpr int OUTW = W - 2 * HALO;
  static_assert(K >= 1 && K <= HALO, "steps per pass must not exceed the halo");
  static_assert(!(EXT && TRACE != kTraceNone), "the probe trace and the records are not kept by EXT kernels");
  // per warp: gy2, gy3, fy1, fy2, fy3 of its columns (PML); then (nf > 0)
  // the DFT ring [K+1 rows][32 lanes][nf][re0, re1, im0, im1] (lane stride
  // padded to an odd number of 16-byte units: conflict-free vector access)
  // and the twiddles [K][nf][cos, -sin]; then the field-row ring [2][NFA][W]
  // and the material-row ring [K+1][NMA][W]
  static_assert(!EXT || CPL == 2, "EXT kernels use 64-column stripes");
  extern __shared__ float smem[];

  const int lane = threadIdx.x & 31;
  const int wid = threadIdx.x >> 5;
  const int nx = a.nx, ny = a.ny;
  const int jw0 = stripe * OUTW - HALO;              // first column of the warp's stripe
  const int j0 = jw0 + lane * CPL;                   // first column of this lane (multiple of 4 or 2)
  const bool vin = (j0 >= 0) && (j0 + CPL <= ny);    // ny % 4 == 0: a vector is wholly in or out
  const bool vout = vin && (lane * CPL >= HALO) && (lane * CPL < HALO + OUTW);

  const int nf = NFC >= 0 ? NFC : (EXT ? a.ext.nf : 0);
  // rows are prefetched one iteration ahead by cp.async; M rows of the
  // DFT and material rings are in use at once (levels 1..K and the next row)
  constexpr int M = K + 1;
  constexpr int NFA = ext_nfields(LOSSY, PML);  // fields in the row ring: dz, hx, hy, [iz], [ihx, ihy]
  constexpr int NMA = LOSSY ? 2 : 1;            // naz, [nbz]
  constexpr int F_IZ = 3, F_IHX = 3 + (LOSSY ? 1 : 0), F_IHY = F_IHX + 1;
  const int ls = ext_lane_stride(nf);
  const int wst = (PML ? 5 * W : 0) + (PF ? ext_warp_floats(K, nf, LOSSY, PML, W) : 0);
  float* const wsm = smem + wid * wst;
  float* cg = wsm + lane * CPL;
  float* const ring = wsm + (PML ? 5 * W : 0);
  float* const tw = ring + M * 32 * ls;
  float* const fring = ring + ext_dft_floats(K, nf) + lane * CPL;  // [2][NFA][W], this lane's columns
  float* const mring = fring + 2 * NFA * W;                         // [M][NMA][W]
  // columns: interior if every column of the stripe lies in 1 .. ny-2 with
  // unit PML coefficients, and neither the source nor the probe is among them
  bool col_ok = (j0 >= 1) && (j0 + CPL - 1 <= ny - 2);
  if (PML) {
#pragma unroll
    for (int c = 0; c < CPL; ++c) {
      const int j = j0 + c;
      const bool ok = (j >= 0) && (j < ny);
      const float gy2 = ok ? __ldg(a.pml.gy2 + j) : 1.f;
      const float gy3 = ok ? __ldg(a.pml.gy3 + j) : 1.f;
      const float fy1 = ok ? __ldg(a.pml.fy1 + j) : 0.f;
      const float fy2 = ok ? __ldg(a.pml.fy2 + j) : 1.f;
      const float fy3 = ok ? __ldg(a.pml.fy3 + j) : 1.f;
      cg[0 * W + c] = gy2;
      cg[1 * W + c] = gy3;
      cg[2 * W + c] = fy1;
      cg[3 * W + c] = fy2;
      cg[4 * W + c] = fy3;
      col_ok &= gy2 == 1.f && gy3 == 1.f && fy1 == 0.f && fy2 == 1.f && fy3 == 1.f;
    }
    __syncwarp();
  }
  const bool src_here = a.src_kind != FDTD_SRC_NONE && a.src_j >= jw0 && a.src_j < jw0 + W;
  const bool probe_here = PROBE && a.probe_j >= jw0 && a.probe_j < jw0 + W;
  // TF/SF: the box's edge columns (inctdz at np-1 and ny-np, incthx at np-2
  // and ny-np, for rows np-1 .. nx-np) make a stripe general; the edge rows
  // np-2 and nx-np (incthy) are bad rows for every stripe (row_ok)
  const int np_edge = TFS ? a.ext.tfsf_npml : 0;
  if (np_edge > 0) {
#pragma unroll
    for (int c = 0; c < CPL; ++c) {
      const int j = j0 + c;
      col_ok &= j != np_edge - 2 && j != np_edge - 1 && j != ny - np_edge;
    }
  }
  const bool cint = __all_sync(FULL, col_ok);
  if constexpr (DFT) {
    for (int x = lane; x < K * nf; x += 32) {
      const int s = x / nf, f = x - s * nf;
      const size_t row = (size_t)(a.t0 + s) * nf + f;  // table row t-1 = t0+s of step t0+s+1
      tw[2 * x] = __ldg(a.ext.dft_cos + row);
      tw[2 * x + 1] = -__ldg(a.ext.dft_sin + row);
    }
    __syncwarp();
  }
  // TF/SF edge columns of this lane: bit 4c+0 D += hxi[np-2]/2, 4c+1 D -=
  // hxi[ny-np]/2, 4c+2 hx += ezi[np-1]/2, 4c+3 hx -= ezi[ny-np]/2
  // (TF bodies run only with np > 0: k_march picks them for edge warps)
  const int np = TFS ? a.ext.tfsf_npml : 0;
  unsigned tcol = 0;
  if (TFS && np > 0) {
#pragma unroll
    for (int c = 0; c < CPL; ++c) {
      const int j = j0 + c;
      if (j == np - 1) tcol |= 1u << (4 * c);
      if (j == ny - np) tcol |= 2u << (4 * c);
      if (j == np - 2) tcol |= 4u << (4 * c);
      if (j == ny - np) tcol |= 8u << (4 * c);
    }
  }
  // rows: bit l of row_ok(b) says row b+l may be touched by an interior
  // iteration (1 .. nx-2, unit PML row coefficients, not the source's or the
  // probe's row when its column is in the stripe)
  auto row_ok = [&](int b) -> unsigned {
    const int row = b + lane;
    bool g = row >= 1 && row <= nx - 2;
    if (PML && g)
      g = __ldg(a.pml.gx2 + row) == 1.f && __ldg(a.pml.gx3 + row) == 1.f && __ldg(a.pml.fx1 + row) == 0.f &&
          __ldg(a.pml.fx2 + row) == 1.f && __ldg(a.pml.fx3 + row) == 1.f;
    if (src_here && row == a.src_i) g = false;
    if (probe_here && row == a.probe_i) g = false;
    if (np_edge > 0 && (row == np_edge - 2 || row == nx - np_edge)) g = false;
    return __ballot_sync(FULL, g);
  };

  // level state: values of the row each level will complete next
  float p_hy[K][CPL], p_hx[K][CPL], p_ihx[K][CPL], p_ihy[K][CPL], p_ez[K][CPL], p_dz[K][CPL], p_iz[K][CPL];
#pragma unroll
  for (int s = 0; s < K; ++s)
#pragma unroll
    for (int c = 0; c < CPL; ++c) {
      p_hy[s][c] = p_hx[s][c] = p_ihx[s][c] = p_ihy[s][c] = 0.f;
      p_ez[s][c] = p_dz[s][c] = p_iz[s][c] = 0.f;
    }

  const int r_begin = max(0, i_s - K);
  const int r_end = i_e - 1 + K;
  bool finite_ok = true;
  const size_t ncell = (size_t)nx * ny;
  int mk = PF ? r_begin % M : 0;  // ring slot of row r (level 1's row); level s uses slot (r - s) mod M
  if constexpr (PF) {
    // rows the levels 2..K read before row r_begin, then row r_begin itself
    int ms = ((r_begin - K + 1) % M + M) % M;
    for (int q = r_begin - K + 1; q < r_begin; ++q) {
      pf_material<CPL, LOSSY>(a, mring + ms * NMA * W, q, nx, ny, j0, vin);
      ms = (ms + 1 == M) ? 0 : ms + 1;
    }
    pf_material<CPL, LOSSY>(a, mring + mk * NMA * W, r_begin, nx, ny, j0, vin);
    pf_fields<CPL, LOSSY, PML>(a, fring + (r_begin & 1) * NFA * W, r_begin, nx, ny, j0, vin);
    if constexpr (DFT)
      pf_dft<CPL, NFC, NFMAX>(a, ring + (mk * 32 + lane) * ls, r_begin, ny, j0, vout && r_begin >= i_s && r_begin < i_e,
                              ncell, nf);
    cp_async_commit();
  }
  // good-row run before the first iteration (rows r_begin-K .. r_begin-1)
  int gbase = r_begin - K;
  unsigned gmask = cint ? row_ok(gbase) : 0u;
  int run = 0;
  if (cint)
    for (int q = r_begin - K; q < r_begin; ++q) run = ((gmask >> (q - gbase)) & 1u) ? run + 1 : 0;

  // one row iteration: row r enters level 1, level s completes row r-s-1
  auto iterate = [&](const int r, auto int_tag) {
    constexpr bool INT = decltype(int_tag)::value;
    float in_dz[CPL], in_iz[CPL], in_hx[CPL], in_hy[CPL], in_ihx[CPL], in_ihy[CPL];
    if constexpr (PF) {
      // row r+1 starts its way in; row r's copies (issued one iteration ago) complete
      const int mn = (mk + 1 == M) ? 0 : mk + 1;
      pf_material<CPL, LOSSY>(a, mring + mn * NMA * W, r + 1, nx, ny, j0, vin);
      pf_fields<CPL, LOSSY, PML>(a, fring + ((r + 1) & 1) * NFA * W, r + 1, nx, ny, j0, vin);
      if constexpr (DFT)
        pf_dft<CPL, NFC, NFMAX>(a, ring + (mn * 32 + lane) * ls, r + 1, ny, j0, vout && r + 1 >= i_s && r + 1 < i_e,
                                ncell, nf);
      cp_async_commit();
      cp_async_wait_1();
      const float* fr = fring + (r & 1) * NFA * W;
      ld_acc2<CPL>(fr + 0 * W, in_dz);
      ld_acc2<CPL>(fr + 1 * W, in_hx);
      ld_acc2<CPL>(fr + 2 * W, in_hy);
      if (LOSSY) ld_acc2<CPL>(fr + F_IZ * W, in_iz);
      else {
#pragma unroll
        for (int c = 0; c < CPL; ++c) in_iz[c] = 0.f;
      }
      if (PML) {
        ld_acc2<CPL>(fr + F_IHX * W, in_ihx);
        ld_acc2<CPL>(fr + F_IHY * W, in_ihy);
      } else {
#pragma unroll
        for (int c = 0; c < CPL; ++c) in_ihx[c] = in_ihy[c] = 0.f;
      }
    } else {
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
      if constexpr (PF) {
        const float* mr = mring + (mk >= s ? mk - s : mk - s + M) * NMA * W;
        ld_acc2<CPL>(mr, naz);
        if (LOSSY) ld_acc2<CPL>(mr + W, nbz);
      } else {
        const bool ok = qok && vin;
        const size_t off = ok ? (size_t)q * ny + j0 : 0;
        ld_row<CPL>(a.naz + off, ok, naz);
        if (LOSSY) ld_row<CPL>(a.nbz + off, ok, nbz);
      }
      float gx3q = 1.f, gx2q = 1.f;
      if (!INT && PML && qok) {
        gx3q = __ldg(a.pml.gx3 + q);
        gx2q = __ldg(a.pml.gx2 + q);
      }
      const float hx_left = __shfl_up_sync(FULL, in_hx[CPL - 1], 1);
      const bool drow = (q >= 1) && (q < nx);
      bool d_tf = false;  // inctdz row (warp-uniform); the interior form meets no TF/SF edge
      float hxi_lo = 0.f, hxi_hi = 0.f;
      if (TFS && !INT) {
        d_tf = q >= np - 1 && q <= nx - np;
        hxi_lo = __ldg(a.ext.inc_h + 2 * s);
        hxi_hi = __ldg(a.ext.inc_h + 2 * s + 1);
      }
      float nd[CPL], ne[CPL], niz[CPL];
#pragma unroll
      for (int c = 0; c < CPL; ++c) {
        const int j = j0 + c;
        const float hxm = (c == 0) ? hx_left : in_hx[c - 1];
        float d = in_dz[c];
        if constexpr (INT) {
          d = d_update_unit(d, in_hy[c], p_hy[s][c], in_hx[c], hxm);
        } else {
          if (drow && j >= 1 && j < ny) {
            const float gy2 = PML ? cg[0 * W + c] : 1.f;
            const float gy3 = PML ? cg[1 * W + c] : 1.f;
            d = d_update(d, in_hy[c], p_hy[s][c], in_hx[c], hxm, gx3q, gy3, gx2q, gy2);
          }
          if (a.src_kind != FDTD_SRC_NONE && q == a.src_i && j == a.src_j) {
            const float v = __ldg(a.src_table + a.t0 + s);
            d = (a.src_kind == FDTD_SRC_HARD) ? v : __fadd_rn(d, v);
          }
          if (TFS) {
            const float d_lo = __fmaf_rn(0.5f, hxi_lo, d), d_hi = __fmaf_rn(-0.5f, hxi_hi, d);
            d = (d_tf && (tcol & (1u << (4 * c)))) ? d_lo : d;
            d = (d_tf && (tcol & (2u << (4 * c)))) ? d_hi : d;
          }
        }
        float izv = in_iz[c];
        const float e = LOSSY ? e_update_lossy(d, izv, naz[c], nbz[c]) : e_update(d, naz[c]);
        nd[c] = d;
        niz[c] = izv;
        ne[c] = e;
        // the probe cell's Ez is recorded by the warp that owns it (output
        // column, row inside the segment), where every level is valid
        if (!INT && PROBE && q == a.probe_i && j == a.probe_j && vout && q >= i_s && q < i_e)
          a.probe_ez[a.t0 + s] = e;
      }

      // ---- running DFT of row q at step t0+s+1 (stored where owned)
      if constexpr (DFT) {
        const bool own = vout && q >= i_s && q < i_e;
        const size_t goff = own ? (size_t)q * ny + j0 : 0;
        const int slot = mk >= s ? mk - s : mk - s + M;
        float* rg = ring + (slot * 32 + lane) * ls;
        const float2* tws = reinterpret_cast<const float2*>(tw) + s * nf;
#pragma unroll
        for (int f = 0; f < NFMAX; ++f) {
          if (NFC < 0 && f >= nf) break;
          float4 v = *reinterpret_cast<const float4*>(rg + 4 * f);  // re0, re1, im0, im1
          const float2 w = tws[f];                                  // cos, -sin
          v.x = __fmaf_rn(w.x, ne[0], v.x);
          v.y = __fmaf_rn(w.x, ne[1], v.y);
          v.z = __fmaf_rn(w.y, ne[0], v.z);
          v.w = __fmaf_rn(w.y, ne[1], v.w);
          if (s == K - 1) {
            if (own) {
              __stcs(reinterpret_cast<float2*>(a.ext.r_pt + f * ncell + goff), make_float2(v.x, v.y));
              __stcs(reinterpret_cast<float2*>(a.ext.i_pt + f * ncell + goff), make_float2(v.z, v.w));
            }
          } else {
            *reinterpret_cast<float4*>(rg + 4 * f) = v;
          }
        }
      }

      // ---- H on row qc (needs Ez of rows qc and q at this level)
      const float ez_right = __shfl_down_sync(FULL, p_ez[s][0], 1);
      const bool hrow = (qc >= 0) && (qc <= nx - 2);
      bool hx_tf = false, hy_tf = false;  // incthx / incthy rows (warp-uniform)
      float ezi_lo = 0.f, ezi_hi = 0.f, hy_w = 0.f;
      float ezr[CPL];
#pragma unroll
      for (int c = 0; c < CPL; ++c) ezr[c] = 0.f;
      if (TFS && !INT) {
        const float* erow = a.ext.inc_e + (size_t)s * ny;
        hx_tf = qc >= np - 1 && qc <= nx - np;
        ezi_lo = __ldg(erow + max(np - 1, 0));
        ezi_hi = __ldg(erow + min(ny - np, ny - 1));
        hy_tf = np > 0 && (qc == np - 2 || qc == nx - np);
        hy_w = (qc == np - 2) ? -0.5f : 0.5f;
        ld_row<CPL>(erow + (vin ? j0 : 0), vin && hy_tf, ezr);
      }
      float fx1 = 0.f, fx2 = 1.f, fx3 = 1.f;
      if (!INT && PML && hrow) {
        fx1 = __ldg(a.pml.fx1 + qc);
        fx2 = __ldg(a.pml.fx2 + qc);
        fx3 = __ldg(a.pml.fx3 + qc);
      }
      float ohx[CPL], ohy[CPL], oihx[CPL], oihy[CPL];
#pragma unroll
      for (int c = 0; c < CPL; ++c) {
        const int j = j0 + c;
        float hxv = p_hx[s][c], hyv = p_hy[s][c], ihxv = p_ihx[s][c], ihyv = p_ihy[s][c];
        const float er = (c == CPL - 1) ? ez_right : p_ez[s][c + 1];
        if constexpr (INT) {
          if (PML)
            h_update_pml_unit(p_ez[s][c], er, ne[c], hxv, hyv, ihxv, ihyv);
          else
            h_update_free(p_ez[s][c], er, ne[c], hxv, hyv);
        } else if (hrow && j >= 0 && j <= ny - 2) {
          if (PML)
            h_update_pml(p_ez[s][c], er, ne[c], hxv, hyv, ihxv, ihyv, fx1, fx2, fx3, cg[2 * W + c], cg[3 * W + c],
                         cg[4 * W + c]);
          else
            h_update_free(p_ez[s][c], er, ne[c], hxv, hyv);
          if (TFS) {
            const float x_lo = __fmaf_rn(0.5f, ezi_lo, hxv), x_hi = __fmaf_rn(-0.5f, ezi_hi, hxv);
            const float y_c = __fmaf_rn(hy_w, ezr[c], hyv);
            hxv = (hx_tf && (tcol & (4u << (4 * c)))) ? x_lo : hxv;
            hxv = (hx_tf && (tcol & (8u << (4 * c)))) ? x_hi : hxv;
            hyv = (hy_tf && j >= np - 1 && j <= ny - np) ? y_c : hyv;
          }
        }
        ohx[c] = hxv;
        ohy[c] = hyv;
        oihx[c] = ihxv;
        oihy[c] = ihyv;
      }

      // ---- recording passes store every level's completed row: the state
      //      after step t0+s+1 (the values level K stores for s = K-1)
      if (REC && vout && qc >= i_s && qc < i_e) {
        const size_t off = (size_t)qc * ny + j0;
        st_row<CPL>(a.rec[s].dz + off, p_dz[s]);
        if (LOSSY) st_row<CPL>(a.rec[s].iz + off, p_iz[s]);
        st_row<CPL>(a.rec[s].hx + off, ohx);
        st_row<CPL>(a.rec[s].hy + off, ohy);
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
    if constexpr (PF) mk = (mk + 1 == M) ? 0 : mk + 1;
  };

  for (int r = r_begin; r <= r_end; ++r) {
    bool interior = false;
    if (cint) {
      if (r - gbase >= 32) {
        gbase += 32;
        gmask = row_ok(gbase);
      }
      run = ((gmask >> (r - gbase)) & 1u) ? run + 1 : 0;
      interior = run > K;  // rows r-K .. r all good
    }
    if (interior)
      iterate(r, std::true_type{});
    else
      iterate(r, std::false_type{});
  }
  if constexpr (PF) cp_async_wait_all();  // the copies of row r_end+1 land before the warp leaves
  if (a.check_finite && __any_sync(FULL, !finite_ok) && lane == 0) raise_status(a.status, ST_NONFINITE);
}

// Warp -> work of the plain kernels (layout: plain_layout): warps
// 0 .. n_int*n_segs-1 take the stripes away from the edges, the rest the
// general stripes at either edge with their shorter segments.  False: no work.
__host__ __device__ inline bool plain_work(const MarchArgs& a, int gw, int& stripe, int& i_s, int& i_e) {
  const int n_int = a.n_stripes - a.n_gen_lo - a.n_gen_hi;
  const int n_main = n_int * a.n_segs;
  if (gw < n_main) {
    stripe = a.n_gen_lo + gw % n_int;
    const int seg = gw / n_int;
    i_s = seg == 0 ? 0 : a.seg_first + (seg - 1) * a.seg_rows;
    i_e = (seg == a.n_segs - 1) ? a.nx : (seg == 0 ? a.seg_first : i_s + a.seg_rows);
  } else {
    const int n_gen = a.n_gen_lo + a.n_gen_hi;
    if (n_gen == 0) return false;
    const int k = gw - n_main;
    const int g = k % n_gen, seg = k / n_gen;
    if (seg >= a.n_segs_g) return false;
    stripe = g < a.n_gen_lo ? g : a.n_stripes - n_gen + g;
    i_s = seg * a.seg_rows_g;
    i_e = i_s + a.seg_rows_g;
  }
  i_e = i_e < a.nx ? i_e : a.nx;
  return i_s < i_e;
}

// Warp -> work: plain_work for every kernel.  With the TF/SF source on, all
// warps carry the edge logic in their general iterations (TF = true); the
// interior iterations skip it where no edge can be met.
template <int K, int CPL, bool LOSSY, bool PML, int WARPS, int TRACE, int NFC>
__global__ void __launch_bounds__(WARPS * 32, CPL == 2 ? (NFC == kPlain ? 4 : kExtMinBlocks) : 1)
    k_march(const MarchArgs a) {
  const int gw = blockIdx.x * WARPS + (threadIdx.x >> 5);
  if constexpr (NFC == kPlain) {
    int stripe, i_s, i_e;
    if (!plain_work(a, gw, stripe, i_s, i_e)) return;  // whole warp leaves; nothing below syncs the block
    march_body<K, CPL, LOSSY, PML, WARPS, TRACE, NFC, false>(a, stripe, i_s, i_e);
  } else {
    int stripe, i_s, i_e;
    if (!plain_work(a, gw, stripe, i_s, i_e)) return;
    if (a.ext.tfsf_npml > 0)
      march_body<K, CPL, LOSSY, PML, WARPS, TRACE, NFC, true>(a, stripe, i_s, i_e);
    else
      march_body<K, CPL, LOSSY, PML, WARPS, TRACE, NFC, false>(a, stripe, i_s, i_e);
  }
}

// Work layout of the fused kernels' single wave of warps (MarchArgs).  The
// stripes that reach column 0, column ny-1 or (with the pml_hint) the
// absorbing layer or the TF/SF box's edge columns run general iterations
// throughout; they get gen_cost times
// as many segments.  In the other stripes only the rows of the layer and the
// grid's first/last rows (plus the K-row cone) iterate in the general form,
// so their first and last segments are shortened by that extra time.
template <int K, int CPL>
long plain_layout(MarchArgs& a, long resident, float G) {
  constexpr int W = 32 * CPL, OUTW = W - 2 * HALO;
  // the absorbing layer and, with TF/SF on, the box's edges (at np-2 ..
  // n-np, next to the layer in the reference's programs)
  const int P = std::max(a.pml_hint > 0 ? a.pml_hint : 0, a.ext.tfsf_npml > 0 ? a.ext.tfsf_npml + 1 : 0);
  auto general = [&](int s) {
    const int lo = s * OUTW - HALO, hi = lo + W - 1;
    return lo < std::max(P, 1) || hi > a.ny - 2 - P;
  };
  int glo = 0, ghi = 0;
  while (glo < a.n_stripes && general(glo)) ++glo;
  while (ghi < a.n_stripes - glo && general(a.n_stripes - 1 - ghi)) ++ghi;
  const int n_int = a.n_stripes - glo - ghi, n_gen = glo + ghi;
  const int mn = min_seg_rows(K);
  if (!(G >= 1.f)) G = 1.f;
  long n_segs = (long)((double)resident / ((double)n_int + (double)G * n_gen));
  if (n_segs < 1) n_segs = 1;
  const long n_segs_g = std::max(1L, (long)(G * n_segs));
  const int rg = std::max((int)((a.nx + n_segs_g - 1) / n_segs_g), mn);
  a.seg_rows_g = rg;
  a.n_segs_g = (a.nx + rg - 1) / rg;
  const int T = (int)((G - 1.f) * (float)(P + K + 1));
  int L = a.nx, f = a.nx, ns = 1;
  if (n_segs > 1) {
    L = std::max((int)((a.nx + 2L * T + n_segs - 1) / n_segs), mn);
    f = std::min(std::max(L - T, mn), a.nx);
    ns = a.nx <= f ? 1 : 1 + (a.nx - f + L - 1) / L;
  }
  a.seg_rows = L;
  a.seg_first = f;
  a.n_segs = ns;
  a.n_gen_lo = glo;
  a.n_gen_hi = ghi;
  return (long)n_int * ns + (long)n_gen * a.n_segs_g;
}

template <int K, int CPL, bool LOSSY, bool PML, int TRACE, int NFC = kPlain>
int launch_t(const MarchArgs& a0, int warps_cfg, int seg_cfg, cudaStream_t st) {
  constexpr int WARPS = kWarps;
  (void)warps_cfg;
  MarchArgs a = a0;
  constexpr int W = 32 * CPL;
  constexpr int OUTW = W - 2 * HALO;
  auto kern = k_march<K, CPL, LOSSY, PML, WARPS, TRACE, NFC>;
  constexpr bool EXT = NFC != kPlain;
  constexpr bool PF = EXT || kPlainPrefetch;
  const int nf = NFC >= 0 ? NFC : (EXT ? a.ext.nf : 0);
  const size_t smem = march_smem_bytes(WARPS, K, nf, LOSSY, PML, W, PF);
  if (smem > 48 * 1024) {
    const cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) {
      fdtd_host::note_cuda_error(e);
      return FDTD_ERR_CUDA;
    }
  }
  a.n_stripes = (a.ny + OUTW - 1) / OUTW;
  int seg_rows = seg_cfg;
  long resident = 0;
  if (seg_rows <= 0) {
    int dev = 0, nsm = 0, blocks_per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, kern, WARPS * 32, smem);
    if (blocks_per_sm < 1) blocks_per_sm = 1;
    resident = (long)nsm * blocks_per_sm * WARPS;
    // one wave of warps: n_stripes * n_segs ~= resident warps
    long n_segs = resident / a.n_stripes;
    if (n_segs < 1) n_segs = 1;
    seg_rows = (int)((a.nx + n_segs - 1) / n_segs);
    // keep the recomputed cone (2K rows per segment) small
    seg_rows = std::max(seg_rows, min_seg_rows(K));
  }
  a.seg_rows = seg_rows;
  a.n_segs = (a.nx + seg_rows - 1) / seg_rows;
  a.seg_first = seg_rows;
  a.n_gen_lo = a.n_gen_hi = 0;
  a.seg_rows_g = seg_rows;
  a.n_segs_g = 0;
  long warps = (long)a.n_stripes * a.n_segs;
  if (resident > 0) {
    // measured defaults: plain 128-column 4.0, plain 64-column 2.5, with the
    // fd2d_3_4 extras 2.0 (2048^2: 108.6 Gcell/s; 84 at 1, 94-105 at 2.5-3)
    const float G = g_cfg.gen_cost > 0.f ? g_cfg.gen_cost : (EXT ? 2.0f : (CPL == 4 ? 4.0f : 2.5f));
    warps = plain_layout<K, CPL>(a, resident, G);
  }
  const int blocks = (int)((warps + WARPS - 1) / WARPS);
  kern<<<blocks, WARPS * 32, smem, st>>>(a);
  return fdtd_host::check_launch();
}

template <int NFC, int K>
int launch_k_ext(const MarchArgs& a, bool lossy, bool pml, cudaStream_t st) {
  if (lossy && pml) return launch_t<K, 2, true, true, false, NFC>(a, g_cfg.warps, g_cfg.seg_rows, st);
  if (lossy) return launch_t<K, 2, true, false, false, NFC>(a, g_cfg.warps, g_cfg.seg_rows, st);
  if (pml) return launch_t<K, 2, false, true, false, NFC>(a, g_cfg.warps, g_cfg.seg_rows, st);
  return launch_t<K, 2, false, false, false, NFC>(a, g_cfg.warps, g_cfg.seg_rows, st);
}

// 64-column stripes only: the DFT ring and the edge masks do not fit the
// 128-column kernel's registers.
template <int NFC>
int launch_ext_nfc(const MarchArgs& a, int k, bool lossy, bool pml, cudaStream_t st) {
  switch (k) {
    case 1: return launch_k_ext<NFC, 1>(a, lossy, pml, st);
    case 2: return launch_k_ext<NFC, 2>(a, lossy, pml, st);
    case 3: return launch_k_ext<NFC, 3>(a, lossy, pml, st);
    case 4: return launch_k_ext<NFC, 4>(a, lossy, pml, st);
    default: return FDTD_ERR_ARG;
  }
}

}  // namespace
}  // namespace fdtd
