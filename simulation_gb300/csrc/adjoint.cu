// Reverse-time (adjoint) step of the lossy 2D TM update with PML, and the
// out-of-place fused pass used to recompute forward states between checkpoints.
//
// No counterpart in the reference (which only runs forward); the forward map
// being differentiated is the reference's step, fd2d/python/fd2d_3_2.py:62-88
// with the lossy E update of fd2d/python/fd2d_3_4.py:131-136 and a point
// source after the D update.
//
// Forward step t maps x = (dz, iz, hx, hy, ihx, ihy) to x':
//   dz' = ca*dz + cb*curl(hy, hx)       ca = gx3*gy3, cb = 0.5*gx2*gy2  (i, j >= 1)
//   dz'[src] = v (hard) or += v (soft)
//   ez  = naz*(dz' - iz);  iz' = iz + nbz*ez
//   cx = ez - ez[j+1], cy = ez - ez[i+1];  ihx' = ihx + cx;  ihy' = ihy + cy
//   hx' = fy3*hx + fy2*(0.5*cx + fx1*ihx');  hy' = fx3*hy - fx2*(0.5*cy + fy1*ihy')
// and the objective adds w/2 * ez[probe]^2 per step (J = sum ez^2 for w = 2).
// Given the adjoints L' of x' this computes the adjoints L of x and adds
// dJ/dnaz, dJ/dnbz on a design box.  L(dz) at a cell needs L'(dz) of its +i
// and +j neighbours after they received their E terms, so the step is either
// two kernels over the grid (fdtd2d_adjoint_step, in place) or one tiled
// kernel with a one-cell halo of that temporary (k_adj_fused, out of place):
//   A: recompute dz', ez at the cell from x; L(ez) from the H adjoints of the
//      cell and its (i, j-1), (i-1, j) neighbours (+ probe seed); E backward;
//      writes L'(dz)+E terms to a temporary and L(iz) in place; gradients;
//   B: D backward: L(dz) = ca*T, L(hy) += cb*T - cb[i+1]*T[i+1],
//      L(hx) += -cb*T + cb[j+1]*T[j+1]; H backward for hx, hy, ihx, ihy.
#include <type_traits>

#include "fd2d_internal.cuh"

namespace fdtd {

namespace {

struct AdjArgs {
  int nx, ny, t;
  fdtd2d_pml pml;
  const float* naz;
  const float* nbz;
  int src_kind, src_i, src_j;
  const float* src_table;
  fdtd2d_fields fwd;  // state before step t
  fdtd2d_fields fwd0;  // state before step t-1 (the two-step kernel only)
  fdtd2d_fields adj;  // adjoints after step t (read)
  fdtd2d_fields out;  // adjoints before step t (written; the same arrays as adj for the two-kernel step)
  float* tmp;
  int probe_i, probe_j;
  float probe_w;
  fdtd2d_box box;
  float* grad_naz;
  float* grad_nbz;
};

// Where the per-cell functions below read the state: straight from global
// memory (GlobalCells), or from a block's shared-memory copy of its tile and
// halo (TileCells).  Both give the same values, so every form of the reverse
// step does the same arithmetic on the same operands.
struct GlobalCells {
  const AdjArgs& a;
  __device__ __forceinline__ size_t n(int i, int j) const { return (size_t)i * a.ny + j; }
  __device__ __forceinline__ float fdz(int i, int j) const { return __ldg(a.fwd.dz + n(i, j)); }
  __device__ __forceinline__ float fiz(int i, int j) const { return __ldg(a.fwd.iz + n(i, j)); }
  __device__ __forceinline__ float fhx(int i, int j) const { return __ldg(a.fwd.hx + n(i, j)); }
  __device__ __forceinline__ float fhy(int i, int j) const { return __ldg(a.fwd.hy + n(i, j)); }
  __device__ __forceinline__ float naz(int i, int j) const { return __ldg(a.naz + n(i, j)); }
  __device__ __forceinline__ float nbz(int i, int j) const { return __ldg(a.nbz + n(i, j)); }
  __device__ __forceinline__ float ldz(int i, int j) const { return __ldg(a.adj.dz + n(i, j)); }
  __device__ __forceinline__ float liz(int i, int j) const { return __ldg(a.adj.iz + n(i, j)); }
  __device__ __forceinline__ float lhx(int i, int j) const { return __ldg(a.adj.hx + n(i, j)); }
  __device__ __forceinline__ float lhy(int i, int j) const { return __ldg(a.adj.hy + n(i, j)); }
  __device__ __forceinline__ float lihx(int i, int j) const { return __ldg(a.adj.ihx + n(i, j)); }
  __device__ __forceinline__ float lihy(int i, int j) const { return __ldg(a.adj.ihy + n(i, j)); }  // PML profile vectors (read through the cache)
  __device__ __forceinline__ float fx1(int i) const { return __ldg(a.pml.fx1 + i); }
  __device__ __forceinline__ float fx2(int i) const { return __ldg(a.pml.fx2 + i); }
  __device__ __forceinline__ float fx3(int i) const { return __ldg(a.pml.fx3 + i); }
  __device__ __forceinline__ float gx2(int i) const { return __ldg(a.pml.gx2 + i); }
  __device__ __forceinline__ float gx3(int i) const { return __ldg(a.pml.gx3 + i); }
  __device__ __forceinline__ float fy1(int j) const { return __ldg(a.pml.fy1 + j); }
  __device__ __forceinline__ float fy2(int j) const { return __ldg(a.pml.fy2 + j); }
  __device__ __forceinline__ float fy3(int j) const { return __ldg(a.pml.fy3 + j); }
  __device__ __forceinline__ float gy2(int j) const { return __ldg(a.pml.gy2 + j); }
  __device__ __forceinline__ float gy3(int j) const { return __ldg(a.pml.gy3 + j); }
};

// UNIT: the tile's rows and columns all have unit PML coefficients and lie
// inside the bounds tested below (k_adj_fused decides per tile).  With
// fy2 = fx2 = 1 and fx1 = fy1 = 0 the general expressions reduce exactly
// (1*x = x, fma(0, x, y) = y up to the sign of a zero), so both forms give
// the same values.
template <bool UNIT, class Cells>
__device__ __forceinline__ float lam_cx(const AdjArgs& a, const Cells& c, int i, int j) {
  // adjoint of cx at (i, j) from hx', ihx' there (0 where H is not applied)
  if constexpr (UNIT) return __fmaf_rn(0.5f, c.lhx(i, j), c.lihx(i, j));
  if (i < 0 || j < 0 || i > a.nx - 2 || j > a.ny - 2) return 0.f;
  const float lhx = c.lhx(i, j);
  const float fy2 = c.fy2(j);
  const float lihx_t = __fmaf_rn(__fmul_rn(fy2, c.fx1(i)), lhx, c.lihx(i, j));
  return __fmaf_rn(__fmul_rn(0.5f, fy2), lhx, lihx_t);
}

template <bool UNIT, class Cells>
__device__ __forceinline__ float lam_cy(const AdjArgs& a, const Cells& c, int i, int j) {
  if constexpr (UNIT) return __fmaf_rn(-0.5f, c.lhy(i, j), c.lihy(i, j));
  if (i < 0 || j < 0 || i > a.nx - 2 || j > a.ny - 2) return 0.f;
  const float lhy = c.lhy(i, j);
  const float fx2 = c.fx2(i);
  const float lihy_t = __fmaf_rn(-__fmul_rn(fx2, c.fy1(j)), lhy, c.lihy(i, j));
  return __fmaf_rn(-__fmul_rn(0.5f, fx2), lhy, lihy_t);
}

// E part of the reverse step at one cell: recomputes dz' and ez from the
// forward state (before step t), takes L(ez) from the H adjoints (+ the probe
// seed), runs the E update backwards.  T = L'(dz) + naz*L(ez~) is the D
// adjoint before the D update is undone; liz the adjoint of iz before the
// step; lezt, diff, ez and liz_in the terms of the cell's dJ/dnaz, dJ/dnbz.
struct AdjE {
  float T, liz, lezt, diff, ez, liz_in;
};

template <bool UNIT, class Cells>
__device__ __forceinline__ AdjE adj_e_core(const AdjArgs& a, const Cells& c, int i, int j, int t) {
  // forward recompute of dz' and ez at this cell (same formulas as the forward)
  float dzp = c.fdz(i, j);
  if constexpr (UNIT)
    dzp = d_update_unit(dzp, c.fhy(i, j), c.fhy(i - 1, j), c.fhx(i, j), c.fhx(i, j - 1));
  else if (i >= 1 && j >= 1)
    dzp = d_update(dzp, c.fhy(i, j), c.fhy(i - 1, j), c.fhx(i, j), c.fhx(i, j - 1), c.gx3(i),
                   c.gy3(j), c.gx2(i), c.gy2(j));
  if (!UNIT && a.src_kind != FDTD_SRC_NONE && i == a.src_i && j == a.src_j) {
    const float v = __ldg(a.src_table + t - 1);
    dzp = (a.src_kind == FDTD_SRC_HARD) ? v : __fadd_rn(dzp, v);
  }
  AdjE r;
  const float izv = a.nbz ? c.fiz(i, j) : 0.f;
  r.diff = __fsub_rn(dzp, izv);
  const float naz = c.naz(i, j);
  r.ez = __fmul_rn(naz, r.diff);
  // adjoint of ez
  float lez = lam_cx<UNIT>(a, c, i, j) - lam_cx<UNIT>(a, c, i, j - 1) + lam_cy<UNIT>(a, c, i, j) -
              lam_cy<UNIT>(a, c, i - 1, j);
  if (i == a.probe_i && j == a.probe_j) lez = __fmaf_rn(a.probe_w, r.ez, lez);
  // E backward
  const float nbz = a.nbz ? c.nbz(i, j) : 0.f;
  r.liz_in = a.nbz ? c.liz(i, j) : 0.f;
  r.lezt = __fmaf_rn(nbz, r.liz_in, lez);
  r.liz = __fmaf_rn(-naz, r.lezt, r.liz_in);
  r.T = __fmaf_rn(naz, r.lezt, c.ldz(i, j));
  return r;
}

// adds the cell's dJ/dnaz, dJ/dnbz of one step when it lies in the design box
__device__ __forceinline__ void adj_grad(const AdjArgs& a, int i, int j, const AdjE& r) {
  const int bi = i - a.box.i0, bj = j - a.box.j0;
  if (a.grad_naz && bi >= 0 && bi < a.box.ni && bj >= 0 && bj < a.box.nj) {
    const size_t b = (size_t)bi * a.box.nj + bj;
    a.grad_naz[b] = __fmaf_rn(r.lezt, r.diff, a.grad_naz[b]);
    if (a.grad_nbz) a.grad_nbz[b] = __fmaf_rn(r.liz_in, r.ez, a.grad_nbz[b]);
  }
}

// adj_e_core at step a.t; with `own`, also writes L(iz) and adds the cell's
// gradient (a cell computed only as a neighbour's halo does neither)
template <bool UNIT = false, class Cells>
__device__ __forceinline__ float adj_e(const AdjArgs& a, const Cells& c, int i, int j, bool own) {
  const AdjE r = adj_e_core<UNIT>(a, c, i, j, a.t);
  if (own) {
    if (a.nbz) a.out.iz[(size_t)i * a.ny + j] = r.liz;
    adj_grad(a, i, j, r);
  }
  return r.T;
}

// cb*T at (i, j): the D adjoint flowing into the curl's H terms (0 where D is
// not applied, or at a hard source whose dz' does not depend on the state)
template <bool UNIT = false, class Cells>
__device__ __forceinline__ float dgrad(const AdjArgs& a, const Cells& c, int i, int j, float T) {
  if constexpr (UNIT) return __fmul_rn(0.5f, T);  // (gx2*gy2)*0.5 = 0.5; no source in the tile
  if (i < 1 || j < 1 || i >= a.nx || j >= a.ny) return 0.f;
  if (a.src_kind == FDTD_SRC_HARD && i == a.src_i && j == a.src_j) return 0.f;
  const float cb = __fmul_rn(__fmul_rn(c.gx2(i), c.gy2(j)), 0.5f);
  return __fmul_rn(cb, T);
}

// D and H part of the reverse step at one cell, given T there (T) and at
// the (i+1, j) and (i, j+1) neighbours (Ti, Tj): L(dz) = ca*T, L(hy) +=
// cb*T - cb[i+1]*T[i+1], L(hx) += -cb*T + cb[j+1]*T[j+1], then H backward.
struct AdjDH {
  float ldz, lhx, lhy, lihx, lihy;
};

template <bool UNIT, class Cells>
__device__ __forceinline__ AdjDH adj_dh_core(const AdjArgs& a, const Cells& c, int i, int j, float T, float Ti,
                                             float Tj) {
  const bool hard_src = !UNIT && (a.src_kind == FDTD_SRC_HARD && i == a.src_i && j == a.src_j);
  AdjDH r;
  if (UNIT) r.ldz = T;  // (gx3*gy3)*T = 1*T
  else if (hard_src) r.ldz = 0.f;
  else if (i >= 1 && j >= 1) r.ldz = __fmul_rn(__fmul_rn(c.gx3(i), c.gy3(j)), T);
  else r.ldz = T;
  const float dg = dgrad<UNIT>(a, c, i, j, T);
  const bool hm = UNIT || ((i <= a.nx - 2) && (j <= a.ny - 2));
  float lhx = c.lhx(i, j), lhy = c.lhy(i, j), lihx = c.lihx(i, j), lihy = c.lihy(i, j);
  if (!UNIT && hm) {
    const float fy2 = c.fy2(j), fx2 = c.fx2(i);
    lihx = __fmaf_rn(__fmul_rn(fy2, c.fx1(i)), lhx, lihx);
    lihy = __fmaf_rn(-__fmul_rn(fx2, c.fy1(j)), lhy, lihy);
    lhx = __fmul_rn(c.fy3(j), lhx);
    lhy = __fmul_rn(c.fx3(i), lhy);
  }
  r.lhy = __fadd_rn(__fadd_rn(lhy, dg), -dgrad<UNIT>(a, c, i + 1, j, Ti));
  r.lhx = __fadd_rn(__fsub_rn(lhx, dg), dgrad<UNIT>(a, c, i, j + 1, Tj));
  r.lihx = lihx;
  r.lihy = lihy;
  return r;
}

template <bool UNIT = false, class Cells>
__device__ __forceinline__ void adj_dh(const AdjArgs& a, const Cells& c, int i, int j, float T, float Ti, float Tj) {
  const size_t n = (size_t)i * a.ny + j;
  const AdjDH r = adj_dh_core<UNIT>(a, c, i, j, T, Ti, Tj);
  a.out.dz[n] = r.ldz;
  a.out.hx[n] = r.lhx;
  a.out.hy[n] = r.lhy;
  a.out.ihx[n] = r.lihx;
  a.out.ihy[n] = r.lihy;
}

// Two-kernel form (in place, T through a full-grid temporary)
__global__ void k_adj_a(const AdjArgs a) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= a.nx || j >= a.ny) return;
  a.tmp[(size_t)i * a.ny + j] = adj_e(a, GlobalCells{a}, i, j, true);
}

__global__ void k_adj_b(const AdjArgs a) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= a.nx || j >= a.ny) return;
  const size_t n = (size_t)i * a.ny + j;
  const float Ti = (i + 1 < a.nx) ? a.tmp[n + a.ny] : 0.f;
  const float Tj = (j + 1 < a.ny) ? a.tmp[n + 1] : 0.f;
  adj_dh(a, GlobalCells{a}, i, j, a.tmp[n], Ti, Tj);
}

// Fused form: one block of 32 x 8 threads takes a kAdjTI x 32 tile.  It first
// copies every value the step reads for the tile, one row and one column of
// halo below and right of it (whose T it needs) and one row and one column
// above and left of that (their neighbours), into shared memory: twelve
// fields over (kAdjTI+2) x 34 cells (widened to 40 for 16-byte copies), all
// copies in flight together.  A tile whose cells all see unit PML
// coefficients, no grid edge and no source takes the unit form.  Then it computes T on the tile and halo, then the D/H part for
// the tile.  It reads the adjoints after step t (a.adj) and writes those
// before it to other arrays (a.out): a halo cell's inputs belong to the
// neighbouring tile, which must not have overwritten them.  Same per-cell
// arithmetic on the same values as the two-kernel form, so the results are
// bitwise equal.  Cells outside the grid are staged as 0 and never used
// (every use is guarded by the grid bounds as in the global form).
constexpr int kAdjTJ = 32, kAdjTI = 16, kAdjThreadsY = 8, kAdjRows = kAdjTI / kAdjThreadsY;
// staged rows i0-1 .. i0+TI and columns j0-4 .. j0+TJ+3: the columns the
// step reads are j0-1 .. j0+TJ; the tile is widened to whole 16-byte groups
// so it is copied with one float4 load per field and group (ny % 4 == 0)
constexpr int kTileR = kAdjTI + 2, kTileC = kAdjTJ + 8, kTileQ = kTileC / 4;
enum { F_FDZ, F_FIZ, F_FHX, F_FHY, F_NAZ, F_NBZ, F_LDZ, F_LIZ, F_LHX, F_LHY, F_LIHX, F_LIHY, F_COUNT };

struct TileCells {
  const float (*t)[kTileR][kTileC];  // [field][row][column]
  int i0, j0;
  const fdtd2d_pml* pml;
  __device__ __forceinline__ float at(int f, int i, int j) const { return t[f][i - i0 + 1][j - j0 + 4]; }
  __device__ __forceinline__ float fdz(int i, int j) const { return at(F_FDZ, i, j); }
  __device__ __forceinline__ float fiz(int i, int j) const { return at(F_FIZ, i, j); }
  __device__ __forceinline__ float fhx(int i, int j) const { return at(F_FHX, i, j); }
  __device__ __forceinline__ float fhy(int i, int j) const { return at(F_FHY, i, j); }
  __device__ __forceinline__ float naz(int i, int j) const { return at(F_NAZ, i, j); }
  __device__ __forceinline__ float nbz(int i, int j) const { return at(F_NBZ, i, j); }
  __device__ __forceinline__ float ldz(int i, int j) const { return at(F_LDZ, i, j); }
  __device__ __forceinline__ float liz(int i, int j) const { return at(F_LIZ, i, j); }
  __device__ __forceinline__ float lhx(int i, int j) const { return at(F_LHX, i, j); }
  __device__ __forceinline__ float lhy(int i, int j) const { return at(F_LHY, i, j); }
  __device__ __forceinline__ float lihx(int i, int j) const { return at(F_LIHX, i, j); }
  __device__ __forceinline__ float lihy(int i, int j) const { return at(F_LIHY, i, j); }  __device__ __forceinline__ float fx1(int i) const { return __ldg(pml->fx1 + i); }
  __device__ __forceinline__ float fx2(int i) const { return __ldg(pml->fx2 + i); }
  __device__ __forceinline__ float fx3(int i) const { return __ldg(pml->fx3 + i); }
  __device__ __forceinline__ float gx2(int i) const { return __ldg(pml->gx2 + i); }
  __device__ __forceinline__ float gx3(int i) const { return __ldg(pml->gx3 + i); }
  __device__ __forceinline__ float fy1(int j) const { return __ldg(pml->fy1 + j); }
  __device__ __forceinline__ float fy2(int j) const { return __ldg(pml->fy2 + j); }
  __device__ __forceinline__ float fy3(int j) const { return __ldg(pml->fy3 + j); }
  __device__ __forceinline__ float gy2(int j) const { return __ldg(pml->gy2 + j); }
  __device__ __forceinline__ float gy3(int j) const { return __ldg(pml->gy3 + j); }
};

// T on the tile and its halo into sT, then the D/H part on the tile
template <bool UNIT>
__device__ __forceinline__ void adj_tile(const AdjArgs& a, const TileCells& c, int i0, int j0,
                                         float (*sT)[kAdjTJ + 1]) {
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int j = j0 + tx;
#pragma unroll
  for (int k = 0; k < kAdjRows; ++k) {
    const int li = ty + kAdjThreadsY * k, i = i0 + li;
    sT[li][tx] = (i < a.nx && j < a.ny) ? adj_e<UNIT>(a, c, i, j, true) : 0.f;
  }
  if (ty == 0) {  // halo row below the tile
    const int i = i0 + kAdjTI;
    sT[kAdjTI][tx] = (i < a.nx && j < a.ny) ? adj_e<UNIT>(a, c, i, j, false) : 0.f;
  } else if (ty == 1 && tx < kAdjTI) {  // halo column right of the tile
    const int i = i0 + tx, jj = j0 + kAdjTJ;
    sT[tx][kAdjTJ] = (i < a.nx && jj < a.ny) ? adj_e<UNIT>(a, c, i, jj, false) : 0.f;
  } else if (ty == 2 && tx == 0) {  // and their corner
    const int i = i0 + kAdjTI, jj = j0 + kAdjTJ;
    sT[kAdjTI][kAdjTJ] = (i < a.nx && jj < a.ny) ? adj_e<UNIT>(a, c, i, jj, false) : 0.f;
  }
  __syncthreads();
  if (j < a.ny) {
#pragma unroll
    for (int k = 0; k < kAdjRows; ++k) {
      const int li = ty + kAdjThreadsY * k, i = i0 + li;
      if (i < a.nx) adj_dh<UNIT>(a, c, i, j, sT[li][tx], sT[li + 1][tx], sT[li][tx + 1]);
    }
  }
}

// cp.async of one 16-byte group into shared memory, zero-filled (nothing
// read) where !ok; src must be a valid address either way
__device__ __forceinline__ void cp_async16(float* dst, const float* src, bool ok) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(src), "r"(ok ? 16u : 0u) : "memory");
}

// Stage tile k's twelve fields (rows i0-1 .. i0+TI, columns j0-4 .. j0+TJ+3)
// into `tile` with one 16-byte cp.async per thread and field.
__device__ __forceinline__ void stage_tile(const AdjArgs& a, float (*tile)[kTileR][kTileC], int i0, int j0, int tid) {
  if (tid >= kTileR * kTileQ) return;
  const float* src[F_COUNT] = {a.fwd.dz, a.fwd.iz, a.fwd.hx, a.fwd.hy, a.naz, a.nbz,
                               a.adj.dz, a.adj.iz, a.adj.hx, a.adj.hy, a.adj.ihx, a.adj.ihy};
  const int r = tid / kTileQ, q = tid - r * kTileQ;
  const int i = i0 - 1 + r, j = j0 - 4 + 4 * q;
  const bool in = i >= 0 && i < a.nx && j >= 0 && j < a.ny;  // a group is wholly in or out
  const size_t n = in ? (size_t)i * a.ny + j : 0;
#pragma unroll
  for (int f = 0; f < F_COUNT; ++f) {
    const bool ok = in && src[f] != nullptr;
    cp_async16(&tile[f][r][4 * q], ok ? src[f] + n : a.naz, ok);
  }
}

// Whether tile (i0, j0) takes the unit form: its rows i0-1 .. i0+TI and
// columns j0-1 .. j0+TJ lie inside 0 .. n-2 with unit PML coefficients and
// the source is not within a cell of it.  Each thread tests its share; the
// caller combines them with __syncthreads_and.
__device__ __forceinline__ bool tile_unit_part(const AdjArgs& a, int i0, int j0, int tid) {
  if (tid < kTileR) {
    const int i = i0 - 1 + tid;
    return i >= 0 && i <= a.nx - 2 && __ldg(a.pml.fx1 + i) == 0.f && __ldg(a.pml.fx2 + i) == 1.f &&
           __ldg(a.pml.fx3 + i) == 1.f && __ldg(a.pml.gx2 + i) == 1.f && __ldg(a.pml.gx3 + i) == 1.f;
  }
  if (tid >= 32 && tid < 32 + kAdjTJ + 2) {
    const int j = j0 - 1 + (tid - 32);
    return j >= 0 && j <= a.ny - 2 && __ldg(a.pml.fy1 + j) == 0.f && __ldg(a.pml.fy2 + j) == 1.f &&
           __ldg(a.pml.fy3 + j) == 1.f && __ldg(a.pml.gy2 + j) == 1.f && __ldg(a.pml.gy3 + j) == 1.f;
  }
  if (tid == 96)
    return a.src_kind == FDTD_SRC_NONE || a.src_i < i0 - 1 || a.src_i > i0 + kAdjTI + 1 || a.src_j < j0 - 1 ||
           a.src_j > j0 + kAdjTJ + 1;
  return true;
}

// One block per tile: stage it (one 16-byte cp.async per thread and field,
// all in flight together), decide the form, compute.  (A persistent variant
// that staged the next tile while computing the current one measured the
// same 27 us per step at 1024^2, with twice the shared memory.)
__global__ void __launch_bounds__(kAdjTJ * kAdjThreadsY) k_adj_fused(const AdjArgs a, int ntj) {
  extern __shared__ float4 adj_smem4[];
  float* adj_smem = reinterpret_cast<float*>(adj_smem4);
  float (*tile)[kTileR][kTileC] = reinterpret_cast<float (*)[kTileR][kTileC]>(adj_smem);
  float (*sT)[kAdjTJ + 1] = reinterpret_cast<float (*)[kAdjTJ + 1]>(adj_smem + F_COUNT * kTileR * kTileC);
  const int tid = threadIdx.y * kAdjTJ + threadIdx.x;
  const int i0 = (blockIdx.x / ntj) * kAdjTI, j0 = (blockIdx.x % ntj) * kAdjTJ;
  stage_tile(a, tile, i0, j0, tid);
  asm volatile("cp.async.commit_group;\n" ::: "memory");
  const bool part = tile_unit_part(a, i0, j0, tid);
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
  const bool unit = __syncthreads_and(part);  // also publishes the staged tile
  const TileCells c{tile, i0, j0, &a.pml};
  if (unit)
    adj_tile<true>(a, c, i0, j0, sT);
  else
    adj_tile<false>(a, c, i0, j0, sT);
}
constexpr size_t kAdjSmem = (size_t)(F_COUNT * kTileR * kTileC + (kAdjTI + 1) * (kAdjTJ + 1)) * sizeof(float);

// ---------------------------------------------------------------- two steps
// k_adj_fused2 undoes steps t and t-1 in one launch.  A block stages a kA2TI x
// 32 tile with a two-cell halo (rows i0-2 .. i0+kA2TI+1, columns j0-4 .. j0+35
// in 16-byte groups) of the adjoints after step t, both forward states (before
// t and before t-1) and the material, then
//   1. T of step t on the tile and a ring of one cell plus one more row below
//      and column right (E1), and L(iz) of step t in place on the ring (R1);
//   2. the D/H part of step t on R1, in place: the staged adjoints become the
//      adjoints after step t-1 there;
//   3. T of step t-1 on the tile plus one row below and one column right (E2);
//   4. the D/H part of step t-1 on the tile, written out.
// Every cell runs the same per-cell functions on the same operands as the
// one-step kernels (a ring cell is the neighbouring tile's cell, computed
// again), so the results are bitwise equal to two launches of k_adj_fused;
// each tile cell adds its gradient terms of step t, then of step t-1.
// Against two one-step launches it stages half the bytes, needs three block
// barriers instead of four and launches once.
// 8 x 32 tiles: 25.7 KB of shared memory (lossless box), 8 blocks per SM.  At
// 1024^2 the reverse took 57.0 ms with 8-row tiles, 59.3 with 16, 65.5 with 24
// and 72.2 with 32: occupancy pays more than the smaller halo share.
constexpr int kA2TI = 8, kA2TJ = 32;  // kA2TI a multiple of 8, at most 60
static_assert(kA2TI % 8 == 0 && kA2TI + 4 <= 64, "tile rows: phase 4 takes 8 rows per pass; unit test ranges");
constexpr int kT2R = kA2TI + 4, kT2C = kA2TJ + 8, kT2Q = kT2C / 4;  // staged rows, columns, 16-byte groups
constexpr int kE1R = kA2TI + 3, kE1C = kA2TJ + 3;                    // E1: rows i0-1 .., columns j0-1 ..
constexpr int kR1R = kA2TI + 2, kR1C = kA2TJ + 2;                    // R1: the same origin
constexpr int kE2R = kA2TI + 1, kE2C = kA2TJ + 1;                    // E2: rows i0 .., columns j0 ..

template <bool LOSSY>
struct A2F;
template <>
struct A2F<true> {
  enum { F1DZ, F1IZ, F1HX, F1HY, F0DZ, F0IZ, F0HX, F0HY, NAZ, NBZ, LDZ, LIZ, LHX, LHY, LIHX, LIHY, COUNT };
};
template <>
struct A2F<false> {
  enum { F1DZ, F1HX, F1HY, F0DZ, F0HX, F0HY, NAZ, LDZ, LHX, LHY, LIHX, LIHY, COUNT, F1IZ = -1, F0IZ = -1,
         NBZ = -1, LIZ = -1 };
};

// STEP 1: step t (state before t, adjoints after t); STEP 0: step t-1 (state
// before t-1, the adjoints after t-1 that phase 2 left in the same arrays)
// the PML profile vectors over the staged rows and columns, in shared memory
enum { PX_FX1, PX_FX2, PX_FX3, PX_GX2, PX_GX3, PX_COUNT };
enum { PY_FY1, PY_FY2, PY_FY3, PY_GY2, PY_GY3, PY_COUNT };
constexpr int kPYC = kA2TJ + 4;  // columns j0-2 .. j0+TJ+1

template <bool LOSSY, int STEP>
struct Tile2Cells {
  using F = A2F<LOSSY>;
  float (*t)[kT2R][kT2C];
  int i0, j0;
  const float (*px)[kT2R];  // [vector][row i - i0 + 2]
  const float (*py)[kPYC];  // [vector][column j - j0 + 2]
  __device__ __forceinline__ float fx1(int i) const { return px[PX_FX1][i - i0 + 2]; }
  __device__ __forceinline__ float fx2(int i) const { return px[PX_FX2][i - i0 + 2]; }
  __device__ __forceinline__ float fx3(int i) const { return px[PX_FX3][i - i0 + 2]; }
  __device__ __forceinline__ float gx2(int i) const { return px[PX_GX2][i - i0 + 2]; }
  __device__ __forceinline__ float gx3(int i) const { return px[PX_GX3][i - i0 + 2]; }
  __device__ __forceinline__ float fy1(int j) const { return py[PY_FY1][j - j0 + 2]; }
  __device__ __forceinline__ float fy2(int j) const { return py[PY_FY2][j - j0 + 2]; }
  __device__ __forceinline__ float fy3(int j) const { return py[PY_FY3][j - j0 + 2]; }
  __device__ __forceinline__ float gy2(int j) const { return py[PY_GY2][j - j0 + 2]; }
  __device__ __forceinline__ float gy3(int j) const { return py[PY_GY3][j - j0 + 2]; }
  __device__ __forceinline__ float at(int f, int i, int j) const { return t[f][i - i0 + 2][j - j0 + 4]; }
  __device__ __forceinline__ float fdz(int i, int j) const { return at(STEP ? F::F1DZ : F::F0DZ, i, j); }
  __device__ __forceinline__ float fiz(int i, int j) const {
    return LOSSY ? at(STEP ? F::F1IZ : F::F0IZ, i, j) : 0.f;
  }
  __device__ __forceinline__ float fhx(int i, int j) const { return at(STEP ? F::F1HX : F::F0HX, i, j); }
  __device__ __forceinline__ float fhy(int i, int j) const { return at(STEP ? F::F1HY : F::F0HY, i, j); }
  __device__ __forceinline__ float naz(int i, int j) const { return at(F::NAZ, i, j); }
  __device__ __forceinline__ float nbz(int i, int j) const { return LOSSY ? at(F::NBZ, i, j) : 0.f; }
  __device__ __forceinline__ float ldz(int i, int j) const { return at(F::LDZ, i, j); }
  __device__ __forceinline__ float liz(int i, int j) const { return LOSSY ? at(F::LIZ, i, j) : 0.f; }
  __device__ __forceinline__ float lhx(int i, int j) const { return at(F::LHX, i, j); }
  __device__ __forceinline__ float lhy(int i, int j) const { return at(F::LHY, i, j); }
  __device__ __forceinline__ float lihx(int i, int j) const { return at(F::LIHX, i, j); }
  __device__ __forceinline__ float lihy(int i, int j) const { return at(F::LIHY, i, j); }
};

template <bool LOSSY>
__device__ __forceinline__ void stage_tile2(const AdjArgs& a, float (*tile)[kT2R][kT2C], int i0, int j0, int tid) {
  constexpr int N = A2F<LOSSY>::COUNT;
  const float* src[16];
  if (LOSSY) {
    const float* s16[16] = {a.fwd.dz,  a.fwd.iz, a.fwd.hx, a.fwd.hy, a.fwd0.dz, a.fwd0.iz, a.fwd0.hx, a.fwd0.hy,
                            a.naz,     a.nbz,    a.adj.dz, a.adj.iz, a.adj.hx,  a.adj.hy,  a.adj.ihx, a.adj.ihy};
    for (int f = 0; f < 16; ++f) src[f] = s16[f];
  } else {
    const float* s12[12] = {a.fwd.dz, a.fwd.hx, a.fwd.hy, a.fwd0.dz, a.fwd0.hx, a.fwd0.hy,
                            a.naz,    a.adj.dz, a.adj.hx, a.adj.hy,  a.adj.ihx, a.adj.ihy};
    for (int f = 0; f < 12; ++f) src[f] = s12[f];
  }
  for (int g = tid; g < kT2R * kT2Q; g += kA2TJ * 8) {
    const int r = g / kT2Q, q = g - r * kT2Q;
    const int i = i0 - 2 + r, j = j0 - 4 + 4 * q;
    const bool in = i >= 0 && i < a.nx && j >= 0 && j < a.ny;  // a group is wholly in or out (ny % 4 == 0)
    const size_t n = in ? (size_t)i * a.ny + j : 0;
#pragma unroll
    for (int f = 0; f < N; ++f) cp_async16(&tile[f][r][4 * q], in ? src[f] + n : a.naz, in);
  }
}

// Copies the PML vectors of the staged rows (i0-2 .. i0+TI+1) and columns
// (j0-2 .. j0+TJ+1) into px/py (0 outside the grid, where no cell reads
// them) and tells whether this thread's share allows the unit form: those
// rows and columns inside 0 .. n-2 with unit PML coefficients, and no source
// near the tile.
__device__ __forceinline__ bool tile2_unit_part(const AdjArgs& a, int i0, int j0, int tid, float (*px)[kT2R],
                                                float (*py)[kPYC]) {
  if (tid < kT2R) {
    const int i = i0 - 2 + tid;
    const bool in = i >= 0 && i < a.nx;
    const float f1 = in ? __ldg(a.pml.fx1 + i) : 0.f, f2 = in ? __ldg(a.pml.fx2 + i) : 0.f;
    const float f3 = in ? __ldg(a.pml.fx3 + i) : 0.f, g2 = in ? __ldg(a.pml.gx2 + i) : 0.f;
    const float g3 = in ? __ldg(a.pml.gx3 + i) : 0.f;
    px[PX_FX1][tid] = f1;
    px[PX_FX2][tid] = f2;
    px[PX_FX3][tid] = f3;
    px[PX_GX2][tid] = g2;
    px[PX_GX3][tid] = g3;
    return i >= 0 && i <= a.nx - 2 && f1 == 0.f && f2 == 1.f && f3 == 1.f && g2 == 1.f && g3 == 1.f;
  }
  if (tid >= 64 && tid < 64 + kPYC) {
    const int c = tid - 64, j = j0 - 2 + c;
    const bool in = j >= 0 && j < a.ny;
    const float f1 = in ? __ldg(a.pml.fy1 + j) : 0.f, f2 = in ? __ldg(a.pml.fy2 + j) : 0.f;
    const float f3 = in ? __ldg(a.pml.fy3 + j) : 0.f, g2 = in ? __ldg(a.pml.gy2 + j) : 0.f;
    const float g3 = in ? __ldg(a.pml.gy3 + j) : 0.f;
    py[PY_FY1][c] = f1;
    py[PY_FY2][c] = f2;
    py[PY_FY3][c] = f3;
    py[PY_GY2][c] = g2;
    py[PY_GY3][c] = g3;
    return j >= 0 && j <= a.ny - 2 && f1 == 0.f && f2 == 1.f && f3 == 1.f && g2 == 1.f && g3 == 1.f;
  }
  if (tid == 128)
    return a.src_kind == FDTD_SRC_NONE || a.src_i < i0 - 2 || a.src_i > i0 + kA2TI + 2 || a.src_j < j0 - 2 ||
           a.src_j > j0 + kA2TJ + 2;
  return true;
}

template <bool UNIT, bool LOSSY>
__device__ __forceinline__ void adj_tile2(const AdjArgs& a, float (*tile)[kT2R][kT2C], int i0, int j0, int tid,
                                          float (*s1)[kE1C], float (*s2)[kE2C], const float (*px)[kT2R],
                                          const float (*py)[kPYC]) {
  using F = A2F<LOSSY>;
  const Tile2Cells<LOSSY, 1> c1{tile, i0, j0, px, py};
  const Tile2Cells<LOSSY, 0> c0{tile, i0, j0, px, py};
  auto in_grid = [&](int i, int j) { return i >= 0 && i < a.nx && j >= 0 && j < a.ny; };
  // A region of R rows x C columns (C > 32) is covered row by row: warp w
  // takes rows w, w+8, ..., its lanes the first 32 columns (consecutive
  // shared-memory words, no bank conflict); the other C-32 columns go to the
  // threads of the warps from R % 8 on, which have one row fewer.
  const int lane = threadIdx.x, w = threadIdx.y, tid_ = w * 32 + lane;
  auto cover = [&](auto R, auto C, auto&& cell) {
    constexpr int kR = decltype(R)::value, kC = decltype(C)::value, kX = kC - 32;
    for (int li = w; li < kR; li += 8) cell(li, lane);
    for (int k = (tid_ + 256 - (kR % 8) * 32) % 256; k < kR * kX; k += 256) {
      const int li = k / kX;
      cell(li, 32 + (k - li * kX));
    }
  };
  // 1. step t: T on E1, L(iz) in place on R1, gradient terms of the tile
  cover(std::integral_constant<int, kE1R>{}, std::integral_constant<int, kE1C>{}, [&](int li, int lj) {
    const int i = i0 - 1 + li, j = j0 - 1 + lj;
    float T = 0.f;
    if (UNIT || in_grid(i, j)) {
      const AdjE r = adj_e_core<UNIT>(a, c1, i, j, a.t);
      T = r.T;
      if (LOSSY && li < kR1R && lj < kR1C) tile[F::LIZ][li + 1][lj + 3] = r.liz;
      if (li >= 1 && li <= kA2TI && lj >= 1 && lj <= kA2TJ) adj_grad(a, i, j, r);
    }
    s1[li][lj] = T;
  });
  __syncthreads();
  // 2. step t: D/H on R1, in place
  cover(std::integral_constant<int, kR1R>{}, std::integral_constant<int, kR1C>{}, [&](int li, int lj) {
    const int i = i0 - 1 + li, j = j0 - 1 + lj;
    if (UNIT || in_grid(i, j)) {
      const AdjDH r = adj_dh_core<UNIT>(a, c1, i, j, s1[li][lj], s1[li + 1][lj], s1[li][lj + 1]);
      tile[F::LDZ][li + 1][lj + 3] = r.ldz;
      tile[F::LHX][li + 1][lj + 3] = r.lhx;
      tile[F::LHY][li + 1][lj + 3] = r.lhy;
      tile[F::LIHX][li + 1][lj + 3] = r.lihx;
      tile[F::LIHY][li + 1][lj + 3] = r.lihy;
    }
  });
  __syncthreads();
  // 3. step t-1: T on E2; L(iz) and gradient terms of the tile
  cover(std::integral_constant<int, kE2R>{}, std::integral_constant<int, kE2C>{}, [&](int li, int lj) {
    const int i = i0 + li, j = j0 + lj;
    float T = 0.f;
    if (UNIT || in_grid(i, j)) {
      const AdjE r = adj_e_core<UNIT>(a, c0, i, j, a.t - 1);
      T = r.T;
      if (li < kA2TI && lj < kA2TJ) {
        if (LOSSY) a.out.iz[(size_t)i * a.ny + j] = r.liz;
        adj_grad(a, i, j, r);
      }
    }
    s2[li][lj] = T;
  });
  __syncthreads();
  // 4. step t-1: D/H on the tile
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int j = j0 + tx;
  if (j < a.ny) {
#pragma unroll
    for (int k = 0; k < kA2TI / 8; ++k) {
      const int li = ty + 8 * k, i = i0 + li;
      if (i < a.nx) adj_dh<UNIT>(a, c0, i, j, s2[li][tx], s2[li + 1][tx], s2[li][tx + 1]);
    }
  }
}

template <bool LOSSY>
constexpr size_t adj2_smem() {
  return (size_t)(A2F<LOSSY>::COUNT * kT2R * kT2C + kE1R * kE1C + kE2R * kE2C + PX_COUNT * kT2R + PY_COUNT * kPYC) *
         sizeof(float);
}

template <bool LOSSY>
__global__ void __launch_bounds__(kA2TJ * 8) k_adj_fused2(const AdjArgs a, int ntj) {
  extern __shared__ float4 adj2_smem4[];
  float* sm = reinterpret_cast<float*>(adj2_smem4);
  float (*tile)[kT2R][kT2C] = reinterpret_cast<float (*)[kT2R][kT2C]>(sm);
  float (*s1)[kE1C] = reinterpret_cast<float (*)[kE1C]>(sm + A2F<LOSSY>::COUNT * kT2R * kT2C);
  float* rest = sm + A2F<LOSSY>::COUNT * kT2R * kT2C + kE1R * kE1C;
  float (*s2)[kE2C] = reinterpret_cast<float (*)[kE2C]>(rest);
  float (*px)[kT2R] = reinterpret_cast<float (*)[kT2R]>(rest + kE2R * kE2C);
  float (*py)[kPYC] = reinterpret_cast<float (*)[kPYC]>(rest + kE2R * kE2C + PX_COUNT * kT2R);
  const int tid = threadIdx.y * kA2TJ + threadIdx.x;
  const int i0 = (blockIdx.x / ntj) * kA2TI, j0 = (blockIdx.x % ntj) * kA2TJ;
  stage_tile2<LOSSY>(a, tile, i0, j0, tid);
  asm volatile("cp.async.commit_group;\n" ::: "memory");
  const bool part = tile2_unit_part(a, i0, j0, tid, px, py);
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
  const bool unit = __syncthreads_and(part);  // also publishes the staged tile and vectors
  if (unit)
    adj_tile2<true, LOSSY>(a, tile, i0, j0, tid, s1, s2, px, py);
  else
    adj_tile2<false, LOSSY>(a, tile, i0, j0, tid, s1, s2, px, py);
}

template <bool LOSSY>
int launch_adj2(const AdjArgs& a, cudaStream_t st) {
  static const cudaError_t attr =
      cudaFuncSetAttribute(k_adj_fused2<LOSSY>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)adj2_smem<LOSSY>());
  if (attr != cudaSuccess) {
    fdtd_host::note_cuda_error(attr);
    return FDTD_ERR_CUDA;
  }
  const int ntj = (a.ny + kA2TJ - 1) / kA2TJ, nti = (a.nx + kA2TI - 1) / kA2TI;
  k_adj_fused2<LOSSY><<<ntj * nti, dim3(kA2TJ, 8), adj2_smem<LOSSY>(), st>>>(a, ntj);
  return fdtd_host::check_launch();
}

}  // namespace

// One reverse step in one launch (k_adj_fused): adjoints after step t from
// adj_in, before it to adj_out (distinct arrays), fwd = the state before t.
int launch_adjoint_fused(const fdtd2d_params& p, int t, const fdtd2d_fields& fwd, const fdtd2d_fields& adj_in,
                         const fdtd2d_fields& adj_out, int probe_i, int probe_j, float probe_w,
                         const fdtd2d_box& box, float* grad_naz, float* grad_nbz, cudaStream_t st) {
  AdjArgs a{};
  a.nx = p.nx;
  a.ny = p.ny;
  a.t = t;
  a.pml = p.pml;
  a.naz = p.naz;
  a.nbz = p.nbz;
  a.src_kind = p.src.kind;
  a.src_i = p.src.i;
  a.src_j = p.src.j;
  a.src_table = p.src.table;
  a.fwd = fwd;
  a.adj = adj_in;
  a.out = adj_out;
  a.tmp = nullptr;
  a.probe_i = probe_i;
  a.probe_j = probe_j;
  a.probe_w = probe_w;
  a.box = box;
  a.grad_naz = grad_naz;
  a.grad_nbz = grad_nbz;
  const dim3 blk(kAdjTJ, kAdjThreadsY);
  const int ntj = (p.ny + kAdjTJ - 1) / kAdjTJ, nti = (p.nx + kAdjTI - 1) / kAdjTI;
  k_adj_fused<<<ntj * nti, blk, kAdjSmem, st>>>(a, ntj);
  return fdtd_host::check_launch();
}

// Steps t and t-1 in one launch (k_adj_fused2): adjoints after step t from
// adj_in, before step t-1 to adj_out; fwd1/fwd0 = the states before t / t-1.
int launch_adjoint_fused2(const fdtd2d_params& p, int t, const fdtd2d_fields& fwd1, const fdtd2d_fields& fwd0,
                          const fdtd2d_fields& adj_in, const fdtd2d_fields& adj_out, int probe_i, int probe_j,
                          float probe_w, const fdtd2d_box& box, float* grad_naz, float* grad_nbz, cudaStream_t st) {
  AdjArgs a{};
  a.nx = p.nx;
  a.ny = p.ny;
  a.t = t;
  a.pml = p.pml;
  a.naz = p.naz;
  a.nbz = p.nbz;
  a.src_kind = p.src.kind;
  a.src_i = p.src.i;
  a.src_j = p.src.j;
  a.src_table = p.src.table;
  a.fwd = fwd1;
  a.fwd0 = fwd0;
  a.adj = adj_in;
  a.out = adj_out;
  a.tmp = nullptr;
  a.probe_i = probe_i;
  a.probe_j = probe_j;
  a.probe_w = probe_w;
  a.box = box;
  a.grad_naz = grad_naz;
  a.grad_nbz = grad_nbz;
  return p.nbz ? launch_adj2<true>(a, st) : launch_adj2<false>(a, st);
}

}  // namespace fdtd

extern "C" {

int fdtd2d_pass(const fdtd2d_params* p, const fdtd2d_fields* in, fdtd2d_fields* out, float* ez, int t0, int k,
                int* status, fdtd_stream_t stream) {
  if (!p || !in || !out || !ez) return FDTD_ERR_NULL;
  if (p->nx < 3 || p->ny < 3 || p->ny % 4) return FDTD_ERR_SIZE;
  if (k < 1 || k > fdtd::march_max_steps_per_pass() || t0 < 0) return FDTD_ERR_ARG;
  if (!in->dz || !in->hx || !in->hy || !out->dz || !out->hx || !out->hy || !p->naz) return FDTD_ERR_NULL;
  if (p->nbz && (!in->iz || !out->iz)) return FDTD_ERR_NULL;
  if (fdtd::has_pml(*p) && (!in->ihx || !in->ihy || !out->ihx || !out->ihy)) return FDTD_ERR_NULL;
  if (p->src.kind != FDTD_SRC_NONE && (!p->src.table || t0 + k > p->src.table_len)) return FDTD_ERR_SIZE;
  if (p->tfsf_npml > 0 || p->nf > 0) return FDTD_ERR_UNSUPPORTED;
  if (in->dz == out->dz) return FDTD_ERR_ARG;
  fdtd::FieldSet fi{in->dz, in->iz, in->hx, in->hy, in->ihx, in->ihy};
  fdtd::FieldSet fo{out->dz, out->iz, out->hx, out->hy, out->ihx, out->ihy};
  return fdtd::launch_march(*p, fi, fo, ez, t0, k, status, nullptr, (cudaStream_t)stream);
}

int fdtd2d_adjoint_step(int t, const fdtd2d_params* p, const fdtd2d_fields* fwd, fdtd2d_fields* adj, float* adj_tmp,
                        int probe_i, int probe_j, float probe_weight, fdtd2d_box box, float* grad_naz,
                        float* grad_nbz, fdtd_stream_t stream) {
  if (!p || !fwd || !adj || !adj_tmp) return FDTD_ERR_NULL;
  if (p->nx < 3 || p->ny < 3) return FDTD_ERR_SIZE;
  if (t < 1) return FDTD_ERR_ARG;
  if (!fdtd::has_pml(*p)) return FDTD_ERR_UNSUPPORTED;  // pass unit profiles for no absorbing layer
  if (!p->naz || !fwd->dz || !fwd->hx || !fwd->hy) return FDTD_ERR_NULL;
  if (!adj->dz || !adj->hx || !adj->hy || !adj->ihx || !adj->ihy) return FDTD_ERR_NULL;
  if (p->nbz && (!fwd->iz || !adj->iz)) return FDTD_ERR_NULL;
  if (p->src.kind != FDTD_SRC_NONE && (!p->src.table || t > p->src.table_len)) return FDTD_ERR_SIZE;
  if (p->tfsf_npml > 0 || p->nf > 0) return FDTD_ERR_UNSUPPORTED;
  if (grad_naz && (box.ni <= 0 || box.nj <= 0 || box.i0 < 0 || box.j0 < 0 || box.i0 + box.ni > p->nx ||
                   box.j0 + box.nj > p->ny))
    return FDTD_ERR_ARG;
  fdtd::AdjArgs a{};
  a.nx = p->nx;
  a.ny = p->ny;
  a.t = t;
  a.pml = p->pml;
  a.naz = p->naz;
  a.nbz = p->nbz;
  a.src_kind = p->src.kind;
  a.src_i = p->src.i;
  a.src_j = p->src.j;
  a.src_table = p->src.table;
  a.fwd = *fwd;
  a.adj = *adj;
  a.out = *adj;
  a.tmp = adj_tmp;
  a.probe_i = probe_i;
  a.probe_j = probe_j;
  a.probe_w = probe_weight;
  a.box = box;
  a.grad_naz = grad_naz;
  a.grad_nbz = grad_nbz;
  const dim3 blk(32, 8);
  const dim3 grd((p->ny + 31) / 32, (p->nx + 7) / 8);
  cudaStream_t st = (cudaStream_t)stream;
  fdtd::k_adj_a<<<grd, blk, 0, st>>>(a);
  int rc = fdtd_host::check_launch();
  if (rc) return rc;
  fdtd::k_adj_b<<<grd, blk, 0, st>>>(a);
  return fdtd_host::check_launch();
}

}  // extern "C"
