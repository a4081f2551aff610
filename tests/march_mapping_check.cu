// Host-only check of the warp -> work layout of the fused passes
// (simulation_gb300/csrc/fd2d_march.cuh), built by tests/test_march_mapping.py
// and run on the CPU (it makes no CUDA call).
//
// One launch is a single wave of warps, each marching down one segment of
// rows of one stripe of columns.  The stripes that hold the absorbing layer,
// the grid's edges or the TF/SF box's edge columns get shorter segments, and
// the other stripes' first and last segments are shortened too
// (plain_layout); plain_work maps a warp to its work.  This program checks,
// with the header's own two functions, over many grid shapes, layer widths,
// TF/SF boxes, wave sizes and cost factors, that every (stripe, row) is owned
// by exactly one warp and that every warp's work lies inside the grid.  It
// also checks that every instantiation's dynamic shared memory fits a block.
#include <algorithm>
#include <cstdio>
#include <vector>

#include "fd2d_march.cuh"

namespace {

int g_fail = 0;

void fail(const char* what, int nx, int ny, int np, int K, int seg_rows, int a, int b) {
  if (g_fail < 20) std::printf("FAIL %s: nx=%d ny=%d hint=%d K=%d seg=%d (%d, %d)\n", what, nx, ny, np, K, seg_rows, a, b);
  ++g_fail;
}

// Dynamic shared memory of every instantiation (launch_t's own formula,
// march_smem_bytes) fits the 227 KB a block may have: 64- and 128-column
// stripes, K = 1..4, 0..8 DFT frequencies (the extras use 64-column stripes
// only).
void check_shared_memory() {
  for (int cpl : {2, 4})
    for (int k = 1; k <= 4; ++k)
      for (int nf = 0; nf <= fdtd::kMarchMaxNf; ++nf)
        for (int lossy = 0; lossy < 2; ++lossy)
          for (int pml = 0; pml < 2; ++pml)
            for (int pf = 0; pf < 2; ++pf) {
              if (cpl == 4 && nf > 0) continue;
              const long bytes = (long)fdtd::march::march_smem_bytes(fdtd::march::kWarps, k, nf, lossy, pml,
                                                                     32 * cpl, pf);
              if (bytes > 227L * 1024) fail("shared memory over 227 KB", cpl, k, nf, lossy, pml, (int)bytes, 0);
            }
}

// The plain kernels' work layout (plain_layout + plain_work, the header's own
// functions): every (stripe, row) owned by exactly one warp, every warp's
// stripe and rows inside the grid, and no more warps than one wave when the
// wave can hold one segment per stripe.
template <int K, int CPLX>
void check_plain(int nx, int ny, int hint, int np, long resident, float G) {
  constexpr int WX = 32 * CPLX, OUTWX = WX - 2 * fdtd::march::HALO;
  fdtd::march::MarchArgs a{};
  a.nx = nx;
  a.ny = ny;
  a.pml_hint = hint;
  a.ext.tfsf_npml = np;
  a.n_stripes = (ny + OUTWX - 1) / OUTWX;
  const long warps = fdtd::plain_layout<K, CPLX>(a, resident, G);
  const int n_gen = a.n_gen_lo + a.n_gen_hi;
  if (n_gen > a.n_stripes) fail("more general stripes than stripes", nx, ny, hint, K, 0, n_gen, a.n_stripes);
  if (resident >= (long)(a.n_stripes - n_gen) + (long)(G * n_gen) + 1 && warps > resident)
    fail("more warps than one wave", nx, ny, hint, K, 0, (int)warps, (int)resident);
  std::vector<int> cover((size_t)a.n_stripes * nx, 0);
  for (long gw = 0; gw < warps + 64; ++gw) {
    int stripe, i_s, i_e;
    if (!fdtd::plain_work(a, (int)gw, stripe, i_s, i_e)) continue;
    if (gw >= warps) {
      fail("work beyond the launched warps", nx, ny, hint, K, 0, (int)gw, (int)warps);
      continue;
    }
    if (stripe < 0 || stripe >= a.n_stripes || i_s < 0 || i_e > nx) {
      fail("work outside the grid", nx, ny, hint, K, 0, stripe, i_s);
      continue;
    }
    for (int r = i_s; r < i_e; ++r) ++cover[(size_t)stripe * nx + r];
  }
  for (int q = 0; q < a.n_stripes; ++q)
    for (int r = 0; r < nx; ++r)
      if (cover[(size_t)q * nx + r] != 1) fail("plain: row not owned exactly once", nx, ny, hint, K, 0, q, r);
}

template <int K>
void sweep_plain() {
  const int sizes_x[] = {3, 9, 67, 130, 300, 1024, 2048, 8192};
  const int sizes_y[] = {4, 8, 68, 132, 300, 1024, 8192};
  for (int nx : sizes_x)
    for (int ny : sizes_y)
      for (int hint : {0, 1, 6, 32, 80})
        for (int np : {0, 2, 8, 32})
          for (long resident : {8L, 608L, 1216L, 2432L})
            for (float G : {1.f, 1.5f, 2.5f, 4.f, 8.f}) {
              if (np > 0 && (2 * np >= nx || 2 * np >= ny)) continue;
              check_plain<K, 2>(nx, ny, hint, np, resident, G);
              check_plain<K, 4>(nx, ny, hint, np, resident, G);
            }
}

}  // namespace

int main() {
  check_shared_memory();
  sweep_plain<1>();
  sweep_plain<2>();
  sweep_plain<3>();
  sweep_plain<4>();
  if (g_fail) {
    std::printf("%d failures\n", g_fail);
    return 1;
  }
  std::printf("ok\n");
  return 0;
}
