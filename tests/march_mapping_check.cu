// Host-only check of the warp -> work mapping of the fused pass with TF/SF
// (simulation_gb300/csrc/fd2d_march.cuh), built by tests/test_march_mapping.py
// and run on the CPU (it makes no CUDA call).
//
// The pass compiles the TF/SF edge logic only into the body that "edge" warps
// run, and halves their segments across extra warps.  Two properties make
// that exact, and this program checks both over many grid shapes with the
// header's own tf_stripe / tf_segment predicates:
//   * every (stripe, row) of the grid is owned by exactly one warp, halves
//     included;
//   * a warp classified as not touching an edge really never updates a cell
//     that a TF/SF correction applies to (an edge column in its stripe, halo
//     included, or an hy edge row among the rows its levels complete).
// The list building and the warp enumeration below restate launch_t and
// k_march's extras branch line for line.  It also checks that every
// instantiation's dynamic shared memory fits a block.
#include <algorithm>
#include <cstdio>
#include <vector>

#include "fd2d_march.cuh"

namespace {

constexpr int CPL = 2;  // the extras kernels use 64-column stripes
constexpr int W = 32 * CPL;
constexpr int OUTW = W - 2 * fdtd::march::HALO;

int g_fail = 0;

void fail(const char* what, int nx, int ny, int np, int K, int seg_rows, int a, int b) {
  if (g_fail < 20) std::printf("FAIL %s: nx=%d ny=%d np=%d K=%d seg=%d (%d, %d)\n", what, nx, ny, np, K, seg_rows, a, b);
  ++g_fail;
}

template <int K>
void check(int nx, int ny, int np, int seg_rows) {
  const int n_stripes = (ny + OUTW - 1) / OUTW;
  const int n_segs = (nx + seg_rows - 1) / seg_rows;
  // halving lists (launch_t)
  std::vector<int> tc, tr;
  bool fits = true;
  if (np > 0) {
    for (int q = 0; q < n_stripes && fits; ++q)
      if (fdtd::tf_stripe<CPL>(np, ny, q)) {
        if (tc.size() == 6) fits = false;
        else tc.push_back(q);
      }
    for (int q = 0; q < n_segs && fits; ++q)
      if (fdtd::tf_segment<K>(np, nx, seg_rows, q)) {
        if (tr.size() == 6) fits = false;
        else tr.push_back(q);
      }
  }
  const int nc = fits ? (int)tc.size() : 0, nr = fits ? (int)tr.size() : 0;
  const long n_base = (long)n_stripes * n_segs;
  const long total = n_base + (long)nc * n_segs + (long)(n_stripes - nc) * nr;

  std::vector<int> cover((size_t)n_stripes * nx, 0);
  for (long gw = 0; gw < total; ++gw) {
    // warp -> work (k_march, extras branch)
    int stripe, seg, half = 0;
    if (gw < n_base) {
      stripe = (int)(gw % n_stripes);
      seg = (int)(gw / n_stripes);
    } else {
      long k = gw - n_base;
      if (k < (long)nc * n_segs) {
        stripe = tc[k / n_segs];
        seg = (int)(k % n_segs);
      } else {
        k -= (long)nc * n_segs;
        if (k >= (long)(n_stripes - nc) * nr) continue;
        seg = tr[k % nr];
        stripe = (int)(k / nr);
        for (int i = 0; i < nc; ++i)
          if (tc[i] <= stripe) ++stripe;
      }
      half = 2;
    }
    const bool tf = np > 0 && (fdtd::tf_stripe<CPL>(np, ny, stripe) || fdtd::tf_segment<K>(np, nx, seg_rows, seg));
    if (tf && half == 0 && (nc > 0 || nr > 0)) half = 1;
    int i_s = seg * seg_rows;
    int i_e = std::min(nx, i_s + seg_rows);
    const int mid = i_s + (i_e - i_s + 1) / 2;
    if (half == 1) i_e = mid;
    if (half == 2) i_s = mid;
    if (i_s >= i_e) continue;
    for (int r = i_s; r < i_e; ++r) ++cover[(size_t)stripe * nx + r];

    if (!tf && np > 0) {
      // columns the warp computes (halo included)
      const int c0 = stripe * OUTW - fdtd::march::HALO, c1 = c0 + W - 1;
      for (int c : {np - 2, np - 1, ny - np})
        if (c >= c0 && c <= c1) fail("edge column in a plain warp", nx, ny, np, K, seg_rows, stripe, c);
      // rows whose H its levels complete: qc = r - s - 1 over the row loop
      const int r_begin = std::max(0, i_s - K), r_end = i_e - 1 + K;
      const int lo = std::max(0, r_begin - K), hi = std::min(nx - 2, r_end - 1);
      for (int row : {np - 2, nx - np})
        if (row >= lo && row <= hi) fail("hy edge row in a plain warp", nx, ny, np, K, seg_rows, seg, row);
    }
  }
  for (int q = 0; q < n_stripes; ++q)
    for (int r = 0; r < nx; ++r)
      if (cover[(size_t)q * nx + r] != 1)
        fail("row not owned exactly once", nx, ny, np, K, seg_rows, q, r);
}

template <int K>
void sweep() {
  const int sizes_x[] = {9, 20, 67, 97, 100, 130, 257, 300, 1000, 2048};
  const int sizes_y[] = {8, 20, 68, 100, 132, 256, 300, 1024, 2048};
  const int nps[] = {0, 2, 3, 8, 32};
  for (int nx : sizes_x)
    for (int ny : sizes_y)
      for (int np : nps) {
        if (np > 0 && (2 * np >= nx || 2 * np >= ny || ny < 7)) continue;
        const int segs[] = {1, 5, 7, 4 * K, 16, 33, 42, 64, nx};
        for (int seg_rows : segs)
          if (seg_rows >= 1) check<K>(nx, ny, np, seg_rows);
      }
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
void check_plain(int nx, int ny, int hint, long resident, float G) {
  constexpr int WX = 32 * CPLX, OUTWX = WX - 2 * fdtd::march::HALO;
  fdtd::march::MarchArgs a{};
  a.nx = nx;
  a.ny = ny;
  a.pml_hint = hint;
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
        for (long resident : {8L, 608L, 2432L})
          for (float G : {1.f, 1.5f, 2.f, 3.f}) {
            check_plain<K, 2>(nx, ny, hint, resident, G);
            check_plain<K, 4>(nx, ny, hint, resident, G);
          }
}

}  // namespace

int main() {
  check_shared_memory();
  sweep_plain<1>();
  sweep_plain<2>();
  sweep_plain<3>();
  sweep_plain<4>();
  sweep<1>();
  sweep<2>();
  sweep<3>();
  sweep<4>();
  if (g_fail) {
    std::printf("%d failures\n", g_fail);
    return 1;
  }
  std::printf("ok\n");
  return 0;
}
