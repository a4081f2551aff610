// Plain fused passes (fdtd2d_step_n, fdtd2d_pass) and the pass dispatch; the
// kernel itself is in fd2d_march.cuh.
#include "fd2d_march.cuh"

namespace fdtd {
namespace march {
MarchConfig g_cfg;
}  // namespace march

namespace {

using namespace march;

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

// Steps per pass when the caller leaves it to the library.  Measured with
// the lossy PML program (CUDA events, 960 steps): at 1024^2, whose fields fit
// in L2, 2 steps per pass run 9.6 us per step against 10.4 for 4 (fewer
// recomputed cone rows in the short segments a small grid needs to fill the
// GPU); at 2048^2 and above 4 are fastest (18.4 against 29.8 us).
int march_default_steps(int nx, int ny) { return (long long)nx * ny < (1LL << 21) ? 2 : HALO; }

namespace {
MarchArgs march_args(const fdtd2d_params& p, const FieldSet& in, const FieldSet& out, float* ez, int t0,
                     int* status, float* probe_ez) {
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
  a.pml_hint = has_pml(p) ? p.pml_cells : 0;
  return a;
}
}  // namespace

bool march_ext_supported(const fdtd2d_params& p) {
  if (p.nf > kMarchMaxNf) return false;
  if (p.tfsf_npml > 0 && p.ny > kLineMaxNy) return false;
  return true;
}

int launch_march_ext(const fdtd2d_params& p, const FieldSet& in, const FieldSet& out, float* ez, int t0, int k,
                     int* status, const MarchExt& ext, cudaStream_t st) {
  MarchArgs a = march_args(p, in, out, ez, t0, status, nullptr);
  a.ext = ext;
  const bool lossy = p.nbz != nullptr;
  const bool pml = has_pml(p);
  switch (p.nf) {
    case 0: return launch_ext_nf0(a, k, lossy, pml, st);
    case 1: return launch_ext_nf1(a, k, lossy, pml, st);
    case 2: return launch_ext_nf2(a, k, lossy, pml, st);
    case 3: return launch_ext_nf3(a, k, lossy, pml, st);
    case 4: return launch_ext_nf4(a, k, lossy, pml, st);
    default: return launch_ext_nfrt(a, k, lossy, pml, st);
  }
}

int launch_march(const fdtd2d_params& p, const FieldSet& in, const FieldSet& out, float* ez, int t0, int k,
                 int* status, float* probe_ez, cudaStream_t st) {
  const MarchArgs a = march_args(p, in, out, ez, t0, status, probe_ez);
  const bool lossy = p.nbz != nullptr;
  const bool pml = has_pml(p);
  // 128-column stripes unless the grid is too small to fill the GPU with
  // them (with the interior iterations they beat 64-column stripes at K = 4:
  // 386 against 350 Gcell/s at 8192^2)
  int cpl = g_cfg.cpl ? g_cfg.cpl : 4;
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

int launch_march_record(const fdtd2d_params& p, const FieldSet& in, const FieldSet& out, float* ez, int t0, int k,
                        const RecSet* rec, cudaStream_t st) {
  if (!has_pml(p) || k < 1 || k > HALO) return FDTD_ERR_UNSUPPORTED;
  MarchArgs a = march_args(p, in, out, ez, t0, nullptr, nullptr);
  for (int s = 0; s < k; ++s) a.rec[s] = rec[s];
  const bool lossy = p.nbz != nullptr;
  auto go = [&](auto kk) -> int {
    constexpr int K = decltype(kk)::value;
    if (lossy) return launch_t<K, 2, true, true, kTraceRecord>(a, g_cfg.warps, g_cfg.seg_rows, st);
    return launch_t<K, 2, false, true, kTraceRecord>(a, g_cfg.warps, g_cfg.seg_rows, st);
  };
  switch (k) {
    case 1: return go(std::integral_constant<int, 1>{});
    case 2: return go(std::integral_constant<int, 2>{});
    case 3: return go(std::integral_constant<int, 3>{});
    default: return go(std::integral_constant<int, 4>{});
  }
}

}  // namespace fdtd

extern "C" int fdtd2d_set_march_config(int cols_per_lane, int warps_per_block, int seg_rows) {
  if (cols_per_lane != 0 && cols_per_lane != 2 && cols_per_lane != 4) return FDTD_ERR_ARG;
  if (seg_rows < 0) return FDTD_ERR_ARG;
  fdtd::march::g_cfg.cpl = cols_per_lane;
  fdtd::march::g_cfg.warps = warps_per_block;
  fdtd::march::g_cfg.seg_rows = seg_rows;
  return FDTD_OK;
}

extern "C" int fdtd2d_set_march_balance(float gen_cost) {
  if (gen_cost != 0.f && (!(gen_cost >= 1.f) || gen_cost > 16.f)) return FDTD_ERR_ARG;
  fdtd::march::g_cfg.gen_cost = gen_cost;
  return FDTD_OK;
}
