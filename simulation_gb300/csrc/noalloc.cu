// fdtd2d_step_n_noalloc: the fused 2D time loop for callers that cannot
// allocate device memory.
//
// Who needs it: code that runs where cudaMalloc is unavailable or forbidden
// (a host application with a fixed memory budget that pre-reserves
// everything, a plugin called inside another framework's stream capture or
// memory pool, an embedded runtime without an allocator of its own).  Such a
// caller still owns the field arrays but cannot provide the ping-pong
// workspace fdtd2d_step_n needs.
//
// What it does: the workspace is a file-scope static device array of
// FDTD2D_NOALLOC_SCRATCH_BYTES (24 MiB: six fields of up to
// FDTD2D_NOALLOC_MAX_CELLS = 1024*1024 cells).  Every GPU that loads this
// library holds that array until the process exits.  The call allocates
// nothing (no cudaMalloc/cudaFree, no allocating library routine): it looks
// the array's device address up once per device and hands it to
// fdtd2d_step_n as the workspace.  Everything else is fdtd2d_step_n's code
// path, unchanged.
//
// Limits and caveats (also in include/fdtd.h):
//   * grids whose workspace exceeds the array are rejected with FDTD_ERR_SIZE,
//     except with TF/SF or the DFT on, where the incident-line tables may not
//     fit beside the fields: those runs go one step per fdtd2d_step_n call
//     (its three-launch form, which needs no workspace);
//   * the first call on a device resolves the array's address with
//     cudaGetSymbolAddress; with lazy module loading that is when the driver
//     reserves the array, so the first call can fail with FDTD_ERR_CUDA when
//     the device is out of memory: make it up front, before any stream
//     capture; the address is kept per device and context, and looked up
//     again when the current context is a new one (after a cudaDeviceReset);
//   * all calls share the one array and it keeps the last call's contents;
//     nothing in it has to start at zero (each call's first pass overwrites
//     it before reading it), but calls whose work overlaps on the GPU (two
//     streams, two host threads) race on it.
#include <dlfcn.h>

#include <mutex>

#include "fdtd_common.cuh"

namespace {

constexpr size_t kScratchBytes = (size_t)FDTD2D_NOALLOC_SCRATCH_BYTES;

// the workspace; only device code may name it directly, host code must use the
// address returned by cudaGetSymbolAddress (the host-side symbol is a stand-in)
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_addr[kMaxDevices] = {nullptr};
unsigned long long g_ctx[kMaxDevices] = {0};  // the context the address belongs to (0: unknown)

// Unique ID of the calling thread's current context (CUDA 12+ driver, found
// in the driver library the runtime has already loaded; nothing is linked),
// or 0 where it cannot be told.  A context created anew (after a
// cudaDeviceReset, say) has a new ID, so the scratch address is looked up again.
unsigned long long current_context_id() {
  using GetCurrent = int (*)(void**);
  using GetId = int (*)(void*, unsigned long long*);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* h = dlopen("libcuda.so.1", RTLD_NOW | RTLD_NOLOAD);
    if (h) {
      get_current = reinterpret_cast<GetCurrent>(dlsym(h, "cuCtxGetCurrent"));
      get_id = reinterpret_cast<GetId>(dlsym(h, "cuCtxGetId"));
    }
  });
  if (!get_current || !get_id) return 0;
  void* ctx = nullptr;
  unsigned long long id = 0;
  if (get_current(&ctx) != 0 || ctx == nullptr || get_id(ctx, &id) != 0) return 0;
  return id;
}

int scratch_address(void** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    fdtd_host::note_cuda_error(e);
    return FDTD_ERR_CUDA;
  }
  if (dev < 0 || dev >= kMaxDevices) return FDTD_ERR_UNSUPPORTED;
  const unsigned long long ctx = current_context_id();
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_addr[dev] || (ctx != 0 && ctx != g_ctx[dev])) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
      fdtd_host::note_cuda_error(e);
      return FDTD_ERR_CUDA;
    }
    g_addr[dev] = p;
    g_ctx[dev] = ctx;
  }
  *out = g_addr[dev];
  return FDTD_OK;
}

}  // namespace

extern "C" int fdtd2d_step_n_noalloc(const fdtd2d_params* p, fdtd2d_state* s, int t0, int nsteps,
                                     int steps_per_pass, fdtd_stream_t stream) {
  if (!p || !s) return FDTD_ERR_NULL;
  if (t0 < 0 || nsteps < 0) return FDTD_ERR_ARG;  // as fdtd2d_step_n, before either path
  if ((long long)p->nx * p->ny > (long long)FDTD2D_NOALLOC_MAX_CELLS) return FDTD_ERR_SIZE;
  const size_t need = fdtd2d_workspace_size(p, steps_per_pass);
  if (need > kScratchBytes) {
    if (p->tfsf_npml <= 0 && p->nf <= 0) return FDTD_ERR_SIZE;
    // one-step calls (three launches each, no workspace); the Inf/NaN test,
    // which every call would otherwise run, runs once after the last step
    fdtd2d_state quiet = *s;
    quiet.status = nullptr;
    for (int i = 0; i < nsteps; ++i) {
      const int rc = fdtd2d_step_n(p, i + 1 == nsteps ? s : &quiet, t0 + i, 1, steps_per_pass, nullptr, 0,
                                   stream);
      if (rc != FDTD_OK) return rc;
    }
    return FDTD_OK;
  }
  void* ws = nullptr;
  if (need > 0) {
    const int rc = scratch_address(&ws);
    if (rc != FDTD_OK) return rc;
  }
  return fdtd2d_step_n(p, s, t0, nsteps, steps_per_pass, ws, need > 0 ? kScratchBytes : 0, stream);
}
