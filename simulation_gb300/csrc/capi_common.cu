// Library-wide C-ABI helpers: version, status codes, CUDA error recording.
#include <atomic>

#include "fdtd_common.cuh"

namespace fdtd_host {

static std::atomic<int> g_last_cuda_error{0};

void note_cuda_error(cudaError_t e) {
  if (e != cudaSuccess) g_last_cuda_error.store((int)e);
}

int check_launch() {
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    note_cuda_error(e);
    return FDTD_ERR_CUDA;
  }
  return FDTD_OK;
}

}  // namespace fdtd_host

extern "C" {

int fdtd_version(void) { return 100; }

const char* fdtd_status_string(int status) {
  switch (status) {
    case FDTD_OK: return "ok";
    case FDTD_ERR_NULL: return "a required pointer is NULL";
    case FDTD_ERR_SIZE: return "grid size, PML width or step count out of range";
    case FDTD_ERR_ALIGN: return "pointer not 16-byte aligned";
    case FDTD_ERR_ARG: return "invalid argument";
    case FDTD_ERR_CUDA: return "CUDA call failed";
    case FDTD_ERR_NONFINITE: return "a field became Inf/NaN";
    case FDTD_ERR_TIMEOUT: return "a bounded device wait ran out";
    case FDTD_ERR_UNSUPPORTED: return "unsupported combination of options";
    case FDTD_ERR_WORKSPACE: return "workspace missing or too small";
    default: return "unknown status";
  }
}

int fdtd_last_cuda_error(void) { return fdtd_host::g_last_cuda_error.load(); }

int fdtd_status_to_error(int device_status) {
  if (device_status & FDTD_STATUS_TIMEOUT) return FDTD_ERR_TIMEOUT;
  if (device_status & FDTD_STATUS_NONFINITE) return FDTD_ERR_NONFINITE;
  if (device_status & FDTD_STATUS_BOUNDS) return FDTD_ERR_SIZE;
  return FDTD_OK;
}

}  // extern "C"
