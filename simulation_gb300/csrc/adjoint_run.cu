// fdtd2d_tm_adjoint: the gradient of J = sum_t (w/2) ez_t[probe]^2 with
// respect to naz (and nbz) over a design box, in one call: a checkpointed
// forward run and the reverse sweep.  No counterpart in the reference (it
// only runs forward); the map being differentiated is its step,
// fd2d/python/fd2d_3_2.py:62-88 with the lossy E update of
// fd2d/python/fd2d_3_4.py:131-136 and a point source after the D update.
//
// Schedule (all in the caller's workspace, nothing allocated):
//   forward   fused passes of up to 4 steps from zero fields; each segment
//             of `checkpoint` steps starts from a stored state (the previous
//             segment's last pass writes it directly) and the probe's Ez is
//             recorded every step; J is summed on the device in double;
//   reverse   segments last first.  A segment's states are recomputed from
//             its checkpoint by recording passes (one pass of 4 steps stores
//             dz, iz, hx, hy after each of its steps), on a second stream,
//             one segment ahead of the sweep (two record buffers, events
//             order their reuse); the sweep runs one fused reverse kernel per
//             two steps (one step for an odd segment's first), the adjoint
//             fields ping-ponging between two sets.
// Results do not depend on the checkpoint interval or on the overlap: every
// recorded state is bitwise the forward's, and each reverse step does the
// same per-cell arithmetic (fdtd2d_adjoint_step's two kernels give the same
// bits).
#include <cstdint>
#include <mutex>
#include <vector>

#include "fd2d_internal.cuh"

namespace fdtd {
int launch_adjoint_fused(const fdtd2d_params& p, int t, const fdtd2d_fields& fwd, const fdtd2d_fields& adj_in,
                         const fdtd2d_fields& adj_out, int probe_i, int probe_j, float probe_w,
                         const fdtd2d_box& box, float* grad_naz, float* grad_nbz, cudaStream_t st);
int launch_adjoint_fused2(const fdtd2d_params& p, int t, const fdtd2d_fields& fwd1, const fdtd2d_fields& fwd0,
                          const fdtd2d_fields& adj_in, const fdtd2d_fields& adj_out, int probe_i, int probe_j,
                          float probe_w, const fdtd2d_box& box, float* grad_naz, float* grad_nbz, cudaStream_t st);
}  // namespace fdtd

namespace {

using namespace fdtd;

constexpr int kMaxK = 4;  // most steps per fused pass (the record buffers of one pass)

size_t slot(const fdtd2d_params* p) { return (((size_t)p->nx * p->ny * sizeof(float)) + 255) & ~(size_t)255; }
int nfields(const fdtd2d_params* p) { return p->nbz ? 6 : 5; }  // dz, [iz], hx, hy, ihx, ihy
int nrec(const fdtd2d_params* p) { return p->nbz ? 4 : 3; }     // dz, [iz], hx, hy

struct Layout {
  int ncp, cp;
  size_t slot;
  char* base;
  // slot indices
  size_t ckpt0, x0, ez, rec0, adj0, jbuf, end;
};

Layout layout(const fdtd2d_params* p, const fdtd2d_adjoint_params* a, void* ws) {
  Layout L{};
  L.cp = a->checkpoint;
  L.ncp = (a->nsteps + L.cp - 1) / L.cp;
  L.slot = slot(p);
  L.base = (char*)ws;
  const int F = nfields(p), R = nrec(p);
  size_t s = 0;
  L.ckpt0 = s;
  s += (size_t)(L.ncp + 1) * F;  // states before segments 0..ncp-1 and the final state
  L.x0 = s;
  s += 2 * (size_t)F;  // pass ping-pong
  L.ez = s;
  s += 1;
  L.rec0 = s;
  s += 2 * (size_t)(L.cp > 1 ? L.cp - 1 : 0) * R;  // two record buffers
  L.adj0 = s;
  s += 2 * (size_t)F;  // adjoint ping-pong
  L.jbuf = s;
  s += 1;  // J accumulator and spare
  L.end = s;
  return L;
}

float* at(const Layout& L, size_t k) { return (float*)(L.base + L.slot * k); }

// F consecutive slots -> fields (iz absent for the lossless update)
fdtd2d_fields fields_at(const fdtd2d_params* p, const Layout& L, size_t k) {
  fdtd2d_fields f{};
  f.dz = at(L, k++);
  if (p->nbz) f.iz = at(L, k++);
  f.hx = at(L, k++);
  f.hy = at(L, k++);
  f.ihx = at(L, k++);
  f.ihy = at(L, k++);
  return f;
}
FieldSet set_of(const fdtd2d_fields& f) { return FieldSet{f.dz, f.iz, f.hx, f.hy, f.ihx, f.ihy}; }
fdtd2d_fields ckpt(const fdtd2d_params* p, const Layout& L, int c) {
  return fields_at(p, L, L.ckpt0 + (size_t)c * nfields(p));
}
fdtd2d_fields xbuf(const fdtd2d_params* p, const Layout& L, int b) {
  return fields_at(p, L, L.x0 + (size_t)b * nfields(p));
}
fdtd2d_fields adjbuf(const fdtd2d_params* p, const Layout& L, int b) {
  return fields_at(p, L, L.adj0 + (size_t)b * nfields(p));
}
// recorded state k (after step t_start+k+1) of record buffer b
RecSet rec(const fdtd2d_params* p, const Layout& L, int b, int k) {
  const int R = nrec(p);
  size_t s = L.rec0 + ((size_t)b * (L.cp - 1) + k) * R;
  RecSet r{};
  r.dz = at(L, s++);
  if (p->nbz) r.iz = at(L, s++);
  r.hx = at(L, s++);
  r.hy = at(L, s++);
  return r;
}

int cuda_rc(cudaError_t e) {
  if (e == cudaSuccess) return FDTD_OK;
  fdtd_host::note_cuda_error(e);
  return FDTD_ERR_CUDA;
}

int zero_fields(const fdtd2d_params* p, const fdtd2d_fields& f, cudaStream_t st) {
  const size_t b = (size_t)p->nx * p->ny * sizeof(float);
  float* all[] = {f.dz, f.iz, f.hx, f.hy, f.ihx, f.ihy};
  for (float* q : all)
    if (q) {
      const int rc = cuda_rc(cudaMemsetAsync(q, 0, b, st));
      if (rc) return rc;
    }
  return FDTD_OK;
}

// J = sum_t (w/2) trace[t]^2 in double, one block
__global__ void k_objective(const float* trace, int n, float w, double* J) {
  __shared__ double part[256];
  double s = 0.0;
  for (int t = threadIdx.x; t < n; t += blockDim.x) {
    const double v = trace[t];
    s += v * v;
  }
  part[threadIdx.x] = s;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) part[threadIdx.x] += part[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) *J = 0.5 * (double)w * part[0];
}

// the reverse sweep's second stream and its events, made once per device
struct Side {
  cudaStream_t stream = nullptr;
  cudaEvent_t fork = nullptr, ready[2] = {nullptr, nullptr}, free_[2] = {nullptr, nullptr};
};
constexpr int kMaxDevices = 64;
std::mutex g_side_mu;
Side g_side[kMaxDevices];

int side_of_device(Side** out) {
  int dev = -1;
  int rc = cuda_rc(cudaGetDevice(&dev));
  if (rc) return rc;
  if (dev < 0 || dev >= kMaxDevices) return FDTD_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lk(g_side_mu);
  Side& s = g_side[dev];
  if (!s.stream) {
    if ((rc = cuda_rc(cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking)))) return rc;
    cudaEvent_t* evs[] = {&s.fork, &s.ready[0], &s.ready[1], &s.free_[0], &s.free_[1]};
    for (cudaEvent_t* e : evs)
      if ((rc = cuda_rc(cudaEventCreateWithFlags(e, cudaEventDisableTiming)))) return rc;
  }
  *out = &s;
  return FDTD_OK;
}

int check(const fdtd2d_params* p, const fdtd2d_adjoint_params* a) {
  if (!p || !a) return FDTD_ERR_NULL;
  if (p->nx < 3 || p->ny < 3 || p->ny % 4) return FDTD_ERR_SIZE;
  if ((long long)p->nx * p->ny > (1LL << 34)) return FDTD_ERR_SIZE;
  if (!has_pml(*p)) return FDTD_ERR_UNSUPPORTED;  // pass unit profiles for no absorbing layer
  const fdtd2d_pml& m = p->pml;
  if (!m.fx2 || !m.fx3 || !m.fy1 || !m.fy2 || !m.fy3 || !m.gx2 || !m.gx3 || !m.gy2 || !m.gy3) return FDTD_ERR_NULL;
  if (!p->naz) return FDTD_ERR_NULL;
  if (((uintptr_t)p->naz & 15u) || ((uintptr_t)p->nbz & 15u)) return FDTD_ERR_ALIGN;
  if (p->tfsf_npml > 0 || p->nf > 0) return FDTD_ERR_UNSUPPORTED;
  if (a->nsteps < 1 || a->checkpoint < 1) return FDTD_ERR_ARG;
  if (p->src.kind < FDTD_SRC_NONE || p->src.kind > FDTD_SRC_SOFT) return FDTD_ERR_ARG;
  if (p->src.kind != FDTD_SRC_NONE) {
    if (!p->src.table) return FDTD_ERR_NULL;
    if (p->src.i < 0 || p->src.i >= p->nx || p->src.j < 0 || p->src.j >= p->ny) return FDTD_ERR_ARG;
    if (a->nsteps > p->src.table_len) return FDTD_ERR_SIZE;
  }
  if (a->probe_i < 0 || a->probe_i >= p->nx || a->probe_j < 0 || a->probe_j >= p->ny) return FDTD_ERR_ARG;
  const fdtd2d_box& b = a->box;
  if (b.ni <= 0 || b.nj <= 0 || b.i0 < 0 || b.j0 < 0 || b.i0 + b.ni > p->nx || b.j0 + b.nj > p->ny)
    return FDTD_ERR_ARG;
  return FDTD_OK;
}

int check_ws(const fdtd2d_params* p, const fdtd2d_adjoint_params* a, void* ws, size_t bytes) {
  if (!ws) return FDTD_ERR_WORKSPACE;
  if ((uintptr_t)ws & 255u) return FDTD_ERR_ALIGN;
  const Layout L = layout(p, a, ws);
  if (bytes < L.slot * L.end) return FDTD_ERR_WORKSPACE;
  return FDTD_OK;
}

int run_forward(const fdtd2d_params* p0, const fdtd2d_adjoint_params* a, float* trace, double* J, void* ws,
                cudaStream_t st) {
  const Layout L = layout(p0, a, ws);
  fdtd2d_params p = *p0;  // the probe of the objective
  p.probe_i = a->probe_i;
  p.probe_j = a->probe_j;
  p.probe_len = a->nsteps;
  int rc = zero_fields(&p, ckpt(&p, L, 0), st);
  if (rc) return rc;
  if ((rc = cuda_rc(cudaMemsetAsync(trace, 0, (size_t)a->nsteps * sizeof(float), st)))) return rc;
  float* ez = at(L, L.ez);
  for (int c = 0; c < L.ncp; ++c) {
    const int t_start = c * L.cp;
    const int len = std::min(L.cp, a->nsteps - t_start);
    const int kk = march_default_steps(p.nx, p.ny);
    const int npass = (len + kk - 1) / kk;
    fdtd2d_fields in = ckpt(&p, L, c);
    for (int i = 0, t = t_start; i < npass; ++i) {
      const int k = std::min(kk, t_start + len - t);
      const fdtd2d_fields out = (i + 1 == npass) ? ckpt(&p, L, c + 1) : xbuf(&p, L, i % 2);
      if ((rc = launch_march(p, set_of(in), set_of(out), ez, t, k, nullptr, trace, st))) return rc;
      in = out;
      t += k;
    }
  }
  if (J) {
    k_objective<<<1, 256, 0, st>>>(trace, a->nsteps, a->probe_weight, J);
    if ((rc = fdtd_host::check_launch())) return rc;
  }
  return FDTD_OK;
}

// states before steps t_start+2 .. t_start+len of segment c into record buffer b
int recompute(const fdtd2d_params* p, const Layout& L, int c, int len, int b, cudaStream_t st) {
  const int t_start = c * L.cp;
  const int t_end = t_start + len - 1;  // the last state needed is after step t_end
  fdtd2d_fields in = ckpt(p, L, c);
  float* ez = at(L, L.ez);
  for (int t = t_start, i = 0; t < t_end; ++i) {
    const int k = std::min(march_default_steps(p->nx, p->ny), t_end - t);
    RecSet r[kMaxK];
    for (int s = 0; s < k; ++s) r[s] = rec(p, L, b, t - t_start + s);
    const fdtd2d_fields out = xbuf(p, L, i % 2);
    const int rc = launch_march_record(*p, set_of(in), set_of(out), ez, t, k, r, st);
    if (rc) return rc;
    in = out;
    t += k;
  }
  return FDTD_OK;
}

int run_reverse(const fdtd2d_params* p, const fdtd2d_adjoint_params* a, float* grad_naz, float* grad_nbz,
                void* ws, cudaStream_t main) {
  const Layout L = layout(p, a, ws);
  Side* side = nullptr;
  int rc = side_of_device(&side);
  if (rc) return rc;
  cudaStream_t ss = side->stream;
  const size_t gb = (size_t)a->box.ni * a->box.nj * sizeof(float);
  if ((rc = zero_fields(p, adjbuf(p, L, 0), main))) return rc;
  if ((rc = cuda_rc(cudaMemsetAsync(grad_naz, 0, gb, main)))) return rc;
  if (grad_nbz && (rc = cuda_rc(cudaMemsetAsync(grad_nbz, 0, gb, main)))) return rc;
  // the side stream starts after everything before this call on the caller's stream
  if ((rc = cuda_rc(cudaEventRecord(side->fork, main)))) return rc;
  if ((rc = cuda_rc(cudaStreamWaitEvent(ss, side->fork, 0)))) return rc;

  auto seg_len = [&](int c) { return std::min(L.cp, a->nsteps - c * L.cp); };
  std::vector<int> order;
  for (int c = L.ncp - 1; c >= 0; --c) order.push_back(c);
  if ((rc = recompute(p, L, order[0], seg_len(order[0]), 0, ss))) return rc;
  if ((rc = cuda_rc(cudaEventRecord(side->ready[0], ss)))) return rc;
  int cur = 0;  // adjoint set holding the adjoints after the step being undone
  for (size_t idx = 0; idx < order.size(); ++idx) {
    const int c = order[idx], b = (int)(idx % 2);
    if (idx + 1 < order.size()) {
      const int nb = 1 - b;
      if (idx >= 1 && (rc = cuda_rc(cudaStreamWaitEvent(ss, side->free_[nb], 0)))) return rc;
      if ((rc = recompute(p, L, order[idx + 1], seg_len(order[idx + 1]), nb, ss))) return rc;
      if ((rc = cuda_rc(cudaEventRecord(side->ready[nb], ss)))) return rc;
    }
    if ((rc = cuda_rc(cudaStreamWaitEvent(main, side->ready[b], 0)))) return rc;
    const int t_start = c * L.cp, len = seg_len(c);
    // the state before step t: the checkpoint, or a recorded state
    auto fwd_of = [&](int t) {
      if (t == t_start + 1) return ckpt(p, L, c);
      const RecSet r = rec(p, L, b, t - t_start - 2);
      return fdtd2d_fields{r.dz, r.iz, r.hx, r.hy, nullptr, nullptr};
    };
    // two steps per launch; an odd segment's first step alone
    for (int t = t_start + len; t > t_start; t -= 2) {
      if (t - 1 > t_start)
        rc = launch_adjoint_fused2(*p, t, fwd_of(t), fwd_of(t - 1), adjbuf(p, L, cur), adjbuf(p, L, 1 - cur),
                                   a->probe_i, a->probe_j, a->probe_weight, a->box, grad_naz, grad_nbz, main);
      else
        rc = launch_adjoint_fused(*p, t, fwd_of(t), adjbuf(p, L, cur), adjbuf(p, L, 1 - cur), a->probe_i,
                                  a->probe_j, a->probe_weight, a->box, grad_naz, grad_nbz, main);
      if (rc) return rc;
      cur = 1 - cur;
    }
    if ((rc = cuda_rc(cudaEventRecord(side->free_[b], main)))) return rc;
  }
  return FDTD_OK;
}

}  // namespace

extern "C" {

size_t fdtd2d_tm_adjoint_workspace_size(const fdtd2d_params* p, const fdtd2d_adjoint_params* a) {
  if (check(p, a) != FDTD_OK) return 0;
  const Layout L = layout(p, a, nullptr);
  return L.slot * L.end;
}

int fdtd2d_tm_adjoint_forward(const fdtd2d_params* p, const fdtd2d_adjoint_params* a, float* trace, double* J,
                              void* workspace, size_t workspace_bytes, fdtd_stream_t stream) {
  int rc = check(p, a);
  if (rc) return rc;
  if (!trace) return FDTD_ERR_NULL;
  if ((rc = check_ws(p, a, workspace, workspace_bytes))) return rc;
  return run_forward(p, a, trace, J, workspace, (cudaStream_t)stream);
}

int fdtd2d_tm_adjoint_reverse(const fdtd2d_params* p, const fdtd2d_adjoint_params* a, float* grad_naz,
                              float* grad_nbz, void* workspace, size_t workspace_bytes, fdtd_stream_t stream) {
  int rc = check(p, a);
  if (rc) return rc;
  if (!grad_naz) return FDTD_ERR_NULL;
  if (grad_nbz && !p->nbz) return FDTD_ERR_ARG;
  if ((rc = check_ws(p, a, workspace, workspace_bytes))) return rc;
  return run_reverse(p, a, grad_naz, grad_nbz, workspace, (cudaStream_t)stream);
}

int fdtd2d_tm_adjoint(const fdtd2d_params* p, const fdtd2d_adjoint_params* a, float* trace, double* J,
                      float* grad_naz, float* grad_nbz, void* workspace, size_t workspace_bytes,
                      fdtd_stream_t stream) {
  int rc = check(p, a);
  if (rc) return rc;
  if (!trace || !grad_naz) return FDTD_ERR_NULL;
  if (grad_nbz && !p->nbz) return FDTD_ERR_ARG;
  if ((rc = check_ws(p, a, workspace, workspace_bytes))) return rc;
  if ((rc = run_forward(p, a, trace, J, workspace, (cudaStream_t)stream))) return rc;
  return run_reverse(p, a, grad_naz, grad_nbz, workspace, (cudaStream_t)stream);
}

}  // extern "C"
