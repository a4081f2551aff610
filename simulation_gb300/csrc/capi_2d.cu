// C-ABI entry points of the 2D TM path: argument checks, then launches.
#include <vector>

#include "fd2d_internal.cuh"

namespace {

using namespace fdtd;

inline bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

int check_params(const fdtd2d_params* p, const fdtd2d_state* s, int t_last, bool need_e, bool need_h) {
  if (!p || !s) return FDTD_ERR_NULL;
  if (p->nx < 3 || p->ny < 3) return FDTD_ERR_SIZE;
  if ((long long)p->nx * p->ny > (1LL << 34)) return FDTD_ERR_SIZE;
  if (!s->dz || !s->ez || !s->hx || !s->hy || !p->naz) return FDTD_ERR_NULL;
  if (p->nbz && !s->iz) return FDTD_ERR_NULL;
  const fdtd2d_pml& m = p->pml;
  const int npml_ptrs = (m.fx1 != nullptr) + (m.fx2 != nullptr) + (m.fx3 != nullptr) + (m.fy1 != nullptr) +
                        (m.fy2 != nullptr) + (m.fy3 != nullptr) + (m.gx2 != nullptr) + (m.gx3 != nullptr) +
                        (m.gy2 != nullptr) + (m.gy3 != nullptr);
  if (npml_ptrs != 0 && npml_ptrs != 10) return FDTD_ERR_NULL;
  if (npml_ptrs == 10 && need_h && (!s->ihx || !s->ihy)) return FDTD_ERR_NULL;
  if (p->src.kind < FDTD_SRC_NONE || p->src.kind > FDTD_SRC_SOFT) return FDTD_ERR_ARG;
  if (p->src.kind != FDTD_SRC_NONE) {
    if (p->src.i < 0 || p->src.i >= p->nx || p->src.j < 0 || p->src.j >= p->ny) return FDTD_ERR_ARG;
    if (!p->src.table) return FDTD_ERR_NULL;
    if (t_last > p->src.table_len) return FDTD_ERR_SIZE;
  }
  if (p->tfsf_npml < 0) return FDTD_ERR_SIZE;
  if (p->tfsf_npml > 0) {
    if (p->tfsf_npml < 2 || 2 * p->tfsf_npml >= p->nx || 2 * p->tfsf_npml >= p->ny || p->ny < 7)
      return FDTD_ERR_SIZE;
    if (!s->ezi || !s->hxi || !s->bc || !p->tfsf_table) return FDTD_ERR_NULL;
    if (t_last > p->tfsf_table_len) return FDTD_ERR_SIZE;
  }
  if (p->nf < 0) return FDTD_ERR_SIZE;
  if (p->nf > 0) {
    if (p->nf > 1024) return FDTD_ERR_SIZE;
    if (!p->dft_cos || !p->dft_sin || !s->r_pt || !s->i_pt) return FDTD_ERR_NULL;
    if (p->tfsf_npml > 0 && (!s->r_in || !s->i_in)) return FDTD_ERR_NULL;
    if (t_last > p->dft_table_len) return FDTD_ERR_SIZE;
  }
  if (s->probe_ez) {
    if (p->probe_i < 0 || p->probe_i >= p->nx || p->probe_j < 0 || p->probe_j >= p->ny) return FDTD_ERR_ARG;
    if (t_last > p->probe_len) return FDTD_ERR_SIZE;
  }
  (void)need_e;
  return FDTD_OK;
}

bool ext_on(const fdtd2d_params* p) { return p->tfsf_npml > 0 || p->nf > 0; }

// what the fused path needs of the parameters alone (the workspace query
// sees only these)
bool fused_params_ok(const fdtd2d_params* p) {
  if (p->ny % 4 != 0) return false;
  return !ext_on(p) || march_ext_supported(*p);
}

bool fused_ok(const fdtd2d_params* p, const fdtd2d_state* s) {
  if (!fused_params_ok(p)) return false;
  if (ext_on(p) && s->probe_ez) return false;  // the probe trace is kept by the plain kernels only
  if (p->nf > 0 && (!aligned16(s->r_pt) || !aligned16(s->i_pt))) return false;
  const void* ptrs[] = {s->dz, s->ez, s->hx, s->hy, p->naz};
  for (const void* q : ptrs)
    if (!aligned16(q)) return false;
  if (p->nbz && (!aligned16(p->nbz) || !aligned16(s->iz))) return false;
  if (has_pml(*p) && (!aligned16(s->ihx) || !aligned16(s->ihy))) return false;
  return true;
}

size_t slot_bytes(const fdtd2d_params* p) {
  const size_t b = (size_t)p->nx * p->ny * sizeof(float);
  return (b + 255) & ~(size_t)255;
}

int nslots(const fdtd2d_params* p) { return 3 + (p->nbz ? 1 : 0) + (has_pml(*p) ? 2 : 0); }

size_t round256(size_t b) { return (b + 255) & ~(size_t)255; }

// incident-line tables of one chunk of steps (TF/SF): inc_e [chunk][ny],
// inc_h [chunk][2]
size_t line_e_bytes(const fdtd2d_params* p) { return round256((size_t)kLineChunkSteps * p->ny * sizeof(float)); }
size_t line_bytes(const fdtd2d_params* p) {
  return p->tfsf_npml > 0 ? line_e_bytes(p) + round256((size_t)kLineChunkSteps * 2 * sizeof(float)) : 0;
}
size_t fused_workspace_bytes(const fdtd2d_params* p) { return slot_bytes(p) * nslots(p) + line_bytes(p); }

// one time step in the reference's order (fd2d/python/fd2d_3_4.py:268-277):
// ezinct, dfield, inctdz, efield, fourier, hxinct, hfield, incthx, incthy in
// three launches (launch_step3), bitwise equal to the nine functions
int step_three_launches(int t, const fdtd2d_params& p, const fdtd2d_state& s, cudaStream_t st) {
  int rc;
  if ((rc = launch_step3(t, p, s, st))) return rc;
  if (s.probe_ez) {
    const cudaError_t e = cudaMemcpyAsync(s.probe_ez + (t - 1), s.ez + (size_t)p.probe_i * p.ny + p.probe_j,
                                          sizeof(float), cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) {
      fdtd_host::note_cuda_error(e);
      return FDTD_ERR_CUDA;
    }
  }
  return FDTD_OK;
}

}  // namespace

extern "C" {

int fdtd2d_dfield(int t, const fdtd2d_params* p, fdtd2d_state* s, fdtd_stream_t stream) {
  int rc = check_params(p, s, t, false, false);
  if (rc) return rc;
  if (t < 1) return FDTD_ERR_ARG;
  return launch_dfield(t, *p, *s, (cudaStream_t)stream);
}

int fdtd2d_efield(const fdtd2d_params* p, fdtd2d_state* s, fdtd_stream_t stream) {
  int rc = check_params(p, s, 0, true, false);
  if (rc) return rc;
  return launch_efield(*p, *s, (cudaStream_t)stream);
}

int fdtd2d_hfield(const fdtd2d_params* p, fdtd2d_state* s, fdtd_stream_t stream) {
  int rc = check_params(p, s, 0, false, true);
  if (rc) return rc;
  return launch_hfield(*p, *s, (cudaStream_t)stream);
}

int fdtd2d_ezinct(const fdtd2d_params* p, fdtd2d_state* s, fdtd_stream_t stream) {
  int rc = check_params(p, s, 0, false, false);
  if (rc) return rc;
  if (p->tfsf_npml <= 0) return FDTD_ERR_ARG;
  return launch_ezinct(*p, *s, (cudaStream_t)stream);
}

int fdtd2d_inctdz(const fdtd2d_params* p, fdtd2d_state* s, fdtd_stream_t stream) {
  int rc = check_params(p, s, 0, false, false);
  if (rc) return rc;
  if (p->tfsf_npml <= 0) return FDTD_ERR_ARG;
  return launch_inctdz(*p, *s, (cudaStream_t)stream);
}

int fdtd2d_hxinct(const fdtd2d_params* p, fdtd2d_state* s, fdtd_stream_t stream) {
  int rc = check_params(p, s, 0, false, false);
  if (rc) return rc;
  if (p->tfsf_npml <= 0) return FDTD_ERR_ARG;
  return launch_hxinct(*p, *s, (cudaStream_t)stream);
}

int fdtd2d_incth(const fdtd2d_params* p, fdtd2d_state* s, fdtd_stream_t stream) {
  int rc = check_params(p, s, 0, false, false);
  if (rc) return rc;
  if (p->tfsf_npml <= 0) return FDTD_ERR_ARG;
  return launch_incth(*p, *s, (cudaStream_t)stream);
}

int fdtd2d_fourier(int t, const fdtd2d_params* p, fdtd2d_state* s, fdtd_stream_t stream) {
  int rc = check_params(p, s, t, false, false);
  if (rc) return rc;
  if (t < 1 || p->nf <= 0) return FDTD_ERR_ARG;
  return launch_fourier(t, *p, *s, (cudaStream_t)stream);
}

size_t fdtd2d_workspace_size(const fdtd2d_params* p, int steps_per_pass) {
  (void)steps_per_pass;
  if (!p || p->nx < 3 || p->ny < 3) return 0;
  if (!fused_params_ok(p)) return 0;
  return fused_workspace_bytes(p);
}

int fdtd2d_step_n(const fdtd2d_params* p, fdtd2d_state* s, int t0, int nsteps, int steps_per_pass, void* workspace,
                  size_t workspace_bytes, fdtd_stream_t stream) {
  if (t0 < 0 || nsteps < 0) return FDTD_ERR_ARG;
  int rc = check_params(p, s, t0 + nsteps, true, true);
  if (rc) return rc;
  if (steps_per_pass < 0 || steps_per_pass > march_max_steps_per_pass()) return FDTD_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  if (nsteps == 0) return FDTD_OK;

  if (!fused_ok(p, s) || nsteps == 1) {
    for (int t = t0 + 1; t <= t0 + nsteps; ++t)
      if ((rc = step_three_launches(t, *p, *s, st))) return rc;
    if (s->status) launch_check_finite(s->ez, (size_t)p->nx * p->ny, s->status, st);
    return fdtd_host::check_launch();
  }

  const size_t need = fused_workspace_bytes(p);
  if (!workspace || workspace_bytes < need) return FDTD_ERR_WORKSPACE;
  if (((uintptr_t)workspace & 255u) != 0) return FDTD_ERR_ALIGN;

  // pass schedule with an even number of passes, so the last pass writes the
  // caller's arrays (split one pass if needed)
  const int K = steps_per_pass == 0 ? march_default_steps(p->nx, p->ny) : steps_per_pass;
  std::vector<int> sched;
  for (int rem = nsteps; rem > 0;) {
    const int k = rem < K ? rem : K;
    sched.push_back(k);
    rem -= k;
  }
  bool copy_back = false;
  if (sched.size() % 2 == 1) {
    size_t idx = sched.size();
    for (size_t i = 0; i < sched.size(); ++i)
      if (sched[i] >= 2) {
        idx = i;
        break;
      }
    if (idx < sched.size()) {
      const int k = sched[idx];
      sched[idx] = k / 2;
      sched.insert(sched.begin() + idx + 1, k - k / 2);
    } else {
      copy_back = true;
    }
  }

  FieldSet user{s->dz, s->iz, s->hx, s->hy, s->ihx, s->ihy};
  FieldSet ws{};
  {
    char* base = (char*)workspace;
    const size_t sb = slot_bytes(p);
    int k = 0;
    ws.dz = (float*)(base + sb * k++);
    ws.hx = (float*)(base + sb * k++);
    ws.hy = (float*)(base + sb * k++);
    if (p->nbz) ws.iz = (float*)(base + sb * k++);
    if (has_pml(*p)) {
      ws.ihx = (float*)(base + sb * k++);
      ws.ihy = (float*)(base + sb * k++);
    }
  }
  MarchExt ext{};
  float* inc_e = nullptr;
  float* inc_h = nullptr;
  if (ext_on(p)) {
    ext.tfsf_npml = p->tfsf_npml;
    ext.nf = p->nf;
    ext.dft_cos = p->dft_cos;
    ext.dft_sin = p->dft_sin;
    ext.r_pt = s->r_pt;
    ext.i_pt = s->i_pt;
    if (p->tfsf_npml > 0) {
      char* lb = (char*)workspace + slot_bytes(p) * nslots(p);
      inc_e = (float*)lb;
      inc_h = (float*)(lb + line_e_bytes(p));
    }
    // (without TF/SF no warp runs the edge logic that reads the tables)
    ext.inc_e = inc_e;
    ext.inc_h = inc_h;
  }
  int t = t0;
  int line_t0 = t0, line_n = 0;  // steps the incident-line tables hold
  for (size_t i = 0; i < sched.size(); ++i) {
    const FieldSet& in = (i % 2 == 0) ? user : ws;
    const FieldSet& out = (i % 2 == 0) ? ws : user;
    // the last pass alone tests the fields it writes for Inf/NaN: a non-finite
    // value never turns finite again under the update (every operation on
    // Inf/NaN yields Inf/NaN, and it spreads to the neighbours each step), so
    // that one test sees anything an earlier pass would have
    int* status = (i + 1 == sched.size()) ? s->status : nullptr;
    if (!ext_on(p)) {
      rc = launch_march(*p, in, out, s->ez, t, sched[i], status, s->probe_ez, st);
    } else {
      if (p->tfsf_npml > 0) {
        if (t + sched[i] > line_t0 + line_n) {  // next chunk of whole passes
          int n = 0;
          for (size_t q = i; q < sched.size() && n + sched[q] <= kLineChunkSteps; ++q) n += sched[q];
          if ((rc = launch_inc_line(*p, *s, t, n, inc_e, inc_h, st))) return rc;
          line_t0 = t;
          line_n = n;
        }
        ext.inc_e = inc_e + (size_t)(t - line_t0) * p->ny;
        ext.inc_h = inc_h + (size_t)(t - line_t0) * 2;
      }
      rc = launch_march_ext(*p, in, out, s->ez, t, sched[i], status, ext, st);
    }
    if (rc) return rc;
    t += sched[i];
  }
  if (copy_back) {
    const size_t b = (size_t)p->nx * p->ny * sizeof(float);
    float* pairs[6][2] = {{user.dz, ws.dz}, {user.hx, ws.hx}, {user.hy, ws.hy},
                          {user.iz, ws.iz}, {user.ihx, ws.ihx}, {user.ihy, ws.ihy}};
    for (auto& pr : pairs)
      if (pr[0] && pr[1]) {
        const cudaError_t e = cudaMemcpyAsync(pr[0], pr[1], b, cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) {
          fdtd_host::note_cuda_error(e);
          return FDTD_ERR_CUDA;
        }
      }
  }
  return FDTD_OK;
}

int fdtd2d_dielectric_cylinder(int nx, int ny, int npml, double rgrid, double dt, double epsr, double sigma,
                               float* naz, float* nbz, fdtd_stream_t stream) {
  if (!naz || !nbz) return FDTD_ERR_NULL;
  if (nx < 3 || ny < 3 || npml < 0 || 2 * npml > nx || 2 * npml > ny) return FDTD_ERR_SIZE;
  if (!(dt > 0) || !(epsr > 0) || sigma < 0) return FDTD_ERR_ARG;
  return launch_dielectric(nx, ny, npml, rgrid, dt, epsr, sigma, naz, nbz, (cudaStream_t)stream);
}

int fdtd_check_finite(const float* x, size_t n, int* status, fdtd_stream_t stream) {
  if (!x || !status) return FDTD_ERR_NULL;
  return launch_check_finite(x, n, status, (cudaStream_t)stream);
}

}  // extern "C"
