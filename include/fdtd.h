/* fdtd.h -- C-ABI of the GB300 (sm_103a) FDTD library, libfdtd_gb300.so.
 *
 * Drop-in replacement for the time-step hot path of dsarvan/simulation:
 *   (a) the 1D Ex/Hy leapfrog of fd1d (free space, dielectric, lossy, D-form,
 *       Debye; two-step-back ABC; Gaussian/sinusoidal hard/soft sources;
 *       running-DFT probes), and
 *   (b) the 2D TM Dz/Ez/Hx/Hy update of fd2d with its 1D-profile PML
 *       (gx2/gx3/gy2/gy3, fx1..fx3, fy1..fy3, ihx/ihy accumulators), lossy
 *       medium (naz/nbz/iz), point sources, TF/SF plane wave and running DFT.
 *
 * Conventions (every entry point):
 *   - returns int: FDTD_OK (0) or a negative FDTD_ERR_* code; nothing throws;
 *   - argument checks happen on the host BEFORE any launch; a failed check
 *     launches nothing and leaves every buffer untouched;
 *   - buffers are caller-owned DEVICE pointers (e.g. torch.Tensor.data_ptr()),
 *     float32, contiguous; 2D arrays are row-major [nx][ny] with j fastest
 *     (n = i*ny + j, as in fd2d/clang/fd2d_3_2.c:33);
 *   - work is enqueued on the given stream (a cudaStream_t; 0 = legacy
 *     default stream) with no host synchronisation, so calls can be captured
 *     into a CUDA graph;
 *   - per-step source values are read from a caller-provided device table
 *     (table[t-1] is the value at step t) computed on the host in float64, so
 *     graph replays need no argument changes;
 *   - calls on one simulation state must be serialised by the caller; any
 *     host thread may call.
 *
 * The reference has no library API: its "interface" is the per-program step
 * functions (dfield/efield/hfield, exfield/hyfield/dxfield, fourier) that mutate
 * caller-owned arrays in place.  Each entry point below names the reference
 * function(s) it replaces, by file:line in dsarvan/simulation.
 */
#ifndef FDTD_GB300_H
#define FDTD_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* every declaration below is exported from the shared library even when it is
 * built with -fvisibility=hidden */
#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

typedef void* fdtd_stream_t; /* a cudaStream_t */

/* ------------------------------------------------------------ status codes */
#define FDTD_OK 0
#define FDTD_ERR_NULL (-1)        /* a required pointer is NULL */
#define FDTD_ERR_SIZE (-2)        /* nx/ny/npml/step counts out of range */
#define FDTD_ERR_ALIGN (-3)       /* a pointer is not 16-byte aligned where required */
#define FDTD_ERR_ARG (-4)         /* any other invalid argument */
#define FDTD_ERR_CUDA (-5)        /* a CUDA call failed (see fdtd_last_cuda_error) */
#define FDTD_ERR_NONFINITE (-6)   /* the device status word reports Inf/NaN */
#define FDTD_ERR_TIMEOUT (-7)     /* a bounded device wait ran out */
#define FDTD_ERR_UNSUPPORTED (-8) /* combination not implemented */
#define FDTD_ERR_WORKSPACE (-9)   /* workspace missing or too small */

/* device status word bits (an int the caller owns; kernels OR bits in) */
#define FDTD_STATUS_NONFINITE 1
#define FDTD_STATUS_TIMEOUT 2
#define FDTD_STATUS_BOUNDS 4

/* source kinds */
#define FDTD_SRC_NONE 0
#define FDTD_SRC_HARD 1 /* field[k] = value   (fd1d/program/fd1d_1_1.py:43, fd2d/python/fd2d_3_1.py:53) */
#define FDTD_SRC_SOFT 2 /* field[k] += value  (fd1d/program/fd1d_1_3.py:57) */

/* library version, e.g. 100 for 0.1.0 */
int fdtd_version(void);
/* human-readable text of an FDTD_ERR_* code */
const char* fdtd_status_string(int status);
/* last CUDA error code recorded by an entry point (0 if none) */
int fdtd_last_cuda_error(void);
/* decode a device status word read back by the caller into FDTD_OK / FDTD_ERR_* */
int fdtd_status_to_error(int device_status);

/* ================================================================= 2D TM */

/* pmlayer, fd2d/python/fd2d_3_2.py:47-52 (device pointers, float32).
 * All ten NULL selects the update without PML or accumulators
 * (fd2d/python/fd2d_3_1.py:57-72). */
typedef struct {
  const float *fx1, *fx2, *fx3; /* [nx] */
  const float *fy1, *fy2, *fy3; /* [ny] */
  const float *gx2, *gx3;       /* [nx] */
  const float *gy2, *gy3;       /* [ny] */
} fdtd2d_pml;

typedef struct {
  int kind;           /* FDTD_SRC_* applied to dz[i][j] right after the D update */
  int i, j;
  const float* table; /* device, table[t-1] = value at step t */
  int table_len;
} fdtd2d_source;

typedef struct {
  int nx, ny;
  fdtd2d_pml pml;
  const float* naz; /* [nx][ny] 1/(eps_r + sigma*dt/eps0), fd2d/python/fd2d_3_4.py:192 */
  const float* nbz; /* [nx][ny] sigma*dt/eps0, or NULL for the lossless E update */
  fdtd2d_source src;
  /* TF/SF plane-wave source of fd2d/python/fd2d_3_4.py:103-170 (0 = off):
   * incident line ezi/hxi along j, boundary at npml-1 .. n-npml. */
  int tfsf_npml;
  const float* tfsf_table; /* device, ezi[3] = tfsf_table[t-1] (gaussian(t,20,8) in the reference) */
  int tfsf_table_len;
  /* running DFT of Ez at every cell, fd2d/python/fd2d_3_4.py:90-99 (nf = 0: off) */
  int nf;
  const float* dft_cos; /* device [table_len][nf]: cos(2*pi*f*dt*t) at row t-1 */
  const float* dft_sin; /* device [table_len][nf] */
  int dft_table_len;
  /* Ez recorded at one cell every step (state.probe_ez, NULL = off):
   * probe_ez[t-1] = ez[probe_i][probe_j] after step t; probe_len entries */
  int probe_i, probe_j;
  int probe_len;
  /* thickness of the absorbing layer in cells (npml of the reference's
   * programs, e.g. fd2d/python/fd2d_3_2.py:133), or 0 if not given.  A hint
   * for laying out the fused kernel's work only: which cells run the cheaper
   * interior update is decided on the device from the PML vectors
   * themselves, so results never depend on it. */
  int pml_cells;
} fdtd2d_params;

typedef struct {
  float *dz, *ez, *iz, *hx, *hy, *ihx, *ihy; /* [nx][ny]; iz NULL if lossless; ihx/ihy NULL without PML */
  float *ezi, *hxi, *bc;                     /* TF/SF incident line [ny] and its ABC state [4] */
  float *r_pt, *i_pt;                        /* DFT [nf][nx][ny] */
  float *r_in, *i_in;                        /* DFT of ezi[6], [nf] */
  int* status;                               /* device status word, may be NULL */
  float* probe_ez;                           /* device [probe_len] Ez trace at the probe cell, or NULL */
} fdtd2d_state;

/* dfield: D update + point source (+ ezi[3] for TF/SF) for step t.
 * Replaces dfield of fd2d/python/fd2d_3_2.py:62-69, fd2d/python/fd2d_3_4.py:113-119,
 * fd2d/cuda/fd2d_3_2.cu:34-49. */
int fdtd2d_dfield(int t, const fdtd2d_params* p, fdtd2d_state* s, fdtd_stream_t stream);
/* efield: Ez (and iz) from Dz. Replaces efield of fd2d/python/fd2d_3_2.py:72-77 and
 * fd2d/python/fd2d_3_4.py:131-136, fd2d/cuda/fd2d_3_4.cu:99-109. */
int fdtd2d_efield(const fdtd2d_params* p, fdtd2d_state* s, fdtd_stream_t stream);
/* hfield: Hx/Hy (+ ihx/ihy). Replaces hfield of fd2d/python/fd2d_3_2.py:80-88,
 * fd2d/python/fd2d_3_1.py:66-72, fd2d/cuda/fd2d_3_2.cu:63-76. */
int fdtd2d_hfield(const fdtd2d_params* p, fdtd2d_state* s, fdtd_stream_t stream);
/* TF/SF and DFT pieces at the reference's granularity
 * (fd2d/python/fd2d_3_4.py:103-110, :123-127, :140-143, :158-170, :90-99). */
int fdtd2d_ezinct(const fdtd2d_params* p, fdtd2d_state* s, fdtd_stream_t stream);
int fdtd2d_inctdz(const fdtd2d_params* p, fdtd2d_state* s, fdtd_stream_t stream);
int fdtd2d_hxinct(const fdtd2d_params* p, fdtd2d_state* s, fdtd_stream_t stream);
int fdtd2d_incth(const fdtd2d_params* p, fdtd2d_state* s, fdtd_stream_t stream);
int fdtd2d_fourier(int t, const fdtd2d_params* p, fdtd2d_state* s, fdtd_stream_t stream);

/* Bytes of device workspace fdtd2d_step_n needs for these params (0 if none):
 * the ping-pong field copies, plus 64 incident-line rows of ny floats with
 * TF/SF on. */
size_t fdtd2d_workspace_size(const fdtd2d_params* p, int steps_per_pass);

/* fdtd2d_step_n: the program's time loop for t = t0+1 .. t0+nsteps, in the
 * reference's step order (fd2d/python/fd2d_3_4.py:268-277).  The core
 * D->source->E->H update is fused into one streaming kernel that keeps
 * `steps_per_pass` (1..4; 0 = library default: 2 below 2^21 cells, else 4) time steps in registers per
 * pass over HBM; `workspace` (fdtd2d_workspace_size bytes, 256-byte aligned)
 * holds the ping-pong copy of the evolving fields.  Results land in the
 * caller's arrays, bitwise equal to calling dfield/efield/hfield per step.
 * TF/SF and the running DFT (nf <= 8) ride in the same fused passes: the
 * incident line is advanced ahead of them in one launch per 64 steps (its
 * tables are part of the workspace), the box-edge corrections and the DFT
 * accumulation happen inside the pass, bitwise equal to the nine per-function
 * calls per step.  Grids with ny % 4 != 0, nf > 8, TF/SF with ny > 16384, a
 * probe trace together with TF/SF or the DFT, or nsteps == 1 run each step as
 * three launches instead (D + ezinct + inctdz; E + fourier + hxinct; H +
 * incthx + incthy; no workspace), with the same results.
 * Replaces the `for t in 1..ns` loops of fd2d/python/fd2d_3_2.py:139-142 and
 * fd2d/cuda/fd2d_3_4.cu:327-336. */
int fdtd2d_step_n(const fdtd2d_params* p, fdtd2d_state* s, int t0, int nsteps, int steps_per_pass,
                  void* workspace, size_t workspace_bytes, fdtd_stream_t stream);

/* Tuning knob of the fused kernel (used by the bench/autotuner): columns per
 * lane (2 or 4; 0 = automatic) and rows per warp segment (0 = automatic, one
 * wave of warps).
 * No reference counterpart. */
int fdtd2d_set_march_config(int cols_per_lane, int warps_per_block, int seg_rows);
/* Tuning knob of the fused kernel's work layout: the time of a general row
 * iteration (PML coefficients, grid edges, source) over an interior one,
 * used to give the stripes and segments that hold the absorbing layer
 * shorter work (1..16; 0 = the measured default for the stripe width).
 * No reference counterpart. */
int fdtd2d_set_march_balance(float gen_cost);

/* fdtd2d_step_n without a caller-provided workspace, for callers that cannot
 * allocate device memory (no cudaMalloc available or allowed where they run).
 * No counterpart in the reference.  The ping-pong workspace is a static device
 * array of FDTD2D_NOALLOC_SCRATCH_BYTES inside this library, held by every GPU
 * that loads it until the process exits; grids needing more (more than
 * FDTD2D_NOALLOC_MAX_CELLS cells) get FDTD_ERR_SIZE.  Allocates nothing itself.
 * The first call on a device looks the array's address up
 * (cudaGetSymbolAddress): with lazy module loading (the CUDA default) that is
 * when the driver reserves the array, so that first call can fail with
 * FDTD_ERR_CUDA if the device is out of memory; make it up front, before any
 * stream capture and before a memory budget is locked.  The address is kept
 * per device and context: the first call in a new context (after a
 * cudaDeviceReset, say) looks it up again, with the same caveat.  All calls
 * share the array (it keeps the
 * last call's contents, none of which must start at zero); calls that overlap
 * on the GPU race on it.  With TF/SF or the DFT on and a workspace larger than
 * the array, each step is one fdtd2d_step_n call of one step instead. */
#define FDTD2D_NOALLOC_MAX_CELLS (1024 * 1024)
#define FDTD2D_NOALLOC_SCRATCH_BYTES (6ull * 4ull * FDTD2D_NOALLOC_MAX_CELLS)
int fdtd2d_step_n_noalloc(const fdtd2d_params* p, fdtd2d_state* s, int t0, int nsteps, int steps_per_pass,
                          fdtd_stream_t stream);

/* ------------------------------------------------ differentiation (adjoint)
 * No counterpart in the reference (it only runs forward).  A reverse sweep
 * over checkpoints: restore a checkpoint, recompute the states of its segment
 * with fdtd2d_pass, then walk the segment backwards with fdtd2d_adjoint_step. */
typedef struct {
  float *dz, *iz, *hx, *hy, *ihx, *ihy; /* [nx][ny] each; iz NULL if lossless */
} fdtd2d_fields;

typedef struct {
  int i0, j0, ni, nj; /* design box: rows i0..i0+ni-1, columns j0..j0+nj-1 */
} fdtd2d_box;

/* One out-of-place fused pass: the fields after steps t0+1..t0+k (k = 1..4)
 * of `in` go to `out`, Ez to `ez` (same kernel and results as fdtd2d_step_n;
 * point source only, ny % 4 == 0, 16-byte aligned buffers). */
int fdtd2d_pass(const fdtd2d_params* p, const fdtd2d_fields* in, fdtd2d_fields* out, float* ez, int t0, int k,
                int* status, fdtd_stream_t stream);

/* Reverse of time step t of the lossy PML update (fd2d/python/fd2d_3_2.py:62-88
 * with fd2d/python/fd2d_3_4.py:131-136) for J = sum_t (probe_weight/2)*ez_t[probe]^2:
 * `fwd` is the state BEFORE step t; `adj` holds the adjoints of the state after
 * step t and receives those before it (in place); `adj_tmp` is [nx][ny]
 * scratch.  Adds dJ/dnaz (and dJ/dnbz if non-NULL) over `box` into grad_naz
 * [ni][nj].  Needs the ten PML vectors (unit profiles for no layer). */
int fdtd2d_adjoint_step(int t, const fdtd2d_params* p, const fdtd2d_fields* fwd, fdtd2d_fields* adj, float* adj_tmp,
                        int probe_i, int probe_j, float probe_weight, fdtd2d_box box, float* grad_naz,
                        float* grad_nbz, fdtd_stream_t stream);

/* The whole gradient in one call.  J = sum over t = 1..nsteps of
 * (probe_weight/2) * ez_t[probe_i][probe_j]^2 for the program `p` run from
 * zero fields (PML required: pass unit profiles for none; point source only;
 * ny % 4 == 0); grad_naz [box.ni][box.nj] receives dJ/dnaz over the box and
 * grad_nbz (optional, lossy only) dJ/dnbz (dJ/deps_r = -naz^2 dJ/dnaz for
 * naz = 1/(eps_r + sigma*dt/eps0)).
 *   forward: fused passes with a stored state every `checkpoint` steps; the
 *            probe's Ez goes to trace [nsteps] (device) and J (device double,
 *            optional) is summed from it;
 *   reverse: segments last first, each recomputed from its checkpoint by
 *            passes that record the state after every step (on a second,
 *            internal stream, one segment ahead), then undone one step per
 *            fused reverse kernel.
 * fdtd2d_tm_adjoint runs both; _forward and _reverse run one each, sharing
 * the workspace (the reverse needs the forward's checkpoints).  The workspace
 * (fdtd2d_tm_adjoint_workspace_size bytes, 256-byte aligned) holds the
 * checkpoints, two segments of recorded states and the ping-pong fields.  The
 * first call on a device creates the internal stream and its events: make it
 * before any stream capture; later calls can be captured.  The gradient does
 * not depend on the checkpoint interval.
 * Replaces the time loop of fd2d/python/fd2d_3_2.py:139-142 (forward) and
 * adds its reverse, which the reference does not have. */
typedef struct {
  int nsteps;
  int checkpoint;
  int probe_i, probe_j;
  float probe_weight;
  fdtd2d_box box;
} fdtd2d_adjoint_params;

size_t fdtd2d_tm_adjoint_workspace_size(const fdtd2d_params* p, const fdtd2d_adjoint_params* a);
int fdtd2d_tm_adjoint_forward(const fdtd2d_params* p, const fdtd2d_adjoint_params* a, float* trace, double* J,
                              void* workspace, size_t workspace_bytes, fdtd_stream_t stream);
int fdtd2d_tm_adjoint_reverse(const fdtd2d_params* p, const fdtd2d_adjoint_params* a, float* grad_naz,
                              float* grad_nbz, void* workspace, size_t workspace_bytes, fdtd_stream_t stream);
int fdtd2d_tm_adjoint(const fdtd2d_params* p, const fdtd2d_adjoint_params* a, float* trace, double* J,
                      float* grad_naz, float* grad_nbz, void* workspace, size_t workspace_bytes,
                      fdtd_stream_t stream);

/* ------------------------------------------------ BF16 tensor-core GEMM
 * D = epilogue(alpha * A.B) on sm_103a tensor cores (tcgen05, TMA, TMEM),
 * FP32 accumulation; used by the neural-operator surrogate (no reference
 * counterpart).  A is [M][K] (K-major, lda >= K) or stored transposed [K][M]
 * (a_mn_major, lda >= M); B is [N][K] (K-major, D = A.B^T) or [K][N]
 * (b_mn_major, D = A.B).  BF16 operands, 16-byte aligned, leading dimensions
 * multiples of 8.  Epilogue: z = alpha*acc + bias[n] + res16[m][n];
 * pre16 = z (optional); y = act ? gelu(z) : z; y += C (accumulate); C = y as
 * FP32 (C32) or BF16 (C16).  `batch` independent products with element strides. */
typedef struct {
  int M, N, K, batch;
  const void* A;
  long long lda, stride_a;
  int a_mn_major;
  const void* B;
  long long ldb, stride_b;
  int b_mn_major;
  float* C32;
  void* C16;
  long long ldc, stride_c;
  const float* bias;
  const void* res16;
  long long ldr, stride_r;
  float alpha;
  int act; /* 0 none, 1 GELU (tanh form) */
  int accumulate;
  void* pre16;
  int mn_lbo, mn_sbo; /* descriptor byte offsets for MN-major tiles (0 = default) */
  /* optional second product accumulated into the same tile before the
   * epilogue: acc = A.B' + A2.B2' (same M, N; its own K2, layouts, strides) */
  int K2;
  const void* A2;
  long long lda2, stride_a2;
  int a2_mn_major;
  const void* B2;
  long long ldb2, stride_b2;
  int b2_mn_major;
} fdtd_gemm_desc;

int fdtd_gemm_bf16(const fdtd_gemm_desc* d, int* status, fdtd_stream_t stream);

/* ------------------------------------------------ surrogate helper kernels
 * Element-wise/reduction pieces of the 1D Fourier-neural-operator surrogate
 * (no reference counterpart); BF16 tensors are passed as void*.  Shapes:
 * rows = B*N positions, C channels, M retained modes, DFT layout [B][C][2M]
 * (cos rows, then -sin rows), mode-major layout [M][B][2C] ([Re | Im]). */
/* lift from cin <= 8 input channels per position: x0 = in P^T + p */
int fno_lift_fwd(long long rows, int C, int cin, const float* in, const float* P, const float* p, void* x0,
                 fdtd_stream_t stream);
int fno_lift_bwd(long long rows, int C, int cin, const float* in, const void* dx0, float* dP, float* dp,
                 fdtd_stream_t stream);
/* Propagation frame of a slab profile: feat [n][nbins][6] = (eps_r-1)/eps_scale of
 * cells 2b-1, 2b, 2b+1 then sigma/sig_scale of the same cells (vacuum = 0);
 * P [n][2*nf] = [Re | Im] of exp(-i sum k(f, cell)) over the cells from probe_in
 * to probe_gap cells behind the last non-vacuum cell, k the complex wavenumber of
 * the lossy 1D Yee update (fd1d/program/fd1d_1_5.py:37-44, :65, :72) at w*dt =
 * wdt[f] (double, device); loss_scale = dt/(2 eps0). */
int fno_propagation(int n, int nbins, const float* feat, int nf, const double* wdt, double eps_scale,
                    double sig_scale, double loss_scale, int probe_in, int probe_gap, float* P,
                    fdtd_stream_t stream);
/* Network inputs from slab layer tables (device arrays, the batched runs'
 * layout): out [n][nbins][6] float32, (eps_r-1)/eps_scale of cells 2b-1, 2b,
 * 2b+1 of run run_idx[q] (run q when run_idx is NULL), then sigma/sig_scale of
 * the same cells; cells outside every layer are vacuum (0). */
int fno_profile_features(int n, const int* run_idx, const int* layer_off, const int* layer_start,
                         const int* layer_end, const double* epsr, const double* sigma, int nbins, double eps_scale,
                         double sig_scale, float* out, fdtd_stream_t stream);
/* out = P (.) y, or conj(P) (.) y when conj_p, for n spectra stored [Re(nf) | Im(nf)] */
int fno_cmul(long long n, int nf, const float* P, const float* y, int conj_p, float* out, fdtd_stream_t stream);
int fno_dft_to_modes(int B, int C, int M, const float* F, void* Fm, fdtd_stream_t stream);
int fno_modes_to_dft(int B, int C, int M, const float* Gm, void* G, fdtd_stream_t stream);
int fno_build_rbig(int M, int C, const float* Rr, const float* Ri, void* Rbig, fdtd_stream_t stream);
int fno_fold_drbig(int M, int C, const float* dRbig, float* dRr, float* dRi, fdtd_stream_t stream);
/* Inference with the lift folded into the first spectral layer (the lift is
 * linear): inputs [B][N][cin] packed as BF16 rows (features, 1, zeros) into
 * out [B][N][ldo] (ldo >= 16, multiple of 8; columns 16.. are zeroed only if
 * write_pad) and, if out_t is not NULL, into out_t [N][B][16]; FP32
 * C[b] = A[b].B for the folded weights; rectangular complex-weight expansion
 * Rbig [M][2Co][2Ci] from Rr, Ri [M][Co][Ci]. */
int fno_pack_inputs(int B, int N, int cin, int ldo, int write_pad, const float* in, void* out, void* out_t,
                    fdtd_stream_t stream);
int fno_small_matmul(int batch, int M, int N, int K, const float* A, const float* B, float* C, fdtd_stream_t stream);
int fno_build_rbig_rect(int M, int Co, int Ci, const float* Rr, const float* Ri, void* Rbig, fdtd_stream_t stream);
int fno_gelu_fwd(long long n, const float* z, void* y, void* pre, fdtd_stream_t stream);
int fno_gelu_bwd(long long n, const void* dy16, const float* dy32, const void* pre, void* dz, fdtd_stream_t stream);
int fno_meanpool(int B, int N, int C, const void* x, void* h, fdtd_stream_t stream);
int fno_meanpool_bwd(int B, int N, int C, const float* dh, void* dx, fdtd_stream_t stream);
int fno_colsum(long long rows, int C, const void* x16, const float* x32, float* out, fdtd_stream_t stream);
int fno_sum_parts(int nb, long long n, const float* parts, float* out, fdtd_stream_t stream);
int fno_mse(int B, int D, const float* o, const float* y, float* dO, float* loss, fdtd_stream_t stream);
/* relative squared error per sample, ||o-y||^2 / max(||y||^2, floor2), averaged over the batch */
int fno_rel_mse(int B, int D, float floor2, const float* o, const float* y, float* dO, float* loss,
                fdtd_stream_t stream);
int fno_adam(long long n, float* w, const float* g, float* m, float* v, float lr, float b1, float b2, float eps,
             int step, void* w16, fdtd_stream_t stream);
int fno_to_bf16(long long n, const float* x, void* y, fdtd_stream_t stream);

/* Lossy-cylinder material map on the device, float64 arithmetic in the order of
 * dielectric() in fd2d/python/fd2d_3_4.py:174-194 (true division m/3):
 * writes naz, nbz [nx][ny]. */
int fdtd2d_dielectric_cylinder(int nx, int ny, int npml, double rgrid, double dt, double epsr,
                               double sigma, float* naz, float* nbz, fdtd_stream_t stream);

/* Amplitude and phase of running-DFT accumulators against the input probe,
 * in double: amp = 1/hypot(r_in, i_in) * hypot(r_pt, i_pt) and phase =
 * atan2(i_pt, r_pt) - atan2(i_in, r_in), for f < nf and k < n, where the
 * accumulators of frequency f are r_pt[f*ld + k] (so a 2D row is r_pt +
 * row*ny with ld = nx*ny) and the input's are r_in[f]; amp/phase [nf][n]
 * (either may be NULL).  Replaces the post-processing of
 * fd1d/program/fd1d_2_2.py:145-146 and fd2d/python/fd2d_3_4.py:280-284. */
int fdtd_dft_amplitude_phase(int nf, long long n, const float* r_pt, const float* i_pt, long long ld,
                             const float* r_in, const float* i_in, double* amp, double* phase,
                             fdtd_stream_t stream);

/* Sets *status_out |= FDTD_STATUS_NONFINITE if any of the n floats is Inf/NaN. */
int fdtd_check_finite(const float* x, size_t n, int* status, fdtd_stream_t stream);

/* ================================================================= 1D */

#define FDTD1D_FORM_CB 0    /* ex += cb*(hy[i-1]-hy[i])            fd1d/program/fd1d_1_3.py:55 */
#define FDTD1D_FORM_CACB 1  /* ex = ca*ex + cb*(hy[i-1]-hy[i])     fd1d/program/fd1d_1_5.py:65 */
#define FDTD1D_FORM_DFORM 2 /* dx/ix with nax/nbx                   fd1d/program/fd1d_2_2.py:74-84 */
#define FDTD1D_FORM_DEBYE 3 /* D-form + Debye sx with ncx/ndx       fd1d/program/fd1d_2_3.py:82-86 */

#define FDTD1D_MAX_PROBES 8
#define FDTD1D_MAX_FUSED_NX 65536

typedef struct {
  int nx;
  int form;                                      /* FDTD1D_FORM_* */
  const float *ca, *cb;                          /* [nx]: CB uses cb; CACB uses ca, cb */
  const float *nax, *nbx, *ncx, *ndx;            /* [nx]: DFORM uses nax, nbx; DEBYE all four */
  int src_kind;                                  /* FDTD_SRC_*; into ex (CB/CACB) or dx (D forms) */
  int src_k;
  const float* src_table;                        /* device, table[t-1] */
  int src_table_len;
  int abc;                                       /* 1: two-step-back ABC, fd1d/program/fd1d_1_2.py:47-48 */
  int nf;                                        /* running DFT frequencies (0 = off) */
  const float* dft_cos;                          /* device [table_len][nf] */
  const float* dft_sin;
  int dft_table_len;
  int nprobe;                                    /* probe cells (<= FDTD1D_MAX_PROBES) */
  int probe_k[FDTD1D_MAX_PROBES];
  int full_dft;                                  /* 1: accumulate every cell into r_pt/i_pt */
} fdtd1d_params;

typedef struct {
  float *ex, *hy;      /* [nx] */
  float *dx, *ix, *sx; /* [nx] D forms (sx: Debye) */
  float* bc;           /* [4] ABC state */
  float *r_pt, *i_pt;  /* [nf][nx] when full_dft */
  float *r_pr, *i_pr;  /* [nprobe][nf] probe DFT accumulators */
  int* status;
} fdtd1d_state;

/* exfield (+ source), fd1d/clang/fd1d_1_3.c:17-23 and fd1d/program/fd1d_1_5.py:65-67;
 * for the D forms: dxfield + exfield, fd1d/program/fd1d_2_2.py:74-84. */
int fdtd1d_efield(int t, const fdtd1d_params* p, fdtd1d_state* s, fdtd_stream_t stream);
/* hyfield: ABC then Hy, fd1d/program/fd1d_2_2.py:87-92, fd1d/clang/fd1d_1_3.c:26-33. */
int fdtd1d_hfield(const fdtd1d_params* p, fdtd1d_state* s, fdtd_stream_t stream);
/* fourier, fd1d/program/fd1d_2_2.py:65-71 (probes and optionally every cell). */
int fdtd1d_fourier(int t, const fdtd1d_params* p, fdtd1d_state* s, fdtd_stream_t stream);
/* fdtd1d_step_n: the program's time loop, t = t0+1 .. t0+nsteps, in one launch
 * (a line of up to 512 cells is held by one warp, warp shuffles carrying the
 * halos; a longer one by a thread block or cluster, with shared and distributed
 * shared memory between warps and blocks).  nx <= FDTD1D_MAX_FUSED_NX
 * (8 blocks x 512 threads x 16 cells); longer lines use the per-function
 * entry points above.
 * Replaces fd1d/program/fd1d_1_3.py:53-62, fd1d/program/fd1d_2_2.py:138-142,
 * fd1d/cuda/fd1d_1_3.cu:78-85. */
int fdtd1d_step_n(const fdtd1d_params* p, fdtd1d_state* s, int t0, int nsteps, fdtd_stream_t stream);

/* ================================================================= batched 1D
 * Thousands of independent lossy 1D runs (ca/cb update of
 * fd1d/program/fd1d_1_5.py:63-72 with a soft source and the two-step-back ABC)
 * of uneven length, each with a piecewise-constant layer table, in one
 * persistent launch; the running DFT of fd1d/program/fd1d_2_2.py:65-71 is
 * accumulated at an entry and an exit probe.  No reference counterpart: the
 * reference runs one program at a time. */
typedef struct {
  int nruns;
  const int* ke;          /* device [nruns]: cells of each run (>= 4) */
  const int* layer_off;   /* device [nruns+1]: run r's layers are layer_off[r] .. layer_off[r+1]-1 */
  int nlayers;
  const int* layer_start; /* device [nlayers]: first cell of the layer */
  const int* layer_end;   /* device [nlayers]: one past its last cell */
  const float* layer_ca;  /* device [nlayers]: ca, cb of the layer (cells outside layers: ca=1, cb=0.5) */
  const float* layer_cb;
  const int* probe_in;    /* device [nruns]: entry probe cell */
  const int* probe_out;   /* device [nruns]: exit probe cell */
  int src_k;              /* soft source cell (all runs), >= 1 */
  const float* src_table; /* device [nsteps] */
  int nsteps;
  int nf;                 /* 1..64 */
  const float* dft_cos;   /* device [nsteps][nf] */
  const float* dft_sin;
} fdtd1d_batch_params;

typedef struct {
  float* spec;      /* device [nruns][4][nf]: re/im at the entry probe, re/im at the exit probe */
  int* done;        /* device [nruns] or NULL: set to 1 when a run of the plan completes;
                       not cleared by the call (zero it once before the groups' calls) */
  int* status;      /* device status word or NULL */
  unsigned* queue;  /* device work counter (one unsigned), reset by the call */
} fdtd1d_batch_out;

/* Host-side planner (no device work): team size per run = ceil(ke/cells_per_thread)
 * threads rounded to whole warps, teams packed first-fit-decreasing into blocks
 * of block_threads.  Writes the plan (int32) to `plan` (NULL: only *plan_len). */
int fdtd1d_batch_plan(const int* ke_host, int nruns, int cells_per_thread, int block_threads, int* plan,
                      size_t plan_ints, int* plan_len);
/* Runs the planned batch: plan_device is the plan copied to the device;
 * cells_per_thread and block_threads must match the plan: cells_per_thread 8 or
 * 16 with blocks of up to 1024 threads, 24, 32 or 40 with up to 512;
 * ctas_per_sm 0 = as many as fit; max_cycles > 0 bounds each block's time for
 * taking new work (FDTD_STATUS_TIMEOUT if work was left). */
int fdtd1d_batch_run(const fdtd1d_batch_params* p, fdtd1d_batch_out* o, const int* plan_device, int plan_len,
                     int nbundles, int cells_per_thread, int block_threads, int ctas_per_sm, long long max_cycles,
                     fdtd_stream_t stream);

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif

#ifdef __cplusplus
}
#endif

#endif /* FDTD_GB300_H */
