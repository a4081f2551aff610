/* fdtd_oracle.c -- plain-C restatement of the reference FDTD step loops.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle / CPU baseline), never the product.
 *
 * Compiled twice by oracle/Makefile:
 *   REAL=double, -ffp-contract=off : the float64 oracle for grids too large for
 *       NumPy; the same operation order as the reference's loops
 *       (fd2d/clang/fd2d_3_4.c:68-127, fd1d/clang/fd1d_1_3.c:17-33) and as
 *       oracle/fd2d.py, so its results equal the NumPy oracle bit for bit;
 *   REAL=float, -O3 -fopenmp     : the CPU baseline timed beside the GPU, the
 *       shape of the reference's float32 benchmark twins
 *       (fd2d/clang/test_3_4.c, fd1d/clang/test_1_3.c).
 *
 * Differences from the reference C, all deliberate:
 *   - the per-step source value comes from a float64 table (t-1 indexed), so
 *     any waveform/position can be replayed (the reference hard-codes them);
 *   - the material map is an input (the reference C's dielectric() divides
 *     integers, fd2d/clang/fd2d_3_4.c:162-163; the Python formula is used);
 *   - OpenMP parallel-for over rows in 2D, like fd2d/clang/fd2d_3_2.c:30-57.
 */
#include <math.h>
#include <stddef.h>
#include <stdlib.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef REAL
#define REAL double
#endif

#define EXPORT __attribute__((visibility("default")))

EXPORT int oracle_real_size(void) { return (int)sizeof(REAL); }

EXPORT int oracle_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

EXPORT void oracle_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

/* ------------------------------------------------------------------- 2D TM
 * pml: 10 vectors fx1,fx2,fx3,fy1,fy2,fy3,gx2,gx3,gy2,gy3 (NULL = no PML: the
 * fd2d_3_1 update).  nbz/iz NULL = lossless E update.  src_kind 0/1/2 =
 * none/hard/soft at dz[si][sj] after the D update. */
EXPORT void oracle_fd2d_steps(int nx, int ny, int t0, int ns, const REAL* const* pml, const REAL* naz,
                              const REAL* nbz, int src_kind, int si, int sj, const double* src_table, REAL* dz,
                              REAL* ez, REAL* iz, REAL* hx, REAL* hy, REAL* ihx, REAL* ihy) {
  const REAL *fx1 = 0, *fx2 = 0, *fx3 = 0, *fy1 = 0, *fy2 = 0, *fy3 = 0, *gx2 = 0, *gx3 = 0, *gy2 = 0, *gy3 = 0;
  if (pml) {
    fx1 = pml[0]; fx2 = pml[1]; fx3 = pml[2]; fy1 = pml[3]; fy2 = pml[4];
    fy3 = pml[5]; gx2 = pml[6]; gx3 = pml[7]; gy2 = pml[8]; gy3 = pml[9];
  }
  for (int t = t0 + 1; t <= t0 + ns; t++) {
    /* dfield, fd2d/python/fd2d_3_2.py:64-67 */
#pragma omp parallel for schedule(static)
    for (int i = 1; i < nx; i++) {
      for (int j = 1; j < ny; j++) {
        const size_t n = (size_t)i * ny + j;
        const REAL curl = hy[n] - hy[n - ny] - hx[n] + hx[n - 1];
        if (pml)
          dz[n] = gx3[i] * gy3[j] * dz[n] + gx2[i] * gy2[j] * (REAL)0.5 * curl;
        else
          dz[n] += (REAL)0.5 * curl;
      }
    }
    if (src_kind == 1) dz[(size_t)si * ny + sj] = (REAL)src_table[t - 1];
    else if (src_kind == 2) dz[(size_t)si * ny + sj] += (REAL)src_table[t - 1];
    /* efield, fd2d/python/fd2d_3_4.py:131-136 */
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nx; i++) {
      for (int j = 0; j < ny; j++) {
        const size_t n = (size_t)i * ny + j;
        if (nbz) {
          ez[n] = naz[n] * (dz[n] - iz[n]);
          iz[n] += nbz[n] * ez[n];
        } else {
          ez[n] = naz[n] * dz[n];
        }
      }
    }
    /* hfield, fd2d/python/fd2d_3_2.py:80-88 */
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nx - 1; i++) {
      for (int j = 0; j < ny - 1; j++) {
        const size_t n = (size_t)i * ny + j;
        if (pml) {
          const REAL cx = ez[n] - ez[n + 1];
          const REAL cy = ez[n] - ez[n + ny];
          ihx[n] += cx;
          ihy[n] += cy;
          hx[n] = fy3[j] * hx[n] + fy2[j] * ((REAL)0.5 * cx + fx1[i] * ihx[n]);
          hy[n] = fx3[i] * hy[n] - fx2[i] * ((REAL)0.5 * cy + fy1[j] * ihy[n]);
        } else {
          hx[n] += (REAL)0.5 * (ez[n] - ez[n + 1]);
          hy[n] -= (REAL)0.5 * (ez[n] - ez[n + ny]);
        }
      }
    }
  }
}

/* ------------------------------------------------------------------- 1D
 * form 0 cb / 1 ca-cb (fd1d/clang/fd1d_1_5.c:25-31) / 2 D-form (nax,nbx) /
 * 3 Debye (nax..ndx).  Source into ex (forms 0,1) or dx (forms 2,3).  Probe
 * DFT (ex at probe cells, cos/sin tables [t-1][nf]) after E, before the ABC.
 * Single-threaded like the reference's 1D C programs. */
EXPORT void oracle_fd1d_steps(int nx, int form, int t0, int ns, const REAL* ca, const REAL* cb, const REAL* nax,
                              const REAL* nbx, const REAL* ncx, const REAL* ndx, int src_kind, int src_k,
                              const double* src_table, int abc, REAL* ex, REAL* hy, REAL* dx, REAL* ix, REAL* sx,
                              REAL* bc, int nf, const double* dcos, const double* dsin, int nprobe,
                              const int* probe_k, REAL* r_pr, REAL* i_pr) {
  for (int t = t0 + 1; t <= t0 + ns; t++) {
    const REAL v = src_kind ? (REAL)src_table[t - 1] : (REAL)0;
    if (form == 0) {
      for (int i = 1; i < nx; i++) ex[i] += cb[i] * (hy[i - 1] - hy[i]);
    } else if (form == 1) {
      for (int i = 1; i < nx; i++) ex[i] = ca[i] * ex[i] + cb[i] * (hy[i - 1] - hy[i]);
    } else {
      for (int i = 1; i < nx; i++) dx[i] += (REAL)0.5 * (hy[i - 1] - hy[i]);
    }
    REAL* sf = (form <= 1) ? ex : dx;
    if (src_kind == 1) sf[src_k] = v;
    else if (src_kind == 2) sf[src_k] += v;
    if (form == 2) {
      for (int i = 1; i < nx; i++) {
        ex[i] = nax[i] * (dx[i] - ix[i]);
        ix[i] += nbx[i] * ex[i];
      }
    } else if (form == 3) {
      for (int i = 1; i < nx; i++) {
        ex[i] = nax[i] * (dx[i] - ix[i] - ncx[i] * sx[i]);
        ix[i] += nbx[i] * ex[i];
        sx[i] = ncx[i] * sx[i] + ndx[i] * ex[i];
      }
    }
    for (int q = 0; q < nprobe; q++)
      for (int f = 0; f < nf; f++) {
        r_pr[q * nf + f] += (REAL)dcos[(size_t)(t - 1) * nf + f] * ex[probe_k[q]];
        i_pr[q * nf + f] -= (REAL)dsin[(size_t)(t - 1) * nf + f] * ex[probe_k[q]];
      }
    if (abc) {
      ex[0] = bc[0];
      bc[0] = bc[1];
      bc[1] = ex[1];
      ex[nx - 1] = bc[3];
      bc[3] = bc[2];
      bc[2] = ex[nx - 2];
    }
    for (int i = 0; i < nx - 1; i++) hy[i] += (REAL)0.5 * (ex[i] - ex[i + 1]);
  }
}

/* Many independent 1D ca/cb runs (the batched-slab workload), one run per
 * OpenMP thread at a time; each run's coefficients come from its layer table
 * exactly as the GPU batch path builds them.  Used as the CPU baseline and as
 * the oracle for sampled runs. */
EXPORT void oracle_fd1d_batch(int nruns, const int* ke, const int* layer_off, const int* layer_start,
                              const int* layer_end, const double* layer_ca, const double* layer_cb, int src_k,
                              const double* src_table, int ns, int nf, const double* dcos, const double* dsin,
                              const int* probe_in, const int* probe_out, REAL* spec /* [nruns][4][nf] */) {
#pragma omp parallel for schedule(dynamic, 1)
  for (int r = 0; r < nruns; r++) {
    const int nx = ke[r];
    REAL* buf = (REAL*)calloc((size_t)4 * nx, sizeof(REAL));
    REAL *ex = buf, *hy = buf + nx, *ca = buf + 2 * (size_t)nx, *cb = buf + 3 * (size_t)nx;
    for (int i = 0; i < nx; i++) {
      ca[i] = (REAL)1.0;
      cb[i] = (REAL)0.5;
    }
    for (int l = layer_off[r]; l < layer_off[r + 1]; l++)
      for (int i = layer_start[l]; i < layer_end[l] && i < nx; i++) {
        ca[i] = (REAL)layer_ca[l];
        cb[i] = (REAL)layer_cb[l];
      }
    REAL bc[4] = {0, 0, 0, 0};
    REAL* sp = spec + (size_t)r * 4 * nf;
    for (int k = 0; k < 4 * nf; k++) sp[k] = 0;
    const int pin = probe_in[r], pout = probe_out[r];
    for (int t = 1; t <= ns; t++) {
      for (int i = 1; i < nx; i++) ex[i] = ca[i] * ex[i] + cb[i] * (hy[i - 1] - hy[i]);
      ex[src_k] += (REAL)src_table[t - 1];
      for (int f = 0; f < nf; f++) {
        const REAL c = (REAL)dcos[(size_t)(t - 1) * nf + f], s = (REAL)dsin[(size_t)(t - 1) * nf + f];
        sp[0 * nf + f] += c * ex[pin];
        sp[1 * nf + f] -= s * ex[pin];
        sp[2 * nf + f] += c * ex[pout];
        sp[3 * nf + f] -= s * ex[pout];
      }
      ex[0] = bc[0];
      bc[0] = bc[1];
      bc[1] = ex[1];
      ex[nx - 1] = bc[3];
      bc[3] = bc[2];
      bc[2] = ex[nx - 2];
      for (int i = 0; i < nx - 1; i++) hy[i] += (REAL)0.5 * (ex[i] - ex[i + 1]);
    }
    free(buf);
  }
}
