"""2D TM FDTD on the GPU: host mirror of the reference's fd2d programs.

Names and argument meanings follow dsarvan/simulation ``fd2d/python``:
``pmlayer``/``pmlparam`` (fd2d/python/fd2d_3_2.py:47-52, :91-100),
``dielectric`` (fd2d/python/fd2d_3_4.py:174-194), the step functions
``dfield``/``efield``/``hfield`` (:113-154) and the TF/SF pieces.  The field
arrays are float32 CUDA tensors, row-major ``[nx][ny]``; every update runs in
``libfdtd_gb300.so`` (C-ABI ``include/fdtd.h``).

``SimTM2D`` keeps one program's parameters and fields and runs its time loop
(``step``) with the fused streaming kernel, optionally as a captured CUDA
graph (``run_graph``).
"""
from __future__ import annotations

from collections import namedtuple

import numpy as np
import torch

from . import _lib
from ._lib import call, ptr
from .sources import dft_tables, to_device, wave_values

EPS0 = 8.854e-12  # fd2d/python/fd2d_3_4.py:180

pmlayer = namedtuple("pmlayer", ("fx1", "fx2", "fx3", "fy1", "fy2", "fy3", "gx2", "gx3", "gy2", "gy3"))


def pml_profiles(nx: int, ny: int, npml: int, grade: float = 0.33) -> dict:
    """The ten PML vectors in float64 (fd2d/python/fd2d_3_2.py:91-100, grade a parameter).

    Same Python scalar arithmetic and order as the reference's ``pmlparam``,
    so the float64 values are identical to it at ``grade=0.33``.
    """
    v = dict(fx1=np.zeros(nx), fx2=np.ones(nx), fx3=np.ones(nx), fy1=np.zeros(ny), fy2=np.ones(ny),
             fy3=np.ones(ny), gx2=np.ones(nx), gx3=np.ones(nx), gy2=np.ones(ny), gy3=np.ones(ny))
    if 2 * npml >= min(nx, ny) and npml > 0:
        raise ValueError(f"npml={npml} too large for a {nx}x{ny} grid")
    for n in range(npml):
        xm = grade * ((npml - n) / npml) ** 3
        xn = grade * ((npml - n - 0.5) / npml) ** 3
        v["fx1"][n] = v["fx1"][nx - 2 - n] = v["fy1"][n] = v["fy1"][ny - 2 - n] = xn
        v["fx2"][n] = v["fx2"][nx - 2 - n] = v["fy2"][n] = v["fy2"][ny - 2 - n] = 1 / (1 + xn)
        v["gx2"][n] = v["gx2"][nx - 1 - n] = v["gy2"][n] = v["gy2"][ny - 1 - n] = 1 / (1 + xm)
        v["fx3"][n] = v["fx3"][nx - 2 - n] = v["fy3"][n] = v["fy3"][ny - 2 - n] = (1 - xn) / (1 + xn)
        v["gx3"][n] = v["gx3"][nx - 1 - n] = v["gy3"][n] = v["gy3"][ny - 1 - n] = (1 - xm) / (1 + xm)
    return v


def pml_cells(pml: pmlayer | None) -> int:
    """Thickness in cells of the absorbing layer a ``pmlayer`` holds (0 for
    none): the longest run of non-unit coefficients at either end of the ten
    vectors.  Read once from the device when a program is set up; the fused
    kernel uses it only to balance its work."""
    if pml is None:
        return 0
    unit = dict(fx1=0.0, fy1=0.0)
    n = 0
    for k in pmlayer._fields:
        v = getattr(pml, k).detach().cpu().numpy()
        bad = np.flatnonzero(v != unit.get(k, 1.0))
        lo, hi = bad[bad < v.size // 2], bad[bad >= v.size // 2]
        if lo.size:
            n = max(n, int(lo.max()) + 1)
        if hi.size:
            n = max(n, int(v.size - hi.min()))
    return n


def pmlparam(nx: int, ny: int, npml: int, grade: float = 0.33, device="cuda") -> pmlayer:
    """``pmlayer`` of float32 device vectors (npml=0: no absorbing layer)."""
    v = pml_profiles(nx, ny, npml, grade)
    return pmlayer(**{k: to_device(a, device) for k, a in v.items()})


def dielectric(nx: int, ny: int, npml: int, rgrid: float, dt: float, epsr: float, sigma: float,
               device="cuda"):
    """(naz, nbz) of the lossy cylinder, computed on the GPU in float64
    (fd2d/python/fd2d_3_4.py:174-194, true division m/3)."""
    naz = torch.empty((nx, ny), dtype=torch.float32, device=device)
    nbz = torch.empty((nx, ny), dtype=torch.float32, device=device)
    call("fdtd2d_dielectric_cylinder", nx, ny, npml, float(rgrid), float(dt), float(epsr), float(sigma),
         ptr(naz), ptr(nbz), _lib.stream_ptr())
    return naz, nbz


class PointSource:
    """Hard (``dz[i,j] = v``) or soft (``+=``) point source with a float64 waveform."""

    def __init__(self, i: int, j: int, wave: tuple, kind: str = "hard"):
        self.i, self.j, self.wave = int(i), int(j), wave
        self.kind = {"hard": _lib.SRC_HARD, "soft": _lib.SRC_SOFT}[kind]


class SimTM2D:
    """One 2D TM program: parameters, fields and its time loop on the GPU.

    ``lossy`` selects the ``naz*(dz-iz)`` E update with ``iz`` (fd2d_3_4);
    otherwise ``ez = naz*dz`` (fd2d_3_2).  ``pml=None`` selects the update
    without PML or accumulators (fd2d_3_1).  ``tfsf_npml`` enables the
    plane-wave source of fd2d_3_3/3_4; ``freq`` the full-field running DFT.
    """

    def __init__(self, nx: int, ny: int, *, pml: pmlayer | None = None, naz=None, nbz=None,
                 source: PointSource | None = None, lossy: bool = True, tfsf_npml: int = 0,
                 freq=None, dt: float = 0.01 / 6e8, ns: int = 1024, device="cuda",
                 check_finite: bool = True, steps_per_pass: int = 0):
        self.nx, self.ny, self.device = nx, ny, torch.device(device)
        self.dt = dt
        self.lossy = lossy
        self.pml = pml
        self.pml_cells = pml_cells(pml)
        self.source = source
        self.tfsf_npml = tfsf_npml
        self.freq = None if freq is None else np.asarray(freq, dtype=np.float64).reshape(-1)
        self.steps_per_pass = steps_per_pass
        z = lambda: torch.zeros((nx, ny), dtype=torch.float32, device=self.device)  # noqa: E731
        self.naz = naz if naz is not None else torch.ones((nx, ny), dtype=torch.float32, device=self.device)
        self.nbz = (nbz if nbz is not None else z()) if lossy else None
        self.dz, self.ez, self.hx, self.hy = z(), z(), z(), z()
        self.iz = z() if lossy else None
        self.ihx = z() if pml is not None else None
        self.ihy = z() if pml is not None else None
        self.ezi = self.hxi = self.bc = None
        if tfsf_npml:
            self.ezi = torch.zeros(ny, dtype=torch.float32, device=self.device)
            self.hxi = torch.zeros(ny, dtype=torch.float32, device=self.device)
            self.bc = torch.zeros(4, dtype=torch.float32, device=self.device)
        self.r_pt = self.i_pt = self.r_in = self.i_in = None
        if self.freq is not None:
            nf = self.freq.size
            self.r_pt = torch.zeros((nf, nx, ny), dtype=torch.float32, device=self.device)
            self.i_pt = torch.zeros_like(self.r_pt)
            self.r_in = torch.zeros(nf, dtype=torch.float32, device=self.device)
            self.i_in = torch.zeros_like(self.r_in)
        self.status = torch.zeros(1, dtype=torch.int32, device=self.device) if check_finite else None
        self.t = 0
        self._ns = 0
        self._tables(ns)
        self._workspace = None
        self._graphs = {}

    # ------------------------------------------------------------ setup
    def _tables(self, ns: int) -> None:
        """(Re)build the per-step tables for t = 1 .. ns."""
        self._ns = ns
        self.src_table = None
        if self.source is not None:
            self.src_table = to_device(wave_values(self.source.wave, 1, ns), self.device)
        self.tfsf_table = None
        if self.tfsf_npml:
            # fd2d/python/fd2d_3_4.py:119: ezi[3] = gaussian(t, 20, 8.0)
            self.tfsf_table = to_device(wave_values(("gauss", 20, 8.0), 1, ns), self.device)
        self.dft_cos = self.dft_sin = None
        if self.freq is not None:
            cs, sn = dft_tables(self.freq, self.dt, 1, ns)
            self.dft_cos, self.dft_sin = to_device(cs, self.device), to_device(sn, self.device)
        self._build_structs()

    def _build_structs(self) -> None:
        p = _lib.Params2D()
        p.nx, p.ny = self.nx, self.ny
        if self.pml is not None:
            for k in pmlayer._fields:
                setattr(p.pml, k, ptr(getattr(self.pml, k)))
            p.pml_cells = self.pml_cells
        p.naz = ptr(self.naz)
        p.nbz = ptr(self.nbz)
        if self.source is not None:
            p.src.kind, p.src.i, p.src.j = self.source.kind, self.source.i, self.source.j
            p.src.table, p.src.table_len = ptr(self.src_table), self._ns
        p.tfsf_npml = self.tfsf_npml
        if self.tfsf_npml:
            p.tfsf_table, p.tfsf_table_len = ptr(self.tfsf_table), self._ns
        if self.freq is not None:
            p.nf = self.freq.size
            p.dft_cos, p.dft_sin, p.dft_table_len = ptr(self.dft_cos), ptr(self.dft_sin), self._ns
        s = _lib.State2D()
        for k in ("dz", "ez", "iz", "hx", "hy", "ihx", "ihy", "ezi", "hxi", "bc", "r_pt", "i_pt", "r_in", "i_in"):
            setattr(s, k, ptr(getattr(self, k)))
        s.status = ptr(self.status)
        self._p, self._s = p, s
        self._graphs = {}

    def _ensure(self, t_last: int) -> None:
        if t_last > self._ns:
            self._tables(max(t_last, 2 * self._ns))

    def workspace(self):
        n = _lib.lib().fdtd2d_workspace_size(self._p, self.steps_per_pass)
        if n and (self._workspace is None or self._workspace.numel() < n):
            self._workspace = torch.empty(n, dtype=torch.uint8, device=self.device)
            self._graphs = {}
        return self._workspace

    # ------------------------------------------------------------ time loop
    def step(self, n: int = 1, steps_per_pass: int | None = None) -> None:
        """Advance ``n`` time steps (t = self.t+1 .. self.t+n) on the current stream."""
        if n <= 0:
            return
        self._ensure(self.t + n)
        ws = self.workspace()
        spp = self.steps_per_pass if steps_per_pass is None else steps_per_pass
        call("fdtd2d_step_n", self._p, self._s, self.t, n, spp, ptr(ws), 0 if ws is None else ws.numel(),
             _lib.stream_ptr())
        self.t += n

    def run_graph(self, n: int, steps_per_pass: int | None = None) -> None:
        """Advance ``n`` steps by replaying a captured CUDA graph of the loop.

        The graph is recorded once per (start step, n) and replayed after; the
        tables and workspace are allocated before capture.
        """
        if n <= 0:
            return
        self._ensure(self.t + n)
        ws = self.workspace()
        spp = self.steps_per_pass if steps_per_pass is None else steps_per_pass
        key = (self.t, n, spp)
        g = self._graphs.get(key)
        if g is None:
            g = torch.cuda.CUDAGraph()
            s = torch.cuda.Stream(device=self.device)
            s.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(s):
                # warm-up launch outside capture is not needed: the C-ABI does
                # no allocation or host sync
                with torch.cuda.graph(g, stream=s):
                    call("fdtd2d_step_n", self._p, self._s, self.t, n, spp, ptr(ws),
                         0 if ws is None else ws.numel(), _lib.stream_ptr(s))
            torch.cuda.current_stream().wait_stream(s)
            self._graphs[key] = g
        g.replay()
        self.t += n

    # reference-granularity drop-ins (one launch per reference function)
    def dfield(self, t: int) -> None:
        self._ensure(t)
        call("fdtd2d_dfield", t, self._p, self._s, _lib.stream_ptr())

    def efield(self) -> None:
        call("fdtd2d_efield", self._p, self._s, _lib.stream_ptr())

    def hfield(self) -> None:
        call("fdtd2d_hfield", self._p, self._s, _lib.stream_ptr())

    def step_per_function(self, n: int = 1) -> None:
        """The reference's loop body, one launch per reference function."""
        self._ensure(self.t + n)
        st = _lib.stream_ptr()
        for t in range(self.t + 1, self.t + n + 1):
            if self.tfsf_npml:
                call("fdtd2d_ezinct", self._p, self._s, st)
            call("fdtd2d_dfield", t, self._p, self._s, st)
            if self.tfsf_npml:
                call("fdtd2d_inctdz", self._p, self._s, st)
            call("fdtd2d_efield", self._p, self._s, st)
            if self.freq is not None:
                call("fdtd2d_fourier", t, self._p, self._s, st)
            if self.tfsf_npml:
                call("fdtd2d_hxinct", self._p, self._s, st)
            call("fdtd2d_hfield", self._p, self._s, st)
            if self.tfsf_npml:
                call("fdtd2d_incth", self._p, self._s, st)
        self.t += n

    # ------------------------------------------------------------ status, state
    def check(self) -> None:
        """Raise FdtdError if a kernel reported a non-finite field (host sync)."""
        if self.status is None:
            return
        v = int(self.status.item())
        if v:
            rc = _lib.lib().fdtd_status_to_error(v)
            raise _lib.FdtdError(rc, f"SimTM2D status word {v:#x} at t={self.t}")

    def amplitude_phase(self, row: int | None = None, j0: int | None = None, j1: int | None = None):
        """(amp, phase) float64 [nf][j1-j0+1] along one row of the DFT against
        the incident line's input (fd2d/python/fd2d_3_4.py:280-284: row
        nx//2-1, columns npml-1 .. ny-npml with npml the TF/SF boundary)."""
        if self.r_pt is None or self.r_in is None:
            raise ValueError("amplitude_phase needs freq=... and tfsf_npml > 0 (the input is ezi[6])")
        npml = self.tfsf_npml
        row = self.nx // 2 - 1 if row is None else row
        j0 = npml - 1 if j0 is None else j0
        j1 = self.ny - npml if j1 is None else j1
        if not (0 <= row < self.nx and 0 <= j0 <= j1 < self.ny):
            raise ValueError("row/columns outside the grid")
        from .output import amplitude_phase
        return amplitude_phase(self.r_pt, self.i_pt, self.r_in, self.i_in, row * self.ny + j0, j1 - j0 + 1)

    def head(self, name: str = "ez", row: int = 2, n: int = 50) -> str:
        """``print(ez[2][0:50])`` of the reference's benchmark twins
        (fd2d/python/test_3_4.py:292): the first ``n`` values of one row."""
        from .output import head
        return head(getattr(self, name)[row], n)

    def save(self, path: str, names=None) -> str:
        """Write the fields to an .npz archive (or .npy files in a directory)."""
        from .output import save
        return save(self, path, names)

    FIELDS = ("dz", "ez", "iz", "hx", "hy", "ihx", "ihy", "ezi", "hxi", "bc", "r_pt", "i_pt", "r_in", "i_in")

    def state_dict(self) -> dict:
        d = {k: getattr(self, k).clone() for k in self.FIELDS if getattr(self, k) is not None}
        d["t"] = self.t
        return d

    def load_state_dict(self, d: dict) -> None:
        for k in self.FIELDS:
            cur = getattr(self, k)
            if cur is not None:
                cur.copy_(d[k])
        self.t = int(d["t"])
        if self.status is not None:
            self.status.zero_()

    def reset(self) -> None:
        for k in self.FIELDS:
            cur = getattr(self, k)
            if cur is not None:
                cur.zero_()
        self.t = 0
        if self.status is not None:
            self.status.zero_()


def benchmark_sim(nx: int = 8192, ny: int = 8192, npml: int = 32, grade: float = 0.333, rgrid: float = 1000,
                  epsr: float = 30.0, sigma: float = 0.3, ns: int = 2000, device="cuda", **kw) -> SimTM2D:
    """The 2D TM PML benchmark program: lossy cylinder of radius ``rgrid`` cells
    (eps_r=30, sigma=0.3 S/m, centre (nx/2-1, ny/2-1)), ``npml``-cell PML with
    cubic grading ``grade``, hard Gaussian Dz point source at (nx/2, ny/2) with
    t0=20, spread=6 (fd2d/python/fd2d_3_1.py:53), dx=1 cm, dt=dx/(2c)."""
    dt = 0.01 / 6e8
    pml = pmlparam(nx, ny, npml, grade, device)
    naz, nbz = dielectric(nx, ny, npml, rgrid, dt, epsr, sigma, device)
    src = PointSource(nx // 2, ny // 2, ("gauss", 20, 6.0), "hard")
    return SimTM2D(nx, ny, pml=pml, naz=naz, nbz=nbz, source=src, lossy=True, ns=ns, device=device, **kw)
