"""Float64 NumPy restatement of the reference's 2D TM FDTD programs (oracle only).

Follows the vectorised form of fd2d/program/fd2d_3_2.py:61-93 (itself
bit-identical to the Numba loops of fd2d/python/fd2d_3_2.py:62-88) and adds
the lossy ``efield``, the cylinder ``dielectric``, the TF/SF plane-wave
functions and the running DFT of fd2d/python/fd2d_3_4.py.

Arrays are row-major ``[nx][ny]`` (``n = i*ny + j``, j fastest), as in
fd2d/clang/fd2d_3_2.c:33.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np
from numpy import pi, cos, sin

EPS0 = 8.854e-12  # fd2d/python/fd2d_3_4.py:180


@dataclass
class PML:
    """The ten 1D PML profile vectors of ``pmlayer`` (fd2d/python/fd2d_3_2.py:47-52)."""
    fx1: np.ndarray
    fx2: np.ndarray
    fx3: np.ndarray
    fy1: np.ndarray
    fy2: np.ndarray
    fy3: np.ndarray
    gx2: np.ndarray
    gx3: np.ndarray
    gy2: np.ndarray
    gy3: np.ndarray


def pml_default(nx: int, ny: int) -> PML:
    """Profiles with no absorbing layer (fd2d/python/fd2d_3_2.py:124-135)."""
    return PML(fx1=np.zeros(nx), fx2=np.ones(nx), fx3=np.ones(nx),
               fy1=np.zeros(ny), fy2=np.ones(ny), fy3=np.ones(ny),
               gx2=np.ones(nx), gx3=np.ones(nx), gy2=np.ones(ny), gy3=np.ones(ny))


def pmlparam(nx: int, ny: int, npml: int, grade: float = 0.33) -> PML:
    """fd2d/python/fd2d_3_2.py:91-100 with the grading constant made a parameter.

    Python-float scalar arithmetic, in the reference's own order, so the
    profiles are bit-identical to the reference's at ``grade=0.33``.
    """
    p = pml_default(nx, ny)
    for n in range(npml):
        xm = grade * ((npml - n) / npml) ** 3
        xn = grade * ((npml - n - 0.5) / npml) ** 3
        p.fx1[n] = p.fx1[nx - 2 - n] = p.fy1[n] = p.fy1[ny - 2 - n] = xn
        p.fx2[n] = p.fx2[nx - 2 - n] = p.fy2[n] = p.fy2[ny - 2 - n] = 1 / (1 + xn)
        p.gx2[n] = p.gx2[nx - 1 - n] = p.gy2[n] = p.gy2[ny - 1 - n] = 1 / (1 + xm)
        p.fx3[n] = p.fx3[nx - 2 - n] = p.fy3[n] = p.fy3[ny - 2 - n] = (1 - xn) / (1 + xn)
        p.gx3[n] = p.gx3[nx - 1 - n] = p.gy3[n] = p.gy3[ny - 1 - n] = (1 - xm) / (1 + xm)
    return p


def dielectric(nx: int, ny: int, npml: int, rgrid: float, dt: float, epsr: float,
               sigma: float, rows: slice | None = None):
    """fd2d/python/fd2d_3_4.py:174-194 (true division ``m/3``), vectorised.

    Each cell inside ``[npml, n-npml)`` gets ``(epsr-1)/9`` and ``sigma/9``
    added once per sub-sample ``(m, n)`` in -1..1 whose distance to
    ``(nx/2-1, ny/2-1)`` is ``<= rgrid``.  The sums are formed by the same
    sequence of float64 additions as the reference loop, so the result is
    bit-identical.  ``rows`` restricts the output to a band of rows.
    """
    r0, r1 = (0, nx) if rows is None else (rows.start, rows.stop)
    naz = np.full((r1 - r0, ny), 1.0)
    nbz = np.full((r1 - r0, ny), 0.0)
    ce = (epsr - 1) / 9
    cs = sigma / 9
    # sequential partial sums: eps_k = 1 + ce + ... (k terms), cond_k likewise
    eps_k = [1.0]
    cond_k = [0.0]
    for _ in range(9):
        eps_k.append(eps_k[-1] + ce)
        cond_k.append(cond_k[-1] + cs)
    eps_k = np.array(eps_k)
    cond_k = np.array(cond_k)
    ia = max(npml, r0)
    ib = min(nx - npml, r1)
    if ib <= ia:
        return naz, nbz
    i = np.arange(ia, ib, dtype=np.float64)[:, None]
    j = np.arange(npml, ny - npml, dtype=np.float64)[None, :]
    cnt = np.zeros((ib - ia, ny - 2 * npml), dtype=np.int64)
    for m in range(-1, 2):
        x = nx / 2 - 1 - i + m / 3
        for n in range(-1, 2):
            y = ny / 2 - 1 - j + n / 3
            d = np.sqrt(x ** 2 + y ** 2)
            cnt += (d <= rgrid)
    epsn = eps_k[cnt]
    cond = cond_k[cnt]
    naz[ia - r0:ib - r0, npml:ny - npml] = 1 / (epsn + cond * dt / EPS0)
    nbz[ia - r0:ib - r0, npml:ny - npml] = cond * dt / EPS0
    return naz, nbz


def gaussian(t: int, t0: float, spread: float) -> float:
    """fd2d/python/fd2d_3_4.py:84-86."""
    return float(np.exp(-0.5 * ((t - t0) / spread) ** 2))


def sinusoidal(t: int, ds: float, freq: float) -> float:
    """fd2d/python/fd2d_3_2.py:55-58."""
    dt = ds / 6e8
    return float(np.sin(2 * np.pi * freq * dt * t))


def dfield(nx, ny, pml: PML, dz, hx, hy) -> None:
    """D update of fd2d/program/fd2d_3_2.py:61-64 (no source)."""
    dz[1:nx, 1:ny] = (pml.gx3[1:nx, None] * pml.gy3[1:ny] * dz[1:nx, 1:ny]
                      + pml.gx2[1:nx, None] * pml.gy2[1:ny] * 0.5
                      * (hy[1:nx, 1:ny] - hy[0:nx - 1, 1:ny] - hx[1:nx, 1:ny] + hx[1:nx, 0:ny - 1]))


def efield(nx, ny, naz, dz, ez, iz=None, nbz=None) -> None:
    """fd2d/program/fd2d_3_2.py:69-71 (lossless) or fd2d/python/fd2d_3_4.py:131-136 (lossy)."""
    if iz is None:
        ez[0:nx, 0:ny] = naz[0:nx, 0:ny] * dz[0:nx, 0:ny]
    else:
        ez[0:nx, 0:ny] = naz[0:nx, 0:ny] * (dz[0:nx, 0:ny] - iz[0:nx, 0:ny])
        iz[0:nx, 0:ny] += nbz[0:nx, 0:ny] * ez[0:nx, 0:ny]


def hfield(nx, ny, pml: PML, ez, ihx, ihy, hx, hy) -> None:
    """fd2d/program/fd2d_3_2.py:74-81."""
    curl_em = ez[0:nx - 1, 0:ny - 1] - ez[0:nx - 1, 1:ny]
    curl_en = ez[0:nx - 1, 0:ny - 1] - ez[1:nx, 0:ny - 1]
    ihx[0:nx - 1, 0:ny - 1] += curl_em
    ihy[0:nx - 1, 0:ny - 1] += curl_en
    hx[0:nx - 1, 0:ny - 1] = (pml.fy3[0:ny - 1] * hx[0:nx - 1, 0:ny - 1]
                              + pml.fy2[0:ny - 1] * (0.5 * curl_em + pml.fx1[0:nx - 1, None] * ihx[0:nx - 1, 0:ny - 1]))
    hy[0:nx - 1, 0:ny - 1] = (pml.fx3[0:nx - 1, None] * hy[0:nx - 1, 0:ny - 1]
                              - pml.fx2[0:nx - 1, None] * (0.5 * curl_en + pml.fy1[0:ny - 1] * ihy[0:nx - 1, 0:ny - 1]))


def hfield_free(nx, ny, ez, hx, hy) -> None:
    """fd2d/python/fd2d_3_1.py:66-72 (no PML)."""
    hx[0:nx - 1, 0:ny - 1] += 0.5 * (ez[0:nx - 1, 0:ny - 1] - ez[0:nx - 1, 1:ny])
    hy[0:nx - 1, 0:ny - 1] -= 0.5 * (ez[0:nx - 1, 0:ny - 1] - ez[1:nx, 0:ny - 1])


# ---- TF/SF plane-wave source (fd2d/python/fd2d_3_4.py:103-170) ----------

def ezinct(ny, ezi, hxi, bc) -> None:
    """fd2d/python/fd2d_3_4.py:103-110."""
    ezi[1:ny] += 0.5 * (hxi[0:ny - 1] - hxi[1:ny])
    ezi[0], bc[0], bc[1] = bc[0], bc[1], ezi[1]
    ezi[ny - 1], bc[3], bc[2] = bc[3], bc[2], ezi[ny - 2]


def inctdz(nx, ny, npml, hxi, dz) -> None:
    """fd2d/python/fd2d_3_4.py:123-127."""
    dz[npml - 1:nx - npml + 1, npml - 1] += 0.5 * hxi[npml - 2]
    dz[npml - 1:nx - npml + 1, ny - npml] -= 0.5 * hxi[ny - npml]


def hxinct(ny, ezi, hxi) -> None:
    """fd2d/python/fd2d_3_4.py:140-143."""
    hxi[0:ny - 1] += 0.5 * (ezi[0:ny - 1] - ezi[1:ny])


def incthx(nx, ny, npml, ezi, hx) -> None:
    """fd2d/python/fd2d_3_4.py:158-162."""
    hx[npml - 1:nx - npml + 1, npml - 2] += 0.5 * ezi[npml - 1]
    hx[npml - 1:nx - npml + 1, ny - npml] -= 0.5 * ezi[ny - npml]


def incthy(nx, ny, npml, ezi, hy) -> None:
    """fd2d/python/fd2d_3_4.py:165-170."""
    hy[npml - 2, npml - 1:ny - npml + 1] -= 0.5 * ezi[npml - 1:ny - npml + 1]
    hy[nx - npml, npml - 1:ny - npml + 1] += 0.5 * ezi[npml - 1:ny - npml + 1]


@dataclass
class State2D:
    nx: int
    ny: int
    dz: np.ndarray = None
    ez: np.ndarray = None
    iz: np.ndarray = None
    hx: np.ndarray = None
    hy: np.ndarray = None
    ihx: np.ndarray = None
    ihy: np.ndarray = None
    ezi: np.ndarray = None
    hxi: np.ndarray = None
    bc: np.ndarray = None
    r_pt: np.ndarray = None
    i_pt: np.ndarray = None
    r_in: np.ndarray = None
    i_in: np.ndarray = None

    def __post_init__(self):
        for k in ("dz", "ez", "iz", "hx", "hy", "ihx", "ihy"):
            if getattr(self, k) is None:
                setattr(self, k, np.zeros((self.nx, self.ny)))
        if self.ezi is None:
            self.ezi = np.zeros(self.ny)
            self.hxi = np.zeros(self.ny)
            self.bc = np.zeros(4)


def run(nx: int, ny: int, ns: int, *, pml: PML | None = None, naz=None, nbz=None,
        src=None, tfsf_npml: int | None = None, freq=None, dt: float = 0.01 / 6e8,
        lossy: bool = True, state: State2D | None = None, t_start: int = 1,
        free_space_h: bool = False) -> State2D:
    """Run ``ns`` steps of the 2D TM program, in the reference's step order.

    Order per step (fd2d/python/fd2d_3_4.py:268-277): [ezinct], dfield,
    point source, [inctdz], efield, [fourier], [hxinct], hfield, [incthx,
    incthy].  ``src`` = (kind, i, j, wave) with kind "hard" (``dz[i,j] = v``,
    fd2d/python/fd2d_3_1.py:53) or "soft" (``+=``); wave as in
    ``oracle.fd1d.source_value``.  ``tfsf_npml`` switches the plane-wave
    source of fd2d_3_3/3_4 on (incident ``ezi[3] = gaussian(t,20,8)``).
    ``freq`` switches the full-field running DFT of :90-99 on.
    """
    from .fd1d import source_value
    pml = pml or pml_default(nx, ny)
    naz = np.ones((nx, ny)) if naz is None else naz
    nbz = np.zeros((nx, ny)) if nbz is None else nbz
    st = state or State2D(nx, ny)
    if freq is not None:
        freq = np.asarray(freq, dtype=np.float64)
        if st.r_pt is None:
            nf = freq.size
            st.r_pt = np.zeros((nf, nx, ny))
            st.i_pt = np.zeros((nf, nx, ny))
            st.r_in = np.zeros(nf)
            st.i_in = np.zeros(nf)
    for t in range(t_start, t_start + ns):
        if tfsf_npml is not None:
            ezinct(ny, st.ezi, st.hxi, st.bc)
        dfield(nx, ny, pml, st.dz, st.hx, st.hy)
        if tfsf_npml is not None:
            st.ezi[3] = gaussian(t, 20, 8.0)
        if src is not None:
            kind, si, sj, wave = src
            v = source_value(t, wave)
            if kind == "hard":
                st.dz[si, sj] = v
            else:
                st.dz[si, sj] += v
        if tfsf_npml is not None:
            inctdz(nx, ny, tfsf_npml, st.hxi, st.dz)
        if lossy:
            efield(nx, ny, naz, st.dz, st.ez, st.iz, nbz)
        else:
            efield(nx, ny, naz, st.dz, st.ez)
        if freq is not None:
            arg = 2 * pi * freq * dt * t
            c, s = cos(arg), sin(arg)
            st.r_in += c * st.ezi[6]
            st.i_in -= s * st.ezi[6]
            st.r_pt += c[:, None, None] * st.ez[None]
            st.i_pt -= s[:, None, None] * st.ez[None]
        if tfsf_npml is not None:
            hxinct(ny, st.ezi, st.hxi)
        if free_space_h:
            hfield_free(nx, ny, st.ez, st.hx, st.hy)
        else:
            hfield(nx, ny, pml, st.ez, st.ihx, st.ihy, st.hx, st.hy)
        if tfsf_npml is not None:
            incthx(nx, ny, tfsf_npml, st.ezi, st.hx)
            incthy(nx, ny, tfsf_npml, st.ezi, st.hy)
    return st


def amplitude_row(st: State2D, npml: int):
    """fd2d/python/fd2d_3_4.py:280-284: amplitude/phase on row nx//2-1."""
    nx, ny = st.nx, st.ny
    nf = st.r_in.size
    amplt = np.zeros((nf, ny))
    phase = np.zeros((nf, ny))
    js = slice(npml - 1, ny - npml + 1)
    for n in range(nf):
        rp = st.r_pt[n, nx // 2 - 1, js]
        ip = st.i_pt[n, nx // 2 - 1, js]
        amplt[n, js] = 1 / np.hypot(st.r_in[n], st.i_in[n]) * np.hypot(rp, ip)
        phase[n, js] = np.arctan2(ip, rp) - np.arctan2(st.i_in[n], st.r_in[n])
    return amplt, phase


def program(name: str) -> dict:
    """Keyword arguments of ``run`` replaying a reference program's main()."""
    nx = ny = 100
    dt = 0.01 / 6e8
    if name == "fd2d_3_1":   # fd2d/python/fd2d_3_1.py:75-97
        return dict(nx=nx, ny=ny, ns=90, src=("hard", nx // 2, ny // 2, ("gauss", 20, 6.0)),
                    lossy=False, free_space_h=True)
    if name == "fd2d_3_2":   # fd2d/python/fd2d_3_2.py:103-147
        return dict(nx=nx, ny=ny, ns=120, pml=pmlparam(nx, ny, 8),
                    src=("hard", nx // 2 - 5, ny // 2 - 5, ("sin", 0.01, 1500e6)), lossy=False)
    if name == "fd2d_3_3":   # fd2d/python/fd2d_3_3.py
        return dict(nx=nx, ny=ny, ns=120, pml=pmlparam(nx, ny, 8), tfsf_npml=8, lossy=False)
    if name == "fd2d_3_4":   # fd2d/python/fd2d_3_4.py:209-284
        rgrid = int(0.15 / 0.01 - 1)
        naz, nbz = dielectric(nx, ny, 8, rgrid, dt, 30.0, 0.30)
        return dict(nx=nx, ny=ny, ns=120, pml=pmlparam(nx, ny, 8), naz=naz, nbz=nbz,
                    tfsf_npml=8, freq=np.array([50e6, 300e6, 700e6]), dt=dt, lossy=True)
    raise KeyError(name)
