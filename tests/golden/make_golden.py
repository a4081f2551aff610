"""Generate the golden fixtures in this folder from the reference's own programs.

Run in a container that holds the dsarvan/simulation checkout (default
``/root/reference``, override with ``FDTD_REFERENCE_ROOT``):

    python tests/golden/make_golden.py

Every array written here comes from executing the reference's Python code
(``oracle.refload`` stubs out matplotlib/numba only): its ``main()`` with the
plotting calls captured, or its own step functions driven in a loop.  Nothing
is computed by this repository's oracle or library.  The fixtures are float64
``.npz`` files; the test suite compares the oracle against them on any machine.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
# the development container's checkout unless FDTD_REFERENCE_ROOT names another
os.environ.setdefault("FDTD_REFERENCE_ROOT", "/root/reference")

from oracle import refload  # noqa: E402

FD1D = ["fd1d_1_1", "fd1d_1_2", "fd1d_1_3", "fd1d_1_4", "fd1d_1_5", "fd1d_2_1", "fd1d_2_2", "fd1d_2_3"]
FD2D = ["fd2d_3_1", "fd2d_3_2", "fd2d_3_3", "fd2d_3_4"]


def golden_fd1d() -> None:
    out = {}
    for name in FD1D:
        cap = refload.run_main_capture(f"fd1d/program/{name}.py", ("visualize", "amplitude"))
        out[f"{name}_ex"] = np.asarray(cap["visualize"][0][-1], dtype=np.float64)
        if cap["amplitude"]:
            out[f"{name}_amp2"] = np.asarray(cap["amplitude"][0][-1], dtype=np.float64)
    # fd1d/problem/problem_1_4/fd1d_1_1.py runs its loop at import time
    mod = refload.load("fd1d/problem/problem_1_4/fd1d_1_1.py")
    out["problem_1_4_ex"] = np.array(mod.ex, dtype=np.float64)
    out["problem_1_4_hy"] = np.array(mod.hy, dtype=np.float64)
    # the D-form step functions of fd1d_2_2 driven directly: all arrays
    m = refload.load("fd1d/program/fd1d_2_2.py")
    nx, ns = 300, 400
    dt = 0.01 / 6e8
    md = m.dielectric(nx, dt, 4.0, 0.04)
    dx, ex, ix, hy, bc = (np.zeros(nx) for _ in range(5))
    bc = np.zeros(4)
    for t in np.arange(1, ns + 1).astype(np.int32):
        m.dxfield(t, nx, dx, hy)
        m.exfield(nx, md, dx, ix, ex)
        m.hyfield(nx, ex, hy, bc)
    for k, v in dict(dx=dx, ex=ex, ix=ix, hy=hy, bc=bc).items():
        out[f"steps_2_2_{k}"] = v
    np.savez_compressed(os.path.join(HERE, "fd1d_programs.npz"), **out)
    print("fd1d_programs.npz:", sorted(out))


def golden_fd2d() -> None:
    out = {}
    for name in FD2D:
        cap = refload.run_main_capture(f"fd2d/python/{name}.py", ("surfaceplot", "amplitudeplot"))
        out[f"{name}_ez"] = np.asarray(cap["surfaceplot"][0][-1], dtype=np.float64)
        if cap["amplitudeplot"]:
            out[f"{name}_amp2"] = np.asarray(cap["amplitudeplot"][0][-1], dtype=np.float64)
            out[f"{name}_naz"] = np.asarray(cap["surfaceplot"][0][5], dtype=np.float64)
    np.savez_compressed(os.path.join(HERE, "fd2d_programs.npz"), **out)
    print("fd2d_programs.npz:", sorted(out))


def golden_fd2d_steps() -> None:
    """Drive fd2d_3_4's own dfield/efield/hfield/pmlparam/dielectric on a
    non-square grid with a hard Gaussian point source (fd2d_3_1's source) --
    a miniature of the lossy-cylinder PML benchmark.  All seven field arrays
    are saved."""
    m = refload.load("fd2d/python/fd2d_3_4.py")
    g = refload.load("fd2d/python/fd2d_3_1.py")
    nx, ny, ns, npml = 48, 40, 160, 6
    dt = 0.01 / 6e8
    pml = m.pmlayer(
        fx1=np.full(nx, 0.0), fx2=np.full(nx, 1.0), fx3=np.full(nx, 1.0),
        fy1=np.full(ny, 0.0), fy2=np.full(ny, 1.0), fy3=np.full(ny, 1.0),
        gx2=np.full(nx, 1.0), gx3=np.full(nx, 1.0), gy2=np.full(ny, 1.0), gy3=np.full(ny, 1.0))
    m.pmlparam(nx, ny, npml, pml)
    md = m.dielectric(nx, ny, npml, 9, dt, 30.0, 0.3)
    dz, ez, iz, hx, hy, ihx, ihy = (np.zeros((nx, ny)) for _ in range(7))
    ezi = np.zeros(ny)
    si, sj = nx // 2, ny // 2
    for t in np.arange(1, ns + 1).astype(np.int32):
        m.dfield(t, nx, ny, pml, ezi, dz, hx, hy)
        dz[si, sj] = g.gaussian(t, 20, 6.0)
        m.efield(nx, ny, md, dz, iz, ez)
        m.hfield(nx, ny, pml, ez, ihx, ihy, hx, hy)
    out = dict(dz=dz, ez=ez, iz=iz, hx=hx, hy=hy, ihx=ihx, ihy=ihy, naz=md.naz, nbz=md.nbz)
    for k in pml._fields:
        out[f"pml_{k}"] = getattr(pml, k)
    out["meta"] = np.array([nx, ny, ns, npml, si, sj, 9], dtype=np.int64)
    np.savez_compressed(os.path.join(HERE, "fd2d_steps_3_4.npz"), **out)
    print("fd2d_steps_3_4.npz:", sorted(out))


if __name__ == "__main__":
    if not refload.available():
        sys.exit(f"reference checkout not found at {refload.REF_ROOT}")
    golden_fd1d()
    golden_fd2d_steps()
    golden_fd2d()
