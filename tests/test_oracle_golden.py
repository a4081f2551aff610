"""The oracle against the golden fixtures produced by the reference's own code.

``tests/golden/make_golden.py`` ran the reference programs (their main() with
plotting captured, or their own step functions) to write the fixtures; here the
float64 NumPy restatement in ``oracle/`` must reproduce them exactly.
"""
import numpy as np
import pytest

from oracle import fd1d, fd2d

FD1D = ["fd1d_1_1", "fd1d_1_2", "fd1d_1_3", "fd1d_1_4", "fd1d_1_5", "fd1d_2_1", "fd1d_2_2", "fd1d_2_3"]


@pytest.mark.parametrize("name", FD1D)
def test_fd1d_program(golden, name):
    g = golden("fd1d_programs.npz")
    st = fd1d.run(**fd1d.program(name))
    np.testing.assert_array_equal(st.ex, g[f"{name}_ex"])
    if f"{name}_amp2" in g:
        amp, _ = fd1d.amplitude_phase(st.r_pt, st.i_pt, st.r_pr[0][:, None], st.i_pr[0][:, None])
        np.testing.assert_array_equal(amp[2], g[f"{name}_amp2"])


def test_problem_1_4(golden):
    g = golden("fd1d_programs.npz")
    st = fd1d.run(**fd1d.program("problem_1_4"))
    np.testing.assert_array_equal(st.ex, g["problem_1_4_ex"])
    np.testing.assert_array_equal(st.hy, g["problem_1_4_hy"])


def test_fd1d_2_2_step_functions(golden):
    g = golden("fd1d_programs.npz")
    dt = 0.01 / 6e8
    nax, nbx = fd1d.dielectric_dform(300, dt, 4.0, 0.04)
    st = fd1d.run(300, 400, "dform", nax=nax, nbx=nbx, src_kind="soft", src_k=1, wave=("gauss", 50, 10.0))
    for k in ("dx", "ex", "ix", "hy", "bc"):
        np.testing.assert_array_equal(getattr(st, k), g[f"steps_2_2_{k}"])


@pytest.mark.parametrize("name", ["fd2d_3_1", "fd2d_3_2", "fd2d_3_3", "fd2d_3_4"])
def test_fd2d_program(golden, name):
    g = golden("fd2d_programs.npz")
    kw = fd2d.program(name)
    st = fd2d.run(**kw)
    np.testing.assert_array_equal(st.ez, g[f"{name}_ez"])
    if f"{name}_amp2" in g:
        amp, _ = fd2d.amplitude_row(st, 8)
        np.testing.assert_array_equal(amp[2], g[f"{name}_amp2"])
        np.testing.assert_array_equal(kw["naz"], g[f"{name}_naz"])


def test_fd2d_steps_lossy_cylinder(golden):
    g = golden("fd2d_steps_3_4.npz")
    nx, ny, ns, npml, si, sj, rgrid = (int(v) for v in g["meta"])
    dt = 0.01 / 6e8
    pml = fd2d.pmlparam(nx, ny, npml)
    for k in ("fx1", "fx2", "fx3", "fy1", "fy2", "fy3", "gx2", "gx3", "gy2", "gy3"):
        np.testing.assert_array_equal(getattr(pml, k), g[f"pml_{k}"])
    naz, nbz = fd2d.dielectric(nx, ny, npml, rgrid, dt, 30.0, 0.3)
    np.testing.assert_array_equal(naz, g["naz"])
    np.testing.assert_array_equal(nbz, g["nbz"])
    st = fd2d.run(nx, ny, ns, pml=pml, naz=naz, nbz=nbz, src=("hard", si, sj, ("gauss", 20, 6.0)))
    for k in ("dz", "ez", "iz", "hx", "hy", "ihx", "ihy"):
        np.testing.assert_array_equal(getattr(st, k), g[k])
