"""2D TM parity on the GPU through the C-ABI (libfdtd_gb300.so).

* programs fd2d_3_1..3_4 against the golden fixtures written by the
  reference's own code (tolerance: spec 1e-5 max-abs/peak and rel-L2);
* the fused streaming kernel against the per-function kernels, BITWISE, for
  odd sizes, every steps-per-pass and pass counts that exercise the ping-pong;
* the lossy-cylinder PML benchmark miniature against the float64 oracle;
* size-independent properties at the full 8192^2 benchmark size.
"""
import numpy as np
import pytest
import torch

from tests.conftest import assert_parity

pytestmark = pytest.mark.gpu


def _np(t):
    return t.detach().cpu().numpy().astype(np.float64)


def _program_sim(name):
    from simulation_gb300 import fd2d as G
    nx = ny = 100
    dt = 0.01 / 6e8
    if name == "fd2d_3_1":
        return G.SimTM2D(nx, ny, pml=None, lossy=False,
                         source=G.PointSource(nx // 2, ny // 2, ("gauss", 20, 6.0))), 90
    if name == "fd2d_3_2":
        return G.SimTM2D(nx, ny, pml=G.pmlparam(nx, ny, 8), lossy=False,
                         source=G.PointSource(nx // 2 - 5, ny // 2 - 5, ("sin", 0.01, 1500e6))), 120
    if name == "fd2d_3_3":
        return G.SimTM2D(nx, ny, pml=G.pmlparam(nx, ny, 8), lossy=False, tfsf_npml=8), 120
    if name == "fd2d_3_4":
        naz, nbz = G.dielectric(nx, ny, 8, int(0.15 / 0.01 - 1), dt, 30.0, 0.30)
        return G.SimTM2D(nx, ny, pml=G.pmlparam(nx, ny, 8), naz=naz, nbz=nbz, lossy=True, tfsf_npml=8,
                         freq=[50e6, 300e6, 700e6], dt=dt), 120
    raise KeyError(name)


def _extras_sim(nx, ny, lossy, pml, tfsf, nf, ns=256):
    from simulation_gb300 import fd2d as G
    dt = 0.01 / 6e8
    naz = nbz = None
    if lossy:
        naz, nbz = G.dielectric(nx, ny, 8, 14, dt, 30.0, 0.30)
    freq = [50e6, 300e6, 700e6, 120e6, 450e6, 900e6, 75e6, 600e6, 222e6][:nf] if nf else None
    return G.SimTM2D(nx, ny, pml=G.pmlparam(nx, ny, 8) if pml else None, naz=naz, nbz=nbz, lossy=lossy,
                     tfsf_npml=8 if tfsf else 0, freq=freq, dt=dt, ns=ns,
                     source=G.PointSource(nx // 3, ny // 3, ("sin", 0.01, 900e6), "soft"))


@pytest.mark.parametrize("nx,ny", [(100, 100), (97, 83), (130, 68)])
@pytest.mark.parametrize("lossy,pml,tfsf,nf", [(True, True, True, 3), (False, True, True, 0), (True, False, True, 1),
                                               (False, False, False, 8), (True, True, False, 2),
                                               (False, True, True, 4), (True, True, True, 6),
                                               (True, True, True, 9)])
def test_extras_bitwise_equal_nine_functions(cuda_lib, nx, ny, lossy, pml, tfsf, nf):
    """With TF/SF and/or the DFT on, fdtd2d_step_n runs fused passes (the
    incident line advanced ahead of them in chunks of 64 steps; ny % 4 == 0,
    nf <= 8) or three launches per step (otherwise); either way every field,
    the incident line, its ABC state and the DFT accumulators equal the nine
    per-function launches bit for bit.  150 steps cross a line chunk; the
    step counts give odd and even pass counts for every steps-per-pass."""
    for spp, ns in ((4, 150), (3, 70), (1, 5), (2, 9), (0, 131)):
        a = _extras_sim(nx, ny, lossy, pml, tfsf, nf)
        b = _extras_sim(nx, ny, lossy, pml, tfsf, nf)
        a.step(ns, steps_per_pass=spp)
        b.step_per_function(ns)
        torch.cuda.synchronize()
        for k in a.FIELDS:
            x, y = getattr(a, k), getattr(b, k)
            if x is None:
                continue
            assert torch.equal(x, y), f"spp={spp} ns={ns}: {k} differs (max {float((x - y).abs().max()):.3e})"


def test_extras_split_calls_and_graph_replay(cuda_lib):
    """Calls that start mid-chunk, a one-step call (three launches) between
    fused calls, and a captured CUDA graph of the fused loop all give the
    per-function result bit for bit."""
    a = _extras_sim(128, 128, True, True, True, 3)
    b = _extras_sim(128, 128, True, True, True, 3)
    c = _extras_sim(128, 128, True, True, True, 3)
    for n in (37, 1, 66, 3):
        a.step(n)
    b.step_per_function(107)
    c.run_graph(50)
    c.run_graph(57)
    torch.cuda.synchronize()
    for k in a.FIELDS:
        if getattr(a, k) is None:
            continue
        assert torch.equal(getattr(a, k), getattr(b, k)), f"split calls: {k}"
        assert torch.equal(getattr(c, k), getattr(b, k)), f"graph: {k}"


def test_extras_fd2d_3_4_at_2048(cuda_lib):
    """The fd2d_3_4 workload of the benchmark (2048^2, PML 32, lossy cylinder,
    TF/SF, 3-frequency DFT): fused passes equal the per-function launches."""
    from simulation_gb300 import fd2d as G
    n = 2048
    dt = 0.01 / 6e8

    def make():
        naz, nbz = G.dielectric(n, n, 32, n // 8, dt, 30.0, 0.30)
        return G.SimTM2D(n, n, pml=G.pmlparam(n, n, 32), naz=naz, nbz=nbz, lossy=True, tfsf_npml=32,
                         freq=[50e6, 300e6, 700e6], dt=dt, ns=200)
    a, b = make(), make()
    a.step(90)
    b.step_per_function(90)
    torch.cuda.synchronize()
    for k in a.FIELDS:
        if getattr(a, k) is None:
            continue
        assert torch.equal(getattr(a, k), getattr(b, k)), k
    assert float(a.r_pt.abs().max()) > 0 and float(a.ez.abs().max()) > 0


@pytest.mark.parametrize("name", ["fd2d_3_1", "fd2d_3_2", "fd2d_3_3", "fd2d_3_4"])
@pytest.mark.parametrize("path", ["fused", "per_function"])
def test_program_vs_golden(cuda_lib, golden, name, path):
    g = golden("fd2d_programs.npz")
    sim, ns = _program_sim(name)
    if path == "fused":
        sim.step(ns)
    else:
        sim.step_per_function(ns)
    torch.cuda.synchronize()
    sim.check()
    assert_parity(_np(sim.ez), g[f"{name}_ez"], what=f"{name} ez")
    if name == "fd2d_3_4":
        np.testing.assert_array_equal(_np(sim.naz), g["fd2d_3_4_naz"].astype(np.float32))
        from oracle import fd2d as O
        st = O.State2D(100, 100)
        st.r_pt, st.i_pt, st.r_in, st.i_in = (_np(x) for x in (sim.r_pt, sim.i_pt, sim.r_in, sim.i_in))
        amp_o, phase_o = O.amplitude_row(st, 8)
        # the reference's post-processing (fd2d/python/fd2d_3_4.py:280-284) on the device
        amp, phase = sim.amplitude_phase()
        np.testing.assert_allclose(amp.cpu().numpy(), amp_o[:, 7:93], rtol=1e-14)
        np.testing.assert_allclose(phase.cpu().numpy(), phase_o[:, 7:93], rtol=0, atol=1e-13)
        err = assert_parity(amp[2].cpu().numpy(), g["fd2d_3_4_amp2"][7:93], tol=1e-5, what="fd2d_3_4 amplitude")
        print(f"\nfd2d_3_4 amplitude vs golden: max/peak {err[0]:.2e} relL2 {err[1]:.2e}")


def test_steps_lossy_cylinder_golden(cuda_lib, golden):
    """All seven fields after 160 steps vs the reference's own fd2d_3_4 functions."""
    from simulation_gb300 import fd2d as G
    g = golden("fd2d_steps_3_4.npz")
    nx, ny, ns, npml, si, sj, rgrid = (int(v) for v in g["meta"])
    dt = 0.01 / 6e8
    naz, nbz = G.dielectric(nx, ny, npml, rgrid, dt, 30.0, 0.3)
    np.testing.assert_array_equal(_np(naz), g["naz"].astype(np.float32))
    np.testing.assert_array_equal(_np(nbz), g["nbz"].astype(np.float32))
    for path in ("fused", "per_function"):
        sim = G.SimTM2D(nx, ny, pml=G.pmlparam(nx, ny, npml), naz=naz, nbz=nbz,
                        source=G.PointSource(si, sj, ("gauss", 20, 6.0)))
        (sim.step if path == "fused" else sim.step_per_function)(ns)
        torch.cuda.synchronize()
        for k in ("dz", "ez", "iz", "hx", "hy", "ihx", "ihy"):
            assert_parity(_np(getattr(sim, k)), g[k], what=f"{path} {k}")


def _mk(nx, ny, npml, lossy, pml, src=True, rgrid=None, grade=0.33):
    from simulation_gb300 import fd2d as G
    dt = 0.01 / 6e8
    naz = nbz = None
    if lossy:
        naz, nbz = G.dielectric(nx, ny, npml, rgrid or min(nx, ny) // 4, dt, 30.0, 0.3)
    return G.SimTM2D(nx, ny, pml=G.pmlparam(nx, ny, npml, grade) if pml else None, naz=naz, nbz=nbz,
                     lossy=lossy, source=G.PointSource(nx // 2, ny // 2, ("gauss", 20, 6.0)) if src else None)


@pytest.mark.parametrize("nx,ny", [(67, 44), (130, 132), (9, 8), (300, 260)])
@pytest.mark.parametrize("lossy,pml", [(True, True), (False, True), (True, False), (False, False)])
def test_fused_bitwise_equals_per_function(cuda_lib, nx, ny, lossy, pml):
    npml = min(6, (min(nx, ny) - 1) // 2 - 1) if pml else 0
    for spp, ns in ((1, 5), (2, 9), (3, 13), (4, 17), (4, 8), (0, 3)):
        a = _mk(nx, ny, npml, lossy, pml)
        b = _mk(nx, ny, npml, lossy, pml)
        a.step(ns, steps_per_pass=spp)
        b.step_per_function(ns)
        torch.cuda.synchronize()
        for k in ("dz", "ez", "iz", "hx", "hy", "ihx", "ihy"):
            x, y = getattr(a, k), getattr(b, k)
            if x is None:
                continue
            assert torch.equal(x, y), f"{nx}x{ny} lossy={lossy} pml={pml} spp={spp} ns={ns}: {k} differs " \
                                      f"(max {float((x - y).abs().max()):.3e})"


def test_segments_and_stripes_bitwise(cuda_lib):
    """Force short row segments so many warps share cone rows; still bitwise."""
    from simulation_gb300 import _lib
    try:
        for cpl, seg in ((4, 7), (2, 5), (4, 64), (2, 33)):
            _lib.call("fdtd2d_set_march_config", cpl, 4, seg)
            a = _mk(200, 136, 8, True, True)
            b = _mk(200, 136, 8, True, True)
            a.step(23, steps_per_pass=4)
            b.step_per_function(23)
            torch.cuda.synchronize()
            for k in ("dz", "ez", "iz", "hx", "hy", "ihx", "ihy"):
                assert torch.equal(getattr(a, k), getattr(b, k)), f"cpl={cpl} seg={seg} {k}"
    finally:
        _lib.call("fdtd2d_set_march_config", 0, 4, 0)


def test_benchmark_miniature_vs_oracle(cuda_lib):
    """The lossy-cylinder PML benchmark at 256^2 (npml 32, grade 0.333) vs float64."""
    from oracle import fd2d as O
    from simulation_gb300 import fd2d as G
    nx = ny = 256
    ns = 400
    dt = 0.01 / 6e8
    sim = G.benchmark_sim(nx, ny, npml=32, grade=0.333, rgrid=60, ns=ns)
    sim.step(ns)
    torch.cuda.synchronize()
    sim.check()
    pml = O.pmlparam(nx, ny, 32, 0.333)
    naz, nbz = O.dielectric(nx, ny, 32, 60, dt, 30.0, 0.3)
    st = O.run(nx, ny, ns, pml=pml, naz=naz, nbz=nbz, src=("hard", nx // 2, ny // 2, ("gauss", 20, 6.0)))
    for k in ("dz", "ez", "iz", "hx", "hy", "ihx", "ihy"):
        assert_parity(_np(getattr(sim, k)), getattr(st, k), what=k)


def test_graph_replay_and_checkpoint(cuda_lib):
    a = _mk(128, 128, 8, True, True)
    b = _mk(128, 128, 8, True, True)
    a.step(40)
    b.run_graph(20)
    snap = b.state_dict()
    b.run_graph(20)
    torch.cuda.synchronize()
    for k in ("dz", "ez", "iz", "hx", "hy", "ihx", "ihy"):
        assert torch.equal(getattr(a, k), getattr(b, k)), k
    c = _mk(128, 128, 8, True, True)
    c.load_state_dict(snap)
    c.step(20)
    torch.cuda.synchronize()
    for k in ("dz", "ez", "iz", "hx", "hy", "ihx", "ihy"):
        assert torch.equal(getattr(a, k), getattr(c, k)), k


def test_nonfinite_status(cuda_lib):
    from simulation_gb300 import _lib
    a = _mk(64, 64, 6, True, True)
    a.naz[40, 40] = float("nan")
    a.step(30)
    torch.cuda.synchronize()
    with pytest.raises(_lib.FdtdError) as e:
        a.check()
    assert e.value.code == -6


def test_full_size_linearity(cuda_lib):
    """8192^2 benchmark grid: doubling the source doubles every field exactly."""
    from simulation_gb300 import fd2d as G
    from simulation_gb300.sources import to_device, wave_values
    a = G.benchmark_sim(ns=64)
    b = G.benchmark_sim(ns=64)
    b.src_table = to_device(2.0 * wave_values(("gauss", 20, 6.0), 1, b._ns))
    b._build_structs()
    a.step(40)
    b.step(40)
    torch.cuda.synchronize()
    a.check()
    # scaling by 2 commutes with every rounding except in the subnormal range
    # (the far tail of the light cone), so: bitwise equality for normal-size
    # values, and an absolute bound at the bottom of the float range
    for k in ("dz", "ez", "iz", "hx", "hy", "ihx", "ihy"):
        x2, y = 2.0 * getattr(a, k), getattr(b, k)
        big = y.abs() > 1e-20
        assert torch.equal(x2[big], y[big]), k
        assert float((x2 - y).abs().max()) <= 1e-35, k
    assert float(a.ez.abs().max()) > 0.0
