"""1D parity on the GPU through the C-ABI.

Every reference fd1d program against the golden fixtures written by the
reference's own code; the fused cluster kernel against the per-function
kernels bitwise; the config-1 case (ke=200, hard source at k=5) against the
float64 oracle.
"""
import numpy as np
import pytest
import torch

from tests.conftest import assert_parity

pytestmark = pytest.mark.gpu

FD1D = ["fd1d_1_1", "fd1d_1_2", "fd1d_1_3", "fd1d_1_4", "fd1d_1_5", "fd1d_2_1", "fd1d_2_2", "fd1d_2_3"]


def _np(t):
    return t.detach().cpu().numpy().astype(np.float64)


@pytest.mark.parametrize("name", FD1D)
def test_program_vs_golden(cuda_lib, golden, name):
    from simulation_gb300 import fd1d as G
    g = golden("fd1d_programs.npz")
    ns = G.PROGRAM_STEPS[name]
    a = G.program(name)
    b = G.program(name)
    a.step(ns)
    b.step_per_function(ns)
    torch.cuda.synchronize()
    a.check()
    assert_parity(_np(a.ex), g[f"{name}_ex"], what=f"{name} ex")
    for k in ("ex", "hy", "dx", "ix", "sx", "bc", "r_pt", "i_pt", "r_pr", "i_pr"):
        x, y = getattr(a, k), getattr(b, k)
        if x is not None:
            assert torch.equal(x, y), f"{name}: fused vs per-function {k}"
    if f"{name}_amp2" in g:
        # the reference's post-processing (fd1d/program/fd1d_2_2.py:145-146) on the device
        amp, phase = a.amplitude_phase()
        rp, ip = _np(a.r_pt), _np(a.i_pt)
        rin, iin = _np(a.r_pr)[0][:, None], _np(a.i_pr)[0][:, None]
        np.testing.assert_allclose(amp.cpu().numpy(), 1 / np.hypot(rin, iin) * np.hypot(rp, ip), rtol=1e-14)
        np.testing.assert_allclose(phase.cpu().numpy(), np.arctan2(ip, rp) - np.arctan2(iin, rin), rtol=0,
                                   atol=1e-13)
        err = assert_parity(amp[2].cpu().numpy(), g[f"{name}_amp2"], tol=1e-5, what=f"{name} amplitude")
        print(f"\n{name} amplitude vs golden: max/peak {err[0]:.2e} relL2 {err[1]:.2e}")


def test_config1_vs_oracle(cuda_lib):
    from oracle import fd1d as O
    from simulation_gb300 import fd1d as G
    a = G.program("config1")
    a.step(1000)
    torch.cuda.synchronize()
    st = O.run(**O.program("config1"))
    assert_parity(_np(a.ex), st.ex, what="ex")
    assert_parity(_np(a.hy), st.hy, what="hy")


@pytest.mark.parametrize("nx", [5, 33, 38000, 65536])
@pytest.mark.parametrize("form", ["cb", "cacb", "dform", "debye"])
def test_fused_bitwise_sizes(cuda_lib, nx, form):
    from simulation_gb300 import fd1d as G
    dt = 0.01 / 6e8
    kw = {}
    if form == "cb":
        kw["cb"] = G.dielectric_cb(nx, 4.0)
    elif form == "cacb":
        kw["ca"], kw["cb"] = G.dielectric_cacb(nx, dt, 4.0, 0.04)
    elif form == "dform":
        kw["nax"], kw["nbx"] = G.dielectric_dform(nx, dt, 4.0, 0.04)
    else:
        kw["nax"], kw["nbx"], kw["ncx"], kw["ndx"] = G.dielectric_debye(nx, dt, 2.0, 1e-9, 2.0, 0.01)
    ns = 60 if nx > 1000 else 300
    probes = (min(3, nx - 1), nx - 2)
    mk = lambda: G.Sim1D(nx, form, src_kind="soft", src_k=min(2, nx - 1), wave=("gauss", 20, 6.0),  # noqa: E731
                         freq=[1e8, 3e8], probes=probes, full_dft=nx < 1000, **kw)
    a, b = mk(), mk()
    a.step(ns)
    b.step_per_function(ns)
    torch.cuda.synchronize()
    for k in ("ex", "hy", "dx", "ix", "sx", "bc", "r_pt", "i_pt", "r_pr", "i_pr"):
        x, y = getattr(a, k), getattr(b, k)
        if x is not None:
            assert torch.equal(x, y), f"{form} nx={nx}: {k} (max {float((x - y).abs().max()):.3e})"


def _coeffs(nx, form):
    from simulation_gb300 import fd1d as G
    dt = 0.01 / 6e8
    if form == "cb":
        return {"cb": G.dielectric_cb(nx, 4.0)}
    if form == "cacb":
        ca, cb = G.dielectric_cacb(nx, dt, 4.0, 0.04)
        return {"ca": ca, "cb": cb}
    if form == "dform":
        nax, nbx = G.dielectric_dform(nx, dt, 4.0, 0.04)
        return {"nax": nax, "nbx": nbx}
    nax, nbx, ncx, ndx = G.dielectric_debye(nx, dt, 2.0, 1e-9, 2.0, 0.01)
    return {"nax": nax, "nbx": nbx, "ncx": ncx, "ndx": ndx}


def _fused_vs_per_function(nx, form, ns, **kw):
    from simulation_gb300 import fd1d as G
    co = _coeffs(nx, form)
    a, b = G.Sim1D(nx, form, **co, **kw), G.Sim1D(nx, form, **co, **kw)
    a.step(ns)
    b.step_per_function(ns)
    torch.cuda.synchronize()
    a.check()
    for k in ("ex", "hy", "dx", "ix", "sx", "bc", "r_pt", "i_pt", "r_pr", "i_pr"):
        x, y = getattr(a, k), getattr(b, k)
        if x is not None:
            assert torch.equal(x, y), f"{form} nx={nx} {kw}: {k} (max {float((x - y).abs().max()):.3e})"


# one warp holds lines of up to 512 cells: 2, 4, 8 or 16 cells per lane; the
# high-side ABC cell at the end of its lane (nx a multiple of the cells per
# lane) or anywhere in it; the source at cell 0, at lane edges, at nx-1
@pytest.mark.parametrize("nx,src_k", [(4, 0), (5, 4), (7, 1), (64, 63), (100, 8), (129, 4), (200, 5), (203, 31),
                                      (256, 128), (257, 16), (480, 479), (511, 0), (512, 15)])
@pytest.mark.parametrize("form", ["cb", "cacb", "dform", "debye"])
def test_warp_kernel_bitwise(cuda_lib, nx, src_k, form):
    hard = (nx + src_k) % 2 == 0
    abc = nx % 3 != 2
    _fused_vs_per_function(nx, form, 250, src_kind="hard" if hard else "soft", src_k=src_k,
                           wave=("gauss", 20, 6.0), abc=abc, freq=[1e8, 3e8, 7e8],
                           probes=(0, nx - 1, nx // 2), full_dft=nx % 2 == 1)


@pytest.mark.parametrize("nx", [200, 201])
def test_warp_kernel_no_source_no_dft(cuda_lib, nx):
    from simulation_gb300 import fd1d as G
    # a nonzero initial field and no source: the ABC alone drives the ends
    co = _coeffs(nx, "cb")
    a, b = G.Sim1D(nx, "cb", src_kind="none", **co), G.Sim1D(nx, "cb", src_kind="none", **co)
    init = torch.sin(torch.arange(nx, dtype=torch.float32, device="cuda") * 0.1)
    for s in (a, b):
        s.ex.copy_(init)
        s.hy.copy_(0.5 * init)
    a.step(300)
    b.step_per_function(300)
    torch.cuda.synchronize()
    for k in ("ex", "hy", "bc"):
        assert torch.equal(getattr(a, k), getattr(b, k)), k


@pytest.mark.parametrize("nx,nf", [(200, 40), (600, 200)])
def test_probe_dft_more_frequencies_than_threads(cuda_lib, nx, nf):
    """nf larger than the fused kernel's lanes (one warp) or threads per block:
    the probe accumulators then live in global memory, same arithmetic."""
    freq = np.linspace(5e7, 9e8, nf)
    _fused_vs_per_function(nx, "dform", 120, src_kind="soft", src_k=3, wave=("gauss", 20, 6.0), freq=freq,
                           probes=(1, nx // 3, nx - 2), full_dft=False)


# the single-warp run without the DFT at 4, 8 and 16 cells per lane, nx a
# multiple of them (the compile-time ABC variant): sources on either side of
# a lane edge, odd step counts, with and without the ABC
@pytest.mark.parametrize("nx,src_k", [(128, 3), (128, 4), (200, 7), (200, 8), (200, 9), (200, 15), (512, 16),
                                      (512, 31), (512, 1)])
@pytest.mark.parametrize("form", ["cb", "cacb"])
def test_warp_kernel_lane_edge_sources_bitwise(cuda_lib, nx, src_k, form):
    hard = src_k % 2 == 1
    for ns, abc in ((301, True), (250, False)):
        _fused_vs_per_function(nx, form, ns, src_kind="hard" if hard else "soft", src_k=src_k,
                               wave=("gauss", 20, 6.0), abc=abc)


@pytest.mark.parametrize("nx", [200, 203, 700])
def test_fused_split_calls_bitwise(cuda_lib, nx):
    """One run as several fused calls (t0 > 0, not on the 32-step source
    chunks of the single-warp kernel) equals the per-function loop: sources,
    ABC state and the running DFT continue across calls."""
    from simulation_gb300 import fd1d as G
    co = _coeffs(nx, "dform")
    kw = dict(src_kind="soft", src_k=3, wave=("gauss", 30, 8.0), freq=[1e8, 4e8], probes=(2, nx - 3),
              full_dft=True, **co)
    a, b = G.Sim1D(nx, "dform", **kw), G.Sim1D(nx, "dform", **kw)
    for n in (37, 100, 1, 163):
        a.step(n)
    b.step_per_function(301)
    torch.cuda.synchronize()
    for k in ("ex", "hy", "dx", "ix", "bc", "r_pt", "i_pt", "r_pr", "i_pr"):
        x, y = getattr(a, k), getattr(b, k)
        assert torch.equal(x, y), f"nx={nx} {k}"
