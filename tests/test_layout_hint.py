"""The work-layout hint SimTM2D passes to the fused kernel (pml_cells): the
thickness of the absorbing layer read from the ten PML vectors, on the host.
Only the balance of the kernel's work depends on it, never its results; the
GPU tests run grids with and without a layer, and the layout itself is
checked on the CPU by tests/march_mapping_check.cu."""
from simulation_gb300 import fd2d as G


def test_pml_cells_from_profiles():
    assert G.pml_cells(None) == 0
    # pmlparam sets n and N-2-n (f*) and n and N-1-n (g*) for n < npml, so the
    # layer reaches npml cells at the low ends and npml+1 at the high ends
    assert G.pml_cells(G.pmlparam(100, 80, 8, device="cpu")) == 9
    assert G.pml_cells(G.pmlparam(8192, 8192, 32, 0.333, device="cpu")) == 33
    assert G.pml_cells(G.pmlparam(64, 64, 0, device="cpu")) == 0
