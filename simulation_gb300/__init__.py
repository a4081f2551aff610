"""GB300-native (sm_103a) FDTD: the time-step hot path of dsarvan/simulation.

``fd1d`` and ``fd2d`` mirror the reference's 1D and 2D programs; all compute
runs in the CUDA library ``libfdtd_gb300.so`` (C-ABI in ``include/fdtd.h``,
built by ``simulation_gb300.build``).  Importing this package does not touch
the GPU; the library is loaded on first use and a missing library raises.
"""
from ._lib import FdtdError, FdtdLibraryError, lib  # noqa: F401

__version__ = "0.1.0"
