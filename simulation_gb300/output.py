"""Outputs of a program run: the reference's printed field slices, array
dumps, and the DFT amplitude/phase post-processing.

The reference's benchmark twins print the first 50 values of a field after
the time loop (``print(ex[0:50])``, fd1d/program/test_1_3.py:70;
``print(ez[2][0:50])``, fd2d/python/test_3_4.py:292) and its programs plot
fields and amplitudes with matplotlib.  Plots stay out of this library; the
same numbers are available as text (``head``) and as ``.npy``/``.npz`` files
(``save``), which any plotting tool reads.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np
import torch

from . import _lib


def head(field, n: int = 50) -> str:
    """Text of ``print(field[0:n])`` for a device field (numpy's formatting
    of the float32 values, as the reference's float32 twins print them)."""
    a = field.detach().reshape(-1)[:n] if isinstance(field, torch.Tensor) else np.asarray(field).reshape(-1)[:n]
    if isinstance(a, torch.Tensor):
        a = a.cpu().numpy()
    return str(a)


def save(sim, path: str, names=None) -> str:
    """Write the program's arrays (default: every field it holds) and its step
    count to ``path``: one ``.npz`` archive, or, if ``path`` is a directory,
    one ``<name>.npy`` per array plus ``t.npy``.  Returns the path."""
    names = [k for k in (names or sim.FIELDS) if getattr(sim, k, None) is not None]
    arrays = {k: getattr(sim, k).detach().cpu().numpy() for k in names}
    arrays["t"] = np.array(sim.t)
    if os.path.isdir(path):
        for k, a in arrays.items():
            np.save(os.path.join(path, f"{k}.npy"), a)
        return path
    np.savez(path, **arrays)
    return path if path.endswith(".npz") else path + ".npz"


def amplitude_phase(r_pt, i_pt, r_in, i_in, offset: int = 0, count: int | None = None):
    """(amp, phase) float64 [nf][count]: the reference's post-processing of the
    running DFT, amp = 1/hypot(r_in, i_in) * hypot(r_pt, i_pt) and phase =
    atan2(i_pt, r_pt) - atan2(i_in, r_in), on the device.  ``r_pt``/``i_pt``
    are [nf][...] float32 accumulators, read from flat element ``offset`` on
    in each frequency's plane; ``r_in``/``i_in`` the input probe's [nf]."""
    nf = r_pt.shape[0]
    ld = r_pt[0].numel()
    count = ld - offset if count is None else count
    if not (0 <= offset and offset + count <= ld):
        raise ValueError("offset/count outside the accumulator plane")
    amp = torch.empty((nf, count), dtype=torch.float64, device=r_pt.device)
    phase = torch.empty_like(amp)
    base_r = r_pt.data_ptr() + 4 * offset
    base_i = i_pt.data_ptr() + 4 * offset
    _lib.call("fdtd_dft_amplitude_phase", nf, count, base_r, base_i, ld, r_in.data_ptr(), i_in.data_ptr(),
              amp.data_ptr(), phase.data_ptr(), _lib.stream_ptr())
    return amp, phase
