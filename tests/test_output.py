"""Output helpers on the host: the reference's printed field slice and array
dumps (fd1d/program/test_1_3.py:70, fd2d/python/test_3_4.py:292).  No GPU:
they only copy tensors out."""
import os

import numpy as np
import torch

from simulation_gb300 import output


class _Sim:
    FIELDS = ("ex", "hy", "dx")

    def __init__(self):
        self.ex = torch.arange(64, dtype=torch.float32) / 7
        self.hy = torch.ones(64, dtype=torch.float32)
        self.dx = None
        self.t = 17


def test_head_matches_numpy_print():
    s = _Sim()
    assert output.head(s.ex) == str(s.ex.numpy()[0:50])
    assert output.head(s.ex, 5) == str(s.ex.numpy()[0:5])


def test_save_npz_and_directory(tmp_path):
    s = _Sim()
    p = output.save(s, str(tmp_path / "fields"))
    with np.load(p) as z:
        assert sorted(z.files) == ["ex", "hy", "t"]
        np.testing.assert_array_equal(z["ex"], s.ex.numpy())
        assert int(z["t"]) == 17
    d = tmp_path / "dir"
    d.mkdir()
    output.save(s, str(d), names=["hy"])
    assert sorted(os.listdir(d)) == ["hy.npy", "t.npy"]
    np.testing.assert_array_equal(np.load(d / "hy.npy"), s.hy.numpy())
