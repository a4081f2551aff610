"""The FP64 torch restatement used to check the adjoint kernel, on CPU:
its forward equals the NumPy oracle, and its autograd gradient agrees with
central finite differences."""
import numpy as np
import torch

from oracle import fd2d as O2
from oracle import torch_fd2d as T

KW = dict(nx=40, ny=36, npml=5, box=(14, 12, 10, 12), src=(8, 18), probe=(30, 18), ns=90,
          wave=("gauss", 20, 6.0), src_kind="soft", sigma_box=0.05, grade=0.33)


def _eps():
    return torch.as_tensor(np.random.default_rng(0).uniform(1, 4, size=(10, 12)), dtype=torch.float64)


def test_torch_forward_equals_numpy_oracle():
    eps = _eps()
    J = float(T.objective(eps, **KW))
    nx, ny = KW["nx"], KW["ny"]
    i0, j0, bi, bj = KW["box"]
    dt = 0.01 / 6e8
    naz = np.ones((nx, ny))
    nbz = np.zeros((nx, ny))
    nb = KW["sigma_box"] * dt / 8.854e-12
    naz[i0:i0 + bi, j0:j0 + bj] = 1 / (eps.numpy() + nb)
    nbz[i0:i0 + bi, j0:j0 + bj] = nb
    st = O2.State2D(nx, ny)
    Jn = 0.0
    for t in range(1, KW["ns"] + 1):
        O2.run(nx, ny, 1, pml=O2.pmlparam(nx, ny, KW["npml"]), naz=naz, nbz=nbz,
               src=("soft", KW["src"][0], KW["src"][1], KW["wave"]), state=st, t_start=t)
        Jn += st.ez[KW["probe"]] ** 2
    assert abs(J - Jn) <= 1e-12 * abs(Jn)


def test_torch_gradient_matches_central_differences():
    eps = _eps()
    J, g = T.gradient(eps, **KW)
    h = 1e-6
    for (a, b) in [(0, 0), (4, 7), (9, 11), (5, 2)]:
        ep, em = eps.clone(), eps.clone()
        ep[a, b] += h
        em[a, b] -= h
        fd = (float(T.objective(ep, **KW)) - float(T.objective(em, **KW))) / (2 * h)
        assert abs(fd - float(g[a, b])) <= 1e-5 * max(abs(fd), 1e-12) + 1e-12, (a, b, fd, float(g[a, b]))
