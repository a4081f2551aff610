"""Import the reference's own Python programs by file path (oracle pinning only).

The reference programs import ``matplotlib``, ``mpl_toolkits.mplot3d`` and
``numba``, none of which is installed here.  This module installs stand-in
modules for them -- plotting calls do nothing, ``numba.jit`` returns the
function unchanged and ``numba.prange`` is ``range`` -- and then loads a
program from the reference tree so its functions (or its ``main()``, with the
plotting functions replaced by capture hooks) can be run in float64.

It needs the reference checkout, which exists only in the development
container; ``tests/golden/make_golden.py`` uses it to write the committed
fixtures that the test suite checks the oracle against everywhere else.
"""
from __future__ import annotations

import importlib.util
import os
import sys
import types

# the checkout's root comes from the environment (tests/golden/make_golden.py
# sets it); unset means no reference here
REF_ROOT = os.environ.get("FDTD_REFERENCE_ROOT", "")


def available() -> bool:
    return bool(REF_ROOT) and os.path.isdir(os.path.join(REF_ROOT, "fd1d")) and \
        os.path.isdir(os.path.join(REF_ROOT, "fd2d"))


class _Anything:
    """Absorbs any attribute access or call (stand-in for pyplot objects)."""

    def __getattr__(self, name):
        return _Anything()

    def __call__(self, *a, **k):
        return _Anything()

    def __iter__(self):
        return iter((_Anything(), _Anything()))

    def __setitem__(self, k, v):
        pass


def _install_stubs() -> None:
    if "matplotlib" not in sys.modules or not getattr(sys.modules["matplotlib"], "_fdtd_stub", False):
        mpl = types.ModuleType("matplotlib")
        mpl._fdtd_stub = True
        mpl.rcParams = {}
        mpl.use = lambda *a, **k: None
        plt = types.ModuleType("matplotlib.pyplot")
        plt.__getattr__ = lambda name: _Anything()
        plt.style = _Anything()
        plt.subplots = lambda *a, **k: (_Anything(), _Anything())
        mpl.pyplot = plt
        anim = types.ModuleType("matplotlib.animation")
        anim.__getattr__ = lambda name: _Anything()
        mpl.animation = anim
        sys.modules["matplotlib"] = mpl
        sys.modules["matplotlib.pyplot"] = plt
        sys.modules["matplotlib.animation"] = anim
        tk = types.ModuleType("mpl_toolkits")
        m3 = types.ModuleType("mpl_toolkits.mplot3d")
        ax3 = types.ModuleType("mpl_toolkits.mplot3d.axes3d")
        tk.mplot3d = m3
        m3.axes3d = ax3
        sys.modules["mpl_toolkits"] = tk
        sys.modules["mpl_toolkits.mplot3d"] = m3
        sys.modules["mpl_toolkits.mplot3d.axes3d"] = ax3
    if "numba" not in sys.modules or not getattr(sys.modules["numba"], "_fdtd_stub", False):
        nb = types.ModuleType("numba")
        nb._fdtd_stub = True

        def jit(*args, **kwargs):
            if len(args) == 1 and callable(args[0]) and not kwargs:
                return args[0]
            return lambda f: f

        nb.jit = jit
        nb.njit = jit
        nb.prange = range
        sys.modules["numba"] = nb


def load(relpath: str, name: str | None = None):
    """Load ``REF_ROOT/relpath`` as a module (its ``main()`` is not run)."""
    _install_stubs()
    path = os.path.join(REF_ROOT, relpath)
    name = name or "ref_" + relpath.replace("/", "_").replace(".py", "")
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    cwd = os.getcwd()
    try:
        # plt.style.use("../pyplot.mplstyle") is stubbed, cwd is irrelevant,
        # but scripts with module-level simulations write nothing either
        spec.loader.exec_module(mod)
    finally:
        os.chdir(cwd)
    return mod


def run_main_capture(relpath: str, hooks: tuple[str, ...]):
    """Run a program's main() and return the arguments its plot calls received.

    ``hooks`` names the module-level plotting functions to replace; each
    returns a list of the argument tuples it was called with.
    """
    mod = load(relpath)
    captured = {h: [] for h in hooks}
    for h in hooks:
        def _cap(*args, _h=h, **kw):
            captured[_h].append(tuple(a.copy() if hasattr(a, "copy") else a for a in args))
        setattr(mod, h, _cap)
    mod.main()
    return captured
