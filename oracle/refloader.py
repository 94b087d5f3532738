"""Loader that imports the unmodified py4DSTEM 0.14.18 ptychography classes from a
source checkout, for use as a parity oracle.

TEST INFRASTRUCTURE ONLY. Nothing in the product package imports this module.
It is used by ``tests/golden/make_golden.py`` (which writes the committed golden
fixtures) and by CPU tests that pin ``oracle/ptycho_np.py`` against the reference's
own code. The source checkout only exists in the build container; every caller
must handle :class:`ReferenceUnavailable`.

The reference cannot be pip-installed here: ``emdfile``, ``pylops``, ``h5py``,
``matplotlib`` and ``skimage`` are absent and ``setup.py:26`` pins ``numpy<2``. The
ptychography path only *imports* those packages (for plotting, HDF5 I/O and the
off-by-default TV constraint); its arithmetic is plain NumPy/SciPy. So this loader:

1. installs a meta-path finder that hands out ``MagicMock`` modules for
   matplotlib, mpl_toolkits, pylops, skimage, h5py and ``py4DSTEM.visualize*``;
2. provides a minimal ``emdfile`` with a ``Custom`` base class and ``tqdmnd``
   (the only two names the hot path uses: ``singleslice_ptychography.py:18,142,847``);
3. registers the ``py4DSTEM`` packages with ``__path__`` pointing into the checkout
   *without running their ``__init__``* (those pull in every subsystem), and
   re-exports the handful of helpers the phase modules import from package level
   (``process/utils/__init__.py:1-15``, ``process/calibration/__init__.py:2``);
4. never writes bytecode into the read-only checkout.
"""

from __future__ import annotations

import importlib
import importlib.abc
import importlib.machinery
import itertools
import os
import sys
import types
from unittest import mock

import numpy as np

# The checkout's location comes from the caller or from this variable; nothing
# in this module assumes a path.
REFERENCE_ENV = "PY4DSTEM_REFERENCE"

_MOCKED_PREFIXES = (
    "matplotlib",
    "mpl_toolkits",
    "pylops",
    "skimage",
    "h5py",
    "py4DSTEM.visualize",
    "colorspacious",
    "dill",
)


class ReferenceUnavailable(RuntimeError):
    """The py4DSTEM source checkout is not present on this machine."""


class _MockLoader(importlib.abc.Loader):
    def create_module(self, spec):
        module = mock.MagicMock(name=spec.name)
        module.__name__ = spec.name
        module.__path__ = []
        module.__spec__ = spec
        return module

    def exec_module(self, module):
        return None


class _MockFinder(importlib.abc.MetaPathFinder):
    def find_spec(self, fullname, path=None, target=None):
        for prefix in _MOCKED_PREFIXES:
            if fullname == prefix or fullname.startswith(prefix + "."):
                return importlib.machinery.ModuleSpec(
                    fullname, _MockLoader(), is_package=True
                )
        return None


class _Custom:
    """Stand-in for ``emdfile.Custom``: only the constructor is used on the path."""

    def __init__(self, name=None, *args, **kwargs):
        self.name = name


def _tqdmnd(*args, **kwargs):
    """Stand-in for ``emdfile.tqdmnd`` (progress bar over an N-d index range)."""
    ranges = [range(a) if isinstance(a, (int, np.integer)) else a for a in args]
    if len(ranges) == 1:
        return iter(ranges[0])
    return itertools.product(*ranges)


def _make_emdfile():
    mod = types.ModuleType("emdfile")
    mod.Custom = _Custom
    mod.tqdmnd = _tqdmnd

    def __getattr__(name):  # Array, Metadata, PointListArray, _read_metadata, ...
        value = mock.MagicMock(name=f"emdfile.{name}")
        setattr(mod, name, value)
        return value

    mod.__getattr__ = __getattr__
    return mod


class DataCube:
    """Duck-typed stand-in for ``py4DSTEM.datacube.DataCube`` as the phase classes
    read it (``phase_base_class.py:485-611``): ``.data`` (Rx,Ry,Qx,Qy), ``.shape``,
    ``.Rshape`` and ``.calibration.get_{R,Q}_pixel_{size,units}()``."""

    def __init__(self, data, r_pixel_size=1.0, r_pixel_units="A",
                 q_pixel_size=1.0, q_pixel_units="mrad"):
        self.data = data
        self.calibration = _Calibration(r_pixel_size, r_pixel_units,
                                        q_pixel_size, q_pixel_units)

    @property
    def shape(self):
        return self.data.shape

    @property
    def Rshape(self):
        return self.data.shape[:2]

    # the diffraction-space reshaping the phase classes call in preprocess()
    # (phase_base_class.py:280-420) runs the reference's own functions
    # (py4DSTEM/preprocess/preprocess.py) on this object
    R_Nx = property(lambda self: self.data.shape[0])
    R_Ny = property(lambda self: self.data.shape[1])
    Q_Nx = property(lambda self: self.data.shape[2])
    Q_Ny = property(lambda self: self.data.shape[3])
    R_N = property(lambda self: self.data.shape[0] * self.data.shape[1])
    Qshape = property(lambda self: self.data.shape[2:])

    def set_dim(self, *args, **kwargs):
        pass

    def calibrate(self):
        pass

    def bin_Q(self, N, dtype=None):
        from py4DSTEM.preprocess.preprocess import bin_data_diffraction

        return bin_data_diffraction(self, N, dtype)

    def pad_Q(self, N=None, output_size=None):
        from py4DSTEM.preprocess.preprocess import pad_data_diffraction

        return pad_data_diffraction(self, pad_factor=N, output_size=output_size)

    def resample_Q(self, N=None, output_size=None, method="bilinear",
                   conserve_array_sums=False):
        from py4DSTEM.preprocess.preprocess import resample_data_diffraction

        return resample_data_diffraction(self, resampling_factor=N, output_size=output_size,
                                         method=method,
                                         conserve_array_sums=conserve_array_sums)


class _Calibration:
    def __init__(self, r_size, r_units, q_size, q_units):
        self._r = (r_size, r_units)
        self._q = (q_size, q_units)

    def get_R_pixel_size(self):
        return self._r[0]

    def get_R_pixel_units(self):
        return self._r[1]

    def get_Q_pixel_size(self):
        return self._q[0]

    def get_Q_pixel_units(self):
        return self._q[1]

    def set_Q_pixel_size(self, size):
        self._q = (size, self._q[1])


def _package(name, path):
    mod = types.ModuleType(name)
    mod.__path__ = [path]
    mod.__package__ = name
    mod.__spec__ = importlib.machinery.ModuleSpec(name, None, is_package=True)
    mod.__spec__.submodule_search_locations = [path]
    sys.modules[name] = mod
    return mod


def _reexport(target, source_name):
    source = importlib.import_module(source_name)
    for key, value in vars(source).items():
        if not key.startswith("__"):
            setattr(target, key, value)


_LOADED = {}


def load_reference(root: str | None = None):
    """Import the reference phase classes and return them in a namespace.

    Returns an object with attributes ``SingleslicePtychography``,
    ``MultislicePtychography``, ``MixedstatePtychography``,
    ``MixedstateMultislicePtychography``, ``PtychographicTomography``, ``DataCube`` (the
    duck type above), ``utils`` (``process/phase/utils.py``) and ``root``.
    """
    root = root or os.environ.get(REFERENCE_ENV)
    if not root:
        raise ReferenceUnavailable(
            f"no py4DSTEM source checkout given: pass root= or set {REFERENCE_ENV}")
    if root in _LOADED:
        return _LOADED[root]
    pkg_root = os.path.join(root, "py4DSTEM")
    if not os.path.isfile(os.path.join(pkg_root, "process", "phase",
                                       "singleslice_ptychography.py")):
        raise ReferenceUnavailable(f"py4DSTEM sources not found under {root}")

    sys.dont_write_bytecode = True
    if not any(isinstance(f, _MockFinder) for f in sys.meta_path):
        sys.meta_path.insert(0, _MockFinder())
    sys.modules.setdefault("emdfile", _make_emdfile())

    top = _package("py4DSTEM", pkg_root)
    top.is_package_lite = True
    top._TESTPATH = ""

    datacube_mod = types.ModuleType("py4DSTEM.datacube")
    datacube_mod.DataCube = DataCube
    sys.modules["py4DSTEM.datacube"] = datacube_mod
    top.datacube = datacube_mod
    top.DataCube = DataCube

    data_mod = types.ModuleType("py4DSTEM.data")
    data_mod.__getattr__ = lambda name: mock.MagicMock(name=f"py4DSTEM.data.{name}")
    sys.modules["py4DSTEM.data"] = data_mod
    top.data = data_mod

    process = _package("py4DSTEM.process", os.path.join(pkg_root, "process"))
    preprocess = _package("py4DSTEM.preprocess", os.path.join(pkg_root, "preprocess"))
    _reexport(preprocess, "py4DSTEM.preprocess.utils")

    putils = _package("py4DSTEM.process.utils",
                      os.path.join(pkg_root, "process", "utils"))
    _reexport(putils, "py4DSTEM.process.utils.utils")
    _reexport(putils, "py4DSTEM.process.utils.multicorr")
    _reexport(putils, "py4DSTEM.process.utils.cross_correlate")
    for name in ("bin2D", "get_maxima_2D", "get_shifted_ar", "filter_2D_maxima",
                 "linear_interpolation_2D"):
        setattr(putils, name, getattr(preprocess, name))

    fit = _package("py4DSTEM.process.fit", os.path.join(pkg_root, "process", "fit"))
    _reexport(fit, "py4DSTEM.process.fit.fit")

    _package("py4DSTEM.process.phase", os.path.join(pkg_root, "process", "phase"))
    calib = _package("py4DSTEM.process.calibration",
                     os.path.join(pkg_root, "process", "calibration"))
    _reexport(calib, "py4DSTEM.process.calibration.origin")
    process.utils = putils
    process.calibration = calib

    single = importlib.import_module(
        "py4DSTEM.process.phase.singleslice_ptychography")
    multi = importlib.import_module("py4DSTEM.process.phase.multislice_ptychography")
    mixed = importlib.import_module("py4DSTEM.process.phase.mixedstate_ptychography")
    mixed_multi = importlib.import_module(
        "py4DSTEM.process.phase.mixedstate_multislice_ptychography")
    tomo = importlib.import_module("py4DSTEM.process.phase.ptychographic_tomography")
    phase_utils = importlib.import_module("py4DSTEM.process.phase.utils")

    ns = types.SimpleNamespace(
        SingleslicePtychography=single.SingleslicePtychography,
        MultislicePtychography=multi.MultislicePtychography,
        MixedstatePtychography=mixed.MixedstatePtychography,
        MixedstateMultislicePtychography=mixed_multi.MixedstateMultislicePtychography,
        PtychographicTomography=tomo.PtychographicTomography,
        DataCube=DataCube,
        utils=phase_utils,
        root=root,
    )
    _LOADED[root] = ns
    return ns
