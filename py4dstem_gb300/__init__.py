"""GB300-native (sm_103a) iterative ptychography: a drop-in for the per-position
forward/adjoint loop of py4DSTEM's SingleslicePtychography,
MultislicePtychography, MixedstatePtychography,
MixedstateMultislicePtychography and PtychographicTomography.

Host code (this package) keeps the reference's Python API and preprocessing;
the reconstruction loop runs in libptycho_gb300.so (csrc/, C ABI in
include/ptycho_gb300.h).
"""

from .datacube import Calibration, DataCube
from .optics import ComplexProbe, electron_wavelength_angstrom
from .io import read, save
from .ptychography import (MixedstateMultislicePtychography, MixedstatePtychography,
                           MultislicePtychography, SingleslicePtychography)
from .tomography import PtychographicTomography

__all__ = [
    "Calibration",
    "ComplexProbe",
    "DataCube",
    "MixedstateMultislicePtychography",
    "MixedstatePtychography",
    "MultislicePtychography",
    "PtychographicTomography",
    "SingleslicePtychography",
    "electron_wavelength_angstrom",
    "read",
    "save",
]

__version__ = "0.1.0"
