"""Minimal 4D-STEM datacube container accepted by the reconstruction classes.

The reconstruction classes read only ``.data`` (Rx, Ry, Qx, Qy), ``.shape``,
``.Rshape`` and ``.calibration.get_{R,Q}_pixel_{size,units}()``
(``py4DSTEM/process/phase/phase_base_class.py:485-611``), so a real
``py4DSTEM.DataCube`` works unchanged. This class is the same duck type for
callers that do not have py4DSTEM installed.
"""

from __future__ import annotations

import numpy as np


class Calibration:
    """Real-space (R) and reciprocal-space (Q) pixel sizes and units."""

    def __init__(self, r_pixel_size=1.0, r_pixel_units="pixels",
                 q_pixel_size=1.0, q_pixel_units="pixels"):
        self._r_size = r_pixel_size
        self._r_units = r_pixel_units
        self._q_size = q_pixel_size
        self._q_units = q_pixel_units

    def get_R_pixel_size(self):
        return self._r_size

    def get_R_pixel_units(self):
        return self._r_units

    def get_Q_pixel_size(self):
        return self._q_size

    def get_Q_pixel_units(self):
        return self._q_units

    def set_R_pixel_size(self, value):
        self._r_size = value

    def set_R_pixel_units(self, value):
        self._r_units = value

    def set_Q_pixel_size(self, value):
        self._q_size = value

    def set_Q_pixel_units(self, value):
        self._q_units = value


class DataCube:
    """4D array of diffraction intensities with its calibration."""

    def __init__(self, data, calibration: Calibration | None = None, **calib):
        self.data = data
        self.calibration = calibration if calibration is not None else Calibration(**calib)

    @property
    def shape(self):
        return self.data.shape

    @property
    def Rshape(self):
        return self.data.shape[:2]

    @property
    def Qshape(self):
        return self.data.shape[2:]

    def copy(self):
        return DataCube(np.array(self.data, copy=True), self.calibration)
