"""Electron-optics helpers on the host: wavelength, aberration symbols, spatial
frequencies and the aperture/aberration probe model used to seed reconstructions.

These mirror, in arithmetic and dtype, the reference's helpers:

* ``electron_wavelength_angstrom`` — ``py4DSTEM/process/utils/utils.py:90-97``
* ``polar_symbols`` / ``polar_aliases`` — ``py4DSTEM/process/phase/utils.py:29-43``
* ``spatial_frequencies`` — ``py4DSTEM/process/phase/utils.py:444-462``
* :class:`ComplexProbe` — ``py4DSTEM/process/phase/utils.py:50-441`` (aperture with
  cosine roll-off, aberration phase chi up to 5th order, corner-centred build)

The probe is built once per reconstruction on the host (it is not on the
per-position path), in complex64 like the reference.
"""

from __future__ import annotations

import math
from typing import Mapping, Tuple

import numpy as np

POLAR_SYMBOLS = (
    "C10", "C12", "phi12",
    "C21", "phi21", "C23", "phi23",
    "C30", "C32", "phi32", "C34", "phi34",
    "C41", "phi41", "C43", "phi43", "C45", "phi45",
    "C50", "C52", "phi52", "C54", "phi54", "C56", "phi56",
)

POLAR_ALIASES = {
    "defocus": "C10",
    "astigmatism": "C12",
    "astigmatism_angle": "phi12",
    "coma": "C21",
    "coma_angle": "phi21",
    "Cs": "C30",
    "C5": "C50",
}

# Physical constants with the precision the reference uses, so wavelengths agree
# to the last bit (``process/utils/utils.py:91-94``).
_ELECTRON_MASS = 9.109383e-31
_ELEMENTARY_CHARGE = 1.602177e-19
_SPEED_OF_LIGHT = 299792458
_PLANCK = 6.62607e-34


def electron_wavelength_angstrom(energy_ev: float) -> float:
    """Relativistic electron wavelength in Angstrom for a beam energy in eV."""
    m, e, c, h = _ELECTRON_MASS, _ELEMENTARY_CHARGE, _SPEED_OF_LIGHT, _PLANCK
    lam = (
        h
        / math.sqrt(2 * m * e * energy_ev)
        / math.sqrt(1 + e * energy_ev / 2 / m / c**2)
        * 10**10
    )
    return lam


def resolve_polar_parameters(parameters: Mapping[str, float], into: dict) -> dict:
    """Write aberration values into ``into`` (keyed by canonical symbol).

    ``defocus`` is stored as ``C10 = -defocus``; other aliases map directly
    (``phase_base_class.py:1788-1809``). Unknown keys raise ``ValueError``.
    """
    for symbol, value in parameters.items():
        if symbol in into:
            into[symbol] = value
        elif symbol == "defocus":
            into[POLAR_ALIASES[symbol]] = -value
        elif symbol in POLAR_ALIASES:
            into[POLAR_ALIASES[symbol]] = value
        else:
            raise ValueError("{} not a recognized parameter".format(symbol))
    return into


def spatial_frequencies(gpts: Tuple[int, int], sampling: Tuple[float, float]):
    """FFT frequencies (float32) of a grid with the given sampling."""
    return tuple(
        np.fft.fftfreq(int(n), d).astype(np.float32) for n, d in zip(gpts, sampling)
    )


class ComplexProbe:
    """Aperture-limited, aberrated electron probe on a corner-centred grid.

    Same parameterisation as the reference probe model: ``semiangle_cutoff`` and
    ``rolloff`` in mrad, aberrations in Angstrom/radians, or an explicit
    ``vacuum_probe_intensity`` aperture. ``build()`` evaluates the Fourier-space
    transfer function, inverse-transforms it and normalises to unit L2 norm.
    """

    def __init__(
        self,
        energy: float,
        gpts: Tuple[int, int],
        sampling: Tuple[float, float],
        semiangle_cutoff: float = np.inf,
        rolloff: float = 2.0,
        vacuum_probe_intensity: np.ndarray = None,
        focal_spread: float = 0.0,
        angular_spread: float = 0.0,
        gaussian_spread: float = 0.0,
        phase_shift: float = 0.0,
        parameters: Mapping[str, float] = None,
        **kwargs,
    ):
        for key in kwargs:
            if key not in POLAR_SYMBOLS and key not in POLAR_ALIASES:
                raise ValueError("{} not a recognized parameter".format(key))
        self._vacuum_probe_intensity = vacuum_probe_intensity
        self._semiangle_cutoff = semiangle_cutoff
        self._rolloff = rolloff
        self._focal_spread = focal_spread
        self._angular_spread = angular_spread
        self._gaussian_spread = gaussian_spread
        self._phase_shift = phase_shift
        self._energy = energy
        self._wavelength = electron_wavelength_angstrom(energy)
        self._gpts = tuple(int(g) for g in gpts)
        self._sampling = tuple(sampling)
        self._parameters = dict(zip(POLAR_SYMBOLS, [0.0] * len(POLAR_SYMBOLS)))
        params = dict(parameters or {})
        params.update(kwargs)
        resolve_polar_parameters(params, self._parameters)

    # -- Fourier-space factors -------------------------------------------------
    def _aperture(self, alpha):
        cutoff = self._semiangle_cutoff / 1000
        if self._vacuum_probe_intensity is not None:
            vpi = np.asarray(self._vacuum_probe_intensity, dtype=np.float32)
            return np.sqrt(np.maximum(vpi, 0))
        if self._semiangle_cutoff == np.inf:
            return np.ones_like(alpha)
        if self._rolloff > 0.0:
            roll = self._rolloff / 1000.0
            taper = 0.5 * (1 + np.cos(np.pi * (alpha - cutoff + roll) / roll))
            taper[alpha > cutoff] = 0.0
            return np.where(alpha > cutoff - roll, taper,
                            np.ones_like(alpha, dtype=np.float32))
        return np.array(alpha < cutoff).astype(np.float32)

    def _chi(self, alpha, phi):
        """Aberration phase (radians), accumulated order by order in float32."""
        p = self._parameters
        alpha2 = alpha**2
        alpha = np.array(alpha)
        chi = np.zeros(alpha.shape, dtype=np.float32)

        def active(*names):
            return any(p[n] != 0.0 for n in names)

        if active("C10", "C12", "phi12"):
            chi += 1 / 2 * alpha2 * (p["C10"] + p["C12"] * np.cos(2 * (phi - p["phi12"])))
        if active("C21", "phi21", "C23", "phi23"):
            chi += 1 / 3 * alpha2 * alpha * (
                p["C21"] * np.cos(phi - p["phi21"]) + p["C23"] * np.cos(3 * (phi - p["phi23"]))
            )
        if active("C30", "C32", "phi32", "C34", "phi34"):
            chi += 1 / 4 * alpha2**2 * (
                p["C30"]
                + p["C32"] * np.cos(2 * (phi - p["phi32"]))
                + p["C34"] * np.cos(4 * (phi - p["phi34"]))
            )
        # The reference tests "phi41" twice and never "phi45" (utils.py:364-369);
        # the same activation rule is kept so probes agree bit for bit.
        if active("C41", "phi41", "C43", "phi43", "C45", "phi41"):
            chi += 1 / 5 * alpha2**2 * alpha * (
                p["C41"] * np.cos(phi - p["phi41"])
                + p["C43"] * np.cos(3 * (phi - p["phi43"]))
                + p["C45"] * np.cos(5 * (phi - p["phi45"]))
            )
        if active("C50", "C52", "phi52", "C54", "phi54", "C56", "phi56"):
            chi += 1 / 6 * alpha2**3 * (
                p["C50"]
                + p["C52"] * np.cos(2 * (phi - p["phi52"]))
                + p["C54"] * np.cos(4 * (phi - p["phi54"]))
                + p["C56"] * np.cos(6 * (phi - p["phi56"]))
            )
        return 2 * np.pi / self._wavelength * chi + self._phase_shift

    def _temporal_envelope(self, alpha):
        return np.exp(
            -((0.5 * np.pi / self._wavelength * self._focal_spread * alpha**2) ** 2)
        ).astype(np.float32)

    def _gaussian_envelope(self, alpha):
        return np.exp(-0.5 * self._gaussian_spread**2 * alpha**2 / self._wavelength**2)

    def _spatial_envelope(self, alpha, phi):
        p = self._parameters
        k = 2 * np.pi / self._wavelength
        c = np.cos
        s = np.sin
        dchi_dk = k * (
            (p["C12"] * c(2.0 * (phi - p["phi12"])) + p["C10"]) * alpha
            + (p["C23"] * c(3.0 * (phi - p["phi23"])) + p["C21"] * c(1.0 * (phi - p["phi21"])))
            * alpha**2
            + (p["C34"] * c(4.0 * (phi - p["phi34"])) + p["C32"] * c(2.0 * (phi - p["phi32"])) + p["C30"])
            * alpha**3
            + (
                p["C45"] * c(5.0 * (phi - p["phi45"]))
                + p["C43"] * c(3.0 * (phi - p["phi43"]))
                + p["C41"] * c(1.0 * (phi - p["phi41"]))
            )
            * alpha**4
            + (
                p["C56"] * c(6.0 * (phi - p["phi56"]))
                + p["C54"] * c(4.0 * (phi - p["phi54"]))
                + p["C52"] * c(2.0 * (phi - p["phi52"]))
                + p["C50"]
            )
            * alpha**5
        )
        dchi_dphi = -k * (
            1 / 2.0 * (2.0 * p["C12"] * s(2.0 * (phi - p["phi12"]))) * alpha
            + 1 / 3.0 * (3.0 * p["C23"] * s(3.0 * (phi - p["phi23"])) + 1.0 * p["C21"] * s(1.0 * (phi - p["phi21"])))
            * alpha**2
            + 1 / 4.0 * (4.0 * p["C34"] * s(4.0 * (phi - p["phi34"])) + 2.0 * p["C32"] * s(2.0 * (phi - p["phi32"])))
            * alpha**3
            + 1 / 5.0
            * (
                5.0 * p["C45"] * s(5.0 * (phi - p["phi45"]))
                + 3.0 * p["C43"] * s(3.0 * (phi - p["phi43"]))
                + 1.0 * p["C41"] * s(1.0 * (phi - p["phi41"]))
            )
            * alpha**4
            + 1 / 6.0
            * (
                6.0 * p["C56"] * s(6.0 * (phi - p["phi56"]))
                + 4.0 * p["C54"] * s(4.0 * (phi - p["phi54"]))
                + 2.0 * p["C52"] * s(2.0 * (phi - p["phi52"]))
            )
            * alpha**5
        )
        return np.exp(
            -np.sign(self._angular_spread)
            * (self._angular_spread / 2 / 1000) ** 2
            * (dchi_dk**2 + dchi_dphi**2)
        )

    def scattering_angles(self):
        kx, ky = spatial_frequencies(self._gpts, self._sampling)
        x = kx * self._wavelength
        y = ky * self._wavelength
        alpha = np.sqrt(x[:, None] ** 2 + y[None, :] ** 2)
        phi = np.arctan2(y[None, :], x[:, None])
        return alpha, phi

    def evaluate_ctf(self):
        """Fourier-space probe (complex64): aberrations x aperture x envelopes."""
        alpha, phi = self.scattering_angles()
        array = np.exp(-1.0j * self._chi(alpha, phi))
        if self._semiangle_cutoff < np.inf or self._vacuum_probe_intensity is not None:
            array *= self._aperture(alpha)
        if self._focal_spread > 0.0:
            array *= self._temporal_envelope(alpha)
        if self._angular_spread > 0.0:
            array *= self._spatial_envelope(alpha, phi)
        if self._gaussian_spread > 0.0:
            array *= self._gaussian_envelope(alpha)
        return array

    def build(self):
        """Real-space, corner-centred probe with unit L2 norm (complex64)."""
        array = np.fft.ifft2(self.evaluate_ctf())
        array = array / np.sqrt((np.abs(array) ** 2).sum())
        self._array = array
        return self
