"""Seeded synthetic ptychography datasets with the shapes of the benchmark workloads.

No public dataset is used. Each workload is generated from a fixed seed:

* object phase = Gaussian atoms (sigma 0.4 A, peak 0.3 rad) on a square lattice
  with a random rotation and offset, plus a Gaussian-smoothed (sigma 4 px)
  N(0, 0.05) rad field; amplitude = exp(-0.1 * phase);
* probe = aperture-limited, defocused probe (:class:`optics.ComplexProbe`);
* raster scan with uniform position jitter;
* diffraction intensities = the ptychographic forward model (sub-pixel Fourier
  shift of the probe, periodic object patch, optional multislice propagation or
  incoherent probe modes, far-field |FFT|^2), scaled to a dose per pattern and
  drawn from a Poisson distribution, stored detector-centred as float32.

The numpy backend (complex128) serves the small parity cases; the torch backend
(complex64 on a CUDA device) generates the large throughput cases quickly. Both
produce a :class:`ScanCase` whose ``datacube`` lives in host memory.
"""

from __future__ import annotations

import dataclasses
import math
from typing import Optional, Sequence

import numpy as np
from scipy.ndimage import gaussian_filter

from .datacube import DataCube
from .optics import ComplexProbe, electron_wavelength_angstrom


@dataclasses.dataclass
class ScanCase:
    """A generated dataset plus the arguments that reconstruct it."""

    name: str
    datacube: DataCube
    scan_positions_ang: np.ndarray
    true_object: np.ndarray
    sampling: float
    ctor_kwargs: dict
    preprocess_kwargs: dict
    reconstruct_kwargs: dict
    probe_modes: Optional[np.ndarray] = None

    @property
    def num_positions(self):
        return int(self.scan_positions_ang.shape[0])


def atom_lattice_phase(shape, sampling, lattice_a, rng, sigma_ang=0.4, peak_rad=0.3):
    """Sum of Gaussian atoms on a randomly rotated, randomly offset square lattice."""
    nx, ny = shape
    theta = rng.uniform(0.0, np.pi / 2)
    offset = rng.uniform(0.0, lattice_a, size=2)
    extent = max(nx, ny) * sampling
    n_cells = int(math.ceil(extent * 1.5 / lattice_a)) + 2
    idx = np.arange(-n_cells, n_cells + 1)
    gi, gj = np.meshgrid(idx, idx, indexing="ij")
    u = gi.ravel() * lattice_a + offset[0]
    v = gj.ravel() * lattice_a + offset[1]
    c, s = np.cos(theta), np.sin(theta)
    cx = nx * sampling / 2
    cy = ny * sampling / 2
    ax = c * u - s * v + cx
    ay = s * u + c * v + cy
    margin = 5 * sigma_ang
    keep = (ax > -margin) & (ax < nx * sampling + margin) & (ay > -margin) & (
        ay < ny * sampling + margin)
    ax, ay = ax[keep], ay[keep]

    phase = np.zeros(shape, dtype=np.float64)
    half = int(math.ceil(4 * sigma_ang / sampling)) + 1
    win = np.arange(-half, half + 1)
    inv2s2 = 1.0 / (2 * sigma_ang**2)
    for x0, y0 in zip(ax, ay):
        px = int(round(x0 / sampling))
        py = int(round(y0 / sampling))
        xs = px + win
        ys = py + win
        dx = xs * sampling - x0
        dy = ys * sampling - y0
        g = peak_rad * np.exp(-(dx[:, None] ** 2 + dy[None, :] ** 2) * inv2s2)
        mx = (xs >= 0) & (xs < nx)
        my = (ys >= 0) & (ys < ny)
        phase[np.ix_(xs[mx], ys[my])] += g[np.ix_(mx, my)]
    return phase


def portable_normal(rng, size):
    """Standard normal variates by Box-Muller from the generator's uniform
    doubles, which every NumPy version and CPU draws identically from the same
    PCG64 state (unlike Generator.normal / Generator.poisson, whose algorithms
    and rounding may differ between NumPy versions and CPUs)."""
    n = int(np.prod(size))
    u = rng.random(2 * ((n + 1) // 2)).reshape(2, -1)
    r = np.sqrt(-2.0 * np.log1p(-u[0]))
    z = np.concatenate([r * np.cos(2 * np.pi * u[1]), r * np.sin(2 * np.pi * u[1])])
    return z[:n].reshape(size)


def portable_poisson(lam, rng):
    """Poisson counts by inversion of the cumulative distribution (SciPy's
    pdtr) against the generator's uniform doubles: the smallest k with
    u <= P(X <= k). A count changes between machines only when a uniform falls
    within rounding (~1e-15) of a cumulative probability, so the counts agree
    across CPUs and library versions with near certainty."""
    from scipy.special import ndtri, pdtr

    lam = np.asarray(lam, dtype=np.float64)
    flat = lam.ravel()
    u = rng.random(flat.size)
    k = np.zeros(flat.size)
    # k = 0 where u <= P(X = 0) = exp(-lambda) (most dark-field pixels)
    rest = np.nonzero(u > np.exp(-flat))[0]
    lr, ur = flat[rest], u[rest]
    # a starting guess from the normal approximation, then exact corrections
    kr = np.maximum(1.0, np.floor(lr + np.sqrt(lr) * ndtri(ur) + 0.5))
    act = np.nonzero(ur > pdtr(kr, lr))[0]
    while act.size:  # too small: step up
        kr[act] += 1
        act = act[ur[act] > pdtr(kr[act], lr[act])]
    act = np.nonzero((kr >= 2) & (ur <= pdtr(kr - 1, lr)))[0]
    while act.size:  # too large: step down (k >= 1 holds: u > P(X = 0))
        kr[act] -= 1
        act = act[(kr[act] >= 2) & (ur[act] <= pdtr(kr[act] - 1, lr[act]))]
    k[rest] = kr
    return k.astype(np.int64).reshape(lam.shape)


def random_object(shape, sampling, rng, lattice_a=3.9, noise_std=0.05, smooth_px=4.0,
                  sigma_ang=0.4, peak_rad=0.3, portable=False):
    """Complex transmission function exp(-0.1 phi) exp(i phi) (complex128)."""
    phase = atom_lattice_phase(shape, sampling, lattice_a, rng, sigma_ang, peak_rad)
    noise = (noise_std * portable_normal(rng, shape) if portable
             else rng.normal(0.0, noise_std, size=shape))
    phase += gaussian_filter(noise, smooth_px)
    return np.exp(-0.1 * phase) * np.exp(1j * phase)


def raster_positions(nx, ny, step, jitter, rng):
    """(nx*ny, 2) raster positions in Angstrom with uniform +-jitter."""
    x = np.arange(nx) * step
    y = np.arange(ny) * step
    xx, yy = np.meshgrid(x, y, indexing="ij")
    pos = np.stack((xx.ravel(), yy.ravel()), axis=-1).astype(np.float64)
    pos += rng.uniform(-jitter, jitter, size=pos.shape)
    return pos


def positions_in_pixels(positions_ang, sampling, roi_shape, object_shape):
    """Pixel positions as the reconstruction will place them: shifted positive,
    divided by the sampling, padded by half the ROI, then centred in the object
    (``phase_base_class.py:1811-1903``, ``singleslice_ptychography.py:467-473``)."""
    pos = np.array(positions_ang, dtype=np.float64)
    pos -= np.min(pos, axis=0).clip(-np.inf, 0)
    pos /= sampling
    pos += np.asarray(roi_shape, dtype=np.float64) / 2
    pos -= pos.mean(0) - np.asarray(object_shape, dtype=np.float64) / 2
    return pos


def _probe_float64(gpts, sampling, energy, semiangle_mrad, rolloff_mrad, defocus,
                   astigmatism=0.0, astigmatism_angle=0.0):
    """The same probe model as optics.ComplexProbe (soft aperture, defocus and
    two-fold astigmatism), evaluated in float64 from end to end: the portable
    generator's intensities must not depend on the platform's float32 math
    library, whose last-bit differences move a Poisson draw now and then."""
    lam = electron_wavelength_angstrom(energy)
    kx = np.fft.fftfreq(int(gpts[0]), sampling)
    ky = np.fft.fftfreq(int(gpts[1]), sampling)
    x = kx * lam
    y = ky * lam
    alpha = np.sqrt(x[:, None] ** 2 + y[None, :] ** 2)
    phi = np.arctan2(y[None, :], x[:, None])
    c10 = -defocus
    chi = 0.5 * alpha ** 2 * (c10 + astigmatism * np.cos(2 * (phi - astigmatism_angle)))
    chi = 2 * np.pi / lam * chi
    cutoff = semiangle_mrad / 1000.0
    roll = rolloff_mrad / 1000.0
    taper = 0.5 * (1 + np.cos(np.pi * (alpha - cutoff + roll) / roll))
    aperture = np.where(alpha > cutoff - roll, np.where(alpha > cutoff, 0.0, taper), 1.0)
    array = np.fft.ifft2(np.exp(-1.0j * chi) * aperture)
    return array / np.sqrt((np.abs(array) ** 2).sum())


def _fresnel(gpts, sampling, wavelength, dz):
    kx = np.fft.fftfreq(gpts[0], sampling)
    ky = np.fft.fftfreq(gpts[1], sampling)
    return np.exp(-1j * np.pi * wavelength * dz * (kx[:, None] ** 2 + ky[None, :] ** 2))


def _simulate_numpy(objects, probes, weights, positions_px, propagators, dose, rng,
                    batch=256, portable=False):
    """Far-field intensities, (J, Sx, Sy) float32, detector-centred, Poisson noise."""
    T = objects.shape[0]
    M, sx, sy = probes.shape
    px, py = objects.shape[-2:]
    J = positions_px.shape[0]
    kx = np.fft.fftfreq(sx)
    ky = np.fft.fftfreq(sy)
    fx = np.fft.fftfreq(sx, 1 / sx).astype(int)
    fy = np.fft.fftfreq(sy, 1 / sy).astype(int)
    probes_f = np.fft.fft2(probes)
    out = np.empty((J, sx, sy), dtype=np.float32)
    for start in range(0, J, batch):
        pos = positions_px[start:start + batch]
        r = np.round(pos)
        frac = pos - r
        rows = (r[:, 0].astype(int)[:, None] + fx[None, :]) % px
        cols = (r[:, 1].astype(int)[:, None] + fy[None, :]) % py
        ramp = np.exp(-2j * np.pi * kx[None, :, None] * frac[:, 0, None, None]) * np.exp(
            -2j * np.pi * ky[None, None, :] * frac[:, 1, None, None])
        intensity = np.zeros((pos.shape[0], sx, sy))
        for m in range(M):
            wave = np.fft.ifft2(probes_f[m][None] * ramp)
            for s in range(T):
                patch = objects[s][rows[:, :, None], cols[:, None, :]]
                wave = wave * patch
                if s + 1 < T:
                    wave = np.fft.ifft2(np.fft.fft2(wave) * propagators[s])
            intensity += weights[m] * np.abs(np.fft.fft2(wave)) ** 2
        intensity *= dose / intensity.sum(axis=(-2, -1), keepdims=True)
        counts = (portable_poisson(intensity, rng) if portable
                  else rng.poisson(intensity)).astype(np.float32)
        out[start:start + batch] = np.fft.fftshift(counts, axes=(-2, -1))
    return out


def _simulate_torch(objects, probes, weights, positions_px, propagators, dose, seed,
                    device, batch=512):
    import torch

    dev = torch.device(device)
    gen = torch.Generator(device=dev)
    gen.manual_seed(int(seed))
    T = objects.shape[0]
    M, sx, sy = probes.shape
    px, py = objects.shape[-2:]
    J = positions_px.shape[0]
    obj = torch.as_tensor(objects.astype(np.complex64), device=dev)
    prf = torch.fft.fft2(torch.as_tensor(probes.astype(np.complex64), device=dev))
    props = (torch.as_tensor(np.asarray(propagators).astype(np.complex64), device=dev)
             if T > 1 else None)
    kx = torch.as_tensor(np.fft.fftfreq(sx), device=dev, dtype=torch.float64)
    ky = torch.as_tensor(np.fft.fftfreq(sy), device=dev, dtype=torch.float64)
    fx = torch.as_tensor(np.fft.fftfreq(sx, 1 / sx).astype(np.int64), device=dev)
    fy = torch.as_tensor(np.fft.fftfreq(sy, 1 / sy).astype(np.int64), device=dev)
    pos_all = torch.as_tensor(positions_px, device=dev, dtype=torch.float64)
    out = np.empty((J, sx, sy), dtype=np.float32)
    for start in range(0, J, batch):
        pos = pos_all[start:start + batch]
        r = torch.round(pos)
        frac = pos - r
        rows = (r[:, 0].long()[:, None] + fx[None, :]) % px
        cols = (r[:, 1].long()[:, None] + fy[None, :]) % py
        ramp = (torch.exp(-2j * math.pi * kx[None, :, None] * frac[:, 0, None, None])
                * torch.exp(-2j * math.pi * ky[None, None, :] * frac[:, 1, None, None])
                ).to(torch.complex64)
        intensity = torch.zeros((pos.shape[0], sx, sy), device=dev, dtype=torch.float32)
        for m in range(M):
            wave = torch.fft.ifft2(prf[m][None] * ramp)
            for s in range(T):
                patch = obj[s][rows[:, :, None], cols[:, None, :]]
                wave = wave * patch
                if s + 1 < T:
                    wave = torch.fft.ifft2(torch.fft.fft2(wave) * props[s])
            intensity += float(weights[m]) * torch.abs(torch.fft.fft2(wave)) ** 2
        intensity *= dose / intensity.sum(dim=(-2, -1), keepdim=True)
        counts = torch.poisson(intensity, generator=gen)
        out[start:start + batch] = torch.fft.fftshift(counts, dim=(-2, -1)).cpu().numpy()
    return out


def make_scan(
    name: str,
    seed: int,
    scan_shape: Sequence[int],
    step_ang: float,
    jitter_ang: float,
    detector: int,
    object_px: int,
    sampling: float = 0.25,
    energy: float = 300e3,
    semiangle: float = 20.0,
    defocus: float = 100.0,
    dose: float = 1e4,
    num_slices: int = 1,
    slice_thickness: float = 20.0,
    num_modes: int = 1,
    mode_weights: Sequence[float] = (1.0,),
    lattice_a: float = 3.9,
    backend: str = "numpy",
    device: str = "cuda",
) -> ScanCase:
    """Generate one seeded scan (see module docstring for the model).

    backend: "numpy" (complex128 model, NumPy's Poisson and normal samplers),
    "portable" (the same model with every random variate drawn from the
    generator's uniform doubles, so that the counts agree across CPUs and NumPy
    versions: the reference fixtures at the timed sizes are regenerated from
    their seed instead of stored), or "torch" (complex64 on a CUDA device)."""
    rng = np.random.default_rng(seed)
    roi = (detector, detector)
    obj_shape = (object_px, object_px)
    portable = backend == "portable"
    objects = np.stack([random_object(obj_shape, sampling, rng, lattice_a=lattice_a,
                                      portable=portable)
                        for _ in range(num_slices)])
    pos_ang = raster_positions(scan_shape[0], scan_shape[1], step_ang, jitter_ang, rng)
    pos_px = positions_in_pixels(pos_ang, sampling, roi, obj_shape)
    wavelength = electron_wavelength_angstrom(energy)

    if portable:
        base = _probe_float64(roi, sampling, energy, semiangle, 2.0, defocus)
    else:
        base = ComplexProbe(energy=energy, gpts=roi, sampling=(sampling, sampling),
                            semiangle_cutoff=semiangle, rolloff=2.0,
                            parameters={"defocus": defocus}).build()._array
    probes = [base.astype(np.complex128)]
    for m in range(1, num_modes):
        if portable:
            z = portable_normal(rng, 2)
            probes.append(_probe_float64(roi, sampling, energy, semiangle, 2.0,
                                         defocus + 20.0 * z[0], abs(10.0 * z[1]),
                                         rng.uniform(0, np.pi)))
            continue
        perturb = {
            "defocus": defocus + rng.normal(0.0, 20.0),
            "astigmatism": abs(rng.normal(0.0, 10.0)),
            "astigmatism_angle": rng.uniform(0, np.pi),
        }
        pm = ComplexProbe(energy=energy, gpts=roi, sampling=(sampling, sampling),
                          semiangle_cutoff=semiangle, rolloff=2.0,
                          parameters=perturb).build()._array
        probes.append(pm.astype(np.complex128))
    probes = np.stack(probes)
    weights = np.asarray(mode_weights[:num_modes], dtype=np.float64)
    weights = weights / weights.sum()
    propagators = [_fresnel(roi, sampling, wavelength, slice_thickness)
                   for _ in range(num_slices - 1)]

    if backend in ("numpy", "portable"):
        patterns = _simulate_numpy(objects, probes, weights, pos_px, propagators, dose, rng,
                                   portable=portable)
    elif backend == "torch":
        patterns = _simulate_torch(objects, probes, weights, pos_px, propagators, dose,
                                   seed, device)
    else:
        raise ValueError(f"unknown backend {backend!r}")

    q_mrad = wavelength * 1e3 / (sampling * detector)
    data = patterns.reshape(scan_shape[0], scan_shape[1], detector, detector)
    dc = DataCube(data, r_pixel_size=step_ang, r_pixel_units="A",
                  q_pixel_size=q_mrad, q_pixel_units="mrad")
    fov = object_px * sampling
    ctor = dict(energy=energy, semiangle_cutoff=semiangle, defocus=defocus,
                initial_scan_positions=pos_ang, object_fov_ang=(fov, fov))
    if num_slices > 1:
        ctor.update(num_slices=num_slices, slice_thicknesses=slice_thickness)
    if num_modes > 1:
        mode_probes = probes * np.sqrt(weights)[:, None, None]
        ctor.update(num_probes=num_modes)
    else:
        mode_probes = None
    pre = dict(force_com_rotation=0.0, force_com_transpose=False,
               plot_center_of_mass=False, plot_rotation=False, plot_probe_overlaps=False)
    return ScanCase(name=name, datacube=dc, scan_positions_ang=pos_ang,
                    true_object=objects if num_slices > 1 else objects[0],
                    sampling=sampling, ctor_kwargs=ctor, preprocess_kwargs=pre,
                    reconstruct_kwargs={}, probe_modes=mode_probes)


def single_slice_cpu_case(seed=0, scan=32, detector=64, object_px=128, step=0.5,
                          backend="numpy", device="cuda"):
    """The CPU-runnable single-slice workload: 32x32 scan at 0.5 A, 64^2 detector,
    128^2 object at 0.25 A, 1e4 e-/pattern; GD step 0.5, batch 64, 16 iterations."""
    case = make_scan("single-slice 32^2 scan, 64^2 det", seed, (scan, scan), step, 0.05,
                     detector, object_px, dose=1e4, backend=backend, device=device)
    case.reconstruct_kwargs = dict(num_iter=16, max_batch_size=64, step_size=0.5,
                                   seed_random=seed)
    return case


def single_slice_throughput_case(seed=0, backend="torch", device="cuda"):
    """The GPU-throughput single-slice workload: 128x128 scan at 0.75 A, 128^2
    detector, 512^2 object, 1e5 e-/pattern; GD, batch 1024, 200 iterations."""
    case = make_scan("single-slice 128^2 scan, 128^2 det", seed, (128, 128), 0.75, 0.05,
                     128, 512, dose=1e5, backend=backend, device=device)
    case.reconstruct_kwargs = dict(num_iter=200, max_batch_size=1024, step_size=0.5,
                                   seed_random=seed)
    return case


def multislice_case(seed=0, num_slices=8, scan=64, backend="numpy", device="cuda",
                    object_px=256):
    """Multislice workload: T slices of 20 A, 64^2 scan at 0.4 A, 128^2 detector,
    300 kV, 25 mrad, defocus 50 A."""
    case = make_scan(f"multislice T={num_slices}", seed, (scan, scan), 0.4, 0.05, 128,
                     object_px, semiangle=25.0, defocus=50.0, dose=1e4,
                     num_slices=num_slices, slice_thickness=20.0, backend=backend,
                     device=device)
    case.reconstruct_kwargs = dict(num_iter=8, max_batch_size=256, step_size=0.5,
                                   seed_random=seed)
    return case


def mixed_state_case(seed=0, scan=32, detector=64, num_modes=4, backend="numpy",
                     device="cuda", object_px=None):
    """Mixed-state workload: M probe modes (weights 0.7/0.15/0.1/0.05), each a
    randomly perturbed aberration of the 300 kV, 20 mrad probe."""
    sampling = 0.25
    if object_px is None:
        span = scan * 0.5 / sampling + detector
        object_px = int(2 ** math.ceil(math.log2(span)))
    case = make_scan(f"mixed-state M={num_modes}", seed, (scan, scan), 0.5, 0.05,
                     detector, object_px, dose=1e4, num_modes=num_modes,
                     mode_weights=(0.7, 0.15, 0.1, 0.05, 0.0, 0.0)[:num_modes] if num_modes <= 4
                     else [1.0 / num_modes] * num_modes,
                     backend=backend, device=device)
    case.reconstruct_kwargs = dict(num_iter=16, max_batch_size=64, step_size=0.5,
                                   seed_random=seed)
    return case


def multiscan_cases(seed=0, num_scans=16, num_modes=4, backend="torch", device="cuda",
                    grid_range=(24, 96), detectors=(64, 96, 128)):
    """Independent mixed-state scans of uneven sizes: square grids drawn uniformly
    from grid_range, detectors from `detectors`, M probe modes (weights
    0.7/0.15/0.1/0.05), 1e4 e-/pattern, 0.5 A step. Returns ScanCases; each
    carries its mode probes as the initial probe guess."""
    rng = np.random.default_rng(seed)
    cases = []
    for k in range(num_scans):
        n = int(rng.integers(grid_range[0], grid_range[1] + 1))
        det = int(rng.choice(detectors))
        cases.append(mixed_state_case(seed=seed * 1000 + k, scan=n, detector=det,
                                      num_modes=num_modes, backend=backend, device=device))
    return cases
