"""Algorithmic work per position update, the numbers every roofline figure uses.

Counting convention: 5 N log2 N real flops per complex 2D FFT of N = Sx*Sy
points (the radix-2 Cooley-Tukey count); elementwise work as listed per variant.
Bytes are the algorithmic HBM traffic of one position update: the amplitude
read, the object patch read and the two staged scatters, each c64 = 8 B and
f32 = 4 B per pixel. The per-batch object and probe read/write (2 * 8 P / B per
position) is negligible and not counted.

Operators counted (reference, py4DSTEM/process/phase/):
  single slice  ptychographic_methods.py:1482-1635, 1818-1908
      1 probe-shift IFFT + 1 FFT + 1 IFFT, ~50 flops/pixel elementwise
  multislice    ptychographic_methods.py:2300-2458
      (4T - 1) FFTs (shift, T-1 forward propagations as FFT/IFFT pairs,
      far-field FFT and IFFT, T-1 back propagations), 50 + 24 (T - 1) flops/pixel
  mixed state   ptychographic_methods.py:2696-3000
      3 FFTs per mode, 20 + 30 M flops/pixel
  mixed-state multislice  ptychographic_methods.py:3102-3258
      the multislice count for every mode
"""

from __future__ import annotations

import math


def fft_flops(n_pixels: int) -> float:
    return 5.0 * n_pixels * math.log2(n_pixels)


def flops_per_position(n_pixels: int, num_slices: int = 1, num_probes: int = 1) -> float:
    f = fft_flops(n_pixels)
    if num_slices > 1 and num_probes > 1:
        # every mode through every slice and back: (4T - 1) transforms per mode
        t, m = num_slices, num_probes
        return m * ((4 * t - 1) * f + (50 + 24 * (t - 1)) * n_pixels)
    if num_slices > 1:
        t = num_slices
        return (4 * t - 1) * f + (50 + 24 * (t - 1)) * n_pixels
    if num_probes > 1:
        m = num_probes
        return 3 * m * f + (20 + 30 * m) * n_pixels
    return 3 * f + 50 * n_pixels


def bytes_per_position(n_pixels: int, num_slices: int = 1, num_probes: int = 1) -> float:
    if num_slices > 1:
        return 4 * n_pixels + 20 * n_pixels * num_slices
    # amplitude 4N + object patch 8N + object-term scatter 8N + |P|^2 scatter 4N
    # (mixed state sums its modes before the scatter)
    return 24 * n_pixels


def bound(flops: float, bytes_: float, fp32_tflops: float, hbm_gbs: float):
    """(name, seconds) of the slower of the FP32 and HBM rooflines for the work."""
    t_flop = flops / (fp32_tflops * 1e12)
    t_hbm = bytes_ / (hbm_gbs * 1e9)
    return ("fp32", t_flop) if t_flop >= t_hbm else ("hbm", t_hbm)
