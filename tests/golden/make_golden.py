"""Generate the golden fixtures of tests/golden/ from the unmodified reference.

Each fixture holds a seeded synthetic datacube (py4dstem_gb300.synthetic), the
arguments of the constructor / preprocess() / reconstruct() calls, and what the
reference py4DSTEM 0.14.18 CPU path (loaded by oracle/refloader.py) returned:
preprocessed state (mean intensity, positions, initial probe and object, FOV
mask, per-pattern amplitude sums) and the reconstruction result (error per
iteration, object, corner-centred probe, final positions, and the per-position
self-consistency errors of the final state).

Run from the repository root in a container that has the reference checkout:

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py
"""

from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
# this script reads the reference checkout of this container
os.environ.setdefault("PY4DSTEM_REFERENCE", "/root/reference")

from oracle.refloader import load_reference  # noqa: E402
from py4dstem_gb300 import synthetic  # noqa: E402

PRE = dict(plot_center_of_mass=False, plot_rotation=False, plot_probe_overlaps=False,
           force_com_rotation=0.0, force_com_transpose=False)

CASES = {
    # the CPU-runnable single-slice workload, full size, default (uniform) start
    "ss_gd_32x32_det64": dict(
        gen=dict(name="ss", seed=0, scan_shape=(32, 32), step_ang=0.5, jitter_ang=0.05,
                 detector=64, object_px=128),
        cls="single", ctor=dict(object_fov_ang=(32.0, 32.0)),
        rec=dict(num_iter=16, max_batch_size=64, step_size=0.5, seed_random=0)),
    # the smaller cases start from a seeded non-uniform object (`guess`): with a
    # uniform start the first far field is exactly zero outside the aperture and
    # the reference's result is set by FFT rounding noise there
    "ss_gd_potential": dict(
        gen=dict(name="ssp", seed=11, scan_shape=(12, 12), step_ang=0.5, jitter_ang=0.05,
                 detector=64, object_px=96),
        cls="single", ctor=dict(object_fov_ang=(24.0, 24.0), object_type="potential"),
        guess=(96, 96),
        rec=dict(num_iter=6, max_batch_size=36, step_size=0.5, seed_random=1)),
    "ss_ap": dict(
        gen=dict(name="ssr", seed=12, scan_shape=(12, 12), step_ang=0.5, jitter_ang=0.05,
                 detector=64, object_px=96),
        cls="single", ctor=dict(object_fov_ang=(24.0, 24.0)), guess=(96, 96),
        rec=dict(num_iter=6, reconstruction_method="DM_AP", reconstruction_parameter=0.0)),
    # projection sets (RAAR) at a 128^2 detector: the grouped kernels' form
    "ss_ap_det128": dict(
        gen=dict(name="sra", seed=38, scan_shape=(6, 6), step_ang=0.5, jitter_ang=0.05,
                 detector=128, object_px=192),
        cls="single", ctor=dict(object_fov_ang=(48.0, 48.0)), guess=(192, 192),
        rec=dict(num_iter=4, reconstruction_method="RAAR", reconstruction_parameter=0.8)),
    "ms_gd_T3": dict(
        gen=dict(name="ms", seed=13, scan_shape=(10, 10), step_ang=0.5, jitter_ang=0.05,
                 detector=64, object_px=96, num_slices=3, slice_thickness=20.0),
        cls="multi", ctor=dict(object_fov_ang=(24.0, 24.0), num_slices=3, slice_thicknesses=20.0),
        guess=(3, 96, 96),
        rec=dict(num_iter=6, max_batch_size=25, step_size=0.5, seed_random=2)),
    # position correction (fix_positions=False) from perturbed scan positions,
    # with both distance limits and the positions centre-of-mass constraint
    "ss_gd_poscorr": dict(
        gen=dict(name="ssc", seed=15, scan_shape=(12, 12), step_ang=0.5, jitter_ang=0.05,
                 detector=64, object_px=96),
        cls="single", ctor=dict(object_fov_ang=(24.0, 24.0)), guess=(96, 96),
        perturb_ang=0.15,
        rec=dict(num_iter=6, max_batch_size=36, step_size=0.5, seed_random=4,
                 fix_positions=False, fix_positions_com=False, positions_step_size=0.5,
                 max_position_update_distance=0.1, max_position_total_distance=0.3)),
    # position correction with the global affine constraint (RANSAC on the global
    # random generator, between the batch shuffles)
    "ss_gd_poscorr_affine": dict(
        gen=dict(name="ssf", seed=36, scan_shape=(12, 12), step_ang=0.5, jitter_ang=0.05,
                 detector=64, object_px=96),
        cls="single", ctor=dict(object_fov_ang=(24.0, 24.0)), guess=(96, 96),
        perturb_ang=0.15,
        rec=dict(num_iter=5, max_batch_size=36, step_size=0.5, seed_random=16,
                 fix_positions=False, positions_step_size=0.5,
                 global_affine_transformation=True)),
    "ms_gd_poscorr": dict(
        gen=dict(name="msc", seed=17, scan_shape=(10, 10), step_ang=0.5, jitter_ang=0.05,
                 detector=64, object_px=96, num_slices=2, slice_thickness=20.0),
        cls="multi", ctor=dict(object_fov_ang=(24.0, 24.0), num_slices=2, slice_thicknesses=20.0),
        guess=(2, 96, 96), perturb_ang=0.15,
        rec=dict(num_iter=5, max_batch_size=25, step_size=0.5, seed_random=6,
                 fix_positions=False, positions_step_size=0.5,
                 max_position_total_distance=0.5)),
    "mixed_gd_poscorr": dict(
        gen=dict(name="mxc", seed=16, scan_shape=(10, 10), step_ang=0.5, jitter_ang=0.05,
                 detector=64, object_px=96, num_modes=2, mode_weights=(0.8, 0.2)),
        cls="mixed", ctor=dict(object_fov_ang=(24.0, 24.0), num_probes=2), global_seed=8,
        guess=(96, 96), perturb_ang=0.15,
        rec=dict(num_iter=5, max_batch_size=25, step_size=0.5, seed_random=5,
                 fix_positions=False, positions_step_size=0.25)),
    # the benchmark's 128^2 detector (radix-16/8 transforms) on a small scan
    "ss_gd_det128": dict(
        gen=dict(name="s128", seed=18, scan_shape=(6, 6), step_ang=0.5, jitter_ang=0.05,
                 detector=128, object_px=192),
        cls="single", ctor=dict(object_fov_ang=(48.0, 48.0)), guess=(192, 192),
        rec=dict(num_iter=4, max_batch_size=18, step_size=0.5, seed_random=7)),
    # position correction at a 128^2 detector (the grouped kernels' far-field
    # keeping form and the grouped correction)
    "ss_gd_poscorr_det128": dict(
        gen=dict(name="scp", seed=37, scan_shape=(8, 8), step_ang=0.5, jitter_ang=0.05,
                 detector=128, object_px=192),
        cls="single", ctor=dict(object_fov_ang=(48.0, 48.0)), guess=(192, 192),
        perturb_ang=0.15,
        rec=dict(num_iter=4, max_batch_size=32, step_size=0.5, seed_random=9,
                 fix_positions=False, fix_positions_com=False, positions_step_size=0.5,
                 max_position_update_distance=0.1, max_position_total_distance=0.3)),
    # a 96^2 detector (radix-8/4/3 transforms) with a detector Fourier mask
    "ss_gd_det96_mask": dict(
        gen=dict(name="s96", seed=19, scan_shape=(8, 8), step_ang=0.5, jitter_ang=0.05,
                 detector=96, object_px=128),
        cls="single", ctor=dict(object_fov_ang=(32.0, 32.0)), guess=(128, 128),
        mask_seed=5,
        rec=dict(num_iter=4, max_batch_size=16, step_size=0.5, seed_random=8)),
    # region_of_interest_shape different from the detector: the far field is
    # resampled onto the detector grid and back in every Fourier projection
    "ss_gd_resample_up": dict(
        gen=dict(name="rsu", seed=30, scan_shape=(12, 12), step_ang=0.5, jitter_ang=0.05,
                 detector=48, object_px=96),
        cls="single", ctor=dict(object_fov_ang=(24.0, 24.0)), guess=(96, 96),
        pre_extra=dict(region_of_interest_shape=(64, 64)),
        rec=dict(num_iter=4, max_batch_size=36, step_size=0.5, seed_random=11)),
    "ss_gd_resample_down_mask": dict(
        gen=dict(name="rsd", seed=31, scan_shape=(12, 12), step_ang=0.5, jitter_ang=0.05,
                 detector=64, object_px=96),
        cls="single", ctor=dict(object_fov_ang=(24.0, 24.0)), guess=(96, 96), mask_seed=6,
        pre_extra=dict(region_of_interest_shape=(48, 48)),
        rec=dict(num_iter=4, max_batch_size=36, step_size=0.5, seed_random=12)),
    "ss_gd_resample_nonsquare": dict(
        gen=dict(name="rsn", seed=32, scan_shape=(10, 10), step_ang=0.5, jitter_ang=0.05,
                 detector=64, object_px=128),
        cls="single", ctor=dict(object_fov_ang=(32.0, 32.0)), guess=(128, 128),
        pre_extra=dict(region_of_interest_shape=(96, 128)),
        rec=dict(num_iter=3, max_batch_size=25, step_size=0.5, seed_random=13)),
    "mixed_gd_resample": dict(
        gen=dict(name="rsm", seed=33, scan_shape=(10, 10), step_ang=0.5, jitter_ang=0.05,
                 detector=64, object_px=96, num_modes=2, mode_weights=(0.8, 0.2)),
        cls="mixed", ctor=dict(object_fov_ang=(24.0, 24.0), num_probes=2), global_seed=14,
        guess=(96, 96), pre_extra=dict(region_of_interest_shape=(48, 48)),
        rec=dict(num_iter=4, max_batch_size=25, step_size=0.5, seed_random=14)),
    "ms_gd_resample": dict(
        gen=dict(name="rss", seed=34, scan_shape=(10, 10), step_ang=0.5, jitter_ang=0.05,
                 detector=48, object_px=96, num_slices=2, slice_thickness=20.0),
        cls="multi", ctor=dict(object_fov_ang=(24.0, 24.0), num_slices=2, slice_thicknesses=20.0),
        guess=(2, 96, 96), pre_extra=dict(region_of_interest_shape=(64, 64)),
        rec=dict(num_iter=4, max_batch_size=25, step_size=0.5, seed_random=15)),
    # mixed-state multislice: two modes through three slices
    "mms_gd_T3M2": dict(
        gen=dict(name="mms", seed=24, scan_shape=(10, 10), step_ang=0.5, jitter_ang=0.05,
                 detector=64, object_px=96, num_slices=3, slice_thickness=20.0, num_modes=2,
                 mode_weights=(0.8, 0.2)),
        cls="mixed_multi", ctor=dict(object_fov_ang=(24.0, 24.0), num_slices=3,
                                     slice_thicknesses=20.0, num_probes=2),
        global_seed=9, guess=(3, 96, 96),
        rec=dict(num_iter=5, max_batch_size=25, step_size=0.5, seed_random=10)),
    # mixed-state multislice at a 128^2 detector: the grouped kernels' form
    "mms_gd_det128": dict(
        gen=dict(name="mmd", seed=39, scan_shape=(6, 6), step_ang=0.5, jitter_ang=0.05,
                 detector=128, object_px=192, num_slices=2, slice_thickness=20.0,
                 num_modes=2, mode_weights=(0.8, 0.2)),
        cls="mixed_multi", ctor=dict(object_fov_ang=(48.0, 48.0), num_slices=2,
                                     slice_thicknesses=20.0, num_probes=2),
        global_seed=11, guess=(2, 192, 192),
        rec=dict(num_iter=3, max_batch_size=18, step_size=0.5, seed_random=12)),
    "mms_ap": dict(
        gen=dict(name="msa", seed=25, scan_shape=(8, 8), step_ang=0.5, jitter_ang=0.05,
                 detector=64, object_px=96, num_slices=2, slice_thickness=20.0, num_modes=2,
                 mode_weights=(0.8, 0.2)),
        cls="mixed_multi", ctor=dict(object_fov_ang=(24.0, 24.0), num_slices=2,
                                     slice_thicknesses=20.0, num_probes=2),
        global_seed=11, guess=(2, 96, 96),
        rec=dict(num_iter=4, reconstruction_method="RAAR", reconstruction_parameter=0.8)),
    "mms_gd_poscorr": dict(
        gen=dict(name="msp", seed=26, scan_shape=(10, 10), step_ang=0.5, jitter_ang=0.05,
                 detector=64, object_px=96, num_slices=2, slice_thickness=20.0, num_modes=2,
                 mode_weights=(0.8, 0.2)),
        cls="mixed_multi", ctor=dict(object_fov_ang=(24.0, 24.0), num_slices=2,
                                     slice_thicknesses=20.0, num_probes=2),
        global_seed=12, guess=(2, 96, 96), perturb_ang=0.15,
        rec=dict(num_iter=4, max_batch_size=25, step_size=0.5, seed_random=11,
                 fix_positions=False, positions_step_size=0.5,
                 max_position_update_distance=0.1, max_position_total_distance=0.5)),
    # optional constraints: probe aperture and amplitude, identical slices
    "ss_gd_probe_constraints": dict(
        gen=dict(name="spc", seed=29, scan_shape=(10, 10), step_ang=0.5, jitter_ang=0.05,
                 detector=64, object_px=96),
        cls="single", ctor=dict(object_fov_ang=(24.0, 24.0)), guess=(96, 96),
        rec=dict(num_iter=4, max_batch_size=25, step_size=0.5, seed_random=12,
                 fix_probe_aperture=True, constrain_probe_amplitude=True,
                 constrain_probe_amplitude_relative_radius=0.4,
                 constrain_probe_amplitude_relative_width=0.08)),
    "mixed_gd_probe_constraints": dict(
        gen=dict(name="mpc", seed=30, scan_shape=(10, 10), step_ang=0.5, jitter_ang=0.05,
                 detector=64, object_px=96, num_modes=2, mode_weights=(0.8, 0.2)),
        cls="mixed", ctor=dict(object_fov_ang=(24.0, 24.0), num_probes=2), global_seed=13,
        guess=(96, 96),
        rec=dict(num_iter=4, max_batch_size=25, step_size=0.5, seed_random=13,
                 fix_probe_aperture=True, constrain_probe_amplitude=True)),
    "ms_gd_identical_slices": dict(
        gen=dict(name="mis", seed=31, scan_shape=(10, 10), step_ang=0.5, jitter_ang=0.05,
                 detector=64, object_px=96, num_slices=3, slice_thickness=20.0),
        cls="multi", ctor=dict(object_fov_ang=(24.0, 24.0), num_slices=3, slice_thicknesses=20.0),
        guess=(3, 96, 96),
        rec=dict(num_iter=4, max_batch_size=25, step_size=0.5, seed_random=14,
                 identical_slices=True)),
    "ss_gd_gaussian": dict(
        gen=dict(name="sgf", seed=32, scan_shape=(10, 10), step_ang=0.5, jitter_ang=0.05,
                 detector=64, object_px=96),
        cls="single", ctor=dict(object_fov_ang=(24.0, 24.0)), guess=(96, 96),
        rec=dict(num_iter=4, max_batch_size=25, step_size=0.5, seed_random=15,
                 gaussian_filter_sigma=0.5)),
    "ms_gd_gaussian_pure_phase": dict(
        gen=dict(name="mgf", seed=33, scan_shape=(10, 10), step_ang=0.5, jitter_ang=0.05,
                 detector=64, object_px=96, num_slices=2, slice_thickness=20.0),
        cls="multi", ctor=dict(object_fov_ang=(24.0, 24.0), num_slices=2, slice_thicknesses=20.0),
        guess=(2, 96, 96),
        rec=dict(num_iter=4, max_batch_size=25, step_size=0.5, seed_random=16,
                 gaussian_filter_sigma=0.4, pure_phase_object=True)),
    # position correction with projection sets (whole-scan batches)
    "ss_ap_poscorr": dict(
        gen=dict(name="sap", seed=34, scan_shape=(10, 10), step_ang=0.5, jitter_ang=0.05,
                 detector=64, object_px=96),
        cls="single", ctor=dict(object_fov_ang=(24.0, 24.0)), guess=(96, 96), perturb_ang=0.15,
        rec=dict(num_iter=4, reconstruction_method="RAAR", reconstruction_parameter=0.9,
                 fix_positions=False, positions_step_size=0.5,
                 max_position_update_distance=0.1)),
    "ms_ap_poscorr": dict(
        gen=dict(name="map", seed=35, scan_shape=(8, 8), step_ang=0.5, jitter_ang=0.05,
                 detector=64, object_px=96, num_slices=2, slice_thickness=20.0),
        cls="multi", ctor=dict(object_fov_ang=(24.0, 24.0), num_slices=2, slice_thicknesses=20.0),
        guess=(2, 96, 96), perturb_ang=0.15,
        rec=dict(num_iter=4, reconstruction_method="DM_AP", reconstruction_parameter=0.0,
                 fix_positions=False, positions_step_size=0.5, max_position_total_distance=0.5)),
    "mixed_ap_poscorr": dict(
        gen=dict(name="xap", seed=36, scan_shape=(8, 8), step_ang=0.5, jitter_ang=0.05,
                 detector=64, object_px=96, num_modes=2, mode_weights=(0.8, 0.2)),
        cls="mixed", ctor=dict(object_fov_ang=(24.0, 24.0), num_probes=2), global_seed=17,
        guess=(96, 96), perturb_ang=0.15,
        rec=dict(num_iter=3, reconstruction_method="RAAR", reconstruction_parameter=0.9,
                 fix_positions=False, positions_step_size=0.5,
                 max_position_update_distance=0.1, max_position_total_distance=0.4)),
    "mixed_gd_M3": dict(
        gen=dict(name="mx", seed=14, scan_shape=(10, 10), step_ang=0.5, jitter_ang=0.05,
                 detector=64, object_px=96, num_modes=3, mode_weights=(0.7, 0.2, 0.1)),
        cls="mixed", ctor=dict(object_fov_ang=(24.0, 24.0), num_probes=3), global_seed=7,
        guess=(96, 96),
        rec=dict(num_iter=6, max_batch_size=25, step_size=0.5, seed_random=3)),
}


# preprocess-only fixtures ("prep_" prefix): the rotation search, masks, crop and
# the other centre-of-mass options that the reconstruction fixtures fix
PRE_CASES = {
    "prep_rotation_curl": dict(
        gen=dict(name="prc", seed=21, scan_shape=(16, 16), step_ang=0.5, jitter_ang=0.05,
                 detector=64, object_px=128),
        ctor=dict(object_fov_ang=(32.0, 32.0)), scan_positions=True,
        pre=dict(plot_center_of_mass=False, plot_rotation=False, plot_probe_overlaps=False)),
    "prep_rotation_div_masks": dict(
        gen=dict(name="prd", seed=22, scan_shape=(14, 18), step_ang=0.5, jitter_ang=0.05,
                 detector=64, object_px=128),
        ctor=dict(object_fov_ang=(32.0, 32.0)), scan_positions=False, positions_mask_seed=3,
        dp_mask_radius=24,
        pre=dict(plot_center_of_mass=False, plot_rotation=False, plot_probe_overlaps=False,
                 maximize_divergence=True, rotation_angles_deg=list(range(-60, 61, 4)),
                 fit_function="parabola")),
    "prep_crop_loop_com": dict(
        gen=dict(name="prx", seed=23, scan_shape=(12, 12), step_ang=0.5, jitter_ang=0.05,
                 detector=64, object_px=128),
        ctor=dict(object_fov_ang=(32.0, 32.0)), scan_positions=True,
        # the forced centre (24.6 px) makes the corner crop 48 x 48, a region of
        # interest the fused kernels support
        pre=dict(plot_center_of_mass=False, plot_rotation=False, plot_probe_overlaps=False,
                 force_com_transpose=True, crop_patterns=True, force_com_shifts=[24.6, 24.6],
                 vectorized_com_calculation=False)),
    # diffraction resampling (the reference's default 'bilinear' and 'fourier') and
    # padding of a 128^2 detector, with a vacuum probe and a detector mask
    "prep_fourier_vacuum": dict(
        gen=dict(name="prf", seed=27, scan_shape=(10, 10), step_ang=0.5, jitter_ang=0.05,
                 detector=128, object_px=160),
        ctor=dict(object_fov_ang=(40.0, 40.0)), scan_positions=True, vacuum=True,
        dp_mask_radius=50,
        pre=dict(plot_center_of_mass=False, plot_rotation=False, plot_probe_overlaps=False,
                 force_com_rotation=0.0, force_com_transpose=False,
                 diffraction_intensities_shape=[64, 64], reshaping_method="fourier")),
    "prep_bilinear_pad": dict(
        gen=dict(name="prb", seed=28, scan_shape=(10, 10), step_ang=0.5, jitter_ang=0.05,
                 detector=128, object_px=160),
        ctor=dict(object_fov_ang=(40.0, 40.0)), scan_positions=True,
        pre=dict(plot_center_of_mass=False, plot_rotation=False, plot_probe_overlaps=False,
                 force_com_rotation=0.0, force_com_transpose=False,
                 diffraction_intensities_shape=[48, 48],
                 padded_diffraction_intensities_shape=[64, 64])),
}


def make_pre_case(ref, name, spec):
    case = synthetic.make_scan(**spec["gen"])
    data = case.datacube.data
    assert np.array_equal(data, np.round(data)) and data.max() < 65535
    q = case.datacube.calibration.get_Q_pixel_size()
    r = case.datacube.calibration.get_R_pixel_size()
    dc = ref.DataCube(data, r_pixel_size=r, r_pixel_units="A", q_pixel_size=q,
                      q_pixel_units="mrad")
    ctor = dict(energy=300e3, semiangle_cutoff=20.0, defocus=100.0, **spec["ctor"])
    arrays = {}
    kw = {}
    if spec["scan_positions"]:
        kw["initial_scan_positions"] = case.scan_positions_ang
    if spec.get("vacuum"):
        # the probe's own aperture intensity, detector-centred, as the vacuum probe
        from py4dstem_gb300.optics import ComplexProbe

        det = spec["gen"]["detector"]
        pr = ComplexProbe(energy=300e3, gpts=(det, det), sampling=(0.25, 0.25),
                          semiangle_cutoff=20.0, rolloff=2.0).build()._array
        vpi = np.fft.fftshift(np.abs(np.fft.fft2(pr)) ** 2).astype(np.float64)
        arrays["vacuum_probe_intensity"] = vpi
        kw["vacuum_probe_intensity"] = vpi.copy()
    if "positions_mask_seed" in spec:
        mrng = np.random.default_rng(spec["positions_mask_seed"])
        pmask = mrng.random(data.shape[:2]) > 0.1
        arrays["positions_mask"] = pmask
        kw["positions_mask"] = pmask.copy()
    pre = dict(spec["pre"])
    if "dp_mask_radius" in spec:
        qx, qy = data.shape[-2:]
        x, y = np.meshgrid(np.arange(qx) - qx / 2, np.arange(qy) - qy / 2, indexing="ij")
        dmask = (x ** 2 + y ** 2) < spec["dp_mask_radius"] ** 2
        arrays["dp_mask"] = dmask
        pre["dp_mask"] = dmask.copy()
    p = ref.SingleslicePtychography(datacube=dc, verbose=False, device="cpu", **ctor, **kw)
    p.preprocess(**pre)
    out = dict(
        com_measured_x=np.asarray(p._com_measured_x), com_measured_y=np.asarray(p._com_measured_y),
        com_fitted_x=np.asarray(p._com_fitted_x), com_fitted_y=np.asarray(p._com_fitted_y),
        com_normalized_x=np.asarray(p._com_normalized_x),
        com_normalized_y=np.asarray(p._com_normalized_y),
        rotation_best_rad=np.float64(p._rotation_best_rad),
        rotation_best_transpose=np.bool_(p._rotation_best_transpose),
        mean_intensity=np.float32(p._mean_diffraction_intensity),
        positions_px=p._positions_px.copy(),
        probe_initial=p._probe.copy(),
        fov_mask=p._object_fov_mask.copy(),
        amplitudes=p._amplitudes.copy(),
    )
    meta = dict(cls="single", ctor=ctor, preprocess={k: v for k, v in pre.items()
                                                     if k != "dp_mask"},
                r_pixel_size=r, q_pixel_size=q, generator=spec["gen"],
                scan_positions=spec["scan_positions"])
    path = os.path.join(HERE, f"{name}.npz")
    np.savez_compressed(path, datacube=data.astype(np.uint16),
                        scan_positions_ang=case.scan_positions_ang, meta=json.dumps(meta),
                        **arrays, **{f"pre_{k}": v for k, v in out.items()})
    print(f"{name}: {os.path.getsize(path) / 1e6:.2f} MB, rotation "
          f"{np.rad2deg(out['rotation_best_rad']):.1f} deg, transpose "
          f"{bool(out['rotation_best_transpose'])}")


def smooth_guess(shape, seed, potential):
    """Seeded smooth random phase (0.3 rad peak) as an initial object."""
    rng = np.random.default_rng(seed)
    f = rng.normal(size=shape)
    k0 = np.fft.fftfreq(shape[-2])
    k1 = np.fft.fftfreq(shape[-1])
    g = np.exp(-(k0[:, None] ** 2 + k1[None] ** 2) * (shape[-1] / 8.0) ** 2)
    ph = np.fft.ifft2(np.fft.fft2(f) * g).real
    ph = 0.3 * ph / np.abs(ph).max()
    return ph.astype(np.float32) if potential else np.exp(1j * ph).astype(np.complex64)


def make_case(ref, name, spec):
    case = synthetic.make_scan(**spec["gen"])
    data = case.datacube.data
    assert np.array_equal(data, np.round(data)) and data.max() < 65535
    q = case.datacube.calibration.get_Q_pixel_size()
    r = case.datacube.calibration.get_R_pixel_size()
    dc = ref.DataCube(data, r_pixel_size=r, r_pixel_units="A", q_pixel_size=q,
                      q_pixel_units="mrad")
    ctor = dict(energy=300e3, semiangle_cutoff=20.0, defocus=100.0, **spec["ctor"])
    cls = {"single": ref.SingleslicePtychography, "multi": ref.MultislicePtychography,
           "mixed": ref.MixedstatePtychography,
           "mixed_multi": ref.MixedstateMultislicePtychography}[spec["cls"]]
    extra = {}
    guess = None
    if "guess" in spec:
        guess = smooth_guess(tuple(spec["guess"]), spec["gen"]["seed"] + 100,
                             ctor.get("object_type") == "potential")
        # the reference aliases the caller's array as its object and updates it
        # in place, so it gets a copy and the fixture keeps the original
        extra["initial_object_guess"] = guess.copy()
    positions = case.scan_positions_ang
    if "perturb_ang" in spec:
        rng = np.random.default_rng(spec["gen"]["seed"] + 200)
        positions = positions + rng.uniform(-spec["perturb_ang"], spec["perturb_ang"],
                                            positions.shape)
    if "global_seed" in spec:
        np.random.seed(spec["global_seed"])
    p = cls(datacube=dc, initial_scan_positions=positions, verbose=False,
            device="cpu", **ctor, **extra)
    pre_kwargs = dict(PRE, **spec.get("pre_extra", {}))
    p.preprocess(**pre_kwargs)
    pre = dict(
        mean_intensity=np.float32(p._mean_diffraction_intensity),
        positions_px=p._positions_px.copy(),
        probe_initial=p._probe.copy(),
        object_initial=p._object.copy(),
        fov_mask=p._object_fov_mask.copy(),
        amplitude_sums=p._amplitudes.astype(np.float64).sum(axis=(-2, -1)),
        amplitude_first=p._amplitudes[0].copy(),
        amplitude_last=p._amplitudes[-1].copy(),
    )
    rec = dict(spec["rec"])
    if "mask_seed" in spec:
        # corner-centred Fourier mask with ~3% dead pixels, used as given
        mrng = np.random.default_rng(spec["mask_seed"])
        det = spec["gen"]["detector"]
        mask = (mrng.random((det, det)) > 0.03).astype(np.float32)
        extra_arrays_mask = {"detector_fourier_mask": mask}
        rec["detector_fourier_mask"] = mask.copy()
    else:
        extra_arrays_mask = {}
    p.reconstruct(progress_bar=False, **rec)
    out = dict(
        error_iterations=np.asarray(p.error_iterations, dtype=np.float64),
        object=p.object,
        probe_corner=np.asarray(p._probe),
        positions_px=np.asarray(p._positions_px).copy(),
        self_consistency_errors=p._return_self_consistency_errors(
            max_batch_size=spec["rec"].get("max_batch_size")),
    )
    meta = dict(cls=spec["cls"], ctor=ctor, preprocess=pre_kwargs, reconstruct=spec["rec"],
                global_seed=spec.get("global_seed"), r_pixel_size=r, q_pixel_size=q,
                generator=spec["gen"])
    path = os.path.join(HERE, f"{name}.npz")
    if guess is not None:
        extra_arrays = {"initial_object_guess": guess}
    else:
        extra_arrays = {}
    extra_arrays.update(extra_arrays_mask)
    np.savez_compressed(
        path, datacube=data.astype(np.uint16), scan_positions_ang=positions,
        meta=json.dumps(meta), **extra_arrays, **{f"pre_{k}": v for k, v in pre.items()},
        **{f"out_{k}": v for k, v in out.items()})
    print(f"{name}: {os.path.getsize(path) / 1e6:.2f} MB, errors {out['error_iterations'][-3:]}")


# Ptychographic tomography: three tilts about the x axis of a 48^3 potential
# volume, each tilt its own seeded synthetic scan. Gradient descent with the
# default collective update (one volume update per iteration), and with the
# sequential update (the volume updated after every tilt) plus shrinkage, both
# from a seeded smooth positive volume (`guess_peak`: its largest voxel). From
# the default zero volume the first gradient steps are ill-conditioned (a change
# of the float32 FFT alone moves the result by 1e-2); the zero-start case keeps
# that default path covered.
TOMO_CASES = {
    "tomo_gd_collective": dict(
        seeds=(40, 41, 42), tilts_deg=(-10.0, 0.0, 12.0), guess_peak=0.03,
        gen=dict(scan_shape=(8, 8), step_ang=0.5, jitter_ang=0.05, detector=48,
                 object_px=64, num_slices=2, slice_thickness=10.0),
        ctor=dict(num_slices=4, object_padding_px=(8, 8)),
        rec=dict(num_iter=3, max_batch_size=16, seed_random=1, step_size=0.5)),
    "tomo_gd_sequential": dict(
        seeds=(43, 44), tilts_deg=(-7.0, 9.0), guess_peak=0.03,
        gen=dict(scan_shape=(8, 8), step_ang=0.5, jitter_ang=0.05, detector=48,
                 object_px=64, num_slices=2, slice_thickness=10.0),
        ctor=dict(num_slices=3, object_padding_px=(8, 8)),
        rec=dict(num_iter=3, max_batch_size=20, seed_random=5, step_size=0.5,
                 collective_measurement_updates=False, shrinkage_rad=1e-3)),
    # the volume's 3D Gaussian blur among the object constraints
    "tomo_gd_gaussian": dict(
        seeds=(40, 41, 42), tilts_deg=(-10.0, 0.0, 12.0), guess_peak=0.03,
        gen=dict(scan_shape=(8, 8), step_ang=0.5, jitter_ang=0.05, detector=48,
                 object_px=64, num_slices=2, slice_thickness=10.0),
        ctor=dict(num_slices=4, object_padding_px=(8, 8)),
        rec=dict(num_iter=3, max_batch_size=16, seed_random=1, step_size=0.5,
                 gaussian_filter_sigma=0.4)),
    "tomo_gd_zero_start": dict(
        seeds=(40, 41, 42), tilts_deg=(-10.0, 0.0, 12.0),
        gen=dict(scan_shape=(8, 8), step_ang=0.5, jitter_ang=0.05, detector=48,
                 object_px=64, num_slices=2, slice_thickness=10.0),
        ctor=dict(num_slices=4, object_padding_px=(8, 8)),
        rec=dict(num_iter=3, max_batch_size=16, seed_random=1, step_size=0.5)),
}


# Tomography preprocess only: one 2D positions mask for every tilt (tiled by
# the reference, with a warning) and forced centre-of-mass shifts for the first
# tilt.
TOMO_PRE_CASES = {
    "tomo_pre_mask_shifts": dict(
        seeds=(45, 46), tilts_deg=(-5.0, 6.0), mask_seed=9,
        gen=dict(scan_shape=(8, 8), step_ang=0.5, jitter_ang=0.05, detector=48,
                 object_px=64, num_slices=2, slice_thickness=10.0),
        ctor=dict(num_slices=3, object_padding_px=(8, 8)),
        pre_extra=dict(force_com_shifts=[[23.6, 24.3], None])),
}


def smooth_volume(shape, seed, peak):
    """Seeded smooth positive potential volume, values in [0.2, 1] x peak."""
    rng = np.random.default_rng(seed)
    f = rng.normal(size=shape)
    k = [np.fft.fftfreq(n) for n in shape]
    g = np.exp(-(k[0][:, None, None] ** 2 + k[1][None, :, None] ** 2
                 + k[2][None, None, :] ** 2) * (shape[-1] / 6.0) ** 2)
    v = np.fft.ifftn(np.fft.fftn(f) * g).real
    v = (v - v.min()) / (v.max() - v.min())
    return (peak * (0.2 + 0.8 * v)).astype(np.float32)


def tilt_matrix(deg):
    """Rotation by `deg` degrees about the x (first, vertical) axis in (x, y, z)."""
    t = np.deg2rad(deg)
    c, s = np.cos(t), np.sin(t)
    return np.array([[1.0, 0.0, 0.0], [0.0, c, -s], [0.0, s, c]])


def tomography_class(ref):
    """The reference class with two defects of py4DSTEM 0.14.18 that stop its
    preprocess() worked around: ptychographic_tomography.py:486-492 calls
    _normalize_diffraction_intensities without its required
    in_place_datacube_modification argument (passed here as False, the default
    of the preprocess() argument of that name), and the constructor never sets
    the _object_fov_ang that _initialize_object reads (set to None here, the
    value that sizes the volume from the scan positions)."""

    class Tomography(ref.PtychographicTomography):
        def __init__(self, *args, **kwargs):
            super().__init__(*args, **kwargs)
            self._object_fov_ang = None

        def _normalize_diffraction_intensities(self, *args, **kwargs):
            if len(args) == 5:
                kwargs.setdefault("in_place_datacube_modification", False)
            return super()._normalize_diffraction_intensities(*args, **kwargs)

    return Tomography


def make_tomo_case(ref, name, spec):
    cases = [synthetic.make_scan(name="tomo", seed=sd, **spec["gen"]) for sd in spec["seeds"]]
    dcs = []
    for c in cases:
        q = c.datacube.calibration.get_Q_pixel_size()
        r = c.datacube.calibration.get_R_pixel_size()
        dcs.append(ref.DataCube(c.datacube.data, r_pixel_size=r, r_pixel_units="A",
                                q_pixel_size=q, q_pixel_units="mrad"))
    mats = np.stack([tilt_matrix(a) for a in spec["tilts_deg"]])
    positions = np.stack([c.scan_positions_ang for c in cases])
    ctor = dict(energy=300e3, semiangle_cutoff=20.0, defocus=100.0, **spec["ctor"])
    cls = tomography_class(ref)
    pre_args = dict(plot_probe_overlaps=False, diffraction_patterns_rotate_degrees=0.0,
                    diffraction_patterns_transpose=False)
    extra, guess = {}, None
    if "guess_peak" in spec:
        # the volume shape comes out of preprocess(): one pass to learn it
        probe_pass = cls(tilt_orientation_matrices=list(mats), datacube=dcs,
                         initial_scan_positions=list(positions), verbose=False, device="cpu",
                         **ctor)
        probe_pass.preprocess(**pre_args)
        guess = smooth_volume(probe_pass._object.shape, spec["seeds"][0] + 100,
                              spec["guess_peak"])
        extra["initial_object_guess"] = guess.copy()
    p = cls(tilt_orientation_matrices=list(mats), datacube=dcs,
            initial_scan_positions=list(positions), verbose=False, device="cpu", **ctor,
            **extra)
    p.preprocess(**pre_args)
    pre = dict(
        mean_intensity=np.asarray(p._mean_diffraction_intensity, dtype=np.float32),
        positions_px=np.asarray(p._positions_px_all).copy(),
        probe_initial=np.stack(p._probes_all).copy(),
        object_initial=p._object.copy(),
        amplitude_sums=np.asarray(p._amplitudes).sum(axis=(-2, -1)),
        propagators=np.asarray(p._propagator_arrays).copy(),
    )
    p.reconstruct(progress_bar=False, **spec["rec"])
    out = dict(
        error_iterations=np.asarray(p.error_iterations, dtype=np.float64),
        object=np.asarray(p.object),
        probes_corner=np.stack(p._probes_all),
    )
    data = np.stack([c.datacube.data for c in cases])
    assert np.array_equal(data, np.round(data)) and data.max() < 65535
    meta = dict(ctor=ctor, preprocess=pre_args, reconstruct=spec["rec"],
                tilts_deg=spec["tilts_deg"], seeds=spec["seeds"], generator=spec["gen"],
                r_pixel_size=[c.datacube.calibration.get_R_pixel_size() for c in cases],
                q_pixel_size=[c.datacube.calibration.get_Q_pixel_size() for c in cases])
    path = os.path.join(HERE, f"{name}.npz")
    if guess is not None:
        extra_arrays = {"initial_object_guess": guess}
    else:
        extra_arrays = {}
    np.savez_compressed(
        path, datacube=data.astype(np.uint16), scan_positions_ang=positions, tilt_matrices=mats,
        meta=json.dumps(meta), **extra_arrays, **{f"pre_{k}": v for k, v in pre.items()},
        **{f"out_{k}": v for k, v in out.items()})
    print(f"{name}: {os.path.getsize(path) / 1e6:.2f} MB, errors {out['error_iterations']}")


def make_tomo_pre_case(ref, name, spec):
    cases = [synthetic.make_scan(name="tomo", seed=sd, **spec["gen"]) for sd in spec["seeds"]]
    dcs = [ref.DataCube(c.datacube.data, r_pixel_size=c.datacube.calibration.get_R_pixel_size(),
                        r_pixel_units="A", q_pixel_size=c.datacube.calibration.get_Q_pixel_size(),
                        q_pixel_units="mrad") for c in cases]
    mats = np.stack([tilt_matrix(a) for a in spec["tilts_deg"]])
    positions = np.stack([c.scan_positions_ang for c in cases])
    mask = np.random.default_rng(spec["mask_seed"]).random(spec["gen"]["scan_shape"]) > 0.15
    ctor = dict(energy=300e3, semiangle_cutoff=20.0, defocus=100.0, **spec["ctor"])
    pre_args = dict(plot_probe_overlaps=False, diffraction_patterns_rotate_degrees=0.0,
                    diffraction_patterns_transpose=False, **spec["pre_extra"])
    cls = tomography_class(ref)
    # the reference indexes the scan positions with the mask: masked positions
    p = cls(tilt_orientation_matrices=list(mats), datacube=dcs,
            initial_scan_positions=[pos[mask.ravel()] for pos in positions],
            positions_mask=mask.copy(), verbose=False, device="cpu", **ctor)
    # the reference writes the per-tilt shifts it used back into the list it got
    p.preprocess(**json.loads(json.dumps(pre_args)))
    pre = dict(
        mean_intensity=np.asarray(p._mean_diffraction_intensity, dtype=np.float32),
        positions_px=np.asarray(p._positions_px_all).copy(),
        cum_counts=np.asarray(p._cum_probes_per_measurement),
        probe_initial=np.stack(p._probes_all).copy(),
        object_initial=p._object.copy(),
        amplitude_sums=np.asarray(p._amplitudes).sum(axis=(-2, -1)),
        propagators=np.asarray(p._propagator_arrays).copy(),
    )
    data = np.stack([c.datacube.data for c in cases])
    meta = dict(ctor=ctor, preprocess=pre_args, tilts_deg=spec["tilts_deg"], seeds=spec["seeds"],
                generator=spec["gen"],
                r_pixel_size=[c.datacube.calibration.get_R_pixel_size() for c in cases],
                q_pixel_size=[c.datacube.calibration.get_Q_pixel_size() for c in cases])
    path = os.path.join(HERE, f"{name}.npz")
    np.savez_compressed(
        path, datacube=data.astype(np.uint16), scan_positions_ang=positions, tilt_matrices=mats,
        positions_mask=mask, meta=json.dumps(meta), **{f"pre_{k}": v for k, v in pre.items()})
    print(f"{name}: {os.path.getsize(path) / 1e6:.2f} MB, patterns {pre['cum_counts']}")


def make_volume_ops(ref):
    """The reference's own volume operations on a seeded random volume:
    _rotate_zxy_volume (float32 and float64 input), _project_sliced_object and
    _expand_sliced_object (ptychographic_methods.py:783-868)."""
    cls = tomography_class(ref)
    p = cls.__new__(cls)
    p._xp = np
    import scipy

    p._scipy = scipy
    rng = np.random.default_rng(7)
    vol = rng.random((20, 24, 28)).astype(np.float32)
    vol64 = rng.normal(size=(20, 24, 28))
    out = {"volume": vol, "volume64": vol64}
    for k, deg in enumerate((-10.0, 12.0, 30.0, 90.0)):
        r = tilt_matrix(deg) @ tilt_matrix(3.0 * k).T
        out[f"matrix_{k}"] = r
        out[f"rot32_{k}"] = p._rotate_zxy_volume(vol, r)
        out[f"rot64_{k}"] = p._rotate_zxy_volume(vol64, r)
    for T in (1, 3, 6, 7):
        sl = p._project_sliced_object(vol, T)
        out[f"project_{T}"] = sl
        upd = (sl * np.float32(0.25)).astype(np.float32)
        out[f"update_{T}"] = upd
        out[f"expand_{T}"] = p._expand_sliced_object(upd, vol.shape[0])
    path = os.path.join(HERE, "tomo_volume_ops.npz")
    np.savez_compressed(path, **out)
    print(f"tomo_volume_ops: {os.path.getsize(path) / 1e6:.2f} MB")


# Workloads at the sizes that are timed ("size_" prefix). Their datacubes are too
# large to commit (1 GiB of counts for the 128 x 128 scan), so a fixture keeps
# the generator arguments and a SHA-256 digest of the uint16 counts instead; the
# GPU test regenerates the counts (synthetic.make_scan with the "portable"
# backend: every random variate from the generator's uniform doubles, Poisson
# counts by inversion, so that the counts agree across CPUs and NumPy versions)
# and checks the digest before it compares anything. The reference's float32
# amplitudes are pinned the same way (digest and per-pattern sums). The float32
# oracle with every FFT rounded through complex128 (the reference's own
# rounding floor) and the float64 oracle run here, on the reference's
# preprocessed state; the fixture keeps their distances and the float64 object
# and probe.
SIZE_CASES = {
    # single-slice throughput workload: 128 x 128 scan at 0.75 A (J = 16384),
    # 128^2 detector, 512^2 object, 1e5 e-/pattern, batch 1024, uniform start
    "size_ss_scan128_det128": dict(
        gen=dict(name="size_ss", seed=1234, scan_shape=(128, 128), step_ang=0.75,
                 jitter_ang=0.05, detector=128, object_px=512, dose=1e5, backend="portable"),
        cls="single", ctor=dict(object_fov_ang=(128.0, 128.0)),
        rec=dict(num_iter=3, max_batch_size=1024, step_size=0.5, seed_random=1234)),
    # multislice through the adjoint: 8 slices of 20 A, 64 x 64 scan at 0.4 A,
    # 128^2 detector, 25 mrad, defocus 50 A
    "size_ms_T8_scan64_det128": dict(
        gen=dict(name="size_ms", seed=2, scan_shape=(64, 64), step_ang=0.4, jitter_ang=0.05,
                 detector=128, object_px=256, semiangle=25.0, defocus=50.0, dose=1e4,
                 num_slices=8, slice_thickness=20.0, backend="portable"),
        cls="multi", ctor=dict(object_fov_ang=(64.0, 64.0), num_slices=8,
                               slice_thicknesses=20.0),
        ctor_optics=dict(semiangle_cutoff=25.0, defocus=50.0),
        rec=dict(num_iter=2, max_batch_size=256, step_size=0.5, seed_random=2)),
    # one scan of the batched mixed-state workload at its largest size: 96 x 96
    # scan, 128^2 detector, 4 modes (weights 0.7 / 0.15 / 0.1 / 0.05) given as the
    # initial probe
    "size_mixed_M4_scan96_det128": dict(
        gen=dict(name="size_mx", seed=3, scan_shape=(96, 96), step_ang=0.5, jitter_ang=0.05,
                 detector=128, object_px=512, dose=1e4, num_modes=4,
                 mode_weights=(0.7, 0.15, 0.1, 0.05), backend="portable"),
        cls="mixed", ctor=dict(object_fov_ang=(128.0, 128.0), num_probes=4),
        probe_guess=True,
        rec=dict(num_iter=2, max_batch_size=256, step_size=0.5, seed_random=3)),
}


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.complex128)
    b = np.asarray(b, dtype=np.complex128)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def counts_digest(data):
    """SHA-256 of the datacube as uint16 counts (C order)."""
    import hashlib

    return hashlib.sha256(np.ascontiguousarray(data.astype(np.uint16)).tobytes()).hexdigest()


def array_digest(a):
    import hashlib

    a = np.ascontiguousarray(a)
    return hashlib.sha256(a.tobytes()).hexdigest() + f":{a.dtype.str}:{list(a.shape)}"


def make_size_case(ref, name, spec):
    import time

    from oracle.ptycho_np import Oracle, State

    t0 = time.time()
    case = synthetic.make_scan(**spec["gen"])
    data = case.datacube.data
    assert np.array_equal(data, np.round(data)) and data.max() < 65535
    q = case.datacube.calibration.get_Q_pixel_size()
    r = case.datacube.calibration.get_R_pixel_size()
    dc = ref.DataCube(data, r_pixel_size=r, r_pixel_units="A", q_pixel_size=q,
                      q_pixel_units="mrad")
    optics = dict(semiangle_cutoff=20.0, defocus=100.0)
    optics.update(spec.get("ctor_optics", {}))
    ctor = dict(energy=300e3, **optics, **spec["ctor"])
    cls = {"single": ref.SingleslicePtychography, "multi": ref.MultislicePtychography,
           "mixed": ref.MixedstatePtychography}[spec["cls"]]
    extra = {}
    probe_guess = None
    if spec.get("probe_guess"):
        probe_guess = np.asarray(case.probe_modes, dtype=np.complex64)
        extra["initial_probe_guess"] = probe_guess.copy()
    print(f"{name}: generated {data.shape} in {time.time() - t0:.0f} s", flush=True)
    p = cls(datacube=dc, initial_scan_positions=case.scan_positions_ang, verbose=False,
            device="cpu", **ctor, **extra)
    p.preprocess(**PRE)
    print(f"{name}: reference preprocess done at {time.time() - t0:.0f} s", flush=True)
    pre = dict(
        mean_intensity=np.float32(p._mean_diffraction_intensity),
        positions_px=p._positions_px.copy(),
        probe_initial=p._probe.copy(),
        object_initial=p._object.copy(),
        fov_mask=p._object_fov_mask.copy(),
        amplitude_sums=p._amplitudes.astype(np.float64).sum(axis=(-2, -1)),
    )
    amp_digest = array_digest(p._amplitudes)
    state = State(
        amplitudes=p._amplitudes.copy(), positions_px=p._positions_px.copy(),
        probe=np.array(p._probe, copy=True), object=np.array(p._object, copy=True),
        mean_intensity=p._mean_diffraction_intensity,
        fov_mask_inverse=p._object_fov_mask_inverse.copy(), object_type=p._object_type,
        num_slices=spec["ctor"].get("num_slices", 1),
        num_probes=spec["ctor"].get("num_probes", 1), mixed=spec["cls"] == "mixed",
        propagators=(np.array(p._propagator_arrays) if spec["cls"] == "multi" else None),
        sampling=tuple(p.sampling))
    p.reconstruct(progress_bar=False, **spec["rec"])
    print(f"{name}: reference reconstruct done at {time.time() - t0:.0f} s", flush=True)
    out = dict(
        error_iterations=np.asarray(p.error_iterations, dtype=np.float64),
        object=p.object,
        probe_corner=np.asarray(p._probe),
    )
    # the oracle on the same state: float32 (must equal the reference), FFTs
    # rounded through complex128 (the floor), float64 (the FP64 model)
    o32 = Oracle(state.copy()).reconstruct(**spec["rec"])
    assert np.array_equal(np.asarray(o32.error_iterations), out["error_iterations"]), name
    assert np.array_equal(o32.object, out["object"]), name
    floor = Oracle(state.copy(), fft_round_trip=True).reconstruct(**spec["rec"])
    o64 = Oracle(state.copy(), "float64").reconstruct(**spec["rec"])
    ref_err = out["error_iterations"]
    stats = dict(
        floor_err=float(np.max(np.abs(np.asarray(floor.error_iterations) - ref_err) / ref_err)),
        floor_obj=rel_l2(floor.object, out["object"]),
        floor_probe=rel_l2(floor.probe, out["probe_corner"]),
        ref_vs_fp64_obj=rel_l2(out["object"], o64.object),
        ref_vs_fp64_probe=rel_l2(out["probe_corner"], o64.probe),
    )
    print(f"{name}: oracle checks done at {time.time() - t0:.0f} s: {stats}", flush=True)
    meta = dict(cls=spec["cls"], ctor=ctor, preprocess=PRE, reconstruct=spec["rec"],
                r_pixel_size=r, q_pixel_size=q, generator=spec["gen"],
                counts_digest=counts_digest(data), amplitudes_digest=amp_digest,
                counts_total=int(data.astype(np.int64).sum()),
                probe_guess=bool(spec.get("probe_guess")), stats=stats)
    path = os.path.join(HERE, f"{name}.npz")
    np.savez_compressed(
        path, scan_positions_ang=case.scan_positions_ang, meta=json.dumps(meta),
        **{f"pre_{k}": v for k, v in pre.items()},
        **{f"out_{k}": v for k, v in out.items()},
        fp64_object=np.asarray(o64.object).astype(
            np.float32 if p._object_type == "potential" else np.complex64),
        fp64_probe=np.asarray(o64.probe).astype(np.complex64))
    print(f"{name}: {os.path.getsize(path) / 1e6:.2f} MB, errors {out['error_iterations']}",
          flush=True)


def main():
    ref = load_reference()
    only = set(sys.argv[1:])
    if "--size" in only:
        only.discard("--size")
        for name, spec in SIZE_CASES.items():
            if not only or name in only:
                make_size_case(ref, name, spec)
        return
    for name, spec in CASES.items():
        if not only or name in only:
            make_case(ref, name, spec)
    for name, spec in PRE_CASES.items():
        if not only or name in only:
            make_pre_case(ref, name, spec)
    for name, spec in TOMO_CASES.items():
        if not only or name in only:
            make_tomo_case(ref, name, spec)
    for name, spec in TOMO_PRE_CASES.items():
        if not only or name in only:
            make_tomo_pre_case(ref, name, spec)
    if not only or "tomo_volume_ops" in only:
        make_volume_ops(ref)


if __name__ == "__main__":
    main()
