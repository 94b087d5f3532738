"""Small seeded reconstruction states and a GPU runner that mirrors
oracle.ptycho_np.Oracle.reconstruct argument for argument."""

import numpy as np

from oracle.ptycho_np import State
from py4dstem_gb300 import engine
from py4dstem_gb300.optics import ComplexProbe, electron_wavelength_angstrom


def make_state(S=64, J=36, modes=1, slices=1, potential=False, seed=0, obj_px=None,
               uniform_object=False):
    """Random but well-conditioned state: non-uniform initial object (no exact
    zeros in the far field), amplitudes from a different true object plus noise."""
    rng = np.random.default_rng(seed)
    Sx, Sy = (S, S) if np.isscalar(S) else (int(S[0]), int(S[1]))
    sampling = 0.25
    n = int(np.ceil(np.sqrt(J)))
    step = 2.3
    span = (n - 1) * step
    P = obj_px or int(max(Sx, Sy) + span + 8)
    probe = ComplexProbe(energy=300e3, gpts=(Sx, Sy), sampling=(sampling, sampling),
                         semiangle_cutoff=20.0, rolloff=2.0,
                         parameters={"defocus": 100.0}).build()._array.astype(np.complex64)
    probe *= np.float32(30.0)
    probes = [probe]
    for m in range(1, modes):
        ramp_x = np.exp(-2j * np.pi * rng.uniform(-0.5, 0.5) * np.fft.fftfreq(Sx))
        ramp_y = np.exp(-2j * np.pi * rng.uniform(-0.5, 0.5) * np.fft.fftfreq(Sy))
        probes.append((probes[-1] * ramp_x[:, None] * ramp_y[None] * 0.5).astype(np.complex64))
    probe_arr = np.stack(probes) if modes > 1 else probe

    def smooth_field(scale):
        f = rng.normal(size=(P, P)) + 1j * rng.normal(size=(P, P))
        k = np.fft.fftfreq(P)
        g = np.exp(-(k[:, None] ** 2 + k[None] ** 2) * (P / 6.0) ** 2)
        out = np.fft.ifft2(np.fft.fft2(f) * g).real
        return scale * out / np.abs(out).max()

    def obj_pair():
        phase = smooth_field(0.6)
        amp = 0.9 + 0.05 * smooth_field(1.0)
        true = amp * np.exp(1j * phase)
        init = true * np.exp(1j * smooth_field(0.1)) * (1 + 0.02 * smooth_field(1.0))
        if uniform_object:
            init = np.ones_like(init)
        return true, init

    pairs = [obj_pair() for _ in range(slices)]
    true = np.stack([p[0] for p in pairs])
    init = np.stack([p[1] for p in pairs])
    if potential:
        init_o = np.angle(init).astype(np.float32)
    else:
        init_o = init.astype(np.complex64)
    if slices == 1:
        init_o = init_o[0]

    g = np.arange(n) * step
    xx, yy = np.meshgrid(g, g, indexing="ij")
    pos = np.stack([xx.ravel(), yy.ravel()], -1)[:J]
    pos = pos + rng.uniform(-0.5, 0.5, size=pos.shape) + (P - span) / 2
    pos = pos.astype(np.float32)

    lam = electron_wavelength_angstrom(300e3)
    props = None
    if slices > 1:
        kx = np.fft.fftfreq(Sx, sampling).astype(np.float32)
        ky = np.fft.fftfreq(Sy, sampling).astype(np.float32)
        h = np.exp(-1j * np.pi * lam * 20.0 * (kx[:, None] ** 2 + ky[None] ** 2))
        props = np.stack([h] * (slices - 1)).astype(np.complex64)

    # amplitudes from the true object (float64 model)
    fx = np.fft.fftfreq(Sx, 1 / Sx).astype(int)
    fy = np.fft.fftfreq(Sy, 1 / Sy).astype(int)
    kk = np.fft.fftfreq(Sx)
    kl = np.fft.fftfreq(Sy)
    amps = np.empty((J, Sx, Sy), np.float32)
    for j in range(J):
        r = np.round(pos[j].astype(np.float64))
        d = pos[j] - r
        rows = (int(r[0]) + fx) % P
        cols = (int(r[1]) + fy) % P
        ramp = np.exp(-2j * np.pi * kk[:, None] * d[0]) * np.exp(-2j * np.pi * kl[None] * d[1])
        inten = np.zeros((Sx, Sy))
        for m in range(modes):
            w = np.fft.ifft2(np.fft.fft2(np.asarray(probes[m], np.complex128)) * ramp)
            for s in range(slices):
                w = w * true[s][np.ix_(rows, cols)]
                if s + 1 < slices:
                    w = np.fft.ifft2(np.fft.fft2(w) * props[s])
            inten += np.abs(np.fft.fft2(w)) ** 2
        amps[j] = np.sqrt(rng.poisson(inten * 0.05) / 0.05).astype(np.float32)
    mean_int = np.float32(np.mean(np.sum(amps.astype(np.float64) ** 2, axis=(-2, -1))))
    fov_inv = np.ones((P, P), bool)
    fov_inv[Sx // 2: P - Sx // 2, Sy // 2: P - Sy // 2] = False
    return State(amplitudes=amps, positions_px=pos, probe=probe_arr, object=init_o,
                 mean_intensity=mean_int, fov_mask_inverse=fov_inv,
                 object_type="potential" if potential else "complex", num_slices=slices,
                 num_probes=modes, mixed=modes > 1, propagators=props)


def gpu_reconstruct(state, num_iter=1, method="GD", a=None, b=None, c=None, max_batch_size=None,
                    seed_random=None, step_size=0.5, normalization_min=1.0, fix_probe=False,
                    fix_probe_com=True, orthogonalize_probe=True, shrinkage_rad=0.0,
                    fix_potential_baseline=True, pure_phase_object=False,
                    object_positivity=True, detector_fourier_mask=None, storage="gpu",
                    return_state=False):
    projection = method != "GD"
    J = state.amplitudes.shape[0]
    order = np.arange(J)
    if max_batch_size is not None:
        np.random.seed(seed_random)
    else:
        max_batch_size = J
    use_mask = bool(fix_potential_baseline and state.fov_mask_inverse.sum() > 0)
    st = engine.create_state(
        roi_shape=(state.roi_shape if state.roi_shape is not None
                   else state.amplitudes.shape[-2:]),
        object_array=state.object, probe_array=state.probe,
        amplitudes=state.amplitudes, positions_px=state.positions_px,
        num_slices=state.num_slices, num_probes=state.num_probes,
        potential=state.object_type == "potential", max_batch=max_batch_size, storage=storage,
        propagators=state.propagators, detector_mask=detector_fourier_mask,
        fov_mask_inverse=state.fov_mask_inverse if use_mask else None, projection=projection,
        mixed_state=state.mixed)
    drv = engine.IterationDriver(
        st, max_batch=max_batch_size, projection=projection, step_size=step_size,
        normalization_min=normalization_min, fix_probe=fix_probe,
        projection_abc=(a or 0.0, b or 0.0, c or 0.0), shrinkage_rad=shrinkage_rad,
        use_mask=use_mask, pure_phase=pure_phase_object and state.object_type == "complex",
        positivity=object_positivity, fix_probe_com=fix_probe_com,
        orthogonalize_probe=orthogonalize_probe, mean_intensity=state.mean_intensity)
    errors = []
    for _ in range(num_iter):
        if not projection:
            np.random.shuffle(order)
        drv.iterate(order)
        errors.append(float(drv.error()))
    obj = st.object.cpu().numpy()
    probe = st.probe.cpu().numpy().reshape(np.shape(state.probe))
    if return_state:
        return obj, probe, errors, st
    return obj, probe, errors


def rel(a, b):
    a = np.asarray(a, dtype=np.complex128)
    b = np.asarray(b, dtype=np.complex128)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))
