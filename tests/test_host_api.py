"""Host-side behaviour of the drop-in classes that needs no GPU."""

import numpy as np
import pytest

from oracle.ptycho_np import Oracle, method_abc
from py4dstem_gb300 import MixedstatePtychography, MultislicePtychography, SingleslicePtychography
from py4dstem_gb300.preprocess import generate_batches
from py4dstem_gb300.ptychography import method_parameters


@pytest.mark.parametrize("J,B", [(1024, 64), (1000, 64), (7, 3), (16384, 1024), (5, 5), (5, 100)])
def test_batches_match_reference_split(J, B):
    ours = list(generate_batches(J, B))
    ref = list(Oracle.batches(J, B))
    assert ours == ref
    assert ours[-1][1] == J


@pytest.mark.parametrize("method,param", [("DM_AP", 0.3), ("RAAR", 0.5), ("RRR", 1.5),
                                          ("SUPERFLIP", 1.0), ("GD", 1.0),
                                          ("difference-map_alternating-projections", 1.0)])
def test_method_parameters(method, param):
    use, a, b, c, _, step = method_parameters(method, param, None, None, None, 0.5)
    kind, ra, rb, rc = method_abc(method, param)
    assert use == (kind == "PS")
    assert (a, b, c) == (ra, rb, rc)


def test_method_parameter_errors():
    with pytest.raises(ValueError):
        method_parameters("DM_AP", 1.5, None, None, None, 0.5)
    with pytest.raises(ValueError):
        method_parameters("generalized-projections", 1.0, 0.1, None, 0.3, 0.5)
    with pytest.raises(ValueError):
        method_parameters("nope", 1.0, None, None, None, 0.5)


def test_constructor_validation():
    with pytest.raises(ValueError):
        SingleslicePtychography(energy=300e3, object_type="weird")
    with pytest.raises(ValueError):
        SingleslicePtychography(energy=300e3, not_an_aberration=1.0)
    with pytest.raises(ValueError):
        SingleslicePtychography(energy=300e3, device="tpu")
    with pytest.raises(ValueError):
        SingleslicePtychography(energy=300e3, storage="disk")
    with pytest.raises(ValueError):
        MixedstatePtychography(energy=300e3)  # num_probes missing
    with pytest.raises(ValueError):
        MultislicePtychography(energy=300e3, num_slices=4, slice_thicknesses=[1.0, 2.0])


def test_polar_parameters():
    p = SingleslicePtychography(energy=300e3, defocus=100, Cs=1e4)
    assert p._polar_parameters["C10"] == -100
    assert p._polar_parameters["C30"] == 1e4
    m = MultislicePtychography(energy=300e3, num_slices=4, slice_thicknesses=10.0, defocus=50,
                               middle_focus=True)
    assert m._polar_parameters["C10"] == -50 - 10.0 * 4 / 2
    assert m._slice_thicknesses.shape == (3,)


def test_preprocess_requires_datacube():
    with pytest.raises(ValueError):
        SingleslicePtychography(energy=300e3).preprocess()


def test_unsupported_options_raise_before_gpu():
    from golden_io import Golden

    g = Golden("ss_gd_potential")
    p = g.build(device="cpu")
    kw = dict(num_iter=1, device="gpu")
    with pytest.raises(NotImplementedError):
        p.reconstruct(fit_probe_aberrations=True, **kw)
    with pytest.raises(NotImplementedError):
        p.reconstruct(q_lowpass=0.5, **kw)

    with pytest.raises(ValueError):
        p.reconstruct(reconstruction_method="DM_AP", max_batch_size=4, **kw)


def test_device_cpu_preprocesses_on_host_and_refuses_to_reconstruct():
    """device="cpu" is the reference's NumPy preprocessing; the reconstruction
    itself runs on the GPU only and says so."""
    from golden_io import Golden

    g = Golden("ss_gd_32x32_det64")
    p = g.build(device="cpu")
    assert p._preprocessed and p._amplitudes.shape[0] == 32 * 32
    with pytest.raises(ValueError, match="GPU only"):
        p.reconstruct(num_iter=1)
    with pytest.raises(ValueError, match="GPU only"):
        p._return_self_consistency_errors()
