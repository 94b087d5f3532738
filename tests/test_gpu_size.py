"""Parity at the sizes that are timed: the single-slice throughput workload
(128 x 128 scan, 128^2 detector, 512^2 object, batch 1024), 8-slice
multislice at a 128^2 detector on a 64 x 64 scan, and a 4-mode mixed-state scan
of 96 x 96 positions at a 128^2 detector.

The fixtures (tests/golden/size_*.npz, written by make_golden.py --size from
the unmodified reference) keep the generator arguments instead of the
datacube. The test regenerates the counts and checks their SHA-256 digest
before comparing anything. Then it runs the public API (constructor, device
preprocess, reconstruct) on the GPU and holds the result to the stated
tolerances: error per iteration within 1e-5 relative, object and probe within
1e-4 relative L2 of the reference, or 3x the reference's own rounding floor
where that floor is larger. The floor is how far the reference itself moves
when its FFTs are evaluated in complex128 and rounded back (make_golden.py
measures it on the same state). From the default uniform start the first far
fields are exactly zero outside the probe aperture, so A exp(i angle F) there
takes a phase set by rounding. On the 128 x 128 scan this puts the floor of the
error history at 5.6e-5, above 1e-5; no float32 implementation other than the
reference's own NumPy calls can come closer. Each result's distance to the
float64 evaluation of the same model is printed beside it.
"""

import glob
import hashlib
import json
import os

import numpy as np
import pytest

from golden_io import GOLDEN_DIR, rel_l2
from py4dstem_gb300 import DataCube, synthetic
from py4dstem_gb300 import ptychography as api

pytestmark = pytest.mark.gpu

TOL_ERR, TOL_OBJ, TOL_PROBE = 1e-5, 1e-4, 1e-4


def size_names():
    return sorted(os.path.splitext(os.path.basename(p))[0]
                  for p in glob.glob(os.path.join(GOLDEN_DIR, "size_*.npz")))


def _digest(a):
    a = np.ascontiguousarray(a)
    return hashlib.sha256(a.tobytes()).hexdigest() + f":{a.dtype.str}:{list(a.shape)}"


class SizeGolden:
    def __init__(self, name):
        z = np.load(os.path.join(GOLDEN_DIR, f"{name}.npz"))
        self.name = name
        self.meta = json.loads(str(z["meta"]))
        self.scan_positions_ang = z["scan_positions_ang"]
        self.pre = {k[4:]: z[k] for k in z.files if k.startswith("pre_")}
        self.out = {k[4:]: z[k] for k in z.files if k.startswith("out_")}
        self.fp64_object = z["fp64_object"]
        self.fp64_probe = z["fp64_probe"]

    def regenerate(self):
        """The seeded counts, checked against the digest of the reference's input."""
        case = synthetic.make_scan(**self.meta["generator"])
        np.testing.assert_array_equal(case.scan_positions_ang, self.scan_positions_ang)
        counts = np.ascontiguousarray(case.datacube.data.astype(np.uint16))
        digest = hashlib.sha256(counts.tobytes()).hexdigest()
        assert digest == self.meta["counts_digest"], (
            f"{self.name}: regenerated counts differ from the reference's input (total "
            f"{int(counts.sum(dtype=np.int64))}, reference {self.meta.get('counts_total')})")
        return case

    def build(self, case):
        m = self.meta
        ctor = dict(m["ctor"])
        ctor["object_fov_ang"] = tuple(ctor["object_fov_ang"])
        cls = {"single": api.SingleslicePtychography, "multi": api.MultislicePtychography,
               "mixed": api.MixedstatePtychography}[m["cls"]]
        if m.get("probe_guess"):
            ctor["initial_probe_guess"] = np.asarray(case.probe_modes, dtype=np.complex64)
        dc = DataCube(case.datacube.data, r_pixel_size=m["r_pixel_size"], r_pixel_units="A",
                      q_pixel_size=m["q_pixel_size"], q_pixel_units="mrad")
        p = cls(datacube=dc, initial_scan_positions=self.scan_positions_ang.copy(),
                verbose=False, device="gpu", **ctor)
        p.preprocess(**m["preprocess"])
        return p


@pytest.mark.parametrize("name", size_names())
def test_size_reconstruction_matches_reference(cuda, name):
    g = SizeGolden(name)
    case = g.regenerate()
    p = g.build(case)
    # the preprocessed state is the reference's (amplitudes bit for bit)
    np.testing.assert_array_equal(p._positions_px, g.pre["positions_px"])
    assert np.float32(p._mean_diffraction_intensity) == g.pre["mean_intensity"]
    amps = p._amplitudes
    amps = amps.cpu().numpy() if hasattr(amps, "cpu") else np.asarray(amps)
    assert _digest(amps) == g.meta["amplitudes_digest"]
    del amps
    assert rel_l2(p._probe, g.pre["probe_initial"]) < 1e-6
    np.testing.assert_array_equal(p._object_fov_mask, g.pre["fov_mask"])

    p.reconstruct(progress_bar=False, **g.meta["reconstruct"])
    ref_err = g.out["error_iterations"]
    err = np.asarray(p.error_iterations)
    d_err = float(np.max(np.abs(err - ref_err) / np.abs(ref_err)))
    d_obj = rel_l2(p.object, g.out["object"])
    d_probe = rel_l2(p._probe, g.out["probe_corner"])
    s = g.meta["stats"]
    print(f"\n{name}: gpu-vs-ref err {d_err:.2e} obj {d_obj:.2e} probe {d_probe:.2e} | "
          f"floor err {s['floor_err']:.2e} obj {s['floor_obj']:.2e} "
          f"probe {s['floor_probe']:.2e} | gpu-vs-fp64 obj "
          f"{rel_l2(p.object, g.fp64_object):.2e} probe {rel_l2(p._probe, g.fp64_probe):.2e} | "
          f"ref-vs-fp64 obj {s['ref_vs_fp64_obj']:.2e} probe {s['ref_vs_fp64_probe']:.2e}")
    assert d_err <= max(TOL_ERR, 3.0 * s["floor_err"])
    assert d_obj <= max(TOL_OBJ, 3.0 * s["floor_obj"])
    assert d_probe <= max(TOL_PROBE, 3.0 * s["floor_probe"])
