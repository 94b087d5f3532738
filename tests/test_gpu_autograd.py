"""The forward model as a torch.autograd.Function (py4dstem_gb300.autograd).

* Its backward (the hand-written adjoint kernel) agrees with central finite
  differences of the FP64 forward model (oracle) on 32 random object pixels and
  32 random probe pixels, for single-slice (complex and potential), multislice,
  mixed-state and mixed-state multislice models.
* Its object gradient is -2N times the reference's summed adjoint term
  (the scatter of conj(P) chi, ptychographic_methods.py:1818-1908), evaluated by
  the float32 oracle; its probe gradient is the exact one (each term back
  through the adjoint of the position's sub-pixel shift).
* Its loss is the reference's batch error.
"""

import numpy as np
import pytest

from gpu_helpers import make_state, rel
from oracle.ptycho_np import Oracle

pytestmark = pytest.mark.gpu

CASES = {
    "single": dict(S=64, J=16),
    "potential": dict(S=64, J=16, potential=True),
    "multislice": dict(S=64, J=16, slices=3),
    "mixed": dict(S=64, J=16, modes=2),
    "mixed_multislice": dict(S=64, J=16, slices=2, modes=2),
    # the multislice workload's depth and detector: 8 slices at 128^2 (a 3 x 3
    # scan keeps the float64 finite differences short)
    "multislice_T8_det128": dict(S=128, J=9, slices=8),
}


def _model(torch, state):
    from py4dstem_gb300.autograd import PtychoForwardModel

    return PtychoForwardModel(state.amplitudes, state.positions_px, np.shape(state.object)[-2:],
                              num_slices=state.num_slices, num_probes=state.num_probes,
                              potential=state.object_type == "potential",
                              propagators=state.propagators, mixed_state=state.mixed,
                              max_batch=7)  # several batches: gradients add over batches


def _loss64(state, obj, probe):
    s = state.copy()
    s.object = obj
    s.probe = probe
    o = Oracle(s, "float64")
    return float(o.forward_batch(np.arange(o.J))[4])


def _tensors(torch, state):
    obj = torch.tensor(np.asarray(state.object), device="cuda", requires_grad=True)
    probe = torch.tensor(np.asarray(state.probe, np.complex64).reshape(
        (state.num_probes,) + state.amplitudes.shape[-2:]), device="cuda", requires_grad=True)
    return obj, probe


@pytest.mark.parametrize("case", list(CASES))
def test_backward_matches_finite_differences(cuda, case):
    torch = cuda
    state = make_state(seed=3, **CASES[case])
    model = _model(torch, state)
    obj, probe = _tensors(torch, state)
    loss = model.loss(obj, probe)
    loss.backward()
    g_obj = obj.grad.cpu().numpy()
    g_probe = probe.grad.cpu().numpy().reshape(np.shape(state.probe))

    rng = np.random.default_rng(0)
    obj0 = np.asarray(state.object, np.float64 if state.object_type == "potential"
                      else np.complex128)
    probe0 = np.asarray(state.probe, np.complex128)
    # 32 object pixels among those the scan touches (non-negligible gradient)
    flat = np.abs(g_obj).ravel()
    cand = np.flatnonzero(flat > 0.05 * flat.max())
    picks = rng.choice(cand, 32, replace=False)
    eps = 1e-4
    worst = 0.0
    for i in picks:
        idx = np.unravel_index(i, obj0.shape)
        parts = [1.0] if state.object_type == "potential" else [1.0, 1j]
        for d in parts:
            op, om = obj0.copy(), obj0.copy()
            op[idx] += eps * d
            om[idx] -= eps * d
            fd = (_loss64(state, op, probe0) - _loss64(state, om, probe0)) / (2 * eps)
            g = g_obj[idx].real if d == 1.0 else g_obj[idx].imag
            worst = max(worst, abs(g - fd) / flat.max())
    assert worst < 2e-3, worst

    flatp = np.abs(g_probe).ravel()
    cand = np.flatnonzero(flatp > 0.05 * flatp.max())
    picks = rng.choice(cand, 32, replace=False)
    worst = 0.0
    for i in picks:
        idx = np.unravel_index(i, probe0.shape)
        for d in (1.0, 1j):
            pp, pm = probe0.copy(), probe0.copy()
            pp[idx] += eps * d
            pm[idx] -= eps * d
            fd = (_loss64(state, obj0, pp) - _loss64(state, obj0, pm)) / (2 * eps)
            g = g_probe[idx].real if d == 1.0 else g_probe[idx].imag
            worst = max(worst, abs(g - fd) / flatp.max())
    assert worst < 2e-3, worst


def test_gradient_is_scaled_reference_adjoint(cuda):
    """dloss/dO = -2N * scatter(conj(P) chi) of the whole scan as one batch."""
    torch = cuda
    state = make_state(seed=4, S=64, J=16)
    model = _model(torch, state)
    obj, probe = _tensors(torch, state)
    loss, g_obj, g_probe = model.loss_and_gradient(obj.detach(), probe.detach())
    o = Oracle(state)
    idx = np.arange(o.J)
    shifted, patches, _, chi, err = o.forward_batch(idx)
    term = o.scatter(o._obj_term(patches, shifted, chi), o.positions_px[idx])
    N = state.amplitudes.shape[-1] * state.amplitudes.shape[-2]
    assert rel(g_obj.cpu().numpy(), -2 * N * term) < 1e-5
    # probe: each position's conj(O) chi back through the adjoint of its shift
    # (two more float32 FFTs per position than the object term: 3e-5)
    y = np.conj(patches).astype(np.complex128) * chi
    frac = o.positions_px[idx] - np.round(o.positions_px[idx])
    k0 = np.fft.fftfreq(y.shape[-2])[None, :, None]
    k1 = np.fft.fftfreq(y.shape[-1])[None, None, :]
    ramp = np.exp(2j * np.pi * (k0 * frac[:, 0, None, None] + k1 * frac[:, 1, None, None]))
    probe_term = np.sum(np.fft.ifft2(np.fft.fft2(y) * ramp), axis=0)
    assert rel(g_probe.cpu().numpy()[0], -2 * N * probe_term) < 3e-5
    assert abs(float(loss) - float(err)) / float(err) < 1e-5
    # the differentiable forward (forward-only kernel) gives the same loss
    assert abs(float(model.loss(obj, probe)) - float(err)) / float(err) < 1e-5


def test_gradient_descent_with_torch_optimizer(cuda):
    """The model trains with a stock torch optimizer; the data error falls."""
    torch = cuda
    state = make_state(seed=5, S=64, J=16)
    model = _model(torch, state)
    obj, probe = _tensors(torch, state)
    opt = torch.optim.SGD([obj], lr=1e-7)
    losses = []
    for _ in range(5):
        opt.zero_grad()
        loss = model.loss(obj, probe.detach())
        loss.backward()
        opt.step()
        losses.append(float(loss))
    assert losses[-1] < losses[0]
    assert probe.grad is None


def test_sixteen_slices_at_128_det_fit_and_report_memory(cuda):
    """16 slices of a 256^2 object at a 128^2 detector, one batch of 1024
    positions: the backward recomputes the batch (forward through every
    slice, then the adjoint) with that batch's per-slice probes in the
    workspace, T B N 12 bytes (3.2 GB here), whatever the scan size. The peak
    device memory of loss and gradient stays within a few times that."""
    torch = cuda
    from py4dstem_gb300.autograd import PtychoForwardModel

    rng = np.random.default_rng(8)
    T, S, P, J = 16, 128, 256, 1024
    amps = rng.random((J, S, S), dtype=np.float32)
    pos = (rng.random((J, 2)) * (P - S) + S / 2).astype(np.float32)
    k = np.fft.fftfreq(S, 0.25)
    h = np.exp(-1j * np.pi * 0.0197 * 20.0 * (k[:, None] ** 2 + k[None] ** 2))
    props = np.stack([h] * (T - 1)).astype(np.complex64)
    torch.cuda.synchronize()
    torch.cuda.reset_peak_memory_stats()
    base = torch.cuda.memory_allocated()
    model = PtychoForwardModel(amps, pos, (P, P), num_slices=T, num_probes=1, potential=False,
                               propagators=props, mixed_state=False, max_batch=J)
    obj = torch.ones((T, P, P), dtype=torch.complex64, device="cuda")
    probe = torch.from_numpy((rng.standard_normal((1, S, S)) + 0j).astype(np.complex64)).cuda()
    loss, g_obj, g_probe = model.loss_and_gradient(obj, probe)
    torch.cuda.synchronize()
    peak = torch.cuda.max_memory_allocated() - base
    stash = T * J * S * S * 12
    print(f"\n16 slices, B=1024, 128^2: peak {peak / 1e9:.2f} GB, slice stash {stash / 1e9:.2f} GB")
    assert np.isfinite(float(loss))
    assert bool(torch.isfinite(g_obj).all()) and bool(torch.isfinite(g_probe).all())
    assert peak < 3 * stash
