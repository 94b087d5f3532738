"""Tensor-core kernels of the learned initializer against the NumPy reference
(tests/nn_reference.py): the BF16 GEMM, the three 3 x 3 convolution passes,
and the whole U-Net's loss and parameter gradients. A last test trains the
network on a fixed batch and checks that the loss falls.

Tolerances: the GPU accumulates bf16 products in float32 and rounds
activations to bf16, as the reference does. So GEMM and convolution outputs
agree to float32 accumulation error: 1e-5 of the output scale for float32
outputs, one bf16 step for bf16 outputs. The U-Net gradients agree to 5%
relative L2 per layer: a rounding difference on one activation can flip its
bf16 value and carry through the layers (5% per layer, cosine above 0.998).
"""

import ctypes

import numpy as np
import pytest

import nn_reference as ref
from py4dstem_gb300 import _native

pytestmark = pytest.mark.gpu


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def _bf16_tensor(torch, a):
    bits = ref.bf16_bits(a)
    return torch.from_numpy(bits.view(np.int16)).cuda()


def _stream(torch):
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _flag(torch):
    return torch.zeros(1, dtype=torch.int32, device="cuda")


@pytest.mark.parametrize("m,n,k", [(128, 32, 64), (300, 48, 200), (1000, 256, 576),
                                   (257, 128, 1152)])
def test_gemm_bf16(cuda, m, n, k):
    torch = cuda
    lib = _native.lib()
    rng = np.random.default_rng(m + n + k)
    a = ref.bf16_round(rng.standard_normal((m, k)).astype(np.float32))
    b = ref.bf16_round(rng.standard_normal((n, k)).astype(np.float32))
    ta, tb = _bf16_tensor(torch, a), _bf16_tensor(torch, b)
    c = torch.full((m, n), float("nan"), dtype=torch.float32, device="cuda")
    err = _flag(torch)
    assert lib.ptycho_nn_gemm_bf16(_p(ta), _p(tb), _p(c), m, n, k, _p(err), _stream(torch)) == 0
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    want = a.astype(np.float64) @ b.astype(np.float64).T
    got = c.cpu().numpy()
    scale = np.sqrt(k)
    assert np.max(np.abs(got - want)) <= 1e-5 * scale * np.max(np.abs(want)) + 1e-4


CONV_CASES = [(2, 16, 16, 8, 32), (1, 32, 64, 32, 64), (2, 8, 16, 192, 64), (1, 16, 32, 96, 32)]


@pytest.mark.parametrize("nb,H,W,cin,cout", CONV_CASES)
def test_conv3x3_forward(cuda, nb, H, W, cin, cout):
    torch = cuda
    lib = _native.lib()
    rng = np.random.default_rng(nb * 7 + cin)
    x = ref.bf16_round(rng.standard_normal((nb, H, W, cin)).astype(np.float32))
    w = ref.bf16_round((rng.standard_normal((cout, 9, cin)) * 0.1).astype(np.float32))
    bias = rng.standard_normal(cout).astype(np.float32)
    tx, tw = _bf16_tensor(torch, x), _bf16_tensor(torch, w)
    tb = torch.from_numpy(bias).cuda()
    ty = torch.empty((nb, H, W, cout), dtype=torch.int16, device="cuda")
    err = _flag(torch)
    for relu in (0, 1):
        assert lib.ptycho_nn_conv3x3_forward(_p(tx), nb, H, W, cin, _p(tw), _p(tb), cout, relu,
                                             _p(ty), _p(err), _stream(torch)) == 0
        torch.cuda.synchronize()
        got = ref.bf16_to_f32(ty.cpu().numpy().view(np.uint16))
        want = ref.conv3x3(x, w, bias, relu=bool(relu))
        # one bf16 rounding of the output (2^-8 relative) plus accumulation error
        tol = 2.0 ** -8 * np.abs(want) + 1e-5 * np.sqrt(9 * cin) * np.max(np.abs(want))
        assert np.all(np.abs(got - want) <= tol + 1e-6)
    assert int(err.item()) == 0


@pytest.mark.parametrize("nb,H,W,cin,cout", CONV_CASES)
def test_conv3x3_backward(cuda, nb, H, W, cin, cout):
    torch = cuda
    lib = _native.lib()
    rng = np.random.default_rng(nb * 11 + cout)
    x = ref.bf16_round(rng.standard_normal((nb, H, W, cin)).astype(np.float32))
    w = ref.bf16_round((rng.standard_normal((cout, 9, cin)) * 0.1).astype(np.float32))
    dy = ref.bf16_round(rng.standard_normal((nb, H, W, cout)).astype(np.float32))
    wt = np.ascontiguousarray(w.transpose(2, 1, 0))  # (cin, 9, cout)
    tx, tdy, twt = _bf16_tensor(torch, x), _bf16_tensor(torch, dy), _bf16_tensor(torch, wt)
    err = _flag(torch)
    dx = torch.empty((nb, H, W, cin), dtype=torch.float32, device="cuda")
    assert lib.ptycho_nn_conv3x3_backward_data(_p(tdy), nb, H, W, cout, _p(twt), cin, _p(dx),
                                               _p(err), _stream(torch)) == 0
    nbytes = lib.ptycho_nn_conv3x3_wgrad_workspace_bytes(nb, H, W, cin, cout)
    ws = torch.empty(nbytes // 4 + 1, dtype=torch.float32, device="cuda")
    dw = torch.empty((cout, 9, cin), dtype=torch.float32, device="cuda")
    db = torch.empty(cout, dtype=torch.float32, device="cuda")
    assert lib.ptycho_nn_conv3x3_backward_weight(_p(tx), _p(tdy), nb, H, W, cin, cout, _p(dw),
                                                 _p(db), _p(ws), nbytes, _p(err),
                                                 _stream(torch)) == 0
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    want_dx = ref.conv3x3_backward_data(dy, w)
    want_dw, want_db = ref.conv3x3_backward_weight(x, dy)
    for got, want, k in ((dx.cpu().numpy(), want_dx, 9 * cout),
                         (dw.cpu().numpy(), want_dw, nb * H * W),
                         (db.cpu().numpy(), want_db, nb * H * W)):
        assert np.max(np.abs(got - want)) <= 1e-5 * np.sqrt(k) * np.max(np.abs(want)) + 1e-4


def _unet(torch, lib, nb, H, W, seed=3):
    params = torch.empty(lib.ptycho_nn_unet_param_bytes(), dtype=torch.uint8, device="cuda")
    assert lib.ptycho_nn_unet_init(_p(params), seed, _stream(torch)) == 0
    wsb = lib.ptycho_nn_unet_workspace_bytes(nb, H, W)
    ws = torch.zeros(wsb, dtype=torch.uint8, device="cuda")
    return params, ws, wsb


def _param(torch, lib, params, layer, field, shape, dtype):
    off = lib.ptycho_nn_unet_param_offset(layer, field)
    assert off >= 0
    n = int(np.prod(shape))
    item = 2 if dtype == "bf16" else 4
    raw = params[off:off + n * item].cpu().numpy()
    if dtype == "bf16":
        return ref.bf16_to_f32(raw.view(np.uint16)).reshape(shape)
    return raw.view(np.float32).reshape(shape).copy()


def _weights(torch, lib, params):
    w = [_param(torch, lib, params, l, 2, (ref.COUT[l], 9, ref.CIN[l]), "f32") for l in range(14)]
    b = [_param(torch, lib, params, l, 3, (ref.COUT[l],), "f32") for l in range(14)]
    hw = _param(torch, lib, params, 14, 2, (32,), "f32")
    hb = _param(torch, lib, params, 14, 3, (1,), "f32")[0]
    return w, b, hw, hb


def test_unet_gradients_match_reference(cuda):
    torch = cuda
    lib = _native.lib()
    nb, H, W = 2, 64, 64
    params, ws, wsb = _unet(torch, lib, nb, H, W)
    rng = np.random.default_rng(5)
    inp = rng.standard_normal((nb, H, W, 2)).astype(np.float32)
    target = (0.3 * rng.standard_normal((nb, H, W))).astype(np.float32)
    w, b, hw, hb = _weights(torch, lib, params)
    # the bf16 copies the kernels use are the rounded master weights
    np.testing.assert_array_equal(_param(torch, lib, params, 4, 0, w[4].shape, "bf16"),
                                  ref.bf16_round(w[4]))
    loss_t = torch.zeros(1, dtype=torch.float32, device="cuda")
    ti = torch.from_numpy(inp).cuda()
    tt = torch.from_numpy(target).cuda()
    assert lib.ptycho_nn_unet_train_step(_p(params), _p(ti), _p(tt), None, float(nb * H * W), nb,
                                         H, W, 0.0, 1, _p(loss_t), _p(ws), wsb,
                                         _stream(torch)) == 0
    assert lib.ptycho_nn_check(_p(ws), nb, H, W, _stream(torch)) == 0
    net = ref.UNetReference(w, b, hw, hb)
    loss, gw, gb, ghw, ghb = net.gradients(inp, target)
    assert abs(float(loss_t.item()) - loss) <= 1e-3 * loss
    rels = []
    for l in range(14):
        got = _param(torch, lib, params, l, 4, gw[l].shape, "f32")
        gotb = _param(torch, lib, params, l, 5, gb[l].shape, "f32")
        rels.append((np.linalg.norm(got - gw[l]) / np.linalg.norm(gw[l]),
                     np.linalg.norm(gotb - gb[l]) / (np.linalg.norm(gb[l]) + 1e-12),
                     float(np.dot(got.ravel(), gw[l].ravel())
                           / (np.linalg.norm(got) * np.linalg.norm(gw[l])))))
    got = _param(torch, lib, params, 14, 4, (32,), "f32")
    head = np.linalg.norm(got - ghw) / np.linalg.norm(ghw)
    print("\nper-layer weight-gradient rel. L2, bias rel. L2, cosine:")
    for l, r in enumerate(rels):
        print(f"  L{l:2d}: {r[0]:.2e} {r[1]:.2e} {r[2]:.6f}")
    print(f"  head: {head:.2e}")
    # the backward pass rounds each layer's pre-activation gradient to bf16, as
    # the reference does; a rounding that lands differently flips one bf16 value,
    # and such differences accumulate towards the input layer
    for l, (rw, rb, cos) in enumerate(rels):
        assert rw < 5e-2 and rb < 5e-2 and cos > 0.998, (l, rw, rb, cos)
    assert head < 1e-2
    assert abs(_param(torch, lib, params, 14, 5, (1,), "f32")[0] - ghb) <= 1e-2 * abs(ghb) + 1e-7


def test_unet_forward_matches_reference_and_is_deterministic(cuda):
    torch = cuda
    lib = _native.lib()
    nb, H, W = 1, 128, 64
    params, ws, wsb = _unet(torch, lib, nb, H, W, seed=9)
    rng = np.random.default_rng(6)
    inp = rng.standard_normal((nb, H, W, 2)).astype(np.float32)
    ti = torch.from_numpy(inp).cuda()
    outs = []
    for _ in range(2):
        out = torch.empty((nb, H, W), dtype=torch.float32, device="cuda")
        assert lib.ptycho_nn_unet_forward(_p(params), _p(ti), nb, H, W, _p(out), _p(ws), wsb,
                                          _stream(torch)) == 0
        outs.append(out.cpu().numpy())
    np.testing.assert_array_equal(outs[0], outs[1])
    want = ref.UNetReference(*_weights(torch, lib, params)).forward(inp)
    assert np.linalg.norm(outs[0] - want) <= 2e-2 * np.linalg.norm(want)


def test_unet_training_lowers_the_loss(cuda):
    torch = cuda
    lib = _native.lib()
    nb, H, W = 4, 64, 64
    params, ws, wsb = _unet(torch, lib, nb, H, W, seed=1)
    rng = np.random.default_rng(7)
    inp = rng.standard_normal((nb, H, W, 2)).astype(np.float32)
    # a target the network can represent: a smooth function of the inputs
    target = (0.5 * np.tanh(inp[..., 0]) - 0.2 * inp[..., 1] ** 2).astype(np.float32)
    ti, tt = torch.from_numpy(inp).cuda(), torch.from_numpy(target).cuda()
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    losses = []
    for step in range(1, 151):
        assert lib.ptycho_nn_unet_train_step(_p(params), _p(ti), _p(tt), None,
                                             float(nb * H * W), nb, H, W, 2e-3, step, _p(loss),
                                             _p(ws), wsb, _stream(torch)) == 0
        losses.append(float(loss.item()))
    assert lib.ptycho_nn_check(_p(ws), nb, H, W, _stream(torch)) == 0
    print(f"\nloss {losses[0]:.4f} -> {losses[-1]:.4f}")
    assert np.all(np.isfinite(losses))
    assert losses[-1] < 0.25 * losses[0]
