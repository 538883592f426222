"""The convolutional preconditioner (tcgen05 BF16 implicit-GEMM convolutions,
input gradients and weight gradients) against a float64 PyTorch reference
of the same network with BF16 rounding at the same points: inputs, weights,
activations and back-propagated gradients."""
import numpy as np
import pytest

import seismic_gb300 as sw
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
F = torch.nn.functional

# Relative L2 bound of forward outputs and weight gradients against the
# reference: the device sums in FP32 in another order, so a BF16 rounding
# of an activation or gradient lands on the other side now and then.
TOL = 5e-3


def _bf16(a):
    return torch.as_tensor(np.asarray(a, np.float32)).to(torch.bfloat16).to(torch.float64)


def _round_bf16(t):
    return t.to(torch.bfloat16).to(torch.float64)


def _unpack(w, channels, three_d=False):
    """Packed w[co][tap][ci], b[co] per layer -> torch (Cout, Cin, kx, kz) weights
    (tap = 3*(dx+1) + (dz+1)), or (Cout, Cin, ky, kx, kz) for 3 x 3 x 3 kernels
    (tap = 9*(dy+1) + 3*(dx+1) + (dz+1))."""
    taps = 27 if three_d else 9
    out, o = [], 0
    for cin, cout in zip(channels[:-1], channels[1:]):
        wl = w[o:o + cout * taps * cin].reshape((cout,) + (3,) * (3 if three_d else 2) + (cin,))
        o += cout * taps * cin
        b = w[o:o + cout]
        o += cout
        perm = (0, 4, 1, 2, 3) if three_d else (0, 3, 1, 2)
        out.append((np.transpose(wl, perm).copy(), b.copy()))
    return out


def _ref_forward(x, w, channels, requires_grad=False, three_d=False):
    """float64 reference of one image x (C, nx, nz) or volume (C, ny, nx, nz):
    BF16 inputs, weights and activations (straight-through), and with
    requires_grad the gradient reaching each layer's output rounded to BF16
    as the device stores it."""
    layers = _unpack(w, channels, three_d)
    conv = F.conv3d if three_d else F.conv2d
    h = _bf16(x)[None]
    params = []
    for l, (wl, b) in enumerate(layers):
        wt = _bf16(wl).requires_grad_(requires_grad)
        bt = torch.as_tensor(b, dtype=torch.float64).requires_grad_(requires_grad)
        params += [wt, bt]
        z = conv(h, wt, bt, padding=1)
        if requires_grad:
            z.register_hook(_round_bf16)
        if l + 1 < len(layers):
            a = torch.relu(z)
            h = a + (_round_bf16(a.detach()) - a.detach())
        else:
            h = z
    return h[0, 0], params


def _ref_gradient(x, t, w, channels, three_d=False):
    """Batch-mean gradient (packed like the weights) and loss."""
    perm = (0, 2, 3, 4, 1) if three_d else (0, 2, 3, 1)
    grads, losses = [], []
    for xi, ti in zip(x, t):
        out, params = _ref_forward(xi, w, channels, requires_grad=True, three_d=three_d)
        loss = 0.5 * torch.mean((out - torch.as_tensor(ti, dtype=torch.float64)) ** 2)
        loss.backward()
        g = []
        for wt, bt in zip(params[0::2], params[1::2]):
            g.append(np.transpose(wt.grad.numpy(), perm).ravel())  # [co][tap][ci]
            g.append(bt.grad.numpy().ravel())
        grads.append(np.concatenate(g))
        losses.append(float(loss))
    return np.mean(grads, axis=0), float(np.mean(losses))


@pytest.fixture(scope="module")
def image():
    rng = np.random.default_rng(4)
    nx, nz = 70, 53                       # not multiples of the 32 x 4 pixel tile
    return rng.standard_normal((2, nx, nz)).astype(np.float32)


@pytest.mark.parametrize("ch", [[2, 32, 32, 32, 1], [2, 16, 16, 16, 1], [3, 8, 24, 1]])
def test_cnn_forward_matches_reference(ctx, image, ch):
    rng = np.random.default_rng(len(ch))
    x = image if ch[0] == 2 else rng.standard_normal((ch[0],) + image.shape[1:]).astype(np.float32)
    net = sw.CNN(ctx, ch, seed=1)
    try:
        w = net.get_weights()
        out = net.forward(x)
    finally:
        net.close()
    ref, _ = _ref_forward(x, w, ch)
    err = rel_l2(out, ref.detach().numpy())
    print(f"cnn {ch} forward rel L2 {err:.2e}")
    assert np.abs(out).max() > 0
    assert err < TOL


@pytest.mark.parametrize("ch,shape", [([2, 32, 32, 32, 1], (70, 53)), ([2, 16, 8, 1], (3, 20)),
                                      ([2, 32, 1], (9, 200))])
def test_cnn_gradient_matches_reference(ctx, ch, shape):
    """Weight and bias gradients of the batch-mean loss (two images) on the
    tensor cores against float64 autograd of the same BF16-rounded network;
    the image shapes include one smaller than a 32 x 4 tile."""
    rng = np.random.default_rng(11)
    nx, nz = shape
    x = rng.standard_normal((2, ch[0], nx, nz)).astype(np.float32)
    t = rng.standard_normal((2, nx, nz)).astype(np.float32)
    net = sw.CNN(ctx, ch, seed=2)
    try:
        w = net.get_weights()
        g, loss = net.gradient(x, t)
        w_after = net.get_weights()
    finally:
        net.close()
    np.testing.assert_array_equal(w, w_after)      # the gradient call leaves the weights
    rg, rloss = _ref_gradient(x, t, w, ch)
    err = rel_l2(g, rg)
    print(f"cnn {ch} {shape} gradient rel L2 {err:.2e}, loss {loss:.6e} ref {rloss:.6e}")
    assert abs(loss - rloss) <= 1e-3 * rloss
    assert err < TOL
    # Every layer's block, not just the largest one.
    o = 0
    for cin, cout in zip(ch[:-1], ch[1:]):
        n = cout * 9 * cin + cout
        assert rel_l2(g[o:o + n], rg[o:o + n]) < 2 * TOL
        o += n


def test_cnn_adam_step_follows_the_gradient(ctx, image):
    """The first Adam step moves each weight by lr * g / (|g| + eps) with the
    gradient of the same batch."""
    ch = [2, 32, 32, 1]
    rng = np.random.default_rng(5)
    target = rng.standard_normal(image.shape[1:]).astype(np.float32)
    net = sw.CNN(ctx, ch, seed=2)
    try:
        w0 = net.get_weights()
        g, _ = net.gradient(image[None], target[None])
        lr = 1e-3
        net.train_step(image[None], target[None], lr=lr)
        w1 = net.get_weights()
    finally:
        net.close()
    expect = w0 - lr * g / (np.abs(g) + 1e-8)
    np.testing.assert_allclose(w1, expect, rtol=0, atol=2e-6)


def test_cnn_training_reduces_loss(ctx):
    """Learns a 3x3 smoothing of the first input channel."""
    rng = np.random.default_rng(6)
    nx, nz, nb = 48, 40, 4
    x = rng.standard_normal((nb, 2, nx, nz)).astype(np.float32)
    k = np.array([[1, 2, 1], [2, 4, 2], [1, 2, 1]], np.float32) / 16.0
    t = np.stack([F.conv2d(torch.as_tensor(x[i, :1])[None], torch.as_tensor(k)[None, None],
                           padding=1)[0, 0].numpy() for i in range(nb)])
    net = sw.CNN(ctx, [2, 32, 32, 1], seed=3)
    try:
        first = net.train_step(x, t, lr=3e-3)
        for _ in range(150):
            last = net.train_step(x, t, lr=3e-3)
    finally:
        net.close()
    assert np.isfinite(last) and last < first / 10


@pytest.mark.parametrize("ch,shape", [([2, 32, 32, 1], (5, 9, 37)), ([2, 16, 8, 1], (3, 4, 70))])
def test_cnn3d_forward_and_gradient_match_reference(ctx, ch, shape):
    """The 3 x 3 x 3 network on volumes (ny, nx, nz): forward output and the
    weight and bias gradients of a two-volume batch against float64 conv3d
    with the same BF16 rounding points."""
    rng = np.random.default_rng(21)
    ny, nx, nz = shape
    x = rng.standard_normal((2, ch[0], ny, nx, nz)).astype(np.float32)
    t = rng.standard_normal((2, ny, nx, nz)).astype(np.float32)
    net = sw.CNN(ctx, ch, seed=4, three_d=True)
    try:
        w = net.get_weights()
        assert w.size == sum(co * 27 * ci + co for ci, co in zip(ch[:-1], ch[1:]))
        out = net.forward(x[0])
        g, loss = net.gradient(x, t)
    finally:
        net.close()
    ref, _ = _ref_forward(x[0], w, ch, three_d=True)
    ferr = rel_l2(out, ref.detach().numpy())
    rg, rloss = _ref_gradient(x, t, w, ch, three_d=True)
    gerr = rel_l2(g, rg)
    print(f"cnn3d {ch} {shape} forward rel L2 {ferr:.2e}, gradient rel L2 {gerr:.2e}")
    assert np.abs(out).max() > 0
    assert ferr < TOL and gerr < TOL
    assert abs(loss - rloss) <= 1e-3 * rloss


def test_cnn3d_training_reduces_loss(ctx):
    """A 3 x 3 x 3 network learns a 3 x 3 x 3 smoothing of its first channel."""
    rng = np.random.default_rng(7)
    nb, ny, nx, nz = 2, 6, 10, 40
    x = rng.standard_normal((nb, 2, ny, nx, nz)).astype(np.float32)
    k = np.ones((3, 3, 3), np.float32) / 27.0
    t = np.stack([F.conv3d(torch.as_tensor(x[i, :1])[None], torch.as_tensor(k)[None, None],
                           padding=1)[0, 0].numpy() for i in range(nb)])
    net = sw.CNN(ctx, [2, 16, 16, 1], seed=3, three_d=True)
    try:
        first = net.train_step(x, t, lr=3e-3)
        for _ in range(120):
            last = net.train_step(x, t, lr=3e-3)
    finally:
        net.close()
    assert np.isfinite(last) and last < first / 10


def test_cnn_image_and_volume_entry_points_do_not_mix(ctx):
    net2, net3 = sw.CNN(ctx, [2, 8, 1]), sw.CNN(ctx, [2, 8, 1], three_d=True)
    try:
        with pytest.raises(sw.SwaveError):
            net3.three_d = False
            net3.forward(np.zeros((2, 5, 40), np.float32))
        with pytest.raises(sw.SwaveError):
            net2.three_d = True
            net2.forward(np.zeros((2, 3, 5, 40), np.float32))
    finally:
        net2.close()
        net3.close()


def test_cnn_rejects_more_than_32_channels(ctx):
    with pytest.raises(sw.SwaveError) as e:
        sw.CNN(ctx, [2, 33, 1])
    assert e.value.code == sw.SW_BAD_PARAM
