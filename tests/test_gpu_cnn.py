"""The convolutional preconditioner (tcgen05 BF16 implicit-GEMM convolutions)
against a float64 PyTorch reference of the same BF16-rounded network."""
import numpy as np
import pytest

import seismic_gb300 as sw
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
F = torch.nn.functional


def _bf16(a):
    return torch.as_tensor(np.asarray(a, np.float32)).to(torch.bfloat16).to(torch.float64)


def _unpack(w, channels):
    """Packed w[co][tap][ci], b[co] per layer -> torch (Cout, Cin, kx, kz) weights."""
    out, o = [], 0
    for cin, cout in zip(channels[:-1], channels[1:]):
        wl = w[o:o + cout * 9 * cin].reshape(cout, 3, 3, cin)   # tap = 3*(dx+1) + (dz+1)
        o += cout * 9 * cin
        b = w[o:o + cout]
        o += cout
        out.append((np.transpose(wl, (0, 3, 1, 2)).copy(), b.copy()))
    return out


def _ref_forward(x, w, channels, requires_grad=False):
    """float64 reference; x (C, nx, nz); BF16 weights and activations like the GPU."""
    layers = _unpack(w, channels)
    h = _bf16(x)[None]
    params = []
    for l, (wl, b) in enumerate(layers):
        wt = _bf16(wl).requires_grad_(requires_grad)
        bt = torch.as_tensor(b, dtype=torch.float64).requires_grad_(requires_grad)
        params += [wt, bt]
        z = F.conv2d(h, wt, bt, padding=1)
        if l + 1 < len(layers):
            a = torch.relu(z)
            # activations are rounded to BF16 on the GPU (straight-through here)
            h = a + (a.detach().to(torch.bfloat16).to(torch.float64) - a.detach())
        else:
            h = z
    return h[0, 0], params


@pytest.fixture(scope="module")
def image():
    rng = np.random.default_rng(4)
    nx, nz = 70, 53                       # not multiples of the 128-pixel tile
    x = rng.standard_normal((2, nx, nz)).astype(np.float32)
    return x


def test_cnn_forward_matches_reference(ctx, image):
    ch = [2, 16, 16, 16, 1]
    net = sw.CNN(ctx, ch, seed=1)
    try:
        w = net.get_weights()
        out = net.forward(image)
    finally:
        net.close()
    ref, _ = _ref_forward(image, w, ch)
    assert np.abs(out).max() > 0
    assert rel_l2(out, ref.detach().numpy()) < 2e-2


def test_cnn_gradient_signs_after_one_adam_step(ctx, image):
    """The first Adam step moves each weight by lr * sign(gradient); the signs
    match the float64 autograd gradient wherever it is not tiny."""
    ch = [2, 8, 1]
    net = sw.CNN(ctx, ch, seed=2)
    rng = np.random.default_rng(5)
    target = rng.standard_normal(image.shape[1:]).astype(np.float32)
    try:
        w0 = net.get_weights()
        lr = 1e-3
        net.train_step(image[None], target[None], lr=lr)
        w1 = net.get_weights()
    finally:
        net.close()
    out, params = _ref_forward(image, w0, ch, requires_grad=True)
    loss = 0.5 * torch.mean((out - torch.as_tensor(target, dtype=torch.float64)) ** 2)
    loss.backward()
    g = []
    for (wt, bt) in zip(params[0::2], params[1::2]):
        gw = wt.grad.numpy()                               # (Cout, Cin, 3, 3)
        g.append(np.transpose(gw, (0, 2, 3, 1)).ravel())  # back to [co][tap][ci]
        g.append(bt.grad.numpy().ravel())
    g = np.concatenate(g)
    step = (w0 - w1) / lr
    big = np.abs(g) > 1e-3 * np.abs(g).max()
    assert big.sum() > 0.5 * g.size
    agree = np.mean(np.sign(step[big]) == np.sign(g[big]))
    assert agree > 0.98


def test_cnn_training_reduces_loss(ctx):
    """Learns a 3x3 smoothing of the first input channel."""
    rng = np.random.default_rng(6)
    nx, nz, nb = 48, 40, 4
    x = rng.standard_normal((nb, 2, nx, nz)).astype(np.float32)
    k = np.array([[1, 2, 1], [2, 4, 2], [1, 2, 1]], np.float32) / 16.0
    t = np.stack([F.conv2d(torch.as_tensor(x[i, :1])[None], torch.as_tensor(k)[None, None],
                           padding=1)[0, 0].numpy() for i in range(nb)])
    net = sw.CNN(ctx, [2, 16, 16, 1], seed=3)
    try:
        first = net.train_step(x, t, lr=3e-3)
        for _ in range(150):
            last = net.train_step(x, t, lr=3e-3)
    finally:
        net.close()
    assert np.isfinite(last) and last < first / 10
