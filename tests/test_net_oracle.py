"""The numpy oracle of the pressure-guess network, on the CPU: BF16 rounding,
the adjoint identities of its convolution gradients, and its backward pass
against central finite differences in plain FP64."""
import numpy as np

from oracle import unet_oracle as U


def test_bf16_round_known_values():
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -2.5, 3.14159265, 65504.0, 1e-40])
    r = U.bf16_round(v)
    assert r[0] == 1.0
    assert r[1] == 1.0            # tie -> even
    assert r[2] == 1.0 + 2 ** -7  # above the tie -> up
    assert r[3] == -2.5
    assert r[4] == 3.140625
    assert r[5] == 65536.0
    # every result is exactly representable: low 16 bits of the FP32 pattern are zero
    assert np.all((r.astype(np.float32).view(np.uint32) & 0xFFFF) == 0)


def test_conv_gradient_adjoints():
    rng = np.random.default_rng(0)
    x = rng.normal(size=(16, 3, 4, 5))
    y = rng.normal(size=(32, 3, 4, 5))
    W = rng.normal(size=(27, 32, 16))
    lhs = np.sum(U.conv3(x, W) * y)
    assert abs(lhs - np.sum(x * U.conv3_dgrad(y, W))) < 1e-9 * abs(lhs) + 1e-9
    assert abs(lhs - np.sum(W * U.conv3_wgrad(x, y))) < 1e-9 * abs(lhs) + 1e-9


def test_pool_up_adjoint():
    rng = np.random.default_rng(1)
    c = rng.normal(size=(8, 2, 3, 4))
    f = rng.normal(size=(8, 4, 6, 8))
    assert abs(np.sum(U.up(c) * f) - np.sum(c * U.down_sum(f))) < 1e-10
    assert np.allclose(U.pool(U.up(c)), c)


def test_layout_roundtrip():
    a = np.arange(16 * 2 * 3 * 4, dtype=np.float64).reshape(16, 2, 3, 4)
    b = U.to_blocked(a)
    assert b.shape == (2, 2, 3, 4, 8)
    assert b[1, 1, 2, 3, 5] == a[13, 1, 2, 3]
    assert np.array_equal(U.from_blocked(b, 16), a)


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(2)
    p = U.init_params(5).astype(np.float64)
    in3 = rng.normal(size=(3, 16, 16, 16))
    gout = rng.normal(size=(16, 16, 16))
    net = U.UNet(p, bf16=False)
    net.forward(in3)
    g = net.backward(gout)
    d = rng.normal(size=p.size)
    h = 1e-8   # small enough that no ReLU input changes sign

    def loss(q):
        return float(np.sum(U.UNet(q, bf16=False).forward(in3) * gout))

    fd = (loss(p + h * d) - loss(p - h * d)) / (2 * h)
    an = float(np.dot(g, d))
    assert abs(fd - an) <= 1e-4 * max(abs(an), 1.0)
    # one layer at a time (a different random direction restricted to it)
    offs, hw, hb, n = U.param_layout()
    for l in (0, 4, 10):
        w, b = offs[l]
        dl = np.zeros(p.size)
        dl[w:b] = rng.normal(size=b - w)
        fd = (loss(p + h * dl) - loss(p - h * dl)) / (2 * h)
        an = float(np.dot(g, dl))
        assert abs(fd - an) <= 1e-4 * max(abs(an), 1.0), (l, fd, an)
