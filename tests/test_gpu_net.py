"""The learned pressure guess on the GPU: tcgen05 descriptor layouts, single
convolutions (forward, data gradient, weight gradient) and the whole U-Net's
forward output and parameter gradients against the numpy oracle
(oracle/unet_oracle.py, run with the same BF16 roundings)."""
import numpy as np
import pytest

from oracle import unet_oracle as U

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def netmod():
    from turbins_gb300 import build
    build.build()
    from turbins_gb300 import net as N
    return N


def _rel(a, b):
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / max(np.linalg.norm(np.ravel(b)), 1e-30))


@pytest.mark.parametrize("mn", [0, 1])
def test_umma_descriptor_layouts(netmod, mn):
    bad = netmod.selftest_umma(mn, 0)
    if bad:
        other = netmod.selftest_umma(mn, 1)
        pytest.fail("mn_major=%d: %d wrong results (%d with LBO/SBO exchanged)" % (mn, bad, other))


@pytest.mark.parametrize("shift", [0, 1, 2, 3, 5, 7])
def test_umma_swizzle128_row_shift(netmod, shift):
    assert netmod.selftest_umma(2, shift) == 0


def test_bounded_wait_times_out_and_context_survives(netmod):
    """A completion wait that nothing satisfies gives up after its limit
    (about 1 s) with an error count instead of hanging; the next launch on the
    same context works."""
    import time
    t0 = time.time()
    bad = netmod.selftest_umma(0, 2)
    assert bad >= 1000000
    assert time.time() - t0 < 30
    assert netmod.selftest_umma(0, 0) == 0


def _bf16_dev(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).to(torch.bfloat16).cuda()


def _to_np(t):
    return t.float().cpu().numpy().astype(np.float64)


CONV_SHAPES = [(128, 4, 3, 16, 32), (256, 2, 2, 32, 16), (32, 8, 4, 64, 128), (8, 4, 4, 128, 64),
               (4, 2, 2, 32, 32), (200, 3, 2, 16, 16)]


@pytest.mark.parametrize("X,Y,Z,cin,cout", CONV_SHAPES)
def test_conv_forward_and_dgrad(netmod, X, Y, Z, cin, cout):
    rng = np.random.default_rng(X * 7 + cin)
    x = U.bf16_round(rng.normal(size=(cin, Z, Y, X)))
    W = rng.normal(0, 0.2, size=(27, cout, cin)).astype(np.float32)
    b = rng.normal(0, 0.1, size=cout).astype(np.float32)
    Wq = U.bf16_round(W)
    xd = _bf16_dev(U.to_blocked(x))
    out = torch.zeros((cout // 8, Z, Y, X, 8), dtype=torch.bfloat16, device="cuda")
    netmod.conv3(X, Y, Z, cin, cout, xd, torch.from_numpy(W).cuda(), torch.from_numpy(b).cuda(), relu=True, out=out)
    got = U.from_blocked(_to_np(out), cout)
    ref = np.maximum(U.conv3(x, Wq, b.astype(np.float64)), 0.0)
    scale = np.abs(ref).max()
    assert np.all(np.abs(got - ref) <= 2.0 ** -8 * np.abs(ref) + 1e-5 * scale)
    # data gradient: dy has cout channels, dx cin
    dy = U.bf16_round(rng.normal(size=(cout, Z, Y, X)))
    dx = torch.zeros((cin // 8, Z, Y, X, 8), dtype=torch.bfloat16, device="cuda")
    netmod.conv3(X, Y, Z, cin, cout, _bf16_dev(U.to_blocked(dy)), torch.from_numpy(W).cuda(), dgrad=True, out=dx)
    got = U.from_blocked(_to_np(dx), cin)
    ref = U.conv3_dgrad(dy, Wq)
    scale = np.abs(ref).max()
    assert np.all(np.abs(got - ref) <= 2.0 ** -8 * np.abs(ref) + 1e-5 * scale)


@pytest.mark.parametrize("X,Y,Z,cin,cout", [(128, 4, 3, 16, 32), (32, 8, 4, 64, 128), (4, 2, 2, 128, 64),
                                            (16, 8, 8, 32, 16), (48, 4, 2, 16, 16)])
def test_conv_wgrad(netmod, X, Y, Z, cin, cout):
    rng = np.random.default_rng(X + cin * 3 + cout)
    x = U.bf16_round(rng.normal(size=(cin, Z, Y, X)))
    dy = U.bf16_round(rng.normal(size=(cout, Z, Y, X)))
    dw = torch.zeros((27, cout, cin), dtype=torch.float32, device="cuda")
    netmod.conv3_wgrad(X, Y, Z, cin, cout, _bf16_dev(U.to_blocked(x)), _bf16_dev(U.to_blocked(dy)), dw)
    ref = U.conv3_wgrad(x, dy)
    got = dw.cpu().numpy().astype(np.float64)
    # FP32 sums of exact BF16 products: bounded by the sum of |terms|
    bound = 1e-5 * U.conv3_wgrad(np.abs(x), np.abs(dy)) + 1e-6
    assert np.all(np.abs(got - ref) <= bound)


@pytest.mark.parametrize("dims", [(32, 16, 16), (128, 16, 16)])
def test_net_forward_backward_vs_oracle(netmod, dims):
    """Forward: every activation of the GPU against the oracle layer applied to
    the GPU's own input of that layer, and the output.  Backward: the oracle's
    backward run on the GPU's activations (so both see the same ReLU masks)
    against the GPU gradients."""
    nx, ny, nz = dims
    rng = np.random.default_rng(nx + 1)
    p = U.init_params(3)
    in3 = rng.normal(size=(3, nz, ny, nx)).astype(np.float32).astype(np.float64)
    gout = (1.0 + 0.5 * rng.normal(size=(nz, ny, nx))).astype(np.float32).astype(np.float64)
    net = netmod.Net(nx, ny, nz, train=True)
    net.set_params(p)
    dout = torch.zeros((nz, ny, nx), dtype=torch.float32, device="cuda")
    net.forward(torch.from_numpy(in3.astype(np.float32)).cuda(), dout)
    net.backward(torch.from_numpy(gout.astype(np.float32)).cuda())
    g = net.get_grads().astype(np.float64)
    A = {k: net.activation(k) for k in net.ACTS}
    orc = U.UNet(p, bf16=True)
    ref_out = orc.forward(in3)
    assert _rel(dout.cpu().numpy(), ref_out) < 1e-2
    # layer by layer on the GPU's own inputs: within one BF16 rounding
    Wq, bs, r = orc.Wq, orc.bs, U.bf16_round
    chain = [("a0", 0, "x0", True), ("a1", 1, "p0", True), ("a2", 2, "p1", True), ("a3", 3, "p2", True),
             ("b3", 4, "a3", True), ("c2", 5, "b3", False), ("b2", 6, "s2", True), ("c1", 7, "b2", False),
             ("b1", 8, "s1", True), ("c0", 9, "b1", False), ("b0", 10, "s0", True)]
    for out_name, l, in_name, relu in chain:
        z = U.conv3(A[in_name], Wq[l], bs[l])
        ref = r(np.maximum(z, 0.0) if relu else z)
        err = np.abs(A[out_name] - ref)
        assert np.all(err <= 2.0 ** -7 * np.abs(ref) + 1e-5 * np.abs(ref).max()), out_name
    for got, ref in ((A["p0"], r(U.pool(A["a0"]))), (A["s2"], r(np.maximum(U.up(A["c2"]) + A["a2"], 0.0)))):
        assert np.all(np.abs(got - ref) <= 2.0 ** -8 * np.abs(ref))
    head = np.einsum("c,czyx->zyx", orc.hw, A["b0"]) + orc.hb
    assert np.abs(dout.cpu().numpy() - head).max() <= 1e-5 * np.abs(head).max()
    # backward on the same activations
    orc.A = A
    ref_g = orc.backward(gout)
    offs, hw, hb, n = U.param_layout()
    for l, (w, b) in enumerate(offs):
        cin, cout, _ = U.LAYERS[l]
        e_w = _rel(g[w:w + 27 * cin * cout], ref_g[w:w + 27 * cin * cout])
        e_b = _rel(g[b:b + cout], ref_g[b:b + cout])
        assert e_w < 1e-2 and e_b < 1e-2, (l, e_w, e_b)
    assert _rel(g[hw:hw + 17], ref_g[hw:hw + 17]) < 1e-4
    net.close()


def test_adam_matches_oracle(netmod):
    """Three Adam steps of the library (k_adam, FP32) on the gradients of its
    own backward pass against the oracle's Adam in float64: each parameter
    within 1e-3 of the step size lr plus 4 FP32 ulps of its value."""
    nx, ny, nz = 32, 16, 16
    rng = np.random.default_rng(3)
    net = netmod.Net(nx, ny, nz, train=True)
    p = U.init_params(2).astype(np.float32)
    net.set_params(p)
    opt = U.Adam(p.size)
    ref = p.astype(np.float64)
    out = torch.zeros((nz, ny, nx), dtype=torch.float32, device="cuda")
    for step, lr in enumerate((1e-3, 1e-3, 2.5e-4)):
        in3 = torch.from_numpy(rng.normal(size=(3, nz, ny, nx)).astype(np.float32)).cuda()
        gout = torch.from_numpy((1.0 + rng.normal(size=(nz, ny, nx))).astype(np.float32)).cuda()
        net.forward(in3, out)
        net.backward(gout)
        g = net.get_grads()
        assert np.count_nonzero(g) > g.size // 2
        net.adam(lr)
        got = net.get_params().astype(np.float64)
        ref = opt.step(ref, g, lr)
        tol = 1e-3 * lr + 4 * np.spacing(np.abs(ref).astype(np.float32)).astype(np.float64)
        bad = np.abs(got - ref) > tol
        assert not bad.any(), (step, int(bad.sum()), float(np.abs(got - ref).max()))
        ref = got          # continue from the library's FP32 parameters
    assert opt.t == 3
    net.close()
