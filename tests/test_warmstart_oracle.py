"""CPU checks of the learned warm start's oracle (oracle/warmstart_net.py):
its vectorised 4D convolution against a direct loop, the parameter count,
bf16 rounding, finite differences against a hand-derived gradient, and the
analytic backward pass against finite differences."""
import numpy as np

from oracle import warmstart_net as W


def test_conv_matches_direct_loop():
    r = np.random.default_rng(0)
    for stride in (1, 2):
        R, ci, co = 4, 3, 2
        x = r.standard_normal((R, R, R, R, ci))
        w = r.standard_normal((81, ci, co))
        b = r.standard_normal(co)
        got = W.conv(x, w, b, 3, stride)
        Ro = R // stride
        want = np.zeros((Ro, Ro, Ro, Ro, co))
        for t in range(Ro):
            for z in range(Ro):
                for y in range(Ro):
                    for xx in range(Ro):
                        acc = b.copy()
                        for tap in range(81):
                            ox, oy, oz, ot = tap % 3, (tap // 3) % 3, (tap // 9) % 3, tap // 27
                            s = (t * stride + ot - 1, z * stride + oz - 1, y * stride + oy - 1,
                                 xx * stride + ox - 1)
                            if all(0 <= q < R for q in s):
                                acc = acc + x[s] @ w[tap]
                        want[t, z, y, xx] = acc
        assert np.allclose(got, want, rtol=1e-12, atol=1e-12)


def test_param_count_and_bf16():
    assert W.num_params() == sum((81 if k == 3 else 1) * a * b + b for a, b, k, *_ in W.LAYERS)
    # bf16 spacing at 1 is 2^-7: 1 + 2^-8 and 1 + 3 * 2^-8 are ties (to even)
    v = np.array([1.0, 1.00390625, 1.001953125, -3.14159, 1.01171875], np.float32)
    q = W.bf16_round(v)
    assert q[0] == 1.0 and q[1] == 1.0 and q[2] == 1.0
    assert q[3] == np.float32(-3.140625) and q[4] == np.float32(1.015625)


def test_fd_gradient_of_output_bias():
    """d loss / d bias of the output layer is 2 mean(pred - target) per channel."""
    r = np.random.default_rng(1)
    R = 4
    p = r.standard_normal(W.num_params()) * 0.05
    i0 = r.standard_normal((R,) * 4) * 0.01
    i1 = r.standard_normal((R,) * 4) * 0.01
    tgt = r.standard_normal((R,) * 4 + (4,))
    pred = W.forward(p, i0, i1)
    n = W.num_params()
    idx = [n - 4, n - 3, n - 2, n - 1]
    fd = W.fd_grad(p, i0, i1, tgt, idx)
    exact = 2.0 * (pred - tgt).reshape(-1, 4).sum(0) / pred.size
    assert np.allclose(fd, exact, rtol=1e-5, atol=1e-8)


def test_analytic_gradient_matches_finite_differences():
    """loss_and_grad (backpropagation) against central differences of the
    loss, for parameters of every layer, weights and biases."""
    r = np.random.default_rng(2)
    R = 4
    p = r.standard_normal(W.num_params()) * 0.05
    i0 = (r.standard_normal((R,) * 4) * 0.004).astype(np.float32)
    i1 = (r.standard_normal((R,) * 4) * 0.004).astype(np.float32)
    tgt = (r.standard_normal((R,) * 4 + (4,)) * 0.5).astype(np.float32)
    loss, g = W.loss_and_grad(p, i0, i1, tgt)
    assert abs(loss - W.loss(p, i0, i1, tgt)) <= 1e-12 * abs(loss)
    assert g.shape == (W.num_params(),)
    idx, off = [], 0
    for cin, cout, ks, *_ in W.LAYERS:
        nw = (81 if ks == 3 else 1) * cin * cout
        idx += list(off + r.choice(nw, 4, replace=False)) + [off + nw + int(r.integers(cout))]
        off += nw + cout
    fd = W.fd_grad(p, i0, i1, tgt, idx, rel=1e-4)
    assert np.abs(g[idx] - fd).max() <= 1e-7 * np.abs(fd).max() + 1e-12
