"""The learned warm start on the GPU: the network's forward pass and its
training gradients against the CPU oracle (oracle/warmstart_net.py,
finite differences), training, and the warm-started solve against the plain
one."""
import numpy as np
import pytest

import ofblend_gb300 as F
from ofblend_gb300 import synth, warmstart
from oracle import warmstart_net as W

pytestmark = pytest.mark.gpu


def rand_case(R, seed):
    r = np.random.default_rng(seed)
    i0 = (r.standard_normal((R,) * 4) * 0.004).astype(np.float32)
    i1 = (r.standard_normal((R,) * 4) * 0.004).astype(np.float32)
    tgt = (r.standard_normal((R,) * 4 + (4,)) * 0.5).astype(np.float32)
    return i0, i1, tgt


def grids(R, i0, i1, tgt):
    d = (R, R, R, R)
    return (F.Grid4Real(dims=d).from_numpy(i0), F.Grid4Real(dims=d).from_numpy(i1),
            F.Grid4Vec4(dims=d).from_numpy(tgt))


def test_forward_matches_oracle(gpu):
    R = 8
    m = F.Model(R, seed=3)
    p = W.bf16_round(m.get_params())  # the values the network computes with
    m.set_params(p)
    i0, i1, tgt = rand_case(R, 1)
    g0, g1, _ = grids(R, i0, i1, tgt)
    out = F.Grid4Vec4(dims=(R,) * 4)
    m.predict(g0, g1, out)
    want = W.forward(p, i0, i1)
    got = out.to_numpy()
    assert np.abs(got - want).max() <= 1e-4 * max(1.0, np.abs(want).max())


def test_gradients_match_finite_differences(gpu):
    R = 8
    m = F.Model(R, seed=4)
    p = W.bf16_round(m.get_params())
    m.set_params(p)
    i0, i1, tgt = rand_case(R, 2)
    loss, g = m.loss_grad(*grids(R, i0, i1, tgt))
    assert abs(loss - W.loss(p, i0, i1, tgt)) <= 1e-4 * abs(loss)
    # parameters from every layer (weights and biases)
    r = np.random.default_rng(5)
    idx, off = [], 0
    for cin, cout, ks, *_ in W.LAYERS:
        nw = (81 if ks == 3 else 1) * cin * cout
        idx += list(off + r.choice(nw, 3, replace=False)) + [off + nw + int(r.integers(cout))]
        off += nw + cout
    fd = W.fd_grad(p, i0, i1, tgt, idx)
    gg = g[idx].astype(np.float64)
    scale = np.abs(fd).max()
    assert np.abs(gg - fd).max() <= 2e-3 * scale + 1e-7, np.c_[gg, fd]


@pytest.mark.parametrize("R", [16, 12, 4])
def test_full_gradient_matches_oracle(gpu, R):
    """At the coarse extent the driver uses (16^4) every tensor-core shape
    runs: unsplit tiles with the bias and ReLU epilogue, split reductions, the
    two-channel first layer, stride-2 input gradients by parity class.  12^4
    has levels 12, 6 and 3 (no power of two); 4^4 has levels of extent 1,
    where every tap but the centre falls off the grid.  The forward pass and the whole
    gradient (every weight and bias) are compared with the oracle's analytic
    backward pass (itself checked against finite differences)."""
    m = F.Model(R, seed=8)
    p = W.bf16_round(m.get_params())
    m.set_params(p)
    i0, i1, tgt = rand_case(R, 3)
    g0, g1, gt = grids(R, i0, i1, tgt)
    out = F.Grid4Vec4(dims=(R,) * 4)
    m.predict(g0, g1, out)
    want = W.forward(p, i0, i1)
    assert np.abs(out.to_numpy() - want).max() <= 1e-4 * max(1.0, np.abs(want).max())
    loss, g = m.loss_grad(g0, g1, gt)
    wloss, wg = W.loss_and_grad(p, i0, i1, tgt)
    assert abs(loss - wloss) <= 1e-4 * abs(wloss)
    off = 0
    gnorm = np.linalg.norm(wg)  # a floor for blocks whose gradient is (nearly) zero
    for l, (cin, cout, ks, *_) in enumerate(W.LAYERS):
        for n in ((81 if ks == 3 else 1) * cin * cout, cout):  # weights, then biases
            a, b = g[off:off + n].astype(np.float64), wg[off:off + n]
            err = np.linalg.norm(a - b)
            assert err <= 1e-3 * np.linalg.norm(b) + 1e-7 * gnorm, (l, n, err, np.linalg.norm(b))
            off += n
    assert off == g.size


def test_training_reduces_loss(gpu):
    R = 8
    m = F.Model(R, seed=6)
    samples = [grids(R, *rand_case(R, 10 + k)) for k in range(4)]
    hist = warmstart.train(m, samples, epochs=30, batch=2, lr=3e-3)
    assert hist[-1] < 0.7 * hist[0], hist


def test_warm_start_in_the_solve(gpu):
    """A network trained on solver outputs of seeded pairs starts the coarsest
    level closer than zero for held-out pairs; the solve then refines as
    usual, and a model that does not help is dropped by the error check."""
    p = dict(wSmooth=0.001, wEnergy=0.0001, cgAccuracy=0.01, postVelBlur=4, cfl=999, multiStep=2,
             minGridSize=20, resetBndWidth=0.1)
    train_s = warmstart.make_samples(48, base_seed=20000, solve_params=p)
    m = F.Model(16, seed=7)
    hist = warmstart.train(m, train_s, epochs=25, batch=8, lr=2e-3)
    assert hist[-1] < 0.5 * hist[0], hist
    m.attach()
    dims = (32, 32, 32, 32)
    gains = []
    for k in range(4):
        s0, s1 = synth.random_pair_scenes(30000 + k)
        g0 = F.Grid4Real(dims=dims).from_numpy(synth.flow_input(s0, dims))
        g1 = F.Grid4Real(dims=dims).from_numpy(synth.flow_input(s1, dims))
        v = F.Grid4Vec4(dims=dims)
        F.opticalFlowMultiscale4d(v, g0, g1, warmStart=True, **p)
        st = F.last_solve_stats()
        e0, e1 = st["warm_start_err"]
        gains.append(e0 - e1)
        assert st["warm_start"] in (0, 1)
        assert st["warm_start"] == (1 if e1 < e0 else 0)
    print("coarse error gains (zero start - prediction):", gains)
    assert np.mean(gains) > 0, gains
    # an untrained model is no better than zero and gets dropped
    m.init(123)
    v = F.Grid4Vec4(dims=dims)
    F.opticalFlowMultiscale4d(v, g0, g1, warmStart=True, **p)
    st = F.last_solve_stats()
    assert st["warm_start"] == (1 if st["warm_start_err"][1] < st["warm_start_err"][0] else 0)
    m.detach()
