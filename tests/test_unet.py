"""Learned warm start (include/plume_net.h): the CUDA U-Net's forward pass and
gradients against the CPU restatement in oracle/unet_oracle.py, training on
GPU-generated pairs, and its use inside the step (a solve that starts from the
network's guess still meets the plain stop test, and falls back to p = 0 when
it does not converge)."""
import numpy as np
import pytest

from cfs_plume_gb300 import _abi
from oracle import unet_oracle as uo

RES = (16, 12, 8)


def random_params(seed, scale=1.0):
    """He-scaled random weights and small random biases in the parameter layout."""
    rng = np.random.default_rng(seed)
    parts = []
    for name, ci, co, _ in uo.LAYERS:
        fan = 27 * (1 if name == "e1a" else ci)
        w = rng.standard_normal((27, ci, co)) * np.sqrt(2.0 / fan) * scale
        if name == "e1a":
            w[:, 1:, :] = 0.0
        parts += [w.ravel(), 0.05 * rng.standard_normal(co)]
    parts += [rng.standard_normal(16) * 0.25, [0.01]]
    return np.concatenate(parts).astype(np.float32)


def smooth_field(rng, res, batch):
    """Random fields with some spatial correlation (a 3-point box blur of noise)."""
    X, Y, Z = res
    a = rng.standard_normal((batch, Z, Y, X))
    for ax in (1, 2, 3):
        a = (np.roll(a, 1, ax) + a + np.roll(a, -1, ax)) / 3.0
    return a.reshape(batch, -1)


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, float) - b) / max(np.linalg.norm(b), 1e-300))


def test_param_count_and_layout():
    assert uo.num_params() == 27 * 13312 + 320 + 17
    p = random_params(0)
    assert p.size == uo.num_params()
    np.testing.assert_array_equal(uo.pack(uo.unpack(p)), p.astype(np.float64))


@pytest.mark.parametrize("loss", ["mse", "energy"])
def test_oracle_gradient_matches_finite_differences(loss):
    """The restated backward pass (float64, no rounding) against central
    differences of the restated forward pass."""
    res, batch = (8, 8, 8), 2
    rng = np.random.default_rng(1)
    params = random_params(2).astype(np.float64)
    inp = smooth_field(rng, res, batch)
    tgt = smooth_field(rng, res, batch)
    o = uo.UNetOracle(params, bf16=False)
    L = lambda q: uo.UNetOracle(q, bf16=False).loss_grad(inp, tgt, res, batch, loss=loss)[0]
    _, grad = o.loss_grad(inp, tgt, res, batch, loss=loss)
    # parameters spread over every layer, each with a gradient well above round-off
    checked = 0
    offsets = np.cumsum([0] + [27 * ci * co + co for _, ci, co, _ in uo.LAYERS])
    for l, (name, ci, co, _) in enumerate(uo.LAYERS):
        lo = offsets[l]
        span = np.arange(lo, lo + 27 * ci * co + co)
        if name == "e1a":  # only input channel 0 is live
            w = np.arange(27 * ci * co).reshape(27, ci, co)[:, 0, :].ravel()
            span = np.concatenate([lo + w, np.arange(lo + 27 * ci * co, lo + 27 * ci * co + co)])
        cand = span[np.argsort(-np.abs(grad[span]))[:3]]
        for k in cand:
            h = 1e-6 * max(1.0, abs(params[k]))
            pp, pm = params.copy(), params.copy()
            pp[k] += h
            pm[k] -= h
            fd = (L(pp) - L(pm)) / (2 * h)
            assert abs(fd - grad[k]) <= 1e-4 * abs(grad[k]) + 1e-9, (name, int(k - lo), fd, grad[k])
            checked += 1
    for k in (offsets[-1], offsets[-1] + 16):  # output layer weight and bias
        h = 1e-6
        pp, pm = params.copy(), params.copy()
        pp[k] += h
        pm[k] -= h
        fd = (L(pp) - L(pm)) / (2 * h)
        assert abs(fd - grad[k]) <= 1e-4 * abs(grad[k]) + 1e-9
        checked += 1
    assert checked == 32


@pytest.fixture(scope="module")
def net():
    from cfs_plume_gb300.net import PlumeNet
    n = PlumeNet(seed=3)
    yield n
    n.close()


@pytest.mark.gpu
def test_forward_matches_oracle(net):
    """BF16 tensor-core forward pass against the restatement with the same
    rounding points; relative L2 tolerance 1e-2 (BF16 has 8 significant bits;
    the two sides accumulate in different orders)."""
    batch = 2
    params = random_params(4)
    net.params = params
    rng = np.random.default_rng(5)
    inp = smooth_field(rng, RES, batch).astype(np.float32)
    y = net.forward(inp, RES)
    ref, _ = uo.UNetOracle(params).forward(inp, RES, batch)
    assert rel(y, ref) < 1e-2
    np.testing.assert_array_equal(net.params, params)


@pytest.mark.gpu
@pytest.mark.parametrize("loss", ["mse", "energy"])
def test_gradients_match_oracle(net, loss):
    """Loss and every layer's weight and bias gradient of the CUDA backward
    pass against the restatement with the same BF16 rounding points: relative
    L2 per tensor <= 1e-2, and closer to it than BF16 rounding itself moves the
    gradient (the restatement without rounding, in float64)."""
    batch = 2
    params = random_params(8)
    net.params = params
    rng = np.random.default_rng(9)
    inp = smooth_field(rng, RES, batch).astype(np.float32)
    tgt = smooth_field(rng, RES, batch).astype(np.float32)
    from cfs_plume_gb300.net import LOSS_ENERGY, LOSS_MSE
    value, grad = net.loss_grad(inp, tgt, RES, loss=LOSS_ENERGY if loss == "energy" else LOSS_MSE)
    lref, gref = uo.UNetOracle(params).loss_grad(inp, tgt, RES, batch, loss=loss)
    _, gexact = uo.UNetOracle(params, bf16=False).loss_grad(inp, tgt, RES, batch, loss=loss)
    assert abs(value - lref) <= 1e-4 * lref
    k = 0
    for name, ci, co, _ in uo.LAYERS:
        nw = 27 * ci * co
        for part, s in (("w", slice(k, k + nw)), ("b", slice(k + nw, k + nw + co))):
            err = rel(grad[s], gref[s])
            # the energy loss weights high frequencies, where the gradient is a
            # difference of large terms and rounding flips count for more
            assert err < (1e-2 if loss == "mse" else 5e-2), (name, part, err)
            assert err < rel(gref[s], gexact[s]), (name, part)
        k += nw + co
    assert rel(grad[k:], gref[k:]) < 1e-3, "out"


@pytest.mark.gpu
def test_gradients_are_deterministic(net):
    net.params = random_params(6)
    rng = np.random.default_rng(7)
    inp = smooth_field(rng, RES, 2).astype(np.float32)
    tgt = smooth_field(rng, RES, 2).astype(np.float32)
    l1, g1 = net.loss_grad(inp, tgt, RES)
    l2, g2 = net.loss_grad(inp, tgt, RES)
    assert l1 == l2
    np.testing.assert_array_equal(g1, g2)


@pytest.mark.gpu
@pytest.mark.parametrize("kind", [0, 1, 2])
def test_pairs_are_normalised_solves(kind):
    """Generated pairs: the input has unit rms over interior cells and the
    target solves A x = input to the stop test -- for solve pairs (b, p), for
    correction pairs (r0 = b - A p_prev, p - p_prev), since
    A (p - p_prev) = b - A p_prev, and for iterate pairs (r_k = b - A x_k,
    p - x_k) with x_k a truncated solve's iterate."""
    from cfs_plume_gb300.net import PairStore
    res = (16, 24, 16)
    ds = PairStore(res, plumes=2, steps=4, skip=1, threads=2, seed=11, kind=kind)
    assert ds.pairs == 6
    X, Y, Z = res
    for i in (0, 5):
        b, p = ds.pair(i)
        b = b.reshape(Z, Y, X)
        p = p.reshape(Z, Y, X).astype(np.float64)
        bi = b[1:-1, 1:-1, 1:-1]
        assert abs(np.sqrt((bi.astype(np.float64) ** 2).mean()) - 1.0) < 1e-2
        assert np.all(b[0] == 0) and np.all(p[:, :, 0] == 0)
        # residual of the 7-point operator with closed walls (missing
        # neighbours on the border drop out of both the diagonal and the sum)
        q = np.zeros_like(p)
        inner = np.zeros_like(p, dtype=bool)
        inner[1:-1, 1:-1, 1:-1] = True
        diag = np.zeros_like(p)
        for ax in range(3):
            for s in (1, -1):
                nb = np.roll(inner, s, ax)
                q += np.where(inner & nb, np.roll(p, s, ax), 0.0)
                diag += (inner & nb)
        r = (bi - (diag * p - q)[1:-1, 1:-1, 1:-1])
        assert np.linalg.norm(r) <= 2e-2 * np.linalg.norm(bi)
    ds.close()


@pytest.mark.gpu
def test_training_reduces_loss():
    from cfs_plume_gb300.net import PairStore, PlumeNet
    res = (16, 24, 16)
    ds = PairStore(res, plumes=4, steps=10, skip=2, threads=4, seed=21)
    n = PlumeNet(seed=1)
    tl, vl, secs = n.train(ds, epochs=6, batch=4, val_pairs=8, lr=2e-3, lr_final=2e-4, seed=3)
    assert np.all(np.isfinite(tl)) and np.all(np.isfinite(vl))
    assert tl[-1] < 0.7 * tl[0], tl
    assert abs(n.scale - ds.target_rms) <= 1e-6 * ds.target_rms
    n.close()
    ds.close()


def _step_pair(res, net, steps, **kw):
    from cfs_plume_gb300.plume import Plume
    plain = Plume(_abi.plume_config(res, **kw))
    learned = Plume(_abi.plume_config(res, warm_start=_abi.WARM_LEARNED, **kw))
    net.attach(learned)
    sp, sl = [], []
    for s in range(steps):
        plain.add_source(s)
        sp.append(plain.step())
        learned.add_source(s)
        sl.append(learned.step())
    out = (plain.field("velocity"), learned.field("velocity"), sp, sl)
    plain.close()
    learned.close()
    return out


@pytest.mark.gpu
def test_learned_start_meets_the_plain_stop_test(net):
    """Every learned-start solve reaches the same rel-L2 1e-6 residual, and the
    velocity stays within 1e-4 relative L2 of the zero-start run."""
    net.params = random_params(12, scale=0.5)
    net.scale = 1.0
    vp, vl, sp, sl = _step_pair((32, 48, 32), net, 4)
    for a, b in zip(sp, sl):
        assert a.converged and b.converged and not b.fallback
        assert b.rel_residual <= 1e-6
    assert rel(vl, vp) < 1e-4


@pytest.mark.gpu
def test_learned_start_falls_back_to_plain(net):
    """With an iteration cap the learned-start solve cannot converge: the step
    reruns plain MIC-PCG from p = 0, flags the fallback and gives the plain
    run's fields bit for bit."""
    net.params = random_params(13)
    net.scale = 1.0
    vp, vl, sp, sl = _step_pair((32, 48, 32), net, 2, max_iters=3)
    assert all(s.fallback for s in sl) and not any(s.fallback for s in sp)
    np.testing.assert_array_equal(vl, vp)


WEIGHTS = __import__("os").path.join(__import__("os").path.dirname(__import__("os").path.dirname(
    __import__("os").path.abspath(__file__))), "cfs_plume_gb300", "weights", "unet_warmstart.bin")


@pytest.mark.gpu
def test_trained_network_saves_iterations():
    """The committed network (trained on 20k correction pairs of 64x96x64
    plumes with the energy loss) against the zero start on an unseen 64x96x64
    plume: fewer
    PCG iterations per step, every solve meeting the same rel-L2 1e-6 test
    without fallback, velocity within 1e-4 relative L2."""
    from cfs_plume_gb300.net import PlumeNet
    n = PlumeNet(path=WEIGHTS)
    vp, vl, sp, sl = _step_pair((64, 96, 64), n, 12)
    n.close()
    ip = np.mean([s.iterations for s in sp[2:]])
    il = np.mean([s.iterations for s in sl[2:]])
    assert not any(s.fallback for s in sl)
    assert all(s.converged and s.rel_residual <= 1e-6 for s in sl)
    assert il < 0.85 * ip, (il, ip)
    assert rel(vl, vp) < 1e-4


@pytest.mark.gpu
def test_tile_shapes_give_identical_outputs(monkeypatch):
    """The autotuner's tile shape never changes a result: the forward pass
    with tuning (fastest shape per layer) equals the fixed smallest shape bit
    for bit."""
    from cfs_plume_gb300.net import PlumeNet
    params = random_params(10)
    rng = np.random.default_rng(11)
    res = (32, 48, 32)
    inp = smooth_field(rng, res, 2).astype(np.float32)
    outs = []
    for off in (True, False):
        if off:
            monkeypatch.setenv("PLUME_CONV_TUNE_OFF", "1")
        else:
            monkeypatch.delenv("PLUME_CONV_TUNE_OFF", raising=False)
        n = PlumeNet(seed=0)
        n.params = params
        outs.append(n.forward(inp, res))
        n.close()
    np.testing.assert_array_equal(outs[0], outs[1])


@pytest.mark.gpu
def test_tcgen05_convolution_matches_mma_sync(monkeypatch):
    """The tensor-core (tcgen05) convolutions against the mma.sync ones on the
    same BF16 inputs and weights: relative L2 below 1e-2 for the whole forward
    pass, the bound of the oracle comparison (both accumulate 27*CIN products
    in FP32, in different orders, and every layer rounds its output to BF16,
    so single elements move by a BF16 ulp and ten layers carry it on), on a
    grid whose edges cut the 16 x 8 x 2 output bricks."""
    from cfs_plume_gb300.net import PlumeNet
    params = random_params(12)
    rng = np.random.default_rng(13)
    res = (36, 44, 28)
    inp = smooth_field(rng, res, 2).astype(np.float32)
    outs = []
    for tc in ("0", "1"):
        monkeypatch.setenv("PLUME_CONV_TC", tc)
        n = PlumeNet(seed=0)
        n.params = params
        outs.append(n.forward(inp, res))
        n.close()
    assert rel(outs[1], outs[0]) < 1e-2, rel(outs[1], outs[0])
