"""The tensor-core MLP (forward, backward, Adam training, site features and
site sums) against the CPU oracle oracle/mlp_oracle.py.

The oracle applies BF16 rounding at the same points as the GPU, so gradients
agree to FP32 accumulation order: relative norm 2e-3 per parameter block, loss
1e-5. Forward outputs: 2e-3 of the largest output.
"""
import numpy as np
import pytest

import leo2d_gb300 as L
from oracle import mlp_oracle as mo
from oracle import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    with L.Context(0) as c:
        yield c


def _blocks():
    off = 0
    for l, d in enumerate(mo.IN_DIM):
        yield f"W{l}", off, off + mo.HID * d
        off += mo.HID * d
        yield f"b{l}", off, off + mo.HID
        off += mo.HID


@pytest.mark.parametrize("n", [64, 256, 1024])
def test_grad_matches_oracle(ctx, n):
    rng = np.random.default_rng(n)
    m = L.Mlp(ctx, seed=3)
    p = m.params()
    assert p.size == mo.param_count()
    x = rng.uniform(-1, 1, (n, mo.N_FEAT)).astype(np.float32)
    t = rng.normal(0, 0.3, (n, mo.OUT)).astype(np.float32)
    loss, g = m.grad(x, t)
    lref, gref = mo.loss_and_grad(p, x, t)
    assert abs(loss - lref) <= 1e-5 * lref
    for name, a, b in _blocks():
        ref = gref[a:b]
        err = np.linalg.norm(g[a:b] - ref) / max(np.linalg.norm(ref), 1e-30)
        assert err < 2e-3, (name, err)
    m.close()


def test_grad_with_loss_weights(ctx):
    rng = np.random.default_rng(7)
    m = L.Mlp(ctx, seed=11)
    w = rng.uniform(0.1, 3.0, mo.OUT).astype(np.float32)
    m.set_loss_weights(w)
    x = rng.uniform(-1, 1, (128, mo.N_FEAT)).astype(np.float32)
    t = rng.normal(0, 0.3, (128, mo.OUT)).astype(np.float32)
    loss, g = m.grad(x, t)
    lref, gref = mo.loss_and_grad(m.params(), x, t, w)
    assert abs(loss - lref) <= 1e-5 * lref
    assert np.linalg.norm(g - gref) / np.linalg.norm(gref) < 2e-3
    m.close()


def test_predict_matches_oracle(ctx):
    rng = np.random.default_rng(5)
    m = L.Mlp(ctx, seed=9)
    x = rng.uniform(-1, 1, (1000, mo.N_FEAT)).astype(np.float32)
    y = m.predict(x)
    ref = mo.forward(m.params(), x)
    assert np.max(np.abs(y - ref)) <= 2e-3 * np.max(np.abs(ref))
    m.close()


def test_set_params_roundtrip(ctx):
    m = L.Mlp(ctx, seed=1)
    p = np.random.default_rng(2).normal(0, 0.05, m.n_params).astype(np.float32)
    m.set_params(p)
    np.testing.assert_array_equal(m.params(), p)
    with pytest.raises(L.Leo2dError):
        m.set_params(np.full(m.n_params, np.nan, np.float32))
    m.close()


def test_training_learns_a_teacher(ctx):
    rng = np.random.default_rng(0)
    teacher = rng.normal(0, 1, mo.param_count())
    Ws, bs = mo.unpack(teacher)
    for l, d in enumerate(mo.IN_DIM):
        Ws[l] *= np.sqrt(1.0 / (mo.N_FEAT if l == 0 else d))
        if l == 0:
            Ws[l][:, mo.N_FEAT:] = 0
        bs[l] *= 0.1
    teacher = mo.pack(Ws, bs)
    x = rng.uniform(-1, 1, (8192, mo.N_FEAT)).astype(np.float32)
    t = mo.forward(teacher, x, exact=True).astype(np.float32)
    m = L.Mlp(ctx, seed=4)
    hist = m.train(x, t, steps=600, batch=1024, lr=2e-3, seed=1)
    assert hist.shape == (600,)
    assert np.all(np.isfinite(hist))
    assert hist[-20:].mean() < 0.05 * hist[:5].mean(), (hist[:5], hist[-5:])
    # held-out rows
    xv = rng.uniform(-1, 1, (2048, mo.N_FEAT)).astype(np.float32)
    tv = mo.forward(teacher, xv, exact=True)
    yv = m.predict(xv)
    assert np.mean((yv - tv) ** 2) < 0.1 * np.mean(tv ** 2)
    m.close()


def test_site_features_and_sum(ctx):
    twist = 1.3
    g = L.make_geom(model=L.MODEL_SIMPLE, size=30, angles_deg=(0.0, twist), energy_rescale=1.0)
    gp = ctx.prepare(g)
    csr = ctx.build_csr(gp)
    x = csr.site_features(twist)
    b = oracle.Built(gp)
    d = b.shift_configs()
    grid = b.index_to_grid.reshape(-1, 4)
    tp = 2 * np.pi
    d0, d1 = d[:, 0], d[:, 1]
    ref = np.stack([np.cos(tp * d0), np.sin(tp * d0), np.cos(tp * d1), np.sin(tp * d1),
                    np.cos(tp * (d0 + d1)), np.sin(tp * (d0 + d1)), np.cos(tp * (d0 - d1)),
                    np.sin(tp * (d0 - d1)), np.cos(2 * tp * d0), np.sin(2 * tp * d0),
                    np.cos(2 * tp * d1), np.sin(2 * tp * d1),
                    np.full_like(d0, np.float32(twist) / np.float32(3.0)),
                    grid[:, 3], grid[:, 2], np.ones_like(d0)], axis=1)
    np.testing.assert_allclose(x, ref, atol=1e-6)
    m = L.Mlp(ctx, seed=2)
    s = m.site_sum(csr, twist)
    y = m.predict(x).astype(np.float64)
    np.testing.assert_allclose(s, y.sum(axis=0), rtol=1e-6, atol=1e-6 * np.abs(y).sum(axis=0).max())
    m.close()


def test_bad_batch_is_rejected(ctx):
    m = L.Mlp(ctx)
    with pytest.raises(L.Leo2dError, match="multiple of 64"):
        m.grad(np.zeros((100, 16), np.float32), np.zeros((100, 256), np.float32))
    m.close()


@pytest.mark.parametrize("n", [1, 127, 129, 1000, 40_000, 100_003])
def test_fused_forward_matches_layered(n):
    """The fused forward (one persistent launch, activations on chip) against
    one GEMM per layer: same BF16 roundings and K order, so the outputs agree to
    FP32 accumulation order (1e-5 of the largest output). The sizes cover a
    single partial tile, a padding tile of the last pair, and several tile
    pairs per CTA."""
    rng = np.random.default_rng(n)
    x = rng.uniform(-1, 1, (n, mo.N_FEAT)).astype(np.float32)
    with L.Context(0) as c:
        m = L.Mlp(c, seed=6)
        c.set_option("mlp_fused", 1)
        y_fused = m.predict(x)
        c.set_option("mlp_fused", 0)
        y_layer = m.predict(x)
        m.close()
    scale = np.max(np.abs(y_layer))
    assert np.max(np.abs(y_fused - y_layer)) <= 1e-5 * scale


def test_fused_site_sum_matches_layered():
    """Site sums of the fused forward (warp transpose-reduce of the outputs, FP64
    per-lane partials) against the layer-by-layer sums over the same flake."""
    twist = 1.1
    with L.Context(0) as c:
        g = L.make_geom(model=L.MODEL_SIMPLE, size=160, angles_deg=(0.0, twist), energy_rescale=1.0)
        csr = c.build_csr(c.prepare(g))
        assert csr.n > 2 * 152 * 128  # several tile pairs per CTA
        m = L.Mlp(c, seed=8)
        c.set_option("mlp_fused", 1)
        s_fused = m.site_sum(csr, twist)
        c.set_option("mlp_fused", 0)
        s_layer = m.site_sum(csr, twist)
        c.set_option("mlp_fused", 1)
        y = m.predict(csr.site_features(twist)).astype(np.float64)
        m.close()
    tol = 1e-6 * np.abs(y).sum(axis=0).max()
    np.testing.assert_allclose(s_fused, s_layer, rtol=1e-6, atol=tol)
    np.testing.assert_allclose(s_fused, y.sum(axis=0), rtol=1e-6, atol=tol)
