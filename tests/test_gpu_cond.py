"""Kubo conductivity moments and transforms against the reference and the oracle.

Per-target moments (the reference's computeCondKPM) are compared with the
golden fixture where the reference defines them (first target, columns
0..P-2) and with the oracle everywhere. The recursion is FP32 with an FP64
moment GEMM: tolerance 1e-4 of the largest moment. The stochastic-trace form is
checked against the oracle on the same Philox vectors, the transforms against
the oracle to 1e-9.
"""
import numpy as np
import pytest

import leo2d_gb300 as L
from oracle import oracle
from tests._golden import load, parse_in

pytestmark = pytest.mark.gpu
FP32_RTOL = 1e-4


@pytest.fixture(scope="module")
def ctx():
    with L.Context(0) as c:
        yield c


def _rel(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


def test_golden_cond_moments(ctx):
    gold = load("flake_cond")
    g, kv = parse_in("flake_cond")
    P = int(gold["meta"][5])
    csr = ctx.build_csr(ctx.prepare(g), keep_zeros=True, with_dx=True)
    tg = gold["targets"].astype(np.int64)
    C = csr.kpm_cond(L.kpm_cfg(P), tg)
    ref = gold["cond_moments"].reshape(len(tg), P, P)
    assert _rel(C[0, :, :P - 1], ref[0, :, :P - 1]) < FP32_RTOL
    rp, col, val, dx, dy = csr.download(dx=True)
    o = oracle.kpm_cond(rp, col, val, dx, tg, P)
    assert _rel(C, o) < FP32_RTOL
    assert np.all(C[:, :, P - 1] == 0.0)


def test_trace_cond_vs_oracle(ctx):
    g = L.make_geom(model=L.MODEL_SIMPLE, size=14, angles_deg=(0.0, 3.0), energy_rescale=1.0)
    csr = ctx.build_csr(ctx.prepare(g), with_dx=True)
    lo, hi = csr.bounds()
    csr.rescale(1.01 * (hi - lo) / 2, -(hi + lo) / 2)
    rp, col, val, dx, dy = csr.download(dx=True)
    M, R, seed = 24, 5, 41
    mu = csr.kpm_cond(L.kpm_cfg(M, R=R, kind=L.VEC_PHASE, seed=seed))
    re, im = oracle.phase_vectors(seed, 0, R, csr.n)
    ref = (oracle.kpm_cond_trace(rp, col, val, dx, re, M) +
           oracle.kpm_cond_trace(rp, col, val, dx, im, M)) / R
    assert _rel(mu, ref) < FP32_RTOL


def test_cond_transform_and_sigma(ctx):
    rng = np.random.default_rng(3)
    P = 40
    M = rng.standard_normal((P, P))
    M = M + M.T
    np.testing.assert_allclose(ctx.cond_transform(M), oracle.cond_transform(M), rtol=1e-9, atol=1e-9)
    E = np.linspace(-1.1, 1.1, 2001)
    s = ctx.cond_sigma(M, E, 1.0, 0.0, 0.5)
    r = oracle.cond_sigma(M, E, 1.0, 0.0, 0.5)
    np.testing.assert_allclose(s, r, rtol=1e-9, atol=1e-9 * np.abs(r).max())


def test_cond_needs_dx(ctx):
    g = L.make_geom(size=6, energy_rescale=13.0)
    csr = ctx.build_csr(ctx.prepare(g))
    with pytest.raises(L.Leo2dError, match="WITH_DX"):
        csr.kpm_cond(L.kpm_cfg(8), [0])


def test_trace_cond_large_product(ctx):
    """256 x 256 trace moments: the moment product runs on the tensor cores over
    several output tiles and K ranges (three TF32 products, FP64 sum)."""
    g = L.make_geom(model=L.MODEL_SIMPLE, size=40, max_R=60.0, angles_deg=(0.0, 2.0), energy_rescale=1.0)
    csr = ctx.build_csr(ctx.prepare(g), with_dx=True)
    lo, hi = csr.bounds()
    csr.rescale(1.01 * (hi - lo) / 2, -(hi + lo) / 2)
    rp, col, val, dx, dy = csr.download(dx=True)
    M, R, seed = 256, 2, 8
    mu = csr.kpm_cond(L.kpm_cfg(M, R=R, kind=L.VEC_PHASE, seed=seed))
    re, im = oracle.phase_vectors(seed, 0, R, csr.n)
    ref = (oracle.kpm_cond_trace(rp, col, val, dx, re, M) + oracle.kpm_cond_trace(rp, col, val, dx, im, M)) / R
    assert _rel(mu, ref) < FP32_RTOL
