"""The tensor-core Chebyshev step (step_kernel = 2) against the gather kernel
and the FP64 oracle.

Three TF32 products per term keep about 22 bits, close to the FP32 recursion
of the gather kernels: moments agree with those to 2e-5 of the largest and with
the FP64 oracle to 1e-4 (the FP32 bar). Repeated runs are bit-identical.
"""
import numpy as np
import pytest

import leo2d_gb300 as L
from oracle import oracle

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


@pytest.fixture(scope="module")
def ctx():
    with L.Context(0) as c:
        yield c


def _flake(ctx, size, twist, model=L.MODEL_SIMPLE):
    g = L.make_geom(model=model, size=size, angles_deg=(0.0, twist), energy_rescale=1.0)
    csr = ctx.build_csr(ctx.prepare(g))
    lo, hi = csr.bounds()
    csr.rescale(1.01 * (hi - lo) / 2, -(hi + lo) / 2)
    return csr


def _run(ctx, variant, fn):
    ctx.set_option("step_kernel", variant)
    try:
        return fn()
    finally:
        ctx.set_option("step_kernel", -1)


@pytest.mark.parametrize("block", [32, 64])
@pytest.mark.parametrize("size,twist,model", [(22, 3.0, L.MODEL_SIMPLE), (37, 1.2, L.MODEL_SIMPLE),
                                             (25, 5.09, L.MODEL_REF)])
def test_tc_dos_matches(ctx, block, size, twist, model):
    csr = _flake(ctx, size, twist, model)
    P, R = 96, block // 2
    cfg = L.kpm_cfg(P, R=R, seed=3, block=block)
    ref = _run(ctx, 0, lambda: csr.kpm_dos(cfg))
    got = _run(ctx, 2, lambda: csr.kpm_dos(cfg))
    assert _rel(got, ref) < 2e-5
    again = _run(ctx, 2, lambda: csr.kpm_dos(cfg))
    np.testing.assert_array_equal(got, again)
    rp, col, val = csr.download()
    re, im = oracle.phase_vectors(3, 0, R, csr.n)
    o = (oracle.kpm_trace(rp, col, val, re, P, literal=False) +
         oracle.kpm_trace(rp, col, val, im, P, literal=False))
    assert _rel(got, o) < 1e-4


def test_tc_ldos_matches(ctx):
    csr = _flake(ctx, 30, 2.0)
    P = 64
    targets = np.arange(0, csr.n, max(1, csr.n // 40))[:32]
    cfg = L.kpm_cfg(P, R=1, block=32)
    ref = _run(ctx, 0, lambda: csr.kpm_ldos(cfg, targets))
    got = _run(ctx, 2, lambda: csr.kpm_ldos(cfg, targets))
    assert _rel(got, ref) < 2e-5
    rp, col, val = csr.download()
    o = oracle.kpm_ldos(rp, col, val, targets, P)
    assert _rel(got, o) < 1e-4


def test_tc_host_vectors_and_rescale(ctx):
    """Host (Gaussian) vectors; after a second rescale the tiles are rebuilt."""
    csr = _flake(ctx, 26, 1.6)
    P, R = 48, 20
    vec = np.random.default_rng(4).normal(size=(R, csr.n))
    cfg = L.kpm_cfg(P, R=R, kind=L.VEC_HOST, block=32)
    ref = _run(ctx, 0, lambda: csr.kpm_dos(cfg, vec))
    got = _run(ctx, 2, lambda: csr.kpm_dos(cfg, vec))
    assert _rel(got, ref) < 2e-5
    csr.rescale(1.5, 0.0)
    ref2 = _run(ctx, 0, lambda: csr.kpm_dos(cfg, vec))
    got2 = _run(ctx, 2, lambda: csr.kpm_dos(cfg, vec))
    assert _rel(got2, ref2) < 2e-5
    assert _rel(got2, got) > 1e-3  # the values really changed
