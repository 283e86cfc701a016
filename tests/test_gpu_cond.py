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


def _flake(ctx, size, twist, with_dx=True, max_R=None):
    g = L.make_geom(model=L.MODEL_SIMPLE, size=size, max_R=max_R, angles_deg=(0.0, twist), energy_rescale=1.0)
    csr = ctx.build_csr(ctx.prepare(g), with_dx=with_dx)
    lo, hi = csr.bounds()
    csr.rescale(1.01 * (hi - lo) / 2, -(hi + lo) / 2)
    return csr


def _opts(ctx, fn, **opts):
    for k, v in opts.items():
        ctx.set_option(k, v)
    try:
        return fn()
    finally:
        ctx.set_option("kubo_velocity", -1)
        ctx.set_option("kubo_chunk", 0)


@pytest.mark.parametrize("size,twist,R,kind", [(13, 3.0, 20, L.VEC_PHASE), (11, 4.4, 7, L.VEC_GAUSSIAN),
                                              (9, 2.0, 3, L.VEC_PHASE)])
def test_velocity_in_step_matches_stored_dx(ctx, size, twist, R, kind):
    """dxH built inside the row-block step from the flake's positions against the
    stored dxH (gather kernels, reference row order) and the FP64 oracle; ragged
    last passes (R not a multiple of the vectors per pass) and row counts that
    leave a partial last row block."""
    csr = _flake(ctx, size, twist)
    M, seed = 32, 17
    cfg = L.kpm_cfg(M, R=R, kind=kind, seed=seed)
    fly = csr.kpm_cond(cfg)
    assert csr.rb_info()[0] == (csr.n + 3) // 4  # the row blocks were built and used
    stored = _opts(ctx, lambda: csr.kpm_cond(cfg), kubo_velocity=0)
    assert _rel(fly, stored) < 2e-5
    if kind == L.VEC_PHASE:  # (Gaussian vectors: the stored-dxH path above is the check)
        rp, col, val, dx, dy = csr.download(dx=True)
        re, im = oracle.phase_vectors(seed, 0, R, csr.n)
        ref = (oracle.kpm_cond_trace(rp, col, val, dx, re, M) + oracle.kpm_cond_trace(rp, col, val, dx, im, M)) / R
        assert _rel(fly, ref) < FP32_RTOL


def test_velocity_in_step_needs_no_stored_dx(ctx):
    """A flake built without LEO2D_CSR_WITH_DX gives the same trace moments; the
    stored-dxH path still asks for it."""
    with_dx = _flake(ctx, 12, 2.5)
    without = _flake(ctx, 12, 2.5, with_dx=False)
    cfg = L.kpm_cfg(24, R=16, kind=L.VEC_PHASE, seed=3)
    np.testing.assert_array_equal(with_dx.kpm_cond(cfg), without.kpm_cond(cfg))
    with pytest.raises(L.Leo2dError, match="WITH_DX"):
        _opts(ctx, lambda: without.kpm_cond(cfg), kubo_velocity=0)


@pytest.mark.parametrize("chunk", [4, 8, 12, 64])
def test_velocity_chunks_of_b_side(ctx, chunk):
    """The B side built in chunks of moments (two-vector carry between chunks,
    each chunk's product into its columns of mu) gives the moments of one chunk."""
    csr = _flake(ctx, 14, 1.8)
    cfg = L.kpm_cfg(48, R=16, kind=L.VEC_PHASE, seed=9)
    whole = csr.kpm_cond(cfg)
    got = _opts(ctx, lambda: csr.kpm_cond(cfg), kubo_chunk=chunk)
    np.testing.assert_allclose(got, whole, rtol=0, atol=1e-12 * np.abs(whole).max())


def test_velocity_step_variants(ctx):
    """Every velocity-step variant (warps, FMA form, batches in flight) gives the
    same moments: the variants change the schedule, not the sums of a row block."""
    csr = _flake(ctx, 15, 2.2)
    cfg = L.kpm_cfg(32, R=16, kind=L.VEC_PHASE, seed=12)
    base = csr.kpm_cond(cfg)
    for w, p, u in ((16, 0, 4), (16, 1, 4), (16, 0, 8), (24, 0, 4)):
        got = _opts(ctx, lambda: csr.kpm_cond(cfg), rb_warps=w, rb_packed=p, rb_unroll=u)
        ctx.set_option("rb_warps", 0)
        ctx.set_option("rb_packed", -1)
        ctx.set_option("rb_unroll", 0)
        assert _rel(got, base) < 1e-6, (w, p, u)


def test_velocity_in_step_on_an_ordered_flake(ctx):
    """With the locality ordering on (what a flake of 1e5 orbitals or more gets by
    default), the DOS default is the 8-row step; the Kubo trace must still take the
    4-row velocity step for the A side, with the B side on the 8-row step, and
    need no stored dxH."""
    csr = _flake(ctx, 13, 3.0, with_dx=False)
    ref_csr = _flake(ctx, 13, 3.0)
    M, R, seed = 32, 16, 5
    cfg = L.kpm_cfg(M, R=R, kind=L.VEC_PHASE, seed=seed)
    ctx.set_option("reorder", 1)
    try:
        fly = csr.kpm_cond(cfg)
        assert csr.rb_info()[0] == (csr.n + 3) // 4  # the velocity step's 4-row blocks
        assert csr.rt_info()[0] == (csr.n + 7) // 8  # the B side's 8-row blocks
    finally:
        ctx.set_option("reorder", -1)
    stored = _opts(ctx, lambda: ref_csr.kpm_cond(cfg), kubo_velocity=0)
    assert _rel(fly, stored) < 2e-5
    rp, col, val, dx, dy = ref_csr.download(dx=True)
    re, im = oracle.phase_vectors(seed, 0, R, csr.n)
    ref = (oracle.kpm_cond_trace(rp, col, val, dx, re, M) + oracle.kpm_cond_trace(rp, col, val, dx, im, M)) / R
    assert _rel(fly, ref) < FP32_RTOL
