"""The row-block Chebyshev step (step_kernel = 3) against the gather kernel and
the FP64 oracle.

The row-block step sums each row over the sorted union of its block's columns
instead of its CSR order, so FP32 moments agree with the gather kernel's to
rounding (2e-5 of the largest) and with the FP64 oracle to 1e-4 (the FP32 bar).
Repeated runs are bit-identical; both FMA forms (scalar and paired FP32) and
every block width give the same results to rounding.
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


def _flake(ctx, size, twist, model=L.MODEL_SIMPLE, keep_zeros=False):
    g = L.make_geom(model=model, size=size, angles_deg=(0.0, twist), energy_rescale=1.0)
    csr = ctx.build_csr(ctx.prepare(g), keep_zeros=keep_zeros)
    lo, hi = csr.bounds()
    csr.rescale(1.01 * (hi - lo) / 2, -(hi + lo) / 2)
    return csr


def _run(ctx, variant, fn, **opts):
    ctx.set_option("step_kernel", variant)
    ctx.set_option("reorder", 1)
    for k, v in opts.items():
        ctx.set_option(k, v)
    try:
        return fn()
    finally:
        ctx.set_option("step_kernel", -1)
        ctx.set_option("reorder", -1)
        ctx.set_option("rb_packed", -1)
        ctx.set_option("rb_warps", 0)
        ctx.set_option("rb_unroll", 0)
        ctx.set_option("rb_window", -1)
        ctx.set_option("reorder_patch_dA", 0)
        ctx.set_option("tile_stages", 2)
        ctx.set_option("tile_chunk", 4)


@pytest.mark.parametrize("size,twist,model", [(22, 3.0, L.MODEL_SIMPLE), (37, 1.2, L.MODEL_SIMPLE),
                                             (25, 5.09, L.MODEL_REF)])
def test_rb_dos_matches(ctx, size, twist, model):
    csr = _flake(ctx, size, twist, model)
    P, R = 96, 16
    cfg = L.kpm_cfg(P, R=R, seed=3, block=32)
    ref = _run(ctx, 0, lambda: csr.kpm_dos(cfg))
    got = _run(ctx, 3, lambda: csr.kpm_dos(cfg))
    blocks, slots, union, max_slots, max_tile = csr.rb_info()
    assert blocks == (csr.n + 3) // 4
    assert union <= slots < union + 4 * blocks
    assert union < csr.nnz and max_slots > 0 and max_tile > 0
    assert _rel(got, ref) < 2e-5
    again = _run(ctx, 3, lambda: csr.kpm_dos(cfg))
    np.testing.assert_array_equal(got, again)
    for opts in ({"rb_packed": 0}, {"rb_warps": 16, "rb_unroll": 4}, {"rb_warps": 32, "rb_packed": 1},
                 {"reorder_patch_dA": 160}, {"rb_window": 1}, {"rb_window": 1, "rb_unroll": 8, "rb_packed": 0}):
        other = _run(ctx, 3, lambda: csr.kpm_dos(cfg), **opts)
        assert _rel(other, got) < 2e-5, opts
    rp, col, val = csr.download()
    re, im = oracle.phase_vectors(3, 0, R, csr.n)
    o = (oracle.kpm_trace(rp, col, val, re, P, literal=False) +
         oracle.kpm_trace(rp, col, val, im, P, literal=False))
    assert _rel(got, o) < 1e-4


@pytest.mark.parametrize("opts", [{"tile_stages": 3}, {"tile_chunk": 1}, {"tile_stages": 4, "tile_chunk": 16},
                                  {"rb_window": 1}, {"rb_window": 1, "tile_chunk": 1, "tile_stages": 3}])
def test_rb_pipeline_shapes(ctx, opts):
    """Stage counts and tile orders change the schedule, not the sums."""
    csr = _flake(ctx, 30, 2.0)
    cfg = L.kpm_cfg(64, R=16, seed=5, block=32)
    base = _run(ctx, 3, lambda: csr.kpm_dos(cfg))
    got = _run(ctx, 3, lambda: csr.kpm_dos(cfg), **opts)
    assert _rel(got, base) < 1e-6


def test_rb_ldos_and_stored_zeros(ctx):
    """Unit start vectors on a matrix that keeps its stored zeros."""
    csr = _flake(ctx, 28, 2.5, keep_zeros=True)
    P = 64
    targets = np.arange(0, csr.n, max(1, csr.n // 40))[:32]
    cfg = L.kpm_cfg(P, R=1, block=32)
    ref = _run(ctx, 0, lambda: csr.kpm_ldos(cfg, targets))
    got = _run(ctx, 3, lambda: csr.kpm_ldos(cfg, targets))
    assert _rel(got, ref) < 2e-5
    rp, col, val = csr.download()
    o = oracle.kpm_ldos(rp, col, val, targets, P)
    assert _rel(got, o) < 1e-4


def test_rb_host_vectors_and_rescale(ctx):
    """Host (Gaussian) vectors; after a second rescale the row blocks are rebuilt."""
    csr = _flake(ctx, 26, 1.6)
    P, R = 48, 20
    vec = np.random.default_rng(4).normal(size=(R, csr.n))
    cfg = L.kpm_cfg(P, R=R, kind=L.VEC_HOST, block=32)
    ref = _run(ctx, 0, lambda: csr.kpm_dos(cfg, vec))
    got = _run(ctx, 3, lambda: csr.kpm_dos(cfg, vec))
    assert _rel(got, ref) < 2e-5
    csr.rescale(1.5, 0.0)
    assert csr.rb_info()[0] == 0  # dropped with the ordered copy
    ref2 = _run(ctx, 0, lambda: csr.kpm_dos(cfg, vec))
    got2 = _run(ctx, 3, lambda: csr.kpm_dos(cfg, vec))
    assert _rel(got2, ref2) < 2e-5
    assert _rel(got2, got) > 1e-3  # the values really changed


def test_rb_ragged_last_block(ctx):
    """Row counts that leave a partial last block (n not a multiple of 4 rows)."""
    for size in (9, 11, 13):
        csr = _flake(ctx, size, 4.0)
        cfg = L.kpm_cfg(32, R=16, seed=9, block=32)
        ref = _run(ctx, 0, lambda: csr.kpm_dos(cfg))
        for window in (0, 1):
            got = _run(ctx, 3, lambda: csr.kpm_dos(cfg), rb_window=window)
            assert _rel(got, ref) < 2e-5, (size, csr.n, window)


@pytest.mark.parametrize("window", [0, 1])
def test_rb_timeout_reports(ctx, window):
    """The bounded wait of the row-block steps: a barrier nobody completes gives
    LEO2D_ERR_TIMEOUT, and the context keeps working afterwards."""
    csr = _flake(ctx, 20, 3.0)
    cfg = L.kpm_cfg(16, R=16, seed=1, block=32)
    ok = _run(ctx, 3, lambda: csr.kpm_dos(cfg), rb_window=window)
    ctx.set_spin_limit(2000)
    ctx.set_option("test_unsatisfied_wait", 1)
    try:
        with pytest.raises(L.Leo2dError) as e:
            _run(ctx, 3, lambda: csr.kpm_dos(cfg), rb_window=window)
        assert e.value.status == L._abi.ERR_TIMEOUT
        assert "wait ran out" in str(e.value)
    finally:
        ctx.set_option("test_unsatisfied_wait", 0)
        ctx.set_spin_limit(0)
    again = _run(ctx, 3, lambda: csr.kpm_dos(cfg), rb_window=window)
    np.testing.assert_array_equal(ok, again)


def test_row_blocks_are_the_default_where_ordered(ctx):
    """With the locality ordering on and no kernel forced, 32-column FP32
    recursions on a real matrix take the 8-row tensor-core row-block step; FP64
    and other widths keep the gather kernels."""
    csr = _flake(ctx, 24, 2.2)
    cfg = L.kpm_cfg(32, R=16, seed=4, block=32)
    ctx.set_option("reorder", 1)
    try:
        mu = csr.kpm_dos(cfg)
        assert csr.rt_info()[0] == (csr.n + 7) // 8
        assert csr.rb_info()[0] == 0
    finally:
        ctx.set_option("reorder", -1)
    ref = _run(ctx, 0, lambda: csr.kpm_dos(cfg))
    assert _rel(mu, ref) < 2e-5
